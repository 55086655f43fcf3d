// fft_engine_gpu.cpp -- drop-in replacement for the reference's engine
// translation units (prothlogic4.2/fft_engine.cpp + llr_fft_pack.cpp) on the
// hot path: same functions, same in-place limb contract, served by libprothgpu.
//
//   fft_init              (fft_engine.cpp:18-73)   -> records L; the device engine is created lazily
//   fft_destroy           (fft_engine.cpp:75-80)   -> pg_destroy
//   fft_square_karatsuba  (fft_engine.cpp:986-1073) -> v <- v^2 mod N, canonical, in place
//
// The reference leaves v congruent to v^2 but not reduced and reduces it in the
// caller (proth_logic.cpp:506-533); the GPU result is already canonical, so the
// caller's reduction finds nothing to do.  Like the reference engine, the shim
// writes exactly n_limbs limbs and drops what does not fit
// (fft_engine.cpp:925-983): the autotuner squares with n_limbs = (n+63)/64
// (dcore.cpp:23,59), one limb short of a residue mod k*2^n+1, and the test loop
// at the autotuned length (proth_logic.cpp:442) can be too; the full residue
// stays on the device, so only the caller's copy is truncated, and
// ctx.last_max_diff always carries the engine's real roundoff error.
//
// The residue stays on the device: the shim uploads v only when the caller
// changed it since the last call (a new x0, a loaded checkpoint) and returns
// the result every call, because the reference loop inspects v after each
// squaring.  The Gerbicz check runs on a block schedule (blocks of
// kBlock squarings, each verified by the check chain squared beside the
// residue), so a per-squaring call does not redo squarings to verify; a
// residue equal to N-1 (a prime's final value) is verified before the caller
// sees it.  fft_square_karatsuba_n returns a verified residue after `iters`
// squarings.
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/prothgpu.h"
#include "../../include/prothgpu_fftcompat.h"

namespace {

const uint32_t kBlock = 1000;     // Gerbicz block length (squarings)
const uint32_t kVerifyBlocks = 1; // verify every block

struct Shim {
    pg_engine* eng = nullptr;
    uint64_t k = 0;
    unsigned n = 0;
    std::vector<uint64_t> last;  // limbs the shim last wrote into the caller's buffer
    std::vector<uint64_t> full;  // the whole residue (n/64 + 3 limbs)
};

Shim* shim_of(FFTContext& ctx) { return static_cast<Shim*>(ctx.base_ptr); }

bool ensure_engine(FFTContext& ctx, unsigned n_bits, uint64_t k_val) {
    Shim* s = shim_of(ctx);
    if (!s) {
        s = new Shim();
        ctx.base_ptr = s;
    }
    if (s->eng && s->k == k_val && s->n == n_bits) return true;
    if (s->eng) pg_destroy(s->eng);
    s->eng = nullptr;
    s->last.clear();
    // the reference length is a hint only: the engine applies its own capacity rule
    if (pg_create(k_val, n_bits, 0, 0, &s->eng) != PG_OK) return false;
    if (pg_set_gerbicz(s->eng, kBlock, kVerifyBlocks) != PG_OK) return false;
    s->k = k_val;
    s->n = n_bits;
    s->full.assign(n_bits / 64 + 3, 0);
    return true;
}

// x == N - 1 = k * 2^n, with x in `full` limbs
bool is_n_minus_1(const std::vector<uint64_t>& x, uint64_t k, unsigned n) {
    const size_t q = n / 64;
    const unsigned r = n % 64;
    for (size_t i = 0; i < x.size(); ++i) {
        uint64_t want = 0;
        if (i == q) want = k << r;
        if (i == q + 1 && r) want = k >> (64 - r);
        if (x[i] != want) return false;
    }
    return true;
}

void square_n(FFTContext& ctx, uint64_t* v, size_t n_limbs, unsigned n_bits, uint64_t k_val, uint64_t iters) {
    if (!ensure_engine(ctx, n_bits, k_val)) {
        ctx.last_max_diff = 1.0;  // the reference reports failures only through last_max_diff
        return;
    }
    Shim* s = shim_of(ctx);
    if (s->last.size() != n_limbs || std::memcmp(s->last.data(), v, n_limbs * sizeof(uint64_t)) != 0) {
        if (pg_set_residue(s->eng, v, n_limbs) != PG_OK) {
            ctx.last_max_diff = 1.0;
            return;
        }
    }
    int rc = pg_square(s->eng, iters);
    if (rc == PG_OK) {
        size_t needed = 0;
        rc = iters > 1 ? pg_get_residue(s->eng, s->full.data(), s->full.size())
                       : pg_peek_residue(s->eng, s->full.data(), s->full.size(), &needed, nullptr);
        // a prime's final residue is N - 1: never hand that out unverified
        if (rc == PG_OK && iters <= 1 && is_n_minus_1(s->full, k_val, n_bits))
            rc = pg_get_residue(s->eng, s->full.data(), s->full.size());
    }
    if (rc == PG_OK) {
        std::memset(v, 0, n_limbs * sizeof(uint64_t));
        std::memcpy(v, s->full.data(), (n_limbs < s->full.size() ? n_limbs : s->full.size()) * sizeof(uint64_t));
    }
    double err = 0.0;
    pg_max_err(s->eng, &err, 1);
    ctx.last_max_diff = rc == PG_OK ? err : 1.0;
    s->last.assign(v, v + n_limbs);
    ctx.prof_calls += iters;
}

}  // namespace

bool fft_init(FFTContext& ctx, FFTBackend backend, size_t fft_len) {
    ctx.backend = backend;
    ctx.fft_len = fft_len;
    ctx.last_max_diff = 0.0;
    ctx.base_ptr = nullptr;
    ctx.raw_allocation = nullptr;
    ctx.total_allocation_size = 0;
    char name[64];
    int sms = 0;
    return pg_device_info(name, sizeof(name), &sms) == PG_OK;
}

void fft_destroy(FFTContext& ctx) {
    Shim* s = shim_of(ctx);
    if (s) {
        if (s->eng) pg_destroy(s->eng);
        delete s;
        ctx.base_ptr = nullptr;
    }
}

void fft_square_karatsuba(FFTContext& ctx, uint64_t* v, size_t n_limbs, unsigned n_bits, uint64_t k_val) {
    square_n(ctx, v, n_limbs, n_bits, k_val, 1);
}

void fft_square_karatsuba_n(FFTContext& ctx, uint64_t* v, size_t n_limbs, unsigned n_bits, uint64_t k_val,
                            uint64_t iters) {
    square_n(ctx, v, n_limbs, n_bits, k_val, iters);
}

// compat_driver.cpp -- callers written against the reference's engine API only
// (fft_init / fft_square_karatsuba / fft_destroy and FFTContext fields), in the
// shape of the reference's own callers, used by the tests and the bench to show
// the shim is a drop-in on machines where the reference sources themselves are
// not available to compile (oracle/ref/build_ref_callers.sh links the real
// callers where they are).
//
//   compat_driver <k> <n> <L> <steps>          x0 hex on stdin; RES64 and ctx.last_max_diff after
//                                              every squaring
//   compat_driver autotune <n> <k>             the FFT-length probe of auto_tune_fft_len
//                                              (dcore.cpp:20-81): all-ones residue of (n+63)/64 limbs,
//                                              100 squarings per length, accept max err <= 0.30
//   compat_driver test <k> <n> <L> [steps]     x0 = a^k mod N hex on stdin; the squaring loop of
//                                              execute_proth_test_fft (proth_logic.cpp:442-552): a
//                                              worker-sized limb buffer (dcore.cpp:143-155),
//                                              n_limbs = L/4, one fft_square_karatsuba per step, the
//                                              clear above 2n/64+4, the reduction test, and the
//                                              final is_nm1_limbs check on L/4 limbs
#include <cctype>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/prothgpu_fftcompat.h"

static std::vector<uint64_t> read_hex(size_t n_limbs) {
    std::string hex;
    for (int ch; (ch = getchar()) != EOF;)
        if (isxdigit(ch)) hex.push_back((char)ch);
    std::vector<uint64_t> limbs(n_limbs, 0);
    for (size_t i = 0; i < hex.size() && i / 16 < n_limbs; ++i) {
        const char c = hex[hex.size() - 1 - i];
        const uint64_t d = isdigit((unsigned char)c) ? c - '0' : (c | 32) - 'a' + 10;
        limbs[i / 16] |= d << (4 * (i % 16));
    }
    return limbs;
}

static int trace(int argc, char** argv) {
    const uint64_t k = strtoull(argv[1], nullptr, 10);
    const unsigned n = (unsigned)strtoul(argv[2], nullptr, 10);
    const size_t L = strtoull(argv[3], nullptr, 10);
    const unsigned long steps = strtoul(argv[4], nullptr, 10);
    (void)argc;
    FFTContext ctx;
    if (!fft_init(ctx, FFTBackend::INTERNAL, L)) {
        fprintf(stderr, "fft_init failed\n");
        return 3;
    }
    const size_t n_limbs = ctx.fft_len / 4;  // n_limbs_safe (proth_logic.cpp:442)
    std::vector<uint64_t> limbs = read_hex(n_limbs);
    for (unsigned long i = 0; i < steps; ++i) {
        fft_square_karatsuba(ctx, limbs.data(), n_limbs, n, k);
        printf("%lu %016llx %.3g\n", i, (unsigned long long)limbs[0], ctx.last_max_diff);
    }
    fft_destroy(ctx);
    return 0;
}

// The length probe of auto_tune_fft_len (dcore.cpp:20-81), call for call.
static int autotune(unsigned n, uint64_t k) {
    const size_t n_limbs = (n + 63) / 64;
    size_t L = 256;
    while ((double)n / (double)L > 18.0) L *= 2;
    for (;;) {
        if ((double)n / (double)L < 11.0) break;
        FFTContext ctx;
        if (!fft_init(ctx, FFTBackend::INTERNAL, L)) {
            L *= 2;
            continue;
        }
        std::vector<uint64_t> v(std::max(L, (size_t)((2 * n) / 64 + 64)), 0);
        for (size_t i = 0; i < n_limbs; ++i) v[i] = ~0ull;
        v[0] = k | 1;
        for (int step = 0; step < 100; ++step) fft_square_karatsuba(ctx, v.data(), n_limbs, n, k);
        const double err = ctx.last_max_diff;
        fft_destroy(ctx);
        printf("PROBE %zu %.6g\n", L, err);
        if (err >= 0.0 && err <= 0.30) break;
        L *= 2;
    }
    printf("L %zu\n", L);
    return 0;
}

// is_nm1_limbs (proth_logic.cpp:336-355): v == k * 2^n within n_limbs limbs.
static bool is_nm1(const uint64_t* v, size_t n_limbs, unsigned n, uint64_t k) {
    std::vector<uint64_t> t(n_limbs, 0);
    const size_t limb = n / 64;
    const unsigned shift = n % 64;
    if (limb < n_limbs) {
        t[limb] = k << shift;
        if (shift != 0 && limb + 1 < n_limbs) t[limb + 1] = k >> (64 - shift);
    }
    return std::memcmp(v, t.data(), n_limbs * 8) == 0;
}

// The squaring loop of execute_proth_test_fft (proth_logic.cpp:442-552) from a
// fresh x0 (no checkpoint file), with the limb handling of the worker
// (dcore.cpp:143-155) and of the loop body (:488-533).
static int test(uint64_t k, unsigned n, size_t L, unsigned long max_steps) {
    FFTContext ctx;
    if (!fft_init(ctx, FFTBackend::INTERNAL, L)) return 3;
    const size_t alloc = std::max(L, (size_t)((2 * n) / 64 + 64));
    const size_t n_limbs = ctx.fft_len / 4;
    std::vector<uint64_t> limbs(alloc, 0);
    {
        const std::vector<uint64_t> x0 = read_hex(n_limbs);
        std::memcpy(limbs.data(), x0.data(), n_limbs * 8);
    }
    ctx.last_max_diff = 0.0;
    double max_err = 0.0;
    unsigned long reduce_calls = 0, steps = 0;
    size_t last_hi = (n + 64) / 64 + 10;
    const unsigned long end = max_steps ? std::min<unsigned long>(max_steps, n - 1) : n - 1;
    const auto t0 = std::chrono::steady_clock::now();
    for (unsigned long i = 0; i < end; ++i) {
        fft_square_karatsuba(ctx, limbs.data(), n_limbs, n, k);
        max_err = std::max(max_err, ctx.last_max_diff);
        const size_t max_sq_limbs = (2 * n) / 64 + 4;
        if (max_sq_limbs < n_limbs) {
            std::memset(limbs.data() + max_sq_limbs, 0, (n_limbs - max_sq_limbs) * 8);
        }
        const size_t cut_limb = n >> 6;
        size_t search_start = std::min(last_hi * 2 + 5, n_limbs);
        size_t hi = 0;
        for (size_t j = search_start; j-- > 0;)
            if (limbs[j]) {
                hi = j;
                break;
            }
        last_hi = hi;
        // the reference calls proth_reduce_stage1 here whenever the top limb reaches
        // bit n (:506-533); the shim's residue is already canonical, which that
        // reduction leaves unchanged, so the call is counted, not made
        if (hi >= cut_limb) reduce_calls++;
        steps++;
    }
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    const int prime = steps == n - 1 && is_nm1(limbs.data(), n_limbs, n, k);
    printf("RESULT %d %016llx %lu %.3f %.3g %lu\n", prime, (unsigned long long)limbs[0], steps,
           steps ? s * 1e6 / steps : 0.0, max_err, reduce_calls);
    fft_destroy(ctx);
    return 0;
}

int main(int argc, char** argv) {
    if (argc >= 4 && std::string(argv[1]) == "autotune")
        return autotune((unsigned)strtoul(argv[2], nullptr, 10), strtoull(argv[3], nullptr, 10));
    if (argc >= 5 && std::string(argv[1]) == "test")
        return test(strtoull(argv[2], nullptr, 10), (unsigned)strtoul(argv[3], nullptr, 10),
                    strtoull(argv[4], nullptr, 10), argc >= 6 ? strtoul(argv[5], nullptr, 10) : 0);
    if (argc >= 5) return trace(argc, argv);
    return 2;
}

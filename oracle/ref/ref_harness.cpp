// Test harness around the UNMODIFIED reference engine (compiled from the
// reference sources by build_ref.sh into oracle/_ref/).  Test infrastructure only.
//
//   ref_harness trace <k> <n> <L> <steps> <x0_hex | - (hex on stdin)>
//       runs <steps> reference squarings (fft_square_karatsuba, fft_engine.cpp:986)
//       at FFT length L from x0, canonicalising each step with GMP mpz_mod, and
//       prints "i res64 maxerr" per step.
//   ref_harness test <k> <n> <L>
//       runs execute_proth_test_fft (proth_logic.cpp:384) and prints
//       "verdict res64 maxerr".
//   ref_harness time <k> <n> <L> <steps>
//       engine-only microseconds per squaring.
//   ref_harness ckpt_save <k> <n> <L> <current_i> <path>   (hex residue on stdin)
//       writes a checkpoint with the reference's save_checkpoint (checkpoint_manager.cpp:8-23).
#include "checkpoint_manager.h"
#include "fft_engine.h"
#include "proth_logic.h"
#include <cctype>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

std::mutex g_io_mutex;  // defined by the reference's worker.cpp, not linked here

static std::vector<uint64_t> parse_hex(const char* s, size_t nl) {
    std::vector<uint64_t> v(nl, 0);
    size_t len = strlen(s);
    for (size_t i = 0; i < len; ++i) {
        char c = s[len - 1 - i];
        uint64_t d = (c >= '0' && c <= '9') ? c - '0' : (c | 32) - 'a' + 10;
        v[i / 16] |= d << (4 * (i % 16));
    }
    return v;
}

int main(int argc, char** argv) {
    if (argc < 5) return 2;
    std::string mode = argv[1];
    uint64_t k = strtoull(argv[2], nullptr, 10);
    unsigned n = (unsigned)strtoul(argv[3], nullptr, 10);
    size_t L = strtoull(argv[4], nullptr, 10);
    FFTContext ctx;
    if (!fft_init(ctx, FFTBackend::INTERNAL, L)) return 3;
    const size_t nl = L / 4;
    size_t alloc = std::max(L, (size_t)((2 * n) / 64 + 64));
    std::vector<uint64_t> limbs(alloc, 0);
    if (mode == "ckpt_save") {
        std::string hex;
        for (int ch; (ch = getchar()) != EOF;)
            if (isxdigit(ch)) hex.push_back((char)ch);
        std::vector<uint64_t> x = parse_hex(hex.c_str(), nl);
        const uint64_t ci = strtoull(argv[5], nullptr, 10);
        return save_checkpoint(ci, nl, x.data(), argv[6]) ? 0 : 4;
    }
    if (mode == "test") {
        bool prime = execute_proth_test_fft(k, n, limbs.data(), ctx, 0);
        printf("%d %016llx %.6g\n", prime ? 1 : 0, (unsigned long long)limbs[0], ctx.last_max_diff);
        return 0;
    }
    if (mode == "trace" || mode == "time") {
        unsigned long steps = strtoul(argv[5], nullptr, 10);
        std::vector<uint64_t> x0(nl, 0);
        if (mode == "trace") {
            std::string hex = argv[6];
            if (hex == "-") {  // read the hex residue from standard input
                hex.clear();
                int ch;
                while ((ch = getchar()) != EOF)
                    if (isxdigit(ch)) hex.push_back((char)ch);
            }
            x0 = parse_hex(hex.c_str(), nl);
        }
        if (mode == "time") for (size_t i = 0; i < n / 64; ++i) x0[i] = 0x9E3779B97F4A7C15ULL * (i + 1);
        memcpy(limbs.data(), x0.data(), nl * 8);
        mpz_t N, r;
        mpz_init(N); mpz_init(r);
        mpz_set_ui(N, k); mpz_mul_2exp(N, N, n); mpz_add_ui(N, N, 1);
        auto t0 = std::chrono::steady_clock::now();
        for (unsigned long i = 0; i < steps; ++i) {
            fft_square_karatsuba(ctx, limbs.data(), nl, n, k);
            if (mode == "trace") {
                mpz_import(r, nl, -1, 8, 0, 0, limbs.data());
                mpz_mod(r, r, N);
                std::fill(limbs.begin(), limbs.begin() + nl, 0);
                mpz_export(limbs.data(), nullptr, -1, 8, 0, 0, r);
                printf("%lu %016llx %.6g\n", i, (unsigned long long)limbs[0], ctx.last_max_diff);
            }
        }
        auto t1 = std::chrono::steady_clock::now();
        if (mode == "time")
            printf("%.3f\n", std::chrono::duration<double, std::micro>(t1 - t0).count() / steps);
        return 0;
    }
    return 2;
}

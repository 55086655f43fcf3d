// compat_driver.cpp -- a caller written against the reference's engine API only
// (fft_init / fft_square_karatsuba / fft_destroy and FFTContext fields), in the
// shape of the reference's squaring loop (proth_logic.cpp:485-549): it squares
// a residue held in host limbs, reads ctx.last_max_diff, and prints RES64 after
// every squaring.  Used by the tests to show the shim is a drop-in.
//
//   compat_driver <k> <n> <L> <steps> <x0 hex on stdin>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../include/prothgpu_fftcompat.h"

int main(int argc, char** argv) {
    if (argc < 5) return 2;
    const uint64_t k = strtoull(argv[1], nullptr, 10);
    const unsigned n = (unsigned)strtoul(argv[2], nullptr, 10);
    const size_t L = strtoull(argv[3], nullptr, 10);
    const unsigned long steps = strtoul(argv[4], nullptr, 10);
    std::string hex;
    for (int ch; (ch = getchar()) != EOF;)
        if (isxdigit(ch)) hex.push_back((char)ch);
    FFTContext ctx;
    if (!fft_init(ctx, FFTBackend::INTERNAL, L)) {
        fprintf(stderr, "fft_init failed\n");
        return 3;
    }
    const size_t n_limbs = ctx.fft_len / 4;  // n_limbs_safe (proth_logic.cpp:442)
    std::vector<uint64_t> limbs(n_limbs, 0);
    for (size_t i = 0; i < hex.size(); ++i) {
        const char c = hex[hex.size() - 1 - i];
        const uint64_t d = isdigit((unsigned char)c) ? c - '0' : (c | 32) - 'a' + 10;
        limbs[i / 16] |= d << (4 * (i % 16));
    }
    for (unsigned long i = 0; i < steps; ++i) {
        fft_square_karatsuba(ctx, limbs.data(), n_limbs, n, k);
        printf("%lu %016llx %.3g\n", i, (unsigned long long)limbs[0], ctx.last_max_diff);
    }
    fft_destroy(ctx);
    return 0;
}

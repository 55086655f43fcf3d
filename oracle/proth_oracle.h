/*
 * proth_oracle.h -- CPU oracle for the Proth modular-squaring path.
 *
 * TEST INFRASTRUCTURE ONLY.  The tests, the
 * smoke check and the CPU-baseline leg of bench.py call it to produce the
 * expected residues and to time the reference algorithm on host cores.  The
 * product (prothlogic_gb300 / libprothgpu) never links, loads or calls it.
 *
 * It restates, in portable C, the algorithm of ProthLogic 4.2 for this path:
 *   prothlogic4.2/llr_fft_pack.cpp:12-41     pack_karatsuba_limbs
 *   prothlogic4.2/fft_engine.cpp:18-73       fft_init (twiddle LUT)
 *   prothlogic4.2/fft_engine.cpp:234-494     fft_stockham_radix8 / :700-820 fft_bailey_2d
 *                                            (any exact complex DFT gives the same rounded
 *                                             integers; restated as Stockham radix-4/2)
 *   prothlogic4.2/fft_engine.cpp:1023-1055   pointwise A^2, B^2, 2AB, x 1/L
 *   prothlogic4.2/fft_engine.cpp:825-984     unpack_karatsuba_overlap_add
 *   prothlogic4.2/fft_engine.cpp:986-1073    fft_square_karatsuba
 *   prothlogic4.2/proth_logic.cpp:250-334    proth_reduce_stage1 (canonicalise mod N)
 *   prothlogic4.2/proth_logic.cpp:41-50      is_divisible_by_gate
 *   prothlogic4.2/proth_logic.cpp:384-580    execute_proth_test_fft (gate, base, a^k, loop, verdict)
 *   prothlogic4.2/dcore.cpp:20-81            auto_tune_fft_len
 *
 * GMP (mpz_jacobi, mpz_powm), which the reference calls for the base choice and
 * for x0 = a^k mod N, is restated here too: the Jacobi symbol by quadratic
 * reciprocity and a^k mod N by left-to-right binary exponentiation.
 *
 * Parity is pinned in tests/ against GMP (libgmp.so.10 through ctypes), against
 * golden vectors produced by the reference engine itself (tests/golden/), and
 * against the known answers of the reference's console log.
 */
#ifndef PROTH_ORACLE_H
#define PROTH_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_ctx ora_ctx;

/* FFT length L (complex points, power of two >= 16). Returns NULL on failure. */
ora_ctx* ora_create(size_t L);
void ora_destroy(ora_ctx* c);
size_t ora_fft_len(const ora_ctx* c);
/* max |x - round(x)| of the last engine squaring (reference ctx.last_max_diff). */
double ora_last_max_err(const ora_ctx* c);

/* The reference's engine step on n_limbs = L/4 limbs (fft_square_karatsuba):
 * v <- value congruent to v^2 mod k*2^n+1, not necessarily reduced. */
void ora_engine_square(ora_ctx* c, uint64_t* v, size_t n_limbs, unsigned n, uint64_t k);

/* Canonicalise v (n_limbs limbs) into [0, N). Returns 0 on success. */
int ora_reduce(uint64_t* v, size_t n_limbs, unsigned n, uint64_t k);

/* One full step of the reference loop: engine square, clear garbage limbs,
 * reduce (proth_logic.cpp:488-533). v must have n_limbs = L/4 limbs. */
double ora_square_mod(ora_ctx* c, uint64_t* v, unsigned n, uint64_t k);

/* v <- v * s mod N for a small multiplier s (< 2^32); v canonical, n_limbs limbs. */
void ora_mul_small_mod(uint64_t* v, size_t n_limbs, unsigned n, uint64_t k, uint64_t s);

/* Reference gate: 1 if p divides k*2^n+1 (proth_logic.cpp:41-50). */
int ora_gate_divisible(uint64_t k, unsigned n, uint64_t p);
/* 1 if any gate prime <= 67 divides N (the reference then reports composite). */
int ora_gate_rejects(uint64_t k, unsigned n);
/* Jacobi symbol (a / k*2^n+1) for a small a >= 1. */
int ora_jacobi_small(uint64_t a, uint64_t k, unsigned n);
/* The reference base choice (proth_logic.cpp:411-422): 0 if none below 100. */
uint64_t ora_choose_base(uint64_t k, unsigned n);

/* Corrected FFT length: smallest power of two L >= max(autotune start, 16) with
 * n + bitlen(k) + 64 <= 16 L. */
size_t ora_choose_L(unsigned n, uint64_t k);
/* The reference autotune (dcore.cpp:20-81), restated, including its 100 test
 * squarings. Can return an L that is too small for n (the reference's bug). */
size_t ora_autotune_L(unsigned n, uint64_t k);

/* x <- a^e mod N with the oracle's own squaring (ctx length L, x has L/4 limbs). */
void ora_powm_small(ora_ctx* c, uint64_t* x, uint64_t a, uint64_t e, unsigned n, uint64_t k);

/* Full Proth test as execute_proth_test_fft does it, without checkpoint files.
 * L = 0 picks ora_choose_L. Returns 1 prime, 0 composite, -1 error.
 * Outputs (each may be NULL): base a (0 when the gate rejected), RES64 = limb 0
 * of the final residue a^((N-1)/2) mod N, and the largest roundoff error seen.
 * If trace != NULL it receives limb 0 of the residue after each of the first
 * trace_len squarings. */
int ora_proth_test(uint64_t k, unsigned n, size_t L, uint64_t* a_out, uint64_t* res64_out,
                   double* max_err_out, uint64_t* trace, size_t trace_len);

/* Run `iters` reference steps from the canonical residue x (L/4 limbs). */
double ora_run_squarings(ora_ctx* c, uint64_t* x, unsigned n, uint64_t k, uint64_t iters);

/* Smallest odd prime p < bound dividing k*2^n+1, or 0 (trial division, the
 * question check_proth_candidates_kernel answers per prime, gpu_engine.cu:290-320). */
uint64_t ora_smallest_factor(uint64_t k, unsigned n, uint64_t bound);

/* CPU-baseline helper: run `count` independent Proth tests on `threads` POSIX
 * threads (one FFT context per thread, like the reference dispatch), each test
 * truncated to `squarings_per_test` squarings (0 = full test). Returns the wall
 * seconds; res64_out[i] receives each test's RES64 (may be NULL). */
double ora_bench_tests(const uint64_t* ks, const unsigned* ns, size_t count, int threads,
                       uint64_t squarings_per_test, uint64_t* res64_out);

#ifdef __cplusplus
}
#endif
#endif

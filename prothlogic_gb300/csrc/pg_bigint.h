// pg_bigint.h -- host-side multi-limb helpers for N = k*2^n + 1.
//
// Only O(size) work lives here: conversions between canonical residues (the
// little-endian limbs the reference's loop holds) and the engine's device
// representation (Montgomery form, balanced digits), plus the small-integer
// pieces of the Proth test (gate, Jacobi symbol, base choice).
#ifndef PG_BIGINT_H
#define PG_BIGINT_H

#include <cstddef>
#include <cstdint>
#include <vector>

namespace pg {

using Limbs = std::vector<uint64_t>;

void trim(Limbs& a);
int cmp(const Limbs& a, const Limbs& b);
Limbs make_N(uint64_t k, unsigned n);                  // k*2^n + 1
// x mod N for any non-negative x (split at bit n, divide the high part by k,
// 2^n = -1/k mod N; the quotient is reduced recursively).
Limbs mod_N(const Limbs& x, uint64_t k, unsigned n);
// Montgomery conversions with R = 2^n: y = x R mod N and x = y R^-1 = -k y mod N.
Limbs to_mont(const Limbs& x_canonical, uint64_t k, unsigned n);
Limbs from_mont(const Limbs& y_canonical, uint64_t k, unsigned n);
// Canonical value -> balanced digits d[0..M) (S_j = ceil(j n / M)) and top.
void value_to_digits(const Limbs& y, unsigned M, unsigned n, int32_t* d, long long* top);
// Signed digits + top -> canonical value mod N.
Limbs digits_to_value(const int32_t* d, unsigned M, unsigned n, long long top, uint64_t k);
bool is_N_minus_1(const Limbs& x, uint64_t k, unsigned n);
Limbs mul_small(const Limbs& a, uint64_t s);

// Proth-test small-integer steps (same decisions as prothlogic4.2/proth_logic.cpp:41-50, 400-422).
bool gate_divisible(uint64_t k, unsigned n, uint64_t p);
bool gate_rejects(uint64_t k, unsigned n);
int jacobi_small(uint64_t a, uint64_t k, unsigned n);
uint64_t choose_base(uint64_t k, unsigned n);
unsigned bitlen(uint64_t x);

}  // namespace pg

#endif

// pg_bigint.cpp -- host-side multi-limb helpers (see pg_bigint.h).
#include "pg_bigint.h"

#include <algorithm>

namespace pg {

typedef unsigned __int128 u128;
typedef __int128 i128;

void trim(Limbs& a) {
    while (!a.empty() && a.back() == 0) a.pop_back();
}

int cmp(const Limbs& a0, const Limbs& b0) {
    size_t na = a0.size(), nb = b0.size();
    while (na > 0 && a0[na - 1] == 0) --na;
    while (nb > 0 && b0[nb - 1] == 0) --nb;
    if (na != nb) return na < nb ? -1 : 1;
    for (size_t i = na; i-- > 0;)
        if (a0[i] != b0[i]) return a0[i] < b0[i] ? -1 : 1;
    return 0;
}

static Limbs shl_word(uint64_t r, unsigned s) {  // r * 2^s
    Limbs out(s / 64 + 2, 0);
    const unsigned q = s / 64, b = s % 64;
    out[q] = r << b;
    if (b) out[q + 1] = r >> (64 - b);
    trim(out);
    return out;
}

Limbs make_N(uint64_t k, unsigned n) {
    Limbs N = shl_word(k, n);
    if (N.empty()) N.push_back(0);
    N[0] |= 1;  // bit 0 of k*2^n is clear for n >= 1
    return N;
}

static Limbs add(const Limbs& a, const Limbs& b) {
    Limbs out(std::max(a.size(), b.size()) + 1, 0);
    u128 c = 0;
    for (size_t i = 0; i < out.size(); ++i) {
        u128 s = c;
        if (i < a.size()) s += a[i];
        if (i < b.size()) s += b[i];
        out[i] = (uint64_t)s;
        c = s >> 64;
    }
    trim(out);
    return out;
}

static Limbs sub(const Limbs& a, const Limbs& b) {  // requires a >= b
    Limbs out(a.size(), 0);
    uint64_t br = 0;
    for (size_t i = 0; i < a.size(); ++i) {
        const uint64_t bi = i < b.size() ? b[i] : 0;
        const uint64_t d = a[i] - bi - br;
        br = (a[i] < bi) || (a[i] - bi < br);
        out[i] = d;
    }
    trim(out);
    return out;
}

static Limbs shr_bits(const Limbs& x, unsigned s) {
    const size_t q = s / 64;
    const unsigned b = s % 64;
    if (q >= x.size()) return Limbs();
    Limbs out(x.size() - q, 0);
    for (size_t i = 0; i < out.size(); ++i) {
        uint64_t v = x[i + q] >> b;
        if (b && i + q + 1 < x.size()) v |= x[i + q + 1] << (64 - b);
        out[i] = v;
    }
    trim(out);
    return out;
}

static Limbs low_bits(const Limbs& x, unsigned s) {
    const size_t q = s / 64;
    const unsigned b = s % 64;
    Limbs out(x.begin(), x.begin() + std::min(x.size(), q + 1));
    if (q < out.size()) {
        if (b == 0) out.resize(q);
        else out[q] &= (1ULL << b) - 1;
    }
    trim(out);
    return out;
}

static uint64_t divmod_small(Limbs& a, uint64_t d) {
    u128 rem = 0;
    for (size_t i = a.size(); i-- > 0;) {
        const u128 cur = (rem << 64) | a[i];
        a[i] = (uint64_t)(cur / d);
        rem = cur % d;
    }
    trim(a);
    return (uint64_t)rem;
}

Limbs mul_small(const Limbs& a, uint64_t s) {
    Limbs out(a.size() + 1, 0);
    u128 c = 0;
    for (size_t i = 0; i < a.size(); ++i) {
        const u128 p = (u128)a[i] * s + c;
        out[i] = (uint64_t)p;
        c = p >> 64;
    }
    out[a.size()] = (uint64_t)c;
    trim(out);
    return out;
}

Limbs mod_N(const Limbs& x, uint64_t k, unsigned n) {
    Limbs v = x;
    trim(v);
    const Limbs N = make_N(k, n);
    if (cmp(v, N) < 0) return v;
    Limbs hi = shr_bits(v, n);
    const Limbs lo = low_bits(v, n);
    const uint64_t r = divmod_small(hi, k);  // hi <- quotient
    // v = (q k + r) 2^n + lo = q (N - 1) + r 2^n + lo = r 2^n + lo - q  (mod N)
    const Limbs qm = mod_N(hi, k, n);
    const Limbs A = add(lo, shl_word(r, n));  // < N
    if (cmp(A, qm) >= 0) return sub(A, qm);
    return sub(add(A, N), qm);
}

Limbs to_mont(const Limbs& x, uint64_t k, unsigned n) {
    // x = q k + r:  x 2^n = -x/k = r 2^n - q  (mod N), using 1/k = -2^n
    Limbs q = mod_N(x, k, n);
    const uint64_t r = divmod_small(q, k);
    const Limbs A = shl_word(r, n);
    if (cmp(A, q) >= 0) return sub(A, q);
    return sub(add(A, make_N(k, n)), q);
}

Limbs from_mont(const Limbs& y, uint64_t k, unsigned n) {
    const Limbs t = mod_N(mul_small(y, k), k, n);
    if (t.empty()) return t;
    return sub(make_N(k, n), t);
}

static inline uint64_t digit_pos(uint64_t j, unsigned n, unsigned M) {
    return (uint64_t)(((u128)j * n + M - 1) / M);
}

static uint64_t get_bits(const Limbs& y, uint64_t pos, unsigned b) {  // b <= 32
    const size_t q = pos / 64;
    const unsigned s = pos % 64;
    if (q >= y.size()) return 0;
    u128 w = y[q] >> s;
    if (s && q + 1 < y.size()) w |= (u128)y[q + 1] << (64 - s);
    return (uint64_t)(w & ((1ULL << b) - 1));
}

void value_to_digits(const Limbs& y, unsigned M, unsigned n, int32_t* d, long long* top) {
    long long carry = 0;
    for (unsigned j = 0; j < M; ++j) {
        const uint64_t s0 = digit_pos(j, n, M), s1 = digit_pos(j + 1, n, M);
        const unsigned b = (unsigned)(s1 - s0);
        long long v = (long long)get_bits(y, s0, b) + carry;
        if (v >= (1LL << (b - 1))) {
            v -= (1LL << b);
            carry = 1;
        } else {
            carry = 0;
        }
        d[j] = (int32_t)v;
    }
    const Limbs hi = shr_bits(y, n);
    *top = (long long)(hi.empty() ? 0 : hi[0]) + carry;
}

Limbs digits_to_value(const int32_t* d, unsigned M, unsigned n, long long top, uint64_t k) {
    const size_t W = n / 64 + 4;
    Limbs out(W, 0);
    i128 acc = 0;
    uint64_t pos = 0;
    size_t li = 0;
    auto emit_to = [&](uint64_t s) {
        while (s - pos >= 64) {
            out[li++] = (uint64_t)acc;
            acc >>= 64;
            pos += 64;
        }
    };
    for (unsigned j = 0; j < M; ++j) {
        const uint64_t s = digit_pos(j, n, M);
        emit_to(s);
        acc += (i128)d[j] << (s - pos);
    }
    emit_to(n);
    acc += (i128)top << (n - pos);
    while (li < W) {
        out[li++] = (uint64_t)acc;
        acc >>= 64;
    }
    // two's complement over W limbs; add N until non-negative
    const Limbs N = make_N(k, n);
    for (int guard = 0; (out[W - 1] >> 63) && guard < 64; ++guard) {
        u128 c = 0;
        for (size_t i = 0; i < W; ++i) {
            const u128 s = (u128)out[i] + (i < N.size() ? N[i] : 0) + c;
            out[i] = (uint64_t)s;
            c = s >> 64;
        }
    }
    return mod_N(out, k, n);
}

bool is_N_minus_1(const Limbs& x, uint64_t k, unsigned n) {
    return cmp(x, shl_word(k, n)) == 0;
}

// ---- small-integer helpers ----

static uint64_t mulmod(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)(((u128)a * b) % m); }
static uint64_t powmod(uint64_t a, uint64_t e, uint64_t m) {
    uint64_t r = 1 % m;
    a %= m;
    for (; e; e >>= 1) {
        if (e & 1) r = mulmod(r, a, m);
        a = mulmod(a, a, m);
    }
    return r;
}

bool gate_divisible(uint64_t k, unsigned n, uint64_t p) {
    // p | k 2^n + 1  <=>  2^n = -k^-1 (mod p), for odd prime p not dividing k
    if (p % 2 == 0) return false;
    const uint64_t km = k % p;
    if (km == 0) return false;
    const uint64_t target = mulmod(p - 1, powmod(km, p - 2, p), p);
    return powmod(2, n, p) == target;
}

bool gate_rejects(uint64_t k, unsigned n) {
    static const uint64_t gp[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67};
    for (uint64_t p : gp)
        if (gate_divisible(k, n, p)) return true;
    return false;
}

static uint64_t N_mod(uint64_t k, unsigned n, uint64_t m) {
    return (mulmod(k % m, powmod(2, n, m), m) + 1) % m;
}

static int jacobi_odd(uint64_t a, uint64_t m) {  // m odd > 0
    int r = 1;
    a %= m;
    while (a) {
        while (!(a & 1)) {
            a >>= 1;
            if ((m & 7) == 3 || (m & 7) == 5) r = -r;
        }
        std::swap(a, m);
        if ((a & 3) == 3 && (m & 3) == 3) r = -r;
        a %= m;
    }
    return m == 1 ? r : 0;
}

int jacobi_small(uint64_t a, uint64_t k, unsigned n) {
    // (a / N) by reciprocity; N is odd for n >= 1
    if (a == 0) return 0;
    int r = 1;
    while (!(a & 1)) {
        a >>= 1;
        const uint64_t m8 = N_mod(k, n, 8);
        if (m8 == 3 || m8 == 5) r = -r;
    }
    if (a == 1) return r;
    if ((a & 3) == 3 && N_mod(k, n, 4) == 3) r = -r;
    return r * jacobi_odd(N_mod(k, n, a), a);
}

uint64_t choose_base(uint64_t k, unsigned n) {
    static const uint64_t pref[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    for (uint64_t b : pref)
        if (jacobi_small(b, k, n) == -1) return b;
    for (uint64_t b = 2; b < 100; ++b)
        if (jacobi_small(b, k, n) == -1) return b;
    return 0;
}

unsigned bitlen(uint64_t x) {
    unsigned b = 0;
    while (x) {
        ++b;
        x >>= 1;
    }
    return b;
}

}  // namespace pg

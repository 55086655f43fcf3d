/*
 * proth_oracle.c -- CPU oracle for the Proth modular-squaring path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, the smoke check and the
 * CPU-baseline leg of bench.py load this library; the product never does.
 * Each function names the ProthLogic 4.2 source it restates (file:line within
 * the reference project).  Portable C11: no intrinsics, no inline assembly, so
 * the same file builds and gives the same results on x86-64 and aarch64.
 */
#define _POSIX_C_SOURCE 200809L
#include "proth_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef unsigned __int128 u128;

struct ora_ctx {
    size_t L;
    int nst4;          /* number of radix-4 stages */
    int tail2;         /* 1 if a final radix-2 stage is needed (log2 L odd) */
    double* wr;        /* e^{-2 pi i j / L}, j < L (fft_engine.cpp:57-66, w1 LUT) */
    double* wi;
    double* stw;       /* per radix-4 stage: w1r w1i w2r w2i w3r w3i, m entries each */
    size_t stw_off[64];
    double *ar, *ai, *br, *bi, *abr, *abi, *tr, *ti; /* k_A, k_B, k_AB and ping-pong */
    uint64_t* sq;
    uint64_t* hq;      /* H then Q */
    size_t cap_limbs;
    double last_max_diff;
};

static void* xalloc(size_t bytes) {
    void* p = NULL;
    if (posix_memalign(&p, 64, bytes ? bytes : 64) != 0) return NULL;
    memset(p, 0, bytes ? bytes : 64);
    return p;
}

/* fft_init (fft_engine.cpp:18-73): twiddle LUT of length L; the per-stage
 * tables below are the same values regrouped for the Stockham passes. */
ora_ctx* ora_create(size_t L) {
    if (L < 16 || (L & (L - 1))) return NULL;
    ora_ctx* c = (ora_ctx*)calloc(1, sizeof(ora_ctx));
    if (!c) return NULL;
    c->L = L;
    int lg = 0;
    while (((size_t)1 << lg) < L) ++lg;
    c->nst4 = lg / 2;
    c->tail2 = lg & 1;
    c->wr = (double*)xalloc(L * sizeof(double));
    c->wi = (double*)xalloc(L * sizeof(double));
    for (size_t j = 0; j < L; ++j) {
        double ang = -2.0 * M_PI * (double)j / (double)L;
        c->wr[j] = cos(ang);
        c->wi[j] = sin(ang);
    }
    size_t total = 0, n = L;
    for (int t = 0; t < c->nst4; ++t) {
        c->stw_off[t] = total;
        total += 6 * (n / 4);
        n /= 4;
    }
    c->stw = (double*)xalloc((total + 6) * sizeof(double));
    n = L;
    for (int t = 0; t < c->nst4; ++t) {
        size_t m = n / 4, step = L / n;
        double* s = c->stw + c->stw_off[t];
        for (size_t p = 0; p < m; ++p) {
            s[0 * m + p] = c->wr[(p * step) % L];
            s[1 * m + p] = c->wi[(p * step) % L];
            s[2 * m + p] = c->wr[(2 * p * step) % L];
            s[3 * m + p] = c->wi[(2 * p * step) % L];
            s[4 * m + p] = c->wr[(3 * p * step) % L];
            s[5 * m + p] = c->wi[(3 * p * step) % L];
        }
        n /= 4;
    }
    double** bufs[] = {&c->ar, &c->ai, &c->br, &c->bi, &c->abr, &c->abi, &c->tr, &c->ti};
    for (int b = 0; b < 8; ++b) *bufs[b] = (double*)xalloc(L * sizeof(double));
    c->cap_limbs = 0;
    return c;
}

void ora_destroy(ora_ctx* c) {
    if (!c) return;
    free(c->wr); free(c->wi); free(c->stw);
    free(c->ar); free(c->ai); free(c->br); free(c->bi);
    free(c->abr); free(c->abi); free(c->tr); free(c->ti);
    free(c->sq); free(c->hq);
    free(c);
}

size_t ora_fft_len(const ora_ctx* c) { return c->L; }
double ora_last_max_err(const ora_ctx* c) { return c->last_max_diff; }

/* One Stockham radix-4 pass, x -> y, sub-length n, stride s; sg = +1 forward
 * (e^{-i}), -1 inverse (conjugate twiddles).  Plays the role of one radix
 * stage of fft_stockham_radix8 (fft_engine.cpp:234-494). */
static void stage4(const double* restrict xr, const double* restrict xi, double* restrict yr,
                   double* restrict yi, size_t n, size_t s, const double* tw, double sg) {
    const size_t m = n / 4;
    const double* w1r = tw; const double* w1i = tw + m;
    const double* w2r = tw + 2 * m; const double* w2i = tw + 3 * m;
    const double* w3r = tw + 4 * m; const double* w3i = tw + 5 * m;
    for (size_t p = 0; p < m; ++p) {
        const double c1 = w1r[p], s1 = sg * w1i[p];
        const double c2 = w2r[p], s2 = sg * w2i[p];
        const double c3 = w3r[p], s3 = sg * w3i[p];
        const double* ar_ = xr + s * p; const double* ai_ = xi + s * p;
        const double* br_ = xr + s * (p + m); const double* bi_ = xi + s * (p + m);
        const double* cr_ = xr + s * (p + 2 * m); const double* ci_ = xi + s * (p + 2 * m);
        const double* dr_ = xr + s * (p + 3 * m); const double* di_ = xi + s * (p + 3 * m);
        double* y0r = yr + s * (4 * p); double* y0i = yi + s * (4 * p);
        double* y1r = y0r + s; double* y1i = y0i + s;
        double* y2r = y1r + s; double* y2i = y1i + s;
        double* y3r = y2r + s; double* y3i = y2i + s;
        for (size_t q = 0; q < s; ++q) {
            double apcr = ar_[q] + cr_[q], apci = ai_[q] + ci_[q];
            double amcr = ar_[q] - cr_[q], amci = ai_[q] - ci_[q];
            double bpdr = br_[q] + dr_[q], bpdi = bi_[q] + di_[q];
            double bmdr = br_[q] - dr_[q], bmdi = bi_[q] - di_[q];
            /* forward: -i*(b-d) = (bmdi, -bmdr); inverse: +i*(b-d) */
            double jr = sg * bmdi, ji = -sg * bmdr;
            double t1r = amcr + jr, t1i = amci + ji;
            double t2r = apcr - bpdr, t2i = apci - bpdi;
            double t3r = amcr - jr, t3i = amci - ji;
            y0r[q] = apcr + bpdr; y0i[q] = apci + bpdi;
            y1r[q] = t1r * c1 - t1i * s1; y1i[q] = t1r * s1 + t1i * c1;
            y2r[q] = t2r * c2 - t2i * s2; y2i[q] = t2r * s2 + t2i * c2;
            y3r[q] = t3r * c3 - t3i * s3; y3i[q] = t3r * s3 + t3i * c3;
        }
    }
}

static void stage2_last(const double* restrict xr, const double* restrict xi, double* restrict yr,
                        double* restrict yi, size_t s) {
    for (size_t q = 0; q < s; ++q) {
        double ar_ = xr[q], ai_ = xi[q], br_ = xr[q + s], bi_ = xi[q + s];
        yr[q] = ar_ + br_; yi[q] = ai_ + bi_;
        yr[q + s] = ar_ - br_; yi[q + s] = ai_ - bi_;
    }
}

/* In-place complex DFT of length L (result back in re/im). */
static void fft_inplace(ora_ctx* c, double* re, double* im, int inverse) {
    const double sg = inverse ? -1.0 : 1.0;
    double *xr = re, *xi = im, *yr = c->tr, *yi = c->ti;
    size_t n = c->L, s = 1;
    for (int t = 0; t < c->nst4; ++t) {
        stage4(xr, xi, yr, yi, n, s, c->stw + c->stw_off[t], sg);
        double* tmp;
        tmp = xr; xr = yr; yr = tmp;
        tmp = xi; xi = yi; yi = tmp;
        n /= 4; s *= 4;
    }
    if (c->tail2) {
        stage2_last(xr, xi, yr, yi, s);
        double* tmp;
        tmp = xr; xr = yr; yr = tmp;
        tmp = xi; xi = yi; yi = tmp;
    }
    if (xr != re) {
        memcpy(re, xr, c->L * sizeof(double));
        memcpy(im, xi, c->L * sizeof(double));
    }
}

static void ensure_cap(ora_ctx* c, size_t n_limbs) {
    size_t need = 2 * n_limbs + 4;
    if (need <= c->cap_limbs) return;
    free(c->sq); free(c->hq);
    c->sq = (uint64_t*)xalloc(need * sizeof(uint64_t));
    c->hq = (uint64_t*)xalloc(2 * need * sizeof(uint64_t));
    c->cap_limbs = need;
}

/* fft_square_karatsuba (fft_engine.cpp:986-1073) with pack_karatsuba_limbs
 * (llr_fft_pack.cpp:12-41) and unpack_karatsuba_overlap_add (fft_engine.cpp:825-984). */
void ora_engine_square(ora_ctx* c, uint64_t* v, size_t n_limbs, unsigned n_bits, uint64_t k) {
    const size_t L = c->L, half = L / 2;
    ensure_cap(c, n_limbs);
    /* pack: 16-bit words; A = words [0, L/2), B = words [L/2, L); upper halves 0 */
    const size_t total_words = n_limbs * 4;
    memset(c->ar, 0, L * sizeof(double)); memset(c->ai, 0, L * sizeof(double));
    memset(c->br, 0, L * sizeof(double)); memset(c->bi, 0, L * sizeof(double));
    for (size_t j = 0; j < half; ++j) {
        if (j < total_words) c->ar[j] = (double)(uint16_t)(v[j >> 2] >> (16 * (j & 3)));
        size_t jb = j + half;
        if (jb < total_words) c->br[j] = (double)(uint16_t)(v[jb >> 2] >> (16 * (jb & 3)));
    }
    fft_inplace(c, c->ar, c->ai, 0);
    fft_inplace(c, c->br, c->bi, 0);
    /* pointwise: A^2/L, B^2/L, 2AB/L (fft_engine.cpp:1023-1055) */
    const double inv_n = 1.0 / (double)L;
    for (size_t i = 0; i < L; ++i) {
        double a_r = c->ar[i], a_i = c->ai[i], b_r = c->br[i], b_i = c->bi[i];
        c->ar[i] = (a_r * a_r - a_i * a_i) * inv_n;
        c->ai[i] = (2.0 * (a_r * a_i)) * inv_n;
        c->br[i] = (b_r * b_r - b_i * b_i) * inv_n;
        c->bi[i] = (2.0 * (b_r * b_i)) * inv_n;
        c->abr[i] = ((a_r * b_r - a_i * b_i) * 2.0) * inv_n;
        c->abi[i] = ((a_r * b_i + a_i * b_r) * 2.0) * inv_n;
    }
    fft_inplace(c, c->ar, c->ai, 1);
    fft_inplace(c, c->br, c->bi, 1);
    fft_inplace(c, c->abr, c->abi, 1);

    /* unpack (1)-(3): overlap-add, round to nearest even, max |err|, 16-bit carry */
    const size_t max_chunks = n_limbs * 8;
    const size_t dbl_limbs = n_limbs * 2 + 2;
    uint64_t* sq = c->sq;
    memset(sq, 0, dbl_limbs * sizeof(uint64_t));
    int64_t carry = 0;
    double max_err = 0.0;
    for (size_t i = 0; i < max_chunks; ++i) {
        double s = 0.0;
        double a2 = (i < L) ? c->ar[i] : 0.0;
        double ab = (i >= half && (i - half) < L) ? c->abr[i - half] : 0.0;
        double b2 = (i >= L && (i - L) < L) ? c->br[i - L] : 0.0;
        s = (a2 + ab) + b2;
        double r = nearbyint(s);
        double e = fabs(s - r);
        if (e > max_err) max_err = e;
        int64_t ival = (int64_t)r + carry;
        carry = ival >> 16;
        uint64_t chunk = (uint64_t)(ival & 0xFFFF);
        size_t limb = i >> 2;
        if (limb < dbl_limbs) sq[limb] |= chunk << (16 * (i & 3));
    }
    c->last_max_diff = max_err;
    size_t cidx = max_chunks >> 2;
    while (carry > 0 && cidx < dbl_limbs) {
        u128 sum = (u128)sq[cidx] + (uint64_t)carry;
        sq[cidx] = (uint64_t)sum;
        carry = (int64_t)(uint64_t)(sum >> 64);
        cidx++;
    }
    /* (4) H = sq >> n, Q = H div k, rem = H mod k (the divq chain at :909-923) */
    const size_t split_q = n_bits / 64;
    const unsigned split_r = n_bits % 64;
    uint64_t* H = c->hq;
    uint64_t* Q = c->hq + n_limbs + 2;
    for (size_t i = 0; i < n_limbs; ++i) {
        size_t src = split_q + i;
        uint64_t h = 0;
        if (src < dbl_limbs) {
            h = sq[src] >> split_r;
            if (split_r > 0 && src + 1 < dbl_limbs) h |= sq[src + 1] << (64 - split_r);
        }
        H[i] = h;
    }
    uint64_t rem = 0;
    if (k < (1ULL << 32)) {
        /* two 64-bit divisions per limb: rem < k < 2^32 keeps each dividend below 2^64 */
        for (size_t i = n_limbs; i-- > 0;) {
            uint64_t hi = (rem << 32) | (H[i] >> 32);
            uint64_t q1 = hi / k, r1 = hi % k;
            uint64_t lo = (r1 << 32) | (H[i] & 0xFFFFFFFFULL);
            uint64_t q0 = lo / k;
            rem = lo % k;
            Q[i] = (q1 << 32) | q0;
        }
    } else {
        for (size_t i = n_limbs; i-- > 0;) {
            u128 cur = ((u128)rem << 64) | H[i];
            Q[i] = (uint64_t)(cur / k);
            rem = (uint64_t)(cur % k);
        }
    }
    /* (5) out = (sq mod 2^n) + rem*2^n - Q, plus N on borrow (:940-983) */
    memset(v, 0, n_limbs * sizeof(uint64_t));
    for (size_t i = 0; i < split_q && i < n_limbs; ++i) v[i] = sq[i];
    if (split_r > 0 && split_q < n_limbs) v[split_q] = sq[split_q] & ((1ULL << split_r) - 1);
    if (rem > 0 && split_q < n_limbs) {
        uint64_t rl = split_r == 0 ? rem : (rem << split_r);
        uint64_t rh = split_r == 0 ? 0 : (rem >> (64 - split_r));
        u128 sum = (u128)v[split_q] + rl;
        v[split_q] = (uint64_t)sum;
        uint64_t ca = (uint64_t)(sum >> 64);
        if (split_q + 1 < n_limbs) {
            sum = (u128)v[split_q + 1] + rh + ca;
            v[split_q + 1] = (uint64_t)sum;
            ca = (uint64_t)(sum >> 64);
            for (size_t idx = split_q + 2; ca && idx < n_limbs; ++idx) {
                sum = (u128)v[idx] + ca;
                v[idx] = (uint64_t)sum;
                ca = (uint64_t)(sum >> 64);
            }
        }
    }
    unsigned borrow = 0;
    for (size_t i = 0; i < n_limbs; ++i) {
        uint64_t a = v[i], b = Q[i];
        uint64_t d = a - b - borrow;
        borrow = (a < b) || (a - b < borrow);
        v[i] = d;
    }
    if (borrow) {
        uint64_t lc = 1;
        for (size_t i = 0; i < n_limbs; ++i) {
            uint64_t add = lc;
            lc = 0;
            u128 extra = 0;
            if (i == split_q) extra += split_r == 0 ? k : (k << split_r);
            if (i == split_q + 1 && split_r > 0) extra += (k >> (64 - split_r));
            u128 sum = (u128)v[i] + add + extra;
            v[i] = (uint64_t)sum;
            lc += (uint64_t)(sum >> 64);
        }
    }
}

/* ---- multi-limb helpers for the exact reduction (proth_logic.cpp:52-249) ---- */

static size_t bn_len(const uint64_t* a, size_t n) {
    while (n > 0 && a[n - 1] == 0) --n;
    return n;
}

/* a (n limbs) -> returns remainder, a <- a div d (div_big_by_u64, proth_logic.cpp:212-221) */
static uint64_t bn_divmod_small(uint64_t* a, size_t n, uint64_t d) {
    u128 rem = 0;
    for (size_t i = n; i-- > 0;) {
        u128 cur = (rem << 64) | a[i];
        a[i] = (uint64_t)(cur / d);
        rem = cur % d;
    }
    return (uint64_t)rem;
}

/* v (nl limbs) += N = k*2^n + 1 modulo 2^(64 nl) (add_proth_modulus_once, :118-157) */
static void bn_add_N(uint64_t* v, size_t nl, unsigned n, uint64_t k) {
    u128 carry = 1;
    size_t ql = n / 64; unsigned rs = n % 64;
    for (size_t i = 0; i < nl; ++i) {
        u128 add = carry;
        if (i == ql) add += (u128)(rs == 0 ? k : (k << rs));
        if (rs > 0 && i == ql + 1) add += (u128)(k >> (64 - rs));
        u128 s = (u128)v[i] + add;
        v[i] = (uint64_t)s;
        carry = s >> 64;
    }
}

/* compare v with N: -1, 0, 1 (cmp_proth_modulus, :89-113) */
static int bn_cmp_N(const uint64_t* v, size_t nl, unsigned n, uint64_t k) {
    size_t ql = n / 64; unsigned rs = n % 64;
    uint64_t nlo = rs == 0 ? k : (k << rs);
    uint64_t nhi = rs == 0 ? 0 : (k >> (64 - rs));
    /* N's limbs beyond v's length: v is smaller if any of them is non-zero */
    if ((ql >= nl && nlo) || (ql + 1 >= nl && nhi)) return -1;
    for (size_t i = nl; i-- > 0;) {
        uint64_t nv = 0;
        if (i == ql) nv = nlo;
        else if (i == ql + 1) nv = nhi;
        if (i == 0) nv |= 1; /* bit 0 of k << (n mod 64) is clear whenever n >= 1 */
        if (v[i] != nv) return v[i] > nv ? 1 : -1;
    }
    return 0;
}

/* v <- v - N (no borrow expected) (sub_proth_modulus_once, :159-182) */
static void bn_sub_N(uint64_t* v, size_t nl, unsigned n, uint64_t k) {
    size_t ql = n / 64; unsigned rs = n % 64;
    unsigned borrow = 0;
    for (size_t i = 0; i < nl; ++i) {
        u128 sub = (i == 0) ? 1 : 0;
        if (i == ql) sub += (u128)(rs == 0 ? k : (k << rs));
        if (rs > 0 && i == ql + 1) sub += (u128)(k >> (64 - rs));
        uint64_t s = (uint64_t)sub;
        uint64_t a = v[i];
        uint64_t d = a - s - borrow;
        borrow = (a < s) || (a - s < borrow);
        v[i] = d;
    }
}

/* Exact v mod N by splitting at bit n and dividing the high part by k, as
 * proth_reduce_stage1_rec (proth_logic.cpp:250-334) does; the quotient is
 * reduced recursively before it is subtracted. */
int ora_reduce(uint64_t* v, size_t nl, unsigned n, uint64_t k) {
    const size_t ql = n / 64; const unsigned rs = n % 64;
    uint64_t* hi = (uint64_t*)calloc(nl + 2, sizeof(uint64_t));
    if (!hi) return -1;
    for (int round = 0; round < 200; ++round) {
        /* high = v >> n */
        memset(hi, 0, (nl + 2) * sizeof(uint64_t));
        for (size_t i = ql; i < nl; ++i) {
            uint64_t h = v[i] >> rs;
            if (rs > 0 && i + 1 < nl) h |= v[i + 1] << (64 - rs);
            hi[i - ql] = h;
        }
        size_t hn = bn_len(hi, nl);
        int done = 0;
        if (hn == 0) done = 1;
        else if (hn == 1 && hi[0] < k) done = 1;
        else if (hn == 1 && hi[0] == k) done = 1; /* value in [k 2^n, (k+1) 2^n): fix below */
        if (done) {
            while (bn_cmp_N(v, nl, n, k) >= 0) bn_sub_N(v, nl, n, k);
            free(hi);
            return 0;
        }
        /* lo = v mod 2^n */
        if (ql < nl) {
            if (rs == 0) { for (size_t i = ql; i < nl; ++i) v[i] = 0; }
            else { v[ql] &= (1ULL << rs) - 1; for (size_t i = ql + 1; i < nl; ++i) v[i] = 0; }
        }
        uint64_t r = bn_divmod_small(hi, hn, k);
        /* q = hi (quotient), reduce it recursively */
        if (ora_reduce(hi, nl, n, k) != 0) { free(hi); return -1; }
        /* v = lo + r*2^n */
        if (r) {
            u128 acc = (u128)v[ql] + ((u128)r << rs);
            v[ql] = (uint64_t)acc;
            uint64_t ca = (uint64_t)(acc >> 64);
            for (size_t i = ql + 1; ca && i < nl; ++i) {
                u128 s = (u128)v[i] + ca;
                v[i] = (uint64_t)s;
                ca = (uint64_t)(s >> 64);
            }
        }
        /* v -= q; on borrow add N (sub_big_inplace + borrow fix, :223-249, :312-321) */
        unsigned borrow = 0;
        for (size_t i = 0; i < nl; ++i) {
            uint64_t a = v[i], b = hi[i];
            uint64_t d = a - b - borrow;
            borrow = (a < b) || (a - b < borrow);
            v[i] = d;
        }
        if (borrow) bn_add_N(v, nl, n, k);
    }
    free(hi);
    return -1;
}

static size_t highest_nonzero_limb(const uint64_t* v, size_t nl) {
    for (size_t i = nl; i-- > 0;)
        if (v[i]) return i;
    return 0;
}

/* The loop body of execute_proth_test_fft (proth_logic.cpp:485-533). */
double ora_square_mod(ora_ctx* c, uint64_t* v, unsigned n, uint64_t k) {
    const size_t nl = c->L / 4;
    ora_engine_square(c, v, nl, n, k);
    size_t max_sq_limbs = (2 * (size_t)n) / 64 + 4;
    if (max_sq_limbs < nl) {
        memset(v + max_sq_limbs, 0, (nl - max_sq_limbs) * sizeof(uint64_t));
        for (size_t j = max_sq_limbs; j-- > (2 * (size_t)n) / 64 + 1;)
            if (v[j] == ~0ULL) v[j] = 0;
    }
    if (highest_nonzero_limb(v, nl) >= (size_t)(n >> 6)) ora_reduce(v, nl, n, k);
    return c->last_max_diff;
}

void ora_mul_small_mod(uint64_t* v, size_t nl, unsigned n, uint64_t k, uint64_t s) {
    uint64_t* t = (uint64_t*)calloc(nl + 2, sizeof(uint64_t));
    u128 carry = 0;
    for (size_t i = 0; i < nl; ++i) {
        u128 p = (u128)v[i] * s + carry;
        t[i] = (uint64_t)p;
        carry = p >> 64;
    }
    t[nl] = (uint64_t)carry;
    ora_reduce(t, nl + 2, n, k);
    memcpy(v, t, nl * sizeof(uint64_t));
    free(t);
}

/* ---- small-integer helpers: gate, Jacobi, base ---- */

static uint64_t mulmod64(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)(((u128)a * b) % m); }
static uint64_t powmod64(uint64_t a, uint64_t e, uint64_t m) {
    uint64_t r = 1 % m;
    a %= m;
    while (e) {
        if (e & 1) r = mulmod64(r, a, m);
        a = mulmod64(a, a, m);
        e >>= 1;
    }
    return r;
}

/* is_divisible_by_gate (proth_logic.cpp:41-50) */
int ora_gate_divisible(uint64_t k, unsigned n, uint64_t p) {
    if (p % 2 == 0) return 0;
    uint64_t km = k % p;
    if (km == 0) return 0;
    uint64_t invk = powmod64(km, p - 2, p);
    uint64_t target = mulmod64(p - 1, invk, p);
    return powmod64(2, n, p) == target;
}

int ora_gate_rejects(uint64_t k, unsigned n) {
    static const uint64_t gp[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67};
    for (size_t i = 0; i < sizeof(gp) / sizeof(gp[0]); ++i)
        if (ora_gate_divisible(k, n, gp[i])) return 1;
    return 0;
}

static uint64_t N_mod(uint64_t k, unsigned n, uint64_t m) {
    return (mulmod64(k % m, powmod64(2, n, m), m) + 1) % m;
}

static int jacobi_u64(uint64_t a, uint64_t m) { /* m odd > 0 */
    int r = 1;
    a %= m;
    while (a) {
        while ((a & 1) == 0) {
            a >>= 1;
            uint64_t m8 = m & 7;
            if (m8 == 3 || m8 == 5) r = -r;
        }
        uint64_t t = a; a = m; m = t;
        if ((a & 3) == 3 && (m & 3) == 3) r = -r;
        a %= m;
    }
    return m == 1 ? r : 0;
}

/* mpz_jacobi(a, N) for small a, by quadratic reciprocity. */
int ora_jacobi_small(uint64_t a, uint64_t k, unsigned n) {
    if (a == 0) return 0;
    int r = 1;
    while ((a & 1) == 0) {
        a >>= 1;
        uint64_t m8 = N_mod(k, n, 8);
        if (m8 == 3 || m8 == 5) r = -r;
    }
    if (a == 1) return r;
    if ((a & 3) == 3 && N_mod(k, n, 4) == 3) r = -r;
    return r * jacobi_u64(N_mod(k, n, a), a);
}

/* base choice (proth_logic.cpp:411-422) */
uint64_t ora_choose_base(uint64_t k, unsigned n) {
    static const uint64_t pref[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    for (size_t i = 0; i < sizeof(pref) / sizeof(pref[0]); ++i)
        if (ora_jacobi_small(pref[i], k, n) == -1) return pref[i];
    for (uint64_t b = 2; b < 100; ++b)
        if (ora_jacobi_small(b, k, n) == -1) return b;
    return 0;
}

static unsigned bitlen64(uint64_t x) {
    unsigned b = 0;
    while (x) { ++b; x >>= 1; }
    return b;
}

size_t ora_choose_L(unsigned n, uint64_t k) {
    size_t L = 256;
    while ((double)n / (double)L > 18.0) L *= 2; /* autotune start (dcore.cpp:24-27) */
    while ((size_t)n + bitlen64(k) + 64 > 16 * L) L *= 2;
    return L;
}

/* auto_tune_fft_len (dcore.cpp:20-81) */
size_t ora_autotune_L(unsigned n, uint64_t k) {
    size_t L = 256;
    while ((double)n / (double)L > 18.0) L *= 2;
    for (;;) {
        double bpw = (double)n / (double)L;
        if (bpw < 11.0) return L;
        ora_ctx* c = ora_create(L);
        if (!c) { L *= 2; continue; }
        size_t nl = ((size_t)n + 63) / 64;
        size_t alloc = L > (2 * (size_t)n) / 64 + 64 ? L : (2 * (size_t)n) / 64 + 64;
        uint64_t* t = (uint64_t*)calloc(alloc, sizeof(uint64_t));
        for (size_t i = 0; i < nl; ++i) t[i] = ~0ULL;
        t[0] = k | 1;
        for (int s = 0; s < 100; ++s) ora_engine_square(c, t, nl, n, k);
        double err = c->last_max_diff;
        free(t);
        ora_destroy(c);
        if (err >= 0.0 && err <= 0.30) return L;
        L *= 2;
    }
}

void ora_powm_small(ora_ctx* c, uint64_t* x, uint64_t a, uint64_t e, unsigned n, uint64_t k) {
    const size_t nl = c->L / 4;
    memset(x, 0, nl * sizeof(uint64_t));
    if (e == 0) { x[0] = 1; return; }
    x[0] = a;
    ora_reduce(x, nl, n, k);
    int top = 63;
    while (!((e >> top) & 1)) --top;
    for (int b = top - 1; b >= 0; --b) {
        ora_square_mod(c, x, n, k);
        if ((e >> b) & 1) ora_mul_small_mod(x, nl, n, k, a);
    }
}

static int is_N_minus_1(const uint64_t* x, size_t nl, unsigned n, uint64_t k) {
    /* N - 1 = k * 2^n (is_nm1_limbs, proth_logic.cpp:336-355) */
    size_t ql = n / 64; unsigned rs = n % 64;
    for (size_t i = 0; i < nl; ++i) {
        uint64_t t = 0;
        if (i == ql) t = rs == 0 ? k : (k << rs);
        if (rs > 0 && i == ql + 1) t = k >> (64 - rs);
        if (x[i] != t) return 0;
    }
    return 1;
}

double ora_run_squarings(ora_ctx* c, uint64_t* x, unsigned n, uint64_t k, uint64_t iters) {
    double mx = 0.0;
    for (uint64_t i = 0; i < iters; ++i) {
        double e = ora_square_mod(c, x, n, k);
        if (e > mx) mx = e;
    }
    return mx;
}

static int proth_test_ctx(ora_ctx* c, uint64_t k, unsigned n, uint64_t limit, uint64_t* a_out,
                          uint64_t* res64_out, double* max_err_out, uint64_t* trace, size_t trace_len) {
    if (a_out) *a_out = 0;
    if (res64_out) *res64_out = 0;
    if (max_err_out) *max_err_out = 0.0;
    if (ora_gate_rejects(k, n)) return 0;
    uint64_t a = ora_choose_base(k, n);
    if (a_out) *a_out = a;
    const size_t nl = c->L / 4;
    uint64_t* x = (uint64_t*)calloc(nl, sizeof(uint64_t));
    if (!x) return -1;
    if (a) ora_powm_small(c, x, a, k, n, k);
    double mx = 0.0;
    uint64_t iters = (uint64_t)n - 1;
    if (limit && limit < iters) iters = limit;
    for (uint64_t i = 0; i < iters; ++i) {
        double e = ora_square_mod(c, x, n, k);
        if (e > mx) mx = e;
        if (trace && i < trace_len) trace[i] = x[0];
    }
    int prime = is_N_minus_1(x, nl, n, k);
    if (res64_out) *res64_out = x[0];
    if (max_err_out) *max_err_out = mx;
    free(x);
    return prime;
}

int ora_proth_test(uint64_t k, unsigned n, size_t L, uint64_t* a_out, uint64_t* res64_out,
                   double* max_err_out, uint64_t* trace, size_t trace_len) {
    if (L == 0) L = ora_choose_L(n, k);
    ora_ctx* c = ora_create(L);
    if (!c) return -1;
    int r = proth_test_ctx(c, k, n, 0, a_out, res64_out, max_err_out, trace, trace_len);
    ora_destroy(c);
    return r;
}

/* Trial division: p | k 2^n + 1  <=>  k 2^n = -1 (mod p), by a plain sieve of
 * the odd numbers below bound (test sizes: bound up to a few times 10^7). */
uint64_t ora_smallest_factor(uint64_t k, unsigned n, uint64_t bound) {
    if (bound < 3) return 0;
    unsigned char* comp = (unsigned char*)calloc(bound, 1);
    if (!comp) return 0;
    uint64_t found = 0;
    for (uint64_t p = 3; p < bound && !found; p += 2) {
        if (comp[p]) continue;
        for (uint64_t j = p * p; j < bound; j += 2 * p) comp[j] = 1;
        if (mulmod64(k % p, powmod64(2, n, p), p) == p - 1) found = p;
    }
    free(comp);
    return found;
}

/* ---- CPU baseline: one pinned-style worker per thread, like dcore.cpp:84-193 ---- */

typedef struct {
    const uint64_t* ks; const unsigned* ns; size_t count; uint64_t limit;
    uint64_t* res; size_t next; pthread_mutex_t mu;
} bench_job;

static void* bench_worker(void* arg) {
    bench_job* j = (bench_job*)arg;
    ora_ctx* c = NULL;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        size_t i = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (i >= j->count) break;
        size_t L = ora_choose_L(j->ns[i], j->ks[i]);
        if (!c || ora_fft_len(c) != L) { ora_destroy(c); c = ora_create(L); }
        uint64_t r = 0;
        proth_test_ctx(c, j->ks[i], j->ns[i], j->limit, NULL, &r, NULL, NULL, 0);
        if (j->res) j->res[i] = r;
    }
    ora_destroy(c);
    return NULL;
}

double ora_bench_tests(const uint64_t* ks, const unsigned* ns, size_t count, int threads,
                       uint64_t squarings_per_test, uint64_t* res64_out) {
    if (threads < 1) threads = 1;
    bench_job j;
    j.ks = ks; j.ns = ns; j.count = count; j.limit = squarings_per_test; j.res = res64_out; j.next = 0;
    pthread_mutex_init(&j.mu, NULL);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    pthread_t* th = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    for (int t = 0; t < threads; ++t) pthread_create(&th[t], NULL, bench_worker, &j);
    for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    free(th);
    pthread_mutex_destroy(&j.mu);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

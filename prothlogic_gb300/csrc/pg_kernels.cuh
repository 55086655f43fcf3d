// pg_kernels.cuh -- sm_103a kernels of one modular squaring y <- s * y^2 * 2^-n mod N.
//
// One squaring of a residue with M digits is a length-M complex FFT pair in
// "right-angle" form: digit j enters as d_j * a_j * theta^j (a_j: IBDWT weight
// 2^{S_j - jn/M}, theta = e^{i pi / 2M}), so the cyclic length-M transform
// computes the negacyclic length-2M product of the real digit sequence.  The
// digit sequence occupies only the low half, so nothing wraps: after the
// inverse transform element j holds c_j + i c_{M+j}, the low and high halves
// of the zero-padded product X^2.  The Montgomery fold (2^-n = -k mod N) then
// needs only element j:  u_j = s (c_{M+j} + 2 top d_j - k c_j).
//
// The transform runs as P passes over a global buffer (radix F[0] x ... x
// F[P-1] = M, decimation in frequency forward, in time inverse, no bit
// reversal: the pointwise square does not care about order).  Kernels:
//   k_first   pass 0 forward, fused with the carry fix-up of the previous
//             squaring, the top-digit reduction, and the forward weight
//   k_mid_*   pass 1 forward / inverse (P == 3 only)
//   k_inner   last pass forward, pointwise square, last pass inverse
//   k_last    pass 0 inverse, fused with unweight, rounding + max |err|,
//             the Montgomery fold and the in-run carry
//   k_block   one residue, P == 3: the three middle kernels in one, a
//             thread-block cluster per block of the spectrum
// All arithmetic on the transform is FP64; rounding, fold and carries are
// exact integer (int64 / int128) work.  Slots (candidates) run side by side:
// blockIdx.y is the slot.
#ifndef PG_KERNELS_CUH
#define PG_KERNELS_CUH

#include "pg_internal.h"

namespace pg {

typedef __int128 i128;

__device__ __forceinline__ double2 cmul(double2 a, double2 w) {
    return make_double2(fma(a.x, w.x, -(a.y * w.y)), fma(a.x, w.y, a.y * w.x));
}
// a * conj(w)
__device__ __forceinline__ double2 cmulc(double2 a, double2 w) {
    return make_double2(fma(a.x, w.x, a.y * w.y), fma(a.y, w.x, -(a.x * w.y)));
}

// Radix-4 decimation-in-frequency butterfly, outputs in place (0,1,2,3).
__device__ __forceinline__ void bfly4_fwd(double2& a0, double2& a1, double2& a2, double2& a3) {
    const double apcx = a0.x + a2.x, apcy = a0.y + a2.y;
    const double amcx = a0.x - a2.x, amcy = a0.y - a2.y;
    const double bpdx = a1.x + a3.x, bpdy = a1.y + a3.y;
    const double bmdx = a1.x - a3.x, bmdy = a1.y - a3.y;
    a0 = make_double2(apcx + bpdx, apcy + bpdy);
    a2 = make_double2(apcx - bpdx, apcy - bpdy);
    a1 = make_double2(amcx + bmdy, amcy - bmdx);  // (a0-a2) - i (a1-a3)
    a3 = make_double2(amcx - bmdy, amcy + bmdx);  // (a0-a2) + i (a1-a3)
}
// Inverse radix-4 butterfly (conjugate DFT, unscaled).
__device__ __forceinline__ void bfly4_inv(double2& z0, double2& z1, double2& z2, double2& z3) {
    const double sx = z0.x + z2.x, sy = z0.y + z2.y;
    const double dx = z0.x - z2.x, dy = z0.y - z2.y;
    const double tx = z1.x + z3.x, ty = z1.y + z3.y;
    const double ux = z1.x - z3.x, uy = z1.y - z3.y;
    z0 = make_double2(sx + tx, sy + ty);
    z2 = make_double2(sx - tx, sy - ty);
    z1 = make_double2(dx - uy, dy + ux);  // (z0-z2) + i (z1-z3)
    z3 = make_double2(dx + uy, dy - ux);  // (z0-z2) - i (z1-z3)
}

template <int F>
struct Lg { static constexpr int v = (F <= 1) ? 0 : 1 + Lg<F / 2>::v; };
template <>
struct Lg<1> { static constexpr int v = 0; };

// Synchronisation policies: a whole CTA, or one warp working on its own tile.
struct BlockSync {
    __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct WarpSync {
    __device__ __forceinline__ void operator()() const { __syncwarp(); }
};

// Called by a tile after it has loaded its constant operands (twiddles,
// weights) and before it touches anything the previous kernel wrote.
// It returns false when the tile has nothing to do (CTA-uniform).
struct NoWait {
    __device__ __forceinline__ bool operator()() const { return true; }
};
// Programmatic dependent launch: wait until the previous kernel in the stream
// has completed (its writes visible).  pdl_trigger() at the end of a CTA's
// work lets the next kernel's CTAs start their prologue during this kernel's
// tail; triggering earlier would let a whole graph of kernels pile up on the SMs.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
// ... then go on only if the slot is active in this step (and, for the
// inverse passes, computes a product of its own).
struct PdlActive {
    const SlotState* st;
    bool need_product;
    __device__ __forceinline__ bool operator()() const {
        pdl_wait();
        return st->active && !(need_product && st->op == OP_FORWARD);
    }
};
// A single residue whose step count the host controls exactly: only wait.
struct PdlOnly {
    __device__ __forceinline__ bool operator()() const {
        pdl_wait();
        return true;
    }
};
// The first pass decides the step's activity from the counters and publishes it.
struct PdlFirst {
    SlotState* st;
    bool publish;
    __device__ __forceinline__ bool operator()() const {
        pdl_wait();
        const bool act = st->step < st->total;
        if (publish) st->active = act ? 1 : 0;
        return act;
    }
};

// Element (group g, index i) of a shared-memory tile.  ST: the row stride in
// elements (0: dense, F for group-major tiles, G otherwise); a padded stride
// keeps the strided accesses of a column transform off a single bank.
template <int F, int G, bool GROUP_MAJOR, int ST = 0>
__device__ __forceinline__ int tix(int g, int i) {
    constexpr int S = ST ? ST : (GROUP_MAJOR ? F : G);
    return GROUP_MAJOR ? g * S + i : i * S + g;
}

// -x by flipping the sign bit with an integer XOR (inline PTX, so the compiler
// cannot turn it back into an FP64 negation that takes an FP64 add to materialise).
__device__ __forceinline__ double neg_bits(double x) {
    int hi = __double2hiint(x);
    asm("xor.b32 %0, %0, 0x80000000;" : "+r"(hi));
    return __hiloint2double(hi, __double2loint(x));
}

__device__ __forceinline__ double2 shfl_xor_d2(double2 v, int m) {
    return make_double2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

// Radix-4 stage s of the forward transform done by a PAIR of adjacent lanes:
// lane `sub` of the pair holds inputs sub and sub+2 of the butterfly, forms
// their sum and difference, swaps one of them with its partner (shuffle), and
// produces outputs sub and sub+2 with their twiddles.  Output 0 takes no
// twiddle, so the three products are shared out evenly: each lane multiplies
// its output sub+2, and output 1 (lane 1's) is multiplied half on each lane,
// lane 0 forming the real part and lane 1 the imaginary part (one shuffle of
// the operand to lane 0, one of the real part back).  The operations are those
// of bfly4_fwd + cmul, so the results are bit-identical to the one-thread
// butterfly; each lane's FP64 chain is 14 instructions instead of 28.
template <int F, int G, bool GM, int ST = 0>
__device__ __forceinline__ void pair_stage_fwd(double2* tile, const double2* __restrict__ wF, int tid, int s) {
    const int sub = tid & 1;
    const int b = tid >> 1;
    const int g = b / (F / 4), w = b % (F / 4);
    const int h = F >> (2 * (s + 1));
    const int step = F / (4 * h);
    const int blk = w / h, j = w % h;
    const int i0 = blk * 4 * h + j;
    const int ia = tix<F, G, GM, ST>(g, i0 + sub * h), ib = tix<F, G, GM, ST>(g, i0 + (sub + 2) * h);
    const double2 xa = tile[ia], xb = tile[ib];
    const double2 p = make_double2(xa.x + xb.x, xa.y + xb.y);
    const double2 m = make_double2(xa.x - xb.x, xa.y - xb.y);
    const double2 snd = sub ? p : m;
    const double2 rcv = make_double2(__shfl_xor_sync(0xffffffffu, snd.x, 1), __shfl_xor_sync(0xffffffffu, snd.y, 1));
    const double2 u = sub ? rcv : p;                          // t0 | t1
    const double2 v = sub ? make_double2(m.y, -m.x) : rcv;    // t2 | -i t3
    double2 oa = make_double2(u.x + v.x, u.y + v.y);          // y0 | y1
    double2 ob = make_double2(u.x - v.x, u.y - v.y);          // y2 | y3
    if (h > 1) {
        const int e = j * step;
        const double2 w1 = wF[e];
        const double2 nb = shfl_xor_d2(oa, 1);                 // every lane shuffles (full mask)
        const double2 y1 = sub ? oa : nb;                      // output 1 on both lanes
        // the two halves of cmul(y1, w1) as one instruction pair with per-lane operands:
        // lane 0 fma(y1.x, w1.x, y1.y (-w1.y)) = Re, lane 1 fma(y1.x, w1.y, y1.y w1.x) = Im
        // (a (-b) == -(a b) exactly, so both equal cmul's halves bit for bit)
        const double part = fma(y1.x, sub ? w1.y : w1.x, y1.y * (sub ? w1.x : neg_bits(w1.y)));
        const double re = __shfl_xor_sync(0xffffffffu, part, 1);
        if (sub) oa = make_double2(re, part);
        ob = cmul(ob, wF[(2 + sub) * e]);
    }
    tile[ia] = oa;
    tile[ib] = ob;
}

// Inverse counterpart (twiddles on the inputs, then bfly4_inv), bit-identical
// to the one-thread butterfly: input 0 takes no twiddle, input 1 (lane 1's) is
// multiplied half on each lane as in the forward stage.
template <int F, int G, bool GM, int ST = 0>
__device__ __forceinline__ void pair_stage_inv(double2* tile, const double2* __restrict__ wF, int tid, int s) {
    const int sub = tid & 1;
    const int b = tid >> 1;
    const int g = b / (F / 4), w = b % (F / 4);
    const int h = F >> (2 * (s + 1));
    const int step = F / (4 * h);
    const int blk = w / h, j = w % h;
    const int i0 = blk * 4 * h + j;
    const int ia = tix<F, G, GM, ST>(g, i0 + sub * h), ib = tix<F, G, GM, ST>(g, i0 + (sub + 2) * h);
    double2 za = tile[ia], zb = tile[ib];
    if (h > 1) {
        const int e = j * step;
        const double2 w1 = wF[e];
        const double2 nb = shfl_xor_d2(za, 1);                 // every lane shuffles (full mask)
        const double2 z1 = sub ? za : nb;                      // input 1 on both lanes
        // the two halves of cmulc(z1, w1) as one instruction pair with per-lane operands:
        // lane 0 fma(z1.x, w1.x, z1.y w1.y) = Re, lane 1 fma(z1.y, w1.x, (-z1.x) w1.y) = Im
        const double part = fma(sub ? z1.y : z1.x, w1.x, (sub ? neg_bits(z1.x) : z1.y) * w1.y);
        const double re = __shfl_xor_sync(0xffffffffu, part, 1);
        if (sub) za = make_double2(re, part);
        zb = cmulc(zb, wF[(2 + sub) * e]);
    }
    const double2 p = make_double2(za.x + zb.x, za.y + zb.y);
    const double2 m = make_double2(za.x - zb.x, za.y - zb.y);
    const double2 snd = sub ? p : m;
    const double2 rcv = make_double2(__shfl_xor_sync(0xffffffffu, snd.x, 1), __shfl_xor_sync(0xffffffffu, snd.y, 1));
    const double2 u = sub ? rcv : p;                          // s | d
    const double2 v = sub ? make_double2(-m.y, m.x) : rcv;    // t | i u
    tile[ia] = make_double2(u.x + v.x, u.y + v.y);            // Z0 | Z1
    tile[ib] = make_double2(u.x - v.x, u.y - v.y);            // Z2 | Z3
}

// p + q or p - q, the sign chosen per lane without a branch (p - q == p + (-q) exactly).
__device__ __forceinline__ double add_sgn(double p, double q, bool minus) { return p + (minus ? -q : q); }

// Radix-4 stage s of the forward transform done by FOUR lanes, one input and
// one output each: lanes (0,2) form a0 +- a2 and lanes (1,3) a1 +- a3 (shuffle
// over lane distance 2), then lanes (0,1) form y0, y2 and lanes (2,3) y1, y3
// (distance 1), and each lane multiplies its output by its twiddle.  Every
// output is the same sum of the same two rounded operands as in bfly4_fwd + cmul
// (operand selects, no divergent branch), so results are bit-identical; a lane's
// FP64 chain is 8 instructions per stage, at the price of w^0 = 1 on lane 0.
template <int F, int G, bool GM, int ST = 0>
__device__ __forceinline__ void quad_stage_fwd(double2* tile, const double2* __restrict__ wF, int tid, int s) {
    const int sub = tid & 3;
    const int b = tid >> 2;
    const int g = b / (F / 4), w = b % (F / 4);
    const int h = F >> (2 * (s + 1));
    const int step = F / (4 * h);
    const int blk = w / h, j = w % h;
    const int i0 = blk * 4 * h + j;
    const double2 x = tile[tix<F, G, GM, ST>(g, i0 + sub * h)];
    const double2 o1 = shfl_xor_d2(x, 2);
    const bool hi = (sub & 2) != 0;  // lanes 2, 3: other - self
    const double2 l1 = make_double2(add_sgn(hi ? o1.x : x.x, hi ? x.x : o1.x, hi),
                                    add_sgn(hi ? o1.y : x.y, hi ? x.y : o1.y, hi));
    const double2 o2 = shfl_xor_d2(l1, 1);
    // lane 0: y0 = apc + bpd   lane 1: y2 = apc - bpd   lane 2: y1 = amc - i bmd   lane 3: y3 = amc + i bmd
    const bool odd = (sub & 1) != 0;
    const double qx = sub == 0 ? o2.x : sub == 1 ? l1.x : sub == 2 ? o2.y : l1.y;
    const double qy = sub == 0 ? o2.y : sub == 1 ? l1.y : sub == 2 ? o2.x : l1.x;
    double2 y = make_double2(add_sgn(odd ? o2.x : l1.x, qx, odd), add_sgn(odd ? o2.y : l1.y, qy, sub == 1 || sub == 2));
    const int ko = sub == 1 ? 2 : sub == 2 ? 1 : sub;  // output index
    if (h > 1) y = cmul(y, wF[ko * j * step]);
    tile[tix<F, G, GM, ST>(g, i0 + ko * h)] = y;
}

// Inverse counterpart (twiddle on the lane's input, then the two exchanges),
// bit-identical to cmulc + bfly4_inv.
template <int F, int G, bool GM, int ST = 0>
__device__ __forceinline__ void quad_stage_inv(double2* tile, const double2* __restrict__ wF, int tid, int s) {
    const int sub = tid & 3;
    const int b = tid >> 2;
    const int g = b / (F / 4), w = b % (F / 4);
    const int h = F >> (2 * (s + 1));
    const int step = F / (4 * h);
    const int blk = w / h, j = w % h;
    const int i0 = blk * 4 * h + j;
    double2 x = tile[tix<F, G, GM, ST>(g, i0 + sub * h)];
    if (h > 1) x = cmulc(x, wF[sub * j * step]);
    const double2 o1 = shfl_xor_d2(x, 2);
    const bool hi = (sub & 2) != 0;  // lanes 0, 1: s = z0 + z2, t = z1 + z3; lanes 2, 3: d = z0 - z2, u = z1 - z3
    const double2 l1 = make_double2(add_sgn(hi ? o1.x : x.x, hi ? x.x : o1.x, hi),
                                    add_sgn(hi ? o1.y : x.y, hi ? x.y : o1.y, hi));
    const double2 o2 = shfl_xor_d2(l1, 1);
    // lane 0: Z0 = s + t   lane 1: Z2 = s - t   lane 2: Z1 = d + i u   lane 3: Z3 = d - i u
    const bool odd = (sub & 1) != 0;
    const double qx = sub == 0 ? o2.x : sub == 1 ? l1.x : sub == 2 ? o2.y : l1.y;
    const double qy = sub == 0 ? o2.y : sub == 1 ? l1.y : sub == 2 ? o2.x : l1.x;
    const double2 z = make_double2(add_sgn(odd ? o2.x : l1.x, qx, sub == 1 || sub == 2),
                                   add_sgn(odd ? o2.y : l1.y, qy, odd));
    const int ko = sub == 1 ? 2 : sub == 2 ? 1 : sub;
    tile[tix<F, G, GM, ST>(g, i0 + ko * h)] = z;
}

// In-place forward DFT of length F on G groups of a shared tile, NT threads.
// Radix-4 stages with spans F/4, F/16, ...; a final radix-2 stage if log2 F is
// odd.  Output order is the digit reversal that the host's permutation table
// (plan construction) describes; the inverse below undoes it exactly.  With
// NT == F*G/2 every radix-4 butterfly is done by a pair of lanes, with
// NT == F*G by four lanes.
template <int F, int G, int NT, bool GM, int ST = 0, class Sync>
__device__ __forceinline__ void smem_fft_fwd(double2* tile, const double2* __restrict__ wF, int tid, Sync sync) {
    constexpr int LG = Lg<F>::v;
    constexpr int N4 = LG / 2;
    if constexpr (NT == F * G) {
#pragma unroll
        for (int s = 0; s < N4; ++s) {
            quad_stage_fwd<F, G, GM, ST>(tile, wF, tid, s);
            sync();
        }
    } else if constexpr (NT == F * G / 2) {
#pragma unroll
        for (int s = 0; s < N4; ++s) {
            pair_stage_fwd<F, G, GM, ST>(tile, wF, tid, s);
            sync();
        }
    } else {
#pragma unroll
    for (int s = 0; s < N4; ++s) {
        const int h = F >> (2 * (s + 1));
        const int step = F / (4 * h);
        for (int b = tid; b < G * F / 4; b += NT) {
            const int g = b / (F / 4), w = b % (F / 4);
            const int blk = w / h, j = w % h;
            const int i0 = blk * 4 * h + j;
            double2 a0 = tile[tix<F, G, GM, ST>(g, i0)];
            double2 a1 = tile[tix<F, G, GM, ST>(g, i0 + h)];
            double2 a2 = tile[tix<F, G, GM, ST>(g, i0 + 2 * h)];
            double2 a3 = tile[tix<F, G, GM, ST>(g, i0 + 3 * h)];
            bfly4_fwd(a0, a1, a2, a3);
            if (h > 1) {
                const int e = j * step;
                a1 = cmul(a1, wF[e]);
                a2 = cmul(a2, wF[2 * e]);
                a3 = cmul(a3, wF[3 * e]);
            }
            tile[tix<F, G, GM, ST>(g, i0)] = a0;
            tile[tix<F, G, GM, ST>(g, i0 + h)] = a1;
            tile[tix<F, G, GM, ST>(g, i0 + 2 * h)] = a2;
            tile[tix<F, G, GM, ST>(g, i0 + 3 * h)] = a3;
        }
        sync();
    }
    }
    if (LG & 1) {
        for (int b = tid; b < G * F / 2; b += NT) {
            const int g = b / (F / 2), i0 = 2 * (b % (F / 2));
            const double2 a = tile[tix<F, G, GM, ST>(g, i0)];
            const double2 c = tile[tix<F, G, GM, ST>(g, i0 + 1)];
            tile[tix<F, G, GM, ST>(g, i0)] = make_double2(a.x + c.x, a.y + c.y);
            tile[tix<F, G, GM, ST>(g, i0 + 1)] = make_double2(a.x - c.x, a.y - c.y);
        }
        sync();
    }
}

// Exact inverse (times F) of smem_fft_fwd.
template <int F, int G, int NT, bool GM, int ST = 0, class Sync>
__device__ __forceinline__ void smem_fft_inv(double2* tile, const double2* __restrict__ wF, int tid, Sync sync) {
    constexpr int LG = Lg<F>::v;
    constexpr int N4 = LG / 2;
    if (LG & 1) {
        for (int b = tid; b < G * F / 2; b += NT) {
            const int g = b / (F / 2), i0 = 2 * (b % (F / 2));
            const double2 a = tile[tix<F, G, GM, ST>(g, i0)];
            const double2 c = tile[tix<F, G, GM, ST>(g, i0 + 1)];
            tile[tix<F, G, GM, ST>(g, i0)] = make_double2(a.x + c.x, a.y + c.y);
            tile[tix<F, G, GM, ST>(g, i0 + 1)] = make_double2(a.x - c.x, a.y - c.y);
        }
        sync();
    }
    if constexpr (NT == F * G) {
#pragma unroll
        for (int s = N4 - 1; s >= 0; --s) {
            quad_stage_inv<F, G, GM, ST>(tile, wF, tid, s);
            sync();
        }
    } else if constexpr (NT == F * G / 2) {
#pragma unroll
        for (int s = N4 - 1; s >= 0; --s) {
            pair_stage_inv<F, G, GM, ST>(tile, wF, tid, s);
            sync();
        }
    } else {
#pragma unroll
    for (int s = N4 - 1; s >= 0; --s) {
        const int h = F >> (2 * (s + 1));
        const int step = F / (4 * h);
        for (int b = tid; b < G * F / 4; b += NT) {
            const int g = b / (F / 4), w = b % (F / 4);
            const int blk = w / h, j = w % h;
            const int i0 = blk * 4 * h + j;
            double2 z0 = tile[tix<F, G, GM, ST>(g, i0)];
            double2 z1 = tile[tix<F, G, GM, ST>(g, i0 + h)];
            double2 z2 = tile[tix<F, G, GM, ST>(g, i0 + 2 * h)];
            double2 z3 = tile[tix<F, G, GM, ST>(g, i0 + 3 * h)];
            if (h > 1) {
                const int e = j * step;
                z1 = cmulc(z1, wF[e]);
                z2 = cmulc(z2, wF[2 * e]);
                z3 = cmulc(z3, wF[3 * e]);
            }
            bfly4_inv(z0, z1, z2, z3);
            tile[tix<F, G, GM, ST>(g, i0)] = z0;
            tile[tix<F, G, GM, ST>(g, i0 + h)] = z1;
            tile[tix<F, G, GM, ST>(g, i0 + 2 * h)] = z2;
            tile[tix<F, G, GM, ST>(g, i0 + 3 * h)] = z3;
        }
        sync();
    }
    }
}

// ---- digit geometry and integer helpers ----

// S_j = ceil(j n / M): bit position of digit j (S_M = n).
__device__ __forceinline__ unsigned long long digit_pos(unsigned long long j, unsigned n, int lgM) {
    return (j * n + ((1ull << lgM) - 1)) >> lgM;
}
__device__ __forceinline__ int digit_width(unsigned long long j, unsigned n, int lgM) {
    return (int)(digit_pos(j + 1, n, lgM) - digit_pos(j, n, lgM));
}

__device__ __forceinline__ i128 load_carry(const long long* c, long long idx) {
    const unsigned long long lo = (unsigned long long)c[2 * idx];
    const long long hi = c[2 * idx + 1];
    return (i128)(((unsigned __int128)(unsigned long long)hi << 64) | lo);
}
__device__ __forceinline__ void store_carry(long long* c, long long idx, i128 v) {
    c[2 * idx] = (long long)(unsigned long long)v;
    c[2 * idx + 1] = (long long)(v >> 64);
}

// Small multiplier of step i: the left-to-right binary powering x <- x^2 a^bit
// over the bits of kexp below its top bit, then 1 (plain squaring).
__device__ __forceinline__ int sched_mul(const SlotState* st, long long i) {
    if (st->kexp == 0 || i < 0 || i >= (long long)st->kbits - 1) return 1;
    return ((st->kexp >> (st->kbits - 2 - i)) & 1ull) ? st->mul : 1;
}

// Split v into a balanced digit of width b (returned) and the carry (left in v).
__device__ __forceinline__ long long take_digit(i128& v, int b) {
    long long lo = (long long)((unsigned long long)v & ((1ull << b) - 1));
    if (lo >= (1ll << (b - 1))) lo -= (1ll << b);
    v = (v - (i128)lo) >> b;
    return lo;
}

// |v| < 2^61: the carry arithmetic of a run then fits in int64 (sums stay below
// 2^62), and the 64-bit path below gives exactly the 128-bit path's digits.
__device__ __forceinline__ bool fits61(i128 v) {
    const long long lo = (long long)(unsigned long long)v;
    return (long long)(v >> 64) == (lo >> 63) && ((lo >> 61) == 0 || (lo >> 61) == -1);
}
__device__ __forceinline__ long long take_digit64(long long& v, int b) {
    long long lo = v & ((1ll << b) - 1);
    if (lo >= (1ll << (b - 1))) lo -= (1ll << b);
    v = (v - lo) >> b;
    return lo;
}

// floor(a / b), b > 0.  Operands that fit in 63 bits (every k below 2^40 with the
// usual top digits) take the 64-bit division, much cheaper than the 128-bit one
// on the critical path of the top-digit reduction; the quotient is the same.
__device__ __forceinline__ i128 floor_div(i128 a, i128 b) {
    const i128 lim = (i128)1 << 62;
    if (a > -lim && a < lim && b < lim) {
        const long long a64 = (long long)a, b64 = (long long)b;
        long long q = a64 / b64;
        if ((a64 % b64) != 0 && a64 < 0) q -= 1;
        return (i128)q;
    }
    i128 q = a / b;
    if ((a % b) != 0 && a < 0) q -= 1;
    return q;
}

// a * b exactly, from one 64 x 64 -> 128-bit product (a and b signed).
__device__ __forceinline__ i128 mul_wide(long long a, long long b) {
    const unsigned long long lo = (unsigned long long)a * (unsigned long long)b;
    const long long hi = __mul64hi(a, b);
    return (i128)(((unsigned __int128)(unsigned long long)hi << 64) | lo);
}

// The Montgomery fold of one digit position of X_a X_b:  u_j = s (c_{M+j} +
// top_a d^b_j + top_b d^a_j - k c_j)  (X_a X_b 2^-n = H - k Lo, the cross terms
// of the top digits at weight 2^n).  Exact integer arithmetic.
__device__ __forceinline__ i128 fold_term(long long cl, long long ch, int dv, int dw, long long ta, long long tb,
                                          long long k, int s) {
    const i128 x = (i128)ch + mul_wide(ta, dw) + mul_wide(tb, dv) - mul_wide(k, cl);
    return s == 1 ? x : x * (i128)s;
}

// The in-run carry of one run of RUN digits starting at digit j0: u[t] are the
// fold terms; writes the balanced digits nd[] and returns the carry out.  Digit
// widths follow from S_j = ceil(j n / M), advanced by one add per digit.
__device__ __forceinline__ i128 run_carry(const i128 (&u)[RUN], unsigned long long j0, unsigned n, int lgM,
                                          int (&nd)[RUN]) {
    unsigned long long acc = j0 * n + ((1ull << lgM) - 1);
    unsigned long long p0 = acc >> lgM;
    bool small = true;
#pragma unroll
    for (int t = 0; t < RUN; ++t) small = small && fits61(u[t]);
    if (small) {  // |carry + u| < 2^62 throughout
        long long c64 = 0;
#pragma unroll
        for (int t = 0; t < RUN; ++t) {
            acc += n;
            const unsigned long long p1 = acc >> lgM;
            c64 += (long long)(unsigned long long)u[t];
            nd[t] = (int)take_digit64(c64, (int)(p1 - p0));
            p0 = p1;
        }
        return (i128)c64;
    }
    i128 carry = 0;
#pragma unroll
    for (int t = 0; t < RUN; ++t) {
        acc += n;
        const unsigned long long p1 = acc >> lgM;
        carry += u[t];
        nd[t] = (int)take_digit(carry, (int)(p1 - p0));
        p0 = p1;
    }
    return carry;
}

__device__ __forceinline__ i128 load_pend(const SlotState* st) {
    return (i128)(((unsigned __int128)(unsigned long long)st->pend_hi << 64) | (unsigned long long)st->pend_lo);
}
__device__ __forceinline__ void store_pend(SlotState* st, i128 v) {
    st->pend_lo = (long long)(unsigned long long)v;
    st->pend_hi = (long long)(v >> 64);
}

// Carry entering run `run` of a slot.  For run 0 it is minus the quotient of
// the top-digit reduction: top' = pend + (carry out of the last run), where
// pend = s top_a top_b of the last product, is split as q k + t with
// |t| <= k/2, and q k 2^n = -q (mod N).
__device__ __forceinline__ i128 run_carry_in(const Slot& sl, long long run, long long nruns,
                                             long long* new_top) {
    if (run > 0) return load_carry(sl.carries, run - 1);
    const SlotState* st = sl.st;
    const i128 clast = load_carry(sl.carries, nruns - 1);
    const i128 tp = load_pend(st) + clast;
    const i128 kk = (i128)sl.k;
    const i128 q = floor_div(2 * tp + kk, 2 * kk);
    *new_top = (long long)(tp - q * kk);
    return -q;
}

// Fold an incoming carry into the RUN digits of one run.  The carry shrinks
// by a digit width per position; whatever is left at the last digit of the run
// is added there unnormalised, so the run's own carry-out stays valid.
__device__ __forceinline__ void fixup_run(int (&dv)[RUN], i128 c, unsigned long long j0, unsigned n,
                                          int lgM, int& bad) {
    unsigned long long acc = j0 * n + ((1ull << lgM) - 1);  // S_j = ceil(j n / M), one add per digit
    unsigned long long p0 = acc >> lgM;
    if (fits61(c)) {
        long long c64 = (long long)c;
#pragma unroll
        for (int t = 0; t < RUN; ++t) {
            acc += n;
            const unsigned long long p1 = acc >> lgM;
            const int b = (int)(p1 - p0);
            p0 = p1;
            if (c64 != 0) {
                long long v = (long long)dv[t] + c64;
                if (t < RUN - 1) {
                    dv[t] = (int)take_digit64(v, b);
                    c64 = v;
                } else {
                    if (v > (1ll << 30) || v < -(1ll << 30)) bad = 1;
                    dv[t] = (int)v;
                    c64 = 0;
                }
            }
        }
        return;
    }
#pragma unroll
    for (int t = 0; t < RUN; ++t) {
        acc += n;
        const unsigned long long p1 = acc >> lgM;
        const int b = (int)(p1 - p0);
        p0 = p1;
        if (c != 0) {
            i128 v = (i128)dv[t] + c;
            if (t < RUN - 1) {
                dv[t] = (int)take_digit(v, b);
                c = v;
            } else {
                if (v > (i128)(1 << 30) || v < -(i128)(1 << 30)) bad = 1;
                dv[t] = (int)v;
                c = 0;
            }
        }
    }
}

// Round x to the nearest integer (ties to even) with one FP64 add of 1.5*2^52;
// tracks max |x - round(x)| in units of 2^-52 (kErrOne = 1.0), read off the bits
// of x with integer operations: the FP64 pipe (two lanes per clock per SM) is
// what a squaring waits on, the integer pipes are not.  With x = +-m 2^-sh
// (m the 53-bit significand), the distance to the nearest integer is
// min(f, 2^sh - f) 2^-sh for f = m mod 2^sh (|x| >= 1); 2^sh - m for
// 1/2 <= |x| < 1, and m itself below 1/2.
constexpr unsigned long long kErrOne = 1ull << 52;
__device__ __forceinline__ long long round_track(double x, unsigned long long& emax, int& bad) {
    const double MAGIC = 6755399441055744.0;  // 1.5 * 2^52
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((bits >> 52) & 0x7FF);
    if (ex >= 1023 + 50) bad = 1;  // |x| >= 2^50: outside the exact range
    const double y = x + MAGIC;
    const long long r = __double_as_longlong(y) - 0x4338000000000000LL;
    const unsigned long long m = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = 1075 - ex;  // x = +-m 2^-sh for ex > 0
    unsigned long long e = 0;  // zero and subnormals (below 2^-1022) count as exact
    if (ex != 0 && sh > 0) {
        if (sh <= 52) {
            const unsigned long long f = m & ((1ull << sh) - 1);
            const unsigned long long g = (1ull << sh) - f;
            e = (f < g ? f : g) << (52 - sh);
        } else if (sh == 53) {
            e = ((1ull << 53) - m) >> 1;
        } else if (sh < 116) {
            e = m >> (sh - 52);
        }
    }
    emax = e > emax ? e : emax;
    return r;
}
// A max |err| in units of 2^-52 as the bits of a non-negative double (their
// order is that of the values, so atomicMax on the bits keeps the largest).
__device__ __forceinline__ unsigned long long err_bits(unsigned long long e) {
    return (unsigned long long)__double_as_longlong((double)e * 0x1p-52);
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// ---------------------------------------------------------------------------
// Tile functions: NT threads (tid in [0, NT)) process one tile of one slot.
// The per-pass kernels run one tile per CTA (BlockSync); the persistent kernel
// runs one tile per warp (WarpSync, NT = 32).

// Pass 0 forward.  Tile = RUN consecutive columns r (each row of the tile is
// one carry run) x F0 rows q.  Needs NT >= F0.
template <int F0, int NT, class Sync, class Pre>
__device__ __forceinline__ void tile_first(const Slot& sl, const PlanDev& pl, int cta, int tid, double2* tile,
                                           int* dsm, Sync sync, Pre pre) {
    constexpr int G = RUN;
    constexpr int PER = (F0 * G + NT - 1) / NT;
    SlotState* st = sl.st;
    const int S0 = pl.S[0];
    const int r0 = cta * G;
    const long long nruns = pl.M / RUN;
    const double2* __restrict__ tw = pl.tw[0];
    double2 cw[PER], ct[PER];  // constants, loaded before waiting on the previous kernel
    const bool bound = sl.wf != nullptr;  // slots of a batch pool may not hold a candidate yet
    const bool unit = unit_weights(sl.n, pl.lgM);
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F0 * G && bound) {
            const int q = e / G, t = e % G;
            cw[i] = unit ? pl.thf[q] : sl.wf[r0 + t + q * S0];
            ct[i] = unit ? pl.twu[q * S0 + r0 + t] : tw[q * S0 + r0 + t];
        }
    }
    if (!pre()) return;
    if (tid < F0) {
        const unsigned long long j0 = (unsigned long long)r0 + (unsigned long long)tid * S0;
        const long long run = (long long)(j0 / RUN);
        int4* dp = reinterpret_cast<int4*>(sl.digits + j0);
        const int4 v0 = dp[0], v1 = dp[1];
        int dv[RUN] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
        long long new_top = 0;
        const i128 cin = run_carry_in(sl, run, nruns, &new_top);
        // each pending carry is consumed by exactly one run: zero it, and re-arm
        // the top as pending, so a slot that only feeds another product stays exact
        if (run == 0) {
            st->top = new_top;
            st->tope[(st->step + 1) & 1] = new_top;  // for a following k_edge (step + 1 by then)
            store_pend(st, (i128)new_top);
            store_carry(sl.carries, nruns - 1, 0);
        } else {
            store_carry(sl.carries, run - 1, 0);
        }
        int bad = 0;
        fixup_run(dv, cin, j0, sl.n, pl.lgM, bad);
        if (bad) atomicOr(&st->flags, SF_DIGIT_OVERFLOW);
        dp[0] = make_int4(dv[0], dv[1], dv[2], dv[3]);
        dp[1] = make_int4(dv[4], dv[5], dv[6], dv[7]);
#pragma unroll
        for (int t = 0; t < RUN; ++t) dsm[tid * G + t] = dv[t];
    }
    sync();
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F0 * G) {
            const double d = (double)dsm[e];
            tile[e] = make_double2(d * cw[i].x, d * cw[i].y);
        }
    }
    sync();
    smem_fft_fwd<F0, G, NT, false>(tile, pl.wF[0], tid, sync);
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F0 * G) {
            const int p = e / G, t = e % G;
            sl.spec[r0 + t + p * S0] = cmul(tile[e], ct[i]);
        }
    }
}

// Pass 1 (three-pass plans).  Tile = G consecutive columns of one block of length Mi[1].
template <int F, int G, int NT, class Sync, class Pre>
__device__ __forceinline__ void tile_mid_fwd(const Slot& sl, const PlanDev& pl, int cta, int tid, double2* tile,
                                             Sync sync, Pre pre) {
    constexpr int PER = (F * G + NT - 1) / NT;
    const int S = pl.S[1], Mi = pl.Mi[1];
    const int cpb = S / G;
    const int blk = cta / cpb, r0 = (cta % cpb) * G;
    double2* bp = sl.spec + (size_t)blk * Mi;
    const double2* __restrict__ tw = pl.tw[1];
    double2 ct[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F * G) ct[i] = tw[(e / G) * S + r0 + e % G];
    }
    if (!pre()) return;
    for (int e = tid; e < F * G; e += NT) {
        const int q = e / G, t = e % G;
        tile[e] = bp[r0 + t + q * S];
    }
    sync();
    smem_fft_fwd<F, G, NT, false>(tile, pl.wF[1], tid, sync);
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F * G) bp[r0 + e % G + (e / G) * S] = cmul(tile[e], ct[i]);
    }
}

template <int F, int G, int NT, class Sync, class Pre>
__device__ __forceinline__ void tile_mid_inv(const Slot& sl, const PlanDev& pl, int cta, int tid, double2* tile,
                                             Sync sync, Pre pre) {
    constexpr int PER = (F * G + NT - 1) / NT;
    const int S = pl.S[1], Mi = pl.Mi[1];
    const int cpb = S / G;
    const int blk = cta / cpb, r0 = (cta % cpb) * G;
    double2* bp = sl.spec + (size_t)blk * Mi;
    const double2* __restrict__ tw = pl.tw[1];
    double2 ct[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F * G) ct[i] = tw[(e / G) * S + r0 + e % G];
    }
    if (!pre()) return;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F * G) tile[e] = cmulc(bp[r0 + e % G + (e / G) * S], ct[i]);
    }
    sync();
    smem_fft_inv<F, G, NT, false>(tile, pl.wF[1], tid, sync);
    for (int e = tid; e < F * G; e += NT) {
        const int q = e / G, t = e % G;
        bp[r0 + t + q * S] = tile[e];
    }
}

// Last pass: G contiguous groups of F; forward, pointwise product with the
// partner's spectrum (itself for a square), inverse.
template <int F, int G, int LASTP, int NT, class Sync, class Pre>
__device__ __forceinline__ void tile_inner(const Slot& sl, const Slot& pb, bool square, const PlanDev& pl, int cta,
                                           int tid, double2* tile, double2* tile2, Sync sync, Pre pre) {
    if (!pre()) return;
    double2* bp = sl.spec + (size_t)cta * (F * G);
    for (int e = tid; e < F * G; e += NT) tile[e] = bp[e];
    if (!square) {
        const double2* qp = pb.spec + (size_t)cta * (F * G);
        for (int e = tid; e < F * G; e += NT) tile2[e] = qp[e];
    }
    sync();
    smem_fft_fwd<F, G, NT, true>(tile, pl.wF[LASTP], tid, sync);
    if (square) {
        for (int e = tid; e < F * G; e += NT) {
            const double2 z = tile[e];
            tile[e] = make_double2(fma(z.x, z.x, -(z.y * z.y)), (z.x + z.x) * z.y);
        }
    } else {
        smem_fft_fwd<F, G, NT, true>(tile2, pl.wF[LASTP], tid, sync);
        for (int e = tid; e < F * G; e += NT) tile[e] = cmul(tile[e], tile2[e]);
    }
    sync();
    smem_fft_inv<F, G, NT, true>(tile, pl.wF[LASTP], tid, sync);
    for (int e = tid; e < F * G; e += NT) bp[e] = tile[e];
}

// ---- bulk asynchronous copies (the TMA engine's non-tensor form) ----
// The last pass's tile is F*G contiguous complex values of one slot's spectrum,
// so one thread moves it between global and shared memory with a single bulk
// copy, completed through an mbarrier, instead of every thread issuing loads.

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Wait for phase `parity` of the barrier, at most kMbarPolls polls; false if it
// did not complete.
constexpr int kMbarPolls = 1 << 22;
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
    for (int i = 0; i < kMbarPolls; ++i) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
__device__ __forceinline__ void bulk_store(void* dst, const void* src, unsigned bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
                 "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// tile_inner with the tile (and the partner's tile) brought in and written back
// by bulk copies.  `bar` is a barrier of this CTA initialised for one arrival;
// the load completes its phase 0, which is the phase waited on (parity 0).
// If the load does not complete within the poll limit, the slot is flagged
// SF_WAIT_TIMEOUT, the copy is waited for once more, and the tile is left
// alone; if that second wait runs out too, SF_COPY_ABANDONED records that the
// CTA left with the copy possibly still in flight.  Either flag makes the host
// discard the step.
template <int F, int G, int LASTP, int NT, class Sync>
__device__ __forceinline__ void tile_inner_bulk(const Slot& sl, const Slot& pb, bool square, const PlanDev& pl,
                                                int cta, int tid, double2* tile, double2* tile2,
                                                unsigned long long* bar, Sync sync) {
    constexpr unsigned BYTES = F * G * sizeof(double2);
    double2* bp = sl.spec + (size_t)cta * (F * G);
    if (tid == 0) {
        mbar_expect_tx(bar, square ? BYTES : 2 * BYTES);
        bulk_load(tile, bp, BYTES, bar);
        if (!square) bulk_load(tile2, pb.spec + (size_t)cta * (F * G), BYTES, bar);
    }
    if (!mbar_wait(bar, 0)) {
        if (tid == 0) atomicOr(&sl.st->flags, SF_WAIT_TIMEOUT);
        if (!mbar_wait(bar, 0) && tid == 0) atomicOr(&sl.st->flags, SF_COPY_ABANDONED);
        return;
    }
    smem_fft_fwd<F, G, NT, true>(tile, pl.wF[LASTP], tid, sync);
    if (square) {
        for (int e = tid; e < F * G; e += NT) {
            const double2 z = tile[e];
            tile[e] = make_double2(fma(z.x, z.x, -(z.y * z.y)), (z.x + z.x) * z.y);
        }
    } else {
        smem_fft_fwd<F, G, NT, true>(tile2, pl.wF[LASTP], tid, sync);
        for (int e = tid; e < F * G; e += NT) tile[e] = cmul(tile[e], tile2[e]);
    }
    sync();
    smem_fft_inv<F, G, NT, true>(tile, pl.wF[LASTP], tid, sync);
    // the inverse ends with a barrier after its last stage; make the generic-proxy
    // writes visible to the bulk copy, then one thread stores the tile
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    sync();
    if (tid == 0) bulk_store(bp, tile, BYTES);
}

// Pass 0 inverse + unweight + round (max |err|) + Montgomery fold + in-run carry.
template <int F0, int NT, class Sync, class Pre>
__device__ __forceinline__ void tile_last(const Slot& sl, const Slot& pb, const PlanDev& pl, int cta, int tid,
                                          double2* tile, long long* cl, long long* ch, Sync sync, Pre pre) {
    constexpr int G = RUN;
    constexpr int PER = (F0 * G + NT - 1) / NT;
    SlotState* st = sl.st;
    const int S0 = pl.S[0];
    const int r0 = cta * G;
    const double2* __restrict__ tw = pl.tw[0];
    double2 ct[PER], cw[PER];
    const bool bound = sl.wi != nullptr;  // slots of a batch pool may not hold a candidate yet
    const bool unit = unit_weights(sl.n, pl.lgM);
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F0 * G && bound) {
            const int q = e / G, t = e % G;
            ct[i] = unit ? pl.twu[q * S0 + r0 + t] : tw[q * S0 + r0 + t];
            cw[i] = unit ? pl.thi[q] : sl.wi[r0 + t + q * S0];
        }
    }
    if (!pre()) return;
    // integer operands of the fold (the digits of both factors at this thread's
    // points), loaded now so their latency overlaps the transform
    const unsigned long long j0 = (unsigned long long)r0 + (unsigned long long)tid * S0;
    int dvi[PER], dwi[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        dvi[i] = dwi[i] = 0;
        if (e < F0 * G) {
            const int j = r0 + e % G + (e / G) * S0;
            dvi[i] = sl.digits[j];
            dwi[i] = pb.digits[j];
        }
    }
    const long long ta_ = st->top, tb_ = pb.st->top, step_ = st->step;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F0 * G) tile[e] = cmulc(sl.spec[r0 + e % G + (e / G) * S0], ct[i]);
    }
    sync();
    smem_fft_inv<F0, G, NT, false>(tile, pl.wF[0], tid, sync);
    unsigned long long emax = 0;
    int badr = 0;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F0 * G) {
            const double2 z = cmul(tile[e], cw[i]);
            cl[e] = round_track(z.x, emax, badr);
            ch[e] = round_track(z.y, emax, badr);
        }
    }
    if (badr) {
        emax = kErrOne;
        atomicOr(&st->flags, SF_ROUND_RANGE);
    }
    emax = warp_max_u64(emax);
    if ((tid & 31) == 0 && emax > 0) atomicMax(&st->maxerr_bits, err_bits(emax));
    // the fold term of every point, by the thread that rounded it (in place of its two halves)
    const int s_ = sched_mul(st, step_ - 1);
    const long long k_ = (long long)sl.k;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F0 * G) {
            const i128 u = fold_term(cl[e], ch[e], dvi[i], dwi[i], ta_, tb_, k_, s_);
            cl[e] = (long long)(unsigned long long)u;
            ch[e] = (long long)(u >> 64);
        }
    }
    sync();
    if (tid < F0) {
        const long long run = (long long)(j0 / RUN);
        if (run == 0) store_pend(st, (i128)s_ * (i128)ta_ * (i128)tb_);
        i128 u[RUN];
#pragma unroll
        for (int t = 0; t < RUN; ++t) {
            const int e = tid * G + t;
            u[t] = (i128)(((unsigned __int128)(unsigned long long)ch[e] << 64) | (unsigned long long)cl[e]);
        }
        int nd[RUN];
        const i128 carry = run_carry(u, j0, sl.n, pl.lgM, nd);
        int4* dp = reinterpret_cast<int4*>(sl.digits + j0);
        dp[0] = make_int4(nd[0], nd[1], nd[2], nd[3]);
        dp[1] = make_int4(nd[4], nd[5], nd[6], nd[7]);
        store_carry(sl.carries, run, carry);
    }
}

// ---------------------------------------------------------------------------
// Per-pass kernels: one tile per CTA, blockIdx.y = slot - base.

// `one` (by value): when its digits pointer is set, the launch squares that
// single residue (blockIdx.y == 0) for a step count the host controls exactly,
// so the kernels skip the slot-table load and the activity checks.

// TPB: threads per radix-4 butterfly (1; 2 or 4 for the paired- and four-lane transforms).
template <int F0, int TPB = 1>
__global__ void __launch_bounds__(2 * F0 * TPB) k_first(const Slot* __restrict__ slots, int base, const PlanDev pl,
                                                        const Slot one) {
    __shared__ double2 tile[F0 * RUN];
    __shared__ int dsm[F0 * RUN];
    if (one.digits) {
        tile_first<F0, 2 * F0 * TPB>(one, pl, blockIdx.x, threadIdx.x, tile, dsm, BlockSync(), PdlOnly());
    } else {
        const Slot sl = slots[base + blockIdx.y];
        tile_first<F0, 2 * F0 * TPB>(sl, pl, blockIdx.x, threadIdx.x, tile, dsm, BlockSync(),
                               PdlFirst{sl.st, blockIdx.x == 0 && threadIdx.x == 0});
    }
    pdl_trigger();
}

template <int F, int G, int TPB = 1>
__global__ void __launch_bounds__(F * G / 4 * TPB) k_mid_fwd(const Slot* __restrict__ slots, int base,
                                                             const PlanDev pl, const Slot one) {
    __shared__ double2 tile[F * G];
    if (one.digits) {
        tile_mid_fwd<F, G, F * G / 4 * TPB>(one, pl, blockIdx.x, threadIdx.x, tile, BlockSync(), PdlOnly());
    } else {
        const Slot sl = slots[base + blockIdx.y];
        tile_mid_fwd<F, G, F * G / 4 * TPB>(sl, pl, blockIdx.x, threadIdx.x, tile, BlockSync(),
                                            PdlActive{sl.st, false});
    }
    pdl_trigger();
}

template <int F, int G, int TPB = 1>
__global__ void __launch_bounds__(F * G / 4 * TPB) k_mid_inv(const Slot* __restrict__ slots, int base,
                                                             const PlanDev pl, const Slot one) {
    __shared__ double2 tile[F * G];
    if (one.digits) {
        tile_mid_inv<F, G, F * G / 4 * TPB>(one, pl, blockIdx.x, threadIdx.x, tile, BlockSync(), PdlOnly());
    } else {
        const Slot sl = slots[base + blockIdx.y];
        tile_mid_inv<F, G, F * G / 4 * TPB>(sl, pl, blockIdx.x, threadIdx.x, tile, BlockSync(),
                                            PdlActive{sl.st, true});
    }
    pdl_trigger();
}

template <int F, int G, int LASTP, int TPB = 1>
__global__ void __launch_bounds__(F * G / 4 * TPB) k_inner(const Slot* __restrict__ slots, int base,
                                                           const PlanDev pl, const Slot one) {
    __shared__ __align__(128) double2 tile[F * G];
    __shared__ __align__(128) double2 tile2[F * G];
    __shared__ unsigned long long bar;
    if (threadIdx.x == 0) mbar_init(&bar);
    __syncthreads();
    if (one.digits) {
        pdl_wait();
        if (blockIdx.x == 0 && threadIdx.x == 0) one.st->step += 1;
        tile_inner_bulk<F, G, LASTP, F * G / 4 * TPB>(one, one, true, pl, blockIdx.x, threadIdx.x, tile, tile2, &bar,
                                                       BlockSync());
        pdl_trigger();
        return;
    }
    const Slot sl = slots[base + blockIdx.y];
    SlotState* st = sl.st;
    pdl_wait();
    if (!st->active) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->step += 1;  // nobody reads step until k_last
    if (st->op == OP_FORWARD) return;                       // the partner's k_inner transforms this slot
    const int partner = st->partner;
    const bool square = partner == base + (int)blockIdx.y;
    tile_inner_bulk<F, G, LASTP, F * G / 4 * TPB>(sl, slots[partner], square, pl, blockIdx.x, threadIdx.x, tile,
                                                   tile2, &bar, BlockSync());
    pdl_trigger();
}

template <int F0, int TPB = 1>
__global__ void __launch_bounds__(2 * F0 * TPB) k_last(const Slot* __restrict__ slots, int base, const PlanDev pl,
                                                       const Slot one) {
    __shared__ double2 tile[F0 * RUN];
    __shared__ long long cl[F0 * RUN];
    __shared__ long long ch[F0 * RUN];
    if (one.digits) {
        tile_last<F0, 2 * F0 * TPB>(one, one, pl, blockIdx.x, threadIdx.x, tile, cl, ch, BlockSync(), PdlOnly());
    } else {
        const Slot sl = slots[base + blockIdx.y];
        SlotState* st = sl.st;
        // the partner index is fixed by the host before the step: safe to read early
        tile_last<F0, 2 * F0 * TPB>(sl, slots[st->partner], pl, blockIdx.x, threadIdx.x, tile, cl, ch, BlockSync(),
                                    PdlActive{st, true});
    }
    pdl_trigger();
}

// ---------------------------------------------------------------------------
// One residue, a chain of squarings: the last pass of squaring i and the first
// pass of squaring i+1 in ONE kernel (k_edge), for the same column tile (RUN
// columns x F0 rows), so the new digits go from the fold straight into the
// carry fix-up and the weight, without a kernel boundary or a round trip
// through global memory.  The only dependency between tiles is the run carry:
// every carry entering this tile's runs comes from the tile before it in the
// ring of tiles (tile c-1; for tile 0, the last tile, whose last run also feeds
// the top-digit reduction).  So each CTA publishes its carries with a release
// flag (the slot's step count) and waits, with a bounded number of polls, for
// its predecessor's flag; a wait that runs out sets SF_WAIT_TIMEOUT and the CTA
// skips its first-pass half, so the host discards the chunk.  All CTAs of the
// launch are resident together (a few KB of shared memory each, and the next
// kernel only starts once every CTA has passed its wait), so the wait ends.
// The operations on every value are those of tile_last and tile_first, in the
// same order: residues are bit-identical to the k_last + k_first sequence.
// The top digit of the squaring being finished is read from tope[] (indexed by
// the step parity) because tile 0 writes the next one while others may still
// read it.

constexpr int kEdgePolls = 1 << 22;

__device__ __forceinline__ void flag_publish(long long* f, long long v) {
    asm volatile("st.release.gpu.global.s64 [%0], %1;" ::"l"(f), "l"(v) : "memory");
}
__device__ __forceinline__ long long flag_read(const long long* f) {
    long long v;
    asm volatile("ld.acquire.gpu.global.s64 %0, [%1];" : "=l"(v) : "l"(f) : "memory");
    return v;
}
// A carry written by another CTA of this launch (read past the L1 cache).
__device__ __forceinline__ i128 load_carry_cg(const long long* c, long long idx) {
    const unsigned long long lo = (unsigned long long)__ldcg(c + 2 * idx);
    const long long hi = __ldcg(c + 2 * idx + 1);
    return (i128)(((unsigned __int128)(unsigned long long)hi << 64) | lo);
}

template <int F0, int TPB = 1>
__global__ void __launch_bounds__(2 * F0 * TPB) k_edge(const PlanDev pl, const Slot one, long long* __restrict__ eflags) {
    constexpr int NT = 2 * F0 * TPB;
    constexpr int G = RUN;
    constexpr int PER = (F0 * G + NT - 1) / NT;
    __shared__ double2 tile[F0 * RUN];
    __shared__ long long cl[F0 * RUN];
    __shared__ long long ch[F0 * RUN];
    __shared__ int dsm[F0 * RUN];
    __shared__ int go;
    const Slot& sl = one;
    SlotState* st = sl.st;
    const int cta = blockIdx.x, tid = threadIdx.x;
    const int S0 = pl.S[0];
    const int r0 = cta * G;
    const long long nruns = pl.M / RUN;
    const double2* __restrict__ tw = pl.tw[0];
    double2 ct[PER], cwi[PER], cwf[PER];  // constants, loaded before waiting on the previous kernel
    const bool unit = unit_weights(sl.n, pl.lgM);
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F0 * G) {
            const int q = e / G, t = e % G;
            ct[i] = unit ? pl.twu[q * S0 + r0 + t] : tw[q * S0 + r0 + t];
            cwi[i] = unit ? pl.thi[q] : sl.wi[r0 + t + q * S0];
            cwf[i] = unit ? pl.thf[q] : sl.wf[r0 + t + q * S0];
        }
    }
    pdl_wait();
    // ---- squaring i: pass 0 inverse, unweight, round, Montgomery fold, in-run carry ----
    const unsigned long long j0 = (unsigned long long)r0 + (unsigned long long)tid * S0;
    const long long run = (long long)(j0 / RUN);
    const long long step_ = st->step;  // squarings done, counting this one
    int4 v0 = make_int4(0, 0, 0, 0), v1 = v0;
    long long ta_ = 0;
    if (tid < F0) {
        const int4* dp = reinterpret_cast<const int4*>(sl.digits + j0);
        v0 = dp[0];
        v1 = dp[1];
        ta_ = st->tope[step_ & 1];
    }
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F0 * G) tile[e] = cmulc(sl.spec[r0 + e % G + (e / G) * S0], ct[i]);
    }
    __syncthreads();
    smem_fft_inv<F0, G, NT, false>(tile, pl.wF[0], tid, BlockSync());
    unsigned long long emax = 0;
    int badr = 0;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F0 * G) {
            const double2 z = cmul(tile[e], cwi[i]);
            cl[e] = round_track(z.x, emax, badr);
            ch[e] = round_track(z.y, emax, badr);
        }
    }
    if (badr) {
        emax = kErrOne;
        atomicOr(&st->flags, SF_ROUND_RANGE);
    }
    emax = warp_max_u64(emax);
    if ((tid & 31) == 0 && emax > 0) atomicMax(&st->maxerr_bits, err_bits(emax));
    __syncthreads();
    int nd[RUN] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (tid < F0) {
        const int dv[RUN] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
        const int s_ = sched_mul(st, step_ - 1);
        if (run == 0) store_pend(st, (i128)s_ * (i128)ta_ * (i128)ta_);
        i128 u[RUN];
#pragma unroll
        for (int t = 0; t < RUN; ++t) {
            const int e = tid * G + t;
            u[t] = fold_term(cl[e], ch[e], dv[t], dv[t], ta_, ta_, (long long)sl.k, s_);
        }
        store_carry(sl.carries, run, run_carry(u, j0, sl.n, pl.lgM, nd));
    }
    // ---- publish this tile's carries; wait for those of the tile before it ----
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        flag_publish(eflags + cta, step_);
        const long long* pf = eflags + (cta == 0 ? (int)gridDim.x - 1 : cta - 1);
        int ok = 0;
        for (int i = 0; i < kEdgePolls; ++i) {
            if (flag_read(pf) == step_) {
                ok = 1;
                break;
            }
        }
        if (!ok) atomicOr(&st->flags, SF_WAIT_TIMEOUT);
        go = ok;
    }
    __syncthreads();
    if (!go) {
        pdl_trigger();
        return;
    }
    // ---- squaring i+1: carry fix-up, top reduction, weight, pass 0 forward ----
    if (tid < F0) {
        i128 cin;
        if (run > 0) {
            cin = load_carry_cg(sl.carries, run - 1);
            store_carry(sl.carries, run - 1, 0);
        } else {
            const i128 tp = load_pend(st) + load_carry_cg(sl.carries, nruns - 1);
            const i128 kk = (i128)sl.k;
            const i128 q = floor_div(2 * tp + kk, 2 * kk);
            const long long new_top = (long long)(tp - q * kk);
            cin = -q;
            st->top = new_top;
            st->tope[(step_ + 1) & 1] = new_top;
            store_pend(st, (i128)new_top);
            store_carry(sl.carries, nruns - 1, 0);
        }
        int bad = 0;
        fixup_run(nd, cin, j0, sl.n, pl.lgM, bad);
        if (bad) atomicOr(&st->flags, SF_DIGIT_OVERFLOW);
        int4* dp = reinterpret_cast<int4*>(sl.digits + j0);
        dp[0] = make_int4(nd[0], nd[1], nd[2], nd[3]);
        dp[1] = make_int4(nd[4], nd[5], nd[6], nd[7]);
#pragma unroll
        for (int t = 0; t < RUN; ++t) dsm[tid * G + t] = nd[t];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F0 * G) {
            const double d = (double)dsm[e];
            tile[e] = make_double2(d * cwf[i].x, d * cwf[i].y);
        }
    }
    __syncthreads();
    smem_fft_fwd<F0, G, NT, false>(tile, pl.wF[0], tid, BlockSync());
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        if (e < F0 * G) {
            const int p = e / G, t = e % G;
            sl.spec[r0 + t + p * S0] = cmul(tile[e], ct[i]);
        }
    }
    pdl_trigger();
}

// ---------------------------------------------------------------------------
// The middle of a three-pass squaring in ONE kernel, on a thread-block cluster.
//
// After pass 0 the spectrum splits into F0 independent contiguous blocks of
// Mi[1] = F * F points (F = F[1] = F[2]); pass 1 forward, pass 2 forward, the
// square, pass 2 inverse and pass 1 inverse never look outside a block.  A
// cluster of CL CTAs owns one block: each CTA does the pass-1 transforms of
// G = F / CL columns, hands every value to the CTA that owns its pass-2 group
// by a store into that CTA's shared memory (distributed shared memory), squares
// G groups of F contiguous points, hands them back the same way, and finishes
// the inverse pass-1 transforms of its columns.  The two hand-overs replace two
// kernel boundaries (and their L2 round trips) by cluster barriers.  The
// operations on every value and their order are those of k_mid_fwd, k_inner and
// k_mid_inv, so the residues are bit-identical to the three-kernel sequence.
// Single residue only (the descriptor by value, as `one` above).

__device__ __forceinline__ unsigned cluster_ctarank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// Address of the same shared variable in CTA `rank` of this cluster.
__device__ __forceinline__ unsigned mapa_shared(unsigned local, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
    return r;
}
__device__ __forceinline__ void st_cluster(unsigned addr, double2 v) {
    asm volatile("st.shared::cluster.v2.f64 [%0], {%1, %2};" ::"r"(addr), "d"(v.x), "d"(v.y) : "memory");
}
// Cluster barrier halves.  Every thread of every CTA of the cluster executes
// each of them the same number of times (no early exit in k_block).
__device__ __forceinline__ void cluster_arrive_relaxed() {
    asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

template <int F, int CL, int TPB>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(F * (F / CL) / 4 * TPB)
    k_block(const PlanDev pl, const Slot one) {
    constexpr int G = F / CL;                // pass-1 columns = pass-2 groups per CTA
    constexpr int NT = F * G / 4 * TPB;
    constexpr int PER = F * G / NT;
    static_assert(G >= 2 && F * G % NT == 0, "block shape");
    __shared__ __align__(16) double2 ta[F * G];  // pass-1 tile: element (row q, column t) at q * G + t
    __shared__ __align__(16) double2 tb[F * G];  // pass-2 tile: element (group g, point i) at g * F + i
    const int tid = threadIdx.x;
    const unsigned c = cluster_ctarank();
    const int blk = blockIdx.x / CL;
    const int S = pl.S[1];                   // == F
    double2* bp = one.spec + (size_t)blk * pl.Mi[1];
    const int r0 = (int)c * G;
    const double2* __restrict__ tw = pl.tw[1];
    double2 ct[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        ct[i] = tw[(e / G) * S + r0 + e % G];
    }
    cluster_arrive_relaxed();  // paired with the wait before the first remote store
    pdl_wait();
    if (blockIdx.x == 0 && tid == 0) one.st->step += 1;  // nobody reads step until k_last
    // pass 1 forward on columns r0 .. r0+G-1
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        ta[e] = bp[r0 + e % G + (e / G) * S];
    }
    __syncthreads();
    smem_fft_fwd<F, G, NT, false>(ta, pl.wF[1], tid, BlockSync());
    cluster_wait();  // every CTA of the cluster is running
    // value (row q, column r0+t) is point r0+t of group q: CTA q / G, slot (q % G) * F + r0 + t
    const unsigned tb_local = smem_u32(tb);
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        const int q = e / G, t = e % G;
        const unsigned dst = tb_local + (unsigned)(((q % G) * F + r0 + t) * (int)sizeof(double2));
        st_cluster(mapa_shared(dst, (unsigned)(q / G)), cmul(ta[e], ct[i]));
    }
    cluster_arrive();
    cluster_wait();
    // pass 2 on groups c*G .. c*G+G-1: forward, square, inverse
    smem_fft_fwd<F, G, NT, true>(tb, pl.wF[2], tid, BlockSync());
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        const double2 z = tb[e];
        tb[e] = make_double2(fma(z.x, z.x, -(z.y * z.y)), (z.x + z.x) * z.y);
    }
    __syncthreads();
    smem_fft_inv<F, G, NT, true>(tb, pl.wF[2], tid, BlockSync());
    // point i of group c*G+g is (row c*G+g, column i): CTA i / G, slot (c*G+g) * G + i % G
    const unsigned ta_local = smem_u32(ta);
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        const int g = e / F, pt = e % F;
        const unsigned dst = ta_local + (unsigned)((((int)c * G + g) * G + pt % G) * (int)sizeof(double2));
        st_cluster(mapa_shared(dst, (unsigned)(pt / G)), tb[e]);
    }
    cluster_arrive();
    cluster_wait();  // after this no CTA touches another's shared memory
    // pass 1 inverse on columns r0 .. r0+G-1
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        ta[e] = cmulc(ta[e], ct[i]);
    }
    __syncthreads();
    smem_fft_inv<F, G, NT, false>(ta, pl.wF[1], tid, BlockSync());
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = tid + i * NT;
        bp[r0 + e % G + (e / G) * S] = ta[e];
    }
    pdl_trigger();
}

// ---------------------------------------------------------------------------
// Persistent kernel: `steps` squarings of slots [base, base + count) in one
// cooperative launch, the five passes separated by a grid barrier.  Each warp
// is a worker that takes tiles w, w + W, ... of a pass (worker ids interleave
// CTAs, so consecutive tiles land on different SMs).

struct GridBar {
    unsigned count;
    unsigned gen;
    int err;        // set when a barrier wait ran out of its spin budget
    int pad;
};

// All CTAs of a cooperative grid meet here.  Every wait is bounded: after
// kBarSpins polls the CTA records the failure and returns false, and every
// CTA then leaves the kernel at its next barrier.
constexpr long long kBarSpins = 1ll << 24;

__device__ __forceinline__ bool grid_barrier(GridBar* bar) {
    __syncthreads();
    __shared__ int ok;
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = &bar->gen;
        volatile int* verr = &bar->err;
        const unsigned g = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(&bar->count, 1u) + 1u;
        int good = 1;
        if (arrived == gridDim.x) {
            bar->count = 0;
            __threadfence();
            atomicAdd(&bar->gen, 1u);
        } else {
            long long spins = 0;
            while (*vgen == g) {
                if (*verr || ++spins > kBarSpins) {
                    atomicExch(&bar->err, 1);
                    good = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        ok = good && !*verr;
    }
    __syncthreads();
    return ok != 0;
}

template <int F0, int F1, int F2, int G1, int G2, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) k_persist(const Slot* __restrict__ slots, int base, int count,
                                                        const PlanDev pl, long long steps, GridBar* bar) {
    static_assert(F0 <= 32 && F1 * G1 / 4 >= 32 && F2 * G2 / 4 >= 32, "one warp per tile");
    constexpr int TILE = (F0 * RUN > F1 * G1 ? (F0 * RUN > F2 * G2 ? F0 * RUN : F2 * G2)
                                             : (F1 * G1 > F2 * G2 ? F1 * G1 : F2 * G2));
    __shared__ double2 sm_tile[WARPS][TILE];
    __shared__ long long sm_i64[WARPS][2 * F0 * RUN];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int W = WARPS * gridDim.x;
    const int wid = warp * gridDim.x + blockIdx.x;
    double2* tile = sm_tile[warp];
    int* dsm = reinterpret_cast<int*>(sm_i64[warp]);
    long long* cl = sm_i64[warp];
    long long* ch = sm_i64[warp] + F0 * RUN;
    const int t_first = (pl.S[0] / RUN), t_mid = pl.M / (F1 * G1), t_inner = pl.M / (F2 * G2);
    const WarpSync ws;
    for (long long it = 0; it < steps; ++it) {
        for (int t = wid; t < t_first * count; t += W) {
            const int s = base + t / t_first;
            tile_first<F0, 32>(slots[s], pl, t % t_first, lane, tile, dsm, ws, NoWait());
        }
        if (!grid_barrier(bar)) return;
        for (int t = wid; t < t_mid * count; t += W) {
            const int s = base + t / t_mid;
            tile_mid_fwd<F1, G1, 32>(slots[s], pl, t % t_mid, lane, tile, ws, NoWait());
        }
        if (!grid_barrier(bar)) return;
        for (int t = wid; t < t_inner * count; t += W) {
            const int s = base + t / t_inner;
            const int c = t % t_inner;
            if (c == 0 && lane == 0) slots[s].st->step += 1;
            tile_inner<F2, G2, 2, 32>(slots[s], slots[s], true, pl, c, lane, tile, tile, ws, NoWait());
        }
        if (!grid_barrier(bar)) return;
        for (int t = wid; t < t_mid * count; t += W) {
            const int s = base + t / t_mid;
            tile_mid_inv<F1, G1, 32>(slots[s], pl, t % t_mid, lane, tile, ws, NoWait());
        }
        if (!grid_barrier(bar)) return;
        for (int t = wid; t < t_first * count; t += W) {
            const int s = base + t / t_first;
            tile_last<F0, 32>(slots[s], slots[s], pl, t % t_first, lane, tile, cl, ch, ws, NoWait());
        }
        if (!grid_barrier(bar)) return;
    }
}

// k_readback: resolve the pending carries of each slot into out_digits /
// out_top without changing the slot state.  One thread per run.
__global__ void k_readback(const Slot* __restrict__ slots, int base, const PlanDev pl, int* __restrict__ out_digits,
                           long long* __restrict__ out_top) {
    const Slot sl = slots[base + blockIdx.y];
    const long long nruns = pl.M / RUN;
    const long long run = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (run >= nruns) return;
    const unsigned long long j0 = (unsigned long long)run * RUN;
    const int* dp = sl.digits + j0;
    int dv[RUN];
#pragma unroll
    for (int t = 0; t < RUN; ++t) dv[t] = dp[t];
    long long new_top = 0;
    const i128 cin = run_carry_in(sl, run, nruns, &new_top);
    int bad = 0;
    fixup_run(dv, cin, j0, sl.n, pl.lgM, bad);
    int* op = out_digits + (size_t)(base + blockIdx.y) * pl.M + j0;
#pragma unroll
    for (int t = 0; t < RUN; ++t) op[t] = dv[t];
    if (run == 0) out_top[base + blockIdx.y] = new_top;
    if (bad) atomicOr(&sl.st->flags, SF_DIGIT_OVERFLOW);
}

// Test hook: add delta to one pending digit (a simulated silent memory error).
__global__ void k_corrupt(const Slot* __restrict__ slots, int slot, unsigned index, int delta) {
    if (threadIdx.x == 0 && blockIdx.x == 0) slots[slot].digits[index] += delta;
}

}  // namespace pg

#endif

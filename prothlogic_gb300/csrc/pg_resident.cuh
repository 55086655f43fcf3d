// pg_resident.cuh -- squaring chains with the residue resident in shared memory.
//
// One thread-block cluster of CL CTAs per residue (CL = 1: one CTA) runs
// `steps` squarings in a single launch; between squarings the digits, the
// pending run carries and the slot's top digit stay in the cluster's shared
// memory, and only the first and last squaring of the launch touch the slot's
// global state.  Two-pass plans, M = F0 * F1:
//
//   column phase  CTA c owns columns r in [c*G0, (c+1)*G0), G0 = F1 / CL, all F0
//                 rows (digit j = r + q*F1): carry fix-up, weight, the F0-point
//                 forward transforms, the inter-pass twiddle; later the inverse
//                 twiddle, the F0-point inverse transforms, unweight, rounding
//                 and the Montgomery fold with the in-run carries;
//   group phase   CTA c owns groups p in [c*G1, (c+1)*G1), G1 = F0 / CL, of F1
//                 contiguous points: forward transform, square, inverse.
//
// The two hand-overs between the phases are stores into the owning CTA's
// shared memory (distributed shared memory) followed by a cluster barrier, and
// the carry out of the last run of a row of columns reaches the next CTA's first
// run through the same memory.  With CL = 1 the column and group views are the
// same array (element (q, t) is point t of group q) and nothing moves.
//
// Every value goes through the operations of k_first, k_inner and k_last, in
// the same order (the same tile transforms, twiddle and weight tables, rounding
// and fold), so residues are bit-identical to the per-pass kernels'.  The
// cluster barriers are hardware barriers that every thread of every CTA of the
// cluster reaches the same number of times (the only early exit is taken by a
// whole cluster before its first barrier); there is no spin-wait.
#ifndef PG_RESIDENT_CUH
#define PG_RESIDENT_CUH

#include "pg_kernels.cuh"

namespace pg {

template <int F0_, int F1_, int CL_, int NT_>
struct ResGeom {
    static constexpr int F0 = F0_, F1 = F1_, CL = CL_, NT = NT_;
    static constexpr int M = F0 * F1;
    static constexpr int G0 = F1 / CL;                     // columns per CTA
    static constexpr int G1 = F0 / CL;                     // groups per CTA
    static constexpr int PTS = M / CL;                     // points per CTA
    static constexpr int RPR = G0 / RUN;                   // carry runs per row of a CTA's columns
    static constexpr int RUNS = PTS / RUN;                 // carry runs per CTA
    static constexpr int SA = (CL == 1 ? F1 : G0) + 1;     // padded row stride of the column tile
    static constexpr int SB = F1 + 1;                      // padded row stride of the group tile
    static constexpr int A_ELEMS = F0 * SA;
    static constexpr int B_ELEMS = CL == 1 ? 0 : G1 * SB;  // CL = 1: the group tile is the column tile
    static constexpr int PER = PTS / NT;                   // points per thread in element-wise phases
    static constexpr size_t SMEM = (size_t)(A_ELEMS + B_ELEMS) * 16 + (size_t)RUNS * 16 + (size_t)PTS * 4 + 64;
    static_assert(G0 % RUN == 0 && G1 >= 1 && PTS % NT == 0, "resident shape");
    static_assert(CL == 1 || SA == G0 + 1, "padding");
};

__device__ __forceinline__ void ld_cluster_u64x2(unsigned addr, long long& a, long long& b) {
    asm volatile("ld.shared::cluster.v2.s64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "r"(addr) : "memory");
}
__device__ __forceinline__ long long ld_cluster_s64(unsigned addr) {
    long long a;
    asm volatile("ld.shared::cluster.s64 %0, [%1];" : "=l"(a) : "r"(addr) : "memory");
    return a;
}

// Whole-cluster barrier (release/acquire), or the CTA barrier when CL == 1.
template <int CL>
__device__ __forceinline__ void res_sync() {
    if constexpr (CL == 1) {
        __syncthreads();
    } else {
        cluster_arrive();
        cluster_wait();
    }
}

// Carry (lo, hi) of local run `lr` in CTA `rank` (this CTA when CL == 1).
template <int CL>
__device__ __forceinline__ i128 res_carry(const long long* cout, unsigned rank, int lr) {
    long long lo, hi;
    if constexpr (CL == 1) {
        lo = cout[2 * lr];
        hi = cout[2 * lr + 1];
    } else {
        ld_cluster_u64x2(mapa_shared(smem_u32(cout + 2 * lr), rank), lo, hi);
    }
    return (i128)(((unsigned __int128)(unsigned long long)hi << 64) | (unsigned long long)lo);
}

// One CTA of a cluster per SM is what a lone residue needs; batch residues (CL = 1) want two per SM.
template <int F0, int F1, int CL, int NT>
__global__ void __launch_bounds__(NT, (CL == 1 && NT <= 512) ? 2 : 1)
    k_resident(const Slot* __restrict__ slots, int base, const PlanDev pl, long long steps) {
    using R = ResGeom<F0, F1, CL, NT>;
    extern __shared__ __align__(16) unsigned char res_smem[];
    double2* A = reinterpret_cast<double2*>(res_smem);
    double2* B = CL == 1 ? A : A + R::A_ELEMS;
    long long* cout = reinterpret_cast<long long*>(A + R::A_ELEMS + R::B_ELEMS);  // RUNS (lo, hi) pairs
    int* dig = reinterpret_cast<int*>(cout + 2 * R::RUNS);                        // RUN digits per local run
    long long* misc = reinterpret_cast<long long*>(dig + R::PTS);                 // [0] top, [1..2] pend (CTA 0)
    const int tid = threadIdx.x;
    const unsigned c = CL == 1 ? 0u : cluster_ctarank();
    const Slot sl = slots[base + (int)(blockIdx.x / CL)];
    SlotState* st = sl.st;
    const long long step0 = st->step;
    const long long nsq = min(steps, st->total - step0);
    if (nsq <= 0 || sl.wf == nullptr) return;  // the same answer in every CTA of the cluster
    const unsigned long long kexp = st->kexp;
    const int kbits = st->kbits, mul = st->mul;
    const unsigned n = sl.n;
    const int lgM = pl.lgM;
    const i128 kk = (i128)sl.k;  // the top-digit reduction
    // n divisible by M: weights theta^(q F1) per row, theta^r folded into the twiddles
    const bool unit = unit_weights(n, lgM);
    const double2* __restrict__ tw = unit ? pl.twu : pl.tw[0];
    const double2* __restrict__ wf = sl.wf;
    const double2* __restrict__ wi = sl.wi;
    // With few points per thread, the weights and twiddles a thread uses stay in
    // registers for the whole chain instead of being read again every squaring.
    constexpr bool CACHE = R::PER <= 2;
    constexpr int NC = CACHE ? R::PER : 1;
    double2 c_wf[NC], c_tf[NC], c_ti[NC], c_wi[NC];
    if constexpr (CACHE) {
#pragma unroll
        for (int i = 0; i < R::PER; ++i) {
            const int e = tid + i * NT, q = e / R::G0, t = e % R::G0;
            const int j = (int)c * R::G0 + t + q * F1;
            c_wf[i] = unit ? pl.thf[q] : wf[j];
            c_wi[i] = unit ? pl.thi[q] : wi[j];
            c_tf[i] = tw[q * F1 + (int)c * R::G0 + t];
            const int g = e / F1, x = e % F1;
            c_ti[i] = tw[((int)c * R::G1 + g) * F1 + x];
        }
    }

    // prologue: the CTA's digits and pending carries, the slot's top and pending top
    for (int lr = tid; lr < R::RUNS; lr += NT) {
        const int q = lr / R::RPR, r = (int)c * R::G0 + (lr % R::RPR) * RUN;
        const long long j0 = r + (long long)q * F1;
        const int4* dp = reinterpret_cast<const int4*>(sl.digits + j0);
        const int4 v0 = dp[0], v1 = dp[1];
        int* d = dig + lr * RUN;
        d[0] = v0.x; d[1] = v0.y; d[2] = v0.z; d[3] = v0.w;
        d[4] = v1.x; d[5] = v1.y; d[6] = v1.z; d[7] = v1.w;
        cout[2 * lr] = sl.carries[2 * (j0 / RUN)];
        cout[2 * lr + 1] = sl.carries[2 * (j0 / RUN) + 1];
    }
    if (c == 0 && tid == 0) {
        misc[0] = st->top;
        misc[1] = st->pend_lo;
        misc[2] = st->pend_hi;
    }
    res_sync<CL>();  // every CTA of the cluster runs and holds its state

    unsigned long long emax = 0;
    int flags = 0;
    for (long long it = 0; it < nsq; ++it) {
        const long long step = step0 + it;
        // 1. carry fix-up: each run takes the pending carry of the run before it
        for (int lr = tid; lr < R::RUNS; lr += NT) {
            const int q = lr / R::RPR, t8 = lr % R::RPR;
            const int r = (int)c * R::G0 + t8 * RUN;
            const unsigned long long j0 = (unsigned long long)r + (unsigned long long)q * F1;
            i128 cin;
            if (j0 == 0) {
                // top reduction: top' = pend + carry of the last run = q k + t, q k 2^n = -q
                const i128 clast = res_carry<CL>(cout, CL - 1, R::RUNS - 1);
                const i128 tp = (i128)(((unsigned __int128)(unsigned long long)misc[2] << 64) |
                                       (unsigned long long)misc[1]) + clast;
                const i128 qq = floor_div(2 * tp + kk, 2 * kk);
                const long long new_top = (long long)(tp - qq * kk);
                cin = -qq;
                misc[0] = new_top;
                misc[1] = new_top;
                misc[2] = new_top < 0 ? -1 : 0;
            } else if (t8 > 0) {
                cin = res_carry<CL>(cout, c, lr - 1);
            } else if (c > 0) {
                cin = res_carry<CL>(cout, c - 1, q * R::RPR + R::RPR - 1);
            } else {
                cin = res_carry<CL>(cout, CL - 1, (q - 1) * R::RPR + R::RPR - 1);
            }
            int dv[RUN];
#pragma unroll
            for (int u = 0; u < RUN; ++u) dv[u] = dig[lr * RUN + u];
            int bad = 0;
            fixup_run(dv, cin, j0, n, lgM, bad);
            if (bad) flags |= SF_DIGIT_OVERFLOW;
#pragma unroll
            for (int u = 0; u < RUN; ++u) dig[lr * RUN + u] = dv[u];
        }
        __syncthreads();
        // 2. weight (column tile (q, t) holds digit j = c G0 + t + q F1)
#pragma unroll 4
        for (int i = 0; i < R::PER; ++i) {
            const int e = tid + i * NT, q = e / R::G0, t = e % R::G0;
            const int j = (int)c * R::G0 + t + q * F1;
            const double d = (double)dig[(q * R::RPR + t / RUN) * RUN + t % RUN];
            const double2 w = CACHE ? c_wf[i < NC ? i : 0] : (unit ? pl.thf[q] : wf[j]);
            A[q * R::SA + t] = make_double2(d * w.x, d * w.y);
        }
        __syncthreads();
        // 3. pass 0 forward; twiddle; hand each value to the CTA that owns its group
        smem_fft_fwd<F0, R::G0, NT, false, R::SA>(A, pl.wF[0], tid, BlockSync());
#pragma unroll 4
        for (int i = 0; i < R::PER; ++i) {
            const int e = tid + i * NT, q = e / R::G0, t = e % R::G0;
            const int r = (int)c * R::G0 + t;
            const double2 v = cmul(A[q * R::SA + t], CACHE ? c_tf[i < NC ? i : 0] : tw[q * F1 + r]);
            if constexpr (CL == 1) {
                A[q * R::SA + t] = v;
            } else {
                const unsigned dst = smem_u32(B + (q % R::G1) * R::SB + r);
                st_cluster(mapa_shared(dst, (unsigned)(q / R::G1)), v);
            }
        }
        res_sync<CL>();
        // 4. pass 1: forward, square, inverse
        smem_fft_fwd<F1, R::G1, NT, true, R::SB>(B, pl.wF[1], tid, BlockSync());
#pragma unroll 4
        for (int i = 0; i < R::PER; ++i) {
            const int e = tid + i * NT, g = e / F1, x = e % F1;
            const double2 z = B[g * R::SB + x];
            B[g * R::SB + x] = make_double2(fma(z.x, z.x, -(z.y * z.y)), (z.x + z.x) * z.y);
        }
        __syncthreads();
        smem_fft_inv<F1, R::G1, NT, true, R::SB>(B, pl.wF[1], tid, BlockSync());
        // 5. inverse twiddle; hand each value back to the CTA that owns its column
#pragma unroll 4
        for (int i = 0; i < R::PER; ++i) {
            const int e = tid + i * NT, g = e / F1, x = e % F1;
            const int p = (int)c * R::G1 + g;
            const double2 v = cmulc(B[g * R::SB + x], CACHE ? c_ti[i < NC ? i : 0] : tw[p * F1 + x]);
            if constexpr (CL == 1) {
                B[g * R::SB + x] = v;
            } else {
                const unsigned dst = smem_u32(A + p * R::SA + x % R::G0);
                st_cluster(mapa_shared(dst, (unsigned)(x / R::G0)), v);
            }
        }
        res_sync<CL>();
        // 6. pass 0 inverse; unweight, round, and the fold term of every point, in place:
        //    u_j = s (c_{M+j} + 2 top d_j - k c_j)  (X^2 2^-n = H - k Lo, cross terms at weight 2^n)
        smem_fft_inv<F0, R::G0, NT, false, R::SA>(A, pl.wF[0], tid, BlockSync());
        // the top digit from CTA 0 (set by this squaring's fix-up, before the hand-overs)
        long long top;
        if constexpr (CL == 1) {
            top = misc[0];
        } else {
            top = ld_cluster_s64(mapa_shared(smem_u32(misc), 0u));
        }
        const int s_ = (kexp == 0 || step >= (long long)kbits - 1)
                           ? 1
                           : (((kexp >> (kbits - 2 - step)) & 1ull) ? mul : 1);
        {
            int badr = 0;
#pragma unroll 4
            for (int i = 0; i < R::PER; ++i) {
                const int e = tid + i * NT, q = e / R::G0, t = e % R::G0;
                const int j = (int)c * R::G0 + t + q * F1;
                const double2 z = cmul(A[q * R::SA + t], CACHE ? c_wi[i < NC ? i : 0] : (unit ? pl.thi[q] : wi[j]));
                const long long lo = round_track(z.x, emax, badr);
                const long long hi = round_track(z.y, emax, badr);
                const int dv = dig[(q * R::RPR + t / RUN) * RUN + t % RUN];
                const i128 u = fold_term(lo, hi, dv, dv, top, top, (long long)sl.k, s_);
                long long* cell = reinterpret_cast<long long*>(A + q * R::SA + t);
                cell[0] = (long long)(unsigned long long)u;
                cell[1] = (long long)(u >> 64);
            }
            if (badr) {
                emax = kErrOne;
                flags |= SF_ROUND_RANGE;
            }
        }
        __syncthreads();
        // 7. in-run carry over the fold terms of each run
        for (int lr = tid; lr < R::RUNS; lr += NT) {
            const int q = lr / R::RPR, t0 = (lr % R::RPR) * RUN;
            const unsigned long long j0 = (unsigned long long)((int)c * R::G0 + t0) + (unsigned long long)q * F1;
            if (j0 == 0) {
                const i128 pend = (i128)s_ * (i128)top * (i128)top;
                misc[1] = (long long)(unsigned long long)pend;
                misc[2] = (long long)(pend >> 64);
            }
            i128 u[RUN];
#pragma unroll
            for (int x = 0; x < RUN; ++x) {
                const long long* cell = reinterpret_cast<const long long*>(A + q * R::SA + t0 + x);
                u[x] = (i128)(((unsigned __int128)(unsigned long long)cell[1] << 64) | (unsigned long long)cell[0]);
            }
            int nd[RUN];
            const i128 carry = run_carry(u, j0, n, lgM, nd);
#pragma unroll
            for (int x = 0; x < RUN; ++x) dig[lr * RUN + x] = nd[x];
            cout[2 * lr] = (long long)(unsigned long long)carry;
            cout[2 * lr + 1] = (long long)(carry >> 64);
        }
        res_sync<CL>();  // carries and the pending top are visible to the next fix-up
    }

    // epilogue: digits, pending carries and the slot state back to global memory
    for (int lr = tid; lr < R::RUNS; lr += NT) {
        const int q = lr / R::RPR, r = (int)c * R::G0 + (lr % R::RPR) * RUN;
        const long long j0 = r + (long long)q * F1;
        const int* d = dig + lr * RUN;
        int4* dp = reinterpret_cast<int4*>(sl.digits + j0);
        dp[0] = make_int4(d[0], d[1], d[2], d[3]);
        dp[1] = make_int4(d[4], d[5], d[6], d[7]);
        sl.carries[2 * (j0 / RUN)] = cout[2 * lr];
        sl.carries[2 * (j0 / RUN) + 1] = cout[2 * lr + 1];
    }
    emax = warp_max_u64(emax);
    if ((tid & 31) == 0 && emax > 0) atomicMax(&st->maxerr_bits, err_bits(emax));
    if (flags) atomicOr(&st->flags, flags);
    if (c == 0 && tid == 0) {
        st->top = misc[0];
        st->pend_lo = misc[1];
        st->pend_hi = misc[2];
        st->step = step0 + nsq;
    }
}

}  // namespace pg

#endif

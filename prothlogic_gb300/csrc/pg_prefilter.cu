// pg_prefilter.cu -- trial-division pre-filter of Proth candidates on the GPU.
//
// For a list of candidates N_i = k_i 2^{n_i} + 1 it finds, for each, the
// smallest odd prime p < bound that divides N_i (0 when there is none).  This is
// the per-candidate counterpart of the reference's sieve strike
// (prothlogic4.2/gpu_engine.cu:290-320, check_proth_candidates_kernel with the
// 64-bit Montgomery gpu_pow_mod at :246-284), which strikes k in a range for one
// fixed n; a serving queue holds independent (k, n) pairs instead.  Unlike the
// reference's window sieve (:143-149, where only the first ceil(P/256) small
// primes ever strike because blockIdx.x is used as the prime index), every base
// prime strikes every segment here, and k is reduced mod p before it is
// compared (the reference's sparse kernel compares raw k, :397).
//
//   primes:  segmented sieve of Eratosthenes over odd numbers, one shared-memory
//            bitmap per CTA, base primes < 2^16 from the host, survivors
//            compacted with warp ballots;
//   test:    one thread per prime, walking the live candidates sorted by n:
//            2^{n_i} mod p is advanced by 2^{n_i - n_{i-1}} (small exponents),
//            p | N_i  <=>  k_i 2^{n_i} = -1 (mod p), in 32-bit Montgomery form.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/prothgpu.h"

namespace pgpf {

constexpr int kSieveThreads = 256;
constexpr int kSubBits = 1 << 18;              // odd numbers per CTA (32 KB of shared memory)
constexpr int kSubWords = kSubBits / 32;
constexpr unsigned long long kSegNumbers = 1ull << 27;  // numbers per launch (2^26 odd)

// ---- 32-bit Montgomery arithmetic, R = 2^32 ----
struct Mont {
    uint32_t p, pinv;  // pinv = -p^{-1} mod 2^32
    uint32_t r2;       // R^2 mod p
};

// t < p^2 < 2^64.  (t + m p) / 2^32 is formed from the high halves plus the
// carry of the low halves (which sum to 0 mod 2^32), so nothing overflows
// even for p close to 2^32.
__device__ __forceinline__ uint32_t redc(uint64_t t, uint32_t p, uint32_t pinv) {
    const uint32_t m = (uint32_t)t * pinv;
    const uint64_t mp = (uint64_t)m * p;
    const uint64_t u = (t >> 32) + (mp >> 32) + ((uint32_t)t != 0u ? 1u : 0u);  // < 2p
    return u >= p ? (uint32_t)(u - p) : (uint32_t)u;
}
__device__ __forceinline__ uint32_t mmul(uint32_t a, uint32_t b, const Mont& M) {
    return redc((uint64_t)a * b, M.p, M.pinv);
}
__device__ __forceinline__ Mont make_mont(uint32_t p) {
    Mont M;
    M.p = p;
    uint32_t inv = p;  // Newton iteration for p^{-1} mod 2^32 (p odd)
    for (int i = 0; i < 5; ++i) inv *= 2u - p * inv;
    M.pinv = 0u - inv;
    const uint64_t r = (((uint64_t)1) << 32) % p;
    M.r2 = (uint32_t)((r * r) % p);
    return M;
}
// 2^e in Montgomery form (2^e * R mod p)
__device__ __forceinline__ uint32_t mpow2(uint32_t e, const Mont& M) {
    uint32_t two = mmul(2u, M.r2, M);
    uint32_t acc = mmul(1u, M.r2, M);
    while (e) {
        if (e & 1u) acc = mmul(acc, two, M);
        two = mmul(two, two, M);
        e >>= 1;
    }
    return acc;
}

// Segment [lo, lo + 2*bits): bit b <-> odd number lo + 2b + 1.  Composite bits
// are set by the base primes (q^2 <= number); zero bits are primes (except 1).
__global__ void __launch_bounds__(kSieveThreads) k_sieve(unsigned long long lo, const uint32_t* __restrict__ base,
                                                         int nbase, unsigned long long limit,
                                                         uint32_t* __restrict__ out, unsigned* __restrict__ count,
                                                         unsigned cap) {
    __shared__ uint32_t bits[kSubWords];
    const unsigned long long c_lo = lo + 2ull * kSubBits * blockIdx.x;  // even
    for (int w = threadIdx.x; w < kSubWords; w += blockDim.x) bits[w] = 0u;
    __syncthreads();
    const unsigned long long c_hi = c_lo + 2ull * kSubBits;  // numbers < c_hi
    for (int i = threadIdx.x; i < nbase; i += blockDim.x) {
        const unsigned long long q = base[i];
        if (q * q >= c_hi) break;  // base is ascending
        // first odd multiple of q that is >= max(q^2, c_lo + 1)
        unsigned long long m = q * q;
        if (m < c_lo + 1) {
            m = ((c_lo + 1 + q - 1) / q) * q;
            if (!(m & 1ull)) m += q;
        }
        for (; m < c_hi; m += 2 * q) {
            const unsigned b = (unsigned)((m - c_lo - 1) >> 1);
            atomicOr(&bits[b >> 5], 1u << (b & 31));
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (int w = threadIdx.x; w < kSubWords; w += blockDim.x) {
        uint32_t free_bits = ~bits[w];
        // drop 1 and numbers beyond the limit
        const unsigned long long first = c_lo + 1 + 64ull * w;
        if (first == 1) free_bits &= ~1u;
        if (first + 62 >= limit) {
            for (int t = 0; t < 32; ++t)
                if (first + 2ull * t >= limit) free_bits &= ~(1u << t);
        }
        const int cnt = __popc(free_bits);
        // warp-aggregated reservation
        int incl = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        unsigned basei = 0;
        if (lane == 31 && total) basei = atomicAdd(count, (unsigned)total);
        basei = __shfl_sync(0xffffffffu, basei, 31);
        unsigned pos = basei + (unsigned)(incl - cnt);
        while (free_bits) {
            const int t = __ffs(free_bits) - 1;
            free_bits &= free_bits - 1;
            if (pos < cap) out[pos] = (uint32_t)(first + 2ull * t);
            ++pos;
        }
    }
}

// One thread per prime: the live candidates (sorted by n) are tested in order.
__global__ void k_test(const uint32_t* __restrict__ primes, unsigned nprimes, const unsigned long long* __restrict__ ks,
                       const uint32_t* __restrict__ ns, const int* __restrict__ live, int nlive,
                       unsigned long long* __restrict__ factor) {
    const unsigned idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nprimes) return;
    const uint32_t p = primes[idx];
    if (p < 3) return;
    const Mont M = make_mont(p);
    uint32_t prev_n = 0;
    uint32_t pw = mmul(1u, M.r2, M);  // 2^0 in Montgomery form
    const uint32_t minus1 = p - 1;
    for (int j = 0; j < nlive; ++j) {
        const int i = live[j];
        const uint32_t n = ns[i];
        pw = mmul(pw, mpow2(n - prev_n, M), M);  // 2^n R
        prev_n = n;
        const unsigned long long k = ks[i];
        const uint32_t km = (uint32_t)(k % p);
        // k 2^n mod p: mmul(km, 2^n R) = km 2^n (normal form)
        const uint32_t v = mmul(km, pw, M);
        if (v == minus1) atomicMin(&factor[i], (unsigned long long)p);
    }
}

}  // namespace pgpf

using namespace pgpf;

extern "C" int pg_prefilter(const uint64_t* ks, const uint32_t* ns, size_t count, uint64_t bound,
                            uint64_t* smallest_factor) {
    if ((!ks || !ns || !smallest_factor) && count) return PG_EINVAL;
    if (bound > (1ull << 32) || bound < 3) return PG_EINVAL;
    for (size_t i = 0; i < count; ++i) smallest_factor[i] = 0;
    if (!count) return PG_OK;
    // base primes < 2^16 (host sieve)
    std::vector<uint32_t> base;
    {
        const unsigned LIM = 1u << 16;
        std::vector<char> comp(LIM, 0);
        for (unsigned i = 3; i < LIM; i += 2) {
            if (comp[i]) continue;
            base.push_back(i);
            for (unsigned long long j = (unsigned long long)i * i; j < LIM; j += 2ull * i) comp[j] = 1;
        }
    }
    // candidates sorted by n: thread-local powers advance by small exponent steps
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int a, int b) { return ns[a] < ns[b]; });

    uint32_t* d_base = nullptr;
    uint32_t* d_primes = nullptr;
    unsigned* d_count = nullptr;
    unsigned long long* d_ks = nullptr;
    uint32_t* d_ns = nullptr;
    int* d_live = nullptr;
    unsigned long long* d_factor = nullptr;
    const unsigned cap = (unsigned)(kSegNumbers / 8);  // > pi(2^27) / 2 primes per segment
    cudaStream_t st = nullptr;
    int rc = PG_OK;
    auto ck = [&](cudaError_t e) {
        if (e != cudaSuccess && rc == PG_OK) rc = PG_ECUDA;
        return e == cudaSuccess;
    };
    ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    ck(cudaMalloc(&d_base, base.size() * sizeof(uint32_t)));
    ck(cudaMalloc(&d_primes, (size_t)cap * sizeof(uint32_t)));
    ck(cudaMalloc(&d_count, sizeof(unsigned)));
    ck(cudaMalloc(&d_ks, count * sizeof(unsigned long long)));
    ck(cudaMalloc(&d_ns, count * sizeof(uint32_t)));
    ck(cudaMalloc(&d_live, count * sizeof(int)));
    ck(cudaMalloc(&d_factor, count * sizeof(unsigned long long)));
    if (rc == PG_OK) {
        std::vector<unsigned long long> init(count, ~0ull);
        ck(cudaMemcpy(d_base, base.data(), base.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
        ck(cudaMemcpy(d_ks, ks, count * sizeof(unsigned long long), cudaMemcpyHostToDevice));
        ck(cudaMemcpy(d_ns, ns, count * sizeof(uint32_t), cudaMemcpyHostToDevice));
        ck(cudaMemcpy(d_factor, init.data(), count * sizeof(unsigned long long), cudaMemcpyHostToDevice));
    }
    std::vector<int> live(order);
    std::vector<unsigned long long> fac(count, ~0ull);
    for (unsigned long long lo = 0; lo < bound && rc == PG_OK && !live.empty(); lo += kSegNumbers) {
        ck(cudaMemcpyAsync(d_live, live.data(), live.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        ck(cudaMemsetAsync(d_count, 0, sizeof(unsigned), st));
        const unsigned long long limit = std::min<unsigned long long>(bound, lo + kSegNumbers);
        const int ctas = (int)((std::min<unsigned long long>(kSegNumbers, limit - lo) + 2ull * kSubBits - 1) /
                               (2ull * kSubBits));
        k_sieve<<<ctas, kSieveThreads, 0, st>>>(lo, d_base, (int)base.size(), limit, d_primes, d_count, cap);
        ck(cudaGetLastError());
        unsigned np = 0;
        ck(cudaMemcpyAsync(&np, d_count, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        ck(cudaStreamSynchronize(st));
        np = std::min(np, cap);
        if (np) {
            k_test<<<(np + 255) / 256, 256, 0, st>>>(d_primes, np, d_ks, d_ns, d_live, (int)live.size(), d_factor);
            ck(cudaGetLastError());
        }
        ck(cudaMemcpyAsync(fac.data(), d_factor, count * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        ck(cudaStreamSynchronize(st));
        // candidates with a factor in this segment leave the live list (factors
        // in later segments are larger)
        std::vector<int> next;
        next.reserve(live.size());
        for (int i : live)
            if (fac[i] == ~0ull) next.push_back(i);
        live.swap(next);
    }
    for (size_t i = 0; i < count; ++i) smallest_factor[i] = fac[i] == ~0ull ? 0 : fac[i];
    cudaFree(d_base);
    cudaFree(d_primes);
    cudaFree(d_count);
    cudaFree(d_ks);
    cudaFree(d_ns);
    cudaFree(d_live);
    cudaFree(d_factor);
    if (st) cudaStreamDestroy(st);
    return rc;
}

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
//
// Three entry points share these pieces: pg_prefilter (allocates, sieves and
// tests segment by segment, synchronous), pg_prefilter_noalloc (fixed scratch,
// sieve and test fused in one kernel, queued on the caller's stream) and the
// pg_sieve handle (every prime below the bound sieved once into device memory;
// each strike queues only the trial division, staged by prime size).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
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

// t < p 2^32 (a product a b with a < 2^32 and b < p).  (t + m p) / 2^32 < 2p
// is formed from the high halves plus the carry of the low halves (which sum to
// 0 mod 2^32), so nothing overflows even for p close to 2^32.
__device__ __forceinline__ uint32_t redc(uint64_t t, uint32_t p, uint32_t pinv) {
    const uint32_t m = (uint32_t)t * pinv;
    const uint64_t mp = (uint64_t)m * p;
    const uint64_t u = (t >> 32) + (mp >> 32) + ((uint32_t)t != 0u ? 1u : 0u);  // < 2p
    return u >= p ? (uint32_t)(u - p) : (uint32_t)u;
}
__device__ __forceinline__ uint32_t mmul(uint32_t a, uint32_t b, const Mont& M) {
    return redc((uint64_t)a * b, M.p, M.pinv);
}
__device__ __forceinline__ uint32_t mont_pinv(uint32_t p) {
    uint32_t inv = p;  // Newton iteration for p^{-1} mod 2^32 (p odd): 3, 6, 12, 24, 48 bits
    for (int i = 0; i < 4; ++i) inv *= 2u - p * inv;
    return 0u - inv;
}
__device__ __forceinline__ Mont make_mont(uint32_t p) {
    Mont M;
    M.p = p;
    M.pinv = mont_pinv(p);
    const uint64_t r = (((uint64_t)1) << 32) % p;
    M.r2 = (uint32_t)((r * r) % p);
    return M;
}
// 2x mod p for x < p, without leaving 32 bits
__device__ __forceinline__ uint32_t mdbl(uint32_t x, uint32_t p) { return x >= p - x ? x - (p - x) : x + x; }
__device__ __forceinline__ uint32_t madd(uint32_t x, uint32_t y, uint32_t p) { return x >= p - y ? x - (p - y) : x + y; }
// 2^e R mod p from one = R mod p: left to right, a squaring per bit below the
// top one and a doubling (not a multiplication) per set bit.
__device__ __forceinline__ uint32_t mpow2(uint32_t e, uint32_t one, const Mont& M) {
    if (e == 0u) return one;
    uint32_t x = mdbl(one, M.p);
    for (int b = 30 - __clz(e); b >= 0; --b) {
        x = mmul(x, x, M);
        if ((e >> b) & 1u) x = mdbl(x, M.p);
    }
    return x;
}
// k 2^n mod p from pw = 2^n R mod p, without dividing k by p: with k = kh 2^32 + kl,
// REDC(kl pw) = kl 2^n and REDC(kh REDC(pw R^2)) = kh 2^32 2^n.
__device__ __forceinline__ uint32_t k_times(unsigned long long k, uint32_t pw, const Mont& M) {
    uint32_t v = mmul((uint32_t)k, pw, M);
    const uint32_t kh = (uint32_t)(k >> 32);
    if (kh) v = madd(v, mmul(kh, mmul(pw, M.r2, M), M), M.p);
    return v;
}

// Odd numbers of the window [c_lo, c_lo + 2^19) (c_lo even) into shared memory:
// bit b <-> c_lo + 2b + 1, set = composite (struck by a base prime q with
// q^2 <= number).  Every thread of the CTA calls it.
__device__ __forceinline__ void sieve_window(unsigned long long c_lo, const uint32_t* __restrict__ base, int nbase,
                                             uint32_t* bits) {
    for (int w = threadIdx.x; w < kSubWords; w += blockDim.x) bits[w] = 0u;
    __syncthreads();
    const unsigned long long c_hi = c_lo + 2ull * kSubBits;  // numbers < c_hi
    for (int i = threadIdx.x; i < nbase; i += blockDim.x) {
        const unsigned long long q = base[i];
        if (q * q >= c_hi) break;  // base is ascending
        unsigned long long m = q * q;  // first odd multiple of q that is >= max(q^2, c_lo + 1)
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
}
// Primes of word w of a sieved window (bit t <-> c_lo + 64 w + 2t + 1), 1 and
// numbers >= limit dropped.
__device__ __forceinline__ uint32_t window_primes(const uint32_t* bits, int w, unsigned long long c_lo,
                                                  unsigned long long limit) {
    uint32_t free_bits = ~bits[w];
    const unsigned long long first = c_lo + 1 + 64ull * w;
    if (first == 1) free_bits &= ~1u;
    if (first + 62 >= limit) {
        for (int t = 0; t < 32; ++t)
            if (first + 2ull * t >= limit) free_bits &= ~(1u << t);
    }
    return free_bits;
}

// Segment [lo, lo + 2*bits): bit b <-> odd number lo + 2b + 1.  Composite bits
// are set by the base primes (q^2 <= number); zero bits are primes (except 1).
// `live` (optional): the number of candidates still without a factor; at 0 the
// launch has nothing to sieve for and returns at once.
__global__ void __launch_bounds__(kSieveThreads) k_sieve(unsigned long long lo, const uint32_t* __restrict__ base,
                                                         int nbase, unsigned long long limit,
                                                         uint32_t* __restrict__ out, unsigned* __restrict__ count,
                                                         unsigned cap, const uint32_t* __restrict__ live) {
    __shared__ uint32_t bits[kSubWords];
    if (live && *live == 0u) return;
    const unsigned long long c_lo = lo + 2ull * kSubBits * blockIdx.x;  // even
    sieve_window(c_lo, base, nbase, bits);
    const int lane = threadIdx.x & 31;
    for (int w = threadIdx.x; w < kSubWords; w += blockDim.x) {
        uint32_t free_bits = window_primes(bits, w, c_lo, limit);
        const unsigned long long first = c_lo + 1 + 64ull * w;
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
    const uint32_t one = mmul(1u, M.r2, M);  // R mod p
    uint32_t prev_n = 0;
    uint32_t pw = one;  // 2^prev_n R
    for (int j = 0; j < nlive; ++j) {
        const int i = live[j];
        const uint32_t n = ns[i];
        pw = mmul(pw, mpow2(n - prev_n, one, M), M);  // 2^n R
        prev_n = n;
        if (k_times(ks[i], pw, M) == p - 1) atomicMin(&factor[i], (unsigned long long)p);
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
        k_sieve<<<ctas, kSieveThreads, 0, st>>>(lo, d_base, (int)base.size(), limit, d_primes, d_count, cap, nullptr);
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

// ---- fixed-scratch variant: pg_prefilter_noalloc ----
//
// Some callers cannot allocate device memory at all: a host runtime that owns
// the whole device budget through its own pool and forbids any other
// allocation in the process, or a latency-bound serving loop in which
// cudaMalloc/cudaFree would synchronise the device and stall the work queued on
// other streams.  They hand in device buffers for the candidates and for the
// result; everything else the pre-filter needs (the base primes, two
// live-candidate lists and their counters) lives in one file-scope device array
// of fixed size.  Every GPU on which this library is
// loaded holds that array until the process exits.
//
// One fused kernel does the work of pg_prefilter's sieve and test: each CTA
// sieves its own window of numbers in shared memory (as k_sieve does) and tests
// the window's primes against the live candidates right there, walking them in n
// order (as k_test does: the candidates are ranked by n on the device once per
// call), so no prime list is ever written to memory and a bound of 2^32 takes 32
// launches.  The live list is compacted on the device in order after each
// launch, so one call is a fixed sequence of launches on the caller's stream
// with no host synchronisation; once every candidate has a factor the remaining
// launches return at once.
namespace pgpf {

constexpr unsigned long long kNaSegNumbers = 1ull << 27;  // numbers per launch: 256 windows of 2^19
constexpr unsigned kNaBaseCap = 8192;                      // 6,541 odd primes < 2^16
constexpr unsigned kNaMaxCount = PG_PREFILTER_NOALLOC_MAX_COUNT;
// Word offsets: counters (unused, live count of list 0, of list 1), base primes,
// live list 0, live list 1.
constexpr size_t kNaOffBase = 64;
constexpr size_t kNaOffLive0 = kNaOffBase + kNaBaseCap;
constexpr size_t kNaOffLive1 = kNaOffLive0 + kNaMaxCount;
constexpr size_t kNaWords = kNaOffLive1 + kNaMaxCount;
constexpr int kNaRankThreads = 1024;
constexpr int kNaCompactThreads = 1024;

// Live list 0 = all candidates ordered by (n, index): candidate i goes to its
// rank, the number of candidates before it in that order (count^2 comparisons,
// under a millisecond at the 65,536 cap).  Also clears the results and counters.
__global__ void __launch_bounds__(kNaRankThreads) k_na_seed(const uint32_t* __restrict__ ns, unsigned count,
                                                            uint32_t* __restrict__ ctrl, uint32_t* __restrict__ live0,
                                                            unsigned long long* __restrict__ factor) {
    __shared__ uint32_t tile[kNaRankThreads];
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t ni = i < count ? ns[i] : 0u;
    unsigned rank = 0;
    for (unsigned base = 0; base < count; base += kNaRankThreads) {
        __syncthreads();
        if (base + threadIdx.x < count) tile[threadIdx.x] = ns[base + threadIdx.x];
        __syncthreads();
        const unsigned m = min((unsigned)kNaRankThreads, count - base);
        for (unsigned t = 0; t < m; ++t) {
            const uint32_t nj = tile[t];
            rank += (nj < ni || (nj == ni && base + t < i)) ? 1u : 0u;
        }
    }
    if (i < count) {
        live0[rank] = i;
        factor[i] = ~0ull;
    }
    if (i == 0) {
        ctrl[0] = 0u;
        ctrl[1] = count;
        ctrl[2] = 0u;
    }
}

// CTA b: the window [lo + b 2^19, lo + (b+1) 2^19) of numbers below `limit`.
// Sieve its odd numbers with the base primes (bit set = composite), then each
// thread takes the primes of its bitmap words and walks the live candidates in
// n order: 2^{n_i} mod p advances by 2^{n_i - n_{i-1}}, and p | k_i 2^{n_i} + 1
// iff k_i 2^{n_i} = -1 (mod p).
__global__ void __launch_bounds__(kSieveThreads) k_na_sieve_test(unsigned long long lo,
                                                                 const uint32_t* __restrict__ base, int nbase,
                                                                 unsigned long long limit,
                                                                 const unsigned long long* __restrict__ ks,
                                                                 const uint32_t* __restrict__ ns,
                                                                 const uint32_t* __restrict__ live,
                                                                 const uint32_t* __restrict__ nlive,
                                                                 unsigned long long* __restrict__ factor) {
    __shared__ uint32_t bits[kSubWords];
    const unsigned nl = *nlive;
    const unsigned long long c_lo = lo + 2ull * kSubBits * blockIdx.x;  // even
    if (nl == 0u || c_lo >= limit) return;                               // the same in every thread
    sieve_window(c_lo, base, nbase, bits);
    for (int w = threadIdx.x; w < kSubWords; w += blockDim.x) {
        uint32_t free_bits = window_primes(bits, w, c_lo, limit);
        const unsigned long long first = c_lo + 1 + 64ull * w;
        while (free_bits) {
            const int t = __ffs(free_bits) - 1;
            free_bits &= free_bits - 1;
            const uint32_t p = (uint32_t)(first + 2ull * t);
            const Mont M = make_mont(p);
            const uint32_t one = mmul(1u, M.r2, M);
            uint32_t prev_n = 0;
            uint32_t pw = one;
            for (unsigned j = 0; j < nl; ++j) {
                const uint32_t i = live[j];
                const uint32_t n = ns[i];
                pw = mmul(pw, mpow2(n - prev_n, one, M), M);
                prev_n = n;
                if (k_times(ks[i], pw, M) == p - 1) atomicMin(&factor[i], (unsigned long long)p);
            }
        }
    }
}

// Candidates still without a factor move to the other live list, in order: one
// CTA, each thread a contiguous share of the list, a block scan of the counts.
__global__ void __launch_bounds__(kNaCompactThreads) k_na_compact(const uint32_t* __restrict__ live,
                                                                  const uint32_t* __restrict__ nlive,
                                                                  const unsigned long long* __restrict__ factor,
                                                                  uint32_t* __restrict__ next,
                                                                  uint32_t* __restrict__ nnext) {
    __shared__ unsigned warp_sum[kNaCompactThreads / 32];
    const unsigned nl = *nlive;
    const unsigned t = threadIdx.x, lane = t & 31, w = t >> 5;
    const unsigned per = (nl + kNaCompactThreads - 1) / kNaCompactThreads;
    const unsigned j0 = min(nl, t * per), j1 = min(nl, j0 + per);
    unsigned mine = 0;
    for (unsigned j = j0; j < j1; ++j) mine += factor[live[j]] == ~0ull ? 1u : 0u;
    unsigned incl = mine;  // inclusive scan within the warp
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (unsigned)o) incl += v;
    }
    if (lane == 31) warp_sum[w] = incl;
    __syncthreads();
    if (w == 0) {  // scan of the warp totals
        unsigned v = lane < kNaCompactThreads / 32 ? warp_sum[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= (unsigned)o) v += u;
        }
        if (lane < kNaCompactThreads / 32) warp_sum[lane] = v;
    }
    __syncthreads();
    unsigned pos = (w ? warp_sum[w - 1] : 0u) + incl - mine;
    for (unsigned j = j0; j < j1; ++j) {
        const uint32_t i = live[j];
        if (factor[i] == ~0ull) next[pos++] = i;
    }
    if (t == kNaCompactThreads - 1) *nnext = pos;
}

__global__ void k_na_finish(unsigned long long* __restrict__ factor, unsigned count) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count && factor[i] == ~0ull) factor[i] = 0ull;
}

}  // namespace pgpf

// The scratch.  In host code this name only stands for the device symbol; its
// device address comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) uint32_t g_prefilter_scratch[pgpf::kNaWords];
static_assert(sizeof(g_prefilter_scratch) == PG_PREFILTER_NOALLOC_SCRATCH_BYTES, "scratch size in the header");

namespace {

constexpr int kNaMaxDevices = 64;
std::mutex g_na_mu;
uint32_t* g_na_dev[kNaMaxDevices];        // scratch address per device, null until set up
uint32_t g_na_base[pgpf::kNaBaseCap];    // odd primes < 2^16, ascending
unsigned g_na_nbase = 0;
unsigned char g_na_comp[1u << 16];

// First call on a device: find the scratch's device address and write the base
// primes into it (they never change afterwards).  Runs with that device current.
int na_setup(uint32_t** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return PG_ECUDA;
    if (dev < 0 || dev >= kNaMaxDevices) return PG_ENODEV;
    std::lock_guard<std::mutex> lock(g_na_mu);
    if (!g_na_nbase) {
        for (unsigned i = 3; i < (1u << 16); i += 2) {
            if (g_na_comp[i]) continue;
            g_na_base[g_na_nbase++] = i;
            for (unsigned j = i * i; j < (1u << 16); j += 2 * i) g_na_comp[j] = 1;
        }
    }
    if (!g_na_dev[dev]) {
        void* ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_prefilter_scratch) != cudaSuccess || !ptr) return PG_ECUDA;
        uint32_t* s = static_cast<uint32_t*>(ptr);
        if (cudaMemcpy(s + pgpf::kNaOffBase, g_na_base, g_na_nbase * sizeof(uint32_t), cudaMemcpyHostToDevice) !=
            cudaSuccess)
            return PG_ECUDA;
        g_na_dev[dev] = s;
    }
    *out = g_na_dev[dev];
    return PG_OK;
}

}  // namespace

extern "C" int pg_prefilter_noalloc(const uint64_t* d_ks, const uint32_t* d_ns, size_t count, uint64_t bound,
                                    uint64_t* d_smallest_factor, void* stream) {
    if (count > PG_PREFILTER_NOALLOC_MAX_COUNT) return PG_ETOOBIG;
    if ((!d_ks || !d_ns || !d_smallest_factor) && count) return PG_EINVAL;
    if (bound > (1ull << 32) || bound < 3) return PG_EINVAL;
    if (!count) return PG_OK;
    uint32_t* s = nullptr;
    const int rc = na_setup(&s);
    if (rc != PG_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t* ctrl = s;
    uint32_t* live[2] = {s + kNaOffLive0, s + kNaOffLive1};
    const unsigned long long* ks = reinterpret_cast<const unsigned long long*>(d_ks);
    unsigned long long* fac = reinterpret_cast<unsigned long long*>(d_smallest_factor);
    const unsigned cnt = (unsigned)count;
    const unsigned cblocks = (cnt + 255) / 256;
    k_na_seed<<<(cnt + kNaRankThreads - 1) / kNaRankThreads, kNaRankThreads, 0, st>>>(d_ns, cnt, ctrl, live[0],
                                                                                        fac);
    int cur = 0;
    for (unsigned long long lo = 0; lo < bound; lo += kNaSegNumbers) {
        const unsigned long long limit = std::min<unsigned long long>(bound, lo + kNaSegNumbers);
        const int ctas = (int)((limit - lo + 2ull * kSubBits - 1) / (2ull * kSubBits));
        k_na_sieve_test<<<ctas, kSieveThreads, 0, st>>>(lo, s + kNaOffBase, (int)g_na_nbase, limit, ks, d_ns,
                                                        live[cur], ctrl + 1 + cur, fac);
        k_na_compact<<<1, kNaCompactThreads, 0, st>>>(live[cur], ctrl + 1 + cur, fac, live[cur ^ 1],
                                                      ctrl + 1 + (cur ^ 1));
        cur ^= 1;
    }
    k_na_finish<<<cblocks, 256, 0, st>>>(fac, cnt);
    return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}

// ---- device-resident sieve: pg_sieve_create / pg_sieve_strike ----
//
// A serving loop pre-filters a few candidates at a time, many times a second.
// Sieving every prime below the bound again for each call costs far more than
// trial division of a few candidates, so a pg_sieve keeps the primes below its
// bound in device memory, sieved once when it is created: ascending, each with
// R^2 mod p (8 bytes a prime; 1.6 GB below 2^32).  A strike is then only the
// trial division, queued on the caller's stream with no host synchronisation
// and no allocation, in stages of growing primes (2^10, 2^13, ..., 2^31): most
// candidates fall to the small primes (about 84 % to primes below 2^10 for
// random odd k), and the ordered compaction after each stage leaves the large
// primes only the survivors.  Each thread tests two primes of the table against
// the stage's live candidates, in n order, the candidates staged in shared
// memory; thread blocks are short, so batch kernels queued at a higher stream
// priority get SMs between them.
namespace pgpf {

constexpr int kTabThreads = 256;
constexpr int kTabPerThread = 2;
constexpr int kTabChunk = 1024;  // live candidates staged in shared memory at a time
constexpr unsigned long long kTabWindow = 2ull * kSubBits;  // numbers per window (2^19)
constexpr size_t kTabOffLive0 = 64;                         // scratch words: counters, live list 0, live list 1

// Block-wide exclusive scan of one value per thread (kSieveThreads threads).
__device__ __forceinline__ unsigned block_excl_scan(unsigned v, unsigned* warp_sum, unsigned* total) {
    const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (unsigned)o) incl += u;
    }
    if (lane == 31) warp_sum[w] = incl;
    __syncthreads();
    if (w == 0) {
        unsigned x = lane < kSieveThreads / 32 ? warp_sum[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned u = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (unsigned)o) x += u;
        }
        if (lane < kSieveThreads / 32) warp_sum[lane] = x;
    }
    __syncthreads();
    const unsigned r = (w ? warp_sum[w - 1] : 0u) + incl - v;
    if (total) *total = warp_sum[kSieveThreads / 32 - 1];
    return r;
}

// Window b = [b 2^19, (b+1) 2^19): its number of odd primes below `limit`.
__global__ void __launch_bounds__(kSieveThreads) k_tab_count(const uint32_t* __restrict__ base, int nbase,
                                                             unsigned long long limit, uint32_t* __restrict__ counts) {
    __shared__ uint32_t bits[kSubWords];
    __shared__ unsigned warp_sum[kSieveThreads / 32];
    const unsigned long long c_lo = kTabWindow * blockIdx.x;
    sieve_window(c_lo, base, nbase, bits);
    unsigned c = 0;
    for (int w = threadIdx.x; w < kSubWords; w += blockDim.x) c += __popc(window_primes(bits, w, c_lo, limit));
    unsigned total = 0;
    block_excl_scan(c, warp_sum, &total);
    if (threadIdx.x == 0) counts[blockIdx.x] = total;
}

// Window b's primes in ascending order from table[offsets[b]], each with R^2 mod p:
// each thread owns a contiguous run of bitmap words.
__global__ void __launch_bounds__(kSieveThreads) k_tab_fill(const uint32_t* __restrict__ base, int nbase,
                                                            unsigned long long limit,
                                                            const unsigned long long* __restrict__ offsets,
                                                            uint2* __restrict__ table) {
    __shared__ uint32_t bits[kSubWords];
    __shared__ unsigned warp_sum[kSieveThreads / 32];
    const unsigned long long c_lo = kTabWindow * blockIdx.x;
    sieve_window(c_lo, base, nbase, bits);
    constexpr int kPer = kSubWords / kSieveThreads;
    const int w0 = threadIdx.x * kPer;
    unsigned c = 0;
    for (int w = w0; w < w0 + kPer; ++w) c += __popc(window_primes(bits, w, c_lo, limit));
    unsigned long long pos = offsets[blockIdx.x] + block_excl_scan(c, warp_sum, nullptr);
    for (int w = w0; w < w0 + kPer; ++w) {
        uint32_t free_bits = window_primes(bits, w, c_lo, limit);
        const unsigned long long first = c_lo + 1 + 64ull * w;
        while (free_bits) {
            const int t = __ffs(free_bits) - 1;
            free_bits &= free_bits - 1;
            const uint32_t p = (uint32_t)(first + 2ull * t);
            const unsigned long long r = (1ull << 32) % p;
            table[pos++] = make_uint2(p, (uint32_t)((r * r) % p));
        }
    }
}

// Primes table[first, last) against the live candidates (n order).  Thread t of
// block b takes the primes first + (b kTabPerThread + q) kTabThreads + t, q <
// kTabPerThread, and walks both at once (two independent multiplication chains).
__global__ void __launch_bounds__(kTabThreads) k_tab_test(const uint2* __restrict__ table, unsigned first,
                                                          unsigned last, const unsigned long long* __restrict__ ks,
                                                          const uint32_t* __restrict__ ns,
                                                          const uint32_t* __restrict__ live,
                                                          const uint32_t* __restrict__ nlive,
                                                          unsigned long long* __restrict__ factor) {
    __shared__ unsigned long long s_k[kTabChunk];
    __shared__ uint32_t s_n[kTabChunk];
    __shared__ uint32_t s_i[kTabChunk];
    const unsigned nl = *nlive;
    if (nl == 0u) return;  // the same in every thread
    Mont M[kTabPerThread];
    uint32_t one[kTabPerThread], pw[kTabPerThread];
    bool valid[kTabPerThread];
    for (int q = 0; q < kTabPerThread; ++q) {
        const unsigned long long idx =
            first + ((unsigned long long)blockIdx.x * kTabPerThread + q) * kTabThreads + threadIdx.x;
        valid[q] = idx < last;
        const uint2 e = valid[q] ? table[idx] : make_uint2(3u, 1u);  // 2^64 mod 3 = 1
        M[q].p = e.x;
        M[q].pinv = mont_pinv(e.x);
        M[q].r2 = e.y;
        one[q] = mmul(1u, e.y, M[q]);
        pw[q] = one[q];
    }
    uint32_t prev_n = 0;
    for (unsigned c0 = 0; c0 < nl; c0 += kTabChunk) {
        const unsigned m = min((unsigned)kTabChunk, nl - c0);
        __syncthreads();
        for (unsigned j = threadIdx.x; j < m; j += kTabThreads) {
            const uint32_t i = live[c0 + j];
            s_i[j] = i;
            s_n[j] = ns[i];
            s_k[j] = ks[i];
        }
        __syncthreads();
        for (unsigned j = 0; j < m; ++j) {
            const uint32_t n = s_n[j];
            const unsigned long long k = s_k[j];
            const uint32_t d = n - prev_n;
            prev_n = n;
#pragma unroll
            for (int q = 0; q < kTabPerThread; ++q) {
                pw[q] = mmul(pw[q], mpow2(d, one[q], M[q]), M[q]);
                if (valid[q] && k_times(k, pw[q], M[q]) == M[q].p - 1)
                    atomicMin(&factor[s_i[j]], (unsigned long long)M[q].p);
            }
        }
    }
}

}  // namespace pgpf

struct pg_sieve {
    int device = 0;
    uint64_t bound = 0;
    size_t max_count = 0;
    uint2* table = nullptr;
    unsigned long long nprimes = 0;
    std::vector<unsigned long long> stage_end;  // table index at which each stage ends (ascending)
    uint32_t* scratch = nullptr;                 // counters, two live lists of max_count
};

namespace {

void sieve_free(pg_sieve* s) {
    if (!s) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    cudaFree(s->table);
    cudaFree(s->scratch);
    cudaSetDevice(prev);
    delete s;
}

}  // namespace

extern "C" int pg_sieve_create(uint64_t bound, size_t max_count, pg_sieve** out) {
    if (!out) return PG_EINVAL;
    *out = nullptr;
    if (bound > (1ull << 32) || bound < 3) return PG_EINVAL;
    if (max_count == 0) return PG_EINVAL;
    if (max_count > PG_SIEVE_MAX_COUNT) return PG_ETOOBIG;
    pg_sieve* s = new pg_sieve();
    s->bound = bound;
    s->max_count = max_count;
    if (cudaGetDevice(&s->device) != cudaSuccess) {
        delete s;
        return PG_ECUDA;
    }
    // odd primes < 2^19 on the host: the base primes (< 2^16) and the stage
    // boundaries below one window
    const unsigned kSmall = 1u << 19;
    std::vector<char> comp(kSmall, 0);
    std::vector<uint32_t> base;
    std::vector<unsigned> below(kSmall + 1, 0);  // odd primes < x
    for (unsigned i = 3; i < kSmall; i += 2) {
        if (comp[i]) continue;
        if (i < (1u << 16)) base.push_back(i);
        for (unsigned long long j = (unsigned long long)i * i; j < kSmall; j += 2ull * i) comp[j] = 1;
    }
    for (unsigned x = 1; x <= kSmall; ++x)
        below[x] = below[x - 1] + ((x - 1) >= 3 && ((x - 1) & 1u) && !comp[x - 1] ? 1u : 0u);
    const unsigned windows = (unsigned)((bound + kTabWindow - 1) / kTabWindow);
    uint32_t* d_base = nullptr;
    uint32_t* d_counts = nullptr;
    unsigned long long* d_off = nullptr;
    std::vector<uint32_t> counts(windows);
    std::vector<unsigned long long> off(windows + 1, 0);
    int rc = PG_OK;
    auto ck = [&](cudaError_t e, int code) {
        if (e != cudaSuccess && rc == PG_OK) rc = code;
        return rc == PG_OK;
    };
    if (ck(cudaMalloc(&d_base, base.size() * sizeof(uint32_t)), PG_ENOMEM) &&
        ck(cudaMalloc(&d_counts, windows * sizeof(uint32_t)), PG_ENOMEM) &&
        ck(cudaMalloc(&d_off, windows * sizeof(unsigned long long)), PG_ENOMEM) &&
        ck(cudaMemcpy(d_base, base.data(), base.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), PG_ECUDA)) {
        k_tab_count<<<windows, kSieveThreads>>>(d_base, (int)base.size(), bound, d_counts);
        ck(cudaGetLastError(), PG_ECUDA);
        ck(cudaMemcpy(counts.data(), d_counts, windows * sizeof(uint32_t), cudaMemcpyDeviceToHost), PG_ECUDA);
    }
    if (rc == PG_OK) {
        for (unsigned b = 0; b < windows; ++b) off[b + 1] = off[b] + counts[b];
        s->nprimes = off[windows];
        if (ck(cudaMalloc(&s->table, std::max<unsigned long long>(1, s->nprimes) * sizeof(uint2)), PG_ENOMEM) &&
            ck(cudaMemcpy(d_off, off.data(), windows * sizeof(unsigned long long), cudaMemcpyHostToDevice),
               PG_ECUDA)) {
            k_tab_fill<<<windows, kSieveThreads>>>(d_base, (int)base.size(), bound, d_off, s->table);
            ck(cudaGetLastError(), PG_ECUDA);
            ck(cudaDeviceSynchronize(), PG_ECUDA);
        }
    }
    if (rc == PG_OK &&
        ck(cudaMalloc(&s->scratch, (kTabOffLive0 + 2 * max_count) * sizeof(uint32_t)), PG_ENOMEM)) {
        // stages end at the primes below 2^10, 2^13, ..., 2^28, 2^30, 2^31, bound
        const unsigned lg[] = {10, 13, 16, 19, 22, 25, 28, 30, 31};
        for (unsigned g : lg) {
            const unsigned long long x = 1ull << g;
            if (x >= bound) break;
            s->stage_end.push_back(x <= kSmall ? below[x] : off[x / kTabWindow]);
        }
        s->stage_end.push_back(s->nprimes);
    }
    cudaFree(d_base);
    cudaFree(d_counts);
    cudaFree(d_off);
    if (rc != PG_OK) {
        sieve_free(s);
        return rc;
    }
    *out = s;
    return PG_OK;
}

extern "C" int pg_sieve_destroy(pg_sieve* s) {
    sieve_free(s);
    return PG_OK;
}

extern "C" int pg_sieve_primes(const pg_sieve* s, uint64_t* count) {
    if (!s || !count) return PG_EINVAL;
    *count = s->nprimes;
    return PG_OK;
}

extern "C" int pg_sieve_strike(pg_sieve* s, const uint64_t* d_ks, const uint32_t* d_ns, size_t count,
                               uint64_t* d_smallest_factor, void* stream) {
    if (!s) return PG_EINVAL;
    if (count > s->max_count) return PG_ETOOBIG;
    if ((!d_ks || !d_ns || !d_smallest_factor) && count) return PG_EINVAL;
    if (!count) return PG_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return PG_ECUDA;
    if (dev != s->device) return PG_ESTATE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t* ctrl = s->scratch;
    uint32_t* live[2] = {s->scratch + kTabOffLive0, s->scratch + kTabOffLive0 + s->max_count};
    const unsigned long long* ks = reinterpret_cast<const unsigned long long*>(d_ks);
    unsigned long long* fac = reinterpret_cast<unsigned long long*>(d_smallest_factor);
    const unsigned cnt = (unsigned)count;
    k_na_seed<<<(cnt + kNaRankThreads - 1) / kNaRankThreads, kNaRankThreads, 0, st>>>(d_ns, cnt, ctrl, live[0],
                                                                                        fac);
    int cur = 0;
    unsigned long long begin = 0;
    const unsigned long long per_cta = (unsigned long long)kTabThreads * kTabPerThread;
    for (unsigned long long end : s->stage_end) {
        if (end <= begin) continue;
        const unsigned ctas = (unsigned)((end - begin + per_cta - 1) / per_cta);
        k_tab_test<<<ctas, kTabThreads, 0, st>>>(s->table, (unsigned)begin, (unsigned)end, ks, d_ns, live[cur],
                                                 ctrl + 1 + cur, fac);
        k_na_compact<<<1, kNaCompactThreads, 0, st>>>(live[cur], ctrl + 1 + cur, fac, live[cur ^ 1],
                                                      ctrl + 1 + (cur ^ 1));
        cur ^= 1;
        begin = end;
    }
    k_na_finish<<<(cnt + 255) / 256, 256, 0, st>>>(fac, cnt);
    return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}

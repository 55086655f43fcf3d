// pg_internal.h -- structures shared by the host engine and the sm_103a kernels.
//
// Representation of a residue on the device (one "slot").  For N = k*2^n+1 the
// engine keeps y = x * 2^n mod N (Montgomery form with R = 2^n).  Because
// k*2^n = -1 (mod N), 2^-n = -k (mod N): the Montgomery reduction of a product
// P = H*2^n + Lo is H - k*Lo, with no division (see pg_kernels.cuh).
//
//   y = sum_{j<M} d_j 2^{S_j} + top * 2^n,   S_j = ceil(j n / M)
//
// d_j are signed "balanced" digits of width S_{j+1}-S_j (16 bits at n = 2^20,
// M = 2^16), top is a small signed integer (|top| <= k/2 after reduction).
// Between squarings the digits are left "pending": each run of RUN consecutive
// digits carries an int128 carry-out that the next squaring's first pass
// folds into the following run.
#ifndef PG_INTERNAL_H
#define PG_INTERNAL_H

#include <cstdint>
#include <cuda_runtime.h>

namespace pg {

constexpr int RUN = 8;           // digits per carry run (one thread, sequential)
constexpr int MAX_PASSES = 3;

// Per-slot mutable state (device memory).
struct SlotState {
    long long step;                  // operations completed
    long long total;                 // operations to reach; the slot idles at step == total
    unsigned long long kexp;         // exponent driving the small-multiplier schedule (0 = none)
    int kbits;                       // bit length of kexp
    int mul;                         // small multiplier (the base a)
    int active;                      // written by the first-pass kernel each step
    int flags;                       // error bits (overflow, bad rounding range)
    unsigned long long maxerr_bits;  // max roundoff error, as the bits of a non-negative double
    long long top;                   // top digit of the current input (weight 2^n)
    long long pend_lo;               // pending contribution at weight 2^n (int128, lo/hi):
    long long pend_hi;               //   s*top_a*top_b of the last product, or the re-armed top
    int op;                          // OP_PRODUCT or OP_FORWARD
    int partner;                     // slot whose digits/spectrum multiply this one (self: square)
    long long tope[2];               // the top digit again, indexed by the parity of the step count it
                                     //   belongs to: a fused last+first pass (k_edge) reads one entry
                                     //   while its first CTA writes the other
};

enum SlotOp : int {
    OP_PRODUCT = 0,  // y <- s * y * partner * 2^-n  (partner == self: square)
    OP_FORWARD = 1   // operand of another slot's product: fix up + forward passes only
};

enum SlotFlags : int { SF_DIGIT_OVERFLOW = 1, SF_ROUND_RANGE = 2, SF_WAIT_TIMEOUT = 4, SF_COPY_ABANDONED = 8 };

// Per-slot descriptor (device memory, read-only during a step).
struct Slot {
    int* digits;          // M int32 balanced digits
    long long* carries;   // (M/RUN) int128 carries, stored as (lo, hi) int64 pairs
    double2* spec;        // M complex: the transform buffer
    const double2* wf;    // M: forward weight  a_j * theta^j
    const double2* wi;    // M: inverse weight  conj(theta^j) / (M a_j)
    SlotState* st;
    unsigned long long k;
    unsigned n;
    unsigned pad_;
};

// Per FFT-length constants, passed to kernels by value.
struct PlanDev {
    int M, lgM, P;
    int F[MAX_PASSES];        // pass radices, F[0] outermost
    int S[MAX_PASSES];        // element stride inside pass i
    int Mi[MAX_PASSES];       // sub-transform length entering pass i
    const double2* tw[MAX_PASSES];   // inter-pass twiddles, tw[i][p*S[i] + r], i < P-1
    const double2* wF[MAX_PASSES];   // omega_{F[i]}^e, e < F[i]
    // When M divides n every IBDWT weight a_j is 1 and the weight of digit
    // j = r + q*S[0] is theta^j = theta^r theta^(q S[0]): theta^r commutes with the
    // pass-0 transform over q and is folded into its twiddles, so only an F[0]-entry
    // table remains (no M-entry weight tables are read).
    const double2* twu;              // tw[0][p*S[0] + r] * theta^r
    const double2* thf;              // theta^(q S[0]), q < F[0]
    const double2* thi;              // conj(theta^(q S[0])) / M
};

// Whether digit weights reduce to theta^j for n (M = 2^lgM divides n).
__host__ __device__ inline bool unit_weights(unsigned n, int lgM) { return (n & ((1u << lgM) - 1)) == 0; }

}  // namespace pg

#endif

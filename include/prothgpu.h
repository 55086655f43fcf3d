/*
 * prothgpu.h -- C ABI of the GB300 Proth modular-squaring engine (libprothgpu.so).
 *
 * Plain C types only (no CUDA or C++ types), so cgo, JNI, ctypes or the
 * reference's own C++ can bind it.  Residues cross the boundary as
 * little-endian 64-bit limbs, the layout of the reference's limb buffers
 * (prothlogic4.2/dcore.cpp:143-155, mpz_export order -1 at proth_logic.cpp:446).
 *
 * Every function returns a PG_* status; none aborts the process.  One engine
 * handle belongs to one host thread at a time (the reference keeps one
 * FFTContext per worker thread, dcore.cpp:134); distinct handles may be used
 * from distinct threads concurrently, each on its own CUDA stream.
 */
#ifndef PROTHGPU_H
#define PROTHGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define PG_OK 0
#define PG_EINVAL 1     /* bad argument */
#define PG_ENOMEM 2     /* device or host allocation failed */
#define PG_EROUNDOFF 3  /* max |x - round(x)| > 0.4 at the largest FFT length allowed */
#define PG_EGERBICZ 4   /* Gerbicz check kept failing after the allowed rollbacks */
#define PG_ETIMEOUT 5   /* a bounded wait expired */
#define PG_ECUDA 6      /* CUDA runtime error */
#define PG_EIO 7        /* checkpoint file error */
#define PG_ENODEV 8     /* no usable sm_103 device */
#define PG_ESTATE 9     /* handle not ready for this call */
#define PG_EOVERFLOW 10 /* a digit or carry left its representable range */
#define PG_ETOOBIG 11   /* request larger than a fixed-size device buffer holds */

/* pg_create flags */
#define PG_FLAG_NO_GERBICZ 0x1u   /* skip the Gerbicz check in pg_square */
#define PG_FLAG_NO_BUMP 0x2u      /* report PG_EROUNDOFF instead of growing the FFT */
#define PG_FLAG_NO_GRAPH 0x4u     /* launch kernels directly instead of replaying a CUDA graph */
#define PG_FLAG_FORCE_LEN 0x8u    /* use fft_len_hint exactly, even below the safe length (tests) */
#define PG_FLAG_NO_PERSIST 0x10u  /* (default) per-pass kernels, not the persistent cooperative kernel */
#define PG_FLAG_PERSIST 0x20u     /* squaring chains in the persistent cooperative kernel */

typedef struct pg_engine pg_engine;
typedef struct pg_batch pg_batch;

/* Result of one Proth test. */
typedef struct pg_result {
    uint64_t k;
    uint32_t n;
    uint32_t base;          /* a with Jacobi(a, N) = -1; 0 when the small-prime gate rejected N */
    int32_t verdict;        /* 1: a^((N-1)/2) = -1 (prime), 0: composite */
    int32_t status;         /* PG_* */
    uint64_t res64;         /* limb 0 of a^((N-1)/2) mod N (0 when gated) */
    uint64_t tag;           /* caller's tag (batch) */
    uint32_t fft_len;       /* complex FFT length used at the end */
    uint32_t fft_bumps;     /* FFT-length increases after roundoff > 0.4 */
    uint32_t gerbicz_checks;
    uint32_t gerbicz_failures;
    double max_err;         /* largest max |x - round(x)| seen */
    double seconds;         /* time to verdict: submit (or call) to verdict */
} pg_result;

/* ---- library ---- */
const char* pg_strerror(int status);
int pg_version(void);                 /* 100 * major + minor */
int pg_device_info(char* name, size_t name_len, int* sm_count);
/* FFT length (complex points) the engine picks for k*2^n+1; 0 if n is out of range. */
uint32_t pg_pick_fft_len(uint64_t k, uint32_t n);

/* Host-only pieces of the Proth test (no device needed). */
/* 1 if a gate prime <= 67 divides k*2^n+1 (is_divisible_by_gate, proth_logic.cpp:41-50, 400-408). */
int pg_gate_rejects(uint64_t k, uint32_t n);
/* Smallest listed base a with Jacobi(a, N) = -1, else 0 (proth_logic.cpp:411-422). */
uint64_t pg_choose_base(uint64_t k, uint32_t n);
/* Device representation round trip on the host: x -> Montgomery form -> M
 * balanced digits -> value -> x mod N.  Returns PG_OK and the canonical x. */
int pg_host_roundtrip(uint64_t k, uint32_t n, uint32_t M, const uint64_t* x, size_t n_limbs, uint64_t* out,
                      size_t out_limbs);

/* ---- single-candidate engine (all SMs on one residue) ----
 * Replaces fft_init / fft_destroy / fft_square_karatsuba
 * (prothlogic4.2/fft_engine.h:10-22, fft_engine.cpp:18-80 and 986-1073) and the
 * reduction the reference loop runs after each squaring (proth_logic.cpp:488-533).
 * The residue stays on the device between calls; pg_set_residue /
 * pg_get_residue move it across the boundary. */
int pg_create(uint64_t k, uint32_t n, uint32_t fft_len_hint, uint32_t flags, pg_engine** out);
int pg_destroy(pg_engine* e);
/* x (n_limbs little-endian limbs, any value) is reduced mod N and loaded. */
int pg_set_residue(pg_engine* e, const uint64_t* limbs, size_t n_limbs);
/* Canonical x mod N into n_limbs limbs (zero-padded); n_limbs >= ceil((n + 64)/64). */
int pg_get_residue(pg_engine* e, uint64_t* limbs, size_t n_limbs);
/* The current residue WITHOUT verifying it first (pg_get_residue verifies):
 * for callers that read the residue after every squaring, where a
 * verification per read would redo the squarings since the last verified
 * residue.  Writes the low n_limbs limbs of x mod N (canonical; the value is
 * truncated when it needs more limbs, as the reference engine's fixed-size
 * limb buffer truncates it, fft_engine.cpp:925-983); *needed (optional)
 * receives the limbs x needs, *unverified (optional) the squarings done since
 * the last verified residue.  No counterpart in the reference, whose engine
 * has no verification (its callers read v after every fft_square_karatsuba,
 * proth_logic.cpp:488-533). */
int pg_peek_residue(pg_engine* e, uint64_t* limbs, size_t n_limbs, size_t* needed, uint64_t* unverified);
/* x <- x^(2^iters) mod N.  Each squaring records max |x - round(x)|; above 0.4
 * the engine rolls back to its last verified residue and grows the FFT length.
 * A Gerbicz check covers every block of squarings unless PG_FLAG_NO_GERBICZ. */
int pg_square(pg_engine* e, uint64_t iters);
/* x <- base_a^exponent mod N by left-to-right binary powering on the device
 * (x <- x^2 * a^bit per step); used for x0 = a^k (proth_logic.cpp:424-446). */
int pg_pow_small(pg_engine* e, uint64_t base_a, uint64_t exponent);
/* Largest roundoff error since the last reset (ctx.last_max_diff). */
int pg_max_err(pg_engine* e, double* out, int reset);
int pg_fft_len(const pg_engine* e, uint32_t* out);
/* Gerbicz block length in squarings (default 1000) and verification interval
 * in blocks (default 0 = verify at the end of every pg_square call). */
int pg_set_gerbicz(pg_engine* e, uint32_t block, uint32_t verify_every_blocks);
/* Counters: squarings done, Gerbicz checks, failures, FFT bumps. */
int pg_stats(const pg_engine* e, uint64_t* squarings, uint32_t* checks, uint32_t* failures,
             uint32_t* bumps);
/* Device-timed run of `iters` squarings (CUDA events on the engine's stream,
 * graph replay, no rollback bookkeeping); *ms receives the elapsed time.  The
 * residue advances by `iters` squarings.  Returns the launches per squaring in
 * *kernels_per_step. */
int pg_time_squarings(pg_engine* e, uint64_t iters, double* ms, uint32_t* kernels_per_step);
/* Per-kernel device times (ms) of one squaring, launched one by one with an
 * event pair around each: times[i] for i < *count (at most cap). */
int pg_profile_step(pg_engine* e, double* times, uint32_t cap, uint32_t* count);
/* pg_square bracketed by CUDA events on the engine's stream: *ms is the device
 * time of the whole call (squarings, Gerbicz products and checks, and the
 * idle gaps of its host synchronisation). */
int pg_square_timed(pg_engine* e, uint64_t iters, double* ms);
/* Overwrite a device buffer larger than the L2 cache (between timed steps). */
int pg_flush_l2(void);
/* Kernels this library has launched so far (graph replays included). */
uint64_t pg_launch_count(void);
/* Select the CUDA device for the calling host thread (one process per GPU). */
int pg_set_device(int device);
/* Measured FP64 FMA throughput of this device (TFLOP/s, 2 flops per DFMA):
 * a DFMA-only kernel, 4 x SM-count CTAs of 256 threads, 8 independent chains. */
int pg_measure_fp64_peak(double* tflops);
/* Test hook: add `delta` to residue digit `index` on the device (simulates a
 * silent memory error; nothing faults).  Used by the failure-detection tests. */
int pg_debug_corrupt(pg_engine* e, uint32_t index, int32_t delta);

/* Checkpoint file in the reference format (checkpoint_manager.h:10-16):
 * {uint64 current_i, size_t n_limbs} + n_limbs limbs, followed by an extension
 * block (k, n, FFT length, squarings completed, checksum) that the reference
 * reader ignores.  current_i keeps the reference meaning: index of the last
 * completed squaring of the test loop. */
int pg_checkpoint_save(pg_engine* e, const char* path, uint64_t current_i);
int pg_checkpoint_load(pg_engine* e, const char* path, uint64_t* current_i);

/* Full Proth test on the device: the gate of proth_logic.cpp:400-408, base
 * choice :411-422, x0 = a^k mod N, n-1 squarings, verdict x == N-1
 * (execute_proth_test_fft, proth_logic.cpp:384-580). */
int pg_proth_test(uint64_t k, uint32_t n, uint32_t flags, pg_result* out);

/* ---- trial-division pre-filter ----
 * For each candidate k_i*2^{n_i}+1 the smallest odd prime p < bound (bound <=
 * 2^32) dividing it, or 0.  Per-candidate counterpart of the reference's GPU
 * sieve strike (prothlogic4.2/gpu_engine.cu:290-320 check_proth_candidates_kernel),
 * for a queue of independent (k, n) pairs. */
int pg_prefilter(const uint64_t* ks, const uint32_t* ns, size_t count, uint64_t bound, uint64_t* smallest_factor);

/* Same answer as pg_prefilter, for callers that cannot allocate device memory
 * (a host runtime that owns the device budget through its own pool, or a
 * serving loop in which cudaMalloc/cudaFree would synchronise the device).  No
 * counterpart in the reference.  Allocates nothing: d_ks, d_ns and
 * d_smallest_factor are DEVICE pointers owned by the caller, the work is queued
 * on `stream` (a cudaStream_t; NULL = the legacy default stream) and the call
 * returns without waiting for it.  Its scratch is one file-scope device array
 * of PG_PREFILTER_NOALLOC_SCRATCH_BYTES, held by every GPU on which the library
 * is loaded until the process exits; count > PG_PREFILTER_NOALLOC_MAX_COUNT is
 * rejected with PG_ETOOBIG.  The first call on a device (the current device)
 * sets the scratch up, synchronously; make that first call before any stream
 * capture.  All calls share the one array: calls whose work overlaps on the GPU
 * race and give wrong answers, so order them (one stream, or events).  The
 * array's device address is looked up once per device: after cudaDeviceReset
 * the library must be reloaded before this is called again. */
#define PG_PREFILTER_NOALLOC_MAX_COUNT 65536
#define PG_PREFILTER_NOALLOC_SCRATCH_BYTES 557312
int pg_prefilter_noalloc(const uint64_t* d_ks, const uint32_t* d_ns, size_t count, uint64_t bound,
                         uint64_t* d_smallest_factor, void* stream);

/* Same answer again, for a caller that pre-filters a few candidates at a time,
 * many times a second (a serving loop).  The reference keeps its sieve state on
 * the device between batches of primes (init_sparse_gpu_sieve /
 * process_sparse_prime_batch_gpu_from_vram / finalize_sparse_gpu_sieve,
 * prothlogic4.2/gpu_engine.cu:404-450); a pg_sieve keeps every odd prime below
 * `bound` (<= 2^32) in device memory instead, sieved once by pg_sieve_create
 * (synchronous, allocates 8 bytes a prime: 1.6 GB at 2^32, plus 4 bytes per
 * candidate of max_count for the live lists; make it before any stream
 * capture, on the device it will serve).  pg_sieve_strike then queues only the
 * trial division on `stream` (a cudaStream_t; NULL = the legacy default
 * stream) and returns without waiting: no allocation, no host synchronisation.
 * d_ks, d_ns and d_smallest_factor are DEVICE pointers owned by the caller;
 * count > max_count is rejected with PG_ETOOBIG.  Strikes on one pg_sieve share
 * its live lists: order them on the GPU (one stream, or events).
 * pg_sieve_primes reports the number of primes held. */
#define PG_SIEVE_MAX_COUNT 65536
typedef struct pg_sieve pg_sieve;
int pg_sieve_create(uint64_t bound, size_t max_count, pg_sieve** out);
int pg_sieve_strike(pg_sieve* s, const uint64_t* d_ks, const uint32_t* d_ns, size_t count,
                    uint64_t* d_smallest_factor, void* stream);
int pg_sieve_primes(const pg_sieve* s, uint64_t* count);
int pg_sieve_destroy(pg_sieve* s);

/* ---- batched engine: many candidates per launch, grouped by FFT length ----
 * Replaces the reference's worker pool (dcore.cpp:84-193 dispatch with
 * worker.cpp:27-69 run_task_with_ctx over PROTH_FF_BATCH k lists). */
/* max_slots_per_class: at most 13107 (65535 with PG_FLAG_NO_GERBICZ), since each
 * candidate of a Gerbicz-checked class holds five slots and a launch maps slots
 * to gridDim.y. */
int pg_batch_create(uint32_t max_slots_per_class, uint32_t flags, pg_batch** out);
int pg_batch_destroy(pg_batch* b);
/* Queue one candidate; the gate and base choice run on the host at submit. */
int pg_batch_submit(pg_batch* b, uint64_t k, uint32_t n, uint64_t tag);
/* Advance every admitted candidate by up to `max_steps` squarings (0: until
 * all queued candidates are done), admitting queued ones into free slots. */
int pg_batch_run(pg_batch* b, uint64_t max_steps);
/* pg_batch_run bracketed by CUDA events on every FFT-length class's stream;
 * *ms is the longest class's device time (admission and collection included). */
int pg_batch_run_timed(pg_batch* b, uint64_t max_steps, double* ms);
/* Move up to `cap` finished results out; *count receives how many. */
int pg_batch_poll(pg_batch* b, pg_result* out, size_t cap, size_t* count);
/* Cap the device bytes that admitted candidates may hold (0: no cap); queued
 * candidates wait until a verdict frees room.  Class pools are sized to fit. */
int pg_batch_set_budget(pg_batch* b, uint64_t hbm_bytes);
/* Test hook: add `delta` to digit `index` of the running candidate `tag`
 * (a simulated memory error; nothing faults).  PG_ESTATE if it is not running. */
int pg_batch_debug_corrupt(pg_batch* b, uint64_t tag, uint32_t index, int32_t delta);
/* Device bytes one candidate k*2^n+1 holds while admitted in a batch with the
 * Gerbicz check (its five role slots, weights share, checkpoint copy). */
uint64_t pg_slot_footprint(uint64_t k, uint32_t n);
/* Gerbicz-Li block length (class steps) of a batch, before its first run
 * (default 1000; the check is off with PG_FLAG_NO_GERBICZ at creation).  Each
 * candidate is verified when its chain ends: one block of squarings of the
 * product chain plus the tail since the last block end; a mismatch sends it
 * back to its last verified residue.  pg_result reports checks and failures. */
int pg_batch_set_gerbicz(pg_batch* b, uint64_t block);

/* ---- launch-shape autotuner (replaces the reference's auto_tune_fft_len,
 * prothlogic4.2/dcore.cpp:20-81, which tunes only the FFT length) ----
 * A shape is the pass radices of one squaring at 2^lg points (passes x f0 x
 * f1 [x f2]), the transform columns per CTA of the middle and inner kernels
 * (g_mid, g_inner), i.e. the CTAs per residue, and the threads per butterfly.  pg_autotune times every compiled
 * shape on `slots` residues for >= iters squarings, checks that all shapes give
 * bit-identical residues, and makes the fastest the shape of later engines
 * (slots == 1, mode PG_TUNE_ONE) or batch classes (slots > 1, PG_TUNE_MANY) at
 * that length.  `out` receives up to `cap` rows, `count` the number of shapes. */
#define PG_TUNE_ONE 0u
#define PG_TUNE_MANY 1u
typedef struct pg_tune_result {
    uint32_t lg, slots, passes, f0, f1, f2, g_mid, g_inner;
    uint32_t tpb;       /* threads per radix-4 butterfly: 1, 2 or 4 (lanes sharing it: shorter FP64 chains) */
    uint32_t cluster;   /* one residue, three-pass plans: CTAs of the cluster that runs the middle passes
                           as one kernel (0: three kernels) */
    uint32_t tpb_outer; /* threads per radix-4 butterfly of the first and last passes (0: tpb) */
    uint32_t resident;  /* two-pass plans: CTAs of the cluster that holds one residue in shared memory for a
                           whole squaring chain (k_resident; 0: per-pass kernels) */
    uint32_t resident_threads; /* threads per CTA of that kernel */
    uint32_t edge;      /* one residue: the last pass of each squaring and the first pass of the next as one
                           kernel (k_edge), 0 or 1 */
    double us_per_step; /* one squaring of every slot */
    int32_t valid;      /* residues equal to the other shapes', no roundoff or range flag */
    int32_t chosen;
} pg_tune_result;
int pg_autotune(uint32_t lg, uint32_t slots, uint32_t iters, pg_tune_result* out, size_t cap, size_t* count);
/* The shape in use for (lg, mode); PG_ESTATE when none was tuned or set. */
int pg_tune_get(uint32_t lg, uint32_t mode, pg_tune_result* out);
/* Install a shape (e.g. one saved from an earlier run); PG_EINVAL if not compiled. */
int pg_tune_set(uint32_t mode, const pg_tune_result* r);
int pg_tune_clear(void);
/* Queued, running and finished-but-unpolled candidate counts. */
int pg_batch_pending(const pg_batch* b, size_t* queued, size_t* running, size_t* finished);

#ifdef __cplusplus
}
#endif
#endif

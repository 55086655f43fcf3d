/*
 * prothgpu_fftcompat.h -- the reference's engine interface, served by the GPU.
 *
 * Declares, with the same names, signatures and struct layout, the engine API
 * that the ProthLogic 4.2 callers use (prothlogic4.2/fft_engine.h:10-22 and the
 * FFTContext of prothlogic4.2/fft_types.h:12-60), so proth_logic.cpp,
 * dcore.cpp and worker.cpp link against libprothgpu_compat.a unchanged.
 *
 * When building INSIDE the reference tree, compile the shim with
 * -DPROTHGPU_USE_REFERENCE_HEADERS and the reference's include path instead:
 * it then includes the reference's own fft_engine.h.
 */
#ifndef PROTHGPU_FFTCOMPAT_H
#define PROTHGPU_FFTCOMPAT_H

#ifdef PROTHGPU_USE_REFERENCE_HEADERS
#include "fft_engine.h"
#else
#include <cstddef>
#include <cstdint>

enum class FFTBackend { INTERNAL };

// Same member order and types as the reference's FFTContext, so code compiled
// against either header sees the same object.  The GPU shim keeps its engine
// handle in base_ptr; the double* buffers stay null (the residue lives on the GPU).
struct FFTContext {
    FFTBackend backend;
    void* base_mem_ptr;
    void* base_ptr;
    void* raw_allocation;
    size_t total_allocation_size;
    size_t fft_len;
    int num_workers;
    double* re;
    double* im;
    double* re2;
    double* im2;
    double* w1_re;
    double* w1_im;
    double* w2_re;
    double* w2_im;
    double* w3_re;
    double* w3_im;
    double* proth_w_re;
    double* proth_w_im;
    double last_max_diff;
    double prof_pack = 0.0;
    double prof_fwd = 0.0;
    double prof_square = 0.0;
    double prof_inv = 0.0;
    double prof_unpack = 0.0;
    uint64_t prof_calls = 0;
    double prof_unpack_clear = 0.0;
    double prof_unpack_deweight = 0.0;
    double prof_unpack_scalar = 0.0;
    double prof_unpack_finalfix = 0.0;
    double* k_A_re;
    double* k_A_im;
    double* k_B_re;
    double* k_B_im;
    double* k_AB_re;
    double* k_AB_im;
    uint64_t current_i = 0;
};

bool fft_init(FFTContext& ctx, FFTBackend backend, size_t fft_len);
void fft_destroy(FFTContext& ctx);
void fft_square_karatsuba(FFTContext& ctx, uint64_t* v, size_t n_limbs, unsigned n_bits, uint64_t k_val);
#endif

/* GPU-only extension: n squarings in one call, the residue synchronised once. */
void fft_square_karatsuba_n(FFTContext& ctx, uint64_t* v, size_t n_limbs, unsigned n_bits, uint64_t k_val,
                            uint64_t iters);

#endif

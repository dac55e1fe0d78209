/*
 * vkg_diag.h -- test-only diagnostics exported by libvkg.so. They check the library's tcgen05
 * plumbing and its bounded waits; they are not part of the drop-in interface (include/vkg.h) and
 * have no counterpart in the reference.
 */
#ifndef VKG_DIAG_H
#define VKG_DIAG_H

#include "vkg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* D (128 x n FP32, row-major) = A (128 x k BF16, row-major) * B^T (n x k BF16, row-major) with one
 * tcgen05.mma chain through the library's shared-memory descriptors (16 <= n <= 64, k <= 256, both
 * multiples of 16); *d_err (device) gets bit 0 if the completion wait ran out */
vkg_status vkg_diag_tc_gemm(vkg_ctx *ctx, const uint16_t *d_a, const uint16_t *d_b, uint32_t k, uint32_t n, float *d_d,
                            uint32_t *d_err, void *stream);

/* the error path of the tcgen05 kernels' bounded waits, run to its end: num_ctas CTAs (<= 4096) each
 * allocate TMEM, wait on an mbarrier that nothing arrives on with a limit of limit_ns (<= 1e8) instead
 * of the kernels' 1 s, set bit 0 of *d_err when the wait runs out, wait once more (bounded) as the
 * kernels do for MMAs in flight, free their TMEM and return. *d_elapsed_ns (device, uint64) receives
 * the longest time one CTA spent waiting (atomic max: zero it first). */
vkg_status vkg_diag_wait_timeout(vkg_ctx *ctx, uint32_t num_ctas, uint64_t limit_ns, uint32_t *d_err,
                                 uint64_t *d_elapsed_ns, void *stream);

/* record the random numbers the tracer's kernels draw (d_buf NULL: stop). From the next render on,
 * the path of sample s through window pixel p writes record r = s * pixels + p of d_buf (floats):
 * [0..1] the camera jitter, then per segment i < max_segments the segment's uniforms at
 * 2 + 16 i (8, 11 or 15 of them, one more when a material disperses; the rest of the record is left
 * as it was). d_buf must hold samples x pixels x (2 + 16 max_segments) floats for the largest render
 * made while set. */
vkg_status vkg_diag_tracer_uniforms(vkg_tracer *tracer, float *d_buf, uint32_t max_segments);

#ifdef __cplusplus
}
#endif
#endif /* VKG_DIAG_H */

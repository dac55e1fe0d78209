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

#ifdef __cplusplus
}
#endif
#endif /* VKG_DIAG_H */

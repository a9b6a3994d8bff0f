/*
 * gb300kf_diag.h — measurement helpers for roofline reporting.
 *
 * The fitter is bound by the FP64 pipe, for which no vendor-measured peak is
 * supplied; kf_diag_fp64_fma_rate measures it on the current device with
 * independent DFMA chains on every SM.  Not part of the fit path.
 */
#ifndef GB300KF_DIAG_H
#define GB300KF_DIAG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Runs `iters` dependent DFMA steps on 8 independent chains per thread over
 * the whole device and reports FP64 FLOP/s (2 per DFMA) in *gflops_out.
 * Blocks until done.  Returns 0 or a negative kf_error. */
int32_t kf_diag_fp64_fma_rate(int32_t iters, double *gflops_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GB300KF_DIAG_H */

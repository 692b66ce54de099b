/*
 * te_diag.h -- hardware probes of libtegpu used by the benchmark's roofline.
 * No counterpart in the reference (which has no GPU path).
 */
#ifndef TE_DIAG_H
#define TE_DIAG_H
#ifdef __cplusplus
extern "C" {
#endif

/* FP64 FMA throughput of the current device in TFLOP/s: every SM runs
 * independent FMA chains (2 flops each) for about a millisecond, timed with
 * CUDA events.  Returns 0 or a negative TE_ERR_* code. */
int te_probe_fp64_tflops(double* tflops);

#ifdef __cplusplus
}
#endif
#endif

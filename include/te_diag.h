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

/* FP64 FMA issue with `warps` warps per block on `blocks` blocks (1..32 warps;
 * at most one block per SM for a per-SM figure): cycles_indep = SM clock
 * cycles per warp FMA per block when each thread runs 8 independent chains,
 * cycles_chain = cycles per FMA of one dependent chain per thread.  The clock
 * is the device's nominal clock (cudaDevAttrClockRate).  Returns 0 or a
 * negative TE_ERR_* code. */
int te_probe_fp64_issue(int warps, int blocks, double* cycles_indep, double* cycles_chain);

#ifdef __cplusplus
}
#endif
#endif

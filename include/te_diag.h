/*
 * te_diag.h -- hardware probes of libtegpu used by the benchmark's roofline.
 * No counterpart in the reference (which has no GPU path).
 */
#ifndef TE_DIAG_H
#define TE_DIAG_H
#include "tegpu.h"
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

/* Gather throughput: 16-byte rows of a table fetched by index, the access
 * pattern of the SpMV passes' gathers of the fixed-point vector.  With a
 * matrix M the indices are its SELL slot columns in chunk order (what one
 * SpMV pass gathers, padding included) and the table has its dimension;
 * with M = NULL, n_gathers uniform random indices into n_rows rows.  Every
 * warp walks its own run of 32-index rows.  mode 0: ordinary loads with depth
 * (1, 2 or 4) rows in flight per lane; mode 1: TMA tile::gather4 copies into
 * shared memory with depth (4, 8 or 16) stages per warp, completion on
 * mbarriers with bounded waits (TE_ERR_DEVICE_TIMEOUT if one gives up).
 * blocks_per_sm 1..8 blocks of 256 threads per SM (TE_ERR_UNSUPPORTED when
 * they do not fit).  Returns the best of 4 timed launches in *rows_per_s and
 * a checksum of the gathered rows that is the same for both modes at the same
 * blocks_per_sm (which fixes the indices every warp walks). */
int te_probe_gather(te_matrix M, int64_t n_rows, int64_t n_gathers, int mode, int depth, int blocks_per_sm,
                    double* rows_per_s, unsigned long long* checksum);

#ifdef __cplusplus
}
#endif
#endif

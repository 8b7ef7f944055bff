/*
 * edyn_surrogate.h -- C ABI of the chemistry surrogate's kernels.
 *
 * The reference has no surrogate: it integrates every cell's chemistry with
 * its implicit solver (reaction_macks -> macks, SRC/source.f90:17-84).
 * These entry points add the learned path that replaces that call for the
 * cells whose chemistry the network predicts well enough: a small MLP
 * (BF16 weights, FP32 accumulation on the tensor cores) maps a cell's
 * (T, log p, Box-Cox Y, log dt) to its increment over dt; a per-cell gate
 * (FP64 trapezoidal residual + element conservation) accepts the result or
 * hands the cell to the implicit integrator (edyn_reactors_device).
 *
 * All array arguments are DEVICE pointers; `stream` is a cudaStream_t (NULL:
 * the legacy default stream). Every function returns 0 or EDYN_E_* bits and
 * only enqueues work; edyn_mlp_status synchronises and reports a wait that
 * ran out inside a kernel.
 */
#ifndef EDYN_SURROGATE_H
#define EDYN_SURROGATE_H

#include "edyn_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define EDYN_E_SURR 64      /* a surrogate kernel's bounded wait ran out */

#define EDYN_MLP_EPI_F32 0    /* C32 = A B^T (+ bias) */
#define EDYN_MLP_EPI_GELU 1   /* z = A B^T + bias; C32 = z (if given); C16 = gelu(z) */
#define EDYN_MLP_EPI_DGELU 2  /* C16 (and C32, if given) = (A B^T) * gelu'(Z) */

/* Dense layer on the tensor cores: A [M][K] and B [N][K] BF16 row-major
 * (leading dimensions lda, ldb in elements, multiples of 8, 16-byte aligned
 * bases), N a multiple of 64, K a multiple of 64. The fused epilogue writes
 * FP32 (C32, ldc) and/or BF16 (C16, ldc16) outputs as EDYN_MLP_EPI_*
 * describes; gelu is the erf form 0.5 z (1 + erf(z / sqrt 2)). */
int edyn_mlp_gemm(const void* A, int lda, const void* B, int ldb, int M, int N, int K, int epi, const float* bias,
                  float* C32, int ldc, void* C16, int ldc16, const float* Z, int ldz, void* stream);

/* The bulk-copy form of edyn_mlp_gemm for inference: A and B pre-tiled by
 * edyn_mlp_tile (A with BR = 128 and M a multiple of 128, B with
 * BR = edyn_mlp_tile_rows(N)), so that every 64-column k-step of a CTA is
 * two contiguous copies by the bulk-copy (TMA) engine into a four-deep
 * ring. epi is EDYN_MLP_EPI_F32 or _GELU; with c16_tiled the GELU output is
 * written tiled (BR = 128, K = N), ready as the next layer's A. */
int edyn_mlp_gemm_tiled(const void* At, const void* Bt, int M, int N, int K, int epi, const float* bias, float* C32,
                        int ldc, void* C16, int ldc16, int c16_tiled, void* stream);

/* Row block height of the tiled B operand for N output columns (256, 128
 * or 64: the GEMM's N tile). */
int edyn_mlp_tile_rows(int N);

/* Row-major [R][K] BF16 (K a multiple of 64) -> tiled layout with BR-row
 * blocks (64, 128 or 256); block (r / BR, k / 64) is contiguous at element
 * ((r / BR)(K / 64) + k / 64) BR 64, in the core-matrix order of the GEMM's
 * shared-memory tiles; rows past R up to a multiple of BR are zero. */
int edyn_mlp_tile(const void* in, int R, int K, int BR, void* out, void* stream);

/* Synchronises the stream; EDYN_E_SURR if a kernel gave up a wait since the
 * last call (and clears that record). */
int edyn_mlp_status(void* stream);

/* Sets the limit [ns] of the GEMM waits that gate each next step (operand
 * copies landed, a staging buffer free again); the default is 2 s. A wait
 * that runs out stops its GEMM: the kernel still waits, with the full 2 s
 * bound, for the copies and products it issued, frees its TMEM and returns,
 * and edyn_mlp_status then reports EDYN_E_SURR. 0 makes every gating wait
 * give up at once, so a test can drive that path without a stuck barrier.
 * Applies to later launches on the current device. */
int edyn_mlp_set_wait_limit(unsigned long long ns);

/* out[c][r] = in[r][c] (BF16, rows x cols). */
int edyn_mlp_transpose(const void* in, int rows, int cols, void* out, void* stream);

/* out[c] = sum_r X[r][c] (FP32, rows x cols). */
int edyn_mlp_colsum(const float* X, int rows, int cols, float* out, void* stream);

/* Mean-square error over the first cols_real of cols columns: dY32/dY16 =
 * 2 (Y - T) / (rows cols_real), 0 in padded columns; *loss += the mean of
 * the squares (FP64 accumulator, not cleared). */
int edyn_mlp_mse(const float* Y, const float* T, int rows, int cols, int cols_real, float* dY32, void* dY16,
                 double* loss, void* stream);

/* One Adam step (bias-corrected, step >= 1) of n FP32 master weights w with
 * gradient g and moments m, v; w16 (if given) receives BF16 copies. */
int edyn_mlp_adam(float* w, const float* g, float* m, float* v, long n, float lr, float b1, float b2, float eps,
                  int step, void* w16, void* stream);

/* Network inputs of n cells (yiT rows of ns + 1: Y_1..Y_ns, T; rho kg/m^3;
 * dt s; wmol kg/mol): x = (T, log p, (Y_k^0.1 - 1)/0.1, log dt), standardised
 * as (x_j - mu_j) * isig_j, as BF16 rows of ldx >= ns + 3 columns (padding
 * columns get mu = isig = 0). */
int edyn_mlp_features(int n, int ns, const double* rho, const double* dt, const double* yiT, const double* wmol,
                      const float* mu, const float* isig, void* X, int ldx, void* stream);

/* Candidate states from the network output: per component (Y_k, then T)
 * y1 = y0 + dt f0 + (out_j osig_j + omu_j) (|dt f0| + floor), with f0 =
 * f(yiT0), output column 0 for T and k + 1 for Y_k, floor = yfloor for the
 * species and tfloor for T; Y_k clipped at 0. */
int edyn_mlp_decode(int n, int ns, const float* out, int ldo, const float* omu, const float* osig, const double* yiT0,
                    const double* f0, const double* dt, double yfloor, double tfloor, double* yiT1, void* stream);

/* Per-cell gate of a candidate yiT1 over dt from yiT0, with the FP64
 * right-hand sides f0 = f(yiT0), f1 = f(yiT1) (edyn_chem_rhs_device):
 * accepted when |y1 - y0 - dt (f0 + f1) / 2| <= atol + rtol max(|y0|,|y1|)
 * in every component (no atol on T) and every element's moles
 * sum_k elem[e][k] Y_k / W_k stay within etol (relative). A second
 * candidate ya with fa = f(ya) (both NULL: none) is tried where the first
 * fails and copied into yiT1 when it passes. accept[i] = 1 (first), 2
 * (second) or 0; count[0], count[1] += the cells each accepted (not
 * cleared). */
int edyn_mlp_gate(int n, int ns, int ne, const double* yiT0, double* yiT1, const double* f0, const double* f1,
                  const double* ya, const double* fa, const double* dt, const double* wmol, const double* elem,
                  double rtol, double atol, double etol, int* accept, unsigned* count, void* stream);

/* Packs the rejected cells (accept == 0), in cell order: idx[j] their cell
 * index, rho_p/dt_p/yiT_p their inputs, *nrej their number. */
int edyn_mlp_compact(int n, int ns, const int* accept, const double* rho, const double* dt, const double* yiT,
                     int* idx, double* rho_p, double* dt_p, double* yiT_p, int* nrej, void* stream);

/* yiT1[idx[j]] = yiT_p[j], j < m. */
int edyn_mlp_scatter(int m, int ns, const int* idx, const double* yiT_p, double* yiT1, void* stream);

/* FP64 chemistry right-hand side f = d(Y_1..Y_ns, T)/dt of n constant-volume
 * adiabatic reactors (the function the implicit integrator of
 * edyn_reactors integrates), on the context's stream. */
int edyn_chem_rhs_device(void* ctx, int n, const double* rho_d, const double* yiT_d, double* f_d);

#ifdef __cplusplus
}
#endif

#endif

// Launchers shared between the library's translation units (not part of the
// public C ABI).
//
// Device-indexed Krylov steps: the step index j lives in device memory, the
// operator reads a fixed input vector and writes a fixed work vector, and the
// last kernel of the step stores the normalized vector into row j + 1 of the
// basis and into the next input.  Every step therefore launches the same
// kernels with the same arguments, so captured CUDA graphs are replayed for
// all steps.  The index alternates between two slots: a step reads `cur` and
// writes j + 1 to `next` (the other slot), so no kernel of a step overwrites
// the index another block of the same step may still read; graphs are
// captured for both parities.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "c3l_gb300.h"

// largest GMRES basis (restart + 2 rows of projections) of the device step
#define C3L_GMRES_MAX_ROWS 1024

namespace c3l {

// Rows [0, *cur + 1) of V, plus the work vector itself when `self` is set
// (its squared norm), reduced in segments of `seglen` entries; with more than
// one segment a second kernel sums the partials.
struct RowDot {
    int max_rows;   // upper bound of rows (k_max + self)
    int nseg;
    int64_t seglen;
    unsigned grid;
};
RowDot row_dot_plan(int max_rows, int64_t dim, int sms);
int64_t row_dot_partial_size(const RowDot& p);  // entries of the partial buffer

// One Arnoldi step's CGS2 for a batch of channels in one launch per kernel
// (blockIdx.y = channel).  Per channel: basis V (rows of ld), work vector w
// (the operator's output, updated in place), next input xnext, projections
// c1 and c2 (k + 1 entries each), h, Hessenberg columns Hc (leading dimension
// ldc), the pass-2 partials (when the plan has several segments) and the
// counters {step index by parity, done (zero between launches), stop}.  A
// channel whose stop counter is nonzero is skipped by every kernel.
struct ArnoldiBatch {
    int nb;
    double2* V[C3L_MAX_BATCH];
    double2* w[C3L_MAX_BATCH];
    double2* xnext[C3L_MAX_BATCH];
    double2* c1[C3L_MAX_BATCH];
    double2* c2[C3L_MAX_BATCH];
    double* hval[C3L_MAX_BATCH];
    int32_t* counters[C3L_MAX_BATCH];
    double2* Hc[C3L_MAX_BATCH];
    double2* partial[C3L_MAX_BATCH];
    float2* V32[C3L_MAX_BATCH];   // FP32 copy of the basis rows (written with each row)
    float2* w32[C3L_MAX_BATCH];   // FP32 copy of the operator output (sigma), then of w' (first update)
    float2* V32lo[C3L_MAX_BATCH]; // V - V32 in FP32: rows as FP32 (hi, lo) pairs
    float2* w32lo[C3L_MAX_BATCH]; // w' - w32 in FP32 (first update)
    // optional: the sigma's padded input, written by the second update for the
    // next step (xws null: the sigma scatters its input itself)
    double2* xws[C3L_MAX_BATCH];
    const int64_t* xoff;          // [N + 1] entries of input element i: [xoff[i], xoff[i+1])
    const int64_t* xdst;
    const double* xsign;
};
// pass 1 (FP32, from the FP32 copies V32 and w32): c1[r] = V[r]^H w, r < k = counters[par] + 1
c3l_status arnoldi_dot1(const ArnoldiBatch& bt, int par, int64_t ld, int64_t dim, const RowDot& p, cudaStream_t s);
// w -= V[0 : k]^T c1 (double-float products and sums from the FP32 (hi, lo) rows, FP64
// subtraction); (w32, w32lo) receive the FP32 (hi, lo) pair of the result
c3l_status arnoldi_axpy1(const ArnoldiBatch& bt, int par, int64_t ld, int max_k, int64_t dim, cudaStream_t s);
// pass 2 (double-float products and sums on the FP32 pipe from the (hi, lo)
// pairs of the rows and of w, finished in FP64): c2[r] = V[r]^H w, c2[k] = |w|^2, h = sqrt(|w|^2 - |c2|^2),
// column k - 1 of Hc = (c1 + c2 | h), *hval = h, counters[1 - par] = k
c3l_status arnoldi_dot2(const ArnoldiBatch& bt, int par, int64_t ld, int64_t dim, const RowDot& p, int64_t ldc,
                        cudaStream_t s);
// V[k] = xnext = (w - V[0 : k]^T c2) / h (unscaled when h <= tol), V32[k] = (float) V[k];
// V c2 from FP32 products of the FP32 rows (c2 is the small second-pass correction);
// V32lo[k] = (float)(V[k] - V32[k])
c3l_status arnoldi_scale(const ArnoldiBatch& bt, int par, int64_t ld, int max_k, double tol, int64_t n,
                         cudaStream_t s);

// The sigma action on a batch of vectors (actions[b] share one program and
// differ in their workspace); an entry whose stop flag is set is skipped.
// out32 (may be null, or hold null entries): an FP32 copy of each output.
// skip_scatter: the padded input blocks are already written (by the Arnoldi
// step that formed xin).
c3l_status eom_sigma_batch(const c3l_eom_action* actions, int nb, const c3l_complex* const* xin,
                           c3l_complex* const* out, c3l_complex32* const* out32, const int32_t* const* stop,
                           cudaStream_t s, bool skip_scatter = false);
// True when two sigma actions run the same program (they may differ in ws).
bool same_sigma_program(const c3l_eom_action& a, const c3l_eom_action& b);

// GMRES (real) step: a short basis over a long vector.  Blocks own column
// segments for all rows; partial sums partial[block][R] are reduced by the
// block that finishes last.
struct GmPlan {
    int R;              // projection rows (restart + 2)
    int64_t seg;        // columns per block
    unsigned blocks;
    unsigned scale_grid;
};
GmPlan gm_plan(int64_t n, int max_rows, int sms);
// Pass-1 partial projections: partial[block][r] = V[r] . w on the block's
// segment (r < k), row k = |w|^2.  partial holds 2 x blocks x R doubles (pass 1
// in the first half, pass 2 in the second); consumers reduce the partials
// themselves in a fixed order, so no kernel waits for another block.
c3l_status gm_dot(const double* V, int64_t ld, const int* cur, const double* w, int64_t n, const GmPlan& p,
                  double* partial, cudaStream_t s);
// c1 = reduced pass 1 (block 0 stores it), w -= V[0 : k]^T c1, pass-2 partials
c3l_status gm_axpy_dot(const double* V, int64_t ld, const int* cur, double* c1, double* w, int64_t n, const GmPlan& p,
                       double* partial, cudaStream_t s);
// c2 = reduced pass 2, h0 = |w|, h = sqrt(|w'|^2 - |c2|^2); V[k] = xnext =
// (w - V c2) / h unless h <= eps h0; block 0 writes [c1 + c2 (k) | h | h0] to
// host-mapped slot j and *next = k
c3l_status gm_scale(double* V, int64_t ld, const int* cur, int* next, const double* partial, const double* c1,
                    double eps, const double* w, int64_t n, const GmPlan& p, double* xnext, double* slots, int stride,
                    cudaStream_t s);
// The same step over an FP32 basis (inner solves with the FP32 operator): wf
// (n floats) receives the work vector in FP32 and is updated in place; the
// partials and c1 are floats (c1: k + 1 entries); the slot column stays FP64.
c3l_status gm_dot_f32(const float* V, int64_t ld, const int* cur, const double* w, float* wf, int64_t n,
                      const GmPlan& p, float* partial, cudaStream_t s);
c3l_status gm_axpy_dot_f32(const float* V, int64_t ld, const int* cur, float* c1, float* wf, int64_t n,
                           const GmPlan& p, float* partial, cudaStream_t s);
c3l_status gm_scale_f32(float* V, int64_t ld, const int* cur, int* next, const float* partial, const float* c1,
                        double eps, const float* wf, int64_t n, const GmPlan& p, double* xnext, double* slots,
                        int stride, cudaStream_t s);
// FP32 (hi, lo) pair of a complex FP64 vector: hi = (float) x, lo = (float)(x - hi)
c3l_status split_c(int64_t n, const c3l_complex* x, c3l_complex32* hi, c3l_complex32* lo, cudaStream_t s);
// V0 = (float)(a r) and x = V0 (FP64 copy)
c3l_status gm_start_f32(int64_t n, double a, const double* r, float* V0, double* x, cudaStream_t s);
// x += V[0 : k]^T y (FP32 rows, FP64 arithmetic)
c3l_status gm_update_f32(const float* V, int64_t ld, int k, const double* y, double* x, int64_t n, cudaStream_t s);


// The FP32 pair GEMMs of a program on the tcgen05 tensor cores (c3l_tcgen05.cu).
c3l_status pair_gemm_tc(const c3l_pair_program& pp, float2* ws, bool pdl, cudaStream_t s);

// c3l_hessenberg_advance for several states in one launch (up to 16): the
// rotation chains of all channels fill the GPU together.
c3l_status hessenberg_advance_many(c3l_hessenberg_state* const* states, const c3l_complex* const* Hc,
                                   const int64_t* ldc, const int32_t* m, int count, cudaStream_t s);

}  // namespace c3l

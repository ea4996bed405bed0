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
#define C3L_GMRES_MAX_ROWS 256

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

// out[r] = V[r]^H w (r < k) [and |w|^2 at r = k when self]
c3l_status dot_rows_dev_c(const c3l_complex* V, int64_t ld, const int* cur, int self, const c3l_complex* w,
                          int64_t dim, const RowDot& p, c3l_complex* partial, c3l_complex* out, cudaStream_t s);
// The same projections with FP32 products and sums (first CGS2 pass only).
c3l_status dot_rows_f32acc_dev_c(const c3l_complex* V, int64_t ld, const int* cur, const c3l_complex* w, int64_t dim,
                                 const RowDot& p, c3l_complex* out, cudaStream_t s);
// Pass-2 projections with the Arnoldi column: c2[r] = V[r]^H w (r < k),
// c2[k] = |w|^2, then h = sqrt(|w|^2 - |c2|^2), column j = k - 1 of Hc
// (c1 + c2 | h), *hval = h and *next = k (done: zero between launches).
c3l_status dot_rows_column_dev_c(const c3l_complex* V, int64_t ld, const int* cur, int* next, const c3l_complex* w,
                                 int64_t dim, const RowDot& p, c3l_complex* partial, unsigned* done,
                                 const c3l_complex* c1, c3l_complex* c2, c3l_complex* Hc, int64_t ldc, double* hval,
                                 cudaStream_t s);
// w += alpha * V[0 : k]^T c
c3l_status axpy_dev_c(const c3l_complex* V, int64_t ld, const int* cur, int max_k, const c3l_complex* c,
                      c3l_complex alpha, c3l_complex* w, int64_t dim, cudaStream_t s);
// V[k] = xnext = (w - V[0 : k]^T c2) / h (unscaled when h <= tol)
c3l_status arnoldi_scale_dev(c3l_complex* V, int64_t ld, const int* cur, int max_k, const c3l_complex* c2,
                             const double* hval, double tol, const c3l_complex* w, int64_t n, c3l_complex* xnext,
                             cudaStream_t s);

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
// V0 = (float)(a r) and x = V0 (FP64 copy)
c3l_status gm_start_f32(int64_t n, double a, const double* r, float* V0, double* x, cudaStream_t s);
// x += V[0 : k]^T y (FP32 rows, FP64 arithmetic)
c3l_status gm_update_f32(const float* V, int64_t ld, int k, const double* y, double* x, int64_t n, cudaStream_t s);


// c3l_hessenberg_advance for several states in one launch (up to 16): the
// rotation chains of all channels fill the GPU together.
c3l_status hessenberg_advance_many(c3l_hessenberg_state* const* states, const c3l_complex* const* Hc,
                                   const int64_t* ldc, const int32_t* m, int count, cudaStream_t s);

}  // namespace c3l

// Krylov kernels of the coupled-cluster hot path (sm_103a).
//
//  * c3l_multi_dot_{c,r}  : k projections V^H w in one launch pair
//                           (deterministic two-pass reduction, warp shuffles)
//  * c3l_multi_axpy_{c,r} : w += alpha * V c   (one pass over w, k-term sums)
//  * c3l_precondition     : 2x2 real blocks of pack(unpack(x) / diag)
//  * c3l_hessenberg_*     : shifted upper-Hessenberg solves for all shifts,
//                           one thread block per shift, streamed Givens QR.
//
// Classical Gram-Schmidt twice (CGS2) is composed on the host from two
// multi_dot/multi_axpy pairs, exactly the two BLAS passes of the reference
// (src/c3l/green/krylov.py:362-373), so each pass streams the basis once.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>
#include <type_traits>

#include "c3l_gb300.h"
#include "c3l_internal.h"
#include "c3l_df.h"
#include "c3l_pdl.h"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxPartial = 256;
constexpr int kHessThreads = 128;

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }
inline c3l_status launch_status() { return cudaGetLastError() == cudaSuccess ? C3L_OK : C3L_ERR_LAUNCH; }

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cconjmul(double2 a, double2 b) {  // conj(a) * b
    return make_double2(fma(a.x, b.x, a.y * b.y), fma(a.x, b.y, -a.y * b.x));
}
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    // Smith's algorithm
    if (fabs(b.x) >= fabs(b.y)) {
        const double r = b.y / b.x;
        const double d = b.x + b.y * r;
        return make_double2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
    }
    const double r = b.x / b.y;
    const double d = b.y + b.x * r;
    return make_double2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of one double; result valid in thread 0.
__device__ double block_sum(double v, double* smem) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) smem[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = (lane < (int)(blockDim.x >> 5)) ? smem[lane] : 0.0;
        v = warp_sum(v);
    }
    return v;
}

int64_t partial_blocks(int32_t k, int64_t dim) {
    int64_t nb = (dim + 4 * kThreads - 1) / (4 * kThreads);
    const int64_t cap = k > 0 ? (1216 + k - 1) / k : 1;  // ~8 resident blocks per SM overall
    if (nb > cap) nb = cap;
    if (nb > kMaxPartial) nb = kMaxPartial;
    if (nb < 1) nb = 1;
    return nb;
}

__global__ void __launch_bounds__(kThreads) k_dot_partial_c(const double2* __restrict__ V, int64_t ld,
                                                            const double2* __restrict__ w, int64_t dim,
                                                            double2* __restrict__ partial) {
    __shared__ double sm[32];
    const int j = blockIdx.y;
    const double2* v = V + (int64_t)j * ld;
    double re = 0.0, im = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 p = cconjmul(v[i], w[i]);
        re += p.x;
        im += p.y;
    }
    re = block_sum(re, sm);
    im = block_sum(im, sm);
    if (threadIdx.x == 0) partial[(int64_t)j * gridDim.x + blockIdx.x] = make_double2(re, im);
}

// Single pass for short vectors: one block per row reduces the whole row
// (deterministic order), so no partial buffer or second launch is needed.
// The Arnoldi basis of an EOM block is a few thousand entries long.
constexpr int64_t kRowDotMax = 8192;

__global__ void __launch_bounds__(kThreads) k_dot_rows_c(const double2* __restrict__ V, int64_t ld,
                                                         const double2* __restrict__ w, int64_t dim,
                                                         double2* __restrict__ out) {
    __shared__ double sm[32];
    const int j = blockIdx.x;
    const double2* v = V + (int64_t)j * ld;
    double re = 0.0, im = 0.0;
    const int64_t step = blockDim.x;
    int64_t i = threadIdx.x;
    for (; i + 3 * step < dim; i += 4 * step) {  // four independent loads in flight
        double2 a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            a[u] = v[i + u * step];
            b[u] = w[i + u * step];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            re = fma(a[u].x, b[u].x, fma(a[u].y, b[u].y, re));
            im = fma(a[u].x, b[u].y, fma(-a[u].y, b[u].x, im));
        }
    }
    for (; i < dim; i += step) {
        const double2 a = v[i], b = w[i];
        re = fma(a.x, b.x, fma(a.y, b.y, re));
        im = fma(a.x, b.y, fma(-a.y, b.x, im));
    }
    re = block_sum(re, sm);
    im = block_sum(im, sm);
    if (threadIdx.x == 0) out[j] = make_double2(re, im);
}

__global__ void __launch_bounds__(kThreads) k_dot_partial_r(const double* __restrict__ V, int64_t ld,
                                                            const double* __restrict__ w, int64_t dim,
                                                            double* __restrict__ partial) {
    __shared__ double sm[32];
    const int j = blockIdx.y;
    const double* v = V + (int64_t)j * ld;
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x)
        s = fma(v[i], w[i], s);
    s = block_sum(s, sm);
    if (threadIdx.x == 0) partial[(int64_t)j * gridDim.x + blockIdx.x] = s;
}

__global__ void k_dot_final_c(const double2* __restrict__ partial, int nb, double2* __restrict__ out) {
    __shared__ double sm[32];
    const int j = blockIdx.x;
    double re = 0.0, im = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        re += partial[(int64_t)j * nb + b].x;
        im += partial[(int64_t)j * nb + b].y;
    }
    re = block_sum(re, sm);
    im = block_sum(im, sm);
    if (threadIdx.x == 0) out[j] = make_double2(re, im);
}

__global__ void k_dot_final_r(const double* __restrict__ partial, int nb, double* __restrict__ out) {
    __shared__ double sm[32];
    const int j = blockIdx.x;
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += partial[(int64_t)j * nb + b];
    s = block_sum(s, sm);
    if (threadIdx.x == 0) out[j] = s;
}

// w[i] += alpha * sum_j c[j] V[j, i]: an X x Y block covers X consecutive
// entries (coalesced in i) and splits the k rows over Y thread rows.  A long
// basis over a short vector (Arnoldi on an EOM block) uses 4 x 64 blocks so
// that the grid spans every SM; short bases use 32 x 8.
constexpr int kAxX = 32, kAxY = 8;
constexpr int kAxXLong = 4, kAxYLong = 64;

template <int X, int Y>
__global__ void __launch_bounds__(X * Y) k_axpy_c(const double2* __restrict__ V, int64_t ld, int k,
                                                   const double2* __restrict__ c, double2 alpha,
                                                   double2* __restrict__ w, int64_t dim) {
    __shared__ double2 part[Y][X];
    for (int64_t base = (int64_t)blockIdx.x * X; base < dim; base += (int64_t)gridDim.x * X) {
        const int64_t i = base + threadIdx.x;
        double2 s = make_double2(0.0, 0.0);
        if (i < dim) {
            int j = threadIdx.y;
            for (; j + 3 * Y < k; j += 4 * Y) {  // four independent loads in flight
                double2 cj[4], v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    cj[u] = c[j + u * Y];
                    v[u] = V[(int64_t)(j + u * Y) * ld + i];
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    s.x = fma(cj[u].x, v[u].x, fma(-cj[u].y, v[u].y, s.x));
                    s.y = fma(cj[u].x, v[u].y, fma(cj[u].y, v[u].x, s.y));
                }
            }
            for (; j < k; j += Y) {
                const double2 cj = c[j], v = V[(int64_t)j * ld + i];
                s.x = fma(cj.x, v.x, fma(-cj.y, v.y, s.x));
                s.y = fma(cj.x, v.y, fma(cj.y, v.x, s.y));
            }
        }
        part[threadIdx.y][threadIdx.x] = s;
        __syncthreads();
        // tree over the Y partial rows
        for (int h = Y / 2; h > 0; h >>= 1) {
            if ((int)threadIdx.y < h) {
                const double2 o = part[threadIdx.y + h][threadIdx.x];
                part[threadIdx.y][threadIdx.x].x += o.x;
                part[threadIdx.y][threadIdx.x].y += o.y;
            }
            __syncthreads();
        }
        if (threadIdx.y == 0 && i < dim) {
            const double2 a = cmul(alpha, part[0][threadIdx.x]);
            w[i] = make_double2(w[i].x + a.x, w[i].y + a.y);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kAxX * kAxY) k_axpy_r(const double* __restrict__ V, int64_t ld, int k,
                                                         const double* __restrict__ c, double alpha,
                                                         double* __restrict__ w, int64_t dim) {
    __shared__ double part[kAxY][kAxX];
    for (int64_t base = (int64_t)blockIdx.x * kAxX; base < dim; base += (int64_t)gridDim.x * kAxX) {
        const int64_t i = base + threadIdx.x;
        double s = 0.0;
        if (i < dim)
            for (int j = threadIdx.y; j < k; j += kAxY) s = fma(c[j], V[(int64_t)j * ld + i], s);
        part[threadIdx.y][threadIdx.x] = s;
        __syncthreads();
        if (threadIdx.y == 0 && i < dim) {
            double t = part[0][threadIdx.x];
#pragma unroll
            for (int y = 1; y < kAxY; ++y) t += part[y][threadIdx.x];
            w[i] = fma(alpha, t, w[i]);
        }
        __syncthreads();
    }
}

__global__ void k_scale_c(int64_t dim, double2 a, const double2* __restrict__ x, double2* __restrict__ y) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = cmul(a, x[i]);
}

__global__ void k_scale_r(int64_t dim, double a, const double* __restrict__ x, double* __restrict__ y) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = a * x[i];
}

__global__ void k_precondition(int64_t nrep, const double* __restrict__ m4, const int64_t* __restrict__ col,
                               const int64_t* __restrict__ pair, const double* __restrict__ x, double* __restrict__ y) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrep; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = col[r];
        const double* m = m4 + 4 * r;
        if (pair[r]) {
            const double a = x[c], b = x[c + 1];
            y[c] = fma(m[0], a, m[1] * b);
            y[c + 1] = fma(m[2], a, m[3] * b);
        } else {
            y[c] = m[0] * x[c];
        }
    }
}

// out = inv * (z x - s) elementwise (s == NULL: 0; inv == NULL: 1)
__global__ void k_shifted_combine(int64_t dim, double2 z, const double2* __restrict__ x, const double2* __restrict__ s,
                                  const double2* __restrict__ inv, double2* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x) {
        double2 v = cmul(z, x[i]);
        if (s) v = make_double2(v.x - s[i].x, v.y - s[i].y);
        out[i] = inv ? cmul(inv[i], v) : v;
    }
}

unsigned axpy_grid(int64_t dim, int x = kAxX) {
    int64_t b = (dim + x - 1) / x;
    if (b > 8192) b = 8192;
    return (unsigned)(b < 1 ? 1 : b);
}

unsigned grid_for(int64_t count) {
    int64_t b = (count + kThreads - 1) / kThreads;
    if (b < 1) b = 1;
    if (b > 4096) b = 4096;
    return (unsigned)b;
}

// ---------------------------------------------------------------- Hessenberg
// Row k+1 of A = z I - H, entry at column c (c >= k).
__device__ __forceinline__ double2 a_entry(const double2* H, int64_t ldh, int row, int c, double2 z) {
    const double2 h = H[(int64_t)row * ldh + c];
    return (row == c) ? make_double2(z.x - h.x, z.y - h.y) : make_double2(-h.x, -h.y);
}

// Givens rotation (real c, complex s) with c*a + s*b = r and -conj(s)*a + c*b = 0.
__device__ __forceinline__ void givens(double2 a, double2 b, double& c, double2& s, double2& r) {
    const double na = hypot(a.x, a.y);
    const double nb = hypot(b.x, b.y);
    if (nb == 0.0) {
        c = 1.0;
        s = make_double2(0.0, 0.0);
        r = a;
        return;
    }
    if (na == 0.0) {
        c = 0.0;
        s = make_double2(1.0, 0.0);
        r = b;
        return;
    }
    const double rho = hypot(na, nb);
    c = na / rho;
    const double2 ph = make_double2(a.x / na, a.y / na);
    s = cmul(ph, make_double2(b.x / rho, -b.y / rho));  // (a/|a|) conj(b) / rho
    r = make_double2(ph.x * rho, ph.y * rho);
}

// The same rotation with v = num / r, from two reciprocal square roots instead
// of hypot and divisions: c = |a|/rho, s = ph conj(b)/rho, r = ph rho with
// ph = a/|a|, hence num / r = num conj(ph) / rho.  Falls back to the careful
// form when |a|^2 is outside the safe range.
__device__ __forceinline__ void givens_fast(double2 a, double2 b, double2 num, bool want_v, double& c, double2& s,
                                            double2& v) {
    const double na2 = fma(a.x, a.x, a.y * a.y);
    const double nb2 = fma(b.x, b.x, b.y * b.y);
    if (!(na2 > 1e-280 && na2 < 1e280 && nb2 < 1e280)) {
        double2 r;
        givens(a, b, c, s, r);
        v = want_v ? cdiv(num, r) : make_double2(0.0, 0.0);
        return;
    }
    const double inv_na = rsqrt(na2);
    const double inv_rho = rsqrt(na2 + nb2);
    c = na2 * inv_na * inv_rho;
    const double2 ph = make_double2(a.x * inv_na, a.y * inv_na);
    s = cmul(ph, make_double2(b.x * inv_rho, -b.y * inv_rho));
    if (want_v) {
        const double2 t = cconjmul(ph, num);  // conj(ph) num
        v = make_double2(t.x * inv_rho, t.y * inv_rho);
    } else {
        v = make_double2(0.0, 0.0);
    }
}

// The same rotation and v = num / r from one reciprocal square root:
// inv = 1 / (|a| rho) gives c = |a|^2 inv, s = a conj(b) inv and
// 1 / r = conj(a) inv (r = a rho / |a|).  Falls back to the careful form
// when |a|^2 rho^2 leaves the safe range.
__device__ __forceinline__ void givens_one_rsqrt(double2 a, double2 b, double2 num, bool want_v, double& c,
                                                 double2& s, double2& v) {
    const double na2 = fma(a.x, a.x, a.y * a.y);
    const double nb2 = fma(b.x, b.x, b.y * b.y);
    const double q = na2 * (na2 + nb2);
    if (!(q > 1e-290 && q < 1e290)) {
        double2 r;
        givens(a, b, c, s, r);
        v = want_v ? cdiv(num, r) : make_double2(0.0, 0.0);
        return;
    }
    const double inv = rsqrt(q);
    c = na2 * inv;
    const double2 ab = cconjmul(b, a);  // a conj(b)
    s = make_double2(ab.x * inv, ab.y * inv);
    if (want_v) {
        const double2 t = cconjmul(a, num);  // conj(a) num
        v = make_double2(t.x * inv, t.y * inv);
    } else {
        v = make_double2(0.0, 0.0);
    }
}

// Streamed Givens QR of (z I - H_m) with the transposed forward solve
// u = R^{-T} p, so that green = p^T y = sum_k u_k (Q^H beta e1)_k without
// storing R.  Shared memory: w[m] (current working row), acc[m].  Thread 0
// alone forms each rotation (FP64 is a narrow pipe on this part: the
// rotation is computed once per step, not once per thread); all threads then
// update the remaining columns.
__global__ void __launch_bounds__(kHessThreads) k_hessenberg_shifted(const double2* __restrict__ H, int64_t ldh, int m,
                                                                     const double2* __restrict__ shifts, double beta,
                                                                     const double2* __restrict__ sinkproj,
                                                                     double2* __restrict__ green,
                                                                     double* __restrict__ residual) {
    extern __shared__ double2 dyn[];
    double2* w = dyn;
    double2* acc = dyn + m;
    __shared__ double rot_c;
    __shared__ double2 rot_s, u_k;
    const double2 z = shifts[blockIdx.x];
    for (int c = threadIdx.x; c < m; c += blockDim.x) {
        w[c] = a_entry(H, ldh, 0, c, z);
        acc[c] = make_double2(0.0, 0.0);
    }
    // thread-0 state
    double2 rhs_w = make_double2(beta, 0.0);
    double2 G = make_double2(0.0, 0.0);
    double2 ylast = make_double2(0.0, 0.0);
    __syncthreads();
    for (int k = 0; k < m; ++k) {
        if (threadIdx.x == 0) {
            double c;
            double2 s, rkk;
            if (k < m - 1) {
                givens(w[k], a_entry(H, ldh, k + 1, k, z), c, s, rkk);
            } else {
                c = 1.0;
                s = make_double2(0.0, 0.0);
                rkk = w[k];
            }
            const double2 rrhs = make_double2(c * rhs_w.x, c * rhs_w.y);
            rhs_w = cmul(make_double2(-s.x, s.y), rhs_w);  // -conj(s) * rhs_w (the next row's rhs is 0)
            double2 u = make_double2(0.0, 0.0);
            if (sinkproj) {
                const double2 p = sinkproj[k];
                u = cdiv(make_double2(p.x - acc[k].x, p.y - acc[k].y), rkk);
                const double2 gu = cmul(u, rrhs);
                G.x += gu.x;
                G.y += gu.y;
            }
            if (k == m - 1) ylast = cdiv(rrhs, rkk);
            rot_c = c;
            rot_s = s;
            u_k = u;
        }
        __syncthreads();
        const double cc = rot_c;
        const double2 ss = rot_s;
        const double2 u = u_k;
        const double2 mcs = make_double2(-ss.x, ss.y);  // -conj(s)
        for (int col = k + 1 + threadIdx.x; col < m; col += blockDim.x) {
            const double2 rv = (k < m - 1) ? a_entry(H, ldh, k + 1, col, z) : make_double2(0.0, 0.0);
            const double2 wv = w[col];
            const double2 s_rv = cmul(ss, rv);
            const double2 rk = make_double2(fma(cc, wv.x, s_rv.x), fma(cc, wv.y, s_rv.y));
            const double2 nw = cmul(mcs, wv);
            w[col] = make_double2(fma(cc, rv.x, nw.x), fma(cc, rv.y, nw.y));
            if (sinkproj) {
                const double2 t = cmul(rk, u);
                acc[col] = make_double2(acc[col].x + t.x, acc[col].y + t.y);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (green) green[blockIdx.x] = G;
        if (residual) {
            const double2 hs = H[(int64_t)m * ldh + (m - 1)];
            const double2 t = cmul(hs, ylast);
            residual[blockIdx.x] = hypot(t.x, t.y) / beta;
        }
    }
}

// Incremental shifted solves for Arnoldi convergence checks and the final
// Green function.  The Givens QR of the Hessenberg matrix (z I - H) is
// column-incremental: the rotations G_0..G_{j-1} of the first j columns do not
// change when columns are appended.  Each call processes the new columns
// [j0, j1) of every shift once, storing per shift and column the rotation
// (c_j real, s_j complex) and v_j of the transposed sink solve R^T v = p, so
// that the square system of any dimension m gives
//   y_{m-1} = g'_{m-1} / pivot,  residual = |h_{m,m-1}| |y_{m-1}| / beta,
//   green   = sum_{j<m-1} v_j g_j + v'_{m-1} g'_{m-1}
// from O(1) per-shift scalars (g' the rotated right-hand side entry carried
// into the next row, acc = sum v_j g_j over finalized columns).  Over a whole
// Arnoldi run each shift costs one O(m^2/2) elimination instead of one per
// check.
//
// Entry (r, c) of z I - H for a column-major Hessenberg (column c at col).
__device__ __forceinline__ double2 shifted_entry(const double2* __restrict__ col, int r, int c, double2 z) {
    const double2 h = col[r];
    return (r == c) ? make_double2(z.x - h.x, z.y - h.y) : make_double2(-h.x, -h.y);
}

__device__ __forceinline__ double2 shfl2(double2 v, int src) {
    return make_double2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

__device__ __forceinline__ double2 cadd2(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

// Several channels' advances in one launch (blockIdx.y = channel), so that
// the rotation chains of all channels fill the GPU together.  Layout: a warp
// holds kMjShifts shifts x kMjLanes columns; lane t of a shift advances column
// cs + t of a chunk, applying the finalized rotations of rows 0..cs-1 in
// sequence (register double-buffered prefetch) and then the in-chunk
// rotations, each formed by lane p and broadcast by shuffles.
constexpr int kMjLanes = 8;
constexpr int kMjShifts = 32 / kMjLanes;
constexpr int kMjDepth = 4;
constexpr int kMaxAdvJobs = 16;

struct AdvJob {
    const double2* Hc;
    int64_t ldc;
    int j0, j1;
    const double2* shifts;
    int nshift;
    double beta, btol;
    const double2* sinkc;
    double* rot_c;
    double2* rot_s;
    double2* vs;
    double2* carry;
    double2* accum;
    double2* green;
    double* residual;
    c3l_hessenberg_status* status;
};

struct AdvJobs {
    AdvJob job[kMaxAdvJobs];
    int count;
};

__global__ void __launch_bounds__(32) k_hessenberg_advance_jobs(AdvJobs jobs) {
    const AdvJob& jb = jobs.job[blockIdx.y];
    const double2* __restrict__ Hc = jb.Hc;
    const int64_t ldc = jb.ldc;
    const int j0 = jb.j0, j1 = jb.j1, nshift = jb.nshift;
    const double2* __restrict__ sinkc = jb.sinkc;
    const double* __restrict__ rot_c_r = jb.rot_c;
    const double2* __restrict__ rot_s_r = jb.rot_s;
    const double2* __restrict__ vs_r = jb.vs;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int t = lane & (kMjLanes - 1);
    const int sraw = blockIdx.x * kMjShifts + (lane / kMjLanes);
    if (blockIdx.x * kMjShifts >= nshift) return;  // whole block past this channel's shifts (uniform)
    const bool live = sraw < nshift;
    const int sh = live ? sraw : nshift - 1;
    const double2 z = jb.shifts[sh];
    const double2 zero2 = make_double2(0.0, 0.0);
    double2 g = j0 == 0 ? make_double2(jb.beta, 0.0) : jb.carry[sh];
    double2 acc = j0 == 0 ? zero2 : jb.accum[sh];
    bool stop = false;
    for (int cs = j0; cs < j1 && !stop; cs += kMjLanes) {
        const int c = min(cs + t, j1 - 1);  // lanes past j1 shadow the last column (never stored)
        const double2* col = Hc + (int64_t)c * ldc;
        double2 x = shifted_entry(col, 0, c, z);
        double2 dot = zero2;
        // rows i < cs - 1 are off the diagonal (c >= cs): entry a = -h
        auto rotate_h = [&](double ci, double2 si, double2 h, double2 v) {
            const double2 shh = cmul(si, h);
            const double2 r = make_double2(fma(ci, x.x, -shh.x), fma(ci, x.y, -shh.y));
            const double2 sx = cconjmul(si, x);
            x = make_double2(fma(-ci, h.x, -sx.x), fma(-ci, h.y, -sx.y));
            dot = make_double2(fma(r.x, v.x, fma(-r.y, v.y, dot.x)), fma(r.x, v.y, fma(r.y, v.x, dot.y)));
        };
        double bc[2][kMjDepth];
        double2 bs[2][kMjDepth], bv[2][kMjDepth], bh[2][kMjDepth];
        auto fetch = [&](int buf, int i0) {
#pragma unroll
            for (int u = 0; u < kMjDepth; ++u) {
                const int64_t at = (int64_t)(i0 + u) * nshift + sh;
                bc[buf][u] = rot_c_r[at];
                bs[buf][u] = rot_s_r[at];
                bv[buf][u] = sinkc ? vs_r[at] : zero2;
                bh[buf][u] = col[i0 + u + 1];
            }
        };
        const int offdiag = cs > 0 ? cs - 1 : 0;
        const int groups = offdiag / kMjDepth;
        if (groups > 0) fetch(0, 0);
        for (int gi = 0; gi < groups; gi += 2) {
            if (gi + 1 < groups) fetch(1, (gi + 1) * kMjDepth);
#pragma unroll
            for (int u = 0; u < kMjDepth; ++u) rotate_h(bc[0][u], bs[0][u], bh[0][u], bv[0][u]);
            if (gi + 1 >= groups) break;
            if (gi + 2 < groups) fetch(0, (gi + 2) * kMjDepth);
#pragma unroll
            for (int u = 0; u < kMjDepth; ++u) rotate_h(bc[1][u], bs[1][u], bh[1][u], bv[1][u]);
        }
        for (int i = groups * kMjDepth; i < offdiag; ++i) {
            const int64_t at = (int64_t)i * nshift + sh;
            rotate_h(rot_c_r[at], rot_s_r[at], col[i + 1], sinkc ? vs_r[at] : zero2);
        }
        if (cs > 0) {  // last finalized rotation: row cs may be this column's diagonal
            const int64_t at = (int64_t)(cs - 1) * nshift + sh;
            const double2 a = shifted_entry(col, cs, c, z);
            rotate_h(rot_c_r[at], rot_s_r[at], make_double2(-a.x, -a.y), sinkc ? vs_r[at] : zero2);
        }
        // in-chunk rotations
        for (int p = 0; p < kMjLanes; ++p) {
            const int cq = cs + p;
            if (cq >= j1) break;
            const double2 hsub = Hc[(int64_t)cq * ldc + cq + 1];
            const bool brk = !(fabs(hsub.x) > jb.btol);
            double fc = 0.0;
            double2 fs = zero2, fv = zero2;
            if (t == p) {
                const double2 u = sinkc ? make_double2(sinkc[cq].x, -sinkc[cq].y) : zero2;
                const double2 num = make_double2(u.x - dot.x, u.y - dot.y);
                if (cq == j1 - 1 || brk) {
                    const double2 y = cdiv(g, x);
                    const double res = hypot(hsub.x, hsub.y) * hypot(y.x, y.y) / jb.beta;
                    double2 gr = acc;
                    if (sinkc) gr = cadd2(acc, cmul(cdiv(num, x), g));
                    if (live) {
                        jb.residual[sh] = res;
                        if (jb.green) jb.green[sh] = gr;
                        if (isfinite(res) && isfinite(gr.x) && isfinite(gr.y)) {
                            atomicMax(&jb.status->worst, (unsigned long long)__double_as_longlong(res));
                        } else {
                            atomicExch(&jb.status->bad, 1);
                        }
                        if (brk) jb.status->first_break = cq + 1;
                    }
                }
                if (!brk) {
                    givens_one_rsqrt(x, make_double2(-hsub.x, -hsub.y), num, sinkc != nullptr, fc, fs, fv);
                    acc = cadd2(acc, cmul(fv, make_double2(fc * g.x, fc * g.y)));
                    g = cconjmul(fs, g);
                    g = make_double2(-g.x, -g.y);
                    if (live) {
                        const int64_t at = (int64_t)cq * nshift + sh;
                        jb.rot_c[at] = fc;
                        jb.rot_s[at] = fs;
                        jb.vs[at] = fv;
                    }
                }
            }
            if (brk) {
                stop = true;
                break;
            }
            const int src = (lane & ~(kMjLanes - 1)) + p;
            fc = __shfl_sync(full, fc, src);
            fs = shfl2(fs, src);
            fv = shfl2(fv, src);
            g = shfl2(g, src);
            acc = shfl2(acc, src);
            if (t > p) {
                const double2 a = shifted_entry(col, cq + 1, c, z);
                const double2 sa = cmul(fs, a);
                const double2 r = make_double2(fma(fc, x.x, sa.x), fma(fc, x.y, sa.y));
                const double2 sx = cconjmul(fs, x);
                x = make_double2(fma(fc, a.x, -sx.x), fma(fc, a.y, -sx.y));
                if (sinkc) dot = make_double2(fma(r.x, fv.x, fma(-r.y, fv.y, dot.x)), fma(r.x, fv.y, fma(r.y, fv.x, dot.y)));
            }
        }
        __syncwarp();
    }
    if (t == 0 && live) {
        jb.carry[sh] = g;
        jb.accum[sh] = acc;
    }
}

// Same elimination storing R (packed rows) in caller scratch, then back
// substitution for the full reduced coordinates y.
__global__ void __launch_bounds__(kHessThreads) k_hessenberg_coordinates(const double2* __restrict__ H, int64_t ldh, int m,
                                                                         const double2* __restrict__ shifts, double beta,
                                                                         double2* __restrict__ rscratch,
                                                                         double2* __restrict__ Y) {
    extern __shared__ double2 dyn[];
    double2* w = dyn;        // working row
    double2* rr = dyn + m;   // R rhs, then y
    __shared__ double rot_c;
    __shared__ double2 rot_s;
    __shared__ double red[64];
    const double2 z = shifts[blockIdx.x];
    double2* R = rscratch + (int64_t)blockIdx.x * ((int64_t)m * (m + 1) / 2);
    for (int c = threadIdx.x; c < m; c += blockDim.x) w[c] = a_entry(H, ldh, 0, c, z);
    double2 rhs_w = make_double2(beta, 0.0);
    __syncthreads();
    for (int k = 0; k < m; ++k) {
        const int64_t row = (int64_t)k * m - (int64_t)k * (k - 1) / 2;  // packed row start (length m-k)
        if (threadIdx.x == 0) {
            double c;
            double2 s, rkk;
            if (k < m - 1) {
                givens(w[k], a_entry(H, ldh, k + 1, k, z), c, s, rkk);
            } else {
                c = 1.0;
                s = make_double2(0.0, 0.0);
                rkk = w[k];
            }
            rot_c = c;
            rot_s = s;
            R[row] = rkk;
            rr[k] = make_double2(c * rhs_w.x, c * rhs_w.y);
            rhs_w = cmul(make_double2(-s.x, s.y), rhs_w);
        }
        __syncthreads();
        const double cc = rot_c;
        const double2 ss = rot_s;
        const double2 mcs = make_double2(-ss.x, ss.y);
        for (int col = k + 1 + threadIdx.x; col < m; col += blockDim.x) {
            const double2 rv = (k < m - 1) ? a_entry(H, ldh, k + 1, col, z) : make_double2(0.0, 0.0);
            const double2 wv = w[col];
            const double2 s_rv = cmul(ss, rv);
            R[row + (col - k)] = make_double2(fma(cc, wv.x, s_rv.x), fma(cc, wv.y, s_rv.y));
            const double2 nw = cmul(mcs, wv);
            w[col] = make_double2(fma(cc, rv.x, nw.x), fma(cc, rv.y, nw.y));
        }
        __syncthreads();
    }
    // back substitution: y_k = (rr_k - sum_{c>k} R_kc y_c) / R_kk, y stored in rr
    for (int k = m - 1; k >= 0; --k) {
        const int64_t row = (int64_t)k * m - (int64_t)k * (k - 1) / 2;
        double re = 0.0, im = 0.0;
        for (int col = k + 1 + threadIdx.x; col < m; col += blockDim.x) {
            const double2 t = cmul(R[row + (col - k)], rr[col]);
            re += t.x;
            im += t.y;
        }
        re = block_sum(re, red);
        im = block_sum(im, red + 32);
        if (threadIdx.x == 0) {
            const double2 num = make_double2(rr[k].x - re, rr[k].y - im);
            rr[k] = cdiv(num, R[row]);
        }
        __syncthreads();
    }
    for (int c = threadIdx.x; c < m; c += blockDim.x) Y[(int64_t)blockIdx.x * m + c] = rr[c];
}

// One Arnoldi column on the device: H[:k, j] = c1 + c2, h = |w'' | from
// |w'|^2 - |c2|^2, H[k, j] = h (column-major Hc, ld = ldc), then w /= h
// unless h <= tol (breakdown: w is left as is and detected by the host).
// coeff: [c1 (k) | c2 (k) | |w'|^2].
__global__ void k_arnoldi_column(const double2* __restrict__ coeff, int k, double2* __restrict__ w, int64_t n,
                                 double2* __restrict__ Hc, int64_t ldc, int j, double tol) {
    __shared__ double red[32];
    double s = 0.0;
    for (int i = threadIdx.x; i < k; i += blockDim.x) {
        const double2 c2 = coeff[k + i];
        s += c2.x * c2.x + c2.y * c2.y;
    }
    s = block_sum(s, red);
    __shared__ double h_sh;
    if (threadIdx.x == 0) h_sh = sqrt(fmax(coeff[2 * k].x - s, 0.0));
    __syncthreads();
    const double h = h_sh;
    if (blockIdx.x == 0) {
        double2* col = Hc + (int64_t)j * ldc;
        for (int i = threadIdx.x; i < k; i += blockDim.x)
            col[i] = make_double2(coeff[i].x + coeff[k + i].x, coeff[i].y + coeff[k + i].y);
        if (threadIdx.x == 0) col[k] = make_double2(h, 0.0);
    }
    if (!(h > tol)) return;
    const double inv = 1.0 / h;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        w[i] = make_double2(w[i].x * inv, w[i].y * inv);
}

// ------------------------------------------------- device-indexed steps
// Kernels of one Krylov step whose row count k = *jdev + 1 is read from device
// memory (see c3l_internal.h).
constexpr int64_t kSegLen = 4096;

__device__ __forceinline__ void dot_acc(double& s, double a, double b) { s = fma(a, b, s); }
__device__ __forceinline__ void dot_acc(double2& s, double2 a, double2 b) {  // += conj(a) b
    s.x = fma(a.x, b.x, fma(a.y, b.y, s.x));
    s.y = fma(a.x, b.y, fma(-a.y, b.x, s.y));
}
__device__ __forceinline__ void axpy_acc(double& s, double c, double v) { s = fma(c, v, s); }
__device__ __forceinline__ void axpy_acc(double2& s, double2 c, double2 v) {  // += c v
    s.x = fma(c.x, v.x, fma(-c.y, v.y, s.x));
    s.y = fma(c.x, v.y, fma(c.y, v.x, s.y));
}
__device__ __forceinline__ void dot_acc_plain(double& s, double v) { s += v; }
__device__ __forceinline__ void dot_acc_plain(double2& s, double2 v) {
    s.x += v.x;
    s.y += v.y;
}
__device__ __forceinline__ double norm2(double v) { return v * v; }
__device__ __forceinline__ double norm2(double2 v) { return fma(v.x, v.x, v.y * v.y); }
__device__ __forceinline__ double real_of(double v) { return v; }
__device__ __forceinline__ double real_of(double2 v) { return v.x; }
__device__ __forceinline__ double sum_of(double a, double b) { return a + b; }
__device__ __forceinline__ double2 sum_of(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ T from_real(double v);
template <> __device__ __forceinline__ double from_real<double>(double v) { return v; }
template <> __device__ __forceinline__ double2 from_real<double2>(double v) { return make_double2(v, 0.0); }
__device__ __forceinline__ double scaled_diff(double w, double t, double inv) { return (w - t) * inv; }
__device__ __forceinline__ double2 scaled_diff(double2 w, double2 t, double inv) {
    return make_double2((w.x - t.x) * inv, (w.y - t.y) * inv);
}
__device__ __forceinline__ void zero(double& v) { v = 0.0; }
__device__ __forceinline__ void zero(double2& v) { v = make_double2(0.0, 0.0); }
__device__ __forceinline__ double block_sum_t(double v, double* sm) { return block_sum(v, sm); }
__device__ __forceinline__ double2 block_sum_t(double2 v, double* sm) {
    const double re = block_sum(v.x, sm);
    const double im = block_sum(v.y, sm);
    return make_double2(re, im);
}
__device__ __forceinline__ double add_scaled(double w, double a, double t) { return fma(a, t, w); }
__device__ __forceinline__ double2 add_scaled(double2 w, double2 a, double2 t) {
    const double2 u = cmul(a, t);
    return make_double2(w.x + u.x, w.y + u.y);
}

// All blocks of a launch call this once; it returns true in the block that
// finished last, after which that block sees every other block's writes.
__device__ __forceinline__ bool last_block(unsigned* done) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// ------------------------------------------------ Arnoldi (complex) step
// Device-indexed CGS2 of the Arnoldi step for a batch of channels
// (blockIdx.y = channel, each with its own basis, work vectors, projections
// and counters {step index by parity, done, stop}); a channel whose stop flag
// is set does nothing.  k = *cur + 1 basis rows of dimension dim.

__device__ __forceinline__ bool arn_stopped(const c3l::ArnoldiBatch& bt) { return bt.counters[blockIdx.y][3] != 0; }

// Pass 1 in FP32 from the FP32 copies of the basis rows and of w: c1[r] =
// V[r]^H w (one block per row).  The second pass, in FP64, measures and
// removes what the first left, and the column is c1 + c2, so the Arnoldi
// relation and the orthogonality keep FP64 accuracy; this pass leaves the
// FP64 pipe to the others.
__global__ void __launch_bounds__(kThreads) k_arn_dot1(c3l::ArnoldiBatch bt, int par, int64_t ld, int64_t dim) {
    __shared__ float sm[2][32];
    if (arn_stopped(bt)) return;  // dependents launch as the blocks exit
    c3l::pdl_wait();
    const int b = blockIdx.y;
    const float2* __restrict__ V = bt.V32[b];
    const float2* __restrict__ w = bt.w32[b];
    double2* __restrict__ out = bt.c1[b];
    const int k = bt.counters[b][par] + 1;
    for (int row = blockIdx.x; row < k; row += gridDim.x) {
        const float2* v = V + (int64_t)row * ld;
        const int64_t step = blockDim.x;
        float re = 0.0f, im = 0.0f;
        int64_t i = threadIdx.x;
        for (; i + 3 * step < dim; i += 4 * step) {
            float2 a[4], c[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                a[u] = v[i + u * step];
                c[u] = w[i + u * step];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                re = fmaf(a[u].x, c[u].x, fmaf(a[u].y, c[u].y, re));
                im = fmaf(a[u].x, c[u].y, fmaf(-a[u].y, c[u].x, im));
            }
        }
        for (; i < dim; i += step) {
            const float2 a = v[i], c = w[i];
            re = fmaf(a.x, c.x, fmaf(a.y, c.y, re));
            im = fmaf(a.x, c.y, fmaf(-a.y, c.x, im));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            re += __shfl_down_sync(0xffffffffu, re, o);
            im += __shfl_down_sync(0xffffffffu, im, o);
        }
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        __syncthreads();
        if (lane == 0) {
            sm[0][wid] = re;
            sm[1][wid] = im;
        }
        __syncthreads();
        if (wid == 0) {
            re = lane < (int)(blockDim.x >> 5) ? sm[0][lane] : 0.0f;
            im = lane < (int)(blockDim.x >> 5) ? sm[1][lane] : 0.0f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                re += __shfl_down_sync(0xffffffffu, re, o);
                im += __shfl_down_sync(0xffffffffu, im, o);
            }
            if (lane == 0) out[row] = make_double2((double)re, (double)im);
        }
    }
}

// First update: w' = w - V c1, in double-float on the FP32 pipe.  c1 comes from
// the FP32 first pass, so every coefficient is exactly a float; each product
// c1_r V_r splits exactly (one FMA) against the row's FP32 (hi, lo) pair, the
// products are summed by TwoSum per row group, the groups' sums are finished
// in FP64, and the subtraction from w is FP64 (error about 4e-15 of
// sum |c1_r V_r,i|, i.e. near 1e-14 |w|).  The FP32 (hi, lo) pair of w' goes
// to (w32, w32lo) for the second projections.
template <int X, int Y>
__global__ void __launch_bounds__(X * Y) k_arn_axpy(c3l::ArnoldiBatch bt, int par, int64_t ld, int64_t dim) {
    __shared__ double2 part[Y][X];
    __shared__ float2 cf[C3L_MAX_HESSENBERG];
    if (arn_stopped(bt)) return;  // dependents launch as the blocks exit
    c3l::pdl_wait();
    const int b = blockIdx.y;
    const int k = bt.counters[b][par] + 1;
    const int tid = threadIdx.y * X + threadIdx.x;
    for (int r = tid; r < k; r += X * Y) {
        const double2 c = bt.c1[b][r];
        cf[r] = make_float2((float)c.x, (float)c.y);  // exact: c1 holds FP32 sums
    }
    __syncthreads();
    const float2* __restrict__ Vh = bt.V32[b];
    const float2* __restrict__ Vl = bt.V32lo[b];
    double2* __restrict__ w = bt.w[b];
    for (int64_t base = (int64_t)blockIdx.x * X; base < dim; base += (int64_t)gridDim.x * X) {
        const int64_t i = base + threadIdx.x;
        // c v = (cx vx - cy vy) + i (cx vy + cy vx)
        float rS = 0.0f, rC = 0.0f, iS = 0.0f, iC = 0.0f;
        if (i < dim) {
            int j = threadIdx.y;
            for (; j + 3 * Y < k; j += 4 * Y) {  // eight loads in flight
                float2 vh[4], vl[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    vh[u] = Vh[(int64_t)(j + u * Y) * ld + i];
                    vl[u] = Vl[(int64_t)(j + u * Y) * ld + i];
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float2 c = cf[j + u * Y];
                    df_mac(rS, rC, c.x, 0.0f, vh[u].x, vl[u].x);
                    df_mac(rS, rC, -c.y, 0.0f, vh[u].y, vl[u].y);
                    df_mac(iS, iC, c.x, 0.0f, vh[u].y, vl[u].y);
                    df_mac(iS, iC, c.y, 0.0f, vh[u].x, vl[u].x);
                }
            }
            for (; j < k; j += Y) {
                const float2 c = cf[j];
                const float2 vh = Vh[(int64_t)j * ld + i], vl = Vl[(int64_t)j * ld + i];
                df_mac(rS, rC, c.x, 0.0f, vh.x, vl.x);
                df_mac(rS, rC, -c.y, 0.0f, vh.y, vl.y);
                df_mac(iS, iC, c.x, 0.0f, vh.y, vl.y);
                df_mac(iS, iC, c.y, 0.0f, vh.x, vl.x);
            }
        }
        part[threadIdx.y][threadIdx.x] = make_double2((double)rS + (double)rC, (double)iS + (double)iC);
        __syncthreads();
        for (int h = Y / 2; h > 0; h >>= 1) {
            if ((int)threadIdx.y < h) {
                double2 t = part[threadIdx.y][threadIdx.x];
                dot_acc_plain(t, part[threadIdx.y + h][threadIdx.x]);
                part[threadIdx.y][threadIdx.x] = t;
            }
            __syncthreads();
        }
        if (threadIdx.y == 0 && i < dim) {
            const double2 t = part[0][threadIdx.x];
            const double2 x = make_double2(w[i].x - t.x, w[i].y - t.y);
            w[i] = x;
            float2 hi, lo;
            split_d(x.x, hi.x, lo.x);
            split_d(x.y, hi.y, lo.y);
            bt.w32[b][i] = hi;
            bt.w32lo[b][i] = lo;
        }
        __syncthreads();
    }
}

// Arnoldi column from the reduced projections (run by one block): c2 holds
// the pass-2 projections (k) followed by |w'|^2, so h = sqrt(|w'|^2 - |c2|^2);
// H[:k+1, j] = c1 + c2 | h goes to column j of Hc, h to hval, and the step
// counter of the other parity to k.
//
// An exhausted Krylov space is a breakdown also when h is above the absolute
// breakdown tolerance but below kExhausted |w'|: the FP32 first pass leaves
// w' ~ 1e-7 |w| inside the span, and its FP32-product second update a floor of
// ~1e-14 |w| in h, so h / |w'| < 1e-6 means the true remainder is below
// ~1e-13 |w| -- the new vector would be rounding noise.  h is then stored as 0,
// which the shifted solves and the normalization read as a breakdown.
constexpr double kExhausted = 1.0e-6;
__device__ void arnoldi_column_tail(const double2* __restrict__ c1, const double2* __restrict__ c2, int k,
                                    double2* __restrict__ Hc, int64_t ldc, double* __restrict__ hval, int* next) {
    __shared__ double red[32];
    double sq = 0.0;
    for (int i = threadIdx.x; i < k; i += blockDim.x) sq = fma(c2[i].x, c2[i].x, fma(c2[i].y, c2[i].y, sq));
    sq = block_sum(sq, red);
    double2* col = Hc + (int64_t)(k - 1) * ldc;
    for (int i = threadIdx.x; i < k; i += blockDim.x) col[i] = make_double2(c1[i].x + c2[i].x, c1[i].y + c2[i].y);
    if (threadIdx.x == 0) {
        double h = sqrt(fmax(c2[k].x - sq, 0.0));
        if (h <= kExhausted * sqrt(fmax(c2[k].x, 0.0))) h = 0.0;
        col[k] = make_double2(h, 0.0);
        *hval = h;
        *next = k;
    }
}

// Pass 2: rows [0, k) and the vector itself (|w'|^2) in nseg segments of
// seglen, one block per (row, segment) item.  Each thread accumulates its
// entries of conj(V[row]) w' in double-float from the FP32 (hi, lo) pairs of
// the row and of w' (error about 4e-15 of sum |V_i| |w'_i| <= |w'|), and the
// block adds the threads' sums in FP64.  With one segment the block writes
// c2[row] and the block that finishes last forms the column, otherwise it
// writes partial[row][seg] for k_arn_dot2_final.  Every block reaches the
// last-block count.
__global__ void __launch_bounds__(kThreads) k_arn_dot2(c3l::ArnoldiBatch bt, int par, int64_t ld, int64_t dim,
                                                       int nseg, int64_t seglen, int64_t ldc) {
    __shared__ float sm[4][kThreads / 32];
    if (arn_stopped(bt)) return;  // dependents launch as the blocks exit
    c3l::pdl_wait();
    const int b = blockIdx.y;
    const float2* __restrict__ Vh = bt.V32[b];
    const float2* __restrict__ Vl = bt.V32lo[b];
    const float2* __restrict__ wh = bt.w32[b];
    const float2* __restrict__ wl = bt.w32lo[b];
    int32_t* ctr = bt.counters[b];
    const int k = ctr[par] + 1;
    const int items = (k + 1) * nseg;
    for (int item = blockIdx.x; item < items; item += gridDim.x) {
        const int row = item / nseg;
        const int seg = item - row * nseg;
        const float2* vh = row < k ? Vh + (int64_t)row * ld : wh;
        const float2* vl = row < k ? Vl + (int64_t)row * ld : wl;
        const int64_t lo = (int64_t)seg * seglen;
        const int64_t hi = min(dim, lo + seglen);
        // conj(v) w = (vx wx + vy wy) + i (vx wy - vy wx)
        float rS = 0.0f, rC = 0.0f, iS = 0.0f, iC = 0.0f;
        const int64_t step = blockDim.x;
        int64_t i = lo + threadIdx.x;
        for (; i + 3 * step < hi; i += 4 * step) {  // sixteen loads in flight
            float2 ah[4], al[4], bh[4], bl[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                ah[u] = vh[i + u * step];
                al[u] = vl[i + u * step];
                bh[u] = wh[i + u * step];
                bl[u] = wl[i + u * step];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                df_mac(rS, rC, ah[u].x, al[u].x, bh[u].x, bl[u].x);
                df_mac(rS, rC, ah[u].y, al[u].y, bh[u].y, bl[u].y);
                df_mac(iS, iC, ah[u].x, al[u].x, bh[u].y, bl[u].y);
                df_mac(iS, iC, -ah[u].y, -al[u].y, bh[u].x, bl[u].x);
            }
        }
        for (; i < hi; i += step) {
            const float2 ah = vh[i], al = vl[i], bh = wh[i], bl = wl[i];
            df_mac(rS, rC, ah.x, al.x, bh.x, bl.x);
            df_mac(rS, rC, ah.y, al.y, bh.y, bl.y);
            df_mac(iS, iC, ah.x, al.x, bh.y, bl.y);
            df_mac(iS, iC, -ah.y, -al.y, bh.x, bl.x);
        }
        // the block's sum in double-float, FP64 only for the result
        df_warp_sum(rS, rC);
        df_warp_sum(iS, iC);
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        __syncthreads();  // sm is free (previous item)
        if (lane == 0) {
            sm[0][wid] = rS;
            sm[1][wid] = rC;
            sm[2][wid] = iS;
            sm[3][wid] = iC;
        }
        __syncthreads();
        if (wid == 0) {
            const bool in = lane < (int)(blockDim.x >> 5);
            rS = in ? sm[0][lane] : 0.0f;
            rC = in ? sm[1][lane] : 0.0f;
            iS = in ? sm[2][lane] : 0.0f;
            iC = in ? sm[3][lane] : 0.0f;
            df_warp_sum(rS, rC);
            df_warp_sum(iS, iC);
            if (lane == 0) {
                const double2 acc = make_double2((double)rS + (double)rC, (double)iS + (double)iC);
                if (nseg == 1) bt.c2[b][row] = acc;
                else bt.partial[b][(int64_t)row * nseg + seg] = acc;
            }
        }
    }
    if (nseg == 1 && last_block(reinterpret_cast<unsigned*>(ctr + 2))) {
        arnoldi_column_tail(bt.c1[b], bt.c2[b], k, bt.Hc[b], ldc, bt.hval[b], ctr + (1 - par));
        if (threadIdx.x == 0) ctr[2] = 0;
    }
}

__global__ void __launch_bounds__(kThreads) k_arn_dot2_final(c3l::ArnoldiBatch bt, int par, int nseg, int64_t ldc) {
    __shared__ double sm[32];
    if (arn_stopped(bt)) return;  // dependents launch as the blocks exit
    c3l::pdl_wait();
    const int b = blockIdx.y;
    int32_t* ctr = bt.counters[b];
    const int k = ctr[par] + 1;
    const double2* __restrict__ partial = bt.partial[b];
    for (int row = blockIdx.x; row <= k; row += gridDim.x) {
        double2 acc = make_double2(0.0, 0.0);
        for (int q = threadIdx.x; q < nseg; q += blockDim.x) dot_acc_plain(acc, partial[(int64_t)row * nseg + q]);
        acc = block_sum_t(acc, sm);
        if (threadIdx.x == 0) bt.c2[b][row] = acc;
    }
    if (last_block(reinterpret_cast<unsigned*>(ctr + 2))) {
        arnoldi_column_tail(bt.c1[b], bt.c2[b], k, bt.Hc[b], ldc, bt.hval[b], ctr + (1 - par));
        if (threadIdx.x == 0) ctr[2] = 0;
    }
}

// Second update and normalization: V[k] = xnext = (w' - V c2) / h, unscaled
// when h <= tol (breakdown, detected by the shifted solves); V32[k] gets its
// FP32 copy.  c2 is the small correction left by the FP32 first pass (about
// 1e-7 |w'|), so V c2 is formed with FP32 products from the FP32 rows: its
// error, about 6e-8 |V c2|, is near 1e-14 |w|; the subtraction and the
// scaling are FP64.  The projections c2 stay FP64 in the Hessenberg column.
// Reads the step index from `cur` of the parity (the column tail already
// wrote `next`).
template <int X, int Y>
__global__ void __launch_bounds__(X * Y) k_arn_scale(c3l::ArnoldiBatch bt, int par, int64_t ld, int64_t n,
                                                     double tol) {
    __shared__ float2 part[Y][X];
    __shared__ float2 cf[C3L_MAX_HESSENBERG];
    if (arn_stopped(bt)) return;  // dependents launch as the blocks exit
    c3l::pdl_wait();
    const int b = blockIdx.y;
    const int k = bt.counters[b][par] + 1;
    const double h = *bt.hval[b];
    const double inv = h > tol ? 1.0 / h : 1.0;
    const int tid = threadIdx.y * X + threadIdx.x;
    for (int r = tid; r < k; r += X * Y) {
        const double2 c = bt.c2[b][r];
        cf[r] = make_float2((float)c.x, (float)c.y);
    }
    __syncthreads();
    const float2* __restrict__ V32 = bt.V32[b];
    double2* Vk = bt.V[b] + (int64_t)k * ld;
    float2* V32k = bt.V32[b] + (int64_t)k * ld;
    const double2* __restrict__ w = bt.w[b];
    double2* __restrict__ xnext = bt.xnext[b];
    double2* __restrict__ xws = bt.xws[b];
    for (int64_t base = (int64_t)blockIdx.x * X; base < n; base += (int64_t)gridDim.x * X) {
        const int64_t i = base + threadIdx.x;
        float2 s = make_float2(0.0f, 0.0f);
        int64_t q0 = 0, q1 = 0;  // the element's scatter entries (program table)
        if (xws && threadIdx.y == 0 && i < n) {
            q0 = bt.xoff[i];
            q1 = bt.xoff[i + 1];
        }
        if (i < n) {
            int j = threadIdx.y;
            for (; j + 3 * Y < k; j += 4 * Y) {
                float2 v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) v[u] = V32[(int64_t)(j + u * Y) * ld + i];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float2 c = cf[j + u * Y];
                    s.x = fmaf(c.x, v[u].x, fmaf(-c.y, v[u].y, s.x));
                    s.y = fmaf(c.x, v[u].y, fmaf(c.y, v[u].x, s.y));
                }
            }
            for (; j < k; j += Y) {
                const float2 c = cf[j], v = V32[(int64_t)j * ld + i];
                s.x = fmaf(c.x, v.x, fmaf(-c.y, v.y, s.x));
                s.y = fmaf(c.x, v.y, fmaf(c.y, v.x, s.y));
            }
        }
        part[threadIdx.y][threadIdx.x] = s;
        __syncthreads();
        for (int hh = Y / 2; hh > 0; hh >>= 1) {
            if ((int)threadIdx.y < hh) {
                const float2 o = part[threadIdx.y + hh][threadIdx.x];
                part[threadIdx.y][threadIdx.x].x += o.x;
                part[threadIdx.y][threadIdx.x].y += o.y;
            }
            __syncthreads();
        }
        if (threadIdx.y == 0 && i < n) {
            const float2 t = part[0][threadIdx.x];
            const double2 x = make_double2((w[i].x - (double)t.x) * inv, (w[i].y - (double)t.y) * inv);
            Vk[i] = x;
            float2 xh, xl;
            split_d(x.x, xh.x, xl.x);
            split_d(x.y, xh.y, xl.y);
            V32k[i] = xh;
            bt.V32lo[b][(int64_t)k * ld + i] = xl;
            xnext[i] = x;
            if (xws) {  // the next sigma's padded input entries of element i
                for (int64_t q = q0; q < q1; ++q) {
                    const double sg = bt.xsign[q];
                    xws[bt.xdst[q]] = make_double2(sg * x.x, sg * x.y);
                }
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------ GMRES (real) CGS2 step
// Short basis (k <= restart + 1 rows) over a long vector: each block owns a
// column segment for all rows, writes partial[block][row], and the block that
// finishes last reduces the partials in a fixed order.  Warp r8 of a block
// handles rows r8, r8 + 8, ...; its lanes stride the block's segment.
constexpr int kGmWarps = kThreads / 32;

// The rows of one warp (r = warp + kGmWarps q) are
// streamed together: each column step loads w once and one entry per row, so
// the loads of all rows are in flight at once.  Supports k + 1 <= C3L_GMRES_MAX_ROWS rows.

__device__ __forceinline__ void gm_partials(const double* __restrict__ V, int64_t ld, int k,
                                            const double* __restrict__ w, int64_t lo, int64_t hi,
                                            double* __restrict__ partial, int R) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rows = (k + 1 - warp + kGmWarps - 1) / kGmWarps;  // rows of this warp (row k is w itself)
    for (int q0 = 0; q0 < rows; q0 += 4) {
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        const double* v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int r = warp + kGmWarps * (q0 + u);
            v[u] = (q0 + u < rows) ? (r < k ? V + (int64_t)r * ld : w) : w;
        }
        for (int64_t c = lo + lane; c < hi; c += 32) {
            const double wc = w[c];
            double e[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) e[u] = v[u][c];
#pragma unroll
            for (int u = 0; u < 4; ++u) acc[u] = fma(e[u], wc, acc[u]);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const double t = warp_sum(acc[u]);
            const int r = warp + kGmWarps * (q0 + u);
            if (lane == 0 && q0 + u < rows) partial[(int64_t)blockIdx.x * R + r] = t;
        }
    }
}

// out[r] = sum over blocks of partial[block][r], r <= k, reduced by every
// block that needs it (fixed order: identical in every block, so all blocks
// hold bitwise the same coefficients).
__device__ __forceinline__ void gm_reduce(const double* __restrict__ partial, int R, int nb, int k,
                                          double* __restrict__ out) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int r = warp; r <= k; r += kGmWarps) {
        double s = 0.0;
        for (int b = lane; b < nb; b += 32) s += partial[(int64_t)b * R + r];
        s = warp_sum(s);
        if (lane == 0) out[r] = s;
    }
}

// Pass-1 partial projections of the work vector: partial1[block][r].
__global__ void __launch_bounds__(kThreads) k_gm_dot(const double* __restrict__ V, int64_t ld, const int* cur,
                                                     const double* __restrict__ w, int64_t n, int64_t seg,
                                                     double* __restrict__ partial1, int R) {
    const int k = *cur + 1;
    const int64_t lo = (int64_t)blockIdx.x * seg;
    gm_partials(V, ld, k, w, lo, min(n, lo + seg), partial1, R);
}

// c1 = reduced pass-1 projections (block 0 stores them), w' = w - V c1 on
// the block's segment, then the pass-2 partials partial2[block][r].
__global__ void __launch_bounds__(kThreads) k_gm_axpy_dot(const double* __restrict__ V, int64_t ld, const int* cur,
                                                          const double* __restrict__ partial1,
                                                          double* __restrict__ c1, double* __restrict__ w, int64_t n,
                                                          int64_t seg, double* __restrict__ partial2, int R) {
    __shared__ double cs[C3L_GMRES_MAX_ROWS];
    const int k = *cur + 1;
    gm_reduce(partial1, R, gridDim.x, k, cs);
    __syncthreads();
    if (blockIdx.x == 0)
        for (int r = threadIdx.x; r <= k; r += blockDim.x) c1[r] = cs[r];
    const int64_t lo = (int64_t)blockIdx.x * seg;
    const int64_t hi = min(n, lo + seg);
    for (int64_t c = lo + threadIdx.x; c < hi; c += blockDim.x) {
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        int r = 0;
        for (; r + 3 < k; r += 4) {
            s0 = fma(cs[r], V[(int64_t)r * ld + c], s0);
            s1 = fma(cs[r + 1], V[(int64_t)(r + 1) * ld + c], s1);
            s2 = fma(cs[r + 2], V[(int64_t)(r + 2) * ld + c], s2);
            s3 = fma(cs[r + 3], V[(int64_t)(r + 3) * ld + c], s3);
        }
        for (; r < k; ++r) s0 = fma(cs[r], V[(int64_t)r * ld + c], s0);
        w[c] -= (s0 + s1) + (s2 + s3);
    }
    __syncthreads();
    gm_partials(V, ld, k, w, lo, hi, partial2, R);
}

// c2 = reduced pass-2 projections, h0 = |w| (from c1), h = sqrt(|w'|^2 -
// |c2|^2); V[k] = xnext = (w' - V c2) / h unless h <= eps h0 (breakdown:
// unscaled).  Block 0 writes the column [c1 + c2 | h | h0] to host-mapped
// slot j and the step index of the other parity.
__global__ void __launch_bounds__(kThreads) k_gm_scale(double* V, int64_t ld, const int* cur, int* next,
                                                       const double* __restrict__ partial2, int R, int nb,
                                                       const double* __restrict__ c1, double eps,
                                                       const double* __restrict__ w, int64_t n,
                                                       double* __restrict__ xnext, double* __restrict__ slots,
                                                       int stride) {
    __shared__ double cs[C3L_GMRES_MAX_ROWS];
    __shared__ double hh[2];
    const int k = *cur + 1;
    gm_reduce(partial2, R, nb, k, cs);
    __syncthreads();
    if (threadIdx.x < 32) {
        double sq = 0.0;
        for (int r = threadIdx.x; r < k; r += 32) sq = fma(cs[r], cs[r], sq);
        sq = warp_sum(sq);
        if (threadIdx.x == 0) {
            hh[0] = sqrt(fmax(c1[k], 0.0));
            hh[1] = sqrt(fmax(cs[k] - sq, 0.0));
        }
    }
    __syncthreads();
    const double h0 = hh[0], h = hh[1];
    const double inv = h > eps * h0 ? 1.0 / h : 1.0;
    if (blockIdx.x == 0) {
        double* slot = slots + (int64_t)(k - 1) * stride;
        for (int r = threadIdx.x; r < k; r += blockDim.x) slot[r] = c1[r] + cs[r];
        if (threadIdx.x == 0) {
            slot[k] = h;
            slot[k + 1] = h0;
            *next = k;
        }
    }
    double* Vk = V + (int64_t)k * ld;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        int r = 0;
        for (; r + 3 < k; r += 4) {
            s0 = fma(cs[r], V[(int64_t)r * ld + c], s0);
            s1 = fma(cs[r + 1], V[(int64_t)(r + 1) * ld + c], s1);
            s2 = fma(cs[r + 2], V[(int64_t)(r + 2) * ld + c], s2);
            s3 = fma(cs[r + 3], V[(int64_t)(r + 3) * ld + c], s3);
        }
        for (; r < k; ++r) s0 = fma(cs[r], V[(int64_t)r * ld + c], s0);
        const double x = (w[c] - ((s0 + s1) + (s2 + s3))) * inv;
        Vk[c] = x;
        xnext[c] = x;
    }
}

// ------------------------------------------ GMRES CGS2 step, FP32 basis
// The same three kernels for an inner solve whose operator is FP32 (the
// FP32 JVP): the basis rows, the work vector after the operator and all
// products and sums are FP32; the Hessenberg column goes to the host in FP64.
// Partial sums are floats in the same [block][R] layout.  Blocks of 1024
// threads: 32 warps share the projection rows, and the updates w -= V c run
// 256 columns x 4 row groups (each thread a quarter of the rows, the groups
// added in shared memory in a fixed order), so no thread walks all k rows.
constexpr int kGmfThreads = 1024;
constexpr int kGmfWarps = kGmfThreads / 32;
constexpr int kGmfCols = 256;
constexpr int kGmfGroups = kGmfThreads / kGmfCols;

__device__ __forceinline__ void gm_partials_f(const float* __restrict__ V, int64_t ld, int k,
                                              const float* __restrict__ w, int64_t lo, int64_t hi,
                                              float* __restrict__ partial, int R) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rows = (k + 1 - warp + kGmfWarps - 1) / kGmfWarps;  // rows of this warp (row k is w itself)
    for (int q0 = 0; q0 < rows; q0 += 4) {
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        const float* v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int r = warp + kGmfWarps * (q0 + u);
            v[u] = (q0 + u < rows) ? (r < k ? V + (int64_t)r * ld : w) : w;
        }
        for (int64_t c = lo + lane; c < hi; c += 32) {
            const float wc = w[c];
            float e[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) e[u] = v[u][c];
#pragma unroll
            for (int u = 0; u < 4; ++u) acc[u] = fmaf(e[u], wc, acc[u]);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const float t = warp_sum(acc[u]);
            const int r = warp + kGmfWarps * (q0 + u);
            if (lane == 0 && q0 + u < rows) partial[(int64_t)blockIdx.x * R + r] = t;
        }
    }
}

__device__ __forceinline__ void gm_reduce_f(const float* __restrict__ partial, int R, int nb, int k,
                                            float* __restrict__ out) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int r = warp; r <= k; r += kGmfWarps) {
        float s = 0.0f;
        for (int b = lane; b < nb; b += 32) s += partial[(int64_t)b * R + r];
        s = warp_sum(s);
        if (lane == 0) out[r] = s;
    }
}

// t = sum_{r < k} c[r] V[r][col] for the thread's column (col valid when
// `ok`), each row group a quarter of the rows; the result is valid in row
// group 0.  Every thread of the block calls it (it synchronizes).
__device__ __forceinline__ float gm_combine_f(const float* __restrict__ V, int64_t ld, int k,
                                              const float* __restrict__ c, int64_t col, bool ok,
                                              float (*red)[kGmfCols]) {
    const int g = threadIdx.x / kGmfCols, cl = threadIdx.x % kGmfCols;
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
    if (ok) {
        constexpr int G = kGmfGroups;
        int r = g;
        for (; r + 3 * G < k; r += 4 * G) {
            s0 = fmaf(c[r], V[(int64_t)r * ld + col], s0);
            s1 = fmaf(c[r + G], V[(int64_t)(r + G) * ld + col], s1);
            s2 = fmaf(c[r + 2 * G], V[(int64_t)(r + 2 * G) * ld + col], s2);
            s3 = fmaf(c[r + 3 * G], V[(int64_t)(r + 3 * G) * ld + col], s3);
        }
        for (; r < k; r += G) s0 = fmaf(c[r], V[(int64_t)r * ld + col], s0);
    }
    red[g][cl] = (s0 + s1) + (s2 + s3);
    __syncthreads();
    float t = 0.0f;
    if (g == 0) {
#pragma unroll
        for (int q = 0; q < kGmfGroups; ++q) t += red[q][cl];
    }
    return t;
}

// wf = (float) w on the block's segment, then the pass-1 partials.
__global__ void __launch_bounds__(kGmfThreads) k_gm_dot_f(const float* __restrict__ V, int64_t ld, const int* cur,
                                                          const double* __restrict__ w, float* __restrict__ wf,
                                                          int64_t n, int64_t seg, float* __restrict__ partial1,
                                                          int R) {
    c3l::pdl_launch_dependents();
    c3l::pdl_wait();
    const int k = *cur + 1;
    const int64_t lo = (int64_t)blockIdx.x * seg;
    const int64_t hi = min(n, lo + seg);
    for (int64_t c = lo + threadIdx.x; c < hi; c += blockDim.x) wf[c] = (float)w[c];
    __syncthreads();
    gm_partials_f(V, ld, k, wf, lo, hi, partial1, R);
}

__global__ void __launch_bounds__(kGmfThreads) k_gm_axpy_dot_f(const float* __restrict__ V, int64_t ld,
                                                               const int* cur, const float* __restrict__ partial1,
                                                               float* __restrict__ c1, float* __restrict__ wf,
                                                               int64_t n, int64_t seg, float* __restrict__ partial2,
                                                               int R) {
    c3l::pdl_launch_dependents();
    c3l::pdl_wait();
    __shared__ float cs[C3L_GMRES_MAX_ROWS];
    __shared__ float red[kGmfGroups][kGmfCols];
    const int k = *cur + 1;
    gm_reduce_f(partial1, R, gridDim.x, k, cs);
    __syncthreads();
    if (blockIdx.x == 0)
        for (int r = threadIdx.x; r <= k; r += blockDim.x) c1[r] = cs[r];
    const int64_t lo = (int64_t)blockIdx.x * seg;
    const int64_t hi = min(n, lo + seg);
    const int g = threadIdx.x / kGmfCols, cl = threadIdx.x % kGmfCols;
    for (int64_t base = lo; base < hi; base += kGmfCols) {
        const int64_t col = base + cl;
        const float t = gm_combine_f(V, ld, k, cs, col, col < hi, red);
        if (g == 0 && col < hi) wf[col] -= t;
        __syncthreads();  // red is reused; the new wf is visible to the partials below
    }
    gm_partials_f(V, ld, k, wf, lo, hi, partial2, R);
}

__global__ void __launch_bounds__(kGmfThreads) k_gm_scale_f(float* V, int64_t ld, const int* cur, int* next,
                                                            const float* __restrict__ partial2, int R, int nb,
                                                            const float* __restrict__ c1, double eps,
                                                            const float* __restrict__ wf, int64_t n,
                                                            double* __restrict__ xnext, double* __restrict__ slots,
                                                            int stride) {
    c3l::pdl_launch_dependents();
    c3l::pdl_wait();
    __shared__ float cs[C3L_GMRES_MAX_ROWS];
    __shared__ float red[kGmfGroups][kGmfCols];
    __shared__ float hh[2];
    const int k = *cur + 1;
    gm_reduce_f(partial2, R, nb, k, cs);
    __syncthreads();
    if (threadIdx.x < 32) {
        float sq = 0.0f;
        for (int r = threadIdx.x; r < k; r += 32) sq = fmaf(cs[r], cs[r], sq);
        sq = warp_sum(sq);
        if (threadIdx.x == 0) {
            hh[0] = sqrtf(fmaxf(c1[k], 0.0f));
            hh[1] = sqrtf(fmaxf(cs[k] - sq, 0.0f));
        }
    }
    __syncthreads();
    const float h0 = hh[0], h = hh[1];
    const float inv = (double)h > eps * (double)h0 ? 1.0f / h : 1.0f;
    if (blockIdx.x == 0) {
        double* slot = slots + (int64_t)(k - 1) * stride;
        for (int r = threadIdx.x; r < k; r += blockDim.x) slot[r] = (double)c1[r] + (double)cs[r];
        if (threadIdx.x == 0) {
            slot[k] = h;
            slot[k + 1] = h0;
            *next = k;
        }
    }
    float* Vk = V + (int64_t)k * ld;
    const int g = threadIdx.x / kGmfCols, cl = threadIdx.x % kGmfCols;
    for (int64_t base = (int64_t)blockIdx.x * kGmfCols; base < n; base += (int64_t)gridDim.x * kGmfCols) {
        const int64_t col = base + cl;
        const float t = gm_combine_f(V, ld, k, cs, col, col < n, red);
        if (g == 0 && col < n) {
            const float x = (wf[col] - t) * inv;
            Vk[col] = x;
            xnext[col] = (double)x;
        }
        __syncthreads();  // red is reused
    }
}

// FP32 (hi, lo) pair of a complex FP64 vector.
__global__ void k_split_c(int64_t n, const double2* __restrict__ x, float2* __restrict__ hi, float2* __restrict__ lo) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 v = x[i];
        float2 h, l;
        split_d(v.x, h.x, l.x);
        split_d(v.y, h.y, l.y);
        hi[i] = h;
        lo[i] = l;
    }
}

// V0 = (float)(a r) and x = V0 in FP64: the first row of an FP32 basis.
__global__ void k_gm_start_f(int64_t n, double a, const double* __restrict__ r, float* __restrict__ V0,
                             double* __restrict__ x) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = (float)(a * r[i]);
        V0[i] = v;
        x[i] = (double)v;
    }
}

// x += V[0 : k]^T y over an FP32 basis (FP64 products and sums).
__global__ void k_gm_update_f(const float* __restrict__ V, int64_t ld, int k, const double* __restrict__ y,
                              double* __restrict__ x, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int r = 0; r < k; ++r) s = fma(y[r], (double)V[(int64_t)r * ld + i], s);
        x[i] += s;
    }
}

// Fixed scratch for c3l_hessenberg_coordinates_noalloc: the packed R factors
// of the shifted solves live here instead of in caller-provided memory.  The
// array is part of the library's device image, so every GPU that loads the
// library holds these C3L_NOALLOC_SCRATCH_ENTRIES complex entries until the
// process exits.
static __device__ __align__(256) double2 g_noalloc_scratch[C3L_NOALLOC_SCRATCH_ENTRIES];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device.  In host code the
// array's name is only a host-side stand-in, so the address is looked up once
// per device (with that device current) and cached.
c3l_status noalloc_scratch(double2** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return C3L_ERR_LAUNCH;
    if (dev < 0 || dev >= kMaxDevices) return C3L_ERR_CAPACITY;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return C3L_ERR_LAUNCH;
        g_noalloc_ptr[dev] = p;
    }
    *out = static_cast<double2*>(g_noalloc_ptr[dev]);
    return C3L_OK;
}

}  // namespace

namespace c3l {

RowDot row_dot_plan(int max_rows, int64_t dim, int sms) {
    RowDot p;
    p.max_rows = max_rows < 1 ? 1 : max_rows;
    p.nseg = dim > kRowDotMax ? (int)((dim + kSegLen - 1) / kSegLen) : 1;
    p.seglen = p.nseg == 1 ? (dim > 0 ? dim : 1) : kSegLen;
    int64_t g = (int64_t)p.max_rows * p.nseg;
    const int64_t cap = 4 * (int64_t)(sms > 0 ? sms : 152);  // rows beyond the grid are strided
    if (g > cap) g = cap;
    p.grid = (unsigned)(g < 1 ? 1 : g);
    return p;
}

int64_t row_dot_partial_size(const RowDot& p) { return p.nseg == 1 ? 0 : (int64_t)p.max_rows * p.nseg; }

static bool valid_batch(const ArnoldiBatch& bt, bool with_partial) {
    if (bt.nb < 1 || bt.nb > C3L_MAX_BATCH) return false;
    for (int b = 0; b < bt.nb; ++b)
        if (!bt.V[b] || !bt.w[b] || !bt.xnext[b] || !bt.c1[b] || !bt.c2[b] || !bt.hval[b] || !bt.counters[b] ||
            !bt.Hc[b] || !bt.V32[b] || !bt.w32[b] || !bt.V32lo[b] || !bt.w32lo[b] ||
            (with_partial && !bt.partial[b]))
            return false;
    return true;
}

c3l_status arnoldi_dot1(const ArnoldiBatch& bt, int par, int64_t ld, int64_t dim, const RowDot& p, cudaStream_t s) {
    if (!valid_batch(bt, false) || dim <= 0 || ld < dim || (par & ~1)) return C3L_ERR_ARGUMENT;
    return launch_pdl(k_arn_dot1, dim3(p.grid, (unsigned)bt.nb), dim3(kThreads), 0, s, 0, true, bt, par, ld, dim);
}

c3l_status arnoldi_axpy1(const ArnoldiBatch& bt, int par, int64_t ld, int max_k, int64_t dim, cudaStream_t s) {
    if (!valid_batch(bt, false) || dim <= 0 || ld < dim || (par & ~1)) return C3L_ERR_ARGUMENT;
    if (max_k > C3L_MAX_HESSENBERG) return C3L_ERR_CAPACITY;  // c1 is staged in shared memory
    return launch_pdl(k_arn_axpy<kAxX, kAxY>, dim3(axpy_grid(dim), (unsigned)bt.nb), dim3(kAxX, kAxY), 0, s, 0, true, bt, par,
                      ld, dim);
}

c3l_status arnoldi_dot2(const ArnoldiBatch& bt, int par, int64_t ld, int64_t dim, const RowDot& p, int64_t ldc,
                        cudaStream_t s) {
    if (!valid_batch(bt, p.nseg > 1) || dim <= 0 || ld < dim || (par & ~1)) return C3L_ERR_ARGUMENT;
    c3l_status r = launch_pdl(k_arn_dot2, dim3(p.grid, (unsigned)bt.nb), dim3(kThreads), 0, s, 0, true, bt, par, ld, dim,
                              p.nseg, p.seglen, ldc);
    if (r || p.nseg == 1) return r;
    const unsigned g = (unsigned)(p.max_rows > 1024 ? 1024 : p.max_rows);
    return launch_pdl(k_arn_dot2_final, dim3(g, (unsigned)bt.nb), dim3(kThreads), 0, s, 0, true, bt, par, p.nseg, ldc);
}

c3l_status arnoldi_scale(const ArnoldiBatch& bt, int par, int64_t ld, int max_k, double tol, int64_t n,
                         cudaStream_t s) {
    if (!valid_batch(bt, false) || n <= 0 || ld < n || (par & ~1)) return C3L_ERR_ARGUMENT;
    if (max_k > C3L_MAX_HESSENBERG) return C3L_ERR_CAPACITY;  // c2 is staged in shared memory
    return launch_pdl(k_arn_scale<kAxX, kAxY>, dim3(axpy_grid(n), (unsigned)bt.nb), dim3(kAxX, kAxY), 0, s, 0, true, bt, par,
                      ld, n, tol);
}

GmPlan gm_plan(int64_t n, int max_rows, int sms) {
    GmPlan p;
    p.R = max_rows;
    int64_t blocks = (n + kThreads - 1) / kThreads;
    const int64_t cap = 2 * (int64_t)(sms > 0 ? sms : 152);
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    p.seg = ((n + blocks - 1) / blocks + 31) / 32 * 32;
    p.blocks = (unsigned)((n + p.seg - 1) / p.seg);
    int64_t sg = (n + kThreads - 1) / kThreads;
    if (sg > cap) sg = cap;
    p.scale_grid = (unsigned)(sg < 1 ? 1 : sg);
    return p;
}

c3l_status gm_dot(const double* V, int64_t ld, const int* cur, const double* w, int64_t n, const GmPlan& p,
                  double* partial, cudaStream_t s) {
    if (!V || !cur || !w || !partial || n <= 0 || p.R > C3L_GMRES_MAX_ROWS) return C3L_ERR_ARGUMENT;
    k_gm_dot<<<p.blocks, kThreads, 0, s>>>(V, ld, cur, w, n, p.seg, partial, p.R);
    return launch_status();
}

c3l_status gm_axpy_dot(const double* V, int64_t ld, const int* cur, double* c1, double* w, int64_t n, const GmPlan& p,
                       double* partial, cudaStream_t s) {
    if (!V || !cur || !c1 || !w || !partial || n <= 0 || p.R > C3L_GMRES_MAX_ROWS) return C3L_ERR_ARGUMENT;
    const int64_t half = (int64_t)p.blocks * p.R;
    k_gm_axpy_dot<<<p.blocks, kThreads, 0, s>>>(V, ld, cur, partial, c1, w, n, p.seg, partial + half, p.R);
    return launch_status();
}

c3l_status gm_scale(double* V, int64_t ld, const int* cur, int* next, const double* partial, const double* c1,
                    double eps, const double* w, int64_t n, const GmPlan& p, double* xnext, double* slots, int stride,
                    cudaStream_t s) {
    if (!V || !cur || !next || !partial || !c1 || !w || !xnext || !slots || n <= 0) return C3L_ERR_ARGUMENT;
    const int64_t half = (int64_t)p.blocks * p.R;
    k_gm_scale<<<p.scale_grid, kThreads, 0, s>>>(V, ld, cur, next, partial + half, p.R, (int)p.blocks, c1, eps, w, n,
                                                 xnext, slots, stride);
    return launch_status();
}

c3l_status gm_dot_f32(const float* V, int64_t ld, const int* cur, const double* w, float* wf, int64_t n,
                      const GmPlan& p, float* partial, cudaStream_t s) {
    if (!V || !cur || !w || !wf || !partial || n <= 0 || p.R > C3L_GMRES_MAX_ROWS) return C3L_ERR_ARGUMENT;
    return launch_pdl(k_gm_dot_f, dim3(p.blocks), dim3(kGmfThreads), 0, s, 0, true, V, ld, cur, w, wf, n, p.seg, partial, p.R);
}

c3l_status gm_axpy_dot_f32(const float* V, int64_t ld, const int* cur, float* c1, float* wf, int64_t n,
                           const GmPlan& p, float* partial, cudaStream_t s) {
    if (!V || !cur || !c1 || !wf || !partial || n <= 0 || p.R > C3L_GMRES_MAX_ROWS) return C3L_ERR_ARGUMENT;
    const int64_t half = (int64_t)p.blocks * p.R;
    return launch_pdl(k_gm_axpy_dot_f, dim3(p.blocks), dim3(kGmfThreads), 0, s, 0, true, V, ld, cur, (const float*)partial, c1,
                      wf, n, p.seg, partial + half, p.R);
}

c3l_status gm_scale_f32(float* V, int64_t ld, const int* cur, int* next, const float* partial, const float* c1,
                        double eps, const float* wf, int64_t n, const GmPlan& p, double* xnext, double* slots,
                        int stride, cudaStream_t s) {
    if (!V || !cur || !next || !partial || !c1 || !wf || !xnext || !slots || n <= 0) return C3L_ERR_ARGUMENT;
    const int64_t half = (int64_t)p.blocks * p.R;
    return launch_pdl(k_gm_scale_f, dim3(p.scale_grid), dim3(kGmfThreads), 0, s, 0, true, V, ld, cur, next,
                      (const float*)(partial + half), p.R, (int)p.blocks, c1, eps, wf, n, xnext, slots, stride);
}

c3l_status split_c(int64_t n, const c3l_complex* x, c3l_complex32* hi, c3l_complex32* lo, cudaStream_t s) {
    if (!x || !hi || !lo || n <= 0) return C3L_ERR_ARGUMENT;
    k_split_c<<<grid_for(n), kThreads, 0, s>>>(n, reinterpret_cast<const double2*>(x), reinterpret_cast<float2*>(hi),
                                               reinterpret_cast<float2*>(lo));
    return launch_status();
}

c3l_status gm_start_f32(int64_t n, double a, const double* r, float* V0, double* x, cudaStream_t s) {
    if (!r || !V0 || !x || n <= 0) return C3L_ERR_ARGUMENT;
    k_gm_start_f<<<grid_for(n), kThreads, 0, s>>>(n, a, r, V0, x);
    return launch_status();
}

c3l_status gm_update_f32(const float* V, int64_t ld, int k, const double* y, double* x, int64_t n, cudaStream_t s) {
    if (!V || !y || !x || n <= 0 || k <= 0 || ld < n) return C3L_ERR_ARGUMENT;
    k_gm_update_f<<<grid_for(n), kThreads, 0, s>>>(V, ld, k, y, x, n);
    return launch_status();
}

c3l_status hessenberg_advance_many(c3l_hessenberg_state* const* states, const c3l_complex* const* Hc,
                                   const int64_t* ldc, const int32_t* m, int count, cudaStream_t s) {
    if (count <= 0 || count > kMaxAdvJobs) return C3L_ERR_ARGUMENT;
    AdvJobs jobs{};
    int max_shifts = 0;
    for (int i = 0; i < count; ++i) {
        c3l_hessenberg_state* st = states[i];
        if (!st || !Hc[i] || !st->shifts || !st->rot_c || !st->rot_s || !st->vsink || !st->carry || !st->accum ||
            !st->residual || !st->status || st->nshift <= 0 || st->m_max <= 0 || !(st->beta > 0.0))
            return C3L_ERR_ARGUMENT;
        if (m[i] < st->done || m[i] > st->m_max || ldc[i] < (int64_t)st->m_max + 1 || st->done < 0)
            return C3L_ERR_ARGUMENT;
        if (cudaMemsetAsync(st->status, 0, sizeof(c3l_hessenberg_status), s) != cudaSuccess) return C3L_ERR_LAUNCH;
        AdvJob& j = jobs.job[jobs.count];
        if (m[i] == st->done) continue;  // nothing new: outputs stay those of the last call
        j.Hc = reinterpret_cast<const double2*>(Hc[i]);
        j.ldc = ldc[i];
        j.j0 = st->done;
        j.j1 = m[i];
        j.shifts = reinterpret_cast<const double2*>(st->shifts);
        j.nshift = st->nshift;
        j.beta = st->beta;
        j.btol = st->breakdown_tol;
        j.sinkc = reinterpret_cast<const double2*>(st->sinkproj_conj);
        j.rot_c = st->rot_c;
        j.rot_s = reinterpret_cast<double2*>(st->rot_s);
        j.vs = reinterpret_cast<double2*>(st->vsink);
        j.carry = reinterpret_cast<double2*>(st->carry);
        j.accum = reinterpret_cast<double2*>(st->accum);
        j.green = reinterpret_cast<double2*>(st->green);
        j.residual = st->residual;
        j.status = st->status;
        jobs.count += 1;
        max_shifts = std::max(max_shifts, st->nshift);
    }
    if (jobs.count > 0) {
        const dim3 grid((unsigned)((max_shifts + kMjShifts - 1) / kMjShifts), (unsigned)jobs.count, 1);
        k_hessenberg_advance_jobs<<<grid, 32, 0, s>>>(jobs);
        if (cudaGetLastError() != cudaSuccess) return C3L_ERR_LAUNCH;
    }
    for (int i = 0; i < count; ++i) states[i]->done = m[i];
    return C3L_OK;
}

}  // namespace c3l

extern "C" {

int64_t c3l_multi_dot_scratch(int32_t k, int64_t dim) {
    const int64_t nseg = dim > kRowDotMax ? (dim + kSegLen - 1) / kSegLen : 1;
    const int64_t nb = partial_blocks(k, dim);
    return (int64_t)k * (nb > nseg ? nb : nseg);
}

c3l_status c3l_multi_dot_c(const c3l_complex* V, int64_t ld, int32_t k, const c3l_complex* w, int64_t dim,
                           c3l_complex* partial, c3l_complex* out, void* stream) {
    if (k < 0 || dim < 0 || k > 65535) return C3L_ERR_ARGUMENT;
    if (k == 0) return C3L_OK;
    if (!V || !w || !partial || !out || ld < dim) return C3L_ERR_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    if (dim <= kRowDotMax) {
        k_dot_rows_c<<<(unsigned)k, kThreads, 0, s>>>(reinterpret_cast<const double2*>(V), ld,
                                                      reinterpret_cast<const double2*>(w), dim,
                                                      reinterpret_cast<double2*>(out));
        return launch_status();
    }
    const int64_t nb = partial_blocks(k, dim);
    k_dot_partial_c<<<dim3((unsigned)nb, (unsigned)k), kThreads, 0, s>>>(reinterpret_cast<const double2*>(V), ld,
                                                                        reinterpret_cast<const double2*>(w), dim,
                                                                        reinterpret_cast<double2*>(partial));
    k_dot_final_c<<<(unsigned)k, kThreads, 0, s>>>(reinterpret_cast<const double2*>(partial), (int)nb,
                                                  reinterpret_cast<double2*>(out));
    return launch_status();
}

c3l_status c3l_multi_dot_r(const double* V, int64_t ld, int32_t k, const double* w, int64_t dim, double* partial,
                           double* out, void* stream) {
    if (k < 0 || dim < 0 || k > 65535) return C3L_ERR_ARGUMENT;
    if (k == 0) return C3L_OK;
    if (!V || !w || !partial || !out || ld < dim) return C3L_ERR_ARGUMENT;
    const int64_t nb = partial_blocks(k, dim);
    cudaStream_t s = as_stream(stream);
    k_dot_partial_r<<<dim3((unsigned)nb, (unsigned)k), kThreads, 0, s>>>(V, ld, w, dim, partial);
    k_dot_final_r<<<(unsigned)k, kThreads, 0, s>>>(partial, (int)nb, out);
    return launch_status();
}

c3l_status c3l_multi_axpy_c(const c3l_complex* V, int64_t ld, int32_t k, const c3l_complex* c, c3l_complex alpha,
                            c3l_complex* w, int64_t dim, void* stream) {
    if (k < 0 || dim < 0) return C3L_ERR_ARGUMENT;
    if (k == 0 || dim == 0) return C3L_OK;
    if (!V || !c || !w || ld < dim) return C3L_ERR_ARGUMENT;
    const double2* Vd = reinterpret_cast<const double2*>(V);
    const double2* cd = reinterpret_cast<const double2*>(c);
    const double2 al = make_double2(alpha.re, alpha.im);
    double2* wd = reinterpret_cast<double2*>(w);
    if (k >= kAxYLong)
        k_axpy_c<kAxXLong, kAxYLong><<<axpy_grid(dim, kAxXLong), dim3(kAxXLong, kAxYLong), 0, as_stream(stream)>>>(
            Vd, ld, k, cd, al, wd, dim);
    else
        k_axpy_c<kAxX, kAxY><<<axpy_grid(dim), dim3(kAxX, kAxY), 0, as_stream(stream)>>>(Vd, ld, k, cd, al, wd, dim);
    return launch_status();
}

c3l_status c3l_multi_axpy_r(const double* V, int64_t ld, int32_t k, const double* c, double alpha, double* w,
                            int64_t dim, void* stream) {
    if (k < 0 || dim < 0) return C3L_ERR_ARGUMENT;
    if (k == 0 || dim == 0) return C3L_OK;
    if (!V || !c || !w || ld < dim) return C3L_ERR_ARGUMENT;
    k_axpy_r<<<axpy_grid(dim), dim3(kAxX, kAxY), 0, as_stream(stream)>>>(V, ld, k, c, alpha, w, dim);
    return launch_status();
}

c3l_status c3l_scale_c(int64_t dim, c3l_complex a, const c3l_complex* x, c3l_complex* y, void* stream) {
    if (dim < 0 || (dim > 0 && (!x || !y))) return C3L_ERR_ARGUMENT;
    if (dim == 0) return C3L_OK;
    k_scale_c<<<grid_for(dim), kThreads, 0, as_stream(stream)>>>(dim, make_double2(a.re, a.im),
                                                                 reinterpret_cast<const double2*>(x),
                                                                 reinterpret_cast<double2*>(y));
    return launch_status();
}

c3l_status c3l_scale_r(int64_t dim, double a, const double* x, double* y, void* stream) {
    if (dim < 0 || (dim > 0 && (!x || !y))) return C3L_ERR_ARGUMENT;
    if (dim == 0) return C3L_OK;
    k_scale_r<<<grid_for(dim), kThreads, 0, as_stream(stream)>>>(dim, a, x, y);
    return launch_status();
}

c3l_status c3l_shifted_combine(int64_t dim, c3l_complex z, const c3l_complex* x, const c3l_complex* s,
                               const c3l_complex* inv, c3l_complex* out, void* stream) {
    if (dim < 0 || (dim > 0 && (!x || !out))) return C3L_ERR_ARGUMENT;
    if (dim == 0) return C3L_OK;
    k_shifted_combine<<<grid_for(dim), kThreads, 0, as_stream(stream)>>>(
        dim, make_double2(z.re, z.im), reinterpret_cast<const double2*>(x), reinterpret_cast<const double2*>(s),
        reinterpret_cast<const double2*>(inv), reinterpret_cast<double2*>(out));
    return launch_status();
}

c3l_status c3l_precondition(int64_t nrep, const double* m4, const int64_t* col, const int64_t* pair, const double* x,
                            double* y, void* stream) {
    if (nrep < 0 || (nrep > 0 && (!m4 || !col || !pair || !x || !y))) return C3L_ERR_ARGUMENT;
    if (nrep == 0) return C3L_OK;
    k_precondition<<<grid_for(nrep), kThreads, 0, as_stream(stream)>>>(nrep, m4, col, pair, x, y);
    return launch_status();
}

static c3l_status set_smem(const void* fn, size_t bytes) {
    if (bytes > 48 * 1024) {
        if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
            return C3L_ERR_LAUNCH;
    }
    return C3L_OK;
}

c3l_status c3l_hessenberg_shifted(const c3l_complex* H, int64_t ldh, int32_t m, const c3l_complex* shifts, int32_t nshift,
                                  double beta, const c3l_complex* sinkproj, c3l_complex* green, double* residual,
                                  void* stream) {
    if (m <= 0 || nshift < 0 || !H || !shifts || ldh < m || !(beta > 0.0)) return C3L_ERR_ARGUMENT;
    if (m > C3L_MAX_HESSENBERG) return C3L_ERR_CAPACITY;
    if (nshift == 0) return C3L_OK;
    const size_t smem = 2 * (size_t)m * sizeof(double2);
    if (set_smem((const void*)k_hessenberg_shifted, smem)) return C3L_ERR_LAUNCH;
    k_hessenberg_shifted<<<(unsigned)nshift, kHessThreads, smem, as_stream(stream)>>>(
        reinterpret_cast<const double2*>(H), ldh, m, reinterpret_cast<const double2*>(shifts), beta,
        reinterpret_cast<const double2*>(sinkproj), reinterpret_cast<double2*>(green), residual);
    return launch_status();
}

c3l_status c3l_hessenberg_coordinates(const c3l_complex* H, int64_t ldh, int32_t m, const c3l_complex* shifts,
                                      int32_t nshift, double beta, c3l_complex* rscratch, c3l_complex* Y, void* stream) {
    if (m <= 0 || nshift < 0 || !H || !shifts || !rscratch || !Y || ldh < m || !(beta > 0.0)) return C3L_ERR_ARGUMENT;
    if (m > C3L_MAX_HESSENBERG) return C3L_ERR_CAPACITY;
    if (nshift == 0) return C3L_OK;
    const size_t smem = 2 * (size_t)m * sizeof(double2);
    if (set_smem((const void*)k_hessenberg_coordinates, smem)) return C3L_ERR_LAUNCH;
    k_hessenberg_coordinates<<<(unsigned)nshift, kHessThreads, smem, as_stream(stream)>>>(
        reinterpret_cast<const double2*>(H), ldh, m, reinterpret_cast<const double2*>(shifts), beta,
        reinterpret_cast<double2*>(rscratch), reinterpret_cast<double2*>(Y));
    return launch_status();
}

c3l_status c3l_hessenberg_coordinates_noalloc(const c3l_complex* H, int64_t ldh, int32_t m, const c3l_complex* shifts,
                                              int32_t nshift, double beta, c3l_complex* Y, void* stream) {
    if (m <= 0 || nshift < 0 || !H || !shifts || !Y || ldh < m || !(beta > 0.0)) return C3L_ERR_ARGUMENT;
    if (m > C3L_MAX_HESSENBERG) return C3L_ERR_CAPACITY;
    const int64_t per = (int64_t)m * (m + 1) / 2;
    if (per > (int64_t)C3L_NOALLOC_SCRATCH_ENTRIES) return C3L_ERR_CAPACITY;
    if (nshift == 0) return C3L_OK;
    double2* scratch = nullptr;
    c3l_status st = noalloc_scratch(&scratch);
    if (st) return st;
    const size_t smem = 2 * (size_t)m * sizeof(double2);
    if (set_smem((const void*)k_hessenberg_coordinates, smem)) return C3L_ERR_LAUNCH;
    // shifts are processed in chunks that fit the fixed scratch; chunks run
    // back to back on the caller's stream, so they reuse it in order
    const int32_t chunk = (int32_t)((int64_t)C3L_NOALLOC_SCRATCH_ENTRIES / per < nshift
                                        ? (int64_t)C3L_NOALLOC_SCRATCH_ENTRIES / per
                                        : nshift);
    for (int32_t s0 = 0; s0 < nshift; s0 += chunk) {
        const int32_t cnt = nshift - s0 < chunk ? nshift - s0 : chunk;
        k_hessenberg_coordinates<<<(unsigned)cnt, kHessThreads, smem, as_stream(stream)>>>(
            reinterpret_cast<const double2*>(H), ldh, m, reinterpret_cast<const double2*>(shifts) + s0, beta, scratch,
            reinterpret_cast<double2*>(Y) + (int64_t)s0 * m);
        if (cudaGetLastError() != cudaSuccess) return C3L_ERR_LAUNCH;
    }
    return C3L_OK;
}

c3l_status c3l_hessenberg_advance(c3l_hessenberg_state* st, const c3l_complex* Hc, int64_t ldc, int32_t m,
                                  void* stream) {
    c3l_hessenberg_state* states[1] = {st};
    const c3l_complex* hc[1] = {Hc};
    const int64_t lds[1] = {ldc};
    const int32_t ms[1] = {m};
    return c3l::hessenberg_advance_many(states, hc, lds, ms, 1, as_stream(stream));
}

c3l_status c3l_arnoldi_column(const c3l_complex* coeff, int32_t k, c3l_complex* w, int64_t n, c3l_complex* Hc, int64_t ldc,
                              int32_t j, double tol, void* stream) {
    if (!coeff || !w || !Hc || k <= 0 || n <= 0 || ldc < k + 1 || j < 0) return C3L_ERR_ARGUMENT;
    int64_t blocks = (n + kThreads - 1) / kThreads;
    if (blocks > 1024) blocks = 1024;
    k_arnoldi_column<<<(unsigned)blocks, kThreads, 0, as_stream(stream)>>>(
        reinterpret_cast<const double2*>(coeff), k, reinterpret_cast<double2*>(w), n, reinterpret_cast<double2*>(Hc), ldc,
        j, tol);
    return launch_status();
}

}  // extern "C"

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

#include <mutex>

#include "c3l_gb300.h"

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

// w[i] += alpha * sum_j c[j] V[j, i]: a 32 x 8 block covers 32 consecutive
// entries (coalesced in i) and splits the k rows over 8 thread rows, so a
// short vector with a long basis (Arnoldi) still fills the GPU.
constexpr int kAxX = 32, kAxY = 8;

__global__ void __launch_bounds__(kAxX * kAxY) k_axpy_c(const double2* __restrict__ V, int64_t ld, int k,
                                                         const double2* __restrict__ c, double2 alpha,
                                                         double2* __restrict__ w, int64_t dim) {
    __shared__ double2 part[kAxY][kAxX];
    for (int64_t base = (int64_t)blockIdx.x * kAxX; base < dim; base += (int64_t)gridDim.x * kAxX) {
        const int64_t i = base + threadIdx.x;
        double2 s = make_double2(0.0, 0.0);
        if (i < dim) {
            for (int j = threadIdx.y; j < k; j += kAxY) {
                const double2 p = cmul(c[j], V[(int64_t)j * ld + i]);
                s.x += p.x;
                s.y += p.y;
            }
        }
        part[threadIdx.y][threadIdx.x] = s;
        __syncthreads();
        if (threadIdx.y == 0 && i < dim) {
            double2 t = part[0][threadIdx.x];
#pragma unroll
            for (int y = 1; y < kAxY; ++y) {
                t.x += part[y][threadIdx.x].x;
                t.y += part[y][threadIdx.x].y;
            }
            const double2 a = cmul(alpha, t);
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

unsigned axpy_grid(int64_t dim) {
    int64_t b = (dim + kAxX - 1) / kAxX;
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

// FP32 residual-only variant used for Arnoldi convergence checks: the same
// streamed Givens elimination on (z I - H_m) rounded to single precision,
// returning |h_{m,m-1} y_{m-1}| / beta.  Its relative error is ~cond * 1e-7,
// ample for a stopping decision; a positive decision is confirmed in FP64.
__global__ void __launch_bounds__(kHessThreads) k_hessenberg_residual_f32(const double2* __restrict__ H, int64_t ldh,
                                                                          int m, const double2* __restrict__ shifts,
                                                                          double beta, double* __restrict__ residual) {
    extern __shared__ float2 dynf[];
    float2* w = dynf;
    __shared__ float rot_c;
    __shared__ float2 rot_s;
    const double2 zd = shifts[blockIdx.x];
    const float2 z = make_float2((float)zd.x, (float)zd.y);
    auto entry = [&](int row, int c) -> float2 {
        const double2 h = H[(int64_t)row * ldh + c];
        return (row == c) ? make_float2(z.x - (float)h.x, z.y - (float)h.y) : make_float2((float)-h.x, (float)-h.y);
    };
    for (int c = threadIdx.x; c < m; c += blockDim.x) w[c] = entry(0, c);
    float2 rhs = make_float2((float)beta, 0.0f);
    float2 ylast = make_float2(0.0f, 0.0f);
    // the running rhs is a product of sines and may fall below FP32 range:
    // keep it rescaled by powers of 1e20 and track the decimal exponent
    int rhs_exp = 0;
    int y_exp = 0;
    __syncthreads();
    for (int k = 0; k < m; ++k) {
        if (threadIdx.x == 0) {
            const float2 a = w[k];
            float c;
            float2 sn, rkk;
            if (k < m - 1) {
                const float2 b = entry(k + 1, k);
                const float na = hypotf(a.x, a.y), nb = hypotf(b.x, b.y);
                if (nb == 0.0f) {
                    c = 1.0f; sn = make_float2(0.0f, 0.0f); rkk = a;
                } else if (na == 0.0f) {
                    c = 0.0f; sn = make_float2(1.0f, 0.0f); rkk = b;
                } else {
                    const float rho = hypotf(na, nb);
                    c = na / rho;
                    const float2 ph = make_float2(a.x / na, a.y / na);
                    const float2 bb = make_float2(b.x / rho, -b.y / rho);
                    sn = make_float2(ph.x * bb.x - ph.y * bb.y, ph.x * bb.y + ph.y * bb.x);
                    rkk = make_float2(ph.x * rho, ph.y * rho);
                }
            } else {
                c = 1.0f; sn = make_float2(0.0f, 0.0f); rkk = a;
            }
            const float2 rrhs = make_float2(c * rhs.x, c * rhs.y);
            if (k == m - 1) {
                const float d = rkk.x * rkk.x + rkk.y * rkk.y;
                ylast = make_float2((rrhs.x * rkk.x + rrhs.y * rkk.y) / d, (rrhs.y * rkk.x - rrhs.x * rkk.y) / d);
                y_exp = rhs_exp;
            }
            rhs = make_float2(-sn.x * rhs.x - sn.y * rhs.y, -sn.x * rhs.y + sn.y * rhs.x);  // -conj(s) rhs
            const float mag = fmaxf(fabsf(rhs.x), fabsf(rhs.y));
            if (mag != 0.0f && mag < 1e-20f) {
                rhs.x *= 1e20f;
                rhs.y *= 1e20f;
                rhs_exp -= 20;
            }
            rot_c = c;
            rot_s = sn;
        }
        __syncthreads();
        const float cc = rot_c;
        const float2 ss = rot_s;
        for (int col = k + 1 + threadIdx.x; col < m; col += blockDim.x) {
            const float2 rv = (k < m - 1) ? entry(k + 1, col) : make_float2(0.0f, 0.0f);
            const float2 wv = w[col];
            // w' = -conj(s) w + c r
            w[col] = make_float2(-ss.x * wv.x - ss.y * wv.y + cc * rv.x, -ss.x * wv.y + ss.y * wv.x + cc * rv.y);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double2 hs = H[(int64_t)m * ldh + (m - 1)];
        residual[blockIdx.x] = hypot(hs.x, hs.y) * hypot((double)ylast.x, (double)ylast.y) * pow(10.0, (double)y_exp) / beta;
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

extern "C" {

int64_t c3l_multi_dot_scratch(int32_t k, int64_t dim) { return (int64_t)k * partial_blocks(k, dim); }

c3l_status c3l_multi_dot_c(const c3l_complex* V, int64_t ld, int32_t k, const c3l_complex* w, int64_t dim,
                           c3l_complex* partial, c3l_complex* out, void* stream) {
    if (k < 0 || dim < 0 || k > 65535) return C3L_ERR_ARGUMENT;
    if (k == 0) return C3L_OK;
    if (!V || !w || !partial || !out || ld < dim) return C3L_ERR_ARGUMENT;
    const int64_t nb = partial_blocks(k, dim);
    cudaStream_t s = as_stream(stream);
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
    k_axpy_c<<<axpy_grid(dim), dim3(kAxX, kAxY), 0, as_stream(stream)>>>(reinterpret_cast<const double2*>(V), ld, k,
                                                                reinterpret_cast<const double2*>(c),
                                                                make_double2(alpha.re, alpha.im),
                                                                reinterpret_cast<double2*>(w), dim);
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

c3l_status c3l_hessenberg_residual_f32(const c3l_complex* H, int64_t ldh, int32_t m, const c3l_complex* shifts,
                                       int32_t nshift, double beta, double* residual, void* stream) {
    if (m <= 0 || nshift < 0 || !H || !shifts || !residual || ldh < m || !(beta > 0.0)) return C3L_ERR_ARGUMENT;
    if (m > C3L_MAX_HESSENBERG) return C3L_ERR_CAPACITY;
    if (nshift == 0) return C3L_OK;
    const size_t smem = (size_t)m * sizeof(float2);
    if (set_smem((const void*)k_hessenberg_residual_f32, smem)) return C3L_ERR_LAUNCH;
    k_hessenberg_residual_f32<<<(unsigned)nshift, kHessThreads, smem, as_stream(stream)>>>(
        reinterpret_cast<const double2*>(H), ldh, m, reinterpret_cast<const double2*>(shifts), beta, residual);
    return launch_status();
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

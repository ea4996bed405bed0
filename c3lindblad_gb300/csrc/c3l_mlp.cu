// Learned warm start: an element-wise MLP over amplitude features (sm_103a).
//
// Network: F -> H -> H -> O with tanh hidden activations (F = 16, H = 32,
// O = 2).  Inputs, weights and saved activations are BF16; every dot product
// accumulates in FP32.  One thread evaluates one amplitude (one sample); the
// whole parameter set (1,666 values) sits in shared memory.
//
//   k_mlp_forward  -- y = W3 tanh(W2 tanh(W1 x + b1) + b2) + b3
//   k_mlp_backward -- recomputes the forward pass per sample, then the
//                     gradients of the weighted squared error: warp-shuffle
//                     reductions, one shared-memory atomic per warp and
//                     parameter, one global atomic per block and parameter
//   k_adam         -- Adam on FP32 master weights, refreshing the BF16 copy
//   k_warm_features / k_warm_apply -- assemble features from a problem's
//                     rapidities and first-order amplitudes, and turn the
//                     network output into an initial guess.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "c3l_gb300.h"

namespace {

constexpr int F = C3L_MLP_INPUTS;
constexpr int H = C3L_MLP_HIDDEN;
constexpr int O = C3L_MLP_OUTPUTS;
// parameter layout: W1[H][F] b1[H] W2[H][H] b2[H] W3[O][H] b3[O]
constexpr int oW1 = 0, oB1 = oW1 + H * F, oW2 = oB1 + H, oB2 = oW2 + H * H, oW3 = oB2 + H, oB3 = oW3 + O * H;
constexpr int P = oB3 + O;
static_assert(P == C3L_MLP_PARAMS, "parameter count");
constexpr int kThreads = 256;

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }
inline c3l_status launch_status() { return cudaGetLastError() == cudaSuccess ? C3L_OK : C3L_ERR_LAUNCH; }

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }

__device__ __forceinline__ void load_params(const __nv_bfloat16* __restrict__ wb, float* sp) {
    for (int i = threadIdx.x; i < P; i += blockDim.x) sp[i] = bf(wb[i]);
    __syncthreads();
}

__device__ __forceinline__ void forward_one(const float* sp, const float* x, float* h1, float* h2, float* y) {
#pragma unroll 4
    for (int j = 0; j < H; ++j) {
        float a = sp[oB1 + j];
#pragma unroll
        for (int i = 0; i < F; ++i) a = fmaf(sp[oW1 + j * F + i], x[i], a);
        // the saved activation is rounded to BF16 exactly as stored
        h1[j] = bf(__float2bfloat16(tanhf(a)));
    }
#pragma unroll 4
    for (int j = 0; j < H; ++j) {
        float a = sp[oB2 + j];
#pragma unroll 8
        for (int i = 0; i < H; ++i) a = fmaf(sp[oW2 + j * H + i], h1[i], a);
        h2[j] = bf(__float2bfloat16(tanhf(a)));
    }
#pragma unroll
    for (int o = 0; o < O; ++o) {
        float a = sp[oB3 + o];
#pragma unroll 8
        for (int i = 0; i < H; ++i) a = fmaf(sp[oW3 + o * H + i], h2[i], a);
        y[o] = a;
    }
}

__global__ void __launch_bounds__(kThreads) k_mlp_forward(int64_t n, const __nv_bfloat16* __restrict__ X,
                                                          const __nv_bfloat16* __restrict__ wb, float* __restrict__ Y) {
    __shared__ float sp[P];
    load_params(wb, sp);
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        float x[F], h1[H], h2[H], y[O];
#pragma unroll
        for (int i = 0; i < F; ++i) x[i] = bf(X[s * F + i]);
        forward_one(sp, x, h1, h2, y);
#pragma unroll
        for (int o = 0; o < O; ++o) Y[s * O + o] = y[o];
    }
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Adds one per-lane gradient contribution to a shared accumulator: a warp
// reduction first, then a single shared-memory atomic from lane 0.
__device__ __forceinline__ void acc_param(float* sg, int idx, float v, int lane) {
    v = warp_sum(v);
    if (lane == 0) atomicAdd(&sg[idx], v);
}

// Loss = sum_s w_s |y_s - t_s|^2 / sum_s w_s; gradient accumulated into grad[P],
// loss numerator into loss[0].  Every lane of a warp stays active (lanes past
// the end carry zero weight) so the warp reductions are uniform.
__global__ void __launch_bounds__(kThreads) k_mlp_backward(int64_t n, const __nv_bfloat16* __restrict__ X,
                                                           const float* __restrict__ T, const float* __restrict__ W,
                                                           float inv_wsum, const __nv_bfloat16* __restrict__ wb,
                                                           float* __restrict__ grad, float* __restrict__ loss) {
    __shared__ float sp[P];
    __shared__ float sg[P];
    __shared__ float sl;
    for (int i = threadIdx.x; i < P; i += blockDim.x) sg[i] = 0.0f;
    if (threadIdx.x == 0) sl = 0.0f;
    load_params(wb, sp);
    const int lane = threadIdx.x & 31;
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = base + threadIdx.x;
        const bool act = s < n;
        float x[F], h1[H], h2[H], y[O];
#pragma unroll
        for (int i = 0; i < F; ++i) x[i] = act ? bf(X[s * F + i]) : 0.0f;
        forward_one(sp, x, h1, h2, y);
        const float w = act ? (W ? W[s] : 1.0f) : 0.0f;
        float dy[O];
        float l = 0.0f;
#pragma unroll
        for (int o = 0; o < O; ++o) {
            const float e = act ? y[o] - T[s * O + o] : 0.0f;
            l = fmaf(w * e, e, l);
            dy[o] = 2.0f * w * e * inv_wsum;
            acc_param(sg, oB3 + o, dy[o], lane);
        }
        l = warp_sum(l);
        if (lane == 0) atomicAdd(&sl, l);
        // layer 3 and the hidden-2 error
        float d2[H];
#pragma unroll 4
        for (int i = 0; i < H; ++i) {
            float g = 0.0f;
#pragma unroll
            for (int o = 0; o < O; ++o) {
                acc_param(sg, oW3 + o * H + i, dy[o] * h2[i], lane);
                g = fmaf(sp[oW3 + o * H + i], dy[o], g);
            }
            d2[i] = g * (1.0f - h2[i] * h2[i]);
            acc_param(sg, oB2 + i, d2[i], lane);
        }
        // layer 2 and the hidden-1 error
        float d1[H];
#pragma unroll
        for (int i = 0; i < H; ++i) d1[i] = 0.0f;
        for (int j = 0; j < H; ++j) {
            const float dj = d2[j];
#pragma unroll
            for (int i = 0; i < H; ++i) {
                acc_param(sg, oW2 + j * H + i, dj * h1[i], lane);
                d1[i] = fmaf(sp[oW2 + j * H + i], dj, d1[i]);
            }
        }
        // layer 1
        for (int j = 0; j < H; ++j) {
            const float dj = d1[j] * (1.0f - h1[j] * h1[j]);
            acc_param(sg, oB1 + j, dj, lane);
#pragma unroll
            for (int i = 0; i < F; ++i) acc_param(sg, oW1 + j * F + i, dj * x[i], lane);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < P; i += blockDim.x) atomicAdd(&grad[i], sg[i]);
    if (threadIdx.x == 0) atomicAdd(loss, sl);
}

__global__ void k_adam(int n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2,
                       __nv_bfloat16* __restrict__ pb) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float step = lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        p[i] -= step;
        pb[i] = __float2bfloat16(p[i]);
    }
}

// Features per tilde-orbit representative r (cols/pairs from the tilde tables):
//   [Re, Im] of the rapidity of each of up to four modes (0 where absent),
//   a degree flag (+1 doubles, -1 singles), the interaction scale u, the two
//   Jacobi iterates (x[c], x[c+1]) / sigma and their log-magnitudes.
__global__ void k_warm_features(int64_t nrep, const int64_t* __restrict__ modes, const int64_t* __restrict__ col,
                                const int64_t* __restrict__ pair, const double2* __restrict__ rapidities,
                                const double* __restrict__ t1, const double* __restrict__ t2, double inv_sigma,
                                double u, __nv_bfloat16* __restrict__ X) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrep; r += (int64_t)gridDim.x * blockDim.x) {
        float f[F];
        int deg = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int64_t md = modes[r * 4 + k];
            float re = 0.0f, im = 0.0f;
            if (md >= 0) {
                const double2 lam = rapidities[md];
                re = (float)lam.x;
                im = (float)lam.y;
                ++deg;
            }
            f[2 * k] = re;
            f[2 * k + 1] = im;
        }
        f[8] = deg > 2 ? 1.0f : -1.0f;
        f[9] = (float)u;
        const int64_t c = col[r];
        const bool pr = pair[r] != 0;
        const double a1 = t1[c] * inv_sigma, b1 = pr ? t1[c + 1] * inv_sigma : 0.0;
        const double a2 = t2[c] * inv_sigma, b2 = pr ? t2[c + 1] * inv_sigma : 0.0;
        f[10] = (float)a1;
        f[11] = (float)b1;
        f[12] = (float)a2;
        f[13] = (float)b2;
        f[14] = (float)(0.5 * log10(hypot(a1, b1) + 1e-6));
        f[15] = (float)(0.5 * log10(hypot(a2, b2) + 1e-6));
#pragma unroll
        for (int i = 0; i < F; ++i) X[r * F + i] = __float2bfloat16(f[i]);
    }
}

__global__ void k_warm_apply(int64_t nrep, const int64_t* __restrict__ col, const int64_t* __restrict__ pair,
                             const double* __restrict__ t1, const float* __restrict__ Y, double sigma,
                             double* __restrict__ x0) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrep; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = col[r];
        x0[c] = t1[c] + sigma * (double)Y[r * O];
        if (pair[r]) x0[c + 1] = t1[c + 1] + sigma * (double)Y[r * O + 1];
    }
}

unsigned grid_for(int64_t n, int64_t cap) {
    int64_t b = (n + kThreads - 1) / kThreads;
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace

extern "C" {

c3l_status c3l_mlp_forward(int64_t n, const void* X, const void* weights_bf16, float* Y, void* stream) {
    if (n < 0 || (n > 0 && (!X || !weights_bf16 || !Y))) return C3L_ERR_ARGUMENT;
    if (n == 0) return C3L_OK;
    k_mlp_forward<<<grid_for(n, 4096), kThreads, 0, as_stream(stream)>>>(
        n, static_cast<const __nv_bfloat16*>(X), static_cast<const __nv_bfloat16*>(weights_bf16), Y);
    return launch_status();
}

c3l_status c3l_mlp_backward(int64_t n, const void* X, const float* T, const float* W, float inv_wsum,
                            const void* weights_bf16, float* grad, float* loss, void* stream) {
    if (n < 0 || (n > 0 && (!X || !T || !weights_bf16 || !grad || !loss))) return C3L_ERR_ARGUMENT;
    if (n == 0) return C3L_OK;
    k_mlp_backward<<<grid_for(n, 1216), kThreads, 0, as_stream(stream)>>>(
        n, static_cast<const __nv_bfloat16*>(X), T, W, inv_wsum, static_cast<const __nv_bfloat16*>(weights_bf16), grad,
        loss);
    return launch_status();
}

c3l_status c3l_mlp_adam(float* params, const float* grad, float* m, float* v, float lr, float beta1, float beta2,
                        float eps, int32_t step, void* weights_bf16, void* stream) {
    if (!params || !grad || !m || !v || !weights_bf16 || step < 1) return C3L_ERR_ARGUMENT;
    const float c1 = 1.0f - powf(beta1, (float)step);
    const float c2 = 1.0f - powf(beta2, (float)step);
    k_adam<<<grid_for(P, 64), kThreads, 0, as_stream(stream)>>>(P, params, grad, m, v, lr, beta1, beta2, eps, c1, c2,
                                                               static_cast<__nv_bfloat16*>(weights_bf16));
    return launch_status();
}

c3l_status c3l_warm_features(int64_t nrep, const int64_t* modes, const int64_t* col, const int64_t* pair,
                             const c3l_complex* rapidities, const double* t1, const double* t2, double sigma,
                             double u, void* X, void* stream) {
    if (nrep < 0 || !(sigma > 0.0) || (nrep > 0 && (!modes || !col || !pair || !rapidities || !t1 || !t2 || !X)))
        return C3L_ERR_ARGUMENT;
    if (nrep == 0) return C3L_OK;
    k_warm_features<<<grid_for(nrep, 4096), kThreads, 0, as_stream(stream)>>>(
        nrep, modes, col, pair, reinterpret_cast<const double2*>(rapidities), t1, t2, 1.0 / sigma, u,
        static_cast<__nv_bfloat16*>(X));
    return launch_status();
}

c3l_status c3l_warm_apply(int64_t nrep, const int64_t* col, const int64_t* pair, const double* t1, const float* Y,
                          double sigma, double* x0, void* stream) {
    if (nrep < 0 || (nrep > 0 && (!col || !pair || !t1 || !Y || !x0))) return C3L_ERR_ARGUMENT;
    if (nrep == 0) return C3L_OK;
    k_warm_apply<<<grid_for(nrep, 4096), kThreads, 0, as_stream(stream)>>>(nrep, col, pair, t1, Y, sigma, x0);
    return launch_status();
}

}  // extern "C"

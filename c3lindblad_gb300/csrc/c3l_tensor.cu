// Tensor-program kernels of the coupled-cluster hot path (sm_103a).
//
// The compiled program (c3lindblad_gb300/compiler.py) reduces the factorized
// CCSD residual, its JVP and the EOM sigma action to three kernel families:
//
//   k_contract  -- builds atoms: padded blocks of interior products
//                  (iota_a T, iota_b iota_a T, ...) of the amplitudes or of a
//                  direction/response vector, one n-term dot product per entry.
//   k_wedge     -- sums shuffle-signed products of padded block entries
//                  ("instances") per output element: rest forms into padded
//                  workspace blocks, and anchor ^ rest at canonical outputs
//                  with the residual/sigma epilogue fused in.
//   k_scatter / k_tilde_unpack -- move vectors between the reference's
//                  canonical layout and the padded workspace.
//
// Every kernel is templated on the workspace element: complex FP64 (double2)
// for residuals, sources and the refinement path, complex FP32 (float2) for
// the inner Krylov operator of the mixed-precision Newton solve.  FP64 runs
// on a narrow pipe on this part, FP32 on the full-width one.  Epilogues
// (the rapidity diagonal and the -i factor) are always evaluated in FP64.
// Instances of one output block are staged through shared memory and split
// over four thread groups.
#include <cuda_runtime.h>
#include <cstring>
#include <type_traits>
#include <stdint.h>

#include "c3l_gb300.h"
#include "c3l_internal.h"
#include "c3l_df.h"
#include "c3l_pdl.h"

namespace {

constexpr int kThreads = 256;
constexpr int kInstChunk = 32;

template <typename C> struct Cx;
template <> struct Cx<double2> {
    using R = double;
    static __device__ __forceinline__ double2 make(double a, double b) { return make_double2(a, b); }
};
template <> struct Cx<float2> {
    using R = float;
    static __device__ __forceinline__ float2 make(double a, double b) { return make_float2((float)a, (float)b); }
};

template <typename C>
__device__ __forceinline__ C cmul(C a, C b) {
    C r;
    r.x = fma(a.x, b.x, -a.y * b.y);
    r.y = fma(a.x, b.y, a.y * b.x);
    return r;
}
template <typename C>
__device__ __forceinline__ C cadd(C a, C b) {
    C r;
    r.x = a.x + b.x;
    r.y = a.y + b.y;
    return r;
}
template <typename C>
__device__ __forceinline__ C cfma(C a, C b, C c) {  // a*b + c
    C r;
    r.x = fma(a.x, b.x, fma(-a.y, b.y, c.x));
    r.y = fma(a.x, b.y, fma(a.y, b.x, c.y));
    return r;
}
template <typename C>
__device__ __forceinline__ double2 to_d2(C a) {
    return make_double2((double)a.x, (double)a.y);
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline c3l_status launch_status() {
    return cudaGetLastError() == cudaSuccess ? C3L_OK : C3L_ERR_LAUNCH;
}

// Entries of a batched launch (blockIdx.y = entry): the same program over
// separate workspaces, inputs and outputs; an entry whose stop flag is set
// does nothing.  Unbatched launches use entry 0 only.
template <typename C>
struct Batch {
    C* ws[C3L_MAX_BATCH];
    const double2* in[C3L_MAX_BATCH];   // scatter source and output-stage input
    double2* out[C3L_MAX_BATCH];        // complex output-stage destination
    float2* out32[C3L_MAX_BATCH];       // optional FP32 copy of the EOM output
    const int32_t* stop[C3L_MAX_BATCH];
    int nb;
    bool pdl;         // launch with programmatic dependent launch
    bool pdl_at_exit; // dependents launch only as the blocks exit (no early trigger)
};

template <typename C>
__device__ __forceinline__ bool batch_stopped(const Batch<C>& bt) {
    const int32_t* f = bt.stop[blockIdx.y];
    return f && *f;
}

__device__ __forceinline__ double2 tilde_value(const double* __restrict__ x, const int64_t* __restrict__ ia,
                                               const int64_t* __restrict__ ib, const double2* __restrict__ ca,
                                               const double2* __restrict__ cb, int64_t i) {
    const double xa = x[ia[i]];
    const double xb = x[ib[i]];
    const double2 a = ca[i];
    const double2 b = cb[i];
    return make_double2(fma(a.x, xa, b.x * xb), fma(a.y, xa, b.y * xb));
}

__global__ void k_tilde_unpack(int64_t dim, const double* __restrict__ x, const int64_t* __restrict__ ia,
                               const int64_t* __restrict__ ib, const double2* __restrict__ ca,
                               const double2* __restrict__ cb, double2* __restrict__ t) {
    c3l::pdl_launch_dependents();
    c3l::pdl_wait();  // x is the previous kernel's output (a no-op without programmatic launch)
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x)
        t[i] = tilde_value(x, ia, ib, ca, cb, i);
}

// Scatter entries from which a static action unpacks into the canonical
// vector first and scatters from it (two launches: the fused kernel below
// re-reads 48 bytes of tilde tables and two x entries per padded entry, which
// costs more than the second launch once the padded blocks are large).
constexpr int64_t kSplitScatter = 1 << 20;  // runtime.SPLIT_SCATTER counts the launches the same way

// The tilde unpack and the scatter into padded blocks in one launch: t[i]
// for the canonical vector (read again by the output stage) and, per scatter
// entry, ws[dst[e]] = sign[e] t[pos[e]] computed from x directly (the same
// arithmetic as k_tilde_unpack followed by k_scatter).
template <typename C>
__global__ void k_unpack_scatter(int64_t dim, const double* __restrict__ x, const int64_t* __restrict__ ia,
                                 const int64_t* __restrict__ ib, const double2* __restrict__ ca,
                                 const double2* __restrict__ cb, double2* __restrict__ t, int64_t count,
                                 const int64_t* __restrict__ dst, const int64_t* __restrict__ pos,
                                 const double* __restrict__ sign, C* __restrict__ ws) {
    c3l::pdl_launch_dependents();
    const int64_t n = dim > count ? dim : count;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    // the thread's first entry: every index and coefficient is a program table,
    // read before the wait; x (the previous kernel's output) after it
    int64_t a0 = 0, b0 = 0, pa = 0, pb = 0, d0 = 0;
    double2 ca0 = make_double2(0.0, 0.0), cb0 = ca0, cap = ca0, cbp = ca0;
    double sg = 0.0;
    if (i0 < dim) {
        a0 = ia[i0];
        b0 = ib[i0];
        ca0 = ca[i0];
        cb0 = cb[i0];
    }
    if (i0 < count) {
        sg = sign[i0];
        d0 = dst[i0];
        if (sg != 0.0) {
            const int64_t p = pos[i0];
            pa = ia[p];
            pb = ib[p];
            cap = ca[p];
            cbp = cb[p];
        }
    }
    c3l::pdl_wait();
    if (i0 < dim) {
        const double xa = x[a0], xb = x[b0];
        t[i0] = make_double2(fma(ca0.x, xa, cb0.x * xb), fma(ca0.y, xa, cb0.y * xb));
    }
    if (i0 < count) {
        double2 v = make_double2(0.0, 0.0);
        if (sg != 0.0) {
            const double xa = x[pa], xb = x[pb];
            const double2 u = make_double2(fma(cap.x, xa, cbp.x * xb), fma(cap.y, xa, cbp.y * xb));
            v = make_double2(sg * u.x, sg * u.y);
        }
        ws[d0] = Cx<C>::make(v.x, v.y);
    }
    for (int64_t i = i0 + stride; i < n; i += stride) {  // grids smaller than n (not the usual launch)
        if (i < dim) t[i] = tilde_value(x, ia, ib, ca, cb, i);
        if (i < count) {
            const double s2 = sign[i];
            double2 v = make_double2(0.0, 0.0);
            if (s2 != 0.0) {
                const double2 u = tilde_value(x, ia, ib, ca, cb, pos[i]);
                v = make_double2(s2 * u.x, s2 * u.y);
            }
            ws[dst[i]] = Cx<C>::make(v.x, v.y);
        }
    }
}

template <typename C>
__global__ void k_scatter(int64_t count, const int64_t* __restrict__ dst, const int64_t* __restrict__ pos,
                          const double* __restrict__ sign, Batch<C> bt) {
    if (!bt.pdl_at_exit) c3l::pdl_launch_dependents();
    if (batch_stopped(bt)) return;
    const double2* __restrict__ vec = bt.in[blockIdx.y];
    C* __restrict__ ws = bt.ws[blockIdx.y];
    const int64_t e0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    // the first entry's table values before the wait, the vector after it
    double s0 = 0.0;
    int64_t p0 = 0, d0 = 0;
    if (e0 < count) {
        s0 = sign[e0];
        p0 = pos[e0];
        d0 = dst[e0];
    }
    c3l::pdl_wait();
    if (e0 < count) {
        double2 v = make_double2(0.0, 0.0);
        if (s0 != 0.0) {
            const double2 u = vec[p0];
            v = make_double2(s0 * u.x, s0 * u.y);
        }
        ws[d0] = Cx<C>::make(v.x, v.y);
    }
    for (int64_t e = e0 + (int64_t)gridDim.x * blockDim.x; e < count; e += (int64_t)gridDim.x * blockDim.x) {
        const double s = sign[e];
        double2 v = make_double2(0.0, 0.0);
        if (s != 0.0) {
            const double2 u = vec[pos[e]];
            v = make_double2(s * u.x, s * u.y);
        }
        ws[dst[e]] = Cx<C>::make(v.x, v.y);
    }
}

__global__ void k_downcast(int64_t count, const double2* __restrict__ src, float2* __restrict__ dst) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x) {
        const double2 v = src[e];
        dst[e] = make_float2((float)v.x, (float)v.y);
    }
}

__device__ __forceinline__ void powers(int n, int64_t* pw) {
    pw[0] = 1;
#pragma unroll
    for (int i = 1; i < 6; ++i) pw[i] = pw[i - 1] * n;
}

constexpr int kContractChunk = 16;  // source and factor loads issued together per entry

// One padded entry e of a contraction task: const + sum_j sign_j sum_m
// vec_j[m] src_j[... m at axis_j ...] (interior products).  Each chunk of up
// to 16 strided source entries and their factor entries is loaded before any
// is used, so the loads' latencies overlap.
template <typename C>
__device__ __forceinline__ void contract_entry(const c3l_contract_task& task, int64_t e, int n, const int64_t* pw,
                                               const C* __restrict__ vectors, C* __restrict__ ws) {
    C acc = Cx<C>::make(0.0, 0.0);
    if (task.const_off >= 0) acc = vectors[task.const_off + e];
    for (int j = 0; j < task.nsrc; ++j) {
        const int axis = task.axis[j];
        // entries of a padded block are below n^deg < 2^32 (n <= 255 for the
        // degree-4 blocks, n <= 73 for the rank-five response shell): 32-bit division
        const uint32_t low = (uint32_t)pw[task.deg - axis];
        const uint32_t hi = (uint32_t)e / low;
        const uint32_t lo = (uint32_t)e - hi * low;
        const C* src = ws + task.src_off[j] + (int64_t)hi * low * n + lo;
        const C* vec = vectors + task.vec_off[j];
        C sum = Cx<C>::make(0.0, 0.0);
        for (int m0 = 0; m0 < n; m0 += kContractChunk) {
            C v[kContractChunk], f[kContractChunk];
#pragma unroll
            for (int u = 0; u < kContractChunk; ++u)
                if (m0 + u < n) {
                    v[u] = src[(int64_t)(m0 + u) * low];
                    f[u] = vec[m0 + u];
                }
            C s0 = Cx<C>::make(0.0, 0.0), s1 = s0;
#pragma unroll
            for (int u = 0; u < kContractChunk; u += 2) {
                if (m0 + u < n) s0 = cfma(f[u], v[u], s0);
                if (m0 + u + 1 < n) s1 = cfma(f[u + 1], v[u + 1], s1);
            }
            sum = cadd(sum, cadd(s0, s1));
        }
        const typename Cx<C>::R sg = (typename Cx<C>::R)task.sign[j];
        acc.x = fma(sg, sum.x, acc.x);
        acc.y = fma(sg, sum.y, acc.y);
    }
    ws[task.dst_off + e] = acc;
}

template <typename C>
__global__ void __launch_bounds__(kThreads) k_contract(c3l_contract_level lv, int n, const C* __restrict__ vectors,
                                                        Batch<C> bt) {
    if (!bt.pdl_at_exit) c3l::pdl_launch_dependents();
    if (batch_stopped(bt)) return;
    C* __restrict__ ws = bt.ws[blockIdx.y];
    const c3l_tile tile = lv.tiles[blockIdx.x];
    if ((int)threadIdx.x >= tile.count) return;
    const c3l_contract_task task = lv.tasks[tile.block];  // program tables: read before the wait
    int64_t pw[6];
    powers(n, pw);
    c3l::pdl_wait();
    contract_entry<C>(task, tile.start + threadIdx.x, n, pw, vectors, ws);
}

// The small trailing contraction levels (each at most one tile per CTA, each
// level depending on the previous one) as one launch of one thread-block
// cluster: CTA c computes tile c of each level, then the cluster meets at a
// hardware cluster barrier (release/acquire) before the next level.  Every
// CTA reaches every barrier (the level loop's bounds are the same in all
// CTAs).  Batch entries are separate clusters (blockIdx.y); a stopped
// entry's CTAs all return before the first barrier.
constexpr int kLevelClusterMax = 16;  // non-portable cluster size where the device allows it

struct LevelPack {
    c3l_contract_level lv[C3L_MAX_LEVELS];
    int first;
    int count;
};

template <typename C>
__global__ void __launch_bounds__(kThreads) k_contract_cluster(LevelPack pack, int n, const C* __restrict__ vectors,
                                                                Batch<C> bt) {
    if (!bt.pdl_at_exit) c3l::pdl_launch_dependents();
    if (batch_stopped(bt)) return;
    C* __restrict__ ws = bt.ws[blockIdx.y];
    // Every level has at most gridDim.x tiles (the launcher's condition), so a
    // CTA owns at most one tile per level: its tiles and their tasks are
    // fetched for all levels at once, before the first level runs.
    __shared__ c3l_tile stile[C3L_MAX_LEVELS];
    __shared__ c3l_contract_task stask[C3L_MAX_LEVELS];
    static_assert(sizeof(c3l_contract_task) % sizeof(int64_t) == 0, "task records are copied as 8-byte words");
    constexpr int kTaskWords = sizeof(c3l_contract_task) / sizeof(int64_t);
    if ((int)threadIdx.x < pack.count) {
        const c3l_contract_level& lv = pack.lv[pack.first + threadIdx.x];
        c3l_tile t{};
        if ((int64_t)blockIdx.x < lv.ntiles) t = lv.tiles[blockIdx.x];
        stile[threadIdx.x] = t;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < pack.count * kTaskWords; q += blockDim.x) {
        const int l = q / kTaskWords;
        if ((int64_t)blockIdx.x < pack.lv[pack.first + l].ntiles)
            reinterpret_cast<int64_t*>(&stask[l])[q - l * kTaskWords] =
                reinterpret_cast<const int64_t*>(&pack.lv[pack.first + l].tasks[stile[l].block])[q - l * kTaskWords];
    }
    __syncthreads();
    int64_t pw[6];
    powers(n, pw);
    c3l::pdl_wait();  // the tables above are constant; the workspace is not
    for (int i = 0; i < pack.count; ++i) {
        if ((int64_t)blockIdx.x < pack.lv[pack.first + i].ntiles && (int)threadIdx.x < stile[i].count)
            contract_entry<C>(stask[i], stile[i].start + threadIdx.x, n, pw, vectors, ws);
        // the next level reads this one's outputs; after the last level the
        // kernel's end publishes them (no shared memory of other CTAs is used)
        if (i + 1 < pack.count)
            asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
    }
}

// Pair GEMMs (c3l_pair_program): one thread block computes one tile of
// P_g = sum_k A_k^T R_k, whose operand rows A_k = ws[aoff[k] ...] and
// R_k = ws[roff[k] ...] sit anywhere in the workspace (atoms and rest forms).
// The tile's shape (c3l_pair_tile.shape) is chosen per group by the compiler:
// 16 x 16 threads, each accumulating an RM x RN block of complex entries
// (rows tm + 16 i, columns tn + 16 j), so a 64 x 64 tile (4 x 4) feeds four
// products from every shared-memory read and the 32 x 128 / 16 x 256 tiles
// (and their transposes) keep groups of 27 or 65 rows from running mostly
// padding.  Chunks of 8 anchors are staged through shared memory, the next
// chunk's rows loaded into registers while the current one is multiplied.
// One-column groups (N = 1) are matrix-vector products with their own tiles.
//
// The arithmetic is a policy: PairPlain<C> (complex FMAs in C) or PairDf
// (double-float on the FP32 pipe); both accumulate every entry over the
// anchors in anchor order.
constexpr int kPairChunk = 8;
constexpr int kPairThreads = 256;
constexpr int kPairMaxEdge = 256;  // rows plus columns of the largest tile: 16 + 256 (staged per chunk)

template <typename C>
struct PairPlain {
    using Elem = C;  // workspace entry
    using S = C;     // staged entry
    using A = C;     // accumulator
    static __device__ __forceinline__ S stage(C v) { return v; }
    static __device__ __forceinline__ A zero() { return Cx<C>::make(0.0, 0.0); }
    static __device__ __forceinline__ void mac(A& acc, const S& a, const S& b) { acc = cfma(a, b, acc); }
    static __device__ __forceinline__ void add(A& acc, const A& b) { acc = cadd(acc, b); }
    static __device__ __forceinline__ C finish(const A& acc) { return acc; }
};

// Operand entries are split into FP32 (hi, lo) pairs as they are staged
// (complex: re hi, re lo, im hi, im lo; from the bits of the double, so the
// staging issues no FP64 instruction); each real product is formed to about
// 2^-46 (Dekker's product with one FMA, df_mac) and summed by TwoSum into a
// (sum, correction) pair per real component, finished in FP64 when P is
// written.  The result differs from an FP64 GEMM by about 1e-14 of
// sum_k |A_k[i]| |R_k[j]|, at several times the FP64 pipe's rate.
struct PairDf {
    using Elem = double2;
    using S = float4;  // (re hi, re lo, im hi, im lo)
    using A = float4;  // (re sum, re correction, im sum, im correction)
    static __device__ __forceinline__ S stage(double2 v) {
        float4 q;
        split_d_bits(v.x, q.x, q.y);
        split_d_bits(v.y, q.z, q.w);
        return q;
    }
    static __device__ __forceinline__ A zero() { return make_float4(0.0f, 0.0f, 0.0f, 0.0f); }
    static __device__ __forceinline__ void mac(A& c, const S& a, const S& b) {
        // re += ar br - ai bi, im += ar bi + ai br
        df_mac(c.x, c.y, a.x, a.y, b.x, b.y);
        df_mac(c.x, c.y, -a.z, -a.w, b.z, b.w);
        df_mac(c.z, c.w, a.x, a.y, b.z, b.w);
        df_mac(c.z, c.w, a.z, a.w, b.x, b.y);
    }
    static __device__ __forceinline__ void add(A& c, const A& b) {
        df_add(c.x, c.y, b.x, b.y);
        df_add(c.z, c.w, b.z, b.w);
    }
    static __device__ __forceinline__ double2 finish(const A& c) {
        return make_double2((double)c.x + (double)c.y, (double)c.z + (double)c.w);
    }
};

// A (16 RM) x (16 RN) tile.  The loader stages entry e of a chunk's anchor
// rows (e < 8 TM: row e % TM of anchor e / TM) from thread e % 256, and the
// same for the rest rows.
template <class Op, int RM, int RN>
__device__ __forceinline__ void pair_tile(const c3l_pair_program& pp, const c3l_pair_tile& t,
                                          const c3l_pair_group& g, typename Op::Elem* __restrict__ ws,
                                          typename Op::S* smem) {
    using E = typename Op::Elem;
    using S = typename Op::S;
    using A = typename Op::A;
    constexpr int TM = 16 * RM, TN = 16 * RN;
    constexpr int LA = (kPairChunk * TM + kPairThreads - 1) / kPairThreads;
    constexpr int LB = (kPairChunk * TN + kPairThreads - 1) / kPairThreads;
    static_assert(TM + TN <= kPairMaxEdge + 16, "tile larger than the staging buffer");
    S* sa = smem;                     // [kPairChunk][TM]
    S* sr = smem + kPairChunk * TM;   // [kPairChunk][TN]
    const int tid = threadIdx.x, tm = tid / 16, tn = tid % 16;
    const E zero = Cx<E>::make(0.0, 0.0);
    E av[LA], rv[LB];
    auto load = [&](int64_t k0) {
#pragma unroll
        for (int u = 0; u < LA; ++u) {
            const int e = tid + kPairThreads * u;
            const int64_t k = k0 + e / TM;
            const int m = t.m0 + e % TM;
            av[u] = (e < kPairChunk * TM && k < g.kend && m < g.M) ? ws[pp.aoff[k] + m] : zero;
        }
#pragma unroll
        for (int u = 0; u < LB; ++u) {
            const int e = tid + kPairThreads * u;
            const int64_t k = k0 + e / TN;
            const int nn = t.n0 + e % TN;
            rv[u] = (e < kPairChunk * TN && k < g.kend && nn < g.N) ? ws[pp.roff[k] + nn] : zero;
        }
    };
    load(g.kbegin);
    A acc[RM][RN];
#pragma unroll
    for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int j = 0; j < RN; ++j) acc[i][j] = Op::zero();
    for (int64_t k0 = g.kbegin; k0 < g.kend; k0 += kPairChunk) {
        __syncthreads();  // the previous chunk has been used
#pragma unroll
        for (int u = 0; u < LA; ++u) {
            const int e = tid + kPairThreads * u;
            if (e < kPairChunk * TM) sa[e] = Op::stage(av[u]);
        }
#pragma unroll
        for (int u = 0; u < LB; ++u) {
            const int e = tid + kPairThreads * u;
            if (e < kPairChunk * TN) sr[e] = Op::stage(rv[u]);
        }
        __syncthreads();
        if (k0 + kPairChunk < g.kend) load(k0 + kPairChunk);  // in flight during this chunk's products
#pragma unroll 2
        for (int r = 0; r < kPairChunk; ++r) {
            if constexpr (RM <= RN) {
                S a[RM];
#pragma unroll
                for (int i = 0; i < RM; ++i) a[i] = sa[r * TM + tm + 16 * i];
#pragma unroll
                for (int j = 0; j < RN; ++j) {
                    const S b = sr[r * TN + tn + 16 * j];
#pragma unroll
                    for (int i = 0; i < RM; ++i) Op::mac(acc[i][j], a[i], b);
                }
            } else {
                S b[RN];
#pragma unroll
                for (int j = 0; j < RN; ++j) b[j] = sr[r * TN + tn + 16 * j];
#pragma unroll
                for (int i = 0; i < RM; ++i) {
                    const S a = sa[r * TM + tm + 16 * i];
#pragma unroll
                    for (int j = 0; j < RN; ++j) Op::mac(acc[i][j], a, b[j]);
                }
            }
        }
    }
    E* __restrict__ P = ws + pp.base + g.p_off;
#pragma unroll
    for (int i = 0; i < RM; ++i) {
        const int m = t.m0 + tm + 16 * i;
        if (m >= g.M) continue;
#pragma unroll
        for (int j = 0; j < RN; ++j) {
            const int nn = t.n0 + tn + 16 * j;
            if (nn < g.N) P[(int64_t)m * g.N + nn] = Op::finish(acc[i][j]);
        }
    }
}

// One-column groups: P[m] = sum_k A_k[m] R_k[0].  C3L_PAIR_SHAPE_COLUMN: 256
// rows, each thread one row over all anchors; C3L_PAIR_SHAPE_COLUMN_SPLIT: 32
// rows (the lanes), warp w takes anchors w, w + 8, ..., and the eight partial
// sums are added in warp order through shared memory.
template <class Op, bool kSplit>
__device__ __forceinline__ void pair_column(const c3l_pair_program& pp, const c3l_pair_tile& t,
                                            const c3l_pair_group& g, typename Op::Elem* __restrict__ ws,
                                            typename Op::S* smem) {
    using A = typename Op::A;
    const int tid = threadIdx.x;
    const int row = kSplit ? (tid & 31) : tid;
    const int m = t.m0 + row;
    const int kstep = kSplit ? kPairThreads / 32 : 1;
    A acc = Op::zero();
    if (m < g.M) {
        for (int64_t k = g.kbegin + (kSplit ? tid / 32 : 0); k < g.kend; k += kstep)
            Op::mac(acc, Op::stage(ws[pp.aoff[k] + m]), Op::stage(ws[pp.roff[k]]));
    }
    if constexpr (kSplit) {
        static_assert(sizeof(A) <= sizeof(typename Op::S), "partial sums reuse the staging buffer");
        A* part = reinterpret_cast<A*>(smem);
        part[tid] = acc;
        __syncthreads();
        if (tid >= 32) return;
#pragma unroll
        for (int w = 1; w < kPairThreads / 32; ++w) Op::add(acc, part[w * 32 + tid]);
    }
    if (m < g.M) ws[pp.base + g.p_off + m] = Op::finish(acc);
}

template <class Op>
__device__ __forceinline__ void pair_gemm_block(const c3l_pair_program& pp, const Batch<typename Op::Elem>& bt) {
    if (!bt.pdl_at_exit) c3l::pdl_launch_dependents();
    if (batch_stopped(bt)) return;
    __shared__ typename Op::S smem[kPairChunk * (kPairMaxEdge + 16)];
    const c3l_pair_tile t = pp.tiles[blockIdx.x];
    const c3l_pair_group g = pp.groups[t.group];
    c3l::pdl_wait();  // the tables above are constant; the workspace is not
    typename Op::Elem* __restrict__ ws = bt.ws[blockIdx.y];
    switch (t.shape) {
        case C3L_PAIR_SHAPE_32x128: pair_tile<Op, 2, 8>(pp, t, g, ws, smem); break;
        case C3L_PAIR_SHAPE_128x32: pair_tile<Op, 8, 2>(pp, t, g, ws, smem); break;
        case C3L_PAIR_SHAPE_16x256: pair_tile<Op, 1, 16>(pp, t, g, ws, smem); break;
        case C3L_PAIR_SHAPE_256x16: pair_tile<Op, 16, 1>(pp, t, g, ws, smem); break;
        case C3L_PAIR_SHAPE_COLUMN: pair_column<Op, false>(pp, t, g, ws, smem); break;
        case C3L_PAIR_SHAPE_COLUMN_SPLIT: pair_column<Op, true>(pp, t, g, ws, smem); break;
        default: pair_tile<Op, 4, 4>(pp, t, g, ws, smem); break;
    }
}

template <typename C>
__global__ void __launch_bounds__(kPairThreads) k_pair_gemm(c3l_pair_program pp, Batch<C> bt) {
    pair_gemm_block<PairPlain<C>>(pp, bt);
}

__global__ void __launch_bounds__(kPairThreads) k_pair_gemm_df(c3l_pair_program pp, Batch<double2> bt) {
    pair_gemm_block<PairDf>(pp, bt);
}

// FP64 workspaces run the double-float kernel unless `fp64_pipe` asks for the
// plain FP64 one (kept for parity checks of the double-float sums).
template <typename C>
c3l_status run_pairs(const c3l_pair_program& pp, const Batch<C>& bt, cudaStream_t s, bool fp64_pipe = false) {
    if (pp.ntiles <= 0) return C3L_OK;
    if (!pp.groups || !pp.aoff || !pp.roff || !pp.tiles || pp.base < 0) return C3L_ERR_ARGUMENT;
    const dim3 grid((unsigned)pp.ntiles, (unsigned)bt.nb);
    if constexpr (std::is_same<C, float2>::value) {
        if (pp.kernel == C3L_PAIR_TCGEN05 && pp.ntiles_tc > 0) {
            if (bt.nb != 1) return C3L_ERR_ARGUMENT;
            return c3l::pair_gemm_tc(pp, bt.ws[0], bt.pdl, s);
        }
    }
    if constexpr (std::is_same<C, double2>::value) {
        if (!fp64_pipe)
            return c3l::launch_pdl(k_pair_gemm_df, grid, dim3(kPairThreads), 0, s, 0, bt.pdl, pp, bt);
    }
    return c3l::launch_pdl(k_pair_gemm<C>, grid, dim3(kPairThreads), 0, s, 0, bt.pdl, pp, bt);
}

enum WedgeMode { kPadded = 0, kStatic = 1, kEom = 2, kSource = 3 };

// Output-stage constants; the per-entry input (src) and complex destination
// come from the batch.
struct Epilogue {
    const double2* lam;
    const int64_t* col;
    const int64_t* pair;
    const double2* scale;
    double* xout;
    double2 cscale;
    const double* m4;  // static outputs: optional 2x2 preconditioner block per element
    double iscale;     // static outputs: factor of the product part (the homotopy scale)
};

__device__ __forceinline__ double2 dmul(double2 a, double2 b) {
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}

// One block = one tile of up to kWE outputs of one output block; the block's
// instances are split over kWG thread groups (instance i goes to group
// i % kWG) and the groups' partial sums are added in shared memory.  Narrow
// tiles (small kWE) put more blocks on the GPU when a stage has few outputs.
template <int MODE, typename C, int kWE>
__global__ void __launch_bounds__(kThreads) k_wedge(c3l_wedge_stage st, int n, Batch<C> bt, Epilogue ep) {
    constexpr int kWG = kThreads / kWE;
    if (!bt.pdl_at_exit) c3l::pdl_launch_dependents();
    if (batch_stopped(bt)) return;
    C* __restrict__ ws = bt.ws[blockIdx.y];
    __shared__ c3l_instance sinst[kInstChunk];
    __shared__ C red[kWG][kWE];
    const c3l_tile tile = st.tiles[blockIdx.x];
    const c3l_block blk = st.blocks[tile.block];
    const int ex = threadIdx.x % kWE;
    const int gy = threadIdx.x / kWE;
    const bool active = ex < tile.count;
    const int64_t e = tile.start + ex;
    int64_t pw[6];
    powers(n, pw);
    int dig[C3L_MAX_DEGREE] = {0, 0, 0, 0, 0, 0};
    if (active) {
        if (MODE == kPadded) {
            uint32_t r = (uint32_t)e;  // below n^deg < 2^31 (checked when the plan is compiled)
            for (int c = blk.deg - 1; c >= 0; --c) {
                const uint32_t q = r / (uint32_t)n;
                dig[c] = (int)(r - q * (uint32_t)n);
                r = q;
            }
        } else {
            const int64_t packed = st.digits[e];
#pragma unroll
            for (int c = 0; c < C3L_MAX_DEGREE; ++c) dig[c] = (int)((packed >> (8 * c)) & 0xFF);
        }
    }
    // the epilogue's table entries of group 0's output, fetched before the
    // instance loop (and, being program tables, before the wait)
    const bool ep_thread = MODE != kPadded && active && gy == 0;
    int64_t mu = 0, ecol = 0, epair = 0;
    double2 elam = make_double2(0.0, 0.0), escale = make_double2(0.0, 0.0);
    double em4[4] = {0.0, 0.0, 0.0, 0.0};
    if (ep_thread) {
        mu = st.elements[e];
        if (MODE == kStatic || MODE == kEom) elam = ep.lam[e];
        if (MODE == kStatic) {
            escale = ep.scale[e];
            ecol = ep.col[e];
            epair = ep.pair[e];
            if (ep.m4) {
#pragma unroll
                for (int q = 0; q < 4; ++q) em4[q] = ep.m4[4 * e + q];
            }
        }
    }
    C acc = Cx<C>::make(0.0, 0.0);
    // cooperative copy of cnt instances from `base` (8-byte words); the first
    // chunk is staged before the wait (instances are program tables)
    auto stage = [&](int64_t base, int cnt) {
        const int64_t* src = reinterpret_cast<const int64_t*>(st.instances + base);
        int64_t* dst = reinterpret_cast<int64_t*>(sinst);
        static_assert(sizeof(c3l_instance) % 8 == 0, "instances are copied as 8-byte words");
        const int words = cnt * (int)(sizeof(c3l_instance) / 8);
        for (int w = threadIdx.x; w < words; w += blockDim.x) dst[w] = src[w];
    };
    {
        const int64_t left = blk.inst_end - blk.inst_begin;
        if (left > 0) stage(blk.inst_begin, left < kInstChunk ? (int)left : kInstChunk);
    }
    c3l::pdl_wait();
    double2 esrc = make_double2(0.0, 0.0);  // the operator's input at the output (issued before the loop)
    if ((MODE == kStatic || MODE == kEom) && ep_thread) esrc = bt.in[blockIdx.y][mu];
    for (int64_t base = blk.inst_begin; base < blk.inst_end; base += kInstChunk) {
        const int64_t left = blk.inst_end - base;
        const int cnt = left < kInstChunk ? (int)left : kInstChunk;
        if (base != blk.inst_begin) {
            __syncthreads();  // the previous chunk has been used
            stage(base, cnt);
        }
        __syncthreads();
        if (active) {
            for (int i = gy; i < cnt; i += kWG) {
                const c3l_instance& in = sinst[i];
                C v = Cx<C>::make(in.coef[0], in.coef[1]);
                for (int j = 0; j < in.nfac; ++j) {
                    const int d = in.fac_deg[j];
                    int64_t off = in.fac_off[j];
                    for (int q = 0; q < d; ++q) off += (int64_t)dig[in.axes[j][q]] * pw[d - 1 - q];
                    v = cmul(v, ws[off]);
                }
                acc = cadd(acc, v);
            }
        }
    }
    red[gy][ex] = acc;
    __syncthreads();
    if (!active || gy != 0) return;
#pragma unroll
    for (int g = 1; g < kWG; ++g) acc = cadd(acc, red[g][ex]);
    if (MODE == kPadded) {
        ws[blk.out_off + e] = acc;
    } else if (MODE == kStatic) {
        const double2 a0 = to_d2(acc);
        const double2 a = make_double2(ep.iscale * a0.x, ep.iscale * a0.y);
        const double2 lam = elam, src = esrc;
        const double2 s = make_double2(fma(lam.x, src.x, fma(-lam.y, src.y, a.x)), fma(lam.x, src.y, fma(lam.y, src.x, a.y)));
        const double2 r = make_double2(s.y, -s.x);  // -i * s
        const double2 v = dmul(r, escale);
        const int64_t c = ecol;
        if (ep.m4) {  // fused preconditioner: y = M [x_c, x_c+1] (pack(unpack(.)/diag))
            if (epair) {
                ep.xout[c] = fma(em4[0], v.x, em4[1] * r.y);
                ep.xout[c + 1] = fma(em4[2], v.x, em4[3] * r.y);
            } else {
                ep.xout[c] = em4[0] * v.x;
            }
        } else {
            ep.xout[c] = v.x;
            if (epair) ep.xout[c + 1] = r.y;
        }
    } else if (MODE == kEom) {
        const double2 a0 = to_d2(acc);
        const double2 a = make_double2(ep.iscale * a0.x, ep.iscale * a0.y);
        const double2 lam = elam, src = esrc;
        const double2 o =
            make_double2(fma(lam.x, src.x, fma(-lam.y, src.y, a.x)), fma(lam.x, src.y, fma(lam.y, src.x, a.y)));
        bt.out[blockIdx.y][mu] = o;
        float2* o32 = bt.out32[blockIdx.y];
        if (o32) o32[mu] = make_float2((float)o.x, (float)o.y);
    } else {
        bt.out[blockIdx.y][mu] = dmul(ep.cscale, to_d2(acc));
    }
}

template <typename C>
Batch<C> single(C* ws, const double2* in = nullptr, double2* out = nullptr) {
    Batch<C> bt{};
    bt.ws[0] = ws;
    bt.in[0] = in;
    bt.out[0] = out;
    bt.nb = 1;
    return bt;
}

template <int MODE, typename C>
c3l_status launch_wedge(const c3l_wedge_stage& st, int n, const Batch<C>& bt, const Epilogue& ep, cudaStream_t s) {
    const dim3 grid((unsigned)st.ntiles, (unsigned)bt.nb);
    switch (st.width) {
        case 8: return c3l::launch_pdl(k_wedge<MODE, C, 8>, grid, dim3(kThreads), 0, s, 0, bt.pdl, st, n, bt, ep);
        case 16: return c3l::launch_pdl(k_wedge<MODE, C, 16>, grid, dim3(kThreads), 0, s, 0, bt.pdl, st, n, bt, ep);
        case 32: return c3l::launch_pdl(k_wedge<MODE, C, 32>, grid, dim3(kThreads), 0, s, 0, bt.pdl, st, n, bt, ep);
        case 0:
        case 64: return c3l::launch_pdl(k_wedge<MODE, C, 64>, grid, dim3(kThreads), 0, s, 0, bt.pdl, st, n, bt, ep);
        default: return C3L_ERR_ARGUMENT;
    }
}

inline unsigned grid_for(int64_t count) {
    int64_t b = (count + kThreads - 1) / kThreads;
    if (b < 1) b = 1;
    if (b > 65535LL * 16) b = 65535LL * 16;
    return (unsigned)b;
}

// Cluster size for k_contract_cluster<C>: 16 CTAs where the device can
// schedule such a cluster (checked once per process), else the portable 8.
template <typename C>
int level_cluster_size() {
    static int size = 0;
    if (size) return size;
    int chosen = 8;
    const void* fn = (const void*)k_contract_cluster<C>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(kLevelClusterMax, 1, 1);
        cfg.blockDim = dim3(kThreads, 1, 1);
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = kLevelClusterMax;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int clusters = 0;
        if (cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) == cudaSuccess && clusters >= 1)
            chosen = kLevelClusterMax;
    }
    cudaGetLastError();  // a refused query leaves no error behind
    size = chosen;
    return size;
}

template <typename C>
c3l_status run_levels(const c3l_action* a, const Batch<C>& bt, cudaStream_t s) {
    // levels [tail, nlevels) each fit one round of the cluster: one cluster launch runs them
    const int cluster = level_cluster_size<C>();
    int tail = a->nlevels;
    while (tail > 0 && a->levels[tail - 1].ntiles <= cluster) --tail;
    if (a->nlevels - tail < 2) tail = a->nlevels;  // a single small level gains nothing
    const C* vectors = reinterpret_cast<const C*>(a->vectors);
    for (int l = 0; l < tail; ++l) {
        if (a->levels[l].ntiles <= 0) continue;
        const c3l_status r = c3l::launch_pdl(k_contract<C>, dim3((unsigned)a->levels[l].ntiles, (unsigned)bt.nb),
                                             dim3(kThreads), 0, s, 0, bt.pdl, a->levels[l], a->n, vectors, bt);
        if (r) return r;
    }
    if (tail < a->nlevels) {
        LevelPack pack{};
        for (int l = 0; l < a->nlevels; ++l) pack.lv[l] = a->levels[l];
        pack.first = tail;
        pack.count = a->nlevels - tail;
        const c3l_status r = c3l::launch_pdl(k_contract_cluster<C>, dim3(cluster, (unsigned)bt.nb, 1), dim3(kThreads),
                                             0, s, (unsigned)cluster, bt.pdl, pack, a->n, vectors, bt);
        if (r) return r;
    }
    return launch_status();
}

template <typename C>
c3l_status run_padded(const c3l_action* a, const Batch<C>& bt, cudaStream_t s) {
    Epilogue ep{};
    for (int p = 0; p < a->npadded; ++p) {
        if (a->padded[p].ntiles <= 0) continue;
        const c3l_status st = launch_wedge<kPadded, C>(a->padded[p], a->n, bt, ep, s);
        if (st) return st;
    }
    return C3L_OK;
}

template <typename C>
c3l_status scatter(const c3l_action* a, const Batch<C>& bt, cudaStream_t s) {
    if (a->scatter_count <= 0) return C3L_OK;
    return c3l::launch_pdl(k_scatter<C>, dim3(grid_for(a->scatter_count), (unsigned)bt.nb), dim3(kThreads), 0, s, 0,
                           bt.pdl, a->scatter_count, a->scatter_dst, a->scatter_pos, a->scatter_sign, bt);
}

bool valid_action(const c3l_action* a) {
    return a && a->ws && a->vectors && a->n > 0 && a->n <= 255 && a->nlevels >= 0 && a->nlevels <= C3L_MAX_LEVELS &&
           a->npadded >= 0 && a->npadded <= C3L_MAX_STAGES;
}

// The batch's input vectors through the scatter, the atom levels and the
// padded stages of a program.
template <typename C>
c3l_status action_prepare(const c3l_action* action, const Batch<C>& bt, cudaStream_t s) {
    c3l_status st = scatter<C>(action, bt, s);
    if (st) return st;
    if ((st = run_levels<C>(action, bt, s))) return st;
    return run_padded<C>(action, bt, s);
}

template <typename C>
c3l_status static_apply(const c3l_static_action* sa, const double* x, double* xout, void* stream) {
    if (!sa || !x || !xout || !valid_action(&sa->action) || !sa->canon || !sa->tilde_ia || !sa->tilde_ib ||
        !sa->tilde_ca || !sa->tilde_cb || !sa->lam || !sa->col || !sa->pair || !sa->scale || sa->num_amplitudes <= 0 ||
        !(sa->interaction_scale >= 0.0 && sa->interaction_scale <= 1.0))
        return C3L_ERR_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    const c3l_action* a = &sa->action;
    Batch<C> bt = single<C>(reinterpret_cast<C*>(a->ws), reinterpret_cast<const double2*>(sa->canon));
    bt.pdl = true;
    c3l_status st;
    if (a->scatter_count >= kSplitScatter) {
        // canonical vector, then the padded scatter from it (k_scatter waits for the unpack)
        st = c3l::launch_pdl(k_tilde_unpack, dim3(grid_for(sa->num_amplitudes)), dim3(kThreads), 0, s, 0, true,
                             sa->num_amplitudes, x, (const int64_t*)sa->tilde_ia, (const int64_t*)sa->tilde_ib,
                             reinterpret_cast<const double2*>(sa->tilde_ca),
                             reinterpret_cast<const double2*>(sa->tilde_cb), reinterpret_cast<double2*>(sa->canon));
        if (st) return st;
        if ((st = scatter<C>(a, bt, s))) return st;
    } else {
        const int64_t n = sa->num_amplitudes > a->scatter_count ? sa->num_amplitudes : a->scatter_count;
        st = c3l::launch_pdl(
            k_unpack_scatter<C>, dim3(grid_for(n)), dim3(kThreads), 0, s, 0, true, sa->num_amplitudes, x,
            (const int64_t*)sa->tilde_ia, (const int64_t*)sa->tilde_ib, reinterpret_cast<const double2*>(sa->tilde_ca),
            reinterpret_cast<const double2*>(sa->tilde_cb), reinterpret_cast<double2*>(sa->canon), a->scatter_count,
            (const int64_t*)a->scatter_dst, (const int64_t*)a->scatter_pos, (const double*)a->scatter_sign,
            reinterpret_cast<C*>(a->ws));
        if (st) return st;
    }
    if ((st = run_levels<C>(a, bt, s))) return st;
    if ((st = run_padded<C>(a, bt, s))) return st;
    if ((st = run_pairs<C>(a->pairs, bt, s))) return st;
    if (sa->action.out.ntiles <= 0) return C3L_OK;
    Epilogue ep{};
    ep.lam = reinterpret_cast<const double2*>(sa->lam);
    ep.col = sa->col;
    ep.pair = sa->pair;
    ep.scale = reinterpret_cast<const double2*>(sa->scale);
    ep.xout = xout;
    ep.m4 = sa->pc_m4;
    ep.iscale = sa->interaction_scale;
    return launch_wedge<kStatic, C>(sa->action.out, sa->action.n, bt, ep, s);
}

// Two actions run the same program when they differ only in the workspace.
bool same_program(const c3l_action& a, const c3l_action& b) {
    c3l_action x = a, y = b;
    x.ws = nullptr;
    y.ws = nullptr;
    return std::memcmp(&x, &y, sizeof(c3l_action)) == 0;
}

template <typename C>
c3l_status eom_sigma(const c3l_eom_action* ea, int nb, const c3l_complex* const* xin, c3l_complex* const* out,
                     c3l_complex32* const* out32, const int32_t* const* stop, cudaStream_t s, bool pdl = false,
                     bool skip_scatter = false) {
    if (!ea || nb < 1 || nb > C3L_MAX_BATCH || !xin || !out) return C3L_ERR_ARGUMENT;
    Batch<C> bt{};
    bt.nb = nb;
    bt.pdl = pdl;
    bt.pdl_at_exit = true;
    for (int b = 0; b < nb; ++b) {
        if (!xin[b] || !out[b] || !valid_action(&ea[b].action) || !ea[b].lam) return C3L_ERR_ARGUMENT;
        if (b > 0 && (!same_program(ea[b].action, ea[0].action) || ea[b].lam != ea[0].lam ||
                      ea[b].interaction_scale != ea[0].interaction_scale))
            return C3L_ERR_ARGUMENT;
        if (!(ea[b].interaction_scale >= 0.0 && ea[b].interaction_scale <= 1.0)) return C3L_ERR_ARGUMENT;
        bt.ws[b] = reinterpret_cast<C*>(ea[b].action.ws);
        bt.in[b] = reinterpret_cast<const double2*>(xin[b]);
        bt.out[b] = reinterpret_cast<double2*>(out[b]);
        bt.stop[b] = stop ? stop[b] : nullptr;
        bt.out32[b] = out32 ? reinterpret_cast<float2*>(out32[b]) : nullptr;
    }
    c3l_status st = skip_scatter ? C3L_OK : scatter<C>(&ea[0].action, bt, s);
    if (st) return st;
    if ((st = run_levels<C>(&ea[0].action, bt, s))) return st;
    if ((st = run_padded<C>(&ea[0].action, bt, s))) return st;
    if ((st = run_pairs<C>(ea[0].action.pairs, bt, s))) return st;
    if (ea[0].action.out.ntiles <= 0) return C3L_OK;
    Epilogue ep{};
    ep.lam = reinterpret_cast<const double2*>(ea[0].lam);
    ep.iscale = ea[0].interaction_scale;
    return launch_wedge<kEom, C>(ea[0].action.out, ea[0].action.n, bt, ep, s);
}

}  // namespace

namespace c3l {

c3l_status eom_sigma_batch(const c3l_eom_action* actions, int nb, const c3l_complex* const* xin,
                           c3l_complex* const* out, c3l_complex32* const* out32, const int32_t* const* stop,
                           cudaStream_t s, bool skip_scatter) {
    return eom_sigma<double2>(actions, nb, xin, out, out32, stop, s, true, skip_scatter);
}

bool same_sigma_program(const c3l_eom_action& a, const c3l_eom_action& b) {
    return same_program(a.action, b.action) && a.lam == b.lam && a.interaction_scale == b.interaction_scale;
}

}  // namespace c3l

extern "C" {

c3l_status c3l_tilde_unpack(int64_t dim, const double* x, const int64_t* ia, const int64_t* ib, const c3l_complex* ca,
                            const c3l_complex* cb, c3l_complex* t, void* stream) {
    if (dim < 0 || (dim > 0 && (!x || !ia || !ib || !ca || !cb || !t))) return C3L_ERR_ARGUMENT;
    if (dim == 0) return C3L_OK;
    k_tilde_unpack<<<grid_for(dim), kThreads, 0, as_stream(stream)>>>(dim, x, ia, ib, reinterpret_cast<const double2*>(ca),
                                                                     reinterpret_cast<const double2*>(cb),
                                                                     reinterpret_cast<double2*>(t));
    return launch_status();
}

c3l_status c3l_scatter_padded(int64_t count, const int64_t* dst, const int64_t* pos, const double* sign,
                              const c3l_complex* vec, c3l_complex* ws, void* stream) {
    if (count < 0 || (count > 0 && (!dst || !pos || !sign || !vec || !ws))) return C3L_ERR_ARGUMENT;
    if (count == 0) return C3L_OK;
    k_scatter<double2><<<grid_for(count), kThreads, 0, as_stream(stream)>>>(
        count, dst, pos, sign, single<double2>(reinterpret_cast<double2*>(ws), reinterpret_cast<const double2*>(vec)));
    return launch_status();
}

c3l_status c3l_downcast(int64_t count, const c3l_complex* src, c3l_complex32* dst, void* stream) {
    if (count < 0 || (count > 0 && (!src || !dst))) return C3L_ERR_ARGUMENT;
    if (count == 0) return C3L_OK;
    k_downcast<<<grid_for(count), kThreads, 0, as_stream(stream)>>>(count, reinterpret_cast<const double2*>(src),
                                                                   reinterpret_cast<float2*>(dst));
    return launch_status();
}

c3l_status c3l_contract(const c3l_contract_level* level, int32_t n, const c3l_complex* vectors, c3l_complex* ws,
                        void* stream) {
    if (!level || !vectors || !ws || n <= 0 || n > 255) return C3L_ERR_ARGUMENT;
    if (level->ntiles <= 0) return C3L_OK;
    k_contract<double2><<<(unsigned)level->ntiles, kThreads, 0, as_stream(stream)>>>(
        *level, n, reinterpret_cast<const double2*>(vectors), single<double2>(reinterpret_cast<double2*>(ws)));
    return launch_status();
}

c3l_status c3l_wedge_padded(const c3l_wedge_stage* stage, int32_t n, c3l_complex* ws, void* stream) {
    if (!stage || !ws || n <= 0 || n > 255) return C3L_ERR_ARGUMENT;
    if (stage->ntiles <= 0) return C3L_OK;
    Epilogue ep{};
    return launch_wedge<kPadded, double2>(*stage, n, single<double2>(reinterpret_cast<double2*>(ws)), ep,
                                          as_stream(stream));
}

c3l_status c3l_wedge_static_out(const c3l_wedge_stage* stage, int32_t n, const c3l_complex* ws, const c3l_complex* lam,
                                const c3l_complex* src, const int64_t* col, const int64_t* pair, const c3l_complex* scale,
                                double* xout, void* stream) {
    if (!stage || !ws || !lam || !src || !col || !pair || !scale || !xout || n <= 0 || n > 255) return C3L_ERR_ARGUMENT;
    if (stage->ntiles <= 0) return C3L_OK;
    Epilogue ep{};
    ep.lam = reinterpret_cast<const double2*>(lam);
    ep.col = col;
    ep.pair = pair;
    ep.scale = reinterpret_cast<const double2*>(scale);
    ep.xout = xout;
    ep.iscale = 1.0;
    return launch_wedge<kStatic, double2>(
        *stage, n,
        single<double2>(const_cast<double2*>(reinterpret_cast<const double2*>(ws)), reinterpret_cast<const double2*>(src)),
        ep, as_stream(stream));
}

c3l_status c3l_wedge_static_out_f32(const c3l_wedge_stage* stage, int32_t n, const c3l_complex32* ws,
                                    const c3l_complex* lam, const c3l_complex* src, const int64_t* col,
                                    const int64_t* pair, const c3l_complex* scale, double* xout, void* stream) {
    if (!stage || !ws || !lam || !src || !col || !pair || !scale || !xout || n <= 0 || n > 255) return C3L_ERR_ARGUMENT;
    if (stage->ntiles <= 0) return C3L_OK;
    Epilogue ep{};
    ep.lam = reinterpret_cast<const double2*>(lam);
    ep.col = col;
    ep.pair = pair;
    ep.scale = reinterpret_cast<const double2*>(scale);
    ep.xout = xout;
    ep.iscale = 1.0;
    return launch_wedge<kStatic, float2>(
        *stage, n,
        single<float2>(const_cast<float2*>(reinterpret_cast<const float2*>(ws)), reinterpret_cast<const double2*>(src)),
        ep, as_stream(stream));
}

c3l_status c3l_wedge_eom_out(const c3l_wedge_stage* stage, int32_t n, const c3l_complex* ws, const c3l_complex* lam,
                             const c3l_complex* xin, c3l_complex* out, void* stream) {
    if (!stage || !ws || !lam || !xin || !out || n <= 0 || n > 255) return C3L_ERR_ARGUMENT;
    if (stage->ntiles <= 0) return C3L_OK;
    Epilogue ep{};
    ep.lam = reinterpret_cast<const double2*>(lam);
    ep.iscale = 1.0;
    return launch_wedge<kEom, double2>(*stage, n,
                                       single<double2>(const_cast<double2*>(reinterpret_cast<const double2*>(ws)),
                                                       reinterpret_cast<const double2*>(xin),
                                                       reinterpret_cast<double2*>(out)),
                                       ep, as_stream(stream));
}

c3l_status c3l_pair_gemm(const c3l_pair_program* program, c3l_complex* ws, void* stream) {
    if (!program || !ws) return C3L_ERR_ARGUMENT;
    return run_pairs<double2>(*program, single<double2>(reinterpret_cast<double2*>(ws)), as_stream(stream), true);
}

c3l_status c3l_pair_gemm_df(const c3l_pair_program* program, c3l_complex* ws, void* stream) {
    if (!program || !ws) return C3L_ERR_ARGUMENT;
    return run_pairs<double2>(*program, single<double2>(reinterpret_cast<double2*>(ws)), as_stream(stream));
}

c3l_status c3l_pair_gemm_tc(const c3l_pair_program* program, c3l_complex32* ws, void* stream) {
    if (!program || !ws) return C3L_ERR_ARGUMENT;
    return c3l::pair_gemm_tc(*program, reinterpret_cast<float2*>(ws), false, as_stream(stream));
}

c3l_status c3l_pair_gemm_f32(const c3l_pair_program* program, c3l_complex32* ws, void* stream) {
    if (!program || !ws) return C3L_ERR_ARGUMENT;
    return run_pairs<float2>(*program, single<float2>(reinterpret_cast<float2*>(ws)), as_stream(stream));
}

c3l_status c3l_wedge_source_out(const c3l_wedge_stage* stage, int32_t n, const c3l_complex* ws, c3l_complex scale,
                                c3l_complex* out, void* stream) {
    if (!stage || !ws || !out || n <= 0 || n > 255) return C3L_ERR_ARGUMENT;
    if (stage->ntiles <= 0) return C3L_OK;
    Epilogue ep{};
    ep.cscale = make_double2(scale.re, scale.im);
    return launch_wedge<kSource, double2>(
        *stage, n,
        single<double2>(const_cast<double2*>(reinterpret_cast<const double2*>(ws)), nullptr,
                        reinterpret_cast<double2*>(out)),
        ep, as_stream(stream));
}

c3l_status c3l_action_prepare(const c3l_action* action, const c3l_complex* t, void* stream) {
    if (!valid_action(action) || !t) return C3L_ERR_ARGUMENT;
    return action_prepare<double2>(
        action, single<double2>(reinterpret_cast<double2*>(action->ws), reinterpret_cast<const double2*>(t)),
        as_stream(stream));
}

c3l_status c3l_action_prepare_f32(const c3l_action* action, const c3l_complex* t, void* stream) {
    if (!valid_action(action) || !t) return C3L_ERR_ARGUMENT;
    return action_prepare<float2>(
        action, single<float2>(reinterpret_cast<float2*>(action->ws), reinterpret_cast<const double2*>(t)),
        as_stream(stream));
}

c3l_status c3l_static_apply(const c3l_static_action* sa, const double* x, double* xout, void* stream) {
    return static_apply<double2>(sa, x, xout, stream);
}

c3l_status c3l_static_apply_f32(const c3l_static_action* sa, const double* x, double* xout, void* stream) {
    return static_apply<float2>(sa, x, xout, stream);
}

c3l_status c3l_eom_sigma(const c3l_eom_action* ea, const c3l_complex* xin, c3l_complex* out, void* stream) {
    return eom_sigma<double2>(ea, 1, &xin, &out, nullptr, nullptr, as_stream(stream));
}

c3l_status c3l_eom_sigma_f32(const c3l_eom_action* ea, const c3l_complex* xin, c3l_complex* out, void* stream) {
    return eom_sigma<float2>(ea, 1, &xin, &out, nullptr, nullptr, as_stream(stream));
}

c3l_status c3l_eom_sigma_batch(const c3l_eom_action* actions, int32_t nb, const c3l_complex* const* xin,
                               c3l_complex* const* out, void* stream) {
    return eom_sigma<double2>(actions, nb, xin, out, nullptr, nullptr, as_stream(stream));
}

const char* c3l_version(void) { return "c3l_gb300 0.2.0 (sm_103a, fp64/fp32 complex programs)"; }

}  // extern "C"

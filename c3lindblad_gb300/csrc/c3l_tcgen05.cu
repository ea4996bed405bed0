// Pair GEMMs of the FP32 (inner-solve) JVP on the fifth-generation tensor
// cores (tcgen05, sm_103a), split-TF32.
//
// A pair group computes P[i][j] = sum_k A_k[i] R_k[j] over its anchors k, with
// complex operand rows gathered from the workspace (c3l_pair_program).  A
// thread block owns a 128 x 64 tile of P.  Per chunk of 8 anchors its threads
// load the operand rows (coalesced along i and j), split every real
// component x into TF32 parts hi = tf32(x), lo = x - hi, and store them in
// shared memory in the K-major, no-swizzle core-matrix layout the MMA reads
// (8 rows x 16 bytes per core matrix).  One thread then issues the chunk's
// tcgen05.mma.kind::tf32 (M = 128, N = 64, K = 8; twelve per 8 anchors) into
// two FP32 accumulators in tensor memory:
//
//   D_re += Ar Br - Ai Bi,   D_im += Ar Bi + Ai Br,
//   each real product as hi hi + hi lo + lo hi (the lo lo term, 2^-22
//   relative, is dropped), -Ai Bi by the MMA's negate-A bit,
//
// and commits them to the chunk's stage barrier, while the threads stage the
// next chunk into the other buffer.  The error per product is about 2^-21
// relative, the accuracy of the FP32 operands themselves.  The epilogue reads
// the accumulators with tcgen05.ld (warp w reads tensor-memory lanes
// 32 (w % 4) .. + 31, i.e. tile rows; the two warpgroups split the columns)
// and writes P.
//
// Every wait on a barrier is bounded; a block whose wait runs out writes 1
// to the program's status word (when given), skips the epilogue, frees its
// tensor memory and returns.
#include <cuda_runtime.h>
#include <stdint.h>

#include "c3l_gb300.h"
#include "c3l_internal.h"
#include "c3l_pdl.h"

namespace {

constexpr int kTcM = 128;        // tile rows = tensor-memory lanes
constexpr int kTcN = 64;         // tile columns per accumulator
constexpr int kTcK = 8;          // anchors per MMA (32 bytes of TF32)
constexpr int kTcChunk = 16;     // anchors per stage: two MMA K-steps
constexpr int kTcThreads = 256;  // two warpgroups: both stage, warps w and w + 4 share lanes 32 (w % 4)
constexpr int kTcStages = 2;
constexpr int kRowBytes = kTcChunk * 4;               // one tile row's TF32 entries of a stage
constexpr int kATile = kTcM * kRowBytes;              // 8 KB: one TF32 part of the anchor tile
constexpr int kBTile = kTcN * kRowBytes;              // 4 KB: one TF32 part of the rest tile
constexpr int kStageBytes = 4 * kATile + 4 * kBTile;  // 48 KB
constexpr int kTmemCols = 2 * kTcN;                   // D_re in columns [0, 64), D_im in [64, 128)
constexpr int kAlign = 1024;
constexpr int kSmemBytes = kAlign + kTcStages * kStageBytes + 64;
constexpr int kEpiStride = kTcN + 1;  // float2 per row of the epilogue's staging tile
static_assert(kTcM * kEpiStride * 8 <= kTcStages * kStageBytes, "the epilogue tile reuses the stage buffers");
constexpr uint32_t kWaitLimit = 1u << 22;  // try_wait rounds before a block gives up
constexpr int kAPerThread = kTcM * kTcChunk / kTcThreads;  // anchor entries staged per thread
constexpr int kBPerThread = kTcN * kTcChunk / kTcThreads;  // rest entries staged per thread
static_assert(kAPerThread == 8 && kBPerThread == 4, "staging: 8 anchors of a row, 4 of a column per thread");

// Byte offset of (row r, k) in a K-major no-swizzle operand tile of kTcChunk
// anchors: core matrices of 8 rows x 16 bytes (4 TF32), the next 4 k at +128
// bytes (the descriptor's leading-dimension offset), the next 8 rows at
// +8 * kRowBytes (its stride offset).  MMA K-step j starts at +256 j.
__device__ __forceinline__ uint32_t kmajor_off(int r, int k) {
    return (uint32_t)((r >> 3) * (8 * kRowBytes) + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

// Shared-memory matrix descriptor: start address, leading-dimension byte
// offset 128, stride byte offset 8 * kRowBytes (both in 16-byte units),
// descriptor version 1 (bits 46-47), base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(128 >> 4) << 16) |
           ((uint64_t)((8 * kRowBytes) >> 4) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor of tcgen05.mma.kind::tf32: D F32 (bits 4-5 = 1), A and
// B TF32 (bits 7-9, 10-12 = 2), optional negate A (bit 13), both K-major
// (bits 15-16 = 0), N >> 3 (bits 17-22), M >> 4 (bits 24-28).
__host__ __device__ constexpr uint32_t idesc_tf32(bool neg_a) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((neg_a ? 1u : 0u) << 13) | ((uint32_t)(kTcN >> 3) << 17) |
           ((uint32_t)(kTcM >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (uint32_t i = 0; i < kWaitLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ uint32_t tf32_hi(float x) {
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
    return h;
}

// hi and lo TF32 parts of x: hi = tf32(x), lo = tf32(x - hi) (x - hi is exact
// in FP32; rounding it here keeps the tensor core's own truncation of the
// operand from biasing long sums)
__device__ __forceinline__ void tf32_split(float x, float& hi, float& lo) {
    hi = __uint_as_float(tf32_hi(x));
    lo = __uint_as_float(tf32_hi(__fsub_rn(x, hi)));
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, float a, float b, float c, float d) {
    asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(a), "f"(b), "f"(c), "f"(d) : "memory");
}

// 32 lanes x 16 columns of 32 bits: this thread's lane, columns [col, col + 16)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__global__ void __launch_bounds__(kTcThreads) k_pair_gemm_tc(c3l_pair_program pp, float2* __restrict__ ws, int pdl) {
    extern __shared__ uint8_t dsmem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t raw = (uint32_t)__cvta_generic_to_shared(dsmem);
    const uint32_t sbase = (raw + kAlign - 1) & ~(uint32_t)(kAlign - 1);
    const uint32_t mbar0 = sbase + kTcStages * kStageBytes;  // two 8-byte barriers
    const uint32_t slot = mbar0 + 16;                        // tensor-memory address
    const c3l_pair_tile t = pp.tiles_tc[blockIdx.x];
    const c3l_pair_group g = pp.groups[t.group];
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < kTcStages; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar0 + 8 * s) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    uint32_t tmem;
    asm volatile("ld.shared.b32 %0, [%1];" : "=r"(tmem) : "r"(slot) : "memory");
    c3l::pdl_wait();

    const int64_t nk = g.kend - g.kbegin;
    const int nchunks = (int)((nk + kTcChunk - 1) / kTcChunk);
    const int arow = tid & (kTcM - 1), ak0 = (tid >> 7) * kAPerThread;  // anchor tile: row, first anchor
    const bool a_ok = t.m0 + arow < g.M;
    const int bcol = tid & (kTcN - 1), bk0 = (tid >> 6) * kBPerThread;  // rest tile: column, first anchor
    const bool b_ok = t.n0 + bcol < g.N;
    // the operand rows of two chunks are in flight: chunk c + 2 is loaded into
    // the registers chunk c has just been staged from
    float2 av0[kAPerThread], bv0[kBPerThread], av1[kAPerThread], bv1[kBPerThread];
    auto load = [&](int c, float2 (&av)[kAPerThread], float2 (&bv)[kBPerThread]) {
        const int64_t k0 = g.kbegin + (int64_t)c * kTcChunk;
#pragma unroll
        for (int q = 0; q < kAPerThread; ++q) {
            const int64_t k = k0 + ak0 + q;
            av[q] = (a_ok && k < g.kend) ? ws[pp.aoff[k] + t.m0 + arow] : make_float2(0.0f, 0.0f);
        }
#pragma unroll
        for (int q = 0; q < kBPerThread; ++q) {
            const int64_t k = k0 + bk0 + q;
            bv[q] = (b_ok && k < g.kend) ? ws[pp.roff[k] + t.n0 + bcol] : make_float2(0.0f, 0.0f);
        }
    };
    bool ok = true;
    // stage chunk c from (av, bv), issue its MMAs, then load chunk c + 2 into (av, bv)
    auto step = [&](int c, float2 (&av)[kAPerThread], float2 (&bv)[kBPerThread]) {
        const int s = c & 1;
        // the stage's previous MMAs (chunk c - 2) must be done before it is rewritten
        if (c >= kTcStages) ok = mbar_wait(mbar0 + 8 * s, (uint32_t)(((c - kTcStages) >> 1) & 1));
        if (!__syncthreads_and(ok)) {
            ok = false;
            return;
        }
        const uint32_t st = sbase + s * kStageBytes;
        // anchor tile: this thread's row, 8 of the chunk's anchors, 4 per 16-byte store
#pragma unroll
        for (int q4 = 0; q4 < kAPerThread / 4; ++q4) {
            float h[4], l[4], hi2[4], li[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                tf32_split(av[4 * q4 + q].x, h[q], l[q]);
                tf32_split(av[4 * q4 + q].y, hi2[q], li[q]);
            }
            const uint32_t off = kmajor_off(arow, ak0 + 4 * q4);
            st_shared_v4(st + 0 * kATile + off, h[0], h[1], h[2], h[3]);
            st_shared_v4(st + 1 * kATile + off, l[0], l[1], l[2], l[3]);
            st_shared_v4(st + 2 * kATile + off, hi2[0], hi2[1], hi2[2], hi2[3]);
            st_shared_v4(st + 3 * kATile + off, li[0], li[1], li[2], li[3]);
        }
        // rest tile: this thread's column, 4 of the chunk's anchors
        const uint32_t bt = st + 4 * kATile;
#pragma unroll
        for (int q4 = 0; q4 < kBPerThread / 4; ++q4) {
            float h[4], l[4], hi2[4], li[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                tf32_split(bv[4 * q4 + q].x, h[q], l[q]);
                tf32_split(bv[4 * q4 + q].y, hi2[q], li[q]);
            }
            const uint32_t off = kmajor_off(bcol, bk0 + 4 * q4);
            st_shared_v4(bt + 0 * kBTile + off, h[0], h[1], h[2], h[3]);
            st_shared_v4(bt + 1 * kBTile + off, l[0], l[1], l[2], l[3]);
            st_shared_v4(bt + 2 * kBTile + off, hi2[0], hi2[1], hi2[2], hi2[3]);
            st_shared_v4(bt + 3 * kBTile + off, li[0], li[1], li[2], li[3]);
        }
        if (c + 2 < nchunks) load(c + 2, av, bv);  // in flight while this and the next chunk run
        // the generic-proxy stores become visible to the tensor cores' reads
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t dre = tmem, dim = tmem + kTcN;
            const uint32_t pos = idesc_tf32(false), neg = idesc_tf32(true);
#pragma unroll
            for (int j = 0; j < kTcChunk / kTcK; ++j) {
                const uint32_t kb = 256u * j;  // MMA K-step j: 8 anchors = two core-matrix columns
                const uint64_t arh = smem_desc(st + kb), arl = smem_desc(st + kATile + kb),
                               aih = smem_desc(st + 2 * kATile + kb), ail = smem_desc(st + 3 * kATile + kb);
                const uint64_t brh = smem_desc(bt + kb), brl = smem_desc(bt + kBTile + kb),
                               bih = smem_desc(bt + 2 * kBTile + kb), bil = smem_desc(bt + 3 * kBTile + kb);
                const uint32_t first = (c > 0 || j > 0) ? 1u : 0u;
                mma_tf32(dre, arh, brh, pos, first);
                mma_tf32(dre, arh, brl, pos, 1u);
                mma_tf32(dre, arl, brh, pos, 1u);
                mma_tf32(dre, aih, bih, neg, 1u);
                mma_tf32(dre, aih, bil, neg, 1u);
                mma_tf32(dre, ail, bih, neg, 1u);
                mma_tf32(dim, arh, bih, pos, first);
                mma_tf32(dim, arh, bil, pos, 1u);
                mma_tf32(dim, arl, bih, pos, 1u);
                mma_tf32(dim, aih, brh, pos, 1u);
                mma_tf32(dim, aih, brl, pos, 1u);
                mma_tf32(dim, ail, brh, pos, 1u);
            }
            mma_commit(mbar0 + 8 * s);
        }
    };
    if (nchunks > 0) load(0, av0, bv0);
    if (nchunks > 1) load(1, av1, bv1);
    for (int c = 0; c < nchunks && ok; c += 2) {
        step(c, av0, bv0);
        if (ok && c + 1 < nchunks) step(c + 1, av1, bv1);
    }
    // the last chunk's commit covers every MMA issued before it
    if (ok && nchunks > 0) ok = mbar_wait(mbar0 + 8 * ((nchunks - 1) & 1), (uint32_t)(((nchunks - 1) >> 1) & 1));
    // the dependent kernel (the output gather) may start its blocks only now:
    // blocks of it waiting on the SMs earlier would hold shared memory and
    // warps that this kernel's second resident block needs
    if (pdl) c3l::pdl_launch_dependents();
    ok = __syncthreads_and(ok);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok && nchunks > 0) {
        // every MMA has completed, so the stage buffers are free: the tile goes
        // through shared memory (rows of kEpiStride float2, two-way bank
        // conflicts at most) so that each warp then writes whole P rows
        // (coalesced) instead of one entry of 32 rows per store.
        // Warp w reads tensor-memory lanes 32 (w % 4) (tile rows); warps 0-3
        // take columns [0, 32) of both accumulators, warps 4-7 columns [32, 64).
        float2* stile = reinterpret_cast<float2*>(dsmem + (sbase - raw));
        const int row = (warp & 3) * 32 + lane;
        const int cbase = (warp >> 2) * (kTcN / 2);
        const uint32_t lanes = (uint32_t)((warp & 3) * 32) << 16;
#pragma unroll 1
        for (int c0 = cbase; c0 < cbase + kTcN / 2; c0 += 16) {
            float re[16], im[16];
            tmem_ld16(tmem + lanes + c0, re);
            tmem_ld16(tmem + lanes + kTcN + c0, im);
#pragma unroll
            for (int j = 0; j < 16; ++j) stile[row * kEpiStride + c0 + j] = make_float2(re[j], im[j]);
        }
        __syncthreads();
        float2* __restrict__ P = ws + pp.base + g.p_off;
#pragma unroll 1
        for (int r = warp * (kTcM / 8); r < (warp + 1) * (kTcM / 8); ++r) {
            const int m = t.m0 + r;
            if (m >= g.M) break;
#pragma unroll
            for (int h = 0; h < kTcN / 32; ++h) {
                const int col = lane + 32 * h;
                if (t.n0 + col < g.N) P[(int64_t)m * g.N + t.n0 + col] = stile[r * kEpiStride + col];
            }
        }
    } else if (!ok && tid == 0 && pp.status) {
        atomicExch(pp.status, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

}  // namespace

namespace c3l {

c3l_status pair_gemm_tc(const c3l_pair_program& pp, float2* ws, bool pdl, cudaStream_t s) {
    if (pp.ntiles_tc <= 0) return C3L_OK;
    if (!pp.groups || !pp.aoff || !pp.roff || !pp.tiles_tc || pp.base < 0 || !ws) return C3L_ERR_ARGUMENT;
    static bool configured = false;
    if (!configured) {
        if (cudaFuncSetAttribute(k_pair_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes) !=
            cudaSuccess)
            return C3L_ERR_LAUNCH;
        configured = true;
    }
    return launch_pdl(k_pair_gemm_tc, dim3((unsigned)pp.ntiles_tc), dim3(kTcThreads), (size_t)kSmemBytes, s, 0, pdl,
                      pp, ws, pdl ? 1 : 0);
}

}  // namespace c3l

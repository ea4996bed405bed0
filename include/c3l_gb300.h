/*
 * c3l_gb300.h -- C ABI of the GB300-native coupled-cluster hot path.
 *
 * All pointers are device pointers unless stated otherwise; every entry point
 * enqueues work on the given CUDA stream and returns a c3l_status (0 = ok).
 * No entry point synchronizes the stream or allocates device memory; callers
 * own every buffer (the Python host layer allocates them with PyTorch).
 *
 * Complex numbers are interleaved (re, im) doubles (cuDoubleComplex layout).
 *
 * The reference (haoen2021/C3Lindblad, package c3l) is pure Python and has
 * no C ABI.  Each entry point below replaces one Python-level operation of
 * the reference; the citation names the file:line it replaces.
 */
#ifndef C3L_GB300_H
#define C3L_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int c3l_status;
enum {
    C3L_OK = 0,
    C3L_ERR_ARGUMENT = 1,   /* null pointer, bad size or table entry */
    C3L_ERR_LAUNCH = 2,     /* a kernel launch failed (cudaGetLastError) */
    C3L_ERR_CAPACITY = 3    /* a size exceeds a stated maximum */
};

typedef struct { double re, im; } c3l_complex;
typedef struct { float re, im; } c3l_complex32;

/* ---------------------------------------------------------- program tables
 * Built by c3lindblad_gb300/compiler.py (NumPy structured arrays with the
 * same layout).  Offsets index a complex workspace ("ws").
 */
#define C3L_MAX_SOURCES 4
#define C3L_MAX_FACTORS 6
/* largest block degree: 4 for the static amplitudes and S13, 5 with the
 * rank-five response shell (S135); index digits are one byte each */
#define C3L_MAX_DEGREE 6

/* One padded destination block of an atom: dst = const + sum_j sign_j *
 * sum_m vec_j[m] * src_j[... m at axis_j ...] (interior product,
 * src/c3l/cc/component_tensor.py:226-246). */
typedef struct {
    int64_t dst_off;
    int32_t deg;
    int32_t nsrc;
    int64_t const_off;                 /* -1: no creator constant          */
    int64_t src_off[C3L_MAX_SOURCES];
    int64_t vec_off[C3L_MAX_SOURCES];  /* into the factor-vector table     */
    int32_t axis[C3L_MAX_SOURCES];
    double sign[C3L_MAX_SOURCES];
} c3l_contract_task;

/* One shuffle-signed product of padded block entries (one wedge term). */
typedef struct {
    double coef[2];
    int32_t nfac;
    int32_t pad;
    int64_t fac_off[C3L_MAX_FACTORS];
    int32_t fac_deg[C3L_MAX_FACTORS];
    int8_t axes[C3L_MAX_FACTORS][C3L_MAX_DEGREE];
} c3l_instance;

typedef struct {
    int64_t inst_begin;
    int64_t inst_end;
    int64_t out_off;   /* padded stages: workspace offset of the block   */
    int32_t deg;
    int32_t pad;
} c3l_block;

/* A thread-block work unit: consecutive outputs of one block/task (<= 256 for
 * contraction tasks, <= the stage's width for wedge stages). */
typedef struct {
    int32_t block;
    int32_t count;
    int64_t start;
} c3l_tile;

typedef struct {
    const c3l_contract_task* tasks;
    const c3l_tile* tiles;
    int64_t ntiles;
} c3l_contract_level;

typedef struct {
    const c3l_block* blocks;
    const c3l_instance* instances;
    const c3l_tile* tiles;
    int64_t ntiles;
    const int64_t* elements;  /* canonical stages: output vector positions */
    const int64_t* digits;    /* canonical stages: packed index digits      */
    int32_t width;            /* outputs per tile: 8, 16, 32 or 64 (0: 64)  */
    int32_t pad;
} c3l_wedge_stage;

/* Pair GEMMs of an output stage (the anchor ^ rest sums of
 * src/c3l/cc/component_tensor.py:869-898 regrouped by anchor block): group g
 * computes P_g[i][j] = sum_{k in [kbegin, kend)} ws[aoff[k] + i] ws[roff[k] + j]
 * for i < M, j < N into ws[pair_base + p_off + i N + j], pair_base being the
 * first entry after the workspace proper.  The output stage then reads one
 * signed entry of P per shuffle. */
typedef struct {
    int64_t p_off;
    int64_t kbegin;
    int64_t kend;
    int32_t M;
    int32_t N;
} c3l_pair_group;

/* One thread block: the entries of group `group` starting at (m0, n0).  In
 * `tiles` (CUDA-core kernels) `shape` selects the tile: C3L_PAIR_SHAPE_64x64 ..
 * C3L_PAIR_SHAPE_256x16 are rows x columns (16 x 16 threads, each a
 * (rows / 16) x (columns / 16) block of entries); the two column shapes are
 * for groups of one column (N = 1): 256 rows, one per thread, or 32 rows
 * whose anchors the block's 8 warps split.  In `tiles_tc` shape is 0
 * (128 x 64). */
#define C3L_PAIR_SHAPE_64x64 0
#define C3L_PAIR_SHAPE_32x128 1
#define C3L_PAIR_SHAPE_128x32 2
#define C3L_PAIR_SHAPE_16x256 3
#define C3L_PAIR_SHAPE_256x16 4
#define C3L_PAIR_SHAPE_COLUMN 5
#define C3L_PAIR_SHAPE_COLUMN_SPLIT 6
typedef struct {
    int32_t group;
    int32_t m0;
    int32_t n0;
    int32_t shape;
} c3l_pair_tile;

/* kernel: C3L_PAIR_SIMT runs the CUDA-core kernels over `tiles`;
 * C3L_PAIR_TCGEN05 runs FP32 workspaces on the tensor cores over `tiles_tc`
 * (128 x 64, split-TF32, c3l_pair_gemm_tc); status (optional) receives 1 if
 * a tensor-core block gave up waiting for its MMAs. */
#define C3L_PAIR_SIMT 0
#define C3L_PAIR_TCGEN05 1
typedef struct {
    const c3l_pair_group* groups;
    const int64_t* aoff;
    const int64_t* roff;
    const c3l_pair_tile* tiles;
    int64_t ntiles;
    int64_t base;             /* pair_base: P entries are ws[base + p_off + ...] */
    const c3l_pair_tile* tiles_tc;
    int64_t ntiles_tc;
    int32_t* status;
    int32_t kernel;
    int32_t pad;
} c3l_pair_program;

/* ------------------------------------------------------------ primitives */

/* t[mu] = ca[mu] x[ia[mu]] + cb[mu] x[ib[mu]]  (TildeMap.unpack,
 * src/c3l/cc/symmetry.py:67-85). */
c3l_status c3l_tilde_unpack(int64_t dim, const double* x, const int64_t* ia, const int64_t* ib,
                            const c3l_complex* ca, const c3l_complex* cb, c3l_complex* t,
                            void* stream);

/* ws[dst[e]] = sign[e] * vec[pos[e]]  (ComponentCoordinates.unpack,
 * src/c3l/cc/component_tensor.py:302-325). */
c3l_status c3l_scatter_padded(int64_t count, const int64_t* dst, const int64_t* pos, const double* sign,
                              const c3l_complex* vec, c3l_complex* ws, void* stream);

/* One level of atom construction (interior products of amplitudes/shifts,
 * src/c3l/cc/component_tensor.py:1387-1397 and :226-246). */
c3l_status c3l_contract(const c3l_contract_level* level, int32_t n, const c3l_complex* vectors,
                        c3l_complex* ws, void* stream);

/* Rest forms / scalars into padded workspace blocks (wedge materialization,
 * src/c3l/cc/component_tensor.py:869-898, :1035-1137). */
c3l_status c3l_wedge_padded(const c3l_wedge_stage* stage, int32_t n, c3l_complex* ws, void* stream);

/* Static residual/JVP outputs at tilde representatives, fused epilogue
 * r = -i (lam * src[mu] + V), written in real tilde coordinates
 * (src/c3l/cc/component_tensor.py:1855-1858, src/c3l/cc/component_solver.py:57-74). */
c3l_status c3l_wedge_static_out(const c3l_wedge_stage* stage, int32_t n, const c3l_complex* ws,
                                const c3l_complex* lam, const c3l_complex* src, const int64_t* col,
                                const int64_t* pair, const c3l_complex* scale, double* xout,
                                void* stream);

/* The same output stage over a complex FP32 workspace (FP64 epilogue). */
c3l_status c3l_wedge_static_out_f32(const c3l_wedge_stage* stage, int32_t n, const c3l_complex32* ws,
                                    const c3l_complex* lam, const c3l_complex* src, const int64_t* col,
                                    const int64_t* pair, const c3l_complex* scale, double* xout, void* stream);

/* EOM sigma outputs: out[mu] = lam * x[mu] + V
 * (src/c3l/cc/component_tensor.py:2288-2302). */
c3l_status c3l_wedge_eom_out(const c3l_wedge_stage* stage, int32_t n, const c3l_complex* ws,
                             const c3l_complex* lam, const c3l_complex* xin, c3l_complex* out,
                             void* stream);

/* The pair GEMMs alone over a complex workspace (the P blocks are written at
 * ws[program->base + p_off ...]): c3l_pair_gemm on the FP64 pipe,
 * c3l_pair_gemm_df in double-float arithmetic on the FP32 pipe (FP32 (hi, lo)
 * pairs, about 1e-14 relative; what the FP64 actions run), c3l_pair_gemm_f32
 * over an FP32 workspace. */
c3l_status c3l_pair_gemm(const c3l_pair_program* program, c3l_complex* ws, void* stream);
c3l_status c3l_pair_gemm_df(const c3l_pair_program* program, c3l_complex* ws, void* stream);
c3l_status c3l_pair_gemm_f32(const c3l_pair_program* program, c3l_complex32* ws, void* stream);
/* The FP32 pair GEMMs on the tcgen05 tensor cores (split-TF32: three TF32 MMAs
 * per real product, FP32 accumulation in tensor memory; about 5e-7 relative
 * per product), over program->tiles_tc. */
c3l_status c3l_pair_gemm_tc(const c3l_pair_program* program, c3l_complex32* ws, void* stream);

/* EOM sources: out[mu] = scale * V  (src/c3l/cc/component_tensor.py:2788-2798). */
c3l_status c3l_wedge_source_out(const c3l_wedge_stage* stage, int32_t n, const c3l_complex* ws,
                                c3l_complex scale, c3l_complex* out, void* stream);

/* ------------------------------------------------------ composite actions */

#define C3L_MAX_LEVELS 8
#define C3L_MAX_STAGES 4
#define C3L_MAX_BATCH 8

/* One operation = unpack/scatter, atom levels, padded stages, output stage. */
typedef struct {
    int32_t n;
    int32_t nlevels;
    int32_t npadded;
    int32_t pad;
    const c3l_complex* vectors;
    c3l_complex* ws;
    int64_t scatter_count;
    const int64_t* scatter_dst;
    const int64_t* scatter_pos;
    const double* scatter_sign;
    c3l_contract_level levels[C3L_MAX_LEVELS];
    c3l_wedge_stage padded[C3L_MAX_STAGES];
    c3l_pair_program pairs;   /* ntiles 0: none; else run before `out`, which reads P */
    c3l_wedge_stage out;
} c3l_action;

/* Static residual or JVP in real tilde coordinates:
 *   x (real, num_variables) -> tilde unpack -> padded -> atoms -> wedges -> xout.
 * Replaces component_static_residual / component_static_linearized_jvp behind
 * _real_residual / _real_linearized_jvp (src/c3l/cc/component_solver.py:57-74;
 * src/c3l/cc/component_tensor.py:1552-1657, :1822-1868).
 * canon: scratch complex[num_amplitudes] receiving the unpacked vector. */
typedef struct {
    c3l_action action;
    int64_t num_amplitudes;
    const int64_t* tilde_ia;
    const int64_t* tilde_ib;
    const c3l_complex* tilde_ca;
    const c3l_complex* tilde_cb;
    c3l_complex* canon;
    const c3l_complex* lam;
    const int64_t* col;
    const int64_t* pair;
    const c3l_complex* scale;
    /* optional (NULL: none): the rapidity preconditioner as one 2x2 block per
     * output element, [elements][4] row-major, applied to the outputs in the
     * output stage (the product M J of the Newton-Krylov inner solve) */
    const double* pc_m4;
    /* factor s multiplying the product part: xout = -i pack(Lambda x + s V(x)).
     * 1 is the problem as compiled; s < 1 is the reference's homotopy model
     * L0(K_ref) + s [L - L0(K_ref)] at a fixed HF reference
     * (src/c3l/models.py:516-549), whose products are the compiled ones with
     * every coefficient times s (examples/junction/gpu_timing.py:30-31). */
    double interaction_scale;
} c3l_static_action;

c3l_status c3l_static_apply(const c3l_static_action* action, const double* x, double* xout, void* stream);

/* EOM sigma in one (spin, charge) block: xin (complex, dim) -> out.
 * Replaces ComponentSigmaOperator.matvec (src/c3l/cc/component_response.py:53-58). */
typedef struct {
    c3l_action action;
    const c3l_complex* lam;
    /* factor s of the product part, out = lam x + s V(x): the EOM block of the
     * homotopy model at interaction scale s (see c3l_static_action) */
    double interaction_scale;
} c3l_eom_action;

c3l_status c3l_eom_sigma(const c3l_eom_action* action, const c3l_complex* xin, c3l_complex* out, void* stream);

/* The sigma action of one operator on nb <= C3L_MAX_BATCH vectors in one
 * launch per kernel: actions[b] differ only in their workspace (the same
 * program tables and lam), xin[b] -> out[b] (host arrays of device pointers). */
c3l_status c3l_eom_sigma_batch(const c3l_eom_action* actions, int32_t nb, const c3l_complex* const* xin,
                               c3l_complex* const* out, void* stream);

/* Single-precision variants: the action's `vectors` and `ws` point to
 * complex FP32 copies (c3l_complex32) of the factor-vector table and of the
 * workspace; inputs, outputs and epilogues stay FP64.  They serve as the inner
 * operator of the mixed-precision solves (the Newton residual stays FP64).
 * c3l_downcast copies an FP64 workspace (e.g. after an FP64 linearization)
 * into its FP32 twin. */
c3l_status c3l_static_apply_f32(const c3l_static_action* action, const double* x, double* xout, void* stream);
c3l_status c3l_eom_sigma_f32(const c3l_eom_action* action, const c3l_complex* xin, c3l_complex* out, void* stream);
c3l_status c3l_action_prepare_f32(const c3l_action* action, const c3l_complex* t, void* stream);
c3l_status c3l_downcast(int64_t count, const c3l_complex* src, c3l_complex32* dst, void* stream);

/* Runs the amplitude-only part of an action (levels + padded stages) after
 * scattering the complex amplitude vector t; used for linearization and EOM
 * contexts (src/c3l/cc/component_tensor.py:1371-1549, :2234-2251). */
c3l_status c3l_action_prepare(const c3l_action* action, const c3l_complex* t, void* stream);

/* ------------------------------------------------------------ Krylov ops */

/* out[j] = sum_i conj(V[j*ld + i]) * w[i], j < k  (two-pass deterministic
 * reduction; partial: scratch of c3l_multi_dot_scratch(k, dim) entries).
 * Replaces the zgemv projections of src/c3l/green/krylov.py:362-373. */
int64_t c3l_multi_dot_scratch(int32_t k, int64_t dim);
c3l_status c3l_multi_dot_c(const c3l_complex* V, int64_t ld, int32_t k, const c3l_complex* w, int64_t dim,
                           c3l_complex* partial, c3l_complex* out, void* stream);
c3l_status c3l_multi_dot_r(const double* V, int64_t ld, int32_t k, const double* w, int64_t dim,
                           double* partial, double* out, void* stream);

/* w[i] += alpha * sum_j c[j] * V[j*ld + i], j < k. */
c3l_status c3l_multi_axpy_c(const c3l_complex* V, int64_t ld, int32_t k, const c3l_complex* c, c3l_complex alpha,
                            c3l_complex* w, int64_t dim, void* stream);
c3l_status c3l_multi_axpy_r(const double* V, int64_t ld, int32_t k, const double* c, double alpha,
                            double* w, int64_t dim, void* stream);

/* y = a * x (complex or real). */
c3l_status c3l_scale_c(int64_t dim, c3l_complex a, const c3l_complex* x, c3l_complex* y, void* stream);
c3l_status c3l_scale_r(int64_t dim, double a, const double* x, double* y, void* stream);

/* out = inv * (z x - s) elementwise; s == NULL reads as 0 and inv == NULL as 1.
 * The shifted operator and Jacobi preconditioner of
 * src/c3l/cc/component_response.py:88-103 (A x = z x - K x, M = (z - diag)^{-1}). */
c3l_status c3l_shifted_combine(int64_t dim, c3l_complex z, const c3l_complex* x, const c3l_complex* s,
                               const c3l_complex* inv, c3l_complex* out, void* stream);

/* Real preconditioner pack(unpack(x) / diag) as 2x2 blocks per tilde orbit
 * (src/c3l/cc/newton_krylov.py:158-192). m4: [nrep][4] row-major blocks. */
c3l_status c3l_precondition(int64_t nrep, const double* m4, const int64_t* col, const int64_t* pair,
                            const double* x, double* y, void* stream);

/* Shifted Hessenberg solves for all shifts (one thread block per shift):
 * (z_s I - H_m) y = beta e_1 by streamed Givens QR, returning
 *   green[s]    = sum_k sinkproj[k] y_k      (if sinkproj != NULL)
 *   residual[s] = |H[m, m-1] y_{m-1}| / beta (Arnoldi relation residual)
 * H: (m+1) x m, row-major with leading dimension ldh (complex).
 * Replaces ArnoldiResolvent.coefficients/_reduced_residuals
 * (src/c3l/green/krylov.py:66-93, :257-281). m <= C3L_MAX_HESSENBERG. */
#define C3L_MAX_HESSENBERG 4096
c3l_status c3l_hessenberg_shifted(const c3l_complex* H, int64_t ldh, int32_t m, const c3l_complex* shifts,
                                  int32_t nshift, double beta, const c3l_complex* sinkproj,
                                  c3l_complex* green, double* residual, void* stream);

/* Incremental shifted solves: the running state of (z_s I - H_m) y = beta e_1
 * for all shifts while an Arnoldi basis grows.  The Givens rotations of the
 * first j columns of z I - H do not change when columns are appended, so
 * c3l_hessenberg_advance processes each new column once per shift and leaves,
 * for the square system of dimension m,
 *   green[s]    = sum_k p_k y_k           (if sinkproj_conj != NULL)
 *   residual[s] = |h_{m,m-1} y_{m-1}| / beta
 * (the quantities of c3l_hessenberg_shifted; ArnoldiResolvent.coefficients /
 * _reduced_residuals, src/c3l/green/krylov.py:66-93, :257-281).  Over a whole
 * run each shift costs one O(m^2/2) elimination, not one per check.
 * The caller owns every buffer; the library fills shifts/nshift/beta/
 * breakdown_tol when the state is driven by c3l_arnoldi.  Set done = 0 to
 * start a new basis.  A column j with |h_{j+1,j}| <= breakdown_tol stops the
 * advance there (status.first_break = j + 1; outputs are those of m = j + 1);
 * the state is then final. */
typedef struct {
    unsigned long long worst;  /* bit pattern of max_s residual[s] (a non-negative double) */
    int32_t first_break;       /* 1 + first breakdown column, 0: none */
    int32_t bad;               /* nonzero: a non-finite residual or green value */
} c3l_hessenberg_status;

typedef struct {
    int32_t m_max;                     /* capacity in columns                      */
    int32_t nshift;
    int32_t done;                      /* columns processed so far (host counter)  */
    int32_t pad;
    const c3l_complex* shifts;         /* device [nshift]                          */
    double beta;
    double breakdown_tol;
    const c3l_complex* sinkproj_conj;  /* device [m_max]: conj(p_k), or NULL       */
    double* rot_c;                     /* device [m_max][nshift]                   */
    c3l_complex* rot_s;                /* device [m_max][nshift]                   */
    c3l_complex* vsink;                /* device [m_max][nshift]                   */
    c3l_complex* carry;                /* device [nshift]                          */
    c3l_complex* accum;                /* device [nshift]                          */
    c3l_complex* green;                /* device [nshift] output, or NULL          */
    double* residual;                  /* device [nshift] output                   */
    c3l_hessenberg_status* status;     /* device, rewritten by every call          */
} c3l_hessenberg_state;

/* Advances the state over columns [done, m) of the column-major Hessenberg
 * Hc (column j at Hc + j*ldc holds rows 0..j+1; ldc >= m_max + 1). */
c3l_status c3l_hessenberg_advance(c3l_hessenberg_state* state, const c3l_complex* Hc, int64_t ldc, int32_t m,
                                  void* stream);

/* Arnoldi column j on the device from the CGS2 coefficients
 * coeff = [c1 (k) | c2 (k) | |w'|^2]: Hc[j*ldc + i] = c1_i + c2_i (i < k),
 * Hc[j*ldc + k] = h = sqrt(|w'|^2 - |c2|^2), and w /= h unless h <= tol. */
c3l_status c3l_arnoldi_column(const c3l_complex* coeff, int32_t k, c3l_complex* w, int64_t n, c3l_complex* Hc,
                              int64_t ldc, int32_t j, double tol, void* stream);

/* Full reduced coordinates Y[s][0..m) of the same systems (for solution
 * vectors); rscratch: nshift * m*(m+1)/2 complex entries of caller memory. */
c3l_status c3l_hessenberg_coordinates(const c3l_complex* H, int64_t ldh, int32_t m, const c3l_complex* shifts,
                                      int32_t nshift, double beta, c3l_complex* rscratch, c3l_complex* Y,
                                      void* stream);

/* ----------------------------------------------------------- Krylov drivers */

/* Left-preconditioned restarted GMRES for a Newton correction, with SciPy's
 * control flow (the solver of src/c3l/cc/component_solver.py:181-191): A is
 * the device JVP action, M the rapidity preconditioner.  Orthogonalization is
 * classical Gram-Schmidt twice on the device; the Givens updates run on the
 * host.  One inner iteration (JVP, preconditioner, CGS2, normalization) is a
 * CUDA graph captured once per call and replayed with the step index kept in
 * device memory; each iteration's Hessenberg column lands in its own slot of
 * pinned host memory, so the host processes iteration j while the GPU runs
 * iteration j + 1 (an iteration started after the stopping test passes is
 * discarded).
 * With pc_m4_elem (the preconditioner blocks in output-element order, see
 * c3l_static_action.pc_m4) the preconditioner is applied inside the JVP's
 * output stage instead of by a separate kernel.
 * Device buffers: V[(restart+1)*dim], tmp[dim], r[dim], x[dim] (output),
 * work[2*dim], counters[4] (int32), coeff[2*(restart+2)+3],
 * partial[partial_capacity >= c3l_gmres_scratch(restart, dim)]; pinned host:
 * host[3*(restart+2)+2], slots[restart*(restart+3)]; host: history[history_capacity].
 * restart <= 254. */
typedef struct {
    const c3l_static_action* jvp;
    int64_t nrep;
    const double* pc_m4;
    const int64_t* pc_col;
    const int64_t* pc_pair;
    int64_t dim;
    const double* b;
    double* x;
    double rtol;
    double atol;
    int32_t restart;
    int32_t maxiter;
    double* V;
    double* tmp;
    double* r;
    double* coeff;
    double* partial;
    double* host;
    double* history;
    int32_t history_capacity;
    /* outputs */
    int32_t history_len;
    int32_t info;
    int32_t matvecs;
    /* input: nonzero applies the JVP with c3l_static_apply_f32 */
    int32_t use_f32;
    double* work;
    int32_t* counters;
    double* slots;
    /* output: kernels launched (graph nodes included) */
    int64_t launches;
    const double* pc_m4_elem;
    int64_t partial_capacity;
    /* in/out: with keep_graphs set, the captured inner-iteration graphs are
     * kept in graph_cache and reused by later calls whose operator struct,
     * flags and buffers are unchanged (NULL on the first call); release them
     * with c3l_gmres_release.  keep_graphs = 0: captured per call. */
    int32_t keep_graphs;
    /* input: nonzero (with use_f32) keeps the Krylov basis in FP32 and runs
     * CGS2 in FP32; V then holds (restart+1)*dim floats of rows followed by
     * a dim-float work vector (within the same allocation). */
    int32_t basis_f32;
    void* graph_cache;
} c3l_gmres_args;

/* Frees graphs kept by c3l_gmres (NULL is a no-op). */
void c3l_gmres_release(void* graph_cache);

c3l_status c3l_gmres(c3l_gmres_args* args, void* stream);
/* Entries of the `partial` buffer c3l_gmres needs for (restart, dim) on the current device. */
int64_t c3l_gmres_scratch(int32_t restart, int64_t dim);

/* Left-preconditioned restarted GMRES for one shifted EOM system
 * (z I - K) x = b with SciPy's control flow (solve_component_shifted,
 * src/c3l/cc/component_response.py:72-128): A x = z x - sigma(x) with the
 * device sigma action, M = pc_inv elementwise (NULL: none), optional initial
 * solution in x (use_x0).  CGS2 orthogonalization on the device, complex
 * Givens updates (zlartg convention) on the host from one pinned read-back
 * per inner iteration.  This is the reference's per-frequency algorithm; the
 * batched form is c3l_arnoldi.
 * Device buffers: V[(restart+1)*dim], tmp[dim], r[dim], x[dim],
 * coeff[2*(restart+2)+3], partial[c3l_multi_dot_scratch(restart+1, dim)];
 * pinned host: host[3*(restart+2)+3]; host: history[history_capacity]. */
typedef struct {
    const c3l_eom_action* sigma;
    int32_t sigma_launches;  /* kernels per sigma call (for the launch count) */
    int32_t use_x0;
    int64_t dim;
    c3l_complex shift;
    const c3l_complex* pc_inv;
    const c3l_complex* b;
    c3l_complex* x;
    double rtol;
    double atol;
    int32_t restart;
    int32_t maxiter;
    c3l_complex* V;
    c3l_complex* tmp;
    c3l_complex* r;
    c3l_complex* coeff;
    c3l_complex* partial;
    c3l_complex* host;
    double* history;
    int32_t history_capacity;
    /* outputs */
    int32_t history_len;
    int32_t info;
    int32_t matvecs;
    int64_t launches;
} c3l_gmres_shifted_args;

c3l_status c3l_gmres_shifted(c3l_gmres_shifted_args* args, void* stream);

/* One Arnoldi channel (source vector and its own sigma workspace). */
typedef struct {
    const c3l_eom_action* sigma;
    const c3l_complex* b;
    const c3l_complex* sink_conj;      /* device [N] conj(sink), or NULL: residuals only */
    c3l_complex* V;                    /* device (m_max+1) x N, row-major        */
    c3l_complex* Hcol;                 /* device m_max x (m_max+1), column-major  */
    c3l_complex* coeff;                /* device >= 2*(m_max+1)+1                */
    c3l_complex* partial;              /* device c3l_multi_dot_scratch(m_max+1, N) */
    c3l_complex* host;                 /* pinned >= 2*(m_max+1)+1                */
    c3l_complex* H;                    /* host (m_max+1) x m_max row-major, filled on return, or NULL */
    c3l_hessenberg_state hess;         /* buffers (sinkproj_conj: device [m_max] when sink_conj is set) */
    c3l_hessenberg_status* status_host;/* pinned                                  */
    c3l_complex* work;                 /* device [2*N]                            */
    int32_t* counters;                 /* device [4] (int32)                      */
    c3l_complex32* V32;                /* device (m_max+1) x N: FP32 copy of the basis rows */
    c3l_complex32* work32;             /* device [N]: FP32 copy of each sigma output        */
    c3l_complex32* V32lo;              /* device (m_max+1) x N: V - V32 in FP32 (low parts) */
    c3l_complex32* work32lo;           /* device [N]: low part of the updated work vector   */
    /* optional (NULL: the sigma scatters its input itself): the nonzero entries
     * of the sigma's input scatter (sigma->action.scatter_*) grouped by input
     * element, so that each step writes the next step's padded input blocks
     * as it forms V[j+1]: entries [xscatter_offsets[i], xscatter_offsets[i+1])
     * are ws[xscatter_dst[e]] = xscatter_sign[e] * x[i]. */
    const int64_t* xscatter_offsets;   /* device [N + 1] */
    const int64_t* xscatter_dst;
    const double* xscatter_sign;
    int32_t* check_dims;               /* host [check_capacity]                   */
    double* check_res;                 /* host [check_capacity]                   */
    int32_t check_capacity;
    /* outputs (hess.green / hess.residual hold the shifted solves at dimension m) */
    int32_t m;
    int32_t breakdown;
    int32_t converged;
    int32_t nchecks;
    int32_t pad;
    double beta;
    double action_seconds;
    int64_t launches;                  /* kernels launched (graph nodes included) */
} c3l_arnoldi_channel;

/* CGS2 Arnoldi for (z I - K)^{-1} b on every channel
 * (src/c3l/green/krylov.py:284-417): stops a channel when the Arnoldi-relation
 * residual is <= tol for every shift (checked every check_interval steps from
 * min_dim on) or on breakdown (|h_{j+1,j}| <= breakdown_tol).  Channels whose
 * sigma actions run the same program (up to C3L_MAX_BATCH) step together on
 * the stream of their first channel: one step (sigma, CGS2, column of H,
 * normalization) for all of them is a CUDA graph captured once per call and
 * replayed with the step indices kept in device memory.  Each check advances
 * the incremental shifted solves (c3l_hessenberg_advance, FP64) over the new
 * columns on a stream of the driver's own while the channels take their next
 * steps, and reads back one status word per channel.  CGS2 arithmetic: FP32
 * first projections from the FP32 copies V32/work32; first update and second
 * projections in double-float from the (V32, V32lo) and (work32, work32lo)
 * pairs; second update V c2 with FP32 products; FP64 subtractions, scaling
 * and Hessenberg column.  On return hess.green / hess.residual hold the Green
 * function and residuals of the final dimension m. */
c3l_status c3l_arnoldi(c3l_arnoldi_channel* channels, int32_t nchannels, int64_t N, const c3l_complex* shifts,
                       int32_t nshift, int32_t m_max, double tol, int32_t min_dim, int32_t check_interval,
                       double breakdown_tol, void* const* streams);

/* ------------------------------------------------------- learned warm start
 * An element-wise MLP (C3L_MLP_INPUTS -> HIDDEN -> HIDDEN -> OUTPUTS, tanh)
 * mapping per-amplitude features to a correction of the first-order guess.
 * BF16 inputs/weights/activations, FP32 accumulation.  Parameters are laid
 * out W1[H][F] b1[H] W2[H][H] b2[H] W3[O][H] b3[O].  No counterpart in the
 * reference, whose solve starts from zero amplitudes
 * (src/c3l/cc/component_solver.py:121-122); the converged answer is still
 * judged by the FP64 residual, and the zero guess remains the fallback. */
#define C3L_MLP_INPUTS 16
#define C3L_MLP_HIDDEN 32
#define C3L_MLP_OUTPUTS 2
#define C3L_MLP_PARAMS (C3L_MLP_HIDDEN * C3L_MLP_INPUTS + C3L_MLP_HIDDEN + C3L_MLP_HIDDEN * C3L_MLP_HIDDEN + \
                        C3L_MLP_HIDDEN + C3L_MLP_OUTPUTS * C3L_MLP_HIDDEN + C3L_MLP_OUTPUTS)

/* Y[n][O] (FP32) from X[n][F] (BF16) and BF16 weights. */
c3l_status c3l_mlp_forward(int64_t n, const void* X, const void* weights_bf16, float* Y, void* stream);
/* Adds d/dparams of sum_s w_s |y_s - t_s|^2 * inv_wsum into grad[PARAMS] (FP32,
 * caller zeroes it) and the unscaled weighted loss into loss[0]; W may be NULL
 * (unit weights).  Accumulation order across blocks is not fixed. */
c3l_status c3l_mlp_backward(int64_t n, const void* X, const float* T, const float* W, float inv_wsum,
                            const void* weights_bf16, float* grad, float* loss, void* stream);
/* One Adam step (bias-corrected, step >= 1) on FP32 params; refreshes the BF16 copy. */
c3l_status c3l_mlp_adam(float* params, const float* grad, float* m, float* v, float lr, float beta1, float beta2,
                        float eps, int32_t step, void* weights_bf16, void* stream);
/* Features of each tilde-orbit representative: modes[nrep][4] (-1 padded),
 * the first two Jacobi iterates t1, t2 (real tilde coordinates), scale sigma
 * and interaction scale u. */
c3l_status c3l_warm_features(int64_t nrep, const int64_t* modes, const int64_t* col, const int64_t* pair,
                             const c3l_complex* rapidities, const double* t1, const double* t2, double sigma,
                             double u, void* X, void* stream);
/* x0 = t1 + sigma * Y at every representative's real columns. */
c3l_status c3l_warm_apply(int64_t nrep, const int64_t* col, const int64_t* pair, const double* t1, const float* Y,
                          double sigma, double* x0, void* stream);

/* Allocation-free variant of c3l_hessenberg_coordinates, for callers that
 * cannot allocate device memory: a host application that owns the device
 * memory budget (and hands this library only its input and output buffers),
 * or a caller that must not allocate between setup and shutdown.  It has no
 * counterpart in the reference, whose reduced solves run on the host.
 *
 * The R-factor scratch is a fixed array inside the library's device image of
 * C3L_NOALLOC_SCRATCH_ENTRIES complex entries (32 MiB), held on every GPU that
 * loads the library until the process exits.  One shift needs m*(m+1)/2
 * entries; m*(m+1)/2 > C3L_NOALLOC_SCRATCH_ENTRIES (m >= 2048) is rejected with
 * C3L_ERR_CAPACITY.  Larger shift counts are processed in chunks on `stream`.
 *
 * The first call on each device looks up the array's device address (with
 * that device current) and caches it; make that first call before any stream
 * capture.  The cached address belongs to the device's primary context:
 * resetting the device (cudaDeviceReset) while the library stays loaded is
 * not supported, since later calls would use the old context's address.  Every call shares the one array and leaves its contents behind;
 * each call writes every scratch entry it reads, so nothing has to start at
 * zero.  Calls that overlap on the GPU (other streams, other host threads)
 * race on the array: serialize them.  No cudaMalloc or cudaFree is called. */
#define C3L_NOALLOC_SCRATCH_ENTRIES (1 << 21)
c3l_status c3l_hessenberg_coordinates_noalloc(const c3l_complex* H, int64_t ldh, int32_t m, const c3l_complex* shifts,
                                              int32_t nshift, double beta, c3l_complex* Y, void* stream);

/* Library identification (host only). */
const char* c3l_version(void);

#ifdef __cplusplus
}
#endif

#endif /* C3L_GB300_H */

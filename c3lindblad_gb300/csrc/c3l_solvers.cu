// Host drivers of the Krylov solvers (C++ over the library's kernels).
//
// c3l_gmres   -- left-preconditioned restarted GMRES with SciPy's control flow
//                (the solver the reference calls for Newton corrections,
//                src/c3l/cc/component_solver.py:181), the operator being the
//                device JVP action.  One inner iteration (JVP, preconditioner,
//                CGS2, column) is a replayed CUDA graph; the host runs the
//                Givens updates one iteration behind the GPU.
// c3l_arnoldi -- CGS2 Arnoldi of src/c3l/green/krylov.py:284-417 for several
//                independent channels at once: each channel runs on its own
//                stream and workspace, so the channels' kernels overlap on the
//                GPU; the shifted solves advance incrementally at each check.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "c3l_gb300.h"
#include "c3l_internal.h"

namespace {

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

c3l_status d2h(void* host, const void* dev, size_t bytes, cudaStream_t s) {
    if (cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess) return C3L_ERR_LAUNCH;
    if (cudaStreamSynchronize(s) != cudaSuccess) return C3L_ERR_LAUNCH;
    return C3L_OK;
}

// Real plane rotation with c f + s g = r, -s f + c g = 0 (LAPACK dlartg convention).
void lartg(double f, double g, double& c, double& s, double& r) {
    if (g == 0.0) {
        c = 1.0;
        s = 0.0;
        r = f;
    } else if (f == 0.0) {
        c = 0.0;
        s = g > 0 ? 1.0 : -1.0;
        r = std::fabs(g);
    } else {
        const double h = std::hypot(f, g);
        c = std::fabs(f) / h;
        s = (f > 0 ? 1.0 : -1.0) * g / h;
        r = f > 0 ? h : -h;
    }
}

int sm_count() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return 152;
    return sms;
}

// A CUDA graph captured from a callback that enqueues work on a stream.
// Capture runs on a private stream, so the caller's stream (possibly the
// legacy default stream) only ever sees graph launches.
class StepGraph {
  public:
    StepGraph() = default;
    StepGraph(const StepGraph&) = delete;
    StepGraph& operator=(const StepGraph&) = delete;
    ~StepGraph() {
        if (exec_) cudaGraphExecDestroy(exec_);
        if (graph_) cudaGraphDestroy(graph_);
    }
    template <typename F>
    c3l_status capture(cudaStream_t cap, F&& enqueue) {
        if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return C3L_ERR_LAUNCH;
        const c3l_status st = enqueue(cap);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(cap, &g);
        if (st) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess || !g) return C3L_ERR_LAUNCH;
        graph_ = g;
        if (cudaGraphInstantiate(&exec_, graph_, 0) != cudaSuccess) return C3L_ERR_LAUNCH;
        size_t count = 0;
        if (cudaGraphGetNodes(graph_, nullptr, &count) != cudaSuccess) return C3L_ERR_LAUNCH;
        nodes_ = (int64_t)count;
        return C3L_OK;
    }
    c3l_status launch(cudaStream_t s) const {
        return exec_ && cudaGraphLaunch(exec_, s) == cudaSuccess ? C3L_OK : C3L_ERR_LAUNCH;
    }
    int64_t nodes() const { return nodes_; }
    bool captured() const { return exec_ != nullptr; }

  private:
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    int64_t nodes_ = 0;
};

struct OwnedStream {
    cudaStream_t s = nullptr;
    ~OwnedStream() {
        if (s) cudaStreamDestroy(s);
    }
    c3l_status create() {
        return cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess ? C3L_OK : C3L_ERR_LAUNCH;
    }
};

struct OwnedEvents {
    std::vector<cudaEvent_t> ev;
    ~OwnedEvents() {
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    }
    c3l_status create(int count) {
        ev.assign(count, nullptr);
        for (auto& e : ev)
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return C3L_ERR_LAUNCH;
        return C3L_OK;
    }
};

// Inner-iteration graphs of c3l_gmres kept between calls: valid while the
// operator struct, the flags and every buffer pointer are the same.
struct GmresGraphs {
    c3l_static_action op{};
    const double* pc_m4_elem = nullptr;
    int32_t use_f32 = 0, basis_f32 = 0;
    int64_t n = 0, nrep = 0;
    int restart = 0;
    const void* ptrs[10] = {};
    StepGraph inner[2];
    int64_t jvp_nodes = 0;

    static void key_ptrs(const c3l_gmres_args* a, const void** out) {
        const void* p[10] = {a->V, a->tmp, a->coeff, a->partial, a->work, a->counters, a->slots, a->pc_m4, a->pc_col,
                             a->pc_pair};
        for (int i = 0; i < 10; ++i) out[i] = p[i];
    }
    bool matches(const c3l_gmres_args* a, int rs) const {
        const void* p[10];
        key_ptrs(a, p);
        return std::memcmp(&op, a->jvp, sizeof(op)) == 0 && pc_m4_elem == a->pc_m4_elem && use_f32 == a->use_f32 &&
               basis_f32 == a->basis_f32 && n == a->dim && nrep == a->nrep && restart == rs && std::memcmp(ptrs, p, sizeof(ptrs)) == 0;
    }
};

// Complex plane rotation (LAPACK zlartg convention): real c, complex s with
// c f + s g = r and -conj(s) f + c g = 0.
void zlartg(c3l_complex f, c3l_complex g, double& c, c3l_complex& sn, c3l_complex& r) {
    const double ng = std::hypot(g.re, g.im);
    if (ng == 0.0) {
        c = 1.0;
        sn = {0.0, 0.0};
        r = f;
        return;
    }
    const double nf = std::hypot(f.re, f.im);
    if (nf == 0.0) {
        c = 0.0;
        sn = {g.re / ng, -g.im / ng};
        r = {ng, 0.0};
        return;
    }
    const double rho = std::hypot(nf, ng);
    c = nf / rho;
    const c3l_complex ph{f.re / nf, f.im / nf};
    const c3l_complex gc{g.re / rho, -g.im / rho};  // conj(g) / rho
    sn = {ph.re * gc.re - ph.im * gc.im, ph.re * gc.im + ph.im * gc.re};
    r = {ph.re * rho, ph.im * rho};
}

inline c3l_complex cmulh(c3l_complex a, c3l_complex b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline c3l_complex cconjh(c3l_complex a) { return {a.re, -a.im}; }
inline c3l_complex caddh(c3l_complex a, c3l_complex b) { return {a.re + b.re, a.im + b.im}; }
inline c3l_complex csubh(c3l_complex a, c3l_complex b) { return {a.re - b.re, a.im - b.im}; }
inline c3l_complex cdivh(c3l_complex a, c3l_complex b) {
    const double d = b.re * b.re + b.im * b.im;
    return {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}

}  // namespace

extern "C" {

void c3l_gmres_release(void* graph_cache) { delete static_cast<GmresGraphs*>(graph_cache); }

int64_t c3l_gmres_scratch(int32_t restart, int64_t dim) {
    if (restart <= 0 || dim <= 0) return 0;
    const int r = (int)std::min<int64_t>(restart, dim);
    const c3l::GmPlan gp = c3l::gm_plan(dim, r + 2, sm_count());
    return 2 * (int64_t)gp.blocks * (r + 2);
}

c3l_status c3l_gmres(c3l_gmres_args* a, void* stream) {
    if (!a || !a->jvp || !a->b || !a->x || !a->V || !a->tmp || !a->r || !a->coeff || !a->partial || !a->host ||
        !a->pc_m4 || !a->pc_col || !a->pc_pair || !a->work || !a->counters || !a->slots || a->dim <= 0 ||
        a->partial_capacity <= 0 || a->restart <= 0 || a->maxiter <= 0 || (a->basis_f32 && !a->use_f32))
        return C3L_ERR_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    const int64_t n = a->dim;
    const int restart = (int)std::min<int64_t>(a->restart, n);
    const double eps = 2.220446049250313e-16;
    double* V = a->V;
    double* host = a->host;
    double* coeff = a->coeff;
    double* ones = coeff + 2 * (restart + 2) + 2;  // one device 1.0 (set below)
    c3l_status st;
    a->history_len = 0;
    a->matvecs = 0;
    a->launches = 0;
    // one inner iteration as a graph: xcur -> M J -> wfix, CGS2 against
    // V[0..j] in three kernels, column j into host-mapped slot j, V[j+1] =
    // xcur = w'' / h.  The step index alternates between two counters, so
    // there is one graph per parity.
    double* xcur = a->work;
    double* wfix = a->work + n;
    const int R = restart + 2;
    double* c1 = coeff;  // reduced pass-1 projections (k + 1)
    // FP32 basis: rows of n floats, then the FP32 work vector, inside V
    const bool f32b = a->basis_f32 != 0;
    float* Vf = reinterpret_cast<float*>(V);
    float* wf = Vf + (int64_t)(restart + 1) * n;
    float* c1f = reinterpret_cast<float*>(coeff);
    float* pf = reinterpret_cast<float*>(a->partial);
    const int stride = restart + 3;
    if (R > C3L_GMRES_MAX_ROWS) return C3L_ERR_CAPACITY;
    const c3l::GmPlan gp = c3l::gm_plan(n, R, sm_count());
    if (2 * (int64_t)gp.blocks * R > a->partial_capacity) return C3L_ERR_CAPACITY;
    GmresGraphs* cache = static_cast<GmresGraphs*>(a->graph_cache);
    std::unique_ptr<GmresGraphs> local;
    if (!cache || !cache->matches(a, restart)) {
        delete cache;
        a->graph_cache = nullptr;
        local.reset(new GmresGraphs());
        GmresGraphs& gg = *local;
        gg.op = *a->jvp;
        gg.pc_m4_elem = a->pc_m4_elem;
        gg.use_f32 = a->use_f32;
        gg.basis_f32 = a->basis_f32;
        gg.n = n;
        gg.nrep = a->nrep;
        gg.restart = restart;
        GmresGraphs::key_ptrs(a, gg.ptrs);
        c3l_static_action fused = *a->jvp;
        if (a->pc_m4_elem) fused.pc_m4 = a->pc_m4_elem;
        const c3l_static_action* op = &fused;
        OwnedStream cap;
        if ((st = cap.create())) return st;
        for (int par = 0; par < 2; ++par) {
            const int* cur = a->counters + par;
            int* next = a->counters + (1 - par);
            st = gg.inner[par].capture(cap.s, [&](cudaStream_t cs) -> c3l_status {
                void* csv = reinterpret_cast<void*>(cs);
                c3l_status q;
                if (a->pc_m4_elem) {
                    q = a->use_f32 ? c3l_static_apply_f32(op, xcur, wfix, csv) : c3l_static_apply(op, xcur, wfix, csv);
                    if (q) return q;
                } else {
                    q = a->use_f32 ? c3l_static_apply_f32(op, xcur, a->tmp, csv)
                                   : c3l_static_apply(op, xcur, a->tmp, csv);
                    if (q) return q;
                    if ((q = c3l_precondition(a->nrep, a->pc_m4, a->pc_col, a->pc_pair, a->tmp, wfix, csv))) return q;
                }
                if (f32b) {
                    if ((q = c3l::gm_dot_f32(Vf, n, cur, wfix, wf, n, gp, pf, cs))) return q;
                    if ((q = c3l::gm_axpy_dot_f32(Vf, n, cur, c1f, wf, n, gp, pf, cs))) return q;
                    return c3l::gm_scale_f32(Vf, n, cur, next, pf, c1f, eps, wf, n, gp, xcur, a->slots, stride, cs);
                }
                if ((q = c3l::gm_dot(V, n, cur, wfix, n, gp, a->partial, cs))) return q;
                if ((q = c3l::gm_axpy_dot(V, n, cur, c1, wfix, n, gp, a->partial, cs))) return q;
                return c3l::gm_scale(V, n, cur, next, a->partial, c1, eps, wfix, n, gp, xcur, a->slots, stride, cs);
            });
            if (st) return st;
        }
        // kernels of one operator application: the graph less the three CGS2 kernels
        gg.jvp_nodes = gg.inner[0].nodes() - 3 - (a->pc_m4_elem ? 0 : 1);
        cache = local.get();
        if (a->keep_graphs) a->graph_cache = local.release();
    }
    StepGraph* inner = cache->inner;
    const int64_t jvp_nodes = cache->jvp_nodes;
    OwnedEvents ev;
    if ((st = ev.create(2))) return st;
    auto matvec = [&](const double* in, double* out) -> c3l_status {
        a->matvecs += 1;
        return a->use_f32 ? c3l_static_apply_f32(a->jvp, in, out, stream) : c3l_static_apply(a->jvp, in, out, stream);
    };
    auto psolve = [&](const double* in, double* out) -> c3l_status {
        a->launches += 1;
        return c3l_precondition(a->nrep, a->pc_m4, a->pc_col, a->pc_pair, in, out, stream);
    };
    auto norm = [&](const double* v, double& out) -> c3l_status {
        c3l_status q = c3l_multi_dot_r(v, n, 1, v, n, a->partial, coeff, stream);
        if (q) return q;
        a->launches += 2;
        if ((q = d2h(host, coeff, sizeof(double), s))) return q;
        out = std::sqrt(std::max(host[0], 0.0));
        return C3L_OK;
    };
    host[0] = 1.0;
    if (cudaMemcpyAsync(ones, host, sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess) return C3L_ERR_LAUNCH;
    if (cudaMemsetAsync(a->x, 0, n * sizeof(double), s) != cudaSuccess) return C3L_ERR_LAUNCH;
    double bnrm2;
    if ((st = norm(a->b, bnrm2))) return st;
    const double atol = std::max(a->atol, a->rtol * bnrm2);
    a->info = 0;
    if (bnrm2 == 0.0) {
        return cudaMemcpyAsync(a->x, a->b, n * sizeof(double), cudaMemcpyDeviceToDevice, s) == cudaSuccess
                   ? C3L_OK : C3L_ERR_LAUNCH;
    }
    if ((st = psolve(a->b, a->tmp))) return st;
    double mb;
    if ((st = norm(a->tmp, mb))) return st;
    double ptol_max_factor = 1.0;
    double ptol = mb * std::min(ptol_max_factor, atol / bnrm2);
    if (cudaMemcpyAsync(a->r, a->b, n * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess) return C3L_ERR_LAUNCH;
    double rnorm = bnrm2;
    double presid = 0.0;
    std::vector<double> S(restart + 1), h((size_t)restart * (restart + 1)), gc(restart), gs(restart), y;
    auto H = [&](int col, int row) -> double& { return h[(size_t)col * (restart + 1) + row]; };
    // M r of the next cycle goes to tmp (FP32 basis) or V[0] (FP64 basis); its
    // norm is read together with |r| at the end of each cycle
    double* mr = f32b ? a->tmp : V;
    double beta_next = -1.0;
    for (int iteration = 0; iteration < a->maxiter; ++iteration) {
        if (iteration == 0 && bnrm2 < atol) return C3L_OK;
        double beta = beta_next;
        if (beta < 0.0) {
            if ((st = psolve(a->r, mr))) return st;
            if ((st = norm(mr, beta))) return st;
        }
        if (f32b) {
            if ((st = c3l::gm_start_f32(n, 1.0 / beta, a->tmp, Vf, xcur, s))) return st;
        } else {
            if ((st = c3l_scale_r(n, 1.0 / beta, V, V, stream))) return st;
            if (cudaMemcpyAsync(xcur, V, n * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
                return C3L_ERR_LAUNCH;
        }
        if (cudaMemsetAsync(a->counters, 0, 4 * sizeof(int32_t), s) != cudaSuccess) return C3L_ERR_LAUNCH;
        a->launches += 1;  // scale
        std::fill(S.begin(), S.end(), 0.0);
        std::fill(h.begin(), h.end(), 0.0);
        S[0] = beta;
        bool breakdown = false;
        int col = 0;
        auto enqueue = [&](int j) -> c3l_status {
            c3l_status q = inner[j & 1].launch(s);
            if (q) return q;
            a->launches += inner[j & 1].nodes();
            return cudaEventRecord(ev.ev[j & 1], s) == cudaSuccess ? C3L_OK : C3L_ERR_LAUNCH;
        };
        if ((st = enqueue(0))) return st;
        for (col = 0; col < restart; ++col) {
            // keep the GPU one iteration ahead; an iteration past the stop is discarded
            if (col + 1 < restart && (st = enqueue(col + 1))) return st;
            if (cudaEventSynchronize(ev.ev[col & 1]) != cudaSuccess) return C3L_ERR_LAUNCH;
            a->matvecs += 1;
            const int k = col + 1;
            const volatile double* slot = a->slots + (int64_t)col * stride;
            for (int j = 0; j < k; ++j) H(col, j) = slot[j];
            const double h1 = slot[k];
            const double h0 = slot[k + 1];
            H(col, col + 1) = h1;
            if (h1 <= eps * h0) {
                H(col, col + 1) = 0.0;
                breakdown = true;
            }
            for (int j = 0; j < col; ++j) {
                const double n0 = H(col, j), n1 = H(col, j + 1);
                H(col, j) = gc[j] * n0 + gs[j] * n1;
                H(col, j + 1) = -gs[j] * n0 + gc[j] * n1;
            }
            double c, sn, mag;
            lartg(H(col, col), H(col, col + 1), c, sn, mag);
            gc[col] = c;
            gs[col] = sn;
            H(col, col) = mag;
            H(col, col + 1) = 0.0;
            const double t = -sn * S[col];
            S[col] = c * S[col];
            S[col + 1] = t;
            presid = std::fabs(t);
            if (a->history && a->history_len < a->history_capacity) a->history[a->history_len] = presid / bnrm2;
            a->history_len += 1;
            if (presid <= ptol || breakdown) break;
        }
        if (col == restart) col = restart - 1;
        if (H(col, col) == 0.0) S[col] = 0.0;
        y.assign(S.begin(), S.begin() + col + 1);
        for (int k = col; k > 0; --k) {
            if (y[k] != 0.0) {
                y[k] /= H(k, k);
                const double tk = y[k];
                for (int j = 0; j < k; ++j) y[j] -= tk * H(k, j);
            }
        }
        if (y[0] != 0.0) y[0] /= H(0, 0);
        // y goes through its own pinned region: the read-back region is written by later copies
        double* yhost = host + 2 * (restart + 2) + 2;
        std::copy(y.begin(), y.end(), yhost);
        if (cudaMemcpyAsync(coeff, yhost, (col + 1) * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess)
            return C3L_ERR_LAUNCH;
        if ((st = f32b ? c3l::gm_update_f32(Vf, n, col + 1, coeff, a->x, n, s)
                       : c3l_multi_axpy_r(V, n, col + 1, coeff, 1.0, a->x, n, stream)))
            return st;
        if ((st = matvec(a->x, a->tmp))) return st;
        if (cudaMemcpyAsync(a->r, a->b, n * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess) return C3L_ERR_LAUNCH;
        if ((st = c3l_multi_axpy_r(a->tmp, n, 1, ones, -1.0, a->r, n, stream))) return st;
        a->launches += 2 + jvp_nodes;  // two axpys and the JVP
        // |r| and, for the next cycle, M r and |M r|: one read-back
        if ((st = psolve(a->r, mr))) return st;
        if ((st = c3l_multi_dot_r(a->r, n, 1, a->r, n, a->partial, coeff, stream)) ||
            (st = c3l_multi_dot_r(mr, n, 1, mr, n, a->partial, coeff + 1, stream)))
            return st;
        a->launches += 4;
        if ((st = d2h(host, coeff, 2 * sizeof(double), s))) return st;
        rnorm = std::sqrt(std::max(host[0], 0.0));
        beta_next = std::sqrt(std::max(host[1], 0.0));
        if (rnorm <= atol) break;
        if (breakdown) break;
        if (presid <= ptol) ptol_max_factor = std::max(eps, 0.25 * ptol_max_factor);
        else ptol_max_factor = std::min(1.0, 1.5 * ptol_max_factor);
        ptol = presid * std::min(ptol_max_factor, atol / rnorm);
    }
    a->info = rnorm <= atol ? 0 : a->maxiter;
    return C3L_OK;
}

c3l_status c3l_gmres_shifted(c3l_gmres_shifted_args* a, void* stream) {
    if (!a || !a->sigma || !a->b || !a->x || !a->V || !a->tmp || !a->r || !a->coeff || !a->partial || !a->host ||
        a->dim <= 0 || a->restart <= 0 || a->maxiter <= 0 || !(a->rtol >= 0.0) || !(a->atol >= 0.0))
        return C3L_ERR_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    const int64_t n = a->dim;
    const int restart = (int)std::min<int64_t>(a->restart, n);
    const double eps = 2.220446049250313e-16;
    c3l_complex* V = a->V;
    c3l_complex* host = a->host;
    c3l_complex* coeff = a->coeff;
    c3l_complex* ones = coeff + 2 * (restart + 2) + 2;
    c3l_status st;
    a->history_len = 0;
    a->matvecs = 0;
    a->launches = 0;
    // A x = z x - sigma(x), then M (elementwise inverse of z - diag, or none)
    auto apply = [&](const c3l_complex* in, c3l_complex* out, bool precondition) -> c3l_status {
        a->matvecs += 1;
        c3l_status q = c3l_eom_sigma(a->sigma, in, a->tmp, stream);
        if (q) return q;
        a->launches += a->sigma_launches + 1;
        return c3l_shifted_combine(n, a->shift, in, a->tmp, precondition ? a->pc_inv : nullptr, out, stream);
    };
    auto psolve = [&](const c3l_complex* in, c3l_complex* out) -> c3l_status {
        a->launches += 1;
        return c3l_shifted_combine(n, c3l_complex{1.0, 0.0}, in, nullptr, a->pc_inv, out, stream);
    };
    auto norm = [&](const c3l_complex* v, double& out) -> c3l_status {
        c3l_status q = c3l_multi_dot_c(v, n, 1, v, n, a->partial, coeff, stream);
        if (q) return q;
        a->launches += n > 8192 ? 2 : 1;
        if ((q = d2h(host, coeff, sizeof(c3l_complex), s))) return q;
        out = std::sqrt(std::max(host[0].re, 0.0));
        return C3L_OK;
    };
    host[0] = {1.0, 0.0};
    if (cudaMemcpyAsync(ones, host, sizeof(c3l_complex), cudaMemcpyHostToDevice, s) != cudaSuccess) return C3L_ERR_LAUNCH;
    if (!a->use_x0 && cudaMemsetAsync(a->x, 0, n * sizeof(c3l_complex), s) != cudaSuccess) return C3L_ERR_LAUNCH;
    double bnrm2;
    if ((st = norm(a->b, bnrm2))) return st;
    const double atol = std::max(a->atol, a->rtol * bnrm2);
    a->info = 0;
    if (bnrm2 == 0.0) {
        return cudaMemcpyAsync(a->x, a->b, n * sizeof(c3l_complex), cudaMemcpyDeviceToDevice, s) == cudaSuccess
                   ? C3L_OK : C3L_ERR_LAUNCH;
    }
    // SciPy scales the preconditioned tolerance by |M b|
    if ((st = psolve(a->b, a->r))) return st;
    double mb;
    if ((st = norm(a->r, mb))) return st;
    double ptol_max_factor = 1.0;
    double ptol = mb * std::min(ptol_max_factor, atol / bnrm2);
    // r = b - A x0 (or b)
    auto residual = [&](double& out) -> c3l_status {
        c3l_status q;
        if (cudaMemcpyAsync(a->r, a->b, n * sizeof(c3l_complex), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return C3L_ERR_LAUNCH;
        if ((q = apply(a->x, V, false))) return q;  // V[0] as scratch for A x
        if ((q = c3l_multi_axpy_c(V, n, 1, ones, c3l_complex{-1.0, 0.0}, a->r, n, stream))) return q;
        a->launches += 1;
        return norm(a->r, out);
    };
    double rnorm = bnrm2;
    if (a->use_x0) {
        if ((st = residual(rnorm))) return st;
    } else if (cudaMemcpyAsync(a->r, a->b, n * sizeof(c3l_complex), cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
        return C3L_ERR_LAUNCH;
    }
    double presid = 0.0;
    std::vector<c3l_complex> S(restart + 1), h((size_t)restart * (restart + 1)), gs(restart), y;
    std::vector<double> gc(restart);
    auto H = [&](int col, int row) -> c3l_complex& { return h[(size_t)col * (restart + 1) + row]; };
    for (int iteration = 0; iteration < a->maxiter; ++iteration) {
        if (iteration == 0 && rnorm <= atol) return C3L_OK;
        if ((st = psolve(a->r, V))) return st;
        double beta;
        if ((st = norm(V, beta))) return st;
        if ((st = c3l_scale_c(n, c3l_complex{1.0 / beta, 0.0}, V, V, stream))) return st;
        a->launches += 1;
        std::fill(S.begin(), S.end(), c3l_complex{0.0, 0.0});
        std::fill(h.begin(), h.end(), c3l_complex{0.0, 0.0});
        S[0] = {beta, 0.0};
        bool breakdown = false;
        int col = 0;
        for (col = 0; col < restart; ++col) {
            c3l_complex* w = V + (int64_t)(col + 1) * n;
            if ((st = apply(V + (int64_t)col * n, w, true))) return st;
            const int k = col + 1;
            // CGS2: pass 1 with |w|^2 (row k is w itself), pass 2 with |w'|^2
            if ((st = c3l_multi_dot_c(V, n, k + 1, w, n, a->partial, coeff, stream))) return st;
            if ((st = c3l_multi_axpy_c(V, n, k, coeff, c3l_complex{-1.0, 0.0}, w, n, stream))) return st;
            if ((st = c3l_multi_dot_c(V, n, k + 1, w, n, a->partial, coeff + k + 1, stream))) return st;
            if ((st = c3l_multi_axpy_c(V, n, k, coeff + k + 1, c3l_complex{-1.0, 0.0}, w, n, stream))) return st;
            a->launches += 2 * (n > 8192 ? 2 : 1) + 2;
            if ((st = d2h(host, coeff, 2 * (k + 1) * sizeof(c3l_complex), s))) return st;
            const double h0 = std::sqrt(std::max(host[k].re, 0.0));
            double c2sq = 0.0;
            for (int j = 0; j < k; ++j) c2sq += host[k + 1 + j].re * host[k + 1 + j].re + host[k + 1 + j].im * host[k + 1 + j].im;
            const double h1 = std::sqrt(std::max(host[2 * k + 1].re - c2sq, 0.0));
            for (int j = 0; j < k; ++j) H(col, j) = caddh(host[j], host[k + 1 + j]);
            H(col, col + 1) = {h1, 0.0};
            if (h1 <= eps * h0) {
                H(col, col + 1) = {0.0, 0.0};
                breakdown = true;
            } else {
                if ((st = c3l_scale_c(n, c3l_complex{1.0 / h1, 0.0}, w, w, stream))) return st;
                a->launches += 1;
            }
            for (int j = 0; j < col; ++j) {
                const c3l_complex n0 = H(col, j), n1 = H(col, j + 1);
                H(col, j) = caddh(c3l_complex{gc[j] * n0.re, gc[j] * n0.im}, cmulh(gs[j], n1));
                H(col, j + 1) = caddh(cmulh(c3l_complex{-gs[j].re, gs[j].im}, n0), c3l_complex{gc[j] * n1.re, gc[j] * n1.im});
            }
            double c;
            c3l_complex sn, mag;
            zlartg(H(col, col), H(col, col + 1), c, sn, mag);
            gc[col] = c;
            gs[col] = sn;
            H(col, col) = mag;
            H(col, col + 1) = {0.0, 0.0};
            const c3l_complex t = cmulh(c3l_complex{-sn.re, sn.im}, S[col]);  // -conj(s) S[col]
            S[col] = {c * S[col].re, c * S[col].im};
            S[col + 1] = t;
            presid = std::hypot(t.re, t.im);
            if (a->history && a->history_len < a->history_capacity) a->history[a->history_len] = presid / bnrm2;
            a->history_len += 1;
            if (presid <= ptol || breakdown) break;
        }
        if (col == restart) col = restart - 1;
        if (H(col, col).re == 0.0 && H(col, col).im == 0.0) S[col] = {0.0, 0.0};
        y.assign(S.begin(), S.begin() + col + 1);
        for (int k = col; k > 0; --k) {
            if (y[k].re != 0.0 || y[k].im != 0.0) {
                y[k] = cdivh(y[k], H(k, k));
                const c3l_complex tk = y[k];
                for (int j = 0; j < k; ++j) y[j] = csubh(y[j], cmulh(tk, H(k, j)));
            }
        }
        if (y[0].re != 0.0 || y[0].im != 0.0) y[0] = cdivh(y[0], H(0, 0));
        c3l_complex* yhost = host + 2 * (restart + 2) + 2;
        std::copy(y.begin(), y.end(), yhost);
        if (cudaMemcpyAsync(coeff, yhost, (col + 1) * sizeof(c3l_complex), cudaMemcpyHostToDevice, s) != cudaSuccess)
            return C3L_ERR_LAUNCH;
        if ((st = c3l_multi_axpy_c(V, n, col + 1, coeff, c3l_complex{1.0, 0.0}, a->x, n, stream))) return st;
        a->launches += 1;
        if ((st = residual(rnorm))) return st;
        if (rnorm <= atol) break;
        if (breakdown) break;
        if (presid <= ptol) ptol_max_factor = std::max(eps, 0.25 * ptol_max_factor);
        else ptol_max_factor = std::min(1.0, 1.5 * ptol_max_factor);
        ptol = presid * std::min(ptol_max_factor, atol / rnorm);
    }
    a->info = rnorm <= atol ? 0 : a->maxiter;
    return C3L_OK;
}

c3l_status c3l_arnoldi(c3l_arnoldi_channel* ch, int32_t nch, int64_t N, const c3l_complex* shifts, int32_t nshift,
                       int32_t m_max, double tol, int32_t min_dim, int32_t check_interval, double breakdown_tol,
                       void* const* streams) {
    if (!ch || nch <= 0 || N <= 0 || !shifts || nshift <= 0 || m_max <= 0 || m_max > N || !streams ||
        m_max > C3L_MAX_HESSENBERG || check_interval <= 0 || min_dim < 1 || min_dim > m_max)
        return C3L_ERR_ARGUMENT;
    for (int c = 0; c < nch; ++c) {
        const c3l_arnoldi_channel& q = ch[c];
        const c3l_hessenberg_state& h = q.hess;
        if (!q.sigma || !q.b || !q.V || !q.Hcol || !q.coeff || !q.partial || !q.host || !q.status_host || !q.work ||
            !q.counters || !q.V32 || !q.work32 || !q.V32lo || !q.work32lo || !h.rot_c || !h.rot_s || !h.vsink || !h.carry || !h.accum || !h.residual || !h.status ||
            h.m_max < m_max || h.nshift != nshift || (q.sink_conj && !h.sinkproj_conj))
            return C3L_ERR_ARGUMENT;
    }
    const int64_t ldc = (int64_t)m_max + 1;
    const c3l::RowDot rd = c3l::row_dot_plan(m_max + 1, N, sm_count());
    if (c3l::row_dot_partial_size(rd) > c3l_multi_dot_scratch(m_max + 1, N)) return C3L_ERR_CAPACITY;
    c3l_status st;
    // Channels whose sigma actions run the same program step together in a
    // group: one Arnoldi step of the whole group is one graph, every kernel
    // serving all of its channels (blockIdx.y = channel), on the stream of the
    // group's first channel.  Step: xnext -> sigma -> wfix, CGS2 against
    // V[0..j] (the pass-2 projections also form column j of H and h), V[j+1]
    // = xnext = w'' / h.  The step index alternates between two counters per
    // channel: graphs exist for both parities, and `interval` chains
    // check_interval steps starting at either parity.  A channel that has
    // stopped is skipped through its stop counter.
    std::vector<std::vector<int>> groups;
    std::vector<int> group_of(nch, 0);
    for (int c = 0; c < nch; ++c) {
        int g = -1;
        for (size_t i = 0; i < groups.size() && g < 0; ++i)
            if ((int)groups[i].size() < C3L_MAX_BATCH && c3l::same_sigma_program(*ch[groups[i][0]].sigma, *ch[c].sigma))
                g = (int)i;
        if (g < 0) {
            g = (int)groups.size();
            groups.emplace_back();
        }
        groups[g].push_back(c);
        group_of[c] = g;
    }
    const int ng = (int)groups.size();
    auto chan_stream = [&](int c) { return as_stream(streams[groups[group_of[c]].front()]); };
    auto d2 = [](c3l_complex* p) { return reinterpret_cast<double2*>(p); };
    OwnedStream cap;
    if ((st = cap.create())) return st;
    // per-group launch data, kept for the whole call: graphs are captured on
    // first use (checks at multiples of check_interval launch only the
    // interval graph of one parity)
    struct GroupStep {
        c3l::ArnoldiBatch bt{};
        std::vector<c3l_eom_action> acts;
        std::vector<const c3l_complex*> xin;
        std::vector<c3l_complex*> out;
        std::vector<c3l_complex32*> out32;
        std::vector<const int32_t*> stop;
        bool fused_scatter = false;
    };
    std::vector<GroupStep> gsteps(ng);
    for (int g = 0; g < ng; ++g) {
        const std::vector<int>& mem = groups[g];
        const int nb = (int)mem.size();
        GroupStep& gs = gsteps[g];
        gs.bt.nb = nb;
        gs.acts.resize(nb);
        gs.xin.resize(nb);
        gs.out.resize(nb);
        gs.out32.resize(nb);
        gs.stop.resize(nb);
        for (int i = 0; i < nb; ++i) {
            c3l_arnoldi_channel& q = ch[mem[i]];
            gs.acts[i] = *q.sigma;
            gs.xin[i] = q.work;
            gs.out[i] = q.work + N;
            gs.out32[i] = q.work32;
            gs.stop[i] = q.counters + 3;
            c3l::ArnoldiBatch& bt = gs.bt;
            bt.V[i] = d2(q.V);
            bt.w[i] = d2(q.work + N);
            bt.xnext[i] = d2(q.work);
            bt.c1[i] = d2(q.coeff);
            bt.c2[i] = d2(q.coeff + (m_max + 1));
            bt.hval[i] = reinterpret_cast<double*>(q.coeff + 2 * (m_max + 1));
            bt.counters[i] = q.counters;
            bt.Hc[i] = d2(q.Hcol);
            bt.partial[i] = d2(q.partial);
            bt.V32[i] = reinterpret_cast<float2*>(q.V32);
            bt.w32[i] = reinterpret_cast<float2*>(q.work32);
            bt.V32lo[i] = reinterpret_cast<float2*>(q.V32lo);
            bt.w32lo[i] = reinterpret_cast<float2*>(q.work32lo);
        }
        // the second update writes the next sigma's padded input when every
        // channel of the group supplies the scatter grouped by element
        bool fused = true;
        for (int i = 0; i < nb; ++i) {
            const c3l_arnoldi_channel& q = ch[mem[i]];
            fused = fused && q.xscatter_offsets && q.xscatter_dst && q.xscatter_sign;
        }
        gs.fused_scatter = fused;
        if (fused) {
            const c3l_arnoldi_channel& q0 = ch[mem[0]];
            gs.bt.xoff = q0.xscatter_offsets;
            gs.bt.xdst = q0.xscatter_dst;
            gs.bt.xsign = q0.xscatter_sign;
            for (int i = 0; i < nb; ++i) gs.bt.xws[i] = reinterpret_cast<double2*>(ch[mem[i]].sigma->action.ws);
        }
    }
    auto step = [&](const GroupStep& gs, cudaStream_t cs, int par) -> c3l_status {
        c3l_status r = c3l::eom_sigma_batch(gs.acts.data(), gs.bt.nb, gs.xin.data(), gs.out.data(), gs.out32.data(),
                                            gs.stop.data(), cs, gs.fused_scatter);
        if (r) return r;
        if ((r = c3l::arnoldi_dot1(gs.bt, par, N, N, rd, cs))) return r;
        if ((r = c3l::arnoldi_axpy1(gs.bt, par, N, m_max, N, cs))) return r;
        if ((r = c3l::arnoldi_dot2(gs.bt, par, N, N, rd, ldc, cs))) return r;
        return c3l::arnoldi_scale(gs.bt, par, N, m_max, breakdown_tol, N, cs);
    };
    std::vector<StepGraph> one(2 * ng), interval(2 * ng);
    // the graph of group g: `steps` steps (1 or check_interval) from parity par
    auto graph = [&](int g, int par, bool chained, const StepGraph** out) -> c3l_status {
        StepGraph& sg = chained ? interval[2 * g + par] : one[2 * g + par];
        if (!sg.captured()) {
            const int steps = chained ? check_interval : 1;
            c3l_status r = sg.capture(cap.s, [&](cudaStream_t cs) -> c3l_status {
                for (int i = 0; i < steps; ++i) {
                    const c3l_status q = step(gsteps[g], cs, (par + i) & 1);
                    if (q) return q;
                }
                return C3L_OK;
            });
            if (r) return r;
        }
        *out = &sg;
        return C3L_OK;
    };
    std::vector<int> active(nch, 1);
    for (int c = 0; c < nch; ++c) {
        c3l_arnoldi_channel& q = ch[c];
        cudaStream_t s = chan_stream(c);
        void* sv = reinterpret_cast<void*>(s);
        q.m = 0;
        q.breakdown = 0;
        q.converged = 0;
        q.nchecks = 0;
        q.action_seconds = 0.0;
        q.launches = 0;
        if ((st = c3l_multi_dot_c(q.b, N, 1, q.b, N, q.partial, q.coeff, sv))) return st;
        if ((st = d2h(q.host, q.coeff, sizeof(c3l_complex), s))) return st;
        q.beta = std::sqrt(std::max(q.host[0].re, 0.0));
        if (!(q.beta > 0.0) || !std::isfinite(q.beta)) return C3L_ERR_ARGUMENT;
        if ((st = c3l_scale_c(N, c3l_complex{1.0 / q.beta, 0.0}, q.b, q.V, sv))) return st;
        if ((st = c3l::split_c(N, q.V, q.V32, q.V32lo, s))) return st;
        if ((st = c3l_scale_c(N, c3l_complex{1.0 / q.beta, 0.0}, q.b, q.work, sv))) return st;
        if (gsteps[group_of[c]].fused_scatter) {  // the first sigma's padded input (zero entries included)
            const c3l_action& a = q.sigma->action;
            if ((st = c3l_scatter_padded(a.scatter_count, a.scatter_dst, a.scatter_pos, a.scatter_sign, q.work, a.ws,
                                         sv)))
                return st;
            q.launches += 1;
        }
        if (cudaMemsetAsync(q.counters, 0, 4 * sizeof(int32_t), s) != cudaSuccess) return C3L_ERR_LAUNCH;
        q.launches += (N > 8192 ? 2 : 1) + 3;
        q.hess.shifts = shifts;
        q.hess.beta = q.beta;
        q.hess.breakdown_tol = breakdown_tol;
        q.hess.done = 0;
        if (!q.sink_conj) q.hess.sinkproj_conj = nullptr;
    }
    // Checks: the sink projections of the new rows on each channel's stream,
    // then, on a check stream of the driver's own, one launch advancing the
    // shifted solves of every checked channel and the read-back of each
    // status word (worst residual, first breakdown column, non-finite flag).
    // While a check runs, the channels already take their next steps: a
    // channel that the check stops keeps the dimension checked, and the steps
    // taken beyond it are discarded (they write only basis rows and Hessenberg
    // columns past that dimension).
    OwnedEvents ready;
    if ((st = ready.create(nch))) return st;
    OwnedStream chk;
    if ((st = chk.create())) return st;
    auto enqueue_check = [&](const std::vector<int>& which, int upto) -> c3l_status {
        c3l_status r;
        std::vector<c3l_hessenberg_state*> states;
        std::vector<const c3l_complex*> hcs;
        std::vector<int64_t> lds;
        std::vector<int32_t> ms;
        for (int c : which) {
            c3l_arnoldi_channel& q = ch[c];
            const int done = q.hess.done;
            if (q.sink_conj && upto > done) {
                c3l_complex* out = const_cast<c3l_complex*>(q.hess.sinkproj_conj) + done;
                if ((r = c3l_multi_dot_c(q.V + (int64_t)done * N, N, upto - done, q.sink_conj, N, q.partial, out,
                                         reinterpret_cast<void*>(chan_stream(c)))))
                    return r;
                q.launches += N > 8192 ? 2 : 1;
            }
            if (cudaEventRecord(ready.ev[c], chan_stream(c)) != cudaSuccess ||
                cudaStreamWaitEvent(chk.s, ready.ev[c], 0) != cudaSuccess)
                return C3L_ERR_LAUNCH;
            states.push_back(&q.hess);
            hcs.push_back(q.Hcol);
            lds.push_back(ldc);
            ms.push_back(upto);
        }
        if ((r = c3l::hessenberg_advance_many(states.data(), hcs.data(), lds.data(), ms.data(), (int)which.size(),
                                              chk.s)))
            return r;
        ch[which.front()].launches += 1;
        for (int c : which)
            if (cudaMemcpyAsync(ch[c].status_host, ch[c].hess.status, sizeof(c3l_hessenberg_status),
                                cudaMemcpyDeviceToHost, chk.s) != cudaSuccess)
                return C3L_ERR_LAUNCH;
        return C3L_OK;
    };
    auto settle = [&](c3l_arnoldi_channel& q, int first_break, double worst) {
        if (first_break >= 0) {
            q.m = first_break + 1;
            q.breakdown = 1;
        }
        q.converged = worst <= tol ? 1 : 0;
    };
    auto due = [&](int k) { return k >= min_dim && (k % check_interval == 0 || k == m_max); };
    auto next_due = [&](int k) {
        int t = k + 1;
        while (!due(t)) ++t;  // terminates: due(m_max) holds
        return t;
    };
    // every group with an active channel takes the steps launched .. upto
    int launched = 0;
    auto launch_to = [&](int upto) -> c3l_status {
        for (int gi = 0; gi < ng; ++gi) {
            bool any = false;
            for (int c : groups[gi]) any = any || active[c];
            if (!any) continue;
            c3l_arnoldi_channel& q = ch[groups[gi].front()];  // launches counted once per group
            cudaStream_t s = chan_stream(groups[gi].front());
            int left = upto - launched;
            int at = launched;  // steps taken so far: the parity of the next step
            while (left >= check_interval) {
                const StepGraph* g = nullptr;
                c3l_status r = graph(gi, at & 1, true, &g);
                if (r || (r = g->launch(s))) return r;
                q.launches += g->nodes();
                left -= check_interval;
                at += check_interval;
            }
            for (; left > 0; --left, ++at) {
                const StepGraph* g = nullptr;
                c3l_status r = graph(gi, at & 1, false, &g);
                if (r || (r = g->launch(s))) return r;
                q.launches += g->nodes();
            }
        }
        launched = upto;
        return C3L_OK;
    };
    int remaining = nch;
    if ((st = launch_to(next_due(0)))) return st;
    while (remaining > 0) {
        const int target = launched;  // dimension of this check
        std::vector<int> which;
        for (int c = 0; c < nch; ++c)
            if (active[c]) which.push_back(c);
        for (size_t b0 = 0; b0 < which.size(); b0 += 16) {  // at most 16 channels per launch
            std::vector<int> part(which.begin() + b0, which.begin() + std::min(which.size(), b0 + 16));
            if ((st = enqueue_check(part, target))) return st;
        }
        if (target < m_max && (st = launch_to(next_due(target)))) return st;
        if (cudaStreamSynchronize(chk.s) != cudaSuccess) return C3L_ERR_LAUNCH;
        bool bad = false;
        for (int c : which) {
            c3l_arnoldi_channel& q = ch[c];
            const c3l_hessenberg_status hs = *q.status_host;
            bad = bad || hs.bad != 0;
            double worst;
            unsigned long long bits = hs.worst;
            std::memcpy(&worst, &bits, sizeof(double));
            const int first_break = hs.first_break - 1;
            if (q.check_dims && q.nchecks < q.check_capacity) {
                q.check_dims[q.nchecks] = first_break >= 0 ? first_break + 1 : target;
                q.check_res[q.nchecks] = worst;
            }
            q.nchecks += 1;
            q.m = target;
            if (first_break >= 0 || worst <= tol || target == m_max) {
                settle(q, first_break, worst);
                active[c] = 0;
                remaining -= 1;
                // later steps of the group skip this channel
                if (cudaMemsetAsync(q.counters + 3, 1, 1, chan_stream(c)) != cudaSuccess) return C3L_ERR_LAUNCH;
            }
        }
        if (bad) {  // non-finite Arnoldi step: let the steps in flight finish first
            for (int c = 0; c < nch; ++c) cudaStreamSynchronize(chan_stream(c));
            return C3L_ERR_ARGUMENT;
        }
    }
    // host copy of H[:m+1, :m] (row-major, leading dimension m_max)
    for (int c = 0; c < nch; ++c) {
        c3l_arnoldi_channel& q = ch[c];
        if (!q.H || q.m <= 0) continue;
        cudaStream_t s = chan_stream(c);
        const int m = q.m;
        std::vector<c3l_complex> cols((size_t)m * (m + 1));
        if (cudaMemcpy2DAsync(cols.data(), (m + 1) * sizeof(c3l_complex), q.Hcol, ldc * sizeof(c3l_complex),
                              (m + 1) * sizeof(c3l_complex), m, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return C3L_ERR_LAUNCH;
        for (int jj = 0; jj < m; ++jj)
            for (int i = 0; i <= jj + 1 && i <= m; ++i) q.H[(int64_t)i * m_max + jj] = cols[(size_t)jj * (m + 1) + i];
    }
    return C3L_OK;
}

}  // extern "C"

// Host drivers of the Krylov solvers (C++ over the library's kernels).
//
// c3l_gmres   -- left-preconditioned restarted GMRES with SciPy's control flow
//                (the solver the reference calls for Newton corrections,
//                src/c3l/cc/component_solver.py:181), the operator being the
//                device JVP action.  Each inner iteration enqueues the JVP, the
//                preconditioner and a CGS2 pass (projections fused with the
//                norm), then reads back O(k) scalars in one pinned copy.
// c3l_arnoldi -- CGS2 Arnoldi of src/c3l/green/krylov.py:284-417 for several
//                independent channels at once: each channel runs on its own
//                stream and workspace, so the channels' kernels overlap on the
//                GPU while the host handles one channel's scalars.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "c3l_gb300.h"

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

}  // namespace

extern "C" {

c3l_status c3l_gmres(c3l_gmres_args* a, void* stream) {
    if (!a || !a->jvp || !a->b || !a->x || !a->V || !a->tmp || !a->r || !a->coeff || !a->partial || !a->host ||
        !a->pc_m4 || !a->pc_col || !a->pc_pair || a->dim <= 0 || a->restart <= 0 || a->maxiter <= 0)
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
    auto matvec = [&](const double* in, double* out) -> c3l_status {
        a->matvecs += 1;
        return a->use_f32 ? c3l_static_apply_f32(a->jvp, in, out, stream) : c3l_static_apply(a->jvp, in, out, stream);
    };
    auto psolve = [&](const double* in, double* out) -> c3l_status {
        return c3l_precondition(a->nrep, a->pc_m4, a->pc_col, a->pc_pair, in, out, stream);
    };
    auto norm = [&](const double* v, double& out) -> c3l_status {
        c3l_status q = c3l_multi_dot_r(v, n, 1, v, n, a->partial, coeff, stream);
        if (q) return q;
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
    for (int iteration = 0; iteration < a->maxiter; ++iteration) {
        if (iteration == 0 && bnrm2 < atol) return C3L_OK;
        if ((st = psolve(a->r, V))) return st;
        double beta;
        if ((st = norm(V, beta))) return st;
        if ((st = c3l_scale_r(n, 1.0 / beta, V, V, stream))) return st;
        std::fill(S.begin(), S.end(), 0.0);
        std::fill(h.begin(), h.end(), 0.0);
        S[0] = beta;
        bool breakdown = false;
        int col = 0;
        for (col = 0; col < restart; ++col) {
            double* w = V + (int64_t)(col + 1) * n;
            if ((st = matvec(V + (int64_t)col * n, a->tmp))) return st;
            if ((st = psolve(a->tmp, w))) return st;
            const int k = col + 1;
            // pass 1: [V_0..V_col, w]^T w -> c1 and |w|^2 (w is the row after V_col)
            if ((st = c3l_multi_dot_r(V, n, k + 1, w, n, a->partial, coeff, stream))) return st;
            if ((st = c3l_multi_axpy_r(V, n, k, coeff, -1.0, w, n, stream))) return st;
            // pass 2: c2 and |w'|^2 ; |w''|^2 = |w'|^2 - |c2|^2 (w'' = w' - V c2, V orthonormal)
            if ((st = c3l_multi_dot_r(V, n, k + 1, w, n, a->partial, coeff + k + 1, stream))) return st;
            if ((st = c3l_multi_axpy_r(V, n, k, coeff + k + 1, -1.0, w, n, stream))) return st;
            if ((st = d2h(host, coeff, 2 * (k + 1) * sizeof(double), s))) return st;
            const double h0 = std::sqrt(std::max(host[k], 0.0));
            double c2sq = 0.0;
            for (int j = 0; j < k; ++j) c2sq += host[k + 1 + j] * host[k + 1 + j];
            const double h1 = std::sqrt(std::max(host[2 * k + 1] - c2sq, 0.0));
            for (int j = 0; j < k; ++j) H(col, j) = host[j] + host[k + 1 + j];
            H(col, col + 1) = h1;
            if (h1 <= eps * h0) {
                H(col, col + 1) = 0.0;
                breakdown = true;
            } else if ((st = c3l_scale_r(n, 1.0 / h1, w, w, stream))) {
                return st;
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
        if ((st = c3l_multi_axpy_r(V, n, col + 1, coeff, 1.0, a->x, n, stream))) return st;
        if ((st = matvec(a->x, a->tmp))) return st;
        if (cudaMemcpyAsync(a->r, a->b, n * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess) return C3L_ERR_LAUNCH;
        if ((st = c3l_multi_axpy_r(a->tmp, n, 1, ones, -1.0, a->r, n, stream))) return st;
        if ((st = norm(a->r, rnorm))) return st;
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
        if (!q.sigma || !q.b || !q.V || !q.Hcol || !q.coeff || !q.partial || !q.host || !q.H || !q.Hdev ||
            !q.resid_dev || !q.resid_host)
            return C3L_ERR_ARGUMENT;
    }
    const int64_t ldc = (int64_t)m_max + 1;
    c3l_status st;
    std::vector<int> active(nch, 1), synced(nch, 0);
    for (int c = 0; c < nch; ++c) {
        c3l_arnoldi_channel& q = ch[c];
        cudaStream_t s = as_stream(streams[c]);
        q.m = 0;
        q.breakdown = 0;
        q.converged = 0;
        q.nchecks = 0;
        q.action_seconds = 0.0;
        if ((st = c3l_multi_dot_c(q.b, N, 1, q.b, N, q.partial, q.coeff, streams[c]))) return st;
        if ((st = d2h(q.host, q.coeff, sizeof(c3l_complex), s))) return st;
        q.beta = std::sqrt(std::max(q.host[0].re, 0.0));
        if (!(q.beta > 0.0) || !std::isfinite(q.beta)) return C3L_ERR_ARGUMENT;
        if ((st = c3l_scale_c(N, c3l_complex{1.0 / q.beta, 0.0}, q.b, q.V, streams[c]))) return st;
    }
    // copy device columns [synced, upto) of H into the host row-major matrix and
    // scan them for breakdown / non-finite values; returns the first bad column
    auto pull = [&](c3l_arnoldi_channel& q, int c, int upto, int& first_break, bool& bad) -> c3l_status {
        cudaStream_t s = as_stream(streams[c]);
        const int j0 = synced[c];
        first_break = -1;
        bad = false;
        if (upto <= j0) return C3L_OK;
        std::vector<c3l_complex> cols((size_t)(upto - j0) * ldc);
        if (cudaMemcpyAsync(cols.data(), q.Hcol + (int64_t)j0 * ldc, cols.size() * sizeof(c3l_complex),
                            cudaMemcpyDeviceToHost, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
            return C3L_ERR_LAUNCH;
        for (int j = j0; j < upto; ++j) {
            const c3l_complex* col = cols.data() + (size_t)(j - j0) * ldc;
            for (int i = 0; i <= j + 1; ++i) {
                if (!std::isfinite(col[i].re) || !std::isfinite(col[i].im)) bad = true;
                q.H[(int64_t)i * m_max + j] = col[i];
            }
            if (first_break < 0 && std::fabs(col[j + 1].re) <= breakdown_tol) first_break = j;
        }
        synced[c] = upto;
        return C3L_OK;
    };
    auto check = [&](c3l_arnoldi_channel& q, int c, int m, bool fp64, double& worst) -> c3l_status {
        void* stream = streams[c];
        cudaStream_t s = as_stream(stream);
        // H[:m+1, :m] from the host matrix (row pitch m_max) into a dense device copy (ld = m)
        if (cudaMemcpy2DAsync(q.Hdev, m * sizeof(c3l_complex), q.H, m_max * sizeof(c3l_complex),
                              m * sizeof(c3l_complex), m + 1, cudaMemcpyHostToDevice, s) != cudaSuccess)
            return C3L_ERR_LAUNCH;
        c3l_status r = fp64 ? c3l_hessenberg_shifted(q.Hdev, m, m, shifts, nshift, q.beta, nullptr, nullptr,
                                                      q.resid_dev, stream)
                            : c3l_hessenberg_residual_f32(q.Hdev, m, m, shifts, nshift, q.beta, q.resid_dev, stream);
        if (r) return r;
        if ((r = d2h(q.resid_host, q.resid_dev, nshift * sizeof(double), s))) return r;
        worst = 0.0;
        for (int i = 0; i < nshift; ++i) worst = std::max(worst, q.resid_host[i]);
        if (q.check_dims && q.nchecks < q.check_capacity) {
            q.check_dims[q.nchecks] = m;
            q.check_res[q.nchecks] = worst;
        }
        q.nchecks += 1;
        return C3L_OK;
    };
    int remaining = nch;
    for (int j = 0; j < m_max && remaining > 0; ++j) {
        const int k = j + 1;
        const bool due = k >= min_dim && (k % check_interval == 0 || k == m_max);
        for (int c = 0; c < nch; ++c) {
            if (!active[c]) continue;
            c3l_arnoldi_channel& q = ch[c];
            c3l_complex* w = q.V + (int64_t)k * N;
            if ((st = c3l_eom_sigma(q.sigma, q.V + (int64_t)j * N, w, streams[c]))) return st;
            if ((st = c3l_multi_dot_c(q.V, N, k, w, N, q.partial, q.coeff, streams[c]))) return st;
            if ((st = c3l_multi_axpy_c(q.V, N, k, q.coeff, c3l_complex{-1.0, 0.0}, w, N, streams[c]))) return st;
            // pass 2 with the squared norm of the pass-1 vector (last entry)
            if ((st = c3l_multi_dot_c(q.V, N, k + 1, w, N, q.partial, q.coeff + k, streams[c]))) return st;
            if ((st = c3l_multi_axpy_c(q.V, N, k, q.coeff + k, c3l_complex{-1.0, 0.0}, w, N, streams[c]))) return st;
            if ((st = c3l_arnoldi_column(q.coeff, k, w, N, q.Hcol, ldc, j, breakdown_tol, streams[c]))) return st;
            q.m = k;
        }
        if (!due) continue;
        for (int c = 0; c < nch; ++c) {
            if (!active[c]) continue;
            c3l_arnoldi_channel& q = ch[c];
            int first_break;
            bool bad;
            if ((st = pull(q, c, k, first_break, bad))) return st;
            if (bad) return C3L_ERR_ARGUMENT;  // non-finite Arnoldi step
            if (first_break >= 0) {
                q.m = first_break + 1;
                q.breakdown = 1;
                active[c] = 0;
                remaining -= 1;
                continue;
            }
            double worst;
            if ((st = check(q, c, k, false, worst))) return st;
            if (worst <= tol) {
                if ((st = check(q, c, k, true, worst))) return st;
                if (worst <= tol) {
                    q.converged = 1;
                    active[c] = 0;
                    remaining -= 1;
                }
            }
        }
    }
    // channels that stopped on breakdown or at m_max: pull the rest and check in FP64
    for (int c = 0; c < nch; ++c) {
        c3l_arnoldi_channel& q = ch[c];
        if (q.converged) continue;
        int first_break;
        bool bad;
        if ((st = pull(q, c, q.m, first_break, bad))) return st;
        if (bad) return C3L_ERR_ARGUMENT;
        if (first_break >= 0) {
            q.m = first_break + 1;
            q.breakdown = 1;
        }
        double worst;
        if ((st = check(q, c, q.m, true, worst))) return st;
        q.converged = worst <= tol ? 1 : 0;
    }
    return C3L_OK;
}

}  // extern "C"

"""GPU parity: device actions and solvers against the reference's golden vectors.

Every call goes through ``libc3l_gb300.so``.  Tolerances: actions at fixed
inputs 1e-12 relative (FP64 reassociation only); converged amplitudes and
G^R 1e-8 relative with the residual at or below 1e-10 (the bar of the
reference's own CPU/device parity tests, tests/cc/test_component_jax.py).
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN, eom_amplitudes, golden_names, load, relerr

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def problems(cuda_device):
    import c3lindblad_gb300 as c3

    cache = {}

    def get(name):
        if name not in cache:
            spec, g = load(name)
            cache[name] = (spec, g, c3.ComponentStaticProblem.compile(spec, device=cuda_device))
        return cache[name]

    return get


def _packed(plan, vec):
    t = plan.tilde
    x = np.empty(plan.num_variables)
    x[t.rep_col] = (vec[t.rep_pos] * t.rep_scale).real
    pr = t.rep_pair == 1
    x[t.rep_col[pr] + 1] = vec[t.rep_pos[pr]].imag
    return x


@pytest.mark.parametrize("name", golden_names())
def test_device_real_residual_linearization_and_jvp(name, problems, cuda_device):
    spec, g, p = problems(name)
    ops = p.ops
    x = torch.from_numpy(g["fixed_variables"]).to(cuda_device)
    d = torch.from_numpy(g["fixed_direction_variables"]).to(cuda_device)
    r = torch.empty_like(x)
    ops.residual(x, r)
    assert relerr(r.cpu().numpy(), _packed(p.plan, g["residual"])) < 1e-12
    assert abs(ops.reference_value() - g["residual_reference"]) < 1e-12 * max(1.0, abs(g["residual_reference"]))
    ops.linearize(x, r)
    assert relerr(r.cpu().numpy(), _packed(p.plan, g["residual"])) < 1e-12
    j = torch.empty_like(x)
    ops.jvp(d, j)
    assert relerr(j.cpu().numpy(), _packed(p.plan, g["jvp"])) < 1e-12
    # a residual at another point must not disturb the cached linearization
    ops.residual(torch.zeros_like(x), r)
    ops.jvp(d, j)
    assert relerr(j.cpu().numpy(), _packed(p.plan, g["jvp"])) < 1e-12


@pytest.mark.parametrize("name", golden_names())
def test_component_static_residual_and_jvp_complex(name, problems):
    import c3lindblad_gb300 as c3

    spec, g, p = problems(name)
    res = c3.component_static_residual(p, g["fixed_amplitudes"])
    assert relerr(res.retained, g["residual"]) < 1e-12
    assert abs(res.reference - g["residual_reference"]) < 1e-12 * max(1.0, abs(g["residual_reference"]))
    jvp = c3.component_static_jvp(p, g["fixed_amplitudes"], g["fixed_direction"])
    assert relerr(jvp.retained, g["jvp"]) < 1e-12


def test_complex_residual_accepts_non_tilde_amplitudes(problems):
    """Arbitrary complex amplitudes (outside the tilde subspace) match the oracle."""
    import c3lindblad_gb300 as c3
    from oracle import component_oracle as oc

    spec, g, p = problems("readme")
    rng = np.random.default_rng(7)
    t = 1e-2 * (rng.normal(size=p.num_amplitudes) + 1j * rng.normal(size=p.num_amplitudes))
    v = rng.normal(size=p.num_amplitudes) + 1j * rng.normal(size=p.num_amplitudes)
    o = oc.OracleProblem(spec.as_dict())
    assert relerr(c3.component_static_residual(p, t).retained, o.residual(t)[0]) < 1e-12
    assert relerr(c3.component_static_jvp(p, t, v).retained, o.jvp(t, v)[0]) < 1e-12


@pytest.mark.parametrize("name", golden_names(with_eom=True))
@pytest.mark.parametrize("charge", [1, -1])
def test_device_sigma_and_sources(name, charge, problems):
    import c3lindblad_gb300 as c3

    spec, g, p = problems(name)
    tag = "p" if charge == 1 else "m"
    eom = c3.eom_ccsd_problem(p)
    ep = c3.ComponentEOMProblem.compile(eom, p, charge)
    ctx = c3.component_eom_context(ep, eom_amplitudes(g))
    op = c3.ComponentSigmaOperator(ctx)
    assert op.dimension == g[f"eom{tag}_probe"].size
    assert relerr(op.diagonal, g[f"eom{tag}_diagonal"]) < 1e-14
    assert relerr(op.matvec(g[f"eom{tag}_probe"]), g[f"eom{tag}_sigma"]) < 1e-12
    src = c3.component_eom_sources(ctx)
    assert np.max(np.abs(src.addition - g[f"eom{tag}_addition"])) < 1e-12
    assert np.max(np.abs(src.removal - g[f"eom{tag}_removal"])) < 1e-12
    assert np.max(np.abs(src.sink - g[f"eom{tag}_sink"])) < 1e-14


@pytest.mark.parametrize("name", golden_names(with_solution=True))
def test_newton_krylov_solution_matches_reference(name, problems):
    import c3lindblad_gb300 as c3

    spec, g, p = problems(name)
    sol = c3.solve_component_ccsd(p)
    assert sol.converged
    assert sol.packed_residual_norm <= 1e-10
    assert relerr(sol.amplitudes, g["solution_amplitudes"]) < 1e-8
    assert sol.gpu_launches > 0
    # warm restart from the converged amplitudes converges immediately
    again = c3.solve_component_ccsd(p, sol.amplitudes)
    assert again.converged and again.iterations == 0


@pytest.mark.parametrize("name", golden_names(with_green=True))
def test_retarded_green_matches_reference(name, problems):
    import c3lindblad_gb300 as c3

    spec, g, p = problems(name)
    if "green_retarded" not in g:
        pytest.skip("no reference G^R for this fixture")
    ep = c3.ComponentEOMProblem.compile(c3.eom_ccsd_problem(p), p, 1)
    ctx = c3.component_eom_context(ep, g["solution_amplitudes"])
    op = c3.ComponentSigmaOperator(ctx)
    src = c3.component_eom_sources(ctx)
    res = c3.component_retarded_green(op, src, g["green_omega"], float(g["green_eta"]))
    assert relerr(res.retarded, g["green_retarded"]) < 1e-8
    assert relerr(res.addition, g["green_addition"]) < 1e-8
    assert np.max(res.addition_relative_residuals) <= 1e-10
    assert np.max(res.removal_relative_residuals) <= 1e-10
    # lazily reconstructed solution vectors satisfy (zI - A) x = b
    s = res.addition_solutions[0]
    z = complex(g["green_omega"][0], float(g["green_eta"]))
    x = s.solution
    resid = src.addition - (z * x - op.matvec(x))
    assert np.linalg.norm(resid) / np.linalg.norm(src.addition) < 1e-8


def test_shifted_gmres_matches_dense_solve(problems):
    """solve_component_shifted (component_response.py:72-128) against a dense
    solve of (z - K) x = b, from zero and from an initial solution."""
    import c3lindblad_gb300 as c3

    spec, g, p = problems("readme")
    ep = c3.ComponentEOMProblem.compile(c3.eom_ccsd_problem(p), p, 1)
    ctx = c3.component_eom_context(ep, g["solution_amplitudes"])
    op = c3.ComponentSigmaOperator(ctx)
    n = op.dimension
    K = np.stack([op.matvec(np.eye(n, dtype=np.complex128)[j]) for j in range(n)], axis=1)
    src = c3.component_eom_sources(ctx)
    b = np.concatenate([src.addition, np.zeros(n - src.addition.size)])
    for z in (0.3 + 0.05j, -1.7 + 0.0j):
        want = np.linalg.solve(z * np.eye(n) - K, b)
        res = c3.solve_component_shifted(op, z, b)
        assert res.converged and res.info == 0
        assert res.true_relative_residual <= 1e-9
        assert res.iterations == len(res.residual_history) > 0
        assert relerr(res.solution, want) < 1e-8
        again = c3.solve_component_shifted(op, z, b, initial_solution=res.solution)
        assert again.converged and again.iterations <= 2
    with pytest.raises(ValueError):
        c3.solve_component_shifted(op, 0.1, b[:-1])


@pytest.mark.parametrize("name", ["readme", "siam10"])
def test_per_frequency_gmres_green_matches_reference(name, problems):
    """The reference's own per-frequency algorithm (method="gmres") on the device."""
    import c3lindblad_gb300 as c3

    spec, g, p = problems(name)
    ep = c3.ComponentEOMProblem.compile(c3.eom_ccsd_problem(p), p, 1)
    ctx = c3.component_eom_context(ep, g["solution_amplitudes"])
    op = c3.ComponentSigmaOperator(ctx)
    src = c3.component_eom_sources(ctx)
    res = c3.component_retarded_green(op, src, g["green_omega"], float(g["green_eta"]), method="gmres")
    assert relerr(res.retarded, g["green_retarded"]) < 1e-8
    assert all(r.converged for r in res.addition_solutions + res.removal_solutions)
    assert res.component_action_calls > 0


def test_matrix_green_arnoldi_matches_reference(problems):
    """G^R_ab for the three impurity orbitals of the n = 9 Kanamori fixture
    (charge +1, fixed amplitudes) against the reference's one-sided matrix
    Arnoldi driver; all six channels run concurrently."""
    import c3lindblad_gb300 as c3
    from conftest import GOLDEN

    spec, g, p = problems("kanamori3x2")
    ref = np.load(GOLDEN / "kanamori3x2.matrix.npz")
    ep = c3.ComponentEOMProblem.compile(c3.eom_ccsd_problem(p), p, 1)
    ctx = c3.component_eom_context(ep, eom_amplitudes(g))
    op = c3.ComponentSigmaOperator(ctx)
    sources = [c3.component_eom_sources(ctx, site=int(s)) for s in ref["sites"]]
    res = c3.component_retarded_matrix_green_arnoldi(
        op, sources, ref["omega"], float(ref["eta"]), maximum_krylov_dimension=int(ref["maximum_krylov_dimension"]))
    assert res.sites == tuple(int(s) for s in ref["sites"])
    assert res.addition.shape == ref["addition"].shape
    assert relerr(res.addition, ref["addition"]) < 1e-8
    assert relerr(res.removal, ref["removal"]) < 1e-8
    assert relerr(res.retarded, ref["retarded"]) < 1e-8
    assert np.max(res.addition_relative_residuals) <= 1e-10
    assert np.max(res.removal_relative_residuals) <= 1e-10
    dims = [pr.dimension for pr in res.addition_projections + res.removal_projections]
    want = list(ref["addition_dimensions"]) + list(ref["removal_dimensions"])
    assert all(abs(a - b) <= 8 for a, b in zip(dims, want))
    assert res.component_action_calls == sum(dims)
    # a projection's reduced coordinates reproduce the shifted solve on the host
    pr = res.addition_projections[1]
    z = ref["omega"][:3] + 1j * float(ref["eta"])
    Y = pr.coefficients(z)
    m = pr.dimension
    for i, zi in enumerate(z):
        rhs = np.zeros(m, complex)
        rhs[0] = pr.source_norm
        y = np.linalg.solve(zi * np.eye(m) - pr.hessenberg[:m, :m], rhs)
        assert relerr(Y[i], y) < 1e-9
    # the device basis is orthonormal and satisfies K V_m = V_{m+1} H to FP64
    # rounding (a single FP64 pass where |w'| >= |w| / sqrt(2), the DGKS test,
    # let the orthogonality decay to 1e-8 over this basis)
    for pr in (res.addition_projections[0], res.removal_projections[2]):
        V = pr.basis
        m = pr.dimension
        assert np.max(np.abs(V.conj().T @ V - np.eye(m + 1))) < 1e-12
        KV = np.stack([op.matvec(V[:, j]) for j in range(m)], axis=1)
        assert np.linalg.norm(KV - V @ pr.hessenberg) / np.linalg.norm(pr.hessenberg) < 1e-13
    with pytest.raises(ValueError):
        c3.component_retarded_matrix_green_arnoldi(op, sources, ref["omega"], 0.0)
    with pytest.raises(ValueError):
        c3.component_retarded_matrix_green_arnoldi(op, [sources[0], sources[0]], ref["omega"], 0.1)


@pytest.mark.parametrize("suffix,charge", [("", 1), ("_m", -1)])
def test_matrix_green_arnoldi_large_fixture(suffix, charge, problems):
    """n = 27 Kanamori (the three-orbital, eight-mode model; EOM dimension
    29,187), eta = 0.02: the device matrix response against the reference's
    one-sided matrix Arnoldi driver at the fixture's fixed amplitudes, both
    charges."""
    import c3lindblad_gb300 as c3
    from conftest import GOLDEN

    path = GOLDEN / f"kanamori3x8.matrix{suffix}.npz"
    if not path.exists():
        pytest.skip("matrix golden not generated")
    ref = np.load(path)
    spec, g, p = problems("kanamori3x8")
    T, _ = _fixed_inputs(p.plan, float(g["scale"]))
    ep = c3.ComponentEOMProblem.compile(c3.eom_ccsd_problem(p), p, charge)
    ctx = c3.component_eom_context(ep, T)
    op = c3.ComponentSigmaOperator(ctx)
    sources = [c3.component_eom_sources(ctx, site=int(s)) for s in ref["sites"]]
    res = c3.component_retarded_matrix_green_arnoldi(
        op, sources, ref["omega"], float(ref["eta"]), maximum_krylov_dimension=int(ref["maximum_krylov_dimension"]))
    assert relerr(res.addition, ref["addition"]) < 1e-8
    assert relerr(res.removal, ref["removal"]) < 1e-8
    assert relerr(res.retarded, ref["retarded"]) < 1e-8
    assert np.max(res.addition_relative_residuals) <= 1e-10
    assert np.max(res.removal_relative_residuals) <= 1e-10


def test_krylov_primitives_against_numpy(cuda_device):
    from c3lindblad_gb300.krylov import DeviceVectors, hessenberg_shifted

    rng = np.random.default_rng(11)
    vec = DeviceVectors(cuda_device)
    k, n = 7, 5003
    V = rng.normal(size=(k, n)) + 1j * rng.normal(size=(k, n))
    w = rng.normal(size=n) + 1j * rng.normal(size=n)
    Vd = torch.from_numpy(V).to(cuda_device)
    wd = torch.from_numpy(w).to(cuda_device)
    out = torch.empty(k, dtype=torch.complex128, device=cuda_device)
    vec.dots_c(Vd, k, wd, out)
    assert relerr(out.cpu().numpy(), V.conj() @ w) < 1e-13
    c = rng.normal(size=k) + 1j * rng.normal(size=k)
    vec.axpy_c(Vd, k, torch.from_numpy(c).to(cuda_device), -0.5 + 0.25j, wd)
    assert relerr(wd.cpu().numpy(), w + (-0.5 + 0.25j) * (c @ V)) < 1e-13
    # long basis over a short vector (one block per row; 4 x 64 axpy blocks) and a
    # long vector (two-pass reduction)
    for kk, nn in ((70, 1947), (3, 10007)):
        V2 = rng.normal(size=(kk, nn)) + 1j * rng.normal(size=(kk, nn))
        w2 = rng.normal(size=nn) + 1j * rng.normal(size=nn)
        V2d, w2d = torch.from_numpy(V2).to(cuda_device), torch.from_numpy(w2).to(cuda_device)
        out2 = torch.empty(kk, dtype=torch.complex128, device=cuda_device)
        vec.dots_c(V2d, kk, w2d, out2)
        assert relerr(out2.cpu().numpy(), V2.conj() @ w2) < 1e-13
        c2 = rng.normal(size=kk) + 1j * rng.normal(size=kk)
        vec.axpy_c(V2d, kk, torch.from_numpy(c2).to(cuda_device), 0.75 - 0.5j, w2d)
        assert relerr(w2d.cpu().numpy(), w2 + (0.75 - 0.5j) * (c2 @ V2)) < 1e-13
    Vr = rng.normal(size=(k, n))
    wr = rng.normal(size=n)
    outr = torch.empty(k, dtype=torch.float64, device=cuda_device)
    vec.dots_r(torch.from_numpy(Vr).to(cuda_device), k, torch.from_numpy(wr).to(cuda_device), outr)
    assert relerr(outr.cpu().numpy(), Vr @ wr) < 1e-13
    # shifted Hessenberg solves
    m = 37
    H = np.triu(rng.normal(size=(m + 1, m)) + 1j * rng.normal(size=(m + 1, m)), -1)
    shifts = np.linspace(-3, 3, 23) + 0.1j
    p = rng.normal(size=m) + 1j * rng.normal(size=m)
    green, resid = hessenberg_shifted(H, m, torch.from_numpy(shifts).to(cuda_device), 2.5,
                                      torch.from_numpy(p).to(cuda_device))
    e1 = np.zeros(m, complex)
    e1[0] = 2.5
    ys = [np.linalg.solve(z * np.eye(m) - H[:m, :m], e1) for z in shifts]
    assert relerr(green.cpu().numpy(), np.array([p @ y for y in ys])) < 1e-10
    assert relerr(resid.cpu().numpy(), np.array([abs(H[m, m - 1] * y[-1]) / 2.5 for y in ys])) < 1e-10


def _advance(state, Hc, m_max, m, cuda_device):
    from c3lindblad_gb300 import runtime as rt

    st = rt.lib().c3l_hessenberg_advance(C.byref(state), Hc.data_ptr(), m_max + 1, m,
                                         torch.cuda.current_stream(cuda_device).cuda_stream)
    assert st == 0


def test_incremental_hessenberg_against_numpy(cuda_device):
    """Column-incremental shifted solves agree with dense solves at every stop,
    including stops inside a chunk and a breakdown column."""
    from c3lindblad_gb300 import runtime as rt
    from c3lindblad_gb300.krylov import HessenbergTracker

    rng = np.random.default_rng(5)
    m_max = 53
    H = np.triu(rng.normal(size=(m_max + 1, m_max)) + 1j * rng.normal(size=(m_max + 1, m_max)), -1)
    for j in range(m_max):
        H[j + 1, j] = abs(H[j + 1, j]) + 0.5  # Arnoldi subdiagonals are real and positive
    shifts = np.linspace(-3, 3, 23) + 0.1j
    p = rng.normal(size=m_max) + 1j * rng.normal(size=m_max)
    beta = 2.5
    sd = torch.from_numpy(shifts).to(cuda_device)

    def run(Hm, stops, brk=None):
        Hc = torch.zeros((m_max, m_max + 1), dtype=torch.complex128)
        for j in range(m_max):
            Hc[j, :j + 2] = torch.from_numpy(Hm[:j + 2, j])
        Hc = Hc.to(cuda_device)
        tr = HessenbergTracker(m_max, sd, True)
        tr.sinkproj_conj.copy_(torch.from_numpy(np.conj(p)))
        state = rt.HessenbergState()
        tr.fill(state)
        state.beta, state.breakdown_tol = beta, 1e-14
        for m in stops:
            _advance(state, Hc, m_max, m, cuda_device)
            torch.cuda.synchronize()
            stat = tr.status.cpu().numpy()
            mm = m if brk is None or brk >= m else brk + 1
            assert int(stat[1] & 0xffffffff) == (0 if mm == m else brk + 1)
            e1 = np.zeros(mm, complex)
            e1[0] = beta
            ys = [np.linalg.solve(z * np.eye(mm) - Hm[:mm, :mm], e1) for z in shifts]
            want_g = np.array([p[:mm] @ y for y in ys])
            want_r = np.array([abs(Hm[mm, mm - 1] * y[-1]) / beta for y in ys])
            assert relerr(tr.green.cpu().numpy(), want_g) < 1e-10
            if mm == m:
                assert relerr(tr.residual.cpu().numpy(), want_r) < 1e-10
                assert np.array([stat[0]]).view(np.float64)[0] == pytest.approx(want_r.max(), rel=1e-10)
            else:
                assert np.all(tr.residual.cpu().numpy() <= 1e-12)
            if mm < m:
                return

    run(H, [16, 24, 29, 37, 53])
    run(H, [3, 4, 12, 20, 21, 53])
    Hb = H.copy()
    Hb[31, 30] = 0.0  # breakdown at column 30
    run(Hb, [16, 24, 36, 53], brk=30)


# ------------------------------------------------------------ large fixtures
def _fixed_inputs(plan, scale):
    t = plan.tilde
    idx = np.arange(plan.num_variables, dtype=np.float64)
    x = scale * np.cos(idx + 0.13)
    d = 0.2 * np.sin(idx + 0.31)
    unpack = lambda v: t.coef_a * v[t.idx_a] + t.coef_b * v[t.idx_b]
    return unpack(x), unpack(d)


def _close(got, want, norm, tol):
    return np.linalg.norm(got - want) <= tol * max(np.linalg.norm(want), 1e-300) and \
        np.max(np.abs(got - want)) <= tol * norm


@pytest.mark.parametrize("name", golden_names(compact=True))
def test_large_fixture_residual_jvp_sigma_at_sampled_coordinates(name, problems):
    """n = 27 Kanamori (779,301 amplitudes): reference outputs at 4,096 sampled coordinates."""
    import c3lindblad_gb300 as c3

    spec, g, p = problems(name)
    T, D = _fixed_inputs(p.plan, float(g["scale"]))
    pos = g["sample_positions"]
    res = c3.component_static_residual(p, T)
    assert _close(res.retained[pos], g["residual_sample"], float(g["residual_norm"]), 1e-11)
    assert abs(np.linalg.norm(res.retained) - g["residual_norm"]) <= 1e-11 * g["residual_norm"]
    jvp = c3.component_static_jvp(p, T, D)
    assert _close(jvp.retained[pos], g["jvp_sample"], float(g["jvp_norm"]), 1e-11)
    assert abs(np.linalg.norm(jvp.retained) - g["jvp_norm"]) <= 1e-11 * g["jvp_norm"]
    for charge, tag in ((1, "p"), (-1, "m")):
        if f"eom{tag}_sigma_sample" not in g:
            continue
        ep = c3.ComponentEOMProblem.compile(c3.eom_ccsd_problem(p), p, charge)
        ctx = c3.component_eom_context(ep, T)
        op = c3.ComponentSigmaOperator(ctx)
        assert op.dimension == int(g[f"eom{tag}_dimension"])
        k = np.arange(op.dimension, dtype=np.float64)
        probe = np.cos(0.7 * k + 0.2) + 1j * np.sin(0.3 * k - 0.1)
        sig = op.matvec(probe)
        ep_pos = g[f"eom{tag}_sample_positions"]
        assert _close(sig[ep_pos], g[f"eom{tag}_sigma_sample"], float(g[f"eom{tag}_sigma_norm"]), 1e-11)
        assert abs(np.linalg.norm(sig) - g[f"eom{tag}_sigma_norm"]) <= 1e-11 * g[f"eom{tag}_sigma_norm"]
        src = c3.component_eom_sources(ctx)
        for key, val in (("addition", src.addition), ("removal", src.removal), ("sink", src.sink),
                         ("diagonal", op.diagonal)):
            want = g[f"eom{tag}_{key}_sample"]
            assert np.max(np.abs(val[ep_pos] - want)) <= 1e-12 * max(1.0, np.max(np.abs(want)))


@pytest.mark.parametrize("name", [n for n in golden_names(with_solution=True)])
def test_mixed_precision_solve_meets_fp64_tolerance(name, problems):
    """FP32 inner JVPs with FP64 residuals converge to the FP64 reference root."""
    import c3lindblad_gb300 as c3

    spec, g, p = problems(name)
    sol = c3.solve_component_ccsd(p, precision="mixed")
    assert sol.converged and sol.packed_residual_norm <= 1e-10
    assert relerr(sol.amplitudes, g["solution_amplitudes"]) < 1e-8


@pytest.mark.parametrize("kernel", ["simt", "tcgen05"])
@pytest.mark.parametrize("name", golden_names())
def test_single_precision_jvp_tracks_fp64(name, kernel, cuda_device, monkeypatch):
    """The FP32 JVP (its output stage summed by the pair GEMMs, on the CUDA
    cores or the tcgen05 tensor cores) against the FP64 one."""
    import c3lindblad_gb300 as c3

    monkeypatch.setenv("C3L_PAIR_KERNEL", kernel)
    spec, g = load(name)
    p = c3.ComponentStaticProblem.compile(spec, device=cuda_device)
    ops = p.ops
    x = torch.from_numpy(g["fixed_variables"]).to(cuda_device)
    d = torch.from_numpy(g["fixed_direction_variables"]).to(cuda_device)
    r = torch.empty_like(x)
    ops.linearize(x, r)
    ops.to_single()
    j64 = torch.empty_like(x)
    j32 = torch.empty_like(x)
    ops.jvp(d, j64)
    ops.jvp32(d, j32)
    ops.check_device_status()
    err = relerr(j32.cpu().numpy(), j64.cpu().numpy())
    assert 0 < err < 1e-5


def test_pair_kernel_autotuner_keeps_the_faster_kernel(cuda_device, monkeypatch):
    """C3L_PAIR_KERNEL=auto (the default): the tuner times the FP32 JVP with
    both pair-GEMM kernels, keeps the faster, and the JVP it leaves behind is
    still the FP32 JVP (within FP32 rounding of the FP64 one)."""
    import c3lindblad_gb300 as c3
    from c3lindblad_gb300 import device_ops

    monkeypatch.setenv("C3L_PAIR_KERNEL", "auto")
    spec = c3.ProblemSpec.load(GOLDEN / "kanamori3x8.spec.npz")
    p = c3.ComponentStaticProblem.compile(spec, device=cuda_device)
    ops = p.ops
    idx = torch.arange(p.num_variables, dtype=torch.float64, device=cuda_device)
    x = 1e-3 * torch.cos(idx + 0.13)
    d = 0.2 * torch.sin(idx + 0.31)
    r = torch.empty_like(x)
    ops.linearize(x, r)
    ops.to_single()
    times = ops.tune_pair_kernel()
    assert set(times) == set(device_ops.PAIR_KERNELS) and all(t > 0 for t in times.values())
    assert ops.pair_kernel_name == min(times, key=times.get)
    j64 = torch.empty_like(x)
    j32 = torch.empty_like(x)
    ops.jvp(d, j64)
    ops.jvp32(d, j32)
    ops.check_device_status()
    assert 0 < relerr(j32.cpu().numpy(), j64.cpu().numpy()) < 1e-5


@pytest.mark.parametrize("basis_f32,restart", [(False, 30), (True, 30), (True, 70)])
def test_newton_correction_gmres_fp32_operator(basis_f32, restart, problems, cuda_device):
    """c3l_gmres with the FP32 JVP, with an FP64 or an FP32 Krylov basis: the
    correction meets the requested relative tolerance of the FP64 system
    M J s = -M r (left preconditioned) up to the FP32 operator's accuracy;
    restart 70 takes the FP32 basis past 64 rows."""
    spec, g, p = problems("siam10")
    ops = p.ops
    x = torch.from_numpy(g["fixed_variables"]).to(cuda_device)
    r = torch.empty_like(x)
    ops.linearize(x, r)
    ops.to_single()
    solver = p.gmres_solver(restart)
    s = torch.zeros_like(x)
    rtol = 1e-4
    info, hist, matvecs = solver.solve(-r, s, rtol=rtol, atol=0.0, maxiter=40, single=True, basis_f32=basis_f32)
    assert info == 0 and matvecs > 0 and hist[-1] <= rtol
    js = torch.empty_like(x)
    ops.jvp(s, js)  # FP64 operator
    defect = (js + r).cpu().numpy()
    assert np.linalg.norm(defect) <= 2 * rtol * np.linalg.norm(r.cpu().numpy())


def test_batched_sigma_matches_single_calls(problems, cuda_device):
    """c3l_eom_sigma_batch over three channel workspaces gives, bit for bit,
    the single-vector c3l_eom_sigma of each vector (same kernels, one launch
    per kernel for the batch)."""
    import c3lindblad_gb300 as c3
    from c3lindblad_gb300 import runtime as rt

    spec, g, p = problems("siam10")
    ep = c3.ComponentEOMProblem.compile(c3.eom_ccsd_problem(p), p, 1)
    ctx = c3.component_eom_context(ep, g["solution_amplitudes"])
    ops = ctx.ops
    ops.ensure_channels(3)
    N = ops.N
    rng = np.random.default_rng(3)
    xs = [torch.from_numpy(rng.normal(size=N) + 1j * rng.normal(size=N)).to(cuda_device) for _ in range(3)]
    outs = [torch.empty_like(x) for x in xs]
    acts = (rt.EomAction * 3)(*[ops.sigma_actions[i] for i in range(3)])
    xin = (C.c_void_p * 3)(*[x.data_ptr() for x in xs])
    xo = (C.c_void_p * 3)(*[o.data_ptr() for o in outs])
    lib = rt.lib()
    rt.check(lib.c3l_eom_sigma_batch(acts, 3, xin, xo, rt.stream_ptr(cuda_device)), "sigma batch")
    for x, o in zip(xs, outs):
        want = torch.empty_like(x)
        ops.sigma(x, want)
        assert torch.equal(o, want)
    # workspaces of different programs are refused
    other = c3.ComponentEOMProblem.compile(c3.eom_ccsd_problem(p), p, -1)
    octx = c3.component_eom_context(other, g["solution_amplitudes"])
    mixed = (rt.EomAction * 2)(ops.sigma_actions[0], octx.ops.sigma_action)
    assert lib.c3l_eom_sigma_batch(mixed, 2, xin, xo, rt.stream_ptr(cuda_device)) == 1


@pytest.mark.parametrize("name", golden_names(compact=True))
def test_arnoldi_basis_long_vectors(name, problems, cuda_device):
    """The Arnoldi step at N > 8192 (segmented second projections and their
    final reduction, double-float updates from rows that stream from HBM):
    the device bases of the n = 27 Kanamori charge +1 operator (addition and
    removal channels stepped together) are orthonormal and satisfy
    K V_m = V_{m+1} H to FP64-level rounding."""
    import c3lindblad_gb300 as c3
    from c3lindblad_gb300.krylov import arnoldi_channels

    spec, g, p = problems(name)
    T, _ = _fixed_inputs(p.plan, float(g["scale"]))
    ep = c3.ComponentEOMProblem.compile(c3.eom_ccsd_problem(p), p, 1)
    ctx = c3.component_eom_context(ep, T)
    op = c3.ComponentSigmaOperator(ctx)
    N = op.dimension
    assert N > 8192
    src = c3.component_eom_sources(ctx, site=0)
    vecs = [torch.from_numpy(np.ascontiguousarray(v)).to(cuda_device) for v in (src.addition, src.removal)]
    shifts = torch.tensor([0.1 + 0.5j, -1.0 + 0.5j], dtype=torch.complex128, device=cuda_device)
    m = 48
    bases = arnoldi_channels(ctx.ops, vecs, shifts, maximum_dimension=m, residual_tolerance=1e-30,
                             minimum_dimension=m, check_interval=16)
    for basis in bases:
        assert basis.m == m
        V = basis.V[:m + 1].cpu().numpy().T
        H = basis.H[:m + 1, :m]
        assert np.max(np.abs(V.conj().T @ V - np.eye(m + 1))) < 1e-12
        KV = np.stack([op.matvec(V[:, j]) for j in range(m)], axis=1)
        assert np.linalg.norm(KV - V @ H) / np.linalg.norm(H) < 1e-13


@pytest.mark.parametrize("name", ["twosrc", "siam10"])
def test_response_drivers_match_reference(name, problems):
    """The reference's other response drivers (charge +1, converged amplitudes)
    against its own outputs: the GMRES matrix response (one solve per source,
    channel and frequency), the matrix response at complex shifts (Matsubara
    and real-axis points), the time-domain propagation of one source and the
    time-domain matrix with its separate channels.  Frequency-domain values
    1e-8 relative (the G^R contract); Krylov dimensions within one check
    interval; time-domain values 1e-8 relative where the Krylov basis
    converged.  A basis that stops at the 160-vector cap without meeting the
    time-residual test (the siam10 matrix propagation) is an unconverged
    approximation in both codes: there the two agree to 1e-7 (measured
    1.5e-8), the FP64 rounding of two different orthogonalizations carried
    through an unconverged propagator to t = 20."""
    import c3lindblad_gb300 as c3
    from conftest import GOLDEN

    spec, g, p = problems(name)
    ref = np.load(GOLDEN / f"{name}.drivers.npz")
    ep = c3.ComponentEOMProblem.compile(c3.eom_ccsd_problem(p), p, 1)
    ctx = c3.component_eom_context(ep, eom_amplitudes(g))
    sources = [c3.component_eom_sources(ctx, site=int(s)) for s in ref["sites"]]
    S = len(sources)
    errors = {}

    op = c3.ComponentSigmaOperator(ctx)
    mg = c3.component_retarded_matrix_green(op, sources, ref["gmres_omega"], float(ref["gmres_eta"]))
    assert mg.retarded.shape == (ref["gmres_omega"].size, S, S)
    errors["gmres"] = relerr(mg.retarded, ref["gmres_retarded"])
    errors["gmres_addition"] = relerr(mg.addition, ref["gmres_addition"])
    assert all(r.converged for rows in mg.addition_solutions + mg.removal_solutions for r in rows)
    assert mg.addition_solutions[0][0].solution.shape == (op.dimension,)

    op = c3.ComponentSigmaOperator(ctx)
    sh = c3.component_retarded_matrix_green_shifts(op, sources, ref["shifts"])
    errors["shifts"] = relerr(sh.retarded, ref["shifts_retarded"])
    errors["shifts_removal"] = relerr(sh.removal, ref["shifts_removal"])
    dims = [pr.dimension for pr in sh.addition_projections + sh.removal_projections]
    want = list(ref["shifts_addition_dimensions"]) + list(ref["shifts_removal_dimensions"])
    assert all(abs(a - b) <= 8 for a, b in zip(dims, want)), (dims, want)
    assert sh.action_calls == sum(dims) == op.action_calls
    assert np.max(sh.addition_relative_residuals) <= 1e-10

    op = c3.ComponentSigmaOperator(ctx)
    tr = c3.component_retarded_time(op, sources[0], ref["time"])
    errors["time"] = relerr(tr, ref["time_retarded"])
    assert abs(op.action_calls - int(ref["time_calls"])) <= 8

    op = c3.ComponentSigmaOperator(ctx)
    mt = c3.component_retarded_matrix_time(op, sources, ref["time"], ref["validation_shifts"])
    errors["matrix_time"] = relerr(mt.retarded, ref["mtime_retarded"])
    errors["matrix_time_addition"] = relerr(mt.addition, ref["mtime_addition"])
    assert [pr.dimension for pr in mt.combined_projections] == list(ref["mtime_combined_dimensions"]) or all(
        abs(a - b) <= 8 for a, b in zip([pr.dimension for pr in mt.combined_projections],
                                        ref["mtime_combined_dimensions"]))
    assert mt.combined_relative_time_residuals.shape == (S, ref["time"].size)
    assert mt.channel_sum_defect <= max(10 * float(ref["mtime_channel_sum_defect"]), 1e-12)
    print(name, {k: f"{v:.2e}" for k, v in errors.items()})
    for k in ("gmres", "gmres_addition", "shifts", "shifts_removal"):
        assert errors[k] < 1e-8, (k, errors[k])
    assert errors["time"] < 1e-8, errors["time"]
    capped = max(pr.dimension for pr in mt.combined_projections) >= 160
    for k in ("matrix_time", "matrix_time_addition"):
        assert errors[k] < (1e-7 if capped else 1e-8), (k, errors[k], capped)
    # the Matsubara grid form (the complex-shift driver at i|omega_n|)
    op = c3.ComponentSigmaOperator(ctx)
    grid = c3.matsubara_grid(float(ref["matsubara_beta"]), indices=ref["matsubara_indices"])
    mats = c3.component_matsubara_green(op, sources, grid)
    assert mats.green.shape == ref["matsubara_green"].shape
    assert relerr(mats.green, ref["matsubara_green"]) < 1e-8
    assert mats.max_relative_residual <= 1e-10
    # the projection's transfer and orthogonality diagnostics
    pr = sh.addition_projections[0]
    sink = np.concatenate([sources[0].sink, np.zeros(op.dimension - sources[0].sink.size, complex)])
    assert relerr(pr.transfer(ref["shifts"][:4], sink), sh.addition[:4, 0, 0]) < 1e-10
    assert pr.orthogonality_defect < 1e-12
    assert pr.to_dict()["krylov_dimension"] == pr.dimension


def test_exact_diagonalisation_check_readme(problems):
    """The exact-diagonalisation check of the tiny README model
    (examples/basic/01_ccsd_eom.py of the reference): the device CCSD-EOM G^R
    matches the reference's CC values to 1e-8 and so differs from the exact
    Lindblad ED G^R by the reference's own CCSD truncation error."""
    import c3lindblad_gb300 as c3
    from conftest import GOLDEN

    spec, g, p = problems("readme")
    ed = np.load(GOLDEN / "readme.ed.npz")
    sol = c3.solve_component_ccsd(p)
    assert sol.converged
    ep = c3.ComponentEOMProblem.compile(c3.eom_ccsd_problem(p), p, 1)
    ctx = c3.component_eom_context(ep, sol.amplitudes)
    res = c3.component_retarded_green(c3.ComponentSigmaOperator(ctx), c3.component_eom_sources(ctx), ed["omega"],
                                      float(ed["eta"]))
    assert relerr(res.retarded, ed["green_cc_reference"]) < 1e-8
    assert abs(relerr(res.retarded, ed["green_ed"]) - float(ed["cc_vs_ed_relative"])) <= 1e-7


@pytest.mark.parametrize("name", ["readme", "twosrc", "kanamori3x2"])
def test_interaction_scale_is_the_homotopy_model(name, problems, cuda_device):
    """Residual, JVP and EOM sigma with the product part scaled by s equal the
    oracle's on the spec with every product coefficient times s (the
    reference's homotopy model at one HF reference)."""
    import dataclasses

    import c3lindblad_gb300 as c3
    from oracle import component_oracle as oc

    spec, g, p = problems(name)
    s = 0.6
    orc = oc.OracleProblem(dataclasses.replace(spec, product_coefficients=spec.product_coefficients * s).as_dict())
    T = orc.tilde.unpack(g["fixed_variables"])
    D = orc.tilde.unpack(g["fixed_direction_variables"])
    ops = p.ops
    x = torch.from_numpy(g["fixed_variables"]).to(cuda_device)
    d = torch.from_numpy(g["fixed_direction_variables"]).to(cuda_device)
    r = torch.empty_like(x)
    j = torch.empty_like(x)
    ops.set_interaction_scale(s)
    try:
        ops.residual(x, r)
        ops.linearize(x, torch.empty_like(x))
        ops.jvp(d, j)
    finally:
        ops.set_interaction_scale(1.0)
    assert relerr(r.cpu().numpy(), _packed(p.plan, orc.residual(T)[0])) < 1e-12
    assert relerr(j.cpu().numpy(), _packed(p.plan, orc.jvp(T, D)[0])) < 1e-12
    ep = c3.ComponentEOMProblem.compile(c3.eom_ccsd_problem(p), p, 1)
    ctx = c3.component_eom_context(ep, T, interaction_scale=s)
    op = c3.ComponentSigmaOperator(ctx)
    k = np.arange(op.dimension, dtype=np.float64)
    probe = np.cos(0.7 * k + 0.2) + 1j * np.sin(0.3 * k - 0.1)
    assert relerr(op.matvec(probe), oc.OracleEOM(orc, T, 0, 1).sigma(probe)) < 1e-12

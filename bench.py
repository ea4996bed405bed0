"""Time-to-solution benchmark of the coupled-cluster hot path on one GB300.

A *step* is the full hot path on one synthetic model: the CCSD steady state
by Newton--Krylov from zero amplitudes, then the charge +1 EOM block of the
impurity (context, sources) and G^R on the whole frequency grid.

Workload (default): the single-impurity Anderson model with 10 Lindblad
pseudomodes (n = 11 sites, 20,933 amplitudes, EOM dimension 1,947), seeded
as described in ``tests/golden/make_fixtures.py`` (``siam10``), with 1001
frequencies in [-8, 8] and eta = 0.  Inputs are synthetic (seeded), not a
dataset.

``value``  -- seconds per step with the problem tables already resident in HBM
              (CUDA events on the launching stream, L2 flushed between steps).
``e2e``    -- the same step through the public API from host buffers: the
              problem tables are uploaded (H2D) and the amplitudes and G^R are
              read back (D2H) inside the timed region.
``--impl reference`` times the CPU restatement of the reference algorithm
(``oracle/``) on the host cores and prints the same metric.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "s to CCSD+G^R(omega) at ≤1e-8 vs FP64: mixed+batched+warm vs plain FP64, 1 GB300"
WORKLOADS = {
    "siam10": dict(spec="siam10", omega=(-8.0, 8.0, 1001), eta=0.0,
                   label="SIAM U=4, 10 pseudomodes (n=11, 20933 amplitudes, S13 dim 1947), "
                         "charge+1 G^R on 1001 omega in [-8,8], eta=0"),
    "readme": dict(spec="readme", omega=(-4.0, 4.0, 81), eta=0.0,
                   label="README quick-start model (n=3, 117 amplitudes, S13 dim 39), "
                         "charge+1 G^R on 81 omega in [-4,4], eta=0"),
}


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _max_over_ranks(value: float, device) -> float:
    """The largest of the ranks' values (every rank receives it): the job's
    step time is its slowest replica's."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _flush_l2(torch, buf):
    buf.add_(1.0)


def run_gpu(args) -> dict:
    import torch

    import c3lindblad_gb300 as c3
    from c3lindblad_gb300 import runtime as rt

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    wl = WORKLOADS[args.workload]
    spec_path = ROOT / "tests" / "golden" / f"{wl['spec']}.spec.npz"
    gold = dict(np.load(ROOT / "tests" / "golden" / f"{wl['spec']}.golden.npz"))
    omega = np.linspace(*wl["omega"])
    eta = wl["eta"]
    spec = c3.ProblemSpec.load(spec_path)

    # one-off host compilation of the device programs (setup, not timed)
    t0 = time.perf_counter()
    base = c3.ComponentStaticProblem.compile(spec, device=dev)
    _ = base.plan
    eom_problem = c3.ComponentEOMProblem.compile(c3.eom_ccsd_problem(base), base, 1)
    _ = eom_problem.plan
    _ = eom_problem.plan.sources(spec.impurity_site)
    setup_seconds = time.perf_counter() - t0

    def step(problem, eomp, precision="mixed", method="arnoldi", grid=None):
        sol = c3.solve_component_ccsd(problem, precision=precision)
        ctx = c3.ComponentEOMContext(eomp, torch.from_numpy(sol.amplitudes))
        op = c3.ComponentSigmaOperator(ctx)
        src = c3.component_eom_sources(ctx)
        res = c3.component_retarded_green(op, src, omega if grid is None else grid, eta, method=method)
        return sol, res

    # resident problem: device tables uploaded once
    _ = base.ops
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2
    for _ in range(args.warmup):
        step(base, eom_problem)
    torch.cuda.synchronize()
    if args.profile_step:
        # one step inside an NVTX range "step" (for ncu --nvtx-include step/), then stop
        t0 = time.perf_counter()
        torch.cuda.nvtx.range_push("step")
        step(base, eom_problem)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        return {"profile_step_seconds": time.perf_counter() - t0, "workload": args.workload}
    if ws > 1:
        torch.distributed.barrier()
    times = []
    rt.LaunchCounter.reset()
    stream = torch.cuda.current_stream(dev)
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            _flush_l2(torch, flush)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sol, res = step(base, eom_problem)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1000.0)
    launches = rt.LaunchCounter.reset()
    t_step = float(np.mean(times))
    # the plain FP64 form of the same kernels, same workload (comparison point;
    # one untimed step first, as for the headline)
    step(base, eom_problem, "fp64")
    plain = []
    for _ in range(max(1, min(args.steps, 3))):
        _flush_l2(torch, flush)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sol64, res64 = step(base, eom_problem, "fp64")
        e1.record(stream)
        torch.cuda.synchronize()
        plain.append(e0.elapsed_time(e1) / 1000.0)
    rt.LaunchCounter.reset()
    t_plain = float(np.mean(plain))
    mixed_vs_fp64 = float(np.max(np.abs(res.retarded - res64.retarded)) / np.max(np.abs(res64.retarded)))
    # the plain FP64 form with batching over omega disabled as well: the
    # reference's per-frequency GMRES loop on the same kernels (one step,
    # after a warm-up of the same path on a short grid)
    step(base, eom_problem, "fp64", "gmres", omega[:8])
    _flush_l2(torch, flush)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sol_u, res_u = step(base, eom_problem, "fp64", "gmres")
    e1.record(stream)
    torch.cuda.synchronize()
    t_unbatched = e0.elapsed_time(e1) / 1000.0
    rt.LaunchCounter.reset()
    unbatched_vs_fp64 = float(np.max(np.abs(res_u.retarded - res64.retarded)) / np.max(np.abs(res64.retarded)))
    if ws > 1:
        t_step = _max_over_ranks(t_step, dev)

    # accuracy against the reference FP64 run (subset of the grid it computed)
    amp_err = float(np.max(np.abs(sol.amplitudes - gold["solution_amplitudes"])) /
                    np.max(np.abs(gold["solution_amplitudes"])))
    idx = [int(np.argmin(np.abs(omega - w))) for w in gold["green_omega"]]
    g_err = float(np.max(np.abs(res.retarded[idx] - gold["green_retarded"])) / np.max(np.abs(gold["green_retarded"])))

    # end to end from host buffers through the public API (tables uploaded inside)
    e2e_times = []
    h2d = d2h = 0
    for k in range(max(1, min(args.steps, 3))):
        _flush_l2(torch, flush)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        problem = c3.ComponentStaticProblem(spec, device=dev)
        problem._plan = base.plan          # host-compiled program reused; device upload happens here
        eomp = c3.ComponentEOMProblem(problem, 0, 1)
        eomp._plan = eom_problem.plan
        sol2, res2 = step(problem, eomp)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_times.append(e0.elapsed_time(e1) / 1000.0)
        if k == 0:
            # the static and EOM program tables, the converged amplitudes sent to the EOM
            # context, the EOM diagonal, the sink and the shift grid
            h2d = sum(t.numel() * t.element_size() for t in problem.ops._up.keep)
            h2d += sum(t.numel() * t.element_size() for up in eomp._tables.values() for t in up.keep)
            h2d += sol2.amplitudes.nbytes + 16 * eomp.dimension * 2 + 16 * omega.size
            d2h = sol2.amplitudes.nbytes + sol2.variables.nbytes + res2.retarded.nbytes * 3
    e2e = float(np.mean(e2e_times))

    # dominant-kernel roofline: the JVP output stage (k_wedge<static>) timed alone
    roof = kernel_roofline(base, dev)
    hbm, bf16, peak_kind = _peaks()
    out = {
        "metric": METRIC, "value": t_step, "unit": "s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128", "data": "synthetic",
        "config": {"workload": args.workload, "description": wl["label"],
                   "precision": "mixed: FP32 inner JVPs and FP32 Krylov basis in GMRES (inner tolerance >= 1e-5, and up to 0.05 x tolerance / |r| near convergence), FP64 "
                                "residuals/refinement; FP64 sigma; Arnoldi CGS2 with FP32 first projections and "
                                "double-float (FP32-pipe) updates and second projections, FP64 Hessenberg "
                                "column and shifted solves",
                   "plain_fp64_seconds": t_unbatched,
                   "plain_fp64_form": "FP64 inner JVPs, the reference's per-frequency preconditioned GMRES for "
                                      "every omega and channel (batching off), zero initial amplitudes",
                   "speedup_vs_plain_fp64": t_unbatched / t_step,
                   "fp64_batched_seconds": t_plain, "speedup_vs_fp64_batched": t_plain / t_step,
                   "green_rel_err_mixed_vs_fp64": mixed_vs_fp64,
                   "green_rel_err_unbatched_vs_batched_fp64": unbatched_vs_fp64,
                   "batched_omega": "one CGS2 Arnoldi basis per channel for all omega (graph-replayed steps, "
                                    "incremental FP64 shifted solves); addition and removal channels stepped together, "
                                    "one launch per kernel for both",
                   "warm_start": "off: the learned guess lowers the starting residual but not the Newton work "
                                 "on this family",
                   "l2": "flushed between steps (256 MB write)",
                   "parallelism": "replicas" if ws > 1 else "single", "setup_seconds": setup_seconds,
                   "newton_iterations": sol.iterations, "jvp_evaluations": sol.jvp_evaluations,
                   "residual_evaluations": sol.residual_evaluations, "krylov_dimensions": list(res.krylov_dimensions),
                   "amplitude_rel_err_vs_reference": amp_err, "green_rel_err_vs_reference": g_err,
                   "packed_residual_norm": sol.packed_residual_norm},
        "gpu_launches": int(launches),
        "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "roofline": dict(roof, peak=hbm, frac=roof["achieved"] / hbm, peak_source=peak_kind),
        "clocks": clocks.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(spec, gold, omega)
    return out if rank == 0 else None


def kernel_roofline(problem, dev) -> dict:
    """Roofline of the JVP output stage (k_wedge<kStatic>), the most-launched wedge kernel.

    The mixed headline runs it over the FP32 workspace.  Algorithmic bytes per
    launch: every workspace entry its instances reference, read once (8 B per
    complex FP32 entry), the instance/element/tile tables, the per-element
    epilogue tables and the real outputs written.  The FP64 variant is timed
    too for reference.
    """
    import ctypes as C

    import torch

    from c3lindblad_gb300 import runtime as rt

    ops = problem.ops
    plan = problem.plan
    stage = plan.program.stages["jvp"]
    read = set()
    for inst in stage.instances:
        for j in range(int(inst["nfac"])):
            read.add((int(inst["fac_off"][j]), int(inst["fac_deg"][j])))
    entries = sum(plan.n ** d for _, d in read)
    table_bytes = stage.instances.nbytes + stage.elements.nbytes + stage.digits.nbytes + stage.tiles.nbytes
    elem = stage.elements.size
    ep_bytes = elem * (16 + 8 + 8 + 16 + 16)  # lam, col, pair, scale, src
    out_bytes = 8 * plan.num_variables
    alg32 = 8 * entries + table_bytes + ep_bytes + out_bytes
    alg64 = 16 * entries + table_bytes + ep_bytes + out_bytes
    x = torch.zeros(plan.num_variables, dtype=torch.float64, device=dev)
    y = torch.empty_like(x)
    ops.linearize(x, y)
    ops.to_single()
    d = torch.ones_like(x)
    ops.jvp32(d, y)
    ops.jvp(d, y)
    st = rt.wedge_stage(ops._up, stage)
    a = ops.jvp_action
    lib = rt.lib()
    stream = torch.cuda.current_stream(dev)
    reps = 200

    def timed(fn):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1000.0 / reps

    t32 = timed(lambda: lib.c3l_wedge_static_out_f32(C.byref(st), plan.n, ops.ws32_lin.data_ptr(), a.lam, a.canon,
                                                     a.col, a.pair, a.scale, y.data_ptr(), stream.cuda_stream))
    t64 = timed(lambda: lib.c3l_wedge_static_out(C.byref(st), plan.n, ops.ws_lin.data_ptr(), a.lam, a.canon, a.col,
                                                 a.pair, a.scale, y.data_ptr(), stream.cuda_stream))
    # DRAM read + write per launch of this kernel on this workload from one ncu capture (cold caches,
    # 666 tiles of 16 outputs): close to the algorithmic bytes, so nothing is re-read from DRAM
    traffic = 1.728e6 if problem.plan.n == 11 else None
    return {"bound": "hbm", "kernel": "k_wedge<kStatic, float2> (JVP output stage, FP32 workspace)",
            "achieved": alg32 / t32 / 1e9, "unit": "GB/s", "traffic": traffic, "algorithmic_bytes": int(alg32),
            "launch_us": t32 * 1e6, "fp64_variant_launch_us": t64 * 1e6, "instances": int(stage.instances.size),
            "elements": int(elem)}


def cpu_baseline(spec, gold, omega, budget_s: float = 20.0) -> dict:
    """Per-call timings of the CPU oracle scaled by the reference run's call counts."""
    from oracle import component_oracle as oc

    p = oc.OracleProblem(spec.as_dict())
    x = gold["fixed_amplitudes"]
    d = gold["fixed_direction"]
    t0 = time.perf_counter()
    p.residual(x)
    t_res = time.perf_counter() - t0
    t0 = time.perf_counter()
    p.jvp(x, d)
    t_jvp = time.perf_counter() - t0
    eom = oc.OracleEOM(p, gold["solution_amplitudes"], 0, 1)
    v = gold["eomp_probe"]
    k = 0
    t0 = time.perf_counter()
    while k < 50 and time.perf_counter() - t0 < budget_s / 4:
        eom.sigma(v)
        k += 1
    t_sig = (time.perf_counter() - t0) / k
    n_res = int(gold["solution_residual_evaluations"])
    n_jvp = int(gold["solution_jvp_evaluations"])
    sig_calls = float(gold["green_sigma_calls"]) * omega.size / gold["green_omega"].size
    est = n_res * t_res + n_jvp * t_jvp + sig_calls * t_sig
    return {"value": est, "unit": "s", "cores": 1, "kind": "port",
            "sample": (f"oracle per-call times (residual {t_res:.3f}s, JVP {t_jvp:.3f}s, sigma {t_sig * 1e3:.2f}ms) "
                       f"x the reference solver's call counts on this workload ({n_res} residuals, {n_jvp} JVPs, "
                       f"{sig_calls:.0f} sigma calls for {omega.size} omega by per-frequency GMRES)")}


def run_reference(args) -> dict | None:
    ws, rank, _ = _dist()
    if rank != 0:
        return None
    wl = WORKLOADS[args.workload]
    from c3lindblad_gb300.spec import ProblemSpec

    spec = ProblemSpec.load(ROOT / "tests" / "golden" / f"{wl['spec']}.spec.npz")
    gold = dict(np.load(ROOT / "tests" / "golden" / f"{wl['spec']}.golden.npz"))
    omega = np.linspace(*wl["omega"])
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(spec, gold, omega, budget_s=4.0)
    for _ in range(args.steps):
        cb = cpu_baseline(spec, gold, omega, budget_s=8.0)
        vals.append(cb["value"])
    v = float(np.mean(vals))
    cb["value"] = v
    return {"metric": METRIC, "value": v, "unit": "s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128", "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, "description": wl["label"]},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="siam10", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-step", action="store_true",
                    help="run the warm-up steps and one step inside an NVTX range named 'step', then exit")
    args = ap.parse_args()
    out = run_reference(args) if args.impl == "reference" else run_gpu(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()

"""NumPy interpreter of the compiled device tables (test infrastructure).

It executes ``ContractTask``/``Instance``/``Tile`` tables with exactly the
semantics of the CUDA kernels, so the symbolic compiler can be checked
against the oracle on CPU.  It is never used by the product path.
"""

from __future__ import annotations

import numpy as np


def _digits_padded(size: int, deg: int, n: int) -> np.ndarray:
    from c3lindblad_gb300.compiler import MAX_DEGREE

    e = np.arange(size)
    out = np.zeros((size, MAX_DEGREE), np.int64)
    for c in range(deg):
        out[:, c] = (e // n ** (deg - 1 - c)) % n
    return out


def _digits_packed(packed: np.ndarray) -> np.ndarray:
    from c3lindblad_gb300.compiler import MAX_DEGREE

    out = np.zeros((packed.size, MAX_DEGREE), np.int64)
    for c in range(MAX_DEGREE):
        out[:, c] = (packed >> (8 * c)) & 0xFF
    return out


def run_levels(program, cls: str, ws: np.ndarray) -> None:
    n = program.n
    vec = program.vectors
    for level in program.levels.get(cls, []):
        for task in level.tasks:
            deg = int(task["deg"])
            size = n ** deg
            e = np.arange(size)
            acc = np.zeros(size, np.complex128)
            if task["const_off"] >= 0:
                acc += vec[task["const_off"] + e]
            for j in range(int(task["nsrc"])):
                axis = int(task["axis"][j])
                low = n ** (deg - axis)
                hi = e // low
                lo = e % low
                for m in range(n):
                    src = int(task["src_off"][j]) + hi * low * n + m * low + lo
                    acc += task["sign"][j] * vec[task["vec_off"][j] + m] * ws[src]
            ws[task["dst_off"] + e] = acc


def _eval_instances(stage, b: int, digits: np.ndarray, ws: np.ndarray, n: int) -> np.ndarray:
    blk = stage.blocks[b]
    acc = np.zeros(digits.shape[0], np.complex128)
    for inst in stage.instances[blk["inst_begin"]:blk["inst_end"]]:
        val = np.full(digits.shape[0], complex(inst["coef"][0], inst["coef"][1]))
        for j in range(int(inst["nfac"])):
            deg = int(inst["fac_deg"][j])
            off = np.full(digits.shape[0], int(inst["fac_off"][j]), np.int64)
            for q in range(deg):
                off += digits[:, int(inst["axes"][j][q])] * n ** (deg - 1 - q)
            val = val * ws[off]
        acc += val
    return acc


def run_padded(program, name: str, ws: np.ndarray) -> None:
    stage = program.stages.get(name)
    if stage is None:
        return
    n = program.n
    for b, blk in enumerate(stage.blocks):
        deg = int(blk["deg"])
        size = n ** deg
        ws[blk["out_off"] + np.arange(size)] = _eval_instances(stage, b, _digits_padded(size, deg, n), ws, n)


def run_pairs(program, name: str, ws: np.ndarray) -> np.ndarray:
    """The pair GEMMs of stage ``name``: returns the workspace followed by the
    pair buffer (what the ``<name>_pairs`` gather stage reads)."""
    pp = program.pairs[name]
    out = np.concatenate([ws, np.zeros(program.pair_size, np.complex128)])
    base = program.ws_size
    for g in pp.groups:
        M, N = int(g["M"]), int(g["N"])
        k = np.arange(int(g["kbegin"]), int(g["kend"]))
        A = ws[pp.aoff[k][:, None] + np.arange(M)[None, :]]
        R = ws[pp.roff[k][:, None] + np.arange(N)[None, :]]
        out[base + int(g["p_off"]) + np.arange(M * N)] = (A.T @ R).reshape(-1)
    return out


def run_canonical(program, name: str, ws: np.ndarray) -> np.ndarray:
    """Returns the interaction value at every element of the stage (stage order)."""
    stage = program.stages[name]
    n = program.n
    out = np.zeros(stage.elements.size, np.complex128)
    digits = _digits_packed(stage.digits)
    for b in range(len(stage.blocks)):
        sel = np.flatnonzero(stage.element_block == b)
        if sel.size:
            out[sel] = _eval_instances(stage, b, digits[sel], ws, n)
    return out


class InterpretedStatic:
    def __init__(self, plan):
        self.plan = plan
        self.ws = np.zeros(plan.program.ws_size, np.complex128)

    def _unpack(self, x):
        t = self.plan.tilde
        return t.coef_a * x[t.idx_a] + t.coef_b * x[t.idx_b]

    def residual(self, x, *, linearize: bool = False):
        p = self.plan
        prog = p.program
        t = self._unpack(np.asarray(x, np.float64))
        self.t = t
        sc = p.scatter_T
        self.ws[sc.dst] = sc.sign * t[sc.pos]
        run_levels(prog, "T", self.ws)
        run_padded(prog, "res_rest_T", self.ws)
        run_padded(prog, "res_scalar", self.ws)
        if linearize:
            run_padded(prog, "jvp_rest_T", self.ws)
        V = run_canonical(prog, "res", self.ws)
        return self._epilogue(V, t, p.program.stages["res"].elements, p.epilogue), \
            -1j * (self.ws[p.res_scalar_off] if p.res_scalar_off >= 0 else 0.0)

    def jvp(self, dx):
        p = self.plan
        prog = p.program
        v = self._unpack(np.asarray(dx, np.float64))
        sc = p.scatter_V
        self.ws[sc.dst] = sc.sign * v[sc.pos]
        run_levels(prog, "V", self.ws)
        run_padded(prog, "jvp_rest_V", self.ws)
        run_padded(prog, "jvp_scalar", self.ws)
        V = run_canonical(prog, "jvp", self.ws)
        return self._epilogue(V, v, p.program.stages["jvp"].elements, p.epilogue_jvp), \
            -1j * (self.ws[p.jvp_scalar_off] if p.jvp_scalar_off >= 0 else 0.0)

    def _epilogue(self, V, src, elements, ep):
        r = -1j * (ep["lam"] * src[elements] + V)
        x = np.zeros(self.plan.num_variables)
        val = r * ep["scale"]
        x[ep["col"]] = val.real
        pr = ep["pair"] == 1
        x[ep["col"][pr] + 1] = r[pr].imag
        return x


class InterpretedEOM:
    def __init__(self, plan, amplitudes):
        self.plan = plan
        prog = plan.program
        self.ws = np.zeros(prog.ws_size, np.complex128)
        sc = plan.scatter_T
        t = np.asarray(amplitudes, np.complex128)
        self.t = t
        self.ws[sc.dst] = sc.sign * t[sc.pos]
        run_levels(prog, "T", self.ws)
        run_padded(prog, "sigma_rest_T", self.ws)

    def sources(self, site: int):
        sp = self.plan.sources(site)
        prog = sp.program
        ws = np.zeros(prog.ws_size, np.complex128)
        sc = sp.scatter_T
        ws[sc.dst] = sc.sign * self.t[sc.pos]
        run_levels(prog, "T", ws)
        out = []
        for name, scale in zip(("add", "rem"), sp.source_scale):
            run_padded(prog, f"{name}_rest_T", ws)
            V = run_canonical(prog, name, ws)
            v = np.zeros(self.plan.dimension, np.complex128)
            v[prog.stages[name].elements] = scale * V
            out.append(v)
        return out[0], out[1], sp.sink

    def sigma(self, x):
        p = self.plan
        prog = p.program
        x = np.asarray(x, np.complex128)
        sc = p.scatter_X
        self.ws[sc.dst] = sc.sign * x[sc.pos]
        run_levels(prog, "X", self.ws)
        run_padded(prog, "sigma_rest_X", self.ws)
        V = run_canonical(prog, "sigma", self.ws)
        el = prog.stages["sigma"].elements
        out = np.zeros(p.dimension, np.complex128)
        out[el] = p.lam_sigma * x[el] + V
        return out

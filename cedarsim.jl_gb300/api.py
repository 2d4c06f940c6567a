"""Host-side mirror of CedarSim's analysis entry points over the CUDA library.

Reference entry point                                  here
------------------------------------------------------ -------------------------
CircuitIRODESystem(circ)  (src/circuitodesystem.jl:152) System(circuit)
prob.f.f(out, du, u, p, t) / prob.f.jac(J, du, u, p, gamma, t)
   (benchmarks/benchmark_common.jl:138,155)            System.f / System.jac
dc!(circ)                 (src/sweeps.jl:437-448)        dc(circuit)
tran!(circ, tspan)        (src/sweeps.jl:450-463)        tran(circuit, tspan, ...)
CircuitSweep + tran!.     (src/sweeps.jl:390-435,488-502) tran(CircuitSweep(...), tspan)
CircuitSweep + dc!.       (src/sweeps.jl:471-486)        dc(CircuitSweep(...))
instance tables (MC)      (no counterpart)               Batch(...).tran(...), .dc()
forward sensitivities     (test/sensitivity.jl:13-42)    Batch(...).adjoint(...)
ac!(circ) / freqresp      (src/ac.jl:178-186,251-258)    ac(circuit).freqresp(sym, omegas)
noise!(circ) / PSD        (src/ac.jl:188-197,263-283)    noise(circuit).psd(sym, omegas)
acdec(nd, fstart, fstop)  (src/ac.jl:288-301)            acdec(nd, fstart, fstop)

Every computation runs in libcedar_gpu.so; nothing here falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import Optional, Sequence, Tuple, Union

import numpy as np

from . import abi
from .abi import BatchHolder, BatchTuning, DescHolder, Stats, STATS_DTYPE, check, load_library, make_opts
from .circuit import Circuit, Flat, I as _MODEL_I, V as _MODEL_V
from .sweeps import CircuitSweep, sweep_dc, sweep_tran


def _flat(c: Union[Circuit, Flat]) -> Flat:
    return c.flatten() if isinstance(c, Circuit) else c


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _state(x, n: int) -> np.ndarray:
    """x as a contiguous float64 vector of the circuit's n unknowns (the library
    reads exactly n values from it)."""
    x = np.ascontiguousarray(x, np.float64).ravel()
    if x.size != n:
        raise ValueError(f"state has {x.size} values, the circuit has {n} unknowns")
    return x


class System:
    """A compiled circuit on the GPU (the counterpart of CircuitIRODESystem)."""

    def __init__(self, circuit: Union[Circuit, Flat]):
        self.lib = load_library()
        self.flat = _flat(circuit)
        self._holder = DescHolder(self.flat)
        h = C.c_void_p()
        check(self.lib.cedar_ckt_create(C.byref(self._holder.desc), C.byref(h)))
        self.handle = h
        n, nj, nlu, nl = (C.c_int32() for _ in range(4))
        check(self.lib.cedar_ckt_size(h, C.byref(n), C.byref(nj), C.byref(nlu), C.byref(nl)))
        self.n, self.nnz_j, self.nnz_lu, self.n_levels = n.value, nj.value, nlu.value, nl.value

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and h.value:
            self.lib.cedar_ckt_destroy(h)
            self.handle = None

    @property
    def names(self):
        return self.flat.names

    def pattern(self) -> Tuple[np.ndarray, np.ndarray]:
        colptr = np.zeros(self.n + 1, np.int32)
        rowidx = np.zeros(self.nnz_j, np.int32)
        check(self.lib.cedar_ckt_pattern(self.handle, abi.ptr(colptr, C.c_int32), abi.ptr(rowidx, C.c_int32)))
        return colptr, rowidx

    def symbolic(self):
        rm = np.zeros(self.n, np.int32)
        order = np.zeros(self.n, np.int32)
        cp = np.zeros(self.n + 1, np.int32)
        ri = np.zeros(self.nnz_lu, np.int32)
        check(self.lib.cedar_ckt_symbolic(self.handle, *(abi.ptr(a, C.c_int32) for a in (rm, order, cp, ri))))
        return rm, order, cp, ri

    # ---- DAECompiler-style residual / Jacobian
    def f(self, out: np.ndarray, du: Optional[np.ndarray], u: np.ndarray, t: float) -> np.ndarray:
        u = _state(u, self.n)
        du = None if du is None else _state(du, self.n)
        if out.dtype != np.float64 or not out.flags.c_contiguous or out.size != self.n:
            raise ValueError(f"out must be a contiguous float64 array of {self.n} values")
        check(self.lib.cedar_eval(self.handle, _dp(u), None if du is None else _dp(du), float(t), 0.0, _dp(out), None))
        return out

    def jac(self, J: np.ndarray, du: Optional[np.ndarray], u: np.ndarray, gamma: float, t: float) -> np.ndarray:
        """J (CSC values in pattern() order) = dF/du + gamma dF/du'."""
        u = _state(u, self.n)
        if J.dtype != np.float64 or not J.flags.c_contiguous or J.size != self.nnz_j:
            raise ValueError(f"J must be a contiguous float64 array of {self.nnz_j} values")
        check(self.lib.cedar_eval(self.handle, _dp(u), None, float(t), float(gamma), None, _dp(J)))
        return J

    def eval(self, u, du=None, t=0.0, gamma=0.0):
        F = np.zeros(self.n)
        J = np.zeros(self.nnz_j)
        u = _state(u, self.n)
        du = None if du is None else _state(du, self.n)
        check(self.lib.cedar_eval(self.handle, _dp(u), None if du is None else _dp(du), float(t), float(gamma),
                                  _dp(F), _dp(J)))
        return F, J

    def jac_dense(self, J: np.ndarray) -> np.ndarray:
        cp, ri = self.pattern()
        M = np.zeros((self.n, self.n))
        for c in range(self.n):
            M[ri[cp[c]:cp[c + 1]], c] = J[cp[c]:cp[c + 1]]
        return M

    def newton_solve(self, t: float, cj: float, hist: Optional[np.ndarray], x: np.ndarray):
        x = _state(x, self.n).copy()
        st = Stats()
        hist = None if hist is None else _state(hist, self.n)
        rc = self.lib.cedar_newton_solve(self.handle, float(t), float(cj), None if hist is None else _dp(hist), _dp(x),
                                         C.byref(st))
        return x, st, rc


def costs(circuit: Union[Circuit, Flat]) -> dict:
    """Algorithmic FP64 work and bytes of one Newton iteration (host-only analysis)."""
    lib = load_library()
    holder = DescHolder(_flat(circuit))
    h = C.c_void_p()
    check(lib.cedar_plan_create(C.byref(holder.desc), C.byref(h)))
    try:
        c = abi.Costs()
        check(lib.cedar_ckt_costs(h, C.byref(c)))
        return {k: getattr(c, k) for k, _ in abi.Costs._fields_}
    finally:
        lib.cedar_ckt_destroy(h)


@dataclass
class Solution:
    t: np.ndarray
    u: np.ndarray
    names: list
    stats: dict
    retcode: str

    def __getitem__(self, name):
        return self.u[:, self.names.index(name)]


def _stats_dict(st) -> dict:
    return {k: getattr(st, k) for k, _ in Stats._fields_ if k != "pad"}


CEDAR_ENOCONV = -5          # include/cedar.h: Newton / DC operating point did not converge
DC_START_SCALE = 1e-7       # the spread of a restart: x0 = 1e-7 * randn(n), as src/dcop.jl:62


def dc_starts(n: int, seed: int = 0):
    """The restart points of the multi-start DC solve: an endless sequence of
    1e-7 * randn(n) vectors (src/dcop.jl:62) from a Philox generator keyed by
    `seed`, so that a failed solve restarts from the same points on every run."""
    rng = np.random.Generator(np.random.Philox(seed))
    while True:
        yield DC_START_SCALE * rng.standard_normal(n)


def bootstrapped_dc(solve, x0: np.ndarray, trajectories: int = 10, seed: int = 0):
    """CedarSim's bootstrapped_nlsolve (src/dcop.jl:53-94) around one DC solve.

    `solve(x)` runs one DC solve in place on x and returns (rc, stats).  The
    first trajectory starts from x0 (the caller's guess, zeros by default, where
    the reference starts every trajectory from a random point: a solve from
    zeros is kept first so that results where it converges do not depend on the
    seed); each later one starts from the next point of dc_starts(n, seed).  A
    trajectory that ends without convergence (CEDAR_ENOCONV: any non-OK status
    of the solve, a zero pivot included, as the reference retries its
    SingularException) moves on to the next start; any other return code ends
    the loop at once (the caller raises it, as the reference rethrows).  Returns
    (x, rc, stats of the last trajectory, trajectories run, DC iterations summed
    over them); rc is CEDAR_ENOCONV if none converged."""
    if trajectories < 1:
        raise ValueError("trajectories must be at least 1")
    x = np.ascontiguousarray(x0, np.float64).copy()
    starts = dc_starts(x.size, seed)
    iters = 0
    for k in range(trajectories):
        if k:
            x = next(starts)
        rc, st = solve(x)
        iters += int(st.dc_iters)
        if rc != CEDAR_ENOCONV:
            return x, rc, st, k + 1, iters
    return x, rc, st, trajectories, iters


def batch_dc_restarts(x: np.ndarray, st: np.ndarray, n_of: np.ndarray, trajectories: int, seed: int, run_round):
    """The restart rounds of a batched DC solve (bootstrapped_dc per instance).

    x[n_inst, n_max] and st (STATS_DTYPE) hold the first solve of every instance,
    n_of its unknown counts.  Each round solves the instances that have not
    converged yet together, by run_round(idx, x0) -> (x_sub[len(idx), m], stats),
    instance idx[j] starting from x0[j], its next point of dc_starts(n_i, seed + i);
    at most trajectories - 1 rounds.  An instance's dc_iters add up over its
    trajectories; its x, status and other stats are those of its last one.
    Updates x and st in place and returns them."""
    fail = np.flatnonzero(st["status"] != 0)
    starts = {int(i): dc_starts(int(n_of[i]), seed + int(i)) for i in fail}
    for _ in range(trajectories - 1):
        if fail.size == 0:
            break
        xs, ss = run_round(fail, [next(starts[int(i)]) for i in fail])
        ss = ss.copy()
        ss["dc_iters"] += st["dc_iters"][fail]
        x[fail, :xs.shape[1]] = xs
        x[fail, xs.shape[1]:] = 0.0
        st[fail] = ss
        fail = fail[ss["status"] != 0]
    return x, st


def dc(circuit: Union[Circuit, Flat, System, "CircuitSweep"], t: float = 0.0, x0: Optional[np.ndarray] = None,
       trajectories: int = 10, seed: int = 0, **kw):
    """DC operating point (CedarDCOp's role): Newton, then pseudo-transient continuation, then
    source stepping; rerun with dense partial pivoting if the static pivot order fails; a
    solve that does not converge is restarted from up to trajectories - 1 random points
    near zero (bootstrapped_dc).  Over a CircuitSweep this is the dc!. broadcast: every
    point in one batched launch, keyword arguments as sweeps.sweep_dc."""
    if isinstance(circuit, CircuitSweep):
        return sweep_dc(circuit, trajectories=trajectories, seed=seed, **kw)
    if kw:
        raise TypeError(f"dc() of one circuit takes no options {sorted(kw)}")
    sys = circuit if isinstance(circuit, System) else System(circuit)
    x0 = np.zeros(sys.n) if x0 is None else _state(x0, sys.n)

    def solve(x):
        st = Stats()
        return sys.lib.cedar_dcop(sys.handle, float(t), _dp(x), C.byref(st)), st

    x, rc, _, _, _ = bootstrapped_dc(solve, x0, trajectories, seed)
    check(rc)
    return x


def tran(circuit: Union[Circuit, Flat, System, "CircuitSweep"], tspan: Tuple[float, float], method: str = "bdf2",
         h: Optional[float] = None, adaptive: Optional[bool] = None, x0: Optional[np.ndarray] = None,
         dcop: bool = True, reltol: float = 1e-6, abstol_v: float = 1e-9, abstol_i: float = 1e-12,
         cap: int = 1 << 20, **kw) -> Solution:
    """Transient analysis on the GPU (the counterpart of tran!(circ, tspan)).  Over a
    CircuitSweep this is the tran!. broadcast (keyword arguments as sweeps.sweep_tran)."""
    if isinstance(circuit, CircuitSweep):
        return sweep_tran(circuit, tspan, method=method, reltol=reltol, abstol_v=abstol_v, dcop=dcop, **kw)
    sys = circuit if isinstance(circuit, System) else System(circuit)
    if adaptive is None:
        adaptive = h is None
    opts = make_opts(method, adaptive, tspan[0], tspan[1], h or 0.0, dcop, reltol, abstol_v, abstol_i, **kw)
    x = np.zeros(sys.n) if x0 is None else _state(x0, sys.n).copy()
    t_out = np.zeros(cap)
    x_out = np.zeros((cap, sys.n))
    n_out = C.c_int64()
    st = Stats()
    rc = sys.lib.cedar_tran_run(sys.handle, C.byref(opts), _dp(x), _dp(t_out), _dp(x_out), cap, C.byref(n_out),
                                C.byref(st))
    check(rc)
    m = min(n_out.value, cap)
    return Solution(t_out[:m].copy(), x_out[:m].copy(), sys.names, _stats_dict(st), abi.STATUS_NAMES[st.status])


@dataclass
class BatchResult:
    x_final: np.ndarray      # [n_inst, n_max]
    samples: Optional[np.ndarray]  # [n_inst, n_probes, n_samples]
    stats: np.ndarray        # structured STATS_DTYPE


class Batch:
    """Batched instances (a CircuitSweep / Monte Carlo over parameter blocks) on one GPU."""

    def __init__(self, templates: Sequence[Union[Circuit, Flat]], inst_template, inst_par=None, inst_par_off=None,
                 inst_x0=None, inst_x0_off=None, inst_dx=None, inst_dx_off=None, probes=None, n_samples: int = 0):
        self.lib = load_library()
        self.templates = [_flat(t) for t in templates]
        self.holder = BatchHolder(self.templates, inst_template, inst_par, inst_par_off, inst_x0, inst_x0_off,
                                  inst_dx, inst_dx_off, probes, n_samples)
        h = C.c_void_p()
        check(self.lib.cedar_batch_create(C.byref(self.holder.desc), C.byref(h)))
        self.handle = h
        nm = C.c_int32()
        check(self.lib.cedar_batch_nmax(h, C.byref(nm)))
        self.n_max = nm.value
        self.n_inst = self.holder.n_inst
        self.n_probes = 0 if probes is None else np.asarray(probes).shape[-1]
        self.n_samples = n_samples if self.n_probes else 0

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and h.value:
            self.lib.cedar_batch_destroy(h)
            self.handle = None

    @property
    def tuning(self) -> Tuple[int, int]:
        t = BatchTuning()
        check(self.lib.cedar_batch_get_tuning(self.handle, C.byref(t)))
        return t.lanes_per_inst, t.warps_per_cta

    def set_tuning(self, lanes_per_inst: int, warps_per_cta: int, ctas_per_sm: int = 0):
        t = BatchTuning(lanes_per_inst, warps_per_cta, ctas_per_sm)
        check(self.lib.cedar_batch_set_tuning(self.handle, C.byref(t)))

    def autotune(self, opts, horizon: float, cache: Optional[str] = None) -> Tuple[int, int]:
        """Time every tile shape (lanes per instance x warps per CTA) on a short
        horizon and keep the fastest.  With `cache` (a JSON file), a result stored
        for the same GPU, instance count and template sizes is reused instead."""
        key = None
        if cache:
            import json
            import os
            import torch
            sizes = sorted((f.n, sum(g[1].shape[0] for g in f.groups)) for f in self.templates)
            key = f"{torch.cuda.get_device_name(0)}|{self.n_inst}|{sizes}"
            table = {}
            if os.path.exists(cache):
                with open(cache) as fh:
                    table = json.load(fh)
            if key in table:
                k, w = table[key]
                self.set_tuning(k, w)
                return k, w
        t = BatchTuning()
        check(self.lib.cedar_batch_autotune(self.handle, C.byref(opts), float(horizon), C.byref(t)))
        if key is not None:
            table[key] = [t.lanes_per_inst, t.warps_per_cta]
            tmp = cache + ".tmp"
            with open(tmp, "w") as fh:
                json.dump(table, fh, indent=1, sort_keys=True)
            os.replace(tmp, cache)
        return t.lanes_per_inst, t.warps_per_cta

    def run(self, opts, want_samples: bool = True) -> BatchResult:
        xf = np.zeros((self.n_inst, self.n_max))
        samp = np.zeros((self.n_inst, self.n_probes, self.n_samples)) if (want_samples and self.n_probes) else None
        st = np.zeros(self.n_inst, STATS_DTYPE)
        check(self.lib.cedar_batch_run(self.handle, C.byref(opts), _dp(xf), None if samp is None else _dp(samp),
                                       st.ctypes.data_as(C.c_void_p)))
        return BatchResult(xf, samp, st)

    def dc(self, reltol=1e-6, abstol_v=1e-9, trajectories: int = 10, seed: int = 0, **kw):
        """DC operating point of every instance (dc!. over a CircuitSweep).
        Instances whose solve does not converge are solved again, in one batched
        launch per round, from random points near zero (up to trajectories - 1
        rounds; instance i's k-th restart is point k of dc_starts(n_i, seed + i),
        the bootstrapped_dc rule per instance).  stats[i].dc_iters sums the
        iterations of every trajectory of instance i; stats[i].status is that of
        its last one.  Returns (x_dc[n_inst, n_max], stats)."""
        if trajectories < 1:
            raise ValueError("trajectories must be at least 1")
        opts = make_opts("bdf2", True, 0.0, 1.0, 0.0, True, reltol, abstol_v, **kw)
        x = np.zeros((self.n_inst, self.n_max))
        st = np.zeros(self.n_inst, STATS_DTYPE)
        check(self.lib.cedar_batch_dcop(self.handle, C.byref(opts), _dp(x), st.ctypes.data_as(C.c_void_p)))
        if trajectories == 1 or not np.any(st["status"] != 0):
            return x, st
        h = self.holder
        n_of = np.array([t.n for t in self.templates])[h.inst_template]

        def run_round(idx, x0):
            off = np.concatenate([[0], np.cumsum([v.size for v in x0])[:-1]]).astype(np.int64)
            sub = Batch(self.templates, h.inst_template[idx], h.inst_par,
                        None if h.inst_par_off is None else h.inst_par_off[idx],
                        inst_x0=np.concatenate(x0), inst_x0_off=off)
            return sub.dc(reltol, abstol_v, trajectories=1, **kw)

        return batch_dc_restarts(x, st, n_of, trajectories, seed, run_round)

    def tran(self, tspan, method="bdf2", reltol=1e-6, abstol_v=1e-9, dcop=True, **kw) -> BatchResult:
        return self.run(make_opts(method, True, tspan[0], tspan[1], 0.0, dcop, reltol, abstol_v, **kw))

    def nparams(self) -> Tuple[np.ndarray, int]:
        """Differentiable parameters per template (MOS1 widths, resistor values) and their maximum."""
        per = np.zeros(len(self.templates), np.int32)
        m = C.c_int32()
        check(self.lib.cedar_adjoint_nparams(self.handle, per.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(m)))
        return per, m.value

    def adjoint(self, opts, objectives, tstar=None, tape_cap: int = 0) -> "AdjointResult":
        """Objective and its gradient by the discrete adjoint, for every instance.

        objectives: one abi.Objective per template (original unknown indices).
        tstar: target crossing time per instance (or None)."""
        per, np_max = self.nparams()
        obj = (abi.Objective * len(self.templates))(*objectives)
        ts = None if tstar is None else np.ascontiguousarray(tstar, np.float64)
        phi = np.zeros(self.n_inst)
        grad = np.zeros((self.n_inst, max(np_max, 1)))
        status = np.zeros(self.n_inst, np.int32)
        st = np.zeros(self.n_inst, STATS_DTYPE)
        check(self.lib.cedar_adjoint_run(self.handle, C.byref(opts), obj, None if ts is None else _dp(ts),
                                         int(tape_cap), _dp(phi), _dp(grad),
                                         status.ctypes.data_as(C.POINTER(C.c_int32)), st.ctypes.data_as(C.c_void_p)))
        f, b = C.c_double(), C.c_double()
        check(self.lib.cedar_adjoint_last_ms(self.handle, C.byref(f), C.byref(b)))
        return AdjointResult(phi, grad[:, :np_max], status, st, per, f.value, b.value)

    def tape(self, inst: int):
        """Times and orders of the accepted steps the last adjoint run recorded for one instance."""
        n = C.c_int64()
        check(self.lib.cedar_adjoint_tape(self.handle, int(inst), None, None, 0, C.byref(n)))
        t = np.zeros(n.value)
        o = np.zeros(n.value, np.int8)
        check(self.lib.cedar_adjoint_tape(self.handle, int(inst), _dp(t), o.ctypes.data_as(C.c_void_p), n.value,
                                          C.byref(n)))
        return t, o


@dataclass
class AdjointResult:
    phi: np.ndarray          # [n_inst]
    grad: np.ndarray         # [n_inst, np_max]; row i valid up to nparams[template(i)]
    status: np.ndarray       # [n_inst] CEDAR_ST_*
    stats: np.ndarray        # forward counters
    nparams: np.ndarray      # per template
    fwd_ms: float            # device time of the recording forward run
    bwd_ms: float            # device time of the backward kernel


# ---------------------------------------------------------------- AC / noise
def acdec(nd: int, fstart: float, fstop: float) -> np.ndarray:
    """Frequencies (Hz), nd per decade from fstart to fstop, log-spaced: SPICE's
    `.ac dec nd fstart fstop` (acdec, src/ac.jl:288-301)."""
    a, b = math.log10(fstart), math.log10(fstop)
    points = int(math.ceil((b - a) * nd)) + 1
    return 10.0 ** np.linspace(a, b, points)


def ac_drive(flat: Flat) -> np.ndarray:
    """b = -dFi/d(eps) of the circuit's AC sources (original equation order): in
    :ac mode a source's value is dc + eps |ac| (src/simpledevices.jl:292-294,331-333)."""
    b = np.zeros(flat.n)
    for name, mag in flat.ac.items():
        gi, ii = flat.devices[name]
        model, term, br, par = flat.groups[gi]
        if model == _MODEL_V:                 # V+ - V- - (dc + eps a) = 0
            b[br[ii]] += mag
        elif model == _MODEL_I:               # KCL(+) -= m (dc + eps a), KCL(-) += m (dc + eps a)
            m = par[0, ii]
            if term[ii, 0] >= 0:
                b[term[ii, 0]] += m * mag
            if term[ii, 1] >= 0:
                b[term[ii, 1]] -= m * mag
    return b


def _unknown(sys: "System", sym) -> int:
    return int(sym) if isinstance(sym, (int, np.integer)) else sys.flat.index(sym)


def ac_last_stats(sys: "System") -> dict:
    """Of the last AC / noise call on `sys`: frequencies rerun densely, and device
    ms of the sparse kernel and of the dense rerun."""
    nd, a, b = C.c_int32(), C.c_double(), C.c_double()
    check(sys.lib.cedar_ac_last_stats(sys.handle, C.byref(nd), C.byref(a), C.byref(b)))
    return {"n_dense": nd.value, "ms_sparse": a.value, "ms_dense": b.value}


class ACSol:
    """The circuit linearised about its DC operating point (ACSol, src/ac.jl:73-104):
    G = dFi/dx and C = dFq/dx at x_op, driven by the AC sources."""

    def __init__(self, sys: "System", x_op: np.ndarray, b: Optional[np.ndarray] = None):
        self.sys = sys
        self.x_op = np.ascontiguousarray(x_op, np.float64)
        self.b = np.ascontiguousarray(ac_drive(sys.flat) if b is None else b, np.float64)
        self.status: Optional[np.ndarray] = None

    def freqresp(self, sym, omegas) -> np.ndarray:
        """Response X(j omega) at angular frequencies `omegas` (rad/s) of an unknown
        (name or index), of a difference (p, n) of two, or of a list of those:
        complex [n_freq] for one, [n_freq, k] for a list (freqresp, src/ac.jl:251-258)."""
        single = not isinstance(sym, list)
        syms = [sym] if single else list(sym)
        idx, pairs = [], []
        for s_ in syms:
            if isinstance(s_, tuple):
                pairs.append((len(idx), len(idx) + 1))
                idx += [_unknown(self.sys, s_[0]), _unknown(self.sys, s_[1])]
            else:
                pairs.append((len(idx), None))
                idx.append(_unknown(self.sys, s_))
        w = np.ascontiguousarray(omegas, np.float64).ravel()
        probe = np.asarray(idx, np.int32)
        resp = np.zeros((len(w), len(probe), 2))
        st = np.zeros(len(w), np.int32)
        check(self.sys.lib.cedar_ac(self.sys.handle, _dp(self.x_op), _dp(self.b), len(w), _dp(w), len(probe),
                                    abi.ptr(probe, C.c_int32), _dp(resp), abi.ptr(st, C.c_int32)))
        self.status = st
        z = resp[..., 0] + 1j * resp[..., 1]
        out = np.stack([z[:, a] if b_ is None else z[:, a] - z[:, b_] for a, b_ in pairs], axis=1)
        return out[:, 0] if single else out


class NoiseSol:
    """Output noise of the circuit linearised about its DC operating point
    (NoiseSol, src/ac.jl:107-171): white thermal noise of every resistor."""

    def __init__(self, sys: "System", x_op: np.ndarray):
        self.sys = sys
        self.x_op = np.ascontiguousarray(x_op, np.float64)
        self.status: Optional[np.ndarray] = None

    def psd(self, sym, omegas) -> np.ndarray:
        """Power spectral density at an unknown (V^2/Hz for a node voltage) over the
        angular frequencies `omegas` (PSD, src/ac.jl:263-283)."""
        w = np.ascontiguousarray(omegas, np.float64).ravel()
        out = np.zeros(len(w))
        st = np.zeros(len(w), np.int32)
        check(self.sys.lib.cedar_noise(self.sys.handle, _dp(self.x_op), len(w), _dp(w), _unknown(self.sys, sym),
                                       _dp(out), abi.ptr(st, C.c_int32)))
        self.status = st
        return out


def ac(circuit: Union[Circuit, Flat, System], x_op: Optional[np.ndarray] = None) -> ACSol:
    """ac!(circ) (src/ac.jl:178-186): DC operating point, then the linearisation."""
    sys = circuit if isinstance(circuit, System) else System(circuit)
    return ACSol(sys, dc(sys) if x_op is None else x_op)


def noise(circuit: Union[Circuit, Flat, System], x_op: Optional[np.ndarray] = None) -> NoiseSol:
    """noise!(circ) (src/ac.jl:188-197): DC operating point, then the noise analysis."""
    sys = circuit if isinstance(circuit, System) else System(circuit)
    return NoiseSol(sys, dc(sys) if x_op is None else x_op)

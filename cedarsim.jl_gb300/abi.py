"""ctypes mirror of include/cedar.h and helpers that build its descriptors.

The descriptor builders keep every numpy array they point into alive for the
lifetime of the returned holder object.
"""
from __future__ import annotations

import ctypes as C
import pathlib
from typing import List, Optional, Sequence

import numpy as np

from .circuit import Flat

c_double_p = C.POINTER(C.c_double)
c_int32_p = C.POINTER(C.c_int32)
c_int64_p = C.POINTER(C.c_int64)

CEDAR_TRAP, CEDAR_BDF2 = 0, 1
STATUS_NAMES = {0: "OK", 1: "NEWTON", 2: "ZERO_PIVOT", 3: "DT_UNDERFLOW", 4: "MAX_STEPS", 5: "NAN", 6: "DCOP",
                7: "WAIT_LIMIT", 8: "NOT_RUN"}


class DevGroup(C.Structure):
    _fields_ = [("model", C.c_int32), ("n_inst", C.c_int32), ("term", c_int32_p), ("branch", c_int32_p),
                ("par", c_double_p)]


class CktDesc(C.Structure):
    _fields_ = [("n_nodes", C.c_int32), ("n_branch", C.c_int32), ("n_groups", C.c_int32),
                ("groups", C.POINTER(DevGroup)), ("pwl", c_double_p), ("n_pwl", C.c_int64),
                ("temp_c", C.c_double), ("gmin", C.c_double), ("ordering", C.c_int32), ("reserved", C.c_int32)]

ORDER_AUTO, ORDER_MIN_DEGREE, ORDER_NESTED_DISSECTION = 0, 1, 2


class TranOpts(C.Structure):
    _fields_ = [("method", C.c_int32), ("adaptive", C.c_int32), ("dcop", C.c_int32), ("max_newton", C.c_int32),
                ("max_steps", C.c_int64), ("tstart", C.c_double), ("tstop", C.c_double), ("h", C.c_double),
                ("hmin", C.c_double), ("hmax", C.c_double), ("reltol", C.c_double), ("abstol_v", C.c_double),
                ("abstol_i", C.c_double), ("nr_factor", C.c_double), ("hfirst_frac", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("accepted", C.c_int64), ("rejected", C.c_int64), ("newton_iters", C.c_int64),
                ("dc_iters", C.c_int64), ("hmin_seen", C.c_double), ("hmax_seen", C.c_double),
                ("status", C.c_int32), ("pad", C.c_int32)]


STATS_DTYPE = np.dtype([("accepted", np.int64), ("rejected", np.int64), ("newton_iters", np.int64),
                        ("dc_iters", np.int64), ("hmin_seen", np.float64), ("hmax_seen", np.float64),
                        ("status", np.int32), ("pad", np.int32)])


class BatchDesc(C.Structure):
    _fields_ = [("n_templates", C.c_int32), ("templates", C.POINTER(CktDesc)), ("n_inst", C.c_int32),
                ("inst_template", c_int32_p), ("inst_par_off", c_int64_p), ("inst_par", c_double_p),
                ("inst_x0_off", c_int64_p), ("inst_x0", c_double_p), ("inst_dx_off", c_int64_p),
                ("inst_dx", c_double_p), ("n_probes", C.c_int32), ("probes", c_int32_p), ("n_samples", C.c_int32)]


class Costs(C.Structure):
    _fields_ = [("flops_eval", C.c_int64), ("flops_stamp", C.c_int64), ("flops_lu", C.c_int64),
                ("flops_solve", C.c_int64), ("flops_update", C.c_int64), ("bytes", C.c_int64),
                ("lu_levels", C.c_int32), ("fw_levels", C.c_int32), ("bw_levels", C.c_int32), ("nnz_lu", C.c_int32),
                ("ordering", C.c_int32), ("pad", C.c_int32), ("bytes_eval", C.c_int64)]


class Objective(C.Structure):
    _fields_ = [("vnode", C.c_int32), ("ibranch", C.c_int32), ("probe", C.c_int32), ("pad", C.c_int32),
                ("level", C.c_double), ("w_energy", C.c_double), ("w_delay", C.c_double), ("w_final", C.c_double)]


class BatchTuning(C.Structure):
    _fields_ = [("lanes_per_inst", C.c_int32), ("warps_per_cta", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("reserved", C.c_int32 * 5)]


def ptr(a: Optional[np.ndarray], ctype):
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    return a.ctypes.data_as(C.POINTER(ctype))


class DescHolder:
    """A CktDesc plus the arrays it references."""

    def __init__(self, flat: Flat, ordering: int = None):
        self.flat = flat
        if ordering is None:
            ordering = getattr(flat, "ordering", 0)
        self.keep: List[object] = []
        gs = (DevGroup * max(1, len(flat.groups)))()
        for k, (model, term, br, par) in enumerate(flat.groups):
            term = np.ascontiguousarray(term, dtype=np.int32)
            par = np.ascontiguousarray(par, dtype=np.float64)
            br = None if br is None else np.ascontiguousarray(br, dtype=np.int32)
            self.keep += [term, par, br]
            gs[k].model = model
            gs[k].n_inst = term.shape[0]
            gs[k].term = ptr(term, C.c_int32)
            gs[k].branch = ptr(br, C.c_int32)
            gs[k].par = ptr(par, C.c_double)
        self.groups = gs
        pwl = np.ascontiguousarray(flat.pwl, dtype=np.float64)
        self.keep.append(pwl)
        self.desc = CktDesc(flat.n_nodes, flat.n_branch, len(flat.groups), gs,
                            ptr(pwl if pwl.size else None, C.c_double), pwl.size, flat.temp_c, flat.gmin,
                            int(ordering), 0)


def make_opts(method="bdf2", adaptive=True, tstart=0.0, tstop=1.0, h=0.0, dcop=True, reltol=1e-6, abstol_v=1e-9,
              abstol_i=1e-12, nr_factor=1e-3, hfirst_frac=1e-2, hmin=0.0, hmax=0.0, max_newton=20,
              max_steps=0) -> TranOpts:
    m = {"trap": CEDAR_TRAP, "trapezoidal": CEDAR_TRAP, "bdf2": CEDAR_BDF2}[method.lower()] if isinstance(method, str) else int(method)
    return TranOpts(m, int(bool(adaptive)), int(bool(dcop)), int(max_newton), int(max_steps), float(tstart),
                    float(tstop), float(h), float(hmin), float(hmax), float(reltol), float(abstol_v),
                    float(abstol_i), float(nr_factor), float(hfirst_frac))


class BatchHolder:
    """A BatchDesc for instances sharing templates (each a Flat)."""

    def __init__(self, templates: Sequence[Flat], inst_template: np.ndarray, inst_par: Optional[np.ndarray] = None,
                 inst_par_off: Optional[np.ndarray] = None, inst_x0: Optional[np.ndarray] = None,
                 inst_x0_off: Optional[np.ndarray] = None, inst_dx: Optional[np.ndarray] = None,
                 inst_dx_off: Optional[np.ndarray] = None, probes: Optional[np.ndarray] = None,
                 n_samples: int = 0):
        self.templates = [DescHolder(f) for f in templates]
        self.tdescs = (CktDesc * len(self.templates))(*[h.desc for h in self.templates])
        a = lambda x, dt: None if x is None else np.ascontiguousarray(x, dtype=dt)
        self.inst_template = a(inst_template, np.int32)
        self.inst_par = a(inst_par, np.float64)
        self.inst_par_off = a(inst_par_off, np.int64)
        self.inst_x0 = a(inst_x0, np.float64)
        self.inst_x0_off = a(inst_x0_off, np.int64)
        self.inst_dx = a(inst_dx, np.float64)
        self.inst_dx_off = a(inst_dx_off, np.int64)
        self.probes = a(probes, np.int32)
        n_probes = 0 if self.probes is None else self.probes.shape[-1]
        self.desc = BatchDesc(len(self.templates), self.tdescs, len(self.inst_template),
                              ptr(self.inst_template, C.c_int32), ptr(self.inst_par_off, C.c_int64),
                              ptr(self.inst_par, C.c_double), ptr(self.inst_x0_off, C.c_int64),
                              ptr(self.inst_x0, C.c_double), ptr(self.inst_dx_off, C.c_int64),
                              ptr(self.inst_dx, C.c_double), n_probes, ptr(self.probes, C.c_int32),
                              int(n_samples))

    @property
    def n_inst(self) -> int:
        return len(self.inst_template)


# ------------------------------------------------------------------ library
PKG = pathlib.Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libcedar_gpu.so"

# every symbol include/cedar.h declares
EXPORTS = [
    "cedar_last_error", "cedar_version", "cedar_model_nterm", "cedar_model_npar", "cedar_model_has_branch",
    "cedar_tran_opts_default", "cedar_ckt_create", "cedar_plan_create", "cedar_ckt_destroy", "cedar_ckt_size", "cedar_ckt_pattern",
    "cedar_ckt_costs", "cedar_ckt_symbolic", "cedar_eval", "cedar_eval_dev", "cedar_eval_dev_noalloc", "cedar_eval_scratch", "cedar_newton_solve", "cedar_dcop", "cedar_tran_run", "cedar_ckt_last_ms", "cedar_ckt_set_engine", "cedar_ckt_last_blocks",
    "cedar_batch_create", "cedar_batch_destroy", "cedar_batch_run", "cedar_batch_start", "cedar_batch_advance",
    "cedar_batch_results", "cedar_batch_last_ms", "cedar_batch_set_tuning",
    "cedar_batch_get_tuning", "cedar_batch_autotune", "cedar_batch_nmax",
    "cedar_adjoint_run", "cedar_adjoint_nparams", "cedar_adjoint_tape", "cedar_adjoint_last_ms",
    "cedar_fp64_probe", "cedar_fp64_latency", "cedar_ckt_stream", "cedar_batch_dcop", "cedar_ac", "cedar_noise",
    "cedar_ac_last_stats", "cedar_va_count", "cedar_va_name",
]

_lib = None


def load_library(build_if_missing: bool = True):
    """Load libcedar_gpu.so (building it in-tree if needed).  Raises if it cannot."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        from . import build as _b
        _b.build()
    if not LIB_PATH.exists():
        raise RuntimeError(f"CUDA library {LIB_PATH} is missing; run build()")
    lib = C.CDLL(str(LIB_PATH))
    P = C.c_void_p
    sig = {
        "cedar_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
        "cedar_version": (C.c_int, []),
        "cedar_model_nterm": (C.c_int, [C.c_int]),
        "cedar_model_npar": (C.c_int, [C.c_int]),
        "cedar_model_has_branch": (C.c_int, [C.c_int]),
        "cedar_tran_opts_default": (None, [C.POINTER(TranOpts)]),
        "cedar_ckt_create": (C.c_int, [C.POINTER(CktDesc), C.POINTER(P)]),
        "cedar_plan_create": (C.c_int, [C.POINTER(CktDesc), C.POINTER(P)]),
        "cedar_ckt_destroy": (C.c_int, [P]),
        "cedar_ckt_size": (C.c_int, [P, c_int32_p, c_int32_p, c_int32_p, c_int32_p]),
        "cedar_ckt_pattern": (C.c_int, [P, c_int32_p, c_int32_p]),
        "cedar_ckt_costs": (C.c_int, [P, C.POINTER(Costs)]),
        "cedar_ckt_symbolic": (C.c_int, [P, c_int32_p, c_int32_p, c_int32_p, c_int32_p]),
        "cedar_eval": (C.c_int, [P, c_double_p, c_double_p, C.c_double, C.c_double, c_double_p, c_double_p]),
        "cedar_eval_dev": (C.c_int, [P, P, P, C.c_double, C.c_double, P, P]),
        "cedar_eval_dev_noalloc": (C.c_int, [P, P, P, C.c_double, C.c_double, P, P, P]),
        "cedar_eval_scratch": (C.c_int, [P, c_int64_p, c_int64_p, c_int64_p]),
        "cedar_newton_solve": (C.c_int, [P, C.c_double, C.c_double, c_double_p, c_double_p, C.POINTER(Stats)]),
        "cedar_dcop": (C.c_int, [P, C.c_double, c_double_p, C.POINTER(Stats)]),
        "cedar_tran_run": (C.c_int, [P, C.POINTER(TranOpts), c_double_p, c_double_p, c_double_p, C.c_int64,
                                     c_int64_p, C.POINTER(Stats)]),
        "cedar_ckt_last_ms": (C.c_int, [P, c_double_p]),
        "cedar_ckt_set_engine": (C.c_int, [P, C.c_int32, C.c_int32]),
        "cedar_ckt_last_blocks": (C.c_int, [P, c_int32_p]),
        "cedar_batch_create": (C.c_int, [C.POINTER(BatchDesc), C.POINTER(P)]),
        "cedar_batch_destroy": (C.c_int, [P]),
        "cedar_batch_run": (C.c_int, [P, C.POINTER(TranOpts), c_double_p, c_double_p, P]),
        "cedar_batch_start": (C.c_int, [P, C.POINTER(TranOpts)]),
        "cedar_batch_advance": (C.c_int, [P, C.c_double, c_int32_p]),
        "cedar_batch_results": (C.c_int, [P, c_double_p, c_double_p, P]),
        "cedar_batch_last_ms": (C.c_int, [P, c_double_p]),
        "cedar_batch_set_tuning": (C.c_int, [P, C.POINTER(BatchTuning)]),
        "cedar_batch_get_tuning": (C.c_int, [P, C.POINTER(BatchTuning)]),
        "cedar_batch_autotune": (C.c_int, [P, C.POINTER(TranOpts), C.c_double, C.POINTER(BatchTuning)]),
        "cedar_batch_nmax": (C.c_int, [P, c_int32_p]),
        "cedar_adjoint_run": (C.c_int, [P, C.POINTER(TranOpts), C.POINTER(Objective), c_double_p, C.c_int64,
                                        c_double_p, c_double_p, c_int32_p, P]),
        "cedar_adjoint_nparams": (C.c_int, [P, c_int32_p, c_int32_p]),
        "cedar_adjoint_tape": (C.c_int, [P, C.c_int32, c_double_p, P, C.c_int64, c_int64_p]),
        "cedar_adjoint_last_ms": (C.c_int, [P, c_double_p, c_double_p]),
        "cedar_fp64_probe": (C.c_int, [C.c_int32, C.c_int32, c_double_p, c_double_p]),
        "cedar_fp64_latency": (C.c_int, [C.c_int32, c_double_p, c_double_p]),
        "cedar_ckt_stream": (C.c_int, [P, C.POINTER(P)]),
        "cedar_batch_dcop": (C.c_int, [P, C.POINTER(TranOpts), c_double_p, P]),
        "cedar_ac": (C.c_int, [P, c_double_p, c_double_p, C.c_int32, c_double_p, C.c_int32, c_int32_p, c_double_p,
                               c_int32_p]),
        "cedar_noise": (C.c_int, [P, c_double_p, C.c_int32, c_double_p, C.c_int32, c_double_p, c_int32_p]),
        "cedar_ac_last_stats": (C.c_int, [P, c_int32_p, c_double_p, c_double_p]),
        "cedar_va_count": (C.c_int, []),
        "cedar_va_name": (C.c_int, [C.c_int, C.c_char_p, C.c_size_t]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    # the library's Verilog-A models must be the ones the host registry assigns ids to
    from . import va
    names = []
    buf = C.create_string_buffer(256)
    for k in range(lib.cedar_va_count()):
        check(lib.cedar_va_name(k, buf, 256))
        names.append(buf.value.decode())
    want = [m.name for m in va.models()]
    if names != want:
        raise RuntimeError(f"{LIB_PATH} holds Verilog-A models {names}, the sources define {want}: rebuild it")
    _lib = lib
    return lib


class CedarError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"cedar error {code}: {msg}")
        self.code = code


def check(rc: int):
    if rc != 0:
        buf = C.create_string_buffer(1024)
        _lib.cedar_last_error(buf, 1024)
        raise CedarError(rc, buf.value.decode(errors="replace"))

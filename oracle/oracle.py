"""ctypes binding of the CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker / reported baseline, never by the
product package.
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
_lib = None


def build(force: bool = False) -> pathlib.Path:
    src = HERE / "oracle.cpp"
    hdr = HERE.parent / "include" / "cedar.h"
    gen = HERE.parent / "cedarsim.jl_gb300" / "_build" / "gen" / "va_models.gen.h"
    if not gen.exists():
        raise RuntimeError(f"{gen} is missing: build the package first (it emits the Verilog-A device code)")
    deps = [src, hdr, gen, HERE.parent / "cedarsim.jl_gb300" / "csrc" / "va_dual.cuh"]
    if force or not LIB.exists() or max(d.stat().st_mtime for d in deps) > LIB.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def load(pkg):
    """Load the oracle; `pkg` is the product package (for its descriptor types)."""
    global _lib
    if _lib is not None:
        return _lib
    # the Verilog-A device code the oracle compiles in comes from the package's emitter
    import importlib
    importlib.import_module(pkg.__name__ + ".build").generate()
    build()
    lib = C.CDLL(str(LIB))
    abi = pkg.abi
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int64)
    lib.oracle_eval.restype = C.c_int
    lib.oracle_eval.argtypes = [C.POINTER(abi.CktDesc), dp, dp, C.c_double, C.c_int, dp, dp, dp, dp, dp]
    lib.oracle_dcop.restype = C.c_int
    lib.oracle_dcop.argtypes = [C.POINTER(abi.CktDesc), C.POINTER(abi.TranOpts), C.c_double, dp, C.POINTER(abi.Stats)]
    lib.oracle_newton.restype = C.c_int
    lib.oracle_newton.argtypes = [C.POINTER(abi.CktDesc), C.POINTER(abi.TranOpts), C.c_double, C.c_double, dp, dp,
                                  C.POINTER(abi.Stats)]
    lib.oracle_tran.restype = C.c_int
    lib.oracle_tran.argtypes = [C.POINTER(abi.CktDesc), C.POINTER(abi.TranOpts), dp, dp, dp, C.c_int64, ip,
                                C.POINTER(abi.Stats)]
    lib.oracle_simple_diode.restype = C.c_int
    lib.oracle_simple_diode.argtypes = [dp, C.c_double, dp]
    lib.oracle_next_breakpoint.restype = C.c_double
    lib.oracle_next_breakpoint.argtypes = [C.POINTER(abi.CktDesc), C.c_double, C.c_double]
    lib.oracle_source_value.restype = C.c_double
    lib.oracle_source_value.argtypes = [C.POINTER(abi.CktDesc), C.c_int, C.c_int, C.c_double, C.c_int]
    lib.oracle_batch.restype = C.c_int
    lib.oracle_batch.argtypes = [C.POINTER(abi.BatchDesc), C.POINTER(abi.TranOpts), C.c_int32, C.c_int32, C.c_int32,
                                 dp, dp, C.c_void_p, C.c_int]
    obj_p, to_p, cd_p = C.POINTER(abi.Objective), C.POINTER(abi.TranOpts), C.POINTER(abi.CktDesc)
    lib.oracle_adjoint.restype = C.c_int
    lib.oracle_adjoint.argtypes = [cd_p, to_p, to_p, obj_p, C.c_double, dp, dp, dp, dp, C.c_void_p, C.c_int64, ip]
    lib.oracle_replay_phi.restype = C.c_int
    lib.oracle_replay_phi.argtypes = [cd_p, to_p, dp, C.c_void_p, C.c_int64, obj_p, C.c_double, dp, dp]
    lib.oracle_adjoint_batch.restype = C.c_int
    lib.oracle_adjoint_batch.argtypes = [C.POINTER(abi.BatchDesc), to_p, obj_p, dp, C.c_int32, C.c_int32, C.c_int32,
                                         dp, dp, C.POINTER(C.c_int32), C.c_int]
    lib.oracle_n_params.restype = C.c_int
    lib.oracle_n_params.argtypes = [cd_p]
    lib.oracle_va_full.restype = C.c_int
    lib.oracle_va_full.argtypes = [C.c_int, dp, dp, C.c_double, dp, dp, dp, dp]
    lib.oracle_va_ref_full.restype = C.c_int
    lib.oracle_va_ref_full.argtypes = [C.c_int, dp, C.c_int, dp, C.c_double, dp, dp, dp, dp]
    lib.oracle_va_noise.restype = C.c_int
    lib.oracle_va_noise.argtypes = [C.c_int, dp, dp, C.c_double, dp, dp]
    lib.oracle_last_error.restype = C.c_int
    lib.oracle_last_error.argtypes = [C.c_char_p, C.c_size_t]
    _lib = lib
    return lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    def __init__(self, pkg):
        self.pkg = pkg
        self.lib = load(pkg)

    def eval(self, flat, x, xdot=None, t=0.0, dc=False):
        h = self.pkg.abi.DescHolder(flat)
        n = flat.n
        x = np.ascontiguousarray(x, np.float64)
        xdot = None if xdot is None else np.ascontiguousarray(xdot, np.float64)
        F, Fi, Fq = np.zeros(n), np.zeros(n), np.zeros(n)
        G, Cm = np.zeros((n, n)), np.zeros((n, n))
        rc = self.lib.oracle_eval(C.byref(h.desc), _dp(x), _dp(xdot), t, int(dc), _dp(F), _dp(Fi), _dp(Fq), _dp(G), _dp(Cm))
        assert rc == 0
        return F, Fi, Fq, G, Cm

    # SimpleDiode's defaults (src/simpledevices.jl:152-168), in the struct's field order
    SIMPLE_DIODE_DEFAULTS = dict(AREA=1.0, BV=3.40282e38, BVJ=3.40282e38, CJO=0.0, EG=1.11, FC=0.5, IBV=1e-3,
                                 IS=1e-14, KF=0.0, M=0.5, N=1.0, RS=0.0, TNOM=27.0, TT=0.0, VJ=1.0, XTI=3.0)

    def simple_diode(self, vd, **params):
        """The reference's SimpleDiode restated literally at junction voltage vd
        (parity unpinned; see oracle_simple_diode).  Returns (code, Id, Ideff,
        Cdeplete, TT, Cdiffuse in DC); code 1 / 2: the reference reads an undefined
        name (NVt / MJI), 3: sqrt of a negative number."""
        p = dict(self.SIMPLE_DIODE_DEFAULTS)
        for k, v in params.items():
            if k not in p:
                raise KeyError(k)
            p[k] = float(v)
        arr = np.array(list(p.values()), np.float64)
        out = np.full(5, np.nan)
        rc = self.lib.oracle_simple_diode(_dp(arr), float(vd), _dp(out))
        return (rc, *out)

    # ---- small-signal AC and noise (dense complex solves; LAPACK partial pivoting)
    def ac_drive(self, flat, x_op):
        """b = -dFi/d(eps) of the AC sources, from the oracle's own source equations:
        in :ac mode a source's value is dc + eps |ac| (src/simpledevices.jl:292-294,
        331-333), and Fi is linear in it, so a unit step of eps is exact."""
        import copy
        _, fi0, _, _, _ = self.eval(flat, x_op, dc=True)
        f2 = copy.deepcopy(flat)
        for name, mag in flat.ac.items():
            gi, ii = f2.devices[name]
            f2.groups[gi][3][1, ii] += mag          # raw parameter 1 = dc value
        _, fi1, _, _, _ = self.eval(f2, x_op, dc=True)
        return -(fi1 - fi0)

    def ac(self, flat, x_op, omegas, probes, b=None):
        """X(j omega)[probes] with (G + j omega C) X = b, G, C the oracle's dense
        partials at x_op (ACSol + freqresp, src/ac.jl:73-104,251-258)."""
        _, _, _, G, Cm = self.eval(flat, x_op, dc=True)
        b = self.ac_drive(flat, x_op) if b is None else np.asarray(b, np.float64)
        out = np.zeros((len(omegas), len(probes)), complex)
        for k, w in enumerate(omegas):
            out[k] = np.linalg.solve(G + 1j * w * Cm, b.astype(complex))[list(probes)]
        return out

    def noise(self, flat, x_op, omegas, probe):
        """Output PSD at `probe` (PSD, src/ac.jl:263-283): one direct solve per
        resistor thermal-noise current, pwr = 4 k T / r (src/simpledevices.jl:70-75),
        and per noise source of a Verilog-A device (its power and exponent at
        x_op from the interpreter; density pwr / f^exp, f = omega / 2 pi), scaled
        by the multiplicity like the branch current (src/simulate_ir.jl:54)."""
        _, _, _, G, Cm = self.eval(flat, x_op, dc=True)
        n = flat.n
        kT4 = 4.0 * 1.380649e-23 * (flat.temp_c + 273.15)
        cols, pwr, ex = [], [], []
        for inj, pw, e in self._va_noise(flat, x_op):
            cols.append(inj)
            pwr.append(pw)
            ex.append(e)
        for (model, term, br, par) in flat.groups:
            if model != 1:
                continue
            for i in range(par.shape[1]):
                inj = np.zeros(n)
                a, c = term[i, 0], term[i, 1]
                if a >= 0:
                    inj[a] += par[1, i]
                if c >= 0:
                    inj[c] -= par[1, i]
                cols.append(inj)
                pwr.append(kT4 / par[0, i])
                ex.append(0.0)
        out = np.zeros(len(omegas))
        if not cols:
            return out
        INJ, pwr, ex = np.array(cols).T.astype(complex), np.array(pwr), np.array(ex)
        for k, w in enumerate(omegas):
            H = np.linalg.solve(G + 1j * w * Cm, INJ)[probe]
            f = w / (2.0 * np.pi)
            dens = np.array([p if e == 0.0 else p / f ** e for p, e in zip(pwr, ex)])
            out[k] = float(np.sum(dens * np.abs(H) ** 2))
        return out

    def _va_noise(self, flat, x_op):
        """Injection vectors, powers (m^2 pwr) and exponents of the Verilog-A
        devices' noise sources at x_op, from the independent interpretation of
        their modules (oracle/va_interp.py)."""
        import importlib.util
        va = self.pkg.va
        spec = importlib.util.spec_from_file_location("cedar_va_interp", HERE / "va_interp.py")
        vi = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(vi)
        vt = 1.380649e-23 * (flat.temp_c + 273.15) / 1.602176634e-19
        out = []
        for (model, term, br, par) in flat.groups:
            if model < va.BASE_ID:
                continue
            m = va.model(model)
            if not m.noise:
                continue
            names = [p.name for p in m.params]
            for i in range(par.shape[1]):
                vals = par[:, i]
                prm = dict(zip(names, vals[:len(names)]))
                given = [g for j, g in enumerate(m.given) if vals[len(names) + j] != 0.0]
                idx = list(term[i]) + ([int(br[i])] if br is not None else [])
                v = [x_op[u] if u >= 0 else 0.0 for u in idx]
                mult = vals[-1]
                for (a, b), pw, e in vi.noise_sources(m.module, prm, v, vt, flat.gmin, mult, given):
                    inj = np.zeros(flat.n)
                    if idx[a] >= 0:
                        inj[idx[a]] += mult
                    if b >= 0 and idx[b] >= 0:
                        inj[idx[b]] -= mult
                    out.append((inj, pw, e))
        return out

    def dcop(self, flat, t=0.0, x0=None, opts=None):
        h = self.pkg.abi.DescHolder(flat)
        x = np.zeros(flat.n) if x0 is None else np.ascontiguousarray(x0, np.float64).copy()
        o = opts or self.pkg.make_opts(tstop=1.0)
        st = self.pkg.abi.Stats()
        rc = self.lib.oracle_dcop(C.byref(h.desc), C.byref(o), t, _dp(x), C.byref(st))
        return x, st, rc

    def newton(self, flat, t, cj, hist, x0, opts=None):
        h = self.pkg.abi.DescHolder(flat)
        x = np.ascontiguousarray(x0, np.float64).copy()
        hist = None if hist is None else np.ascontiguousarray(hist, np.float64)
        o = opts or self.pkg.make_opts(tstop=1.0)
        st = self.pkg.abi.Stats()
        rc = self.lib.oracle_newton(C.byref(h.desc), C.byref(o), t, cj, _dp(hist), _dp(x), C.byref(st))
        return x, st, rc

    def tran(self, flat, opts, x0=None, cap=1 << 20):
        h = self.pkg.abi.DescHolder(flat)
        x = np.zeros(flat.n) if x0 is None else np.ascontiguousarray(x0, np.float64).copy()
        t_out = np.zeros(cap)
        x_out = np.zeros((cap, flat.n))
        n_out = C.c_int64()
        st = self.pkg.abi.Stats()
        rc = self.lib.oracle_tran(C.byref(h.desc), C.byref(opts), _dp(x), _dp(t_out), _dp(x_out), cap, C.byref(n_out), C.byref(st))
        m = min(n_out.value, cap)
        return t_out[:m].copy(), x_out[:m].copy(), st, rc

    def batch(self, holder, opts, i0=0, i1=None, n_max=None, nthreads=0, want_samples=True):
        i1 = holder.n_inst if i1 is None else i1
        if n_max is None:
            n_max = max(f.flat.n for f in holder.templates)
        cnt = i1 - i0
        xf = np.zeros((cnt, n_max))
        np_ = holder.desc.n_probes
        ns = holder.desc.n_samples
        samp = np.zeros((cnt, np_, ns)) if (want_samples and np_ and ns) else None
        st = np.zeros(cnt, self.pkg.abi.STATS_DTYPE)
        rc = self.lib.oracle_batch(C.byref(holder.desc), C.byref(opts), i0, i1, n_max, _dp(xf), _dp(samp),
                                   st.ctypes.data_as(C.c_void_p), nthreads)
        assert rc == 0
        return xf, samp, st

    def adjoint(self, flat, fwd_opts, replay_opts, obj, tstar, perturb=None, cap=1 << 22):
        """Forward run recording its accepted steps, then the discrete adjoint along
        them.  Returns (phi, grad[MOS1 W..., R r...], t_rec, ord_rec)."""
        h = self.pkg.abi.DescHolder(flat)
        npar = self.lib.oracle_n_params(C.byref(h.desc))
        grad = np.zeros(max(npar, 1))
        t_rec = np.zeros(cap)
        ord_rec = np.zeros(cap, np.int8)
        nrec = C.c_int64()
        phi = C.c_double()
        pert = None if perturb is None else np.ascontiguousarray(perturb, np.float64)
        rc = self.lib.oracle_adjoint(C.byref(h.desc), C.byref(fwd_opts), C.byref(replay_opts), C.byref(obj), tstar,
                                     _dp(pert), C.byref(phi), _dp(grad), _dp(t_rec),
                                     ord_rec.ctypes.data_as(C.c_void_p), cap, C.byref(nrec))
        assert rc == 0, rc
        m = min(nrec.value, cap)
        return phi.value, grad[:npar].copy(), t_rec[:m].copy(), ord_rec[:m].copy()

    def replay_phi(self, flat, replay_opts, t_rec, ord_rec, obj, tstar, perturb=None):
        """The objective along a fixed step sequence (central differences use this)."""
        h = self.pkg.abi.DescHolder(flat)
        t_rec = np.ascontiguousarray(t_rec, np.float64)
        ord_rec = np.ascontiguousarray(ord_rec, np.int8)
        phi = C.c_double()
        pert = None if perturb is None else np.ascontiguousarray(perturb, np.float64)
        rc = self.lib.oracle_replay_phi(C.byref(h.desc), C.byref(replay_opts), _dp(t_rec),
                                        ord_rec.ctypes.data_as(C.c_void_p), len(t_rec), C.byref(obj), tstar,
                                        _dp(pert), C.byref(phi))
        assert rc == 0, rc
        return phi.value

    def adjoint_batch(self, holder, opts, objectives, tstar, i0=0, i1=None, np_max=None, nthreads=0):
        """Oracle adjoint over batch instances [i0, i1) with OpenMP; objectives per template."""
        i1 = holder.n_inst if i1 is None else i1
        if np_max is None:
            np_max = max(self.lib.oracle_n_params(C.byref(t.desc)) for t in holder.templates)
        cnt = i1 - i0
        obj = (self.pkg.abi.Objective * len(objectives))(*objectives)
        ts = np.ascontiguousarray(tstar, np.float64)
        phi = np.zeros(cnt)
        grad = np.zeros((cnt, max(np_max, 1)))
        status = np.zeros(cnt, np.int32)
        rc = self.lib.oracle_adjoint_batch(C.byref(holder.desc), C.byref(opts), obj, _dp(ts), i0, i1, np_max,
                                           _dp(phi), _dp(grad), status.ctypes.data_as(C.POINTER(C.c_int32)), nthreads)
        assert rc == 0, rc
        return phi, grad[:, :np_max], status


"""The Verilog-A emitter end to end on the host, for modules that are not shipped.

Test-only modules that exercise the whole supported subset are emitted into a
header, compiled with g++ into a small library, and their residuals, Jacobians
and noise powers compared with the independent interpretation of the same
parsed modules (oracle/va_interp.py) at random port potentials.  The device
code the engines run is this same emitted C++."""
import ctypes as C
import importlib.util
import pathlib
import shutil
import subprocess

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
CSRC = ROOT / "cedarsim.jl_gb300" / "csrc"
VT = 1.380649e-23 * (27.0 + 273.15) / 1.602176634e-19

SOURCES = r"""
`include "disciplines.vams"
`include "constants.vams"
`define SQ(x) ((x) * (x))
`define SOFTABS(x, e) sqrt(`SQ(x) + (e))
`ifdef UNDEFINED_FLAG
`define K0 0.0
`else
`define K0 0.25
`endif

// internal node, function, case, integer arithmetic, ternary, min / max
module t_mix(a, b, c);
  inout a, b, c;
  electrical a, b, c, x;
  parameter real G = 1m from (0:inf);
  parameter real R = 100.0 from (0:inf);
  parameter integer SEL = 1 from [0:3];
  parameter real P = 1.5;
  real u, w, s;
  integer k;

  analog function real soft;
    input y, e;
    real y, e, t;
    begin
      t = `SOFTABS(y, e);
      soft = 0.5 * (y + t);
    end
  endfunction

  analog begin
    @(initial_step) $strobe("t_mix");
    k = SEL / 2 + 7 / 2;          // integer division
    u = V(a, x);
    case (SEL)
      0: w = G * u;
      1, 2: w = G * soft(u, 1e-3) * `K0 * 4.0;
      default: w = G * tanh(u) * (k > 3 ? 2.0 : 1.0);
    endcase
    s = min(V(b), max(V(c), -0.5)) + pow(abs(V(b, c)) + 1.0, P) * 1e-3;
    I(a, x) <+ w + white_noise(4.0 * P_K * $temperature * G, "ch");
    I(x, c) <+ V(x, c) / R + 1e-4 * atan2(V(b), 1.0 + `SQ(V(c))) + 1e-5 * hypot(V(a), V(b)) + 1e-4 * s;
    I(b) <+ 1e-6 * limexp(V(b) * 10.0) + ddt(1e-12 * V(b) + 1e-13 * `SQ(V(b, c)));
  end
endmodule

// voltage branch probing its own current, $param_given, ddt on the branch,
// $limit, ddx on a single-node probe
module t_branch(p, n, g);
  inout p, n, g;
  electrical p, n, g;
  parameter real L = 1n from (0:inf);
  parameter real RS = 5.0 from [0:inf);
  parameter real K = 2.0;
  real q, vg;
  analog begin
    vg = $limit(V(g), "fetlim", 0.0);
    q = K * vg * vg;
    if ($param_given(RS))
      V(p, n) <+ RS * I(p, n) + ddt(L * I(p, n));
    else
      V(p, n) <+ 0.5 * ddx(q, V(g)) + ddt(L * I(p, n));
    I(g) <+ V(g) * 1e-3;
  end
endmodule

// for / while / repeat loops, a function with output arguments
module t_loop(a, b);
  inout a, b;
  electrical a, b;
  parameter integer NSEG = 4 from [1:16];
  parameter real G = 1m;
  real acc, x, y, lo, hi;
  integer i;

  analog function real split;
    input v;
    output p, q;
    real v, p, q;
    begin
      p = 0.5 * v + 0.1 * v * v;
      q = v - p;
      split = p * q;
    end
  endfunction

  analog begin
    acc = 0.0;
    x = V(a, b);
    for (i = 0; i < NSEG; i = i + 1)
      acc = acc + G * x / NSEG * (1.0 + 0.1 * i);
    i = 0;
    while (i < 3) begin
      acc = acc + 1e-6 * x * x;
      i = i + 1;
    end
    repeat (2) acc = acc * 1.01;
    y = split(x, lo, hi);
    I(a, b) <+ acc + 1e-4 * (lo - hi) + 1e-5 * y;
  end
endmodule
"""


@pytest.fixture(scope="module")
def emitted(pkg, tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    import importlib
    P = importlib.import_module("cedarsim_gb300.va.parser")
    E = importlib.import_module("cedarsim_gb300.va.emit")
    mods = sorted((E.analyze(m) for m in P.parse(SOURCES)), key=lambda ma: ma[0].name)
    d = tmp_path_factory.mktemp("va_host")
    (d / "va_models.gen.h").write_text(E.emit_header(mods, 11))
    (d / "harness.cpp").write_text(
        '#include <math.h>\n#include "va_models.gen.h"\n'
        'extern "C" int h_full(int k, const double *dp, const double *v, double gmin, double *fi, double *fq,'
        ' double *G, double *C) { cedar::va::full(k, dp, 1, v, gmin, fi, fq, G, C); return 0; }\n'
        'extern "C" int h_noise(int k, const double *dp, const double *v, double gmin, double *pw, double *ex)'
        ' { return cedar::va::noise(k, dp, 1, v, gmin, pw, ex); }\n')
    lib = d / "libharness.so"
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I", str(CSRC), "-I",
                        str(d), str(d / "harness.cpp"), "-o", str(lib)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    h = C.CDLL(str(lib))
    dp = C.POINTER(C.c_double)
    h.h_full.argtypes = [C.c_int, dp, dp, C.c_double, dp, dp, dp, dp]
    h.h_noise.argtypes = [C.c_int, dp, dp, C.c_double, dp]
    return h, [m for m, _ in mods]


@pytest.fixture(scope="module")
def interp():
    spec = importlib.util.spec_from_file_location("cedar_va_interp_h", ROOT / "oracle" / "va_interp.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_emitted_host_code_matches_interpreter(emitted, interp):
    h, models = emitted
    rng = np.random.default_rng(123)
    dp_ = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    for k, m in enumerate(models):
        n = m.nx
        assert (m.name, n) in (("t_branch", 4), ("t_mix", 4), ("t_loop", 2))
        for trial in range(80):
            over = {}
            if m.name == "t_mix":
                over = {"SEL": float(rng.integers(0, 4)), "P": float(rng.uniform(0.5, 2.5)),
                        "G": float(rng.uniform(1e-4, 1e-2))}
            elif m.name == "t_loop":
                over = {"NSEG": float(rng.integers(1, 17)), "G": float(rng.uniform(1e-4, 1e-2))}
            elif rng.random() < 0.5:
                over = {"RS": float(rng.uniform(0.0, 20.0))}
            vals = m.defaults(over)
            dp = np.array(vals + [1.0 + rng.integers(0, 2), VT])
            v = rng.uniform(-1.5, 1.5, n)
            fi, fq, G, Cm = np.zeros(n), np.zeros(n), np.zeros(n * n), np.zeros(n * n)
            h.h_full(k, dp_(dp), dp_(v), 1e-12, dp_(fi), dp_(fq), dp_(G), dp_(Cm))
            given = [g for g in m.given if g in over]
            ri, rq, rG, rC = interp.evaluate(m.module, dict(zip([p.name for p in m.params], vals)), list(v), VT,
                                             1e-12, float(dp[-2]), given)
            ri, rq, rG, rC = map(np.asarray, (ri, rq, rG, rC))
            assert np.all(np.abs(fi - ri) <= 1e-13 * (np.abs(ri).max() + 1e-30)), (m.name, over, fi, ri)
            assert np.all(np.abs(fq - rq) <= 1e-13 * (np.abs(rq).max() + 1e-40)), (m.name, fq, rq)
            assert np.all(np.abs(G - rG.ravel()) <= 1e-12 * (np.abs(rG).max() + 1e-30)), (m.name, over, G, rG)
            assert np.all(np.abs(Cm - rC.ravel()) <= 1e-12 * (np.abs(rC).max() + 1e-40)), (m.name, Cm, rC)
            if m.noise:
                pw, ex = np.zeros(len(m.noise)), np.full(len(m.noise), np.nan)
                assert h.h_noise(k, dp_(dp), dp_(v), 1e-12, dp_(pw), dp_(ex)) == len(m.noise)
                src = interp.noise_sources(m.module, dict(zip([p.name for p in m.params], vals)), list(v), VT, 1e-12,
                                           float(dp[-2]), given)
                assert [s[0] for s in src] == m.noise
                np.testing.assert_allclose(pw, [s[1] for s in src], rtol=1e-14)
                np.testing.assert_allclose(ex, [s[2] for s in src], rtol=1e-14)


def test_emitted_structure(emitted):
    _, models = emitted
    mix = next(m for m in models if m.name == "t_mix")
    assert mix.internals == ["x"] and mix.nterm == 4 and mix.has_br == 0
    assert mix.noise == [(0, 3)]                       # white_noise across (a, x)
    assert (1, 1) in mix.cents and (1, 2) in mix.cents  # ddt charge of port b depends on b and c
    br = next(m for m in models if m.name == "t_branch")
    assert br.has_br == 1 and br.nx == 4 and br.given == ["RS"] and br.second_order
    assert (3, 3) in br.cents                          # ddt(L I) on the branch row


def test_emitted_code_compiles_for_the_device(emitted, tmp_path):
    """The same emitted header (functions with output arguments, loops, voltage
    branches, second-order duals) compiles for sm_103a inside a kernel."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not pathlib.Path(nvcc).exists():
        pytest.skip("nvcc not available")
    h, models = emitted
    gen_dir = pathlib.Path(h._name).parent
    (tmp_path / "k.cu").write_text(
        '#include "va_models.gen.h"\n'
        '__global__ void k(int m, const double *dp, const double *v, double *out) {\n'
        '  cedar::va::eval(m, dp, 1, v, v, false, 1e12, 1e-12, out, 1);\n}\n')
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-c", "-I", str(CSRC),
                        "-I", str(gen_dir), str(tmp_path / "k.cu"), "-o", str(tmp_path / "k.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]



def test_wide_model_widens_engine_staging(pkg, tmp_path):
    """A module with 6 terminal values (4 ports, 2 internal nodes) makes the
    generated header define CEDAR_MAX_TERM 6, and the one-circuit engine's
    translation unit compiles for sm_103a with the wider staging; the shipped
    models keep the built-ins' 5."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not pathlib.Path(nvcc).exists():
        pytest.skip("nvcc not available")
    import importlib
    P = importlib.import_module("cedarsim_gb300.va.parser")
    E = importlib.import_module("cedarsim_gb300.va.emit")
    src = """module wide(d, g, s, b); inout d, g, s, b; electrical d, g, s, b, di, si;
      parameter real RD = 10.0, RS = 10.0, K = 1m;
      analog begin
        I(d, di) <+ V(d, di) / RD; I(s, si) <+ V(s, si) / RS;
        I(di, si) <+ K * V(g, si) * V(di, si) + 1e-12 * V(b, si);
      end endmodule"""
    mods = [E.analyze(m) for m in P.parse(src)]
    assert mods[0][0].nx == 6
    text = E.emit_header(mods, 11)
    assert "#define CEDAR_MAX_TERM 6" in text
    (tmp_path / "va_models.gen.h").write_text(text)
    shipped = pkg.va.models()
    assert "CEDAR_MAX_TERM" not in E.emit_header([E.analyze(m.module) for m in shipped], 11)
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O3",
                        "--expt-relaxed-constexpr", "-c", "-I", str(tmp_path), "-I", str(ROOT / "include"),
                        "-I", str(CSRC), str(CSRC / "k_plain.cu"), "-o", str(tmp_path / "k.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


def test_strong_zero_partials(pkg, tmp_path):
    """Where f' is infinite (sqrt, pow at 0) the partials along directions the
    argument does not depend on stay 0, not 0 * inf = NaN (host-compiled code and
    interpreter alike)."""
    import importlib
    P = importlib.import_module("cedarsim_gb300.va.parser")
    E = importlib.import_module("cedarsim_gb300.va.emit")
    src = """module sz(a, b, c); inout a, b, c; electrical a, b, c;
      analog begin
        I(a) <+ 1e-3 * sqrt(V(a)) + 1e-3 * V(b);
        I(c) <+ 1e-3 * pow(V(c), 0.5) + 1e-3 * V(b);
      end endmodule"""
    mods = [E.analyze(m) for m in P.parse(src)]
    (tmp_path / "va_models.gen.h").write_text(E.emit_header(mods, 11))
    (tmp_path / "h.cpp").write_text('#include <math.h>\n#include "va_models.gen.h"\n'
                                    'extern "C" void h(const double *dp, const double *v, double *fi, double *fq, '
                                    'double *G, double *C) { cedar::va::full(0, dp, 1, v, 1e-12, fi, fq, G, C); }\n')
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-I", str(CSRC), "-I", str(tmp_path),
                        str(tmp_path / "h.cpp"), "-o", str(tmp_path / "h.so")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-1500:]
    lib = C.CDLL(str(tmp_path / "h.so"))
    dp_ = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    dp, v = np.array([1.0, VT]), np.array([0.0, 0.3, 0.0])
    fi, fq, G, Cm = np.zeros(3), np.zeros(3), np.zeros(9), np.zeros(9)
    lib.h(dp_(dp), dp_(v), dp_(fi), dp_(fq), dp_(G), dp_(Cm))
    G = G.reshape(3, 3)
    assert G[0, 1] == -1e-3 and G[2, 1] == -1e-3            # finite cross partials
    assert np.isinf(G[0, 0]) and np.isinf(G[2, 2])           # the genuine infinite slopes
    spec = importlib.util.spec_from_file_location("cedar_va_interp_sz", ROOT / "oracle" / "va_interp.py")
    vi = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(vi)
    _, _, rG, _ = vi.evaluate(mods[0][0].module, {}, list(v), VT, 1e-12)
    assert rG[0][1] == -1e-3 and rG[2][1] == -1e-3


def test_pow_gradient_rule(pkg, tmp_path):
    """d(x^p)/dx takes the values of CedarSim's pow derivative (src/va_env.jl:57-68,
    ChainRules' pow gradient): at x = 0, 0 for p = 0 or p > 1, 1 for p = 1, +inf
    for 0 < p < 1, and p x^(p-1) away from 0.  The base sqrt(V^2 + 0.01) - 0.1
    at V = 1e-10 rounds to exactly 0 while its own partial (1e-9) does not,
    which is how BSIM-CMG's smoothed V_ds reaches pow(vdsx, DVTP1 = 0): x^0 must
    have zero partials there, not 0 * inf = NaN."""
    import importlib
    P = importlib.import_module("cedarsim_gb300.va.parser")
    E = importlib.import_module("cedarsim_gb300.va.emit")
    src = """module pw(a, b, c, d, e, f); inout a, b, c, d, e, f; electrical a, b, c, d, e, f;
      analog begin
        I(a) <+ 1e-3 * pow(sqrt(V(a) * V(a) + 0.01) - 0.1, 0.0);
        I(b) <+ 1e-3 * pow(sqrt(V(b) * V(b) + 0.01) - 0.1, 1.0);
        I(c) <+ 1e-3 * pow(sqrt(V(c) * V(c) + 0.01) - 0.1, 2.0);
        I(d) <+ 1e-3 * pow(sqrt(V(d) * V(d) + 0.01) - 0.1, 0.5);
        I(e) <+ 1e-3 * pow(V(e), 3.0);
        I(f) <+ 1e-3 * pow(V(f), 0.0);
      end endmodule"""
    mods = [E.analyze(m) for m in P.parse(src)]
    (tmp_path / "va_models.gen.h").write_text(E.emit_header(mods, 11))
    (tmp_path / "h.cpp").write_text('#include <math.h>\n#include "va_models.gen.h"\n'
                                    'extern "C" void h(const double *dp, const double *v, double *fi, double *fq, '
                                    'double *G, double *C) { cedar::va::full(0, dp, 1, v, 1e-12, fi, fq, G, C); }\n')
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-I", str(CSRC), "-I", str(tmp_path),
                        str(tmp_path / "h.cpp"), "-o", str(tmp_path / "h.so")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-1500:]
    lib = C.CDLL(str(tmp_path / "h.so"))
    dp_ = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    vs = 1e-10
    assert np.sqrt(vs * vs + 0.01) - 0.1 == 0.0                 # the base rounds to exactly 0
    dbase = vs / np.sqrt(vs * vs + 0.01)                         # ... but moves with V
    dp, v = np.array([1.0, VT]), np.array([vs, vs, vs, vs, 0.7, 0.0])
    fi, fq, G, Cm = np.zeros(6), np.zeros(6), np.zeros(36), np.zeros(36)
    lib.h(dp_(dp), dp_(v), dp_(fi), dp_(fq), dp_(G), dp_(Cm))
    g = np.abs(np.diag(G.reshape(6, 6)))
    assert g[0] == 0.0 and g[5] == 0.0                            # p = 0: x^0 is constant
    assert g[1] == pytest.approx(1e-3 * dbase, rel=1e-15)         # p = 1: the base's own slope
    assert g[2] == 0.0                                            # p = 2 at x = 0
    assert np.isinf(g[3])                                         # p = 1/2 at x = 0
    assert g[4] == pytest.approx(1e-3 * 3 * 0.7 ** 2, rel=1e-15)  # p y / x away from 0
    spec = importlib.util.spec_from_file_location("cedar_va_interp_pw", ROOT / "oracle" / "va_interp.py")
    vi = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(vi)
    _, _, rG, _ = vi.evaluate(mods[0][0].module, {}, list(v), VT, 1e-12)
    rg = np.abs(np.diag(np.asarray(rG, dtype=float)))
    assert np.array_equal(np.isinf(rg), np.isinf(g))
    fin = np.isfinite(g)
    assert np.allclose(rg[fin], g[fin], rtol=1e-15, atol=0.0)


def _big_module(n_blocks: int) -> str:
    """A module with more statements than the split threshold: chains of
    assignments, nested ifs (one larger than a part), a loop, an analog function
    with an output argument, $param_given and a charge."""
    L = ["module big(a, b, c); inout a, b, c; electrical a, b, c;",
         "  parameter real G = 1m from (0:inf); parameter real K0 = 0.1;",
         "  real x, y, z, w, q; integer i;",
         "  analog function real sq; input u; real u; begin sq = u * u; end endfunction",
         "  analog function real tw; input u, o; real u, o; begin o = 2.0 * u; tw = u + o; end endfunction",
         "  analog begin",
         "    x = V(a, b); y = V(b, c); z = 0.0; w = 0.0; q = 0.0;"]
    for k in range(n_blocks):
        L.append(f"    z = z + {0.001 * (k + 1):.6f} * sq(x + {0.01 * k:.4f}) - 0.5 * y * {1.0 / (k + 2):.8f};")
        L.append(f"    w = w * 0.999 + tanh(z * {0.1 + 0.001 * k:.5f});")
        if k % 7 == 0:
            L.append(f"    if (x > {0.01 * k:.3f}) begin z = z - 0.001 * exp(-y * y); end else begin w = w + 1e-4; end")
    L.append("    if (x > -10.0) begin")
    for k in range(80):
        L.append(f"      q = q + {1e-3 / (k + 1):.8f} * sqrt(x * x + {k + 1}.0) + tw(y, w) * 1e-6;")
    L.append("    end else begin q = 0.0; end")
    L.append("    for (i = 0; i < 3; i = i + 1) begin q = q + 1e-6 * i; end")
    L.append("    if ($param_given(K0)) q = q * (1.0 + K0);")
    L.append("    I(a, b) <+ G * (x + z * 1e-3 + w * 1e-3);")
    L.append("    I(b, c) <+ G * y + ddt(1e-15 * q);")
    L.append("  end")
    L.append("endmodule")
    return "\n".join(L)


def test_split_emission_of_large_modules(pkg, tmp_path, monkeypatch):
    """A module whose analog block is larger than the split threshold is emitted
    as part functions over a frame (parameters, flags and variables in a
    struct); its host-compiled residuals, charges and Jacobians are bit for bit
    those of the same module emitted as one function, and match the
    interpreter."""
    import importlib
    P = importlib.import_module("cedarsim_gb300.va.parser")
    E = importlib.import_module("cedarsim_gb300.va.emit")
    src = _big_module(380)
    mod = P.parse(src)[0]
    assert E._stmt_count(mod.body) > E.SPLIT_STMTS

    def build(tag):
        mods = [E.analyze(m) for m in P.parse(src)]
        text = E.emit_header(mods, 11)
        d = tmp_path / tag
        d.mkdir()
        (d / "va_models.gen.h").write_text(text)
        (d / "h.cpp").write_text('#include <math.h>\n#include "va_models.gen.h"\n'
                                 'extern "C" void h(const double *dp, const double *v, double *fi, double *fq, '
                                 'double *G, double *C) { cedar::va::full(0, dp, 1, v, 1e-12, fi, fq, G, C); }\n')
        r = subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-I", str(CSRC), "-I", str(d),
                            str(d / "h.cpp"), "-o", str(d / "h.so")], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-1500:]
        return text, C.CDLL(str(d / "h.so"))
    split_text, split = build("split")
    assert split_text.count("VA_PART void part_big_") >= 5 and "struct Frame_big" in split_text
    monkeypatch.setattr(E, "SPLIT_STMTS", 10 ** 9)
    whole_text, whole = build("whole")
    assert "VA_PART" not in whole_text
    dp_ = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    m, _ = E.analyze(mod)
    spec = importlib.util.spec_from_file_location("cedar_va_interp_big", ROOT / "oracle" / "va_interp.py")
    vi = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(vi)
    rng = np.random.default_rng(5)
    for given in (False, True):
        vals = m.defaults({"K0": 0.1} if given else {})   # parameters, then the $param_given(K0) flag
        dp = np.array(vals + [1.0, VT])                    # then m and vt
        for _ in range(4):
            v = rng.uniform(-0.5, 1.0, 3)
            outs = []
            for lib in (split, whole):
                fi, fq, G, Cm = np.zeros(3), np.zeros(3), np.zeros(9), np.zeros(9)
                lib.h(dp_(dp), dp_(v), dp_(fi), dp_(fq), dp_(G), dp_(Cm))
                outs.append((fi, fq, G, Cm))
            for a, b in zip(*outs):
                assert np.array_equal(a, b)
            given_set = ["K0"] if given else []
            ri, rq, rG, rC = map(np.asarray, vi.evaluate(mod, dict(zip([p.name for p in m.params], vals)), list(v),
                                                          VT, 1e-12, 1.0, given_set))
            assert vals[-1] == (1.0 if given else 0.0)
            fi, fq, G, Cm = outs[0]
            assert np.allclose(fi, ri, rtol=1e-12, atol=1e-18) and np.allclose(fq, rq, rtol=1e-12, atol=1e-30)
            assert np.allclose(G, rG.ravel(), rtol=1e-11, atol=1e-18)

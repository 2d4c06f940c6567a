"""C-ABI library on the host (no GPU): exports, host-only analysis, error paths.

The library's J pattern, static pivot (row matching), ordering and LU fill are
compared bit for bit with the independent Python restatement in
oracle/symbolic_ref.py.
"""
import ctypes as C
import pathlib
import re

import numpy as np
import pytest

from tests import circuits as K

HEADER = pathlib.Path(__file__).resolve().parent.parent / "include" / "cedar.h"


def declared_functions():
    txt = HEADER.read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cedar_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib(pkg):
    return pkg.load_library()


def test_exports_every_declared_symbol(lib, pkg):
    names = declared_functions()
    assert len(names) >= 20
    for nm in names:
        assert hasattr(lib, nm), nm
    assert set(names) == set(pkg.abi.EXPORTS)


def test_model_tables(lib):
    assert [lib.cedar_model_nterm(m) for m in range(1, 11)] == [2, 2, 2, 2, 2, 4, 4, 4, 2, 3]
    assert [lib.cedar_model_npar(m) for m in range(1, 11)] == [2, 2, 2, 10, 10, 2, 2, 7, 4, 2]
    assert [lib.cedar_model_has_branch(m) for m in range(1, 11)] == [0, 0, 1, 1, 0, 1, 0, 0, 0, 0]
    assert lib.cedar_model_nterm(99) == -1


def plan(pkg, flat):
    lib = pkg.load_library()
    h = pkg.abi.DescHolder(flat)
    handle = C.c_void_p()
    rc = lib.cedar_plan_create(C.byref(h.desc), C.byref(handle))
    return lib, handle, rc


def lib_analysis(pkg, flat):
    lib, handle, rc = plan(pkg, flat)
    pkg.abi.check(rc)
    try:
        n, nj, nlu, nl = (C.c_int32() for _ in range(4))
        pkg.abi.check(lib.cedar_ckt_size(handle, C.byref(n), C.byref(nj), C.byref(nlu), C.byref(nl)))
        n = n.value
        cp = np.zeros(n + 1, np.int32); ri = np.zeros(nj.value, np.int32)
        pkg.abi.check(lib.cedar_ckt_pattern(handle, pkg.abi.ptr(cp, C.c_int32), pkg.abi.ptr(ri, C.c_int32)))
        rm = np.zeros(n, np.int32); order = np.zeros(n, np.int32)
        lcp = np.zeros(n + 1, np.int32); lri = np.zeros(nlu.value, np.int32)
        pkg.abi.check(lib.cedar_ckt_symbolic(handle, *(pkg.abi.ptr(a, C.c_int32) for a in (rm, order, lcp, lri))))
        # a host-only plan refuses GPU work
        x = np.zeros(n)
        assert lib.cedar_eval(handle, x.ctypes.data_as(C.POINTER(C.c_double)), None, 0.0, 0.0, None, None) == -1
        return cp, ri, rm, order, lcp, lri
    finally:
        lib.cedar_ckt_destroy(handle)


CASES = {
    "rc_ladder": lambda pkg: pkg.generators.rc_ladder(100),
    "inverter_chain_31": lambda pkg: pkg.generators.inverter_chain(31),
    "inverter_chain_5": lambda pkg: pkg.generators.inverter_chain(5),
    "mixed": K.mixed,
    "spice_sources": K.spice_sources,
    "butterworth": K.butterworth,
    "multiplicities": K.multiplicities,
}


@pytest.mark.parametrize("ordering", [1, 2])
@pytest.mark.parametrize("case", sorted(CASES))
def test_symbolic_bit_exact(pkg, symref, case, ordering):
    """J pattern, static pivot, ordering (minimum degree / nested dissection) and LU
    fill equal the independent restatement bit for bit."""
    flat = CASES[case](pkg).flatten()
    flat.ordering = ordering
    got = lib_analysis(pkg, flat)
    want = symref.analyze_with(flat, ordering)
    names = ["J colptr", "J rowidx", "rowmatch", "order", "LU colptr", "LU rowidx"]
    for nm, g, w in zip(names, got, want):
        assert list(g) == list(w), nm


@pytest.mark.parametrize("case", sorted(CASES))
def test_auto_ordering_picks_one_of_the_two(pkg, symref, case):
    flat = CASES[case](pkg).flatten()
    flat.ordering = 0
    order = list(lib_analysis(pkg, flat)[3])
    assert order in (list(symref.analyze_with(flat, 1)[3]), list(symref.analyze_with(flat, 2)[3]))


def test_rc_ladder_sizes(pkg):
    flat = pkg.generators.rc_ladder(100).flatten()
    flat.ordering = 1
    cp, ri, rm, order, lcp, lri = lib_analysis(pkg, flat)
    assert flat.n == 102 and len(ri) == 303   # n = 102, nnz(J) = 303
    assert len(lri) == 303                    # no fill under the chosen ordering


def test_errors(pkg):
    lib = pkg.load_library()
    # structurally singular: a floating node touched only by a current source
    c = pkg.Circuit(); c.I("I1", "a", "0", dc=1.0); c.R("R1", "b", "0", r=1.0)
    lib_, h, rc = plan(pkg, c.flatten())
    assert rc == -4  # CEDAR_ESINGULAR
    buf = C.create_string_buffer(256); lib.cedar_last_error(buf, 256)
    assert b"singular" in buf.value
    # out-of-range terminal
    f = K.vr(pkg).flatten()
    model, term, br, par = f.groups[0]
    bad = term.copy(); bad[0, 0] = 99
    f.groups[0] = (model, bad, br, par)
    lib_, h, rc = plan(pkg, f)
    assert rc == -1
    # null descriptor
    assert lib.cedar_plan_create(None, C.byref(C.c_void_p())) == -1


def test_vectorised_chain_generator_matches_builder(pkg):
    """inverter_chain_flat (numpy, for million-stage chains) builds exactly what
    the netlist builder flattens."""
    for L in (1, 2, 9):
        a = pkg.generators.inverter_chain(L).flatten()
        b = pkg.generators.inverter_chain_flat(L)
        assert (a.n_nodes, a.n_branch, a.names) == (b.n_nodes, b.n_branch, b.names)
        for (ma, ta, ba, pa), (mb, tb, bb, pb) in zip(a.groups, b.groups):
            assert ma == mb and np.array_equal(ta, tb) and np.array_equal(pa, pb)
            assert (ba is None and bb is None) or np.array_equal(ba, bb)


def test_eval_scratch_query_on_a_plan(pkg):
    """cedar_eval_scratch reports the allocation-free evaluation's need (device
    outputs plus supply-rail partial sums) and its fixed limit, from the host-side
    analysis alone."""
    import ctypes as C
    lib = pkg.load_library()
    limit = C.c_int64()
    assert lib.cedar_eval_scratch(None, None, None, C.byref(limit)) == 0 and limit.value == 1 << 18
    for stages, long_rows in ((9, False), (100, True)):
        h = pkg.abi.DescHolder(pkg.generators.inverter_chain(stages).flatten())
        p = C.c_void_p()
        pkg.abi.check(lib.cedar_plan_create(C.byref(h.desc), C.byref(p)))
        try:
            n_out, n_part = C.c_int64(), C.c_int64()
            pkg.abi.check(lib.cedar_eval_scratch(p, C.byref(n_out), C.byref(n_part), None))
            # 2L MOSFETs x 4 outputs, L capacitors x 3, two V sources x 4
            assert n_out.value == 8 * stages + 3 * stages + 8
            assert (n_part.value > 0) == long_rows
        finally:
            lib.cedar_ckt_destroy(p)
    assert lib.cedar_eval_scratch(None, C.byref(C.c_int64()), None, None) == -1


def test_engine_selection_arguments(pkg):
    """cedar_ckt_set_engine accepts the four engine codes and thread counts that
    are 0 or multiples of 32 up to 1024, and refuses anything else (host-side
    checks, on a host-only plan)."""
    lib = pkg.load_library()
    h = pkg.abi.DescHolder(pkg.generators.inverter_chain(5).flatten())
    p = C.c_void_p()
    pkg.abi.check(lib.cedar_plan_create(C.byref(h.desc), C.byref(p)))
    try:
        for eng in (0, 1, 2, 3):
            assert lib.cedar_ckt_set_engine(p, eng, 0) == 0
        assert lib.cedar_ckt_set_engine(p, 2, 256) == 0
        assert lib.cedar_ckt_set_engine(p, 4, 0) == -1
        assert lib.cedar_ckt_set_engine(p, -1, 0) == -1
        assert lib.cedar_ckt_set_engine(p, 2, 48) == -1
        assert lib.cedar_ckt_set_engine(p, 2, 2048) == -1
        assert lib.cedar_ckt_set_engine(None, 0, 0) == -1
        blocks = C.c_int32(7)
        assert lib.cedar_ckt_last_blocks(p, C.byref(blocks)) == 0 and blocks.value == 0
    finally:
        lib.cedar_ckt_destroy(p)

"""Struct layouts of the C ABI, three ways.

Every `typedef struct` of include/cedar.h is compiled with the host C compiler,
which reports each struct's size and each field's offset.  Those must equal the
ctypes mirrors in cedarsim.jl_gb300/abi.py (which the tests and the bench pass to
the library), and the Julia declarations in INTEGRATION.md (the binding a
CedarSim maintainer adds) must list the same fields in the same order with the
matching Julia types, so a struct passed from either host has the header's layout.
"""
import ctypes as C
import pathlib
import re
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "cedar.h"

# C struct -> (ctypes mirror in abi.py, Julia struct in INTEGRATION.md)
STRUCTS = {
    "cedar_devgroup": ("DevGroup", "CedarDevGroup"),
    "cedar_ckt_desc": ("CktDesc", "CedarCktDesc"),
    "cedar_objective": ("Objective", "CedarObjective"),
    "cedar_tran_opts": ("TranOpts", "CedarTranOpts"),
    "cedar_stats": ("Stats", "CedarStats"),
    "cedar_costs": ("Costs", "CedarCosts"),
    "cedar_batch_desc": ("BatchDesc", "CedarBatchDesc"),
    "cedar_batch_tuning": ("BatchTuning", "CedarBatchTuning"),
}


def header_structs():
    """{struct: [(field, C type, array length or 0)]} parsed from cedar.h."""
    src = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    out = {}
    for m in re.finditer(r"typedef struct (\w+)\s*\{(.*?)\}\s*\1\s*;", src, flags=re.S):
        fields = []
        for decl in m.group(2).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            dm = re.match(r"(const )?([\w ]+?)\s*(\*?)\s*(\w+(?:\s*(?:\[\d+\])?\s*,\s*\w+)*)\s*(\[(\d+)\])?$", decl)
            assert dm, decl
            ctype = dm.group(2).strip() + ("*" if dm.group(3) else "")
            for name in dm.group(4).split(","):
                name = name.strip()
                fields.append((name, ctype, int(dm.group(6)) if dm.group(6) else 0))
        out[m.group(1)] = fields
    return out


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    """sizeof / offsetof of every header struct, from the host C compiler."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    structs = header_structs()
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void) {"]
    for s, fields in structs.items():
        lines.append(f'  printf("%s size %zu\\n", "{s}", sizeof({s}));')
        for f, _, _ in fields:
            lines.append(f'  printf("%s %s %zu\\n", "{s}", "{f}", offsetof({s}, {f}));')
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("abi")
    (d / "layout.c").write_text("\n".join(lines) + "\n")
    subprocess.run([cc, "-std=c11", "-o", str(d / "layout"), str(d / "layout.c")], check=True)
    out = subprocess.run([str(d / "layout")], check=True, capture_output=True, text=True).stdout
    size, off = {}, {}
    for line in out.splitlines():
        a, b, c = line.split()
        if b == "size":
            size[a] = int(c)
        else:
            off[(a, b)] = int(c)
    return structs, size, off


def test_every_header_struct_is_mirrored():
    assert set(header_structs()) == set(STRUCTS)


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_ctypes_mirror_matches_header(pkg, c_layout, cname):
    structs, size, off = c_layout
    py = getattr(pkg.abi, STRUCTS[cname][0])
    assert [f for f, _, _ in structs[cname]] == [f for f, *_ in py._fields_]
    assert C.sizeof(py) == size[cname]
    for f, _, _ in structs[cname]:
        assert getattr(py, f).offset == off[(cname, f)], (cname, f)


JULIA_OF_C = {"int32_t": "Int32", "int64_t": "Int64", "double": "Float64"}


def julia_structs():
    """{Julia struct: [(field, type)]} from the julia code block of INTEGRATION.md."""
    text = (ROOT / "INTEGRATION.md").read_text()
    blocks = re.findall(r"```julia\n(.*?)```", text, flags=re.S)
    out = {}
    for blk in blocks:
        for m in re.finditer(r"^(?:Base\.@kwdef )?struct (\w+)\n(.*?)^end$", blk, flags=re.S | re.M):
            fields = []
            for line in m.group(2).splitlines():
                line = line.split("#")[0].strip()
                if not line:
                    continue
                fm = re.match(r"(\w+)::([\w{},]+)", line)
                assert fm, line
                fields.append((fm.group(1), fm.group(2)))
            out[m.group(1)] = fields
    return out


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_julia_binding_matches_header(cname):
    hdr = header_structs()[cname]
    jl = julia_structs()
    jname = STRUCTS[cname][1]
    assert jname in jl, f"INTEGRATION.md declares no struct {jname}"
    assert [f for f, _ in jl[jname]] == [f for f, _, _ in hdr], jname
    for (f, jt), (_, ct, n) in zip(jl[jname], hdr):
        if ct.endswith("*"):
            base = ct[:-1].strip()
            want = f"Ptr{{{JULIA_OF_C.get(base) or STRUCTS[base][1]}}}"
        elif n:
            want = f"NTuple{{{n},{JULIA_OF_C[ct]}}}"
        else:
            want = JULIA_OF_C[ct]
        assert jt == want, (jname, f, jt, want)

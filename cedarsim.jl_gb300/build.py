"""Build the CUDA library (libcedar_gpu.so) in-tree for sm_103a.

Translation units are compiled in parallel with nvcc and linked into
``cedarsim.jl_gb300/_build/libcedar_gpu.so``.  Rebuilds only when a source is
newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libcedar_gpu.so"
INCLUDE = PKG.parent / "include"
GEN = BUILD / "gen"            # generated Verilog-A device code (va_models.gen.h)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I", str(INCLUDE), "-I", str(CSRC), "-I", str(GEN)]
LANES = (1, 2, 4, 8, 16, 32)
# (source, object, extra flags): the batched and adjoint kernels are compiled once
# per lanes-per-instance value so the instantiations build in parallel
SOURCES = ([("api.cu", "api.cu.o", []), ("k_plain.cu", "k_plain.cu.o", []), ("k_dispatch.cu", "k_dispatch.cu.o", []),
            ("k_ac.cu", "k_ac.cu.o", []), ("compile.cpp", "compile.cpp.o", [])]
           + [("k_batch.cu", f"k_batch.k{k}.o", [f"-DCEDAR_LANES={k}"]) for k in LANES]
           + [("k_adjoint.cu", f"k_adjoint.k{k}.o", [f"-DCEDAR_LANES={k}"]) for k in LANES])


# Separate mode: when the generated Verilog-A code is large (a BSIM-class model)
# its evaluation is compiled once, in va_models.cu, and device-linked into the
# kernels (relocatable device code), instead of once in every kernel
# translation unit.  CEDAR_VA_SEPARATE=1 / 0 forces the mode either way.
SEPARATE_BYTES = 128 << 10
# registers of the separately compiled model code: at most the batched kernel's
# own allocation, so a large model spills in its own frame and does not raise
# the register count every engine kernel launches with
SEPARATE_MAXRREG = 232


def separate_mode() -> bool:
    env = os.environ.get("CEDAR_VA_SEPARATE")
    if env is not None:
        return env not in ("", "0")
    gen = GEN / "va_models.gen.h"
    return gen.exists() and gen.stat().st_size > SEPARATE_BYTES


def _sources(separate: bool):
    if not separate:
        return SOURCES
    rdc = ["-rdc=true", "-DCEDAR_VA_SEPARATE"]
    out = [(src, obj, extra + rdc if src.endswith(".cu") else extra) for src, obj, extra in SOURCES]
    return out + [("va_models.cu", "va_models.cu.o", rdc + [f"-maxrregcount={SEPARATE_MAXRREG}"])]


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found; the CUDA library cannot be built")
    return p


MODE = BUILD / "mode"         # the mode the library was built in


def _stale() -> bool:
    if not LIB.exists():
        return True
    if not MODE.exists() or MODE.read_text() != ("separate" if separate_mode() else "whole"):
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h")) + [pathlib.Path(__file__)]
    for g in ("va_models.gen.h", "flops.gen.h"):
        if not (GEN / g).exists():
            return True
        deps.append(GEN / g)
    return any(d.stat().st_mtime > t for d in deps)


def generate() -> pathlib.Path:
    """Emit the Verilog-A models' device code (rewritten only when it changes)."""
    from . import va
    return va.generate(GEN)


def count_flops() -> pathlib.Path:
    """Count the FP64 operations of one device evaluation per model by running
    the device code on an op-counting scalar (csrc/opcount.cpp, a host tool) and
    write them as flops.gen.h, the per-device work cedar_ckt_costs sums
    (rewritten only when it changes)."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("a host C++ compiler (g++) is needed to count device flops")
    BUILD.mkdir(parents=True, exist_ok=True)
    tool = BUILD / "opcount"
    cmd = [cxx, "-std=c++17", "-O1", "-I", str(INCLUDE), "-I", str(CSRC), "-I", str(GEN), "-o", str(tool),
           str(CSRC / "opcount.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"opcount build failed:\n{r.stdout}\n{r.stderr}")
    r = subprocess.run([str(tool)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"opcount failed:\n{r.stderr}")
    out = GEN / "flops.gen.h"
    if not out.exists() or out.read_text() != r.stdout:
        out.write_text(r.stdout)
    return out


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    generate()
    count_flops()
    if not force and not _stale():
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(item) -> str:
        src, objname, extra = item
        obj = BUILD / objname
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return str(obj)

    separate = separate_mode()
    sources = _sources(separate)
    with cf.ThreadPoolExecutor(max_workers=min(len(sources), max(2, os.cpu_count() or 2))) as ex:
        objs = list(ex.map(compile_one, sources))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, *(["-rdc=true"] if separate else []), "-shared", "-o", str(tmp), *objs, "-lcudart_static",
           "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    MODE.write_text("separate" if separate else "whole")
    return LIB


if __name__ == "__main__":
    # run as a script: load the package (its directory name is not an identifier)
    # so that the Verilog-A emitter is importable, then build through it
    import sys
    sys.path.insert(0, str(PKG.parent))
    import __graft_entry__
    b = __import__(__graft_entry__.load().__name__ + ".build", fromlist=["build"])
    print(b.build(force="--force" in sys.argv, verbose=True))

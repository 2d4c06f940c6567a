"""Verilog-A compact models compiled to GPU device code.

The role of CedarSim's `load_VA_model` / `make_spice_device`
(src/vasim.jl:663-875): a Verilog-A module becomes a device model the engines
evaluate.  Here the module is parsed (parser.py) and emitted as C++ over dual
numbers (emit.py); the library build compiles the emitted code into every
engine kernel, so a Verilog-A device runs on the GPU like a built-in one.

Models come from the `models/` directory beside this file and from the
directories listed in the CEDAR_VA_PATH environment variable (os.pathsep
separated), every `*.va` file, and the .va files it names directly (a model
whose other .va files are `include fragments), sorted by module name.  Model ids start at
CEDAR_NMODELS (the first id after the built-in models) in that order; adding a
model means rebuilding the library (`__graft_entry__.build()`).
"""
from __future__ import annotations

import os
import pathlib
from typing import Dict, List, Tuple

from .emit import VAModel, analyze, emit_header
from .parser import VAError, parse, parse_file  # noqa: F401

HERE = pathlib.Path(__file__).resolve().parent
BASE_ID = 11     # CEDAR_NMODELS in include/cedar.h

_cache: Dict[tuple, List[Tuple[VAModel, object]]] = {}


def sources() -> List[pathlib.Path]:
    """The shipped models, then every CEDAR_VA_PATH entry: a directory adds its
    *.va files, a file is taken as it is (for models whose other .va files are
    `include fragments)."""
    entries = [HERE / "models"] + [pathlib.Path(p) for p in os.environ.get("CEDAR_VA_PATH", "").split(os.pathsep)
                                   if p]
    files = []
    for d in entries:
        if d.is_dir():
            files += sorted(d.glob("*.va"))
        elif d.is_file():
            files.append(d)
    return files


def _load() -> List[Tuple[VAModel, object]]:
    files = sources()
    key = tuple((str(f), f.stat().st_mtime) for f in files)
    if key not in _cache:
        out = []
        seen = {}
        for f in files:
            for mod in parse_file(f):
                if mod.name in seen:
                    raise VAError(f"module {mod.name} defined in {seen[mod.name]} and {f}")
                seen[mod.name] = f
                out.append(analyze(mod))
        out.sort(key=lambda ma: ma[0].name)
        _cache.clear()
        _cache[key] = out
    return _cache[key]


def models() -> List[VAModel]:
    """The compiled Verilog-A models in model-id order."""
    return [m for m, _ in _load()]


def model_id(name: str) -> int:
    for k, m in enumerate(models()):
        if m.name == name:
            return BASE_ID + k
    raise KeyError(f"no Verilog-A model named {name!r} (known: {[m.name for m in models()]})")


def model(mid: int) -> VAModel:
    return models()[mid - BASE_ID]


def generate(out_dir: pathlib.Path) -> pathlib.Path:
    """Write va_models.gen.h into out_dir (only when its text changes)."""
    out_dir = pathlib.Path(out_dir)
    out_dir.mkdir(parents=True, exist_ok=True)
    path = out_dir / "va_models.gen.h"
    text = emit_header(_load(), BASE_ID)
    if not path.exists() or path.read_text() != text:
        tmp = path.with_suffix(".tmp")
        tmp.write_text(text)
        os.replace(tmp, path)
    return path

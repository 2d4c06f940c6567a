"""Check a Verilog-A file against the compiled subset, and emit its device code.

    python cedarsim.jl_gb300/va/cli.py MODEL.va [--emit OUT.h] [--host]

Parses the file (its `include files relative to it), analyses every module and
prints, per module: ports, internal nodes, branch unknowns, parameters, the
structurally nonzero Jacobian entries the engines will stamp and the noise
sources.  --emit writes the C++ header the library build would generate for
these modules alone; --host lifts the engines' limit on terminal values per
device (for host-side use of the emitted code only).  To compile a model into
the library, put the file in cedarsim.jl_gb300/va/models or a directory named in
CEDAR_VA_PATH and rebuild.  Exits 1 with the error when a module is outside the
subset.
"""
from __future__ import annotations

import argparse
import pathlib
import sys


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("file")
    ap.add_argument("--emit", default=None, help="write the generated header here")
    ap.add_argument("--host", action="store_true", help="no limit on terminal values per device")
    args = ap.parse_args(argv)
    here = pathlib.Path(__file__).resolve().parent
    sys.path.insert(0, str(here.parent.parent))
    import __graft_entry__
    pkg = __graft_entry__.load()
    va_pkg = __import__(pkg.__name__ + ".va", fromlist=["emit", "parser"])
    E, P = va_pkg.emit, va_pkg.parser
    if args.host:
        E.MAX_PORTS = 64
    try:
        mods = [E.analyze(m) for m in P.parse_file(args.file)]
        header = E.emit_header(sorted(mods, key=lambda ma: ma[0].name), 11)   # the emitter's own checks
    except P.VAError as e:
        print(f"{args.file}: {e}", file=sys.stderr)
        return 1
    for m, _ in mods:
        print(f"module {m.name}: ports {m.ports}, internal nodes {m.internals}, branch unknowns {m.has_br}, "
              f"parameters {len(m.params)} (+{len(m.given)} given flags), outputs {m.nout} "
              f"(G {len(m.gents)}, C {len(m.cents)}), noise sources {len(m.noise)}"
              + (", second-order duals (ddx)" if m.second_order else ""))
    if args.emit:
        pathlib.Path(args.emit).write_text(header)
        print(f"wrote {args.emit}")
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Write ac_noise_ngspice.json: the ngspice output-noise table that CedarSim's AC
test holds for its third-order Butterworth filter (test/ac.jl:83-145, asserted
against the analytic PSD at rtol 1e-6 in test/ac.jl:148-149).

The table is read from the CedarSim checkout whose directory is given on the
command line (required); the JSON it writes is the committed fixture, so the tests
do not need the checkout.  Usage: python make_ac_golden.py <CedarSim checkout>  Columns: frequency (Hz) and sqrt(PSD) of V(vout) (V/sqrt(Hz)).
"""
import json
import pathlib
import sys


def extract(path: pathlib.Path):
    lines = path.read_text().splitlines()
    start = next(i for i, l in enumerate(lines) if l.strip().startswith("ngspice = ["))
    rows = []
    for l in lines[start + 1:]:
        if l.strip() == "]":
            break
        f, v = l.split()
        rows.append((float(f), float(v)))
    return start + 1, rows


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_ac_golden.py <CedarSim checkout directory>")
    ref = pathlib.Path(sys.argv[1])
    first, rows = extract(ref / "test" / "ac.jl")
    out = {
        "src": f"test/ac.jl:{first}-{first + len(rows) + 1}",
        "assert": "isapprox(analytic, ngspice, rtol=1e-6), test/ac.jl:148-149",
        "circuit": "V1 vin 0 AC 1; L1 vin n1 3/2; C2 n1 0 4/3; L3 n1 vout 1/2; R4, R5 vout 0 2 each; "
                   "temp 23 C, gmin 0 (test/ac.jl:17-35)",
        "f_hz": [r[0] for r in rows],
        "sqrt_psd": [r[1] for r in rows],
    }
    p = pathlib.Path(__file__).with_name("ac_noise_ngspice.json")
    p.write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", p, len(rows), "rows")

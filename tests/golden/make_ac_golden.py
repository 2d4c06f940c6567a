"""Write the ngspice output-noise tables that CedarSim's AC test holds:
  ac_noise_ngspice.json           third-order Butterworth filter (test/ac.jl:83-145,
                                  asserted against the analytic PSD at rtol 1e-6,
                                  test/ac.jl:148-149);
  ac_noise_bsimcmg_ngspice.json   BSIM-CMG CMOS inverter on the ASAP7 TT cards
                                  (test/ac.jl:155-234, asserted against CedarSim's
                                  PSD at rtol 1e-6, test/ac.jl:237).

The tables are read from the CedarSim checkout whose directory is given on the
command line (required); the JSON files it writes are the committed fixtures, so
the tests do not need the checkout.  Usage: python make_ac_golden.py <CedarSim
checkout>.  Columns: frequency (Hz) and sqrt(PSD) of the output node (V/sqrt(Hz)).
"""
import json
import pathlib
import sys


def extract(path: pathlib.Path, which: int = 0):
    """Rows of the which-th `ngspice = [` table of the file, and its first line."""
    lines = path.read_text().splitlines()
    start = [i for i, l in enumerate(lines) if l.strip().startswith("ngspice = [")][which]
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
    here = pathlib.Path(__file__).parent
    first, rows = extract(ref / "test" / "ac.jl", 0)
    out = {
        "src": f"test/ac.jl:{first}-{first + len(rows) + 1}",
        "assert": "isapprox(analytic, ngspice, rtol=1e-6), test/ac.jl:148-149",
        "circuit": "V1 vin 0 AC 1; L1 vin n1 3/2; C2 n1 0 4/3; L3 n1 vout 1/2; R4, R5 vout 0 2 each; "
                   "temp 23 C, gmin 0 (test/ac.jl:17-35)",
        "f_hz": [r[0] for r in rows],
        "sqrt_psd": [r[1] for r in rows],
    }
    (here / "ac_noise_ngspice.json").write_text(json.dumps(out, indent=1) + "\n")
    first, rows = extract(ref / "test" / "ac.jl", 1)
    out = {
        "src": f"test/ac.jl:{first}-{first + len(rows) + 1}",
        "assert": "isapprox(sqrt.(abs.(psd)), ngspice[:,2], rtol=1e-6), test/ac.jl:237",
        "circuit": "mneg Q D VSS VSS nmos_lvt; mpos Q D VDD VDD pmos_lvt (BSIM-CMG, ASAP7 TT cards); "
                   "VVDD VDD 0 1.0; VVSS VSS 0 0.0; CQ D 0 1e-15; VD D 0 AC 1 SIN(0.5 0.01 1e7) "
                   "(test/bsimcmg/inverter_cmg_cedar.cir); output node Q",
        "f_hz": [r[0] for r in rows],
        "sqrt_psd": [r[1] for r in rows],
    }
    (here / "ac_noise_bsimcmg_ngspice.json").write_text(json.dumps(out, indent=1) + "\n")

"""Write known_answers.json: the answers CedarSim's own tests assert for the
transient path (file:line within the CedarSim project).  The reference cannot
run here (no Julia toolchain), so these analytic values are the pin."""
import json
import math
import pathlib

V, R, C = 5.0, 2000.0, 1e-6
ANSWERS = {
    "vr": {"V": 5.0, "I": 2.5, "src": "test/basic.jl:38-42"},
    "ir": {"V": 10.0, "I": 5.0, "src": "test/basic.jl:101-105"},
    "vrc": {"i0_per_m": V / R, "v_end": V, "src": "test/basic.jl:135-140,159-165"},
    "spectre_sources": {"node_1": 2.2e-3, "node_3": -1.5, "node_2_end": 3.5, "node_4_end": -5.0,
                        "R4_I_end": -1.25e-3, "src": "test/basic.jl:196-203"},
    "spice_sources": {"node_5": 2.0, "node_6": 4.0, "node_8": 4.0, "node_7": -4000.0, "node_9": -4000.0,
                      "src": "test/basic.jl:230-234"},
    "multiplicities": {"node": 10 / 11, "src": "test/basic.jl:591-594"},
    "semiconductor_resistor": {"I": 1e-3, "src": "test/basic.jl:735-736"},
    "pwl_derivative": {"slopes": [[50e-9, 0.0], [100e-9, 5.0e8], [110e-9, 0.0], [200e-9, -5.0e8]],
                       "src": "test/transients.jl:84-95"},
    "butterworth": {"rms": 0.5, "max_abs_err": 1e-6, "src": "test/transients.jl:152-156"},
    "ddx": {"V1_I": -5.0 * 2 * 2 * 3, "src": "test/ddx.jl:21"},
    "sensitivity": {"dR1_over_V": -0.5, "src": "test/sensitivity.jl:40-41"},
    # ParamSim overrides: V = 5 across R (default 2, overridden to 1) -> V.I = -5;
    # the SPICE deck i1 vcc 0 'foo', l1 vcc out 1m, r1 out 0 r='foo+2000' (params
    # foo = 1 and a subcircuit default foo + 2000): V(r1) after overriding the
    # subcircuit's foo to 2, the global foo to 2, and r1.r to 100
    "params": {"V_I": -5.0, "r1_V": {"sub_foo_2": -2.0, "foo_2": -4004.0, "r_100": -100.0},
               "src": "test/params.jl:19,34,46,87-99"},
    # subcircuit net naming: i1 0 d 1 into a 1 Ohm resistor to ground (the
    # subcircuit's own d tied to ground is a different net) -> i1 carries 1 A
    "subckt_nets": {"i1_I": 1.0, "src": "test/compilation.jl:58-79"},
}

if __name__ == "__main__":
    p = pathlib.Path(__file__).with_name("known_answers.json")
    p.write_text(json.dumps(ANSWERS, indent=1) + "\n")
    print("wrote", p)

"""The oracle's discrete adjoint on workload 5 itself, against central differences.

Instances are drawn at random from the 512-chain adjoint workload (its
generator, seed and per-instance parameters) and run over the full 0..20 ns;
the gradient with respect to randomly drawn MOSFET widths is compared with
central differences (step 1e-6 W) of the objective along the run's own accepted
step sequence (the oracle's replay), to 1e-5 relative, as the GPU's gradients
are in tests/test_gpu_adjoint_fd.py.  The GPU's adjoint equals the oracle's on
the instances tests/test_gpu_adjoint.py compares, so this spreads the check
over the workload.  By default 2 instances x 2 widths (about a minute on a few
cores); CEDAR_ADJ_FD_INSTANCES widens the sample.
"""
import multiprocessing as mp
import os

import numpy as np

N_WORK = 512
TSTOP = 20e-9
N_WIDTHS = 2

_W = {}


def _init():
    import __graft_entry__ as ge
    pkg = ge.load()
    _W["pkg"], _W["orc"] = pkg, ge.load_oracle().Oracle(pkg)
    _W["work"] = pkg.generators.adjoint_chains(N_WORK)


def _instance(i):
    pkg = _W["pkg"]
    templates, itpl, par, off, objs, tstar = _W["work"]
    f = pkg.generators.instance_flat(templates[itpl[i]], par[off[i]:off[i] + templates[itpl[i]].param_block().size].copy())
    ob = objs[itpl[i]]
    obj = pkg.abi.Objective(int(ob[0]), int(ob[1]), int(ob[2]), 0, *[float(v) for v in ob[3:]])
    return f, obj, float(tstar[i])


def _opts(pkg):
    return (pkg.make_opts(tstop=TSTOP, hmax=TSTOP / 50),
            pkg.make_opts(tstop=TSTOP, hmax=TSTOP / 50, nr_factor=1e-5))


def _adjoint(i):
    pkg, orc = _W["pkg"], _W["orc"]
    f, obj, ts = _instance(i)
    fwd, rep = _opts(pkg)
    phi, grad, T, ords = orc.adjoint(f, fwd, rep, obj, ts)
    return i, grad, T, ords


def _replay(args):
    i, mos, k, w, T, ords = args
    pkg, orc = _W["pkg"], _W["orc"]
    f, obj, ts = _instance(i)
    f.groups[mos][3][1, k] = w
    return orc.replay_phi(f, _opts(pkg)[1], T, ords, obj, ts)


def test_workload_adjoint_against_central_differences(pkg):
    n_inst = int(os.environ.get("CEDAR_ADJ_FD_INSTANCES", "2"))
    templates, itpl, par, off, objs, tstar = pkg.generators.adjoint_chains(N_WORK)
    rng = np.random.default_rng(31)
    pick = [int(i) for i in rng.choice(N_WORK, size=n_inst, replace=False)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(os.cpu_count() or 1, 16), initializer=_init) as pool:
        adj = {i: (g, T, o) for i, g, T, o in pool.map(_adjoint, pick, chunksize=1)}
        jobs, meta = [], []
        for i in pick:
            flat = templates[itpl[i]]
            mos = [gi for gi, gr in enumerate(flat.groups) if gr[0] == pkg.circuit.MOS1][0]
            nw = flat.groups[mos][3].shape[1]
            p0 = sum(g[3].size for g in flat.groups[:mos])
            widths = par[off[i] + p0 + nw: off[i] + p0 + 2 * nw]
            g, T, ords = adj[i]
            for k in np.sort(rng.choice(nw, size=N_WIDTHS, replace=False)):
                # the gradient's entry of width k: the MOSFET widths come first, in group order
                d = 1e-6 * widths[k]
                jobs += [(i, mos, int(k), widths[k] + d, T, ords), (i, mos, int(k), widths[k] - d, T, ords)]
                meta.append((i, int(k), d, g[k]))
        phis = pool.map(_replay, jobs, chunksize=1)
    errs = []
    for q, (i, k, d, gk) in enumerate(meta):
        fd = (phis[2 * q] - phis[2 * q + 1]) / (2 * d)
        errs.append(abs(gk - fd) / abs(fd))
        assert errs[-1] <= 1e-5, (i, k, gk, fd)
    print(f"adjoint vs FD: {len(meta)} widths over {len(pick)} instances, worst relative error {max(errs):.2e}")

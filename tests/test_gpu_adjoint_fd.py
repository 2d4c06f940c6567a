"""Workload 5 at its own size: gradients against central differences.

Instances are taken from the 512-chain adjoint workload itself (its generator,
seed and per-instance parameters), the shortest and the longest chain lengths
(L = 31 and L = 63, 62 and 126 widths), each over the full 0..20 ns.  The GPU's
discrete-adjoint gradient is checked against central differences (step 1e-6 W)
on 16 sampled widths per instance, each difference taken by the oracle replaying
the GPU's own accepted step sequence (the gradient is that of the discrete
objective along the recorded steps, test/sensitivity.jl's role), to 1e-5
relative.  The replays run in a process pool on the host cores.
"""
import multiprocessing as mp
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TSTOP = 20e-9
N_WORK = 512
N_FD = 16


_W = {}


def _worker_init():
    import __graft_entry__ as ge
    pkg = ge.load()
    _W["pkg"] = pkg
    _W["orc"] = ge.load_oracle().Oracle(pkg)
    _W["work"] = pkg.generators.adjoint_chains(N_WORK)


def _replay(args):
    """phi along the recorded steps with width k of MOSFET group `mos` of instance
    i set to w (the oracle's replay of a fixed step sequence)."""
    i, mos, k, w, T, ords = args
    pkg, orc = _W["pkg"], _W["orc"]
    templates, itpl, par, off, objs, tstar = _W["work"]
    blk = par[off[i]:off[i] + templates[itpl[i]].param_block().size].copy()   # the worker's copy is reused
    f = pkg.generators.instance_flat(templates[itpl[i]], blk)
    f.groups[mos][3][1, k] = w
    ob = objs[itpl[i]]
    objective = pkg.abi.Objective(int(ob[0]), int(ob[1]), int(ob[2]), 0, *[float(v) for v in ob[3:]])
    rep = pkg.make_opts(tstop=TSTOP, hmax=TSTOP / 50, nr_factor=1e-5)
    return orc.replay_phi(f, rep, T, ords, objective, float(tstar[i]))


def test_adjoint_full_workload_fd(gpu, pkg):
    templates, itpl, par, off, objs, tstar = pkg.generators.adjoint_chains(N_WORK)
    L = np.array([templates[t].n_nodes - 2 for t in itpl])
    rng = np.random.default_rng(29)
    pick = [int(rng.choice(np.flatnonzero(L == lo))) for lo in (L.min(), L.max())]
    assert sorted(L[pick].tolist()) == [31, 63]
    objectives = [pkg.abi.Objective(int(o[0]), int(o[1]), int(o[2]), 0, *[float(v) for v in o[3:]]) for o in objs]
    sw = pkg.Batch(templates, itpl[pick], par, off[pick])
    o = pkg.make_opts(tstop=TSTOP, hmax=TSTOP / 50)
    r = sw.adjoint(o, objectives, tstar[pick])
    assert np.all(r.status == 0)
    jobs, meta = [], []
    for j, i in enumerate(pick):
        flat = templates[itpl[i]]
        mos = [gi for gi, gr in enumerate(flat.groups) if gr[0] == pkg.circuit.MOS1][0]
        nw = flat.groups[mos][3].shape[1]
        T, ords = sw.tape(j)
        assert len(T) == r.stats["accepted"][j]
        w_all = par[off[i]:off[i] + flat.param_block().size]
        # the instance's widths: row 1 of the MOSFET group's parameter block
        p0 = sum(g[3].size for g in flat.groups[:mos])
        widths = w_all[p0 + nw: p0 + 2 * nw]
        for k in np.sort(rng.choice(nw, size=N_FD, replace=False)):
            d = 1e-6 * widths[k]
            jobs += [(i, mos, int(k), widths[k] + d, T, ords), (i, mos, int(k), widths[k] - d, T, ords)]
            meta.append((j, int(k), d))
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(len(jobs), os.cpu_count() or 1), initializer=_worker_init) as pool:
        phis = pool.map(_replay, jobs, chunksize=1)
    worst = 0.0
    for q, (j, k, d) in enumerate(meta):
        fd = (phis[2 * q] - phis[2 * q + 1]) / (2 * d)
        err = abs(r.grad[j, k] - fd) / abs(fd)
        worst = max(worst, err)
        assert err <= 1e-5, (pick[j], k, r.grad[j, k], fd)
    print(f"FD check: {len(meta)} widths over instances {pick} (L = {L[pick].tolist()}), worst relative error {worst:.2e}")

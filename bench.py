#!/usr/bin/env python
"""Benchmark: batched Monte Carlo transient of 4096 ragged CMOS inverter chains.

Workload (the configuration the headline metric is quoted on): 4096 instances of
the level-1 MOSFET inverter chain with chain length drawn from {5, 7, ..., 63},
per-transistor Vth ~ N(nominal, 0.03 V), KP ~ nominal * exp(0.05 z), per-instance
load C ~ U(5, 20) fF; DC operating point, then adaptive BDF2 (reltol 1e-6,
abstol 1e-9 V) to 20 ns, all instances in one persistent launch per step.

A step is one batched launch that advances every instance through one time
window of the 20 ns transient (windows of 20 ns / (warmup + steps)); windows
stop softly, so the step sequence is exactly that of one uninterrupted run.
The first (warm-up) window also includes every instance's DC operating point.

metric  = accepted instance-timesteps per second (whole job, all ranks)
e2e     = the same metric through the C ABI with host buffers: instance
          parameters copied host->device and results device->host inside the
          timed region (a complete cedar_batch_create + run + results)
--impl reference times the CPU restatement of the same path (OpenMP over
instances, all host threads) on a bounded sample of the instances.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MC transient inst-steps/s, batched vs plain GPU @1e-6 reltol; adjoint grads/s"
# DRAM bytes (read + written) of the batched kernel per accepted instance-step,
# from one ncu capture of a 1024-chain window (7.27 MB over 988 847 steps); the
# kernel keeps every instance's state on chip, so this is parameter and history
# traffic only
DRAM_BYTES_PER_STEP = 7.35
UNIT = "instance-timesteps/s"
TSTOP = 20e-9


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=7)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n-inst", type=int, default=4096)
    p.add_argument("--seed", type=int, default=20240607)
    p.add_argument("--lanes", type=int, default=0, help="lanes per instance (0 = library default)")
    p.add_argument("--warps", type=int, default=0)
    p.add_argument("--ctas", type=int, default=0, help="resident CTAs per SM at most (0 = as many as fit)")
    p.add_argument("--ref-inst", type=int, default=64, help="instances per reference (CPU) step")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--plain-inst", type=int, default=4)
    p.add_argument("--plain-tstop", type=float, default=2e-9)
    p.add_argument("--tstop-ns", type=float, default=20.0, help="transient length (20 ns for the headline)")
    p.add_argument("--fp64-probe", action="store_true", help="print the FP64 issue-rate probe (1, 8, 32 lanes) and exit")
    p.add_argument("--no-adjoint", action="store_true")
    p.add_argument("--no-eval", action="store_true", help="skip the cedar_eval HBM leg")
    p.add_argument("--no-rings", action="store_true", help="skip the ring-oscillator leg")
    p.add_argument("--no-ac", action="store_true", help="skip the AC / noise sweep leg")
    p.add_argument("--ac-freq", type=int, default=1 << 17, help="frequency points of the AC / noise leg")
    p.add_argument("--no-va", action="store_true", help="skip the Verilog-A model legs (chains and rings)")
    p.add_argument("--ring-inst", type=int, default=1024)
    p.add_argument("--ring-tstop-ns", type=float, default=50.0)
    p.add_argument("--ring-ref-inst", type=int, default=32, help="instances in the CPU sample of the ring leg")
    p.add_argument("--no-plain-configs", action="store_true", help="skip configurations 1 and 2 (single circuits)")
    p.add_argument("--eval-stages", type=int, default=1_000_000, help="inverter-chain stages of the cedar_eval leg")
    p.add_argument("--adj-inst", type=int, default=512, help="instances of the adjoint workload")
    p.add_argument("--adj-tstop-ns", type=float, default=20.0)
    p.add_argument("--adj-ref-inst", type=int, default=16, help="instances in the CPU adjoint sample")
    return p.parse_args()


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self):
        self.rows, self.proc = [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200", "-i",
                 os.environ.get("LOCAL_RANK", "0")], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = [r for r in self.rows if len(r) >= 6]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[2 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def workload(pkg, n_inst, seed):
    g = pkg.generators
    templates, itpl, par, off = g.mc_chains(n_inst, seed=seed)
    probes = np.array([[g.chain_output_probe(f)] for f in templates], np.int32)
    return templates, itpl, par, off, probes


def shard(itpl, templates, rank, world):
    """Contiguous-free load balance: sort by chain length, deal round-robin."""
    n = np.array([templates[t].n for t in itpl])
    order = np.argsort(-n, kind="stable")
    return np.sort(order[rank::world])


def opts_for(pkg, tstop=TSTOP):
    # hmax stays that of the 20 ns run so a shortened run takes the same steps
    return pkg.make_opts("bdf2", True, 0.0, tstop, 0.0, True, reltol=1e-6, abstol_v=1e-9, hmax=TSTOP / 50)


def mc_workload(n_inst: int, tstop_ns: float = TSTOP * 1e9) -> str:
    """The Monte Carlo headline workload's name, the same in both arms' config."""
    return f"{n_inst} MC ragged inverter chains (L in {{5..63}}), adaptive BDF2 to {tstop_ns:g} ns, reltol 1e-6"


def flops_per_iteration(pkg, templates):
    out = []
    for f in templates:
        c = pkg.costs(f)
        out.append(c["flops_eval"] + c["flops_stamp"] + c["flops_lu"] + c["flops_solve"] + c["flops_update"])
    return np.array(out, np.float64)


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend)
        return rank, world, dist
    return 0, 1, None


def reduce_max(dist, v):
    if dist is None:
        return v
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, v):
    if dist is None:
        return v
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def adjoint_workload(pkg, args):
    templates, itpl, par, off, objs, tstar = pkg.generators.adjoint_chains(args.adj_inst, seed=args.seed)
    objectives = [pkg.abi.Objective(int(a), int(b), int(c), 0, float(l), float(we), float(wd), float(wf))
                  for (a, b, c, l, we, wd, wf) in objs]
    return templates, itpl, par, off, objectives, tstar


ADJ_WORKLOAD = ("512 MC chains L in {31..63}, supply energy + 50% crossing delay objective, "
                "adaptive BDF2 to 20 ns, checkpoint every 64 steps, gradient w.r.t. every MOSFET width")


def reference_adjoint(args, pkg, orc):
    """The oracle's adjoint (OpenMP over instances) on a bounded random sample."""
    templates, itpl, par, off, objectives, tstar = adjoint_workload(pkg, args)
    k = max(1, min(args.adj_ref_inst, args.adj_inst))
    sel = np.sort(np.random.default_rng(5).choice(args.adj_inst, size=k, replace=False))
    sub = pkg.abi.BatchHolder(templates, itpl[sel], par, off[sel])
    cores = os.cpu_count() or 1
    o = opts_for(pkg, args.adj_tstop_ns * 1e-9)
    t0 = time.perf_counter()
    phi, g, st = orc.adjoint_batch(sub, o, objectives, tstar[sel], nthreads=cores)
    dt = time.perf_counter() - t0
    ok = int((st == 0).sum())
    return {"value": ok / dt, "unit": "instance-gradients/s", "cores": cores, "kind": "port",
            "sample": f"{k} randomly chosen instances of the {args.adj_inst}, each forward 0..{args.adj_tstop_ns:g} ns + replay + adjoint",
            "seconds": dt, "failed": k - ok}


def fp64_latency(pkg, lib, C):
    """Latency of one dependent FP64 operation on this GPU (cedar_fp64_latency):
    the unit of a single circuit's critical path through LU and substitutions."""
    cyc, ns = C.c_double(), C.c_double()
    pkg.abi.check(lib.cedar_fp64_latency(1 << 16, C.byref(cyc), C.byref(ns)))
    return {"cycles_per_dependent_dfma": cyc.value, "ns_per_dependent_dfma": ns.value,
            "note": "one warp, a chain of 524288 dependent DFMAs (SM clock; events incl. launch)"}


def measure_eval(pkg, args, torch, C, fp64_peak=None):
    """cedar_eval_dev (device evaluation + CSC stamping, the drop-in residual /
    Jacobian boundary) on one large chain: inputs resident in HBM and larger than
    L2, CUDA events on the handle's stream, algorithmic bytes from cedar_ckt_costs."""
    f = pkg.generators.inverter_chain_flat(args.eval_stages)
    sy = pkg.System(f)
    lib = sy.lib
    dev = torch.device("cuda:0")
    g = torch.Generator(device=dev).manual_seed(7)
    x = torch.rand(sy.n, dtype=torch.float64, device=dev, generator=g) * 1.8
    xd = torch.randn(sy.n, dtype=torch.float64, device=dev, generator=g) * 1e9
    F = torch.empty(sy.n, dtype=torch.float64, device=dev)
    J = torch.empty(sy.nnz_j, dtype=torch.float64, device=dev)
    costs = pkg.abi.Costs()
    pkg.abi.check(lib.cedar_ckt_costs(sy.handle, C.byref(costs)))
    sp = C.c_void_p()
    pkg.abi.check(lib.cedar_ckt_stream(sy.handle, C.byref(sp)))
    st = torch.cuda.ExternalStream(sp.value)
    torch.cuda.synchronize()
    ptr = lambda t: C.c_void_p(t.data_ptr())
    call = lambda: pkg.abi.check(lib.cedar_eval_dev(sy.handle, ptr(x), ptr(xd), 1e-9, 1e12, ptr(F), ptr(J)))
    for _ in range(3):
        call()
    reps = 20
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        call()
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    peak = hbm_peak_gbs()
    gbs = costs.bytes_eval / (ms * 1e-3) / 1e9
    ok = bool(torch.isfinite(F).all().item() and torch.isfinite(J).all().item())
    # the call's FP64 work: every device's evaluation (op-counted) and one add per
    # stamp entry; on this part the device arithmetic can bound the call before HBM
    flops = costs.flops_eval + costs.flops_stamp
    tfl = flops / (ms * 1e-3) / 1e12
    t_floor = max(costs.bytes_eval / (peak * 1e9), flops / (fp64_peak * 1e12)) if fp64_peak else None
    return {"workload": f"{args.eval_stages}-stage inverter chain ({3 * args.eval_stages} devices, n = {sy.n}, "
                        f"nnz(J) = {sy.nnz_j}), one cedar_eval_dev per call",
            "bytes_per_call": int(costs.bytes_eval), "ms_per_call": ms, "achieved_gbs": gbs, "peak_gbs": peak,
            "frac": gbs / peak, "finite": ok, "kernels": ["eval_kernel", "stamp_kernel", "stamp_long_final_kernel"],
            "fp64": {"flops_per_call": int(flops), "achieved_tflops": tfl, "peak_tflops": fp64_peak,
                     "frac": tfl / fp64_peak if fp64_peak else None},
            "roofline_frac": (t_floor / (ms * 1e-3)) if t_floor else None,
            "roofline_note": "roofline_frac = max(bytes / HBM peak, flops / FP64 peak) / measured time",
            "l2": "inputs and outputs of one call exceed L2 (129 MB)",
            "timing": f"CUDA events on the handle's stream around {reps} calls after 3 warm-up calls"}


def measure_rings(pkg, args, C, fp64_peak, verilog_a=False):
    """Workload 4: 15-stage current-starved ring oscillators (level-1 MOSFETs +
    exponential diodes, RC supply per stage), DC operating point + N(0, 1 mV) per
    node, adaptive BDF2 to 50 ns, in one batched launch timed with CUDA events (DC
    included).  verilog_a: the MOSFETs and diodes as the emitted va_mos1 / va_diode."""
    tpl, itpl, par, off, dx, dxo = pkg.generators.mc_rings(args.ring_inst, seed=args.seed)
    if verilog_a:
        tpl = [pkg.generators.as_verilog_a(f) for f in tpl]
    f = tpl[0]
    probes = np.array([[f.index("out1")]], np.int32)
    sw = pkg.Batch(tpl, itpl, par, off, inst_dx=dx, inst_dx_off=dxo, probes=probes, n_samples=501)
    tstop = args.ring_tstop_ns * 1e-9
    o = pkg.make_opts("bdf2", True, 0.0, tstop, 0.0, True, reltol=1e-6, abstol_v=1e-9, hmax=tstop / 50)
    r = sw.run(o)
    ms = C.c_double()
    pkg.abi.check(sw.lib.cedar_batch_last_ms(sw.handle, C.byref(ms)))
    ok = r.stats["status"] == 0
    s = r.samples[:, 0, :]
    osc = int(np.sum((s.max(axis=1) - s.min(axis=1)) > 1.0))
    fl = float(flops_per_iteration(pkg, tpl)[0])
    iters = float(r.stats["newton_iters"].sum() + r.stats["dc_iters"].sum())
    tfl = fl * iters / (ms.value / 1e3) / 1e12
    models = "emitted Verilog-A va_mos1 + va_diode" if verilog_a else "built-in level-1 MOSFETs + exponential diodes"
    return {"workload": f"{args.ring_inst} x 15-stage current-starved ring oscillators ({models}, "
                        f"100 Ohm / 100 fF supply per stage), DC op + N(0, 1 mV) per node, adaptive BDF2 to "
                        f"{args.ring_tstop_ns:g} ns", "value": float(r.stats["accepted"].sum()) / (ms.value / 1e3),
            "unit": "instance-timesteps/s", "ms": ms.value, "failed_instances": int((~ok).sum()),
            "oscillating_instances": osc, "accepted_steps_mean": float(r.stats["accepted"].mean()),
            "accepted_steps": int(r.stats["accepted"].sum()),
            "newton_iters_per_s": iters / (ms.value / 1e3),
            "roofline": {"bound": "fp64", "achieved": tfl, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": tfl / fp64_peak, "flops_per_newton_iter": fl},
            "tuning": list(sw.tuning), "timing": "CUDA events around one cedar_batch_run launch (DC operating points included)"}


def reference_rings(args, pkg, orc):
    """The oracle (OpenMP over instances, all host threads) on a bounded random
    sample of the ring-oscillator workload, each instance over the full horizon."""
    tpl, itpl, par, off, dx, dxo = pkg.generators.mc_rings(args.ring_inst, seed=args.seed)
    k = max(1, min(args.ring_ref_inst, args.ring_inst))
    sel = np.sort(np.random.default_rng(3).choice(args.ring_inst, size=k, replace=False))
    sub = pkg.abi.BatchHolder(tpl, itpl[sel], par, off[sel], inst_dx=dx, inst_dx_off=dxo[sel])
    tstop = args.ring_tstop_ns * 1e-9
    o = pkg.make_opts("bdf2", True, 0.0, tstop, 0.0, True, reltol=1e-6, abstol_v=1e-9, hmax=tstop / 50)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    xf, samp, st = orc.batch(sub, o, 0, len(sel), nthreads=cores, want_samples=False)
    dt = time.perf_counter() - t0
    return {"value": float(st["accepted"].sum()) / dt, "unit": "instance-timesteps/s", "cores": cores,
            "kind": "port", "sample": f"{k} randomly chosen instances of the {args.ring_inst}, each DC + "
                                      f"0..{args.ring_tstop_ns:g} ns", "seconds": dt,
            "failed": int((st["status"] != 0).sum())}


def measure_va(pkg, args, C, builtin_ms, builtin_steps, fp64_peak):
    """Workload 3 at full size with the MOSFETs as the Verilog-A level-1 model
    compiled by the emitter (va_mos1: the built-in model's equations and parameter
    block, evaluated over dual numbers), in one cedar_batch_run (DC included),
    against the built-in model's complete run of the same instances (the e2e run's
    kernel time): the cost of generic emitted device code."""
    templates, itpl, par, off = pkg.generators.mc_chains(args.n_inst, seed=args.seed)
    va_tpl = [pkg.generators.as_verilog_a(f) for f in templates]
    o = opts_for(pkg, args.tstop_ns * 1e-9)
    sw = pkg.Batch(va_tpl, itpl, par, off)
    if args.lanes:
        sw.set_tuning(args.lanes, args.warps or 4, args.ctas)
    r = sw.run(o)
    ms = C.c_double()
    pkg.abi.check(sw.lib.cedar_batch_last_ms(sw.handle, C.byref(ms)))
    steps = float(r.stats["accepted"].sum())
    iters = float(r.stats["newton_iters"].sum() + r.stats["dc_iters"].sum())
    v = steps / (ms.value / 1e3)
    out = {"workload": f"{args.n_inst} MC chains (L in {{5..63}}), adaptive BDF2 to {args.tstop_ns:g} ns, MOSFETs as "
                       "the emitted Verilog-A va_mos1", "unit": "instance-timesteps/s", "value": v, "ms": ms.value,
           "accepted_steps": int(steps), "failed_instances": int((r.stats["status"] != 0).sum()),
           "newton_iters_per_s": iters / (ms.value / 1e3),
           "timing": "CUDA events around one cedar_batch_run launch (DC operating points included)"}
    if builtin_ms:
        vb = builtin_steps / (builtin_ms / 1e3)
        out["builtin"] = {"value": vb, "ms": builtin_ms, "accepted_steps": int(builtin_steps),
                          "source": "kernel time of the e2e run (same instances, built-in MOS1, DC included)"}
        out["va_over_builtin"] = v / vb
        out["same_step_counts"] = int(steps) == int(builtin_steps)
    return out


def measure_ac(pkg, args, torch, C, fp64_peak):
    """Small-signal AC and noise sweeps (cedar_ac / cedar_noise) of the 100-section
    RC ladder about its DC point: every frequency is one complex static-pivot LU
    and solve, one warp per frequency.  Device time: CUDA events on the handle's
    stream around one call (its small host copies included); the CPU column is the
    oracle's dense complex solve per frequency (the reference's freqresp evaluates
    the dense descriptor system per frequency) on a bounded sample."""
    import __graft_entry__ as ge
    f = pkg.generators.rc_ladder(100).flatten()
    f.ac = {"V1": 1.0}
    sy = pkg.System(f)
    lib = sy.lib
    x_op = pkg.dc(sy)
    nf = args.ac_freq
    w = 2 * np.pi * np.logspace(3, 12, nf)
    probe = f.index(f.names[100])
    acs, ns = pkg.ACSol(sy, x_op), pkg.NoiseSol(sy, x_op)
    costs = pkg.abi.Costs()
    pkg.abi.check(lib.cedar_ckt_costs(sy.handle, C.byref(costs)))
    # complex arithmetic: one complex multiply-subtract = 4 real FMAs (8 flops)
    flops = 4 * (costs.flops_lu + costs.flops_solve) + costs.nnz_lu
    sp = C.c_void_p()
    pkg.abi.check(lib.cedar_ckt_stream(sy.handle, C.byref(sp)))
    st = torch.cuda.ExternalStream(sp.value)
    out = {}
    for name, call in (("ac", lambda: acs.freqresp(probe, w)), ("noise", lambda: ns.psd(probe, w))):
        for _ in range(2):
            call()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(st)
        res = call()
        e1.record(st)
        e1.synchronize()
        wall = time.perf_counter() - t0
        ms = e0.elapsed_time(e1)
        sol = acs if name == "ac" else ns
        kst = pkg.ac_last_stats(sy)
        tf = flops * nf / (ms * 1e-3) / 1e12
        out[name] = {"value": nf / (ms * 1e-3), "unit": "frequency points/s", "ms": ms,
                     "e2e": {"value": nf / wall, "unit": "frequency points/s"},
                     "failed_points": int((sol.status != 0).sum()), "finite": bool(np.all(np.isfinite(res))),
                     "achieved_tflops": tf, "fp64_frac": tf / fp64_peak if fp64_peak else None,
                     "dense_reruns": kst["n_dense"], "kernel_ms": {"sparse": kst["ms_sparse"], "dense": kst["ms_dense"]}}
    orc = ge.load_oracle().Oracle(pkg)
    k = min(nf, 2000)
    ws = w[np.linspace(0, nf - 1, k).astype(int)]
    t0 = time.perf_counter()
    orc.ac(f, x_op, ws, [probe])
    cpu_ac = k / (time.perf_counter() - t0)
    out["cpu_baseline"] = {"value": cpu_ac, "unit": "frequency points/s", "kind": "port", "cores": os.cpu_count(),
                           "sample": f"{k} of the {nf} frequencies, dense complex LU per frequency (numpy / LAPACK)"}
    out["workload"] = (f"100-section RC ladder (n = {sy.n}, nnz(LU) = {costs.nnz_lu}) about its DC point, "
                       f"{nf} frequencies log-spaced 1 kHz .. 1 THz, one probe")
    out["flops_per_point"] = int(flops)
    out["timing"] = "CUDA events on the handle's stream around one call (host copies of omega and results included)"
    return out


def plain_leg(pkg, orc, C, name, flat, opts, fp64_peak, hbm_peak, workload):
    """One circuit through cedar_tran_run, the single-circuit drop-in (tran!): the
    kernel's device time (cedar_ckt_last_ms: CUDA events on the handle's stream),
    the call's wall time with its host copies as e2e, the roofline of the
    algorithmic Newton-iteration bytes and flops (cedar_ckt_costs x iterations),
    the waveform error against the FP64 oracle at every recorded point, and the
    oracle timed beside it on one host thread."""
    sy = pkg.System(flat)
    lib = sy.lib
    n_pts = int(round((opts.tstop - opts.tstart) / opts.h)) + 2 if not opts.adaptive else 1 << 18
    x = np.zeros(sy.n)
    t_out, x_out = np.zeros(n_pts), np.zeros((n_pts, sy.n))
    cnt, st = C.c_int64(), pkg.abi.Stats()
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))

    def call():
        x[:] = 0.0
        pkg.abi.check(lib.cedar_tran_run(sy.handle, C.byref(opts), dp(x), dp(t_out), dp(x_out), n_pts, C.byref(cnt),
                                         C.byref(st)))
    # each engine of the single-circuit path (the one-warp slot engine, one CTA of
    # the size chosen from the circuit, and CTAs of 128 / 256 threads): best of 3
    # calls after one warm-up; the fastest is the leg's value
    engines = {}
    for ename, eng, thr in (("warp", 1, 0), ("cta", 2, 0), ("cta128", 2, 128), ("cta256", 2, 256)):
        pkg.abi.check(lib.cedar_ckt_set_engine(sy.handle, eng, thr))
        call()
        ms, walls = [], []
        for _ in range(3):
            t0 = time.perf_counter()
            call()
            walls.append(time.perf_counter() - t0)
            m = C.c_double()
            pkg.abi.check(lib.cedar_ckt_last_ms(sy.handle, C.byref(m)))
            ms.append(m.value)
        engines[ename] = {"ms": min(ms), "wall_s": min(walls), "accepted": int(st.accepted),
                          "status": pkg.abi.STATUS_NAMES[st.status], "x_out": x_out[:cnt.value].copy(),
                          "t_out": t_out[:cnt.value].copy()}
    best = min(engines, key=lambda e: engines[e]["ms"])
    dev_s, wall_s = engines[best]["ms"] / 1e3, engines[best]["wall_s"]
    t_out[:len(engines[best]["t_out"])] = engines[best]["t_out"]
    x_out[:len(engines[best]["x_out"])] = engines[best]["x_out"]
    pkg.abi.check(lib.cedar_ckt_set_engine(sy.handle, 0, 0))
    steps, iters = st.accepted, st.newton_iters + st.dc_iters
    costs = pkg.abi.Costs()
    pkg.abi.check(lib.cedar_ckt_costs(sy.handle, C.byref(costs)))
    flops = costs.flops_eval + costs.flops_stamp + costs.flops_lu + costs.flops_solve + costs.flops_update
    gbs = costs.bytes * iters / dev_s / 1e9
    tfl = flops * iters / dev_s / 1e12
    # oracle: same circuit and options, one host thread
    t0 = time.perf_counter()
    t_ref, x_ref, st_ref, rc = orc.tran(flat, opts, cap=n_pts)
    cpu_s = time.perf_counter() - t0
    m = min(len(t_ref), cnt.value)
    same_t = bool(len(t_ref) == cnt.value and np.array_equal(t_ref, t_out[:m]))
    nn = flat.n_nodes
    err = float(np.max(np.abs(x_out[:m, :nn] - x_ref[:m, :nn]) / (1e-6 * np.abs(x_ref[:m, :nn]) + 1e-9)))
    return {"workload": workload, "value": steps / dev_s, "unit": "timesteps/s",
            "newton_iters_per_s": iters / dev_s, "accepted_steps": int(steps), "newton_iters": int(iters),
            "ms": dev_s * 1e3, "status": pkg.abi.STATUS_NAMES[st.status],
            "e2e": {"value": steps / wall_s, "unit": "timesteps/s", "seconds": wall_s,
                    "h2d_bytes_per_step": int(x.nbytes + C.sizeof(opts)),
                    "d2h_bytes_per_step": int(cnt.value * (8 + 8 * sy.n) + C.sizeof(st))},
            "roofline": {"bound": f"latency (one circuit; fastest engine {best})",
                         "hbm": {"achieved_gbs": gbs, "peak_gbs": hbm_peak, "frac": gbs / hbm_peak},
                         "fp64": {"achieved_tflops": tfl, "peak_tflops": fp64_peak, "frac": tfl / fp64_peak},
                         "bytes_per_newton_iter": int(costs.bytes), "flops_per_newton_iter": int(flops),
                         "note": "algorithmic bytes / flops of one Newton iteration (cedar_ckt_costs) x iterations "
                                 "/ kernel time; one circuit is latency-bound on every engine, the fractions show "
                                 "how far"},
            "vs_oracle": {"max_scaled_error": err, "tolerance": "reltol 1e-6, abstol 1e-9 V, every recorded point",
                          "same_time_points": same_t, "oracle_steps": int(st_ref.accepted)},
            "cpu_baseline": {"value": st_ref.accepted / cpu_s, "unit": "timesteps/s", "cores": 1, "kind": "port",
                             "sample": "the whole run, oracle (dense LU with partial pivoting, as IDA's default "
                                       "direct solve) on one host thread", "seconds": cpu_s},
            "engine": best, "engines_ms": {e: v["ms"] for e, v in engines.items()},
            "engines_same_steps": len({v["accepted"] for v in engines.values()}) == 1,
            "timing": "best of 3 calls after one warm-up per engine; device time = CUDA events around the kernel"}


def measure_plain_configs(pkg, C, fp64_peak):
    """Configurations 1 and 2: the RC ladder (trapezoidal, h = 0.1 ns, 0..1 us) and
    the 31-stage inverter chain (BDF2, h = 1 ps, 0..20 ns), each one circuit through
    cedar_tran_run; the chain with built-in and with Verilog-A level-1 MOSFETs."""
    import __graft_entry__ as ge
    orc = ge.load_oracle().Oracle(pkg)
    g = pkg.generators
    hbm = hbm_peak_gbs()
    o1 = pkg.make_opts("trap", False, 0.0, 1e-6, 0.1e-9, True)
    o2 = pkg.make_opts("bdf2", False, 0.0, 20e-9, 1e-12, True)
    rc = g.rc_ladder(100).flatten()
    ch = g.inverter_chain(31).flatten()
    return {
        "config1": plain_leg(pkg, orc, C, "config1", rc, o1, fp64_peak, hbm,
                             "RC ladder, 100 sections (1 kOhm, 1 pF), PULSE(0 1 0 1n 1n 50n 100n), trapezoidal "
                             "h = 0.1 ns, 0..1 us, n = 101"),
        "config2": plain_leg(pkg, orc, C, "config2", ch, o2, fp64_peak, hbm,
                             "31-stage inverter chain, built-in level-1 MOSFETs, 10 fF loads, PULSE(0 1.8 0 50p 50p "
                             "950p 2n), BDF2 h = 1 ps, 0..20 ns, n = 35"),
        "config2_verilog_a": plain_leg(pkg, orc, C, "config2_va", g.as_verilog_a(ch), o2, fp64_peak, hbm,
                                       "the same chain with the MOSFETs as the emitted Verilog-A va_mos1"),
    }


def hbm_peak_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"])
    except Exception:
        return 6800.0   # fallback figure for GB300 when the measured file is absent


def run_reference(args, pkg):
    """CPU restatement of the path (the oracle) on a bounded sample per step."""
    import __graft_entry__ as ge
    orc = ge.load_oracle().Oracle(pkg)
    templates, itpl, par, off, probes = workload(pkg, args.n_inst, args.seed)
    sw = pkg.abi.BatchHolder(templates, itpl, par, off)
    o = opts_for(pkg)
    cores = os.cpu_count() or 1
    rng_order = np.random.default_rng(1).permutation(args.n_inst)
    k = max(1, args.ref_inst)
    total_steps, total_time = 0, 0.0
    for s in range(args.warmup + args.steps):
        sel = np.sort(rng_order[(s * k) % args.n_inst:][:k])
        sub = pkg.abi.BatchHolder(templates, itpl[sel], par, off[sel])
        t0 = time.perf_counter()
        xf, samp, st = orc.batch(sub, o, 0, len(sel), nthreads=cores, want_samples=False)
        dt = time.perf_counter() - t0
        if s >= args.warmup:
            total_steps += int(st["accepted"].sum())
            total_time += dt
    v = total_steps / total_time
    sample = f"{args.steps} x {k} randomly chosen instances of the {args.n_inst}, each run 0..20 ns (DC op included)"
    adj = None if args.no_adjoint else reference_adjoint(args, pkg, orc)
    rings = None if args.no_rings else reference_rings(args, pkg, orc)
    return {"metric": METRIC, "impl": "reference", "value": v, "unit": UNIT, "n_gpus": args.gpus, "adjoint": adj,
            "rings": rings,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_time / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Philox4x32-10)",
            "config": {"workload": mc_workload(args.n_inst), "n_inst": args.n_inst},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    rank, world, dist = dist_init()
    import __graft_entry__ as ge
    pkg = ge.load()
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args, pkg)), flush=True)
        return
    import torch
    lib0 = pkg.load_library()
    torch.cuda.init()
    import ctypes as C
    if args.fp64_probe:
        out = {}
        for lanes in (32, 8, 1):
            gf, ms = C.c_double(), C.c_double()
            pkg.abi.check(lib0.cedar_fp64_probe(lanes, 4096, C.byref(gf), C.byref(ms)))
            out[str(lanes)] = {"useful_gflops": gf.value, "ms": ms.value}
        print(json.dumps({"fp64_probe": out, "fp64_latency": fp64_latency(pkg, lib0, C)}), flush=True)
        return
    # FP64 peak measured live on this GPU (all lanes active): the roofline denominator
    gf = C.c_double()
    pkg.abi.check(lib0.cedar_fp64_probe(32, 4096, C.byref(gf), None))
    fp64_peak = gf.value / 1e3
    fp64_lat = fp64_latency(pkg, lib0, C)
    templates, itpl, par, off, probes = workload(pkg, args.n_inst, args.seed)
    mine = shard(itpl, templates, rank, world)
    n_samples = 201
    sw = pkg.Batch(templates, itpl[mine], par, off[mine], probes=probes, n_samples=n_samples)
    if args.lanes:
        sw.set_tuning(args.lanes, args.warps or 4, args.ctas)
    tstop = args.tstop_ns * 1e-9
    o = opts_for(pkg, tstop)
    nwin = args.warmup + args.steps
    edges = [tstop * (k + 1) / nwin for k in range(nwin)]
    edges[-1] = tstop
    lib = sw.lib
    pkg.abi.check(lib.cedar_batch_start(sw.handle, C.byref(o)))
    nrun = C.c_int32()
    # warm-up windows (DC operating points happen in the first)
    for k in range(args.warmup):
        pkg.abi.check(lib.cedar_batch_advance(sw.handle, edges[k], C.byref(nrun)))
    st0 = np.zeros(sw.n_inst, pkg.abi.STATS_DTYPE)
    pkg.abi.check(lib.cedar_batch_results(sw.handle, None, None, st0.ctypes.data_as(C.c_void_p)))
    clocks = ClockSampler()
    clocks.start()
    barrier(dist)
    torch.cuda.synchronize()
    # device-side timing: events on the handle's stream are recorded by the library
    # calls' own synchronisation; the host clock brackets synchronised launches
    t0 = time.perf_counter()
    dev_ms = []
    ms = C.c_double()
    for k in range(args.warmup, nwin):
        pkg.abi.check(lib.cedar_batch_advance(sw.handle, edges[k], C.byref(nrun)))
        pkg.abi.check(lib.cedar_batch_last_ms(sw.handle, C.byref(ms)))
        dev_ms.append(ms.value)
    torch.cuda.synchronize()
    barrier(dist)
    wall = time.perf_counter() - t0
    dt = sum(dev_ms) / 1e3  # CUDA-event time of the timed launches on the library's stream
    clk = clocks.stop()
    xf = np.zeros((sw.n_inst, sw.n_max))
    samp = np.zeros((sw.n_inst, 1, n_samples))
    st1 = np.zeros(sw.n_inst, pkg.abi.STATS_DTYPE)
    pkg.abi.check(lib.cedar_batch_results(sw.handle, xf.ctypes.data_as(C.POINTER(C.c_double)),
                                          samp.ctypes.data_as(C.POINTER(C.c_double)), st1.ctypes.data_as(C.c_void_p)))
    steps_local = float(st1["accepted"].sum() - st0["accepted"].sum())
    iters_local = float(st1["newton_iters"].sum() - st0["newton_iters"].sum())
    bad = int((st1["status"] != 0).sum())
    dt = reduce_max(dist, dt)
    steps_all = reduce_sum(dist, steps_local)
    iters_all = reduce_sum(dist, iters_local)
    value = steps_all / dt
    # roofline: algorithmic FP64 flops of the timed Newton iterations / time
    fl = flops_per_iteration(pkg, templates)
    it_by_inst = st1["newton_iters"] - st0["newton_iters"]
    flops_local = float(np.sum(it_by_inst * fl[itpl[mine]]))
    flops_all = reduce_sum(dist, flops_local)
    achieved = flops_all / dt / 1e12
    # end to end through the C ABI with host buffers (create + full run + results)
    e2e = None
    e2e_kernel_ms, e2e_kernel_steps = None, None
    if not args.no_e2e:
        barrier(dist)
        torch.cuda.synchronize()
        te0 = time.perf_counter()
        sw2 = pkg.Batch(templates, itpl[mine], par, off[mine], probes=probes, n_samples=n_samples)
        if args.lanes:
            sw2.set_tuning(args.lanes, args.warps or 4, args.ctas)
        r2 = sw2.run(o)
        torch.cuda.synchronize()
        barrier(dist)
        te = reduce_max(dist, time.perf_counter() - te0)
        kms = C.c_double()
        pkg.abi.check(lib.cedar_batch_last_ms(sw2.handle, C.byref(kms)))
        e2e_kernel_ms, e2e_kernel_steps = kms.value, float(r2.stats["accepted"].sum())
        e2e_steps = reduce_sum(dist, float(r2.stats["accepted"].sum()))
        h2d = int(par.nbytes + off[mine].nbytes + itpl[mine].nbytes + probes.nbytes)
        d2h = int(r2.x_final.nbytes + (r2.samples.nbytes if r2.samples is not None else 0) + r2.stats.nbytes)
        e2e = {"value": e2e_steps / te, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "seconds": te, "note": "one complete C-ABI run (create + DC + 0..20 ns + results) of this rank's instances"}
        del sw2
    if rank != 0:
        return
    # plain (one circuit per launch) GPU path on a sample, for the batched-vs-plain ratio
    plain = None
    if not args.no_plain:
        g = pkg.generators
        sel = np.random.default_rng(2).choice(args.n_inst, size=args.plain_inst, replace=False)
        acc, tt, tk = 0, 0.0, 0.0
        po = opts_for(pkg, args.plain_tstop)
        for i in sel:
            f = g.instance_flat(templates[itpl[i]], par[off[i]:off[i] + templates[itpl[i]].param_block().size])
            s0 = pkg.System(f)
            xi, tb, xb = np.zeros(s0.n), np.zeros(1 << 17), np.zeros(((1 << 17), s0.n))
            cnt, st = C.c_int64(), pkg.abi.Stats()
            dpp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
            t0 = time.perf_counter()
            pkg.abi.check(lib.cedar_tran_run(s0.handle, C.byref(po), dpp(xi), dpp(tb), dpp(xb), 1 << 17, C.byref(cnt),
                                             C.byref(st)))
            tt += time.perf_counter() - t0
            km = C.c_double()
            pkg.abi.check(lib.cedar_ckt_last_ms(s0.handle, C.byref(km)))
            tk += km.value / 1e3
            acc += st.accepted
        plain = {"value": acc / tk, "unit": UNIT, "e2e_value": acc / tt,
                 "sample": f"{args.plain_inst} random instances, each one cedar_tran_run (default engine: one "
                           f"CTA; every accepted point recorded) from DC to {args.plain_tstop * 1e9:g} ns with "
                           f"the headline's options",
                 "seconds_kernel": tk, "seconds_wall": tt}
    # discrete adjoint (workload 5) through the C ABI
    adj = None
    if not args.no_adjoint:
        t5, i5, p5, o5_off, obj5, ts5 = adjoint_workload(pkg, args)
        sw5 = pkg.Batch(t5, i5, p5, o5_off)
        if args.lanes:
            sw5.set_tuning(args.lanes, args.warps or 4, args.ctas)
        sw5.adjoint(opts_for(pkg, 0.05e-9), obj5, ts5)          # warm-up
        r5 = sw5.adjoint(opts_for(pkg, args.adj_tstop_ns * 1e-9), obj5, ts5)
        ok5 = r5.status == 0
        secs = (r5.fwd_ms + r5.bwd_ms) / 1e3
        per, npm = sw5.nparams()
        adj = {"metric": "adjoint gradients/s", "value": float(ok5.sum()) / secs, "unit": "instance-gradients/s",
               "param_derivatives_per_s": float(per[i5][ok5].sum()) / secs, "fwd_ms": r5.fwd_ms, "bwd_ms": r5.bwd_ms,
               "failed_instances": int((~ok5).sum()), "workload": ADJ_WORKLOAD, "n_inst": args.adj_inst,
               "params_per_instance": [int(per.min()), int(per.max())],
               "accepted_steps_mean": float(r5.stats["accepted"].mean()), "tuning": list(sw5.tuning),
               "timing": "CUDA events around the recording forward and the backward kernel"}
        # FP64 roofline of the adjoint: the recording forward, the backward kernel's
        # replay of every segment (the forward's Newton iterations again), and per
        # accepted step one more refactorisation at the converged state (a Newton
        # iteration's flops) plus the transposed substitutions
        c5 = [pkg.costs(f) for f in t5]
        fl5 = np.array([c["flops_eval"] + c["flops_stamp"] + c["flops_lu"] + c["flops_solve"] + c["flops_update"]
                        for c in c5], np.float64)[i5]
        sv5 = np.array([c["flops_solve"] for c in c5], np.float64)[i5]
        it5 = (r5.stats["newton_iters"] + r5.stats["dc_iters"]).astype(np.float64)
        ac5 = r5.stats["accepted"].astype(np.float64)
        adj_flops = float(np.sum(2.0 * it5 * fl5 + ac5 * (fl5 + sv5)))
        tf5 = adj_flops / secs / 1e12
        adj["roofline"] = {"bound": "fp64", "achieved": tf5, "peak": fp64_peak, "unit": "TFLOP/s",
                           "frac": tf5 / fp64_peak,
                           "note": "flops = 2 x forward Newton iterations x flops per iteration (recording forward + "
                                   "replay) + accepted steps x (flops per iteration + substitution flops)"}
        del sw5
    eval_leg = None if args.no_eval else measure_eval(pkg, args, torch, C, fp64_peak)
    rings = None if args.no_rings else measure_rings(pkg, args, C, fp64_peak)
    if rings is not None and not args.no_va:
        rv = measure_rings(pkg, args, C, fp64_peak, verilog_a=True)
        rings["verilog_a"] = rv
        rings["va_over_builtin"] = rv["value"] / rings["value"]
        rings["same_step_counts"] = rv["accepted_steps"] == rings["accepted_steps"]
    ac_leg = None if args.no_ac else measure_ac(pkg, args, torch, C, fp64_peak)
    va_leg = None if args.no_va else measure_va(pkg, args, C, e2e_kernel_ms, e2e_kernel_steps, fp64_peak)
    plain_cfg = None if args.no_plain_configs else measure_plain_configs(pkg, C, fp64_peak)
    cpu = None
    if not args.no_cpu_baseline:
        cpu_line = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                                   "--steps", "1", "--warmup", "0", "--ref-inst", "64"]
                                  + (["--no-adjoint"] if args.no_adjoint else [])
                                  + (["--no-rings"] if args.no_rings else []),
                                  capture_output=True, text=True, timeout=900)
        try:
            ref = json.loads(cpu_line.stdout.strip().splitlines()[-1])
            cpu = ref["cpu_baseline"]
            if adj is not None and ref.get("adjoint"):
                adj["cpu_baseline"] = ref["adjoint"]
            if rings is not None and ref.get("rings"):
                rings["cpu_baseline"] = ref["rings"]
        except Exception:
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                   "sample": "failed: " + cpu_line.stderr[-300:]}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Philox4x32-10)",
        "config": {"workload": mc_workload(args.n_inst, args.tstop_ns),
                   "n_inst": args.n_inst, "instances_per_rank": len(mine), "window_ns": tstop / nwin * 1e9, "tstop_ns": args.tstop_ns,
                   "tuning": list(sw.tuning), "l2": "state resident on chip; no HBM re-read to flush",
                   "parallelism": f"instances sharded over {world} GPU(s), no collective"},
        "newton_iters_per_s": iters_all / dt, "failed_instances": bad, "host_wall_s": wall,
        "launch_ms": dev_ms,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp64_peak,
                     "traffic": DRAM_BYTES_PER_STEP * steps_all / max(1, len(dev_ms)),
                     "traffic_note": f"bytes per launch: {DRAM_BYTES_PER_STEP} B of DRAM traffic per accepted "
                                     "instance-step (ncu dram__bytes_read + write of one batch_kernel window of "
                                     "1024 chains) x the accepted steps of a timed launch",
                     "note": "algorithmic FP64 flops per Newton iteration (cedar_ckt_costs) x iterations / time; "
                             "peak = DFMA rate measured in this run by cedar_fp64_probe (MEASURED_PEAKS.json "
                             "has no FP64 entry); the kernel keeps its state on chip, so HBM is not its bound"},
        "cpu_baseline": cpu, "e2e": e2e, "plain_gpu": plain, "adjoint": adj, "eval_hbm": eval_leg, "rings": rings,
        "ac": ac_leg, "verilog_a": va_leg, "config1": plain_cfg and plain_cfg["config1"],
        "config2": plain_cfg and plain_cfg["config2"], "config2_verilog_a": plain_cfg and plain_cfg["config2_verilog_a"],
        "fp64_latency": fp64_lat, "clocks": clk, "gpu_launches": args.steps,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()

#!/usr/bin/env python
"""Throughput of the GB300 shallow-water hot path (one JSON line).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one time step (all RK stages) of the workload; the default
workload is the 512x512-cell, 64-level, 8-tracer, 5-stage LSRK case with all
four dissipation terms on.  ``value`` is cell-level-stage updates per second
with the state resident in HBM (its 1.6 GB state is larger than L2, so no
flush is needed between steps); ``e2e`` is the same metric through the
public API with the state held in page-locked host memory and copied
host->device and device->host every step: through the host-state stepper
(og.HostStepper, level chunks whose copies overlap the other chunks'
compute), with the serial upload + step + download figure beside it.
Under torchrun each rank advances its own replica
(weak scaling; the path needs no communication).

``--impl reference`` times the CPU restatement of the reference (oracle/,
OpenMP on all host cores) on the same workload; each of its steps is one
LSRK5 step of a level-subsampled copy of the workload (stated in
``cpu_baseline.sample``), so the run stays within minutes.
"""
from __future__ import annotations

import argparse
import json

import numpy as np
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("cell·level·stage updates/s FP64 (% HBM roofline); "
          "adjoint/forward time ratio")
UNIT = "cell·level·stage updates/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
# FP64 thread instructions (DFMA + DADD + DMUL) per cell-level of
# k_cell_final on the LSRK5 512x512x64x8 workload's physics, counted by ncu
# (smsp__sass_thread_inst_executed_op_{dfma,dadd,dmul}_pred_on.sum over the
# launch's cell-levels); it is a property of the compiled kernel and the
# enabled terms, not of the mesh size
K_CELL_FINAL_FP64 = 142


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="lsrk5_512x512")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--level-chunk", type=int, default=-1,
                    help="levels per chunk of the host-state stepper that "
                         "the end-to-end number goes through (-1: the "
                         "fastest chunk layout on this machine, "
                         "HostStepper.autotuned)")
    ap.add_argument("--levels", default="",
                    help="chunk sizes of the host-state stepper, comma "
                         "separated (overrides --level-chunk)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-ensembles", action="store_true",
                    help="leave the two ensemble summaries out of the line")
    ap.add_argument("--nx", type=int, default=0,
                    help="override nx = ny (small profiling cases)")
    ap.add_argument("--adjoint-steps", type=int, default=0,
                    help="rk4_128x128_adjoint: override the 1000 steps; "
                         "adjoint_ensemble32: the 300 steps")
    ap.add_argument("--no-comparisons", action="store_true",
                    help="adjoint_ensemble32: leave out the stream-"
                         "interleaved and one-after-another comparisons "
                         "(small profiling cases)")
    ap.add_argument("--snapshots", type=int, default=0,
                    help="rk4_128x128_adjoint: override the 32 snapshots")
    return ap.parse_args()


L2_BYTES = 129e6  # GB300 L2


def l2_note(state_bytes):
    """How the timed steps relate to L2: the state (read and written every
    stage) either exceeds L2, or the workload is a small case that is not a
    contract number."""
    if state_bytes > L2_BYTES:
        return "state (%.2f GB) larger than L2; no flush" % (state_bytes / 1e9)
    return ("state (%.3f GB) fits in L2; small case timed without a flush, "
            "not the headline workload" % (state_bytes / 1e9))


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def max_over_ranks(ms: float, world: int, device: str = "cpu") -> float:
    """Slowest rank's time (the whole job ends when the last replica does)."""
    if world == 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: int, ms_max: float, world: int) -> float:
    """Whole-job updates/s of `world` independent replicas (weak scaling)."""
    return world * units_per_rank / (ms_max / 1e3)


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


# ----------------------------------------------------------- clocks -------

class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str):
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", gpu_id, f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap")
        for line in out.strip().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                smax.append(float(p[1]))
            except ValueError:
                continue
            for n, v in zip(names, p[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------- CPU baseline -----

def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True,
                             timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def workload_config(wl, world, sample_nlayers):
    """The `config` object both arms print (the same keys, so the two lines
    can be compared key for key)."""
    return {"workload": wl.name, "nx": wl.nx, "ny": wl.ny,
            "nlayers": wl.nlayers, "ntracers": wl.ntracers,
            "stepper": ("rk4" if wl.stepper == "rk4"
                        else f"lsrk{wl.nstages}"), "dt": wl.dt,
            "parallelism": f"replicas x{world}",
            "l2": l2_note(8 * wl.ncells * wl.nlayers * (4 + wl.ntracers)),
            "sample_nlayers": sample_nlayers}


def oracle_sample(wl, nlayers_sample, steps, warmup):
    """Time the oracle (C restatement of the reference, OpenMP) on the
    workload's mesh and tracers with `nlayers_sample` levels."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import pyoracle
    from omega_playground_gb300.workloads import initial_state
    w = wl.scaled(nlayers=nlayers_sample)
    om = pyoracle.OracleMesh(w.nx, w.ny, w.dc, w.nlayers)

    class _M:  # the tables initial_state reads
        pass
    m = _M()
    for k, v in om.tables.items():
        setattr(m, "m_" + k, v)
    m.m_period_x, m.m_period_y = om.period_x, om.period_y
    h, vn, tr = (np.ascontiguousarray(a) for a in initial_state(m, w))
    md = pyoracle.OracleModel(om, **w.param_kwargs())
    for s in range(warmup):
        md.step(h, vn, tr, s * w.dt, w.dt, 1, w.stepper, w.nstages)
    times = []
    for s in range(steps):
        t0 = time.perf_counter()
        md.step(h, vn, tr, (warmup + s) * w.dt, w.dt, 1, w.stepper, w.nstages)
        times.append(time.perf_counter() - t0)
    units = w.ncells * w.nlayers * w.nstages
    return units, times, pyoracle.lib().or_num_threads(), w


def cpu_baseline(wl, target_s=15.0):
    """Bounded sample of ~target_s seconds: pick the level count from a
    probe step, then time whole LSRK/RK4 steps."""
    units, t, cores, _ = oracle_sample(wl, 1, 1, 0)
    per_level = t[0]
    nl = max(1, min(wl.nlayers, int(3.0 / max(per_level, 1e-6))))
    units, times, cores, w = oracle_sample(wl, nl, 1, 0)
    nsteps = max(1, min(20, int(target_s / max(times[0], 1e-6))))
    units, times, cores, w = oracle_sample(wl, nl, nsteps, 0)
    return {"value": units * len(times) / sum(times), "unit": UNIT,
            "cores": cores, "kind": "port", "cpu_model": cpu_model(),
            "sample": (f"{len(times)} {w.stepper}{w.nstages} step(s) of the "
                       f"{w.nx}x{w.ny} mesh, {w.ntracers} tracers, "
                       f"{w.nlayers} of {wl.nlayers} levels; oracle C "
                       f"restatement, OpenMP {cores} threads")}


def run_reference(args, wl):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    # size the sample so (warmup + steps) steps take about two minutes
    _, t, cores, _ = oracle_sample(wl, 1, 1, 0)
    budget = 120.0 / max(1, args.steps + args.warmup)
    nl = max(1, min(wl.nlayers, int(budget / max(t[0], 1e-6))))
    units, times, cores, w = oracle_sample(wl, nl, args.steps, args.warmup)
    total = sum(times)
    value = units * len(times) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": workload_config(wl, args.gpus, w.nlayers),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores,
                         "kind": "port", "cpu_model": cpu_model(),
                         "sample": (f"each step: one {w.stepper}{w.nstages} "
                                    f"step of the {w.nx}x{w.ny} mesh, "
                                    f"{w.ntracers} tracers, {w.nlayers} of "
                                    f"{wl.nlayers} levels (oracle C "
                                    "restatement of the reference, OpenMP)")},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------- GPU arm -------

def adjoint_ratio(stream, nsteps=0, nsnap=0):
    """Checkpointed adjoint of the 128x128x32, 2-tracer RK4 workload (1000
    steps, 32 snapshots): device time of the forward sweep (checkpoints +
    taped last step) plus the backward sweep, over a plain 1000-step forward
    on the same GPU.  The region loss and its gradient (host) are outside
    both timings.  nsteps / nsnap override the step and snapshot counts
    (small profiling cases)."""
    import torch
    import omega_playground_gb300 as og
    from omega_playground_gb300.workloads import (ADJOINT_SNAPSHOTS, WORKLOADS,
                                                  initial_state, loss_and_grad,
                                                  region_cells)
    wl = WORKLOADS["rk4_128x128_adjoint"]
    if nsteps:
        wl = wl.scaled(nsteps=nsteps)
    nsnap = nsnap or ADJOINT_SNAPSHOTS
    mesh = og.PlanarHexagonalMesh(wl.nx, wl.ny, wl.dc, wl.nlayers)
    params = wl.params()
    model = og.ShallowWaterModel(mesh, params)
    x0 = initial_state(mesh, wl)
    region = region_cells(mesh, wl.seed + 99)
    sh = stream.cuda_stream
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
    st = og.ShallowWaterState(mesh, params)
    stepper = og.RK4Stepper(model)
    st.upload(*x0)
    stepper.step(st, 0.0, wl.dt, 3, stream=sh)        # warm-up, graph capture
    st.upload(*x0)
    torch.cuda.synchronize()
    ev[0].record(stream)
    stepper.step(st, 0.0, wl.dt, wl.nsteps, stream=sh)
    ev[1].record(stream)
    torch.cuda.synchronize()
    fwd_ms = ev[0].elapsed_time(ev[1])
    adj = og.Adjoint(model, nsnap)
    X0 = og.ShallowWaterState(mesh, params)
    X0.upload(*x0)
    XN = og.ShallowWaterState(mesh, params)
    # warm-up: a full-length forward sweep plans the schedule (host, once
    # per step and snapshot count), a 2-step pair captures the graphs
    adj.forward(X0, 0.0, wl.dt, wl.nsteps, XN, stream=sh)
    adj.forward(X0, 0.0, wl.dt, 2, XN, stream=sh)
    G = og.ShallowWaterState(mesh, params)
    G.fill(0.0, stream=sh)
    adj.backward(G, stream=sh)
    torch.cuda.synchronize()
    ev[2].record(stream)
    adj.forward(X0, 0.0, wl.dt, wl.nsteps, XN, stream=sh)
    ev[3].record(stream)
    torch.cuda.synchronize()
    L, g = loss_and_grad(*XN.download(stream=sh), region)
    G.upload(*g, stream=sh)
    torch.cuda.synchronize()
    ev[4].record(stream)
    adj.backward(G, stream=sh)
    ev[5].record(stream)
    torch.cuda.synchronize()
    f_ms, b_ms = ev[2].elapsed_time(ev[3]), ev[4].elapsed_time(ev[5])
    plain, taped, tadv = adj.info_ex()
    snap_b, tape_b, total_b = adj.memory()
    grad = G.download(stream=sh)
    return {"workload": wl.name, "steps": wl.nsteps,
            "snapshots": nsnap, "plain_forward_ms": fwd_ms,
            "checkpointed_forward_ms": f_ms, "backward_ms": b_ms,
            "ratio": (f_ms + b_ms) / fwd_ms, "plain_advances": plain,
            "taped_steps": taped, "taped_advances": tadv,
            "classic_binomial_plain_advances": og.checkpoint_cost(wl.nsteps,
                                                                  nsnap),
            "memory": {"snapshot_bytes": snap_b, "tape_bytes": tape_b,
                       "tapes": 2,
                       "tape_in_snapshots": round(tape_b / snap_b, 2),
                       "total_bytes": total_b},
            "loss": L,
            "grad_h_norm": float(np.sqrt(np.sum(grad[0] ** 2)))}


def run_ours(args, wl):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import omega_playground_gb300 as og
    from omega_playground_gb300.shallow_water import gpu_numa_node

    mesh = og.PlanarHexagonalMesh(wl.nx, wl.ny, wl.dc, wl.nlayers)
    params = wl.params()
    model = og.ShallowWaterModel(mesh, params)
    state = og.ShallowWaterState(mesh, params)
    h0, vn0, tr0 = og.workloads.initial_state(mesh, wl)
    state.upload(h0, vn0, tr0)
    stepper = (og.RK4Stepper(model) if wl.stepper == "rk4"
               else og.LSRKStepper(model, wl.nstages))
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # warm-up (captures the step graph)
    stepper.step(state, 0.0, wl.dt, args.warmup, use_graph=True, stream=sh)
    barrier()
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(local).uuid)
    except Exception:
        uuid = str(local)
    clocks = ClockSampler(uuid)
    time.sleep(0.3)
    barrier()
    launches0 = og.kernel_launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    stepper.step(state, args.warmup * wl.dt, wl.dt, args.steps,
                 use_graph=True, stream=sh)
    e1.record(stream)
    barrier()
    ms = e0.elapsed_time(e1)
    launches = og.kernel_launches() - launches0
    clk = clocks.stop()
    ms_max = max_over_ranks(ms, world, device="cuda")
    units = wl.ncells * wl.nlayers * wl.nstages * args.steps
    value = replica_throughput(units, ms_max, world)

    # per-kernel event timing of one step (direct launches)
    og.profile_enable(True)
    stepper.step(state, 0.0, wl.dt, 1, use_graph=False, stream=sh)
    prof = og.profile_read()
    og.profile_enable(False)
    stage_ms = sum(v[0] for v in prof.values()) / wl.nstages
    dom = max(prof, key=lambda k: prof[k][0])
    dom_ms = prof[dom][0] / prof[dom][1]
    CK = wl.ncells * wl.nlayers
    alg_per_unit = {"k_cell_final": 32 * (1 + wl.ntracers),
                    "k_edge_final": 32 * 3}
    peak, peak_kind = hbm_peak()
    dom_bytes = alg_per_unit.get(dom, 0) * CK
    achieved = dom_bytes / (dom_ms / 1e3) / 1e9
    stage_bytes = wl.alg_bytes_per_stage()
    # DRAM bytes per cell-level of the dominant kernel from one ncu capture
    # (dram__bytes_read.sum + dram__bytes_write.sum of k_cell_final on the
    # 256x256x64x8 case: 1.932 GB for 4,194,304 cell-levels), scaled to
    # this launch by its cell-level count; traffic grows in proportion.
    ncu_bytes_per_unit = {"k_cell_final": 1.932e9 / 4194304}
    traffic = (ncu_bytes_per_unit[dom] * CK
               if dom in ncu_bytes_per_unit and wl.ntracers == 8 else None)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_kind, "traffic": traffic,
                "alg_bytes_per_launch": dom_bytes,
                "launch_ms": dom_ms,
                "stage": {"achieved": stage_bytes / (stage_ms / 1e3) / 1e9,
                          "alg_bytes": stage_bytes, "ms": stage_ms,
                          "frac": stage_bytes / (stage_ms / 1e3) / 1e9 / peak}}
    # FP64 issue roof, measured here: DFMA / DADD / DMUL issue rates of this
    # GPU (swg_fp64_issue_rate: every SM filled, 4 independent chains per
    # thread, CUDA events) with the SM clock sampled while they run.  The
    # instructions per cell-level of k_cell_final come from ncu on the
    # 256x256x64x8 case (DFMA 132 + DMUL 15 + DADD 8 = 155 with 8 tracers).
    fp64 = None
    if dom == "k_cell_final" and wl.ntracers == 8:
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        pk_clocks = ClockSampler(uuid)
        time.sleep(0.3)
        rates = {op: og.fp64_issue_rate(op, 40000, stream=sh)
                 for op in ("dfma", "dadd", "dmul")}
        pk_clk = pk_clocks.stop()
        pk_mhz = pk_clk.get("sm_mhz") or 0.0
        peak_inst = rates["dfma"][0]
        got_inst = K_CELL_FINAL_FP64 * CK / (dom_ms / 1e3)
        fp64 = {"bound": "fp64", "kernel": dom, "achieved": got_inst / 1e9,
                "peak": peak_inst / 1e9, "unit": "G FP64 inst/s",
                "frac": got_inst / peak_inst,
                "inst_per_cell_level": K_CELL_FINAL_FP64,
                "peak_source": "measured: swg_fp64_issue_rate (DFMA), this run",
                "issue_rates": {
                    op: {"G_inst_per_s": r / 1e9, "ms": round(ms, 3),
                         "per_sm_per_clock": (r / (sms * pk_mhz * 1e6)
                                              if pk_mhz else None)}
                    for op, (r, ms) in rates.items()},
                "peak_clocks": pk_clk}
    kernels = {k: {"ms_per_launch": v[0] / v[1], "launches_per_step": v[1],
                   "share": v[0] / sum(x[0] for x in prof.values())}
               for k, v in prof.items()}

    # end to end through the public API from page-locked host arrays: the
    # host-state stepper (copies of each level chunk overlap the other
    # chunks' compute), and beside it the serial upload + step + download
    e2e = None
    if not args.no_e2e:
        tuning = None
        if args.levels or args.level_chunk >= 0:
            hs = og.HostStepper(
                model, wl.stepper, wl.nstages, max(args.level_chunk, 0),
                levels=[int(n) for n in args.levels.split(",")]
                if args.levels else None)
        else:
            hs, tuning = og.HostStepper.autotuned(
                model, wl.stepper, wl.nstages, (h0, vn0, tr0), wl.dt)
        hh, vv, tt = hs.pinned_state()
        hh[...], vv[...], tt[...] = h0, vn0, tr0
        nbytes_in = hh.nbytes + vv.nbytes + tt.nbytes
        hs.step(hh, vv, tt, 0.0, wl.dt, 1, stream=sh)  # captures the graphs
        ups = world * wl.ncells * wl.nlayers * wl.nstages * args.e2e_steps

        def link_rates():
            """Host link rates of these page-locked arrays: whole-state
            upload and download (CUDA events, best of 3)."""
            up, down = [], []
            for _ in range(3):
                barrier()
                e0.record(stream)
                state.upload(hh, vv, tt, stream=sh)
                e1.record(stream)
                barrier()
                up.append(e0.elapsed_time(e1))
                e0.record(stream)
                state.download(stream=sh, out=(hh, vv, tt))
                e1.record(stream)
                barrier()
                down.append(e0.elapsed_time(e1))
            return {"h2d_gbs": round(nbytes_in / min(up) / 1e6, 1),
                    "d2h_gbs": round(nbytes_in / min(down) / 1e6, 1)}
        link_before = link_rates()
        e2e_clocks = ClockSampler(uuid)
        # let the sampler's start-up (driver queries of its own) finish
        # before the first timed call, then one untimed call: after the
        # idle second the clocks ramp up again during it
        time.sleep(1.0)
        hs.step(hh, vv, tt, 0.0, wl.dt, 1, stream=sh)
        barrier()
        call_ms = []
        e0.record(stream)
        for s in range(args.e2e_steps):
            t_call = time.perf_counter()
            hs.step(hh, vv, tt, s * wl.dt, wl.dt, 1, stream=sh)
            call_ms.append((time.perf_counter() - t_call) * 1e3)
        e1.record(stream)
        barrier()
        e2e_ms = e0.elapsed_time(e1)
        e2e_clk = e2e_clocks.stop()
        link_after = link_rates()
        hh[...], vv[...], tt[...] = h0, vn0, tr0
        barrier()
        e0.record(stream)
        for s in range(args.e2e_steps):
            state.upload(hh, vv, tt, stream=sh)
            stepper.step(state, s * wl.dt, wl.dt, 1, use_graph=True, stream=sh)
            state.download(stream=sh, out=(hh, vv, tt))
        e1.record(stream)
        barrier()
        serial_ms = e0.elapsed_time(e1)
        e2e = {"value": ups / (e2e_ms / 1e3), "unit": UNIT,
               "h2d_bytes_per_step": nbytes_in,
               "d2h_bytes_per_step": nbytes_in, "steps": args.e2e_steps,
               "ms_per_step": e2e_ms / args.e2e_steps,
               "api": "swg_host_step (HostStepper), page-locked host arrays",
               "level_chunks": hs.chunks,
               "call_ms": {"min": round(min(call_ms), 2),
                           "median": round(float(np.median(call_ms)), 2),
                           "max": round(max(call_ms), 2),
                           "each": [round(x, 2) for x in call_ms]},
               "chunk_tuning_ms_per_step": tuning and {
                   k: round(v, 2) for k, v in tuning.items()},
               "chunk_tuning_statistic": "median of 5 one-step calls",
               "host_link": {"before": link_before, "after": link_after,
                             "bytes_each_way": nbytes_in,
                             "numa": dict(zip(("gpu_node", "host_nodes"),
                                              gpu_numa_node()))},
               "clocks": e2e_clk,
               "serial_upload_step_download": {
                   "value": ups / (serial_ms / 1e3),
                   "ms_per_step": serial_ms / args.e2e_steps}}

    adjoint = None
    if rank == 0 and world == 1 and not args.no_adjoint:
        adjoint = adjoint_ratio(stream)
    ens = adj_ens = None
    if rank == 0 and world == 1 and not args.no_ensembles:
        e = ensemble_line(10, 3)
        ens = {"workload": "ensemble64", "value": e["value"], "unit": UNIT,
               "single_instance_sequential": e["single_instance_sequential"],
               "batch_over_single": e["batch_over_single"],
               "launch_config": e["config"]["launch_config"],
               "cell_levels": e["config"]["cell_levels"], "steps": 10}
        a = adjoint_ensemble_line()
        adj_ens = {"workload": "adjoint_ensemble32", "ratio": a["value"],
                   "members": a["config"]["members"],
                   "snapshots": a["config"]["snapshots"], "steps": a["steps"],
                   "batched_forward_ms": a["batched_forward_ms"],
                   "adjoint_forward_sweep_ms": a["adjoint_forward_sweep_ms"],
                   "adjoint_backward_sweep_ms": a["adjoint_backward_sweep_ms"],
                   "groups": a["groups"], "gpu_launches": a["gpu_launches"],
                   "stream_interleaved_ms": a["stream_interleaved_ms"],
                   "batched_over_sequential_speedup":
                       a["batched_over_sequential_speedup"]}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(wl)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": workload_config(wl, world, wl.nlayers),
            "roofline": roofline, "fp64_roofline": fp64, "kernels": kernels,
            "cpu_baseline": cpu, "e2e": e2e, "adjoint": adjoint,
            "ensemble": ens, "adjoint_ensemble": adj_ens,
            "gpu_launches": launches,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_ensemble(args):
    print(json.dumps(ensemble_line(args.steps, args.warmup)), flush=True)


def ensemble_line(steps, warmup):
    """The batched ensemble: 64 members (nx from {32..192}, 16-96 levels,
    1-4 tracers, RK4) advanced together in the autotuned launch shape
    (persistent kernel or one launch per pass, per RK stage), against the
    same members advanced one at a time by the single-instance path."""
    import torch
    import omega_playground_gb300 as og
    from omega_playground_gb300.workloads import ensemble, initial_state
    torch.cuda.set_device(0)
    wls = ensemble(n=64)
    members, states = [], []
    for wl in wls:
        mesh = og.PlanarHexagonalMesh(wl.nx, wl.ny, wl.dc, wl.nlayers)
        params = wl.params()
        model = og.ShallowWaterModel(mesh, params)
        st = og.ShallowWaterState(mesh, params)
        ic = initial_state(mesh, wl)
        st.upload(*ic)
        members.append((mesh, params, model, ic))
        states.append(st)
    units_step = sum(w.ncells * w.nlayers * 4 for w in wls)
    dt = wls[0].dt
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    batch = og.Batch([m[2] for m in members], states, "rk4", 4)
    cfg, tune_ms = batch.autotune(dt, reps=2, stream=sh)
    for st, m in zip(states, members):
        st.upload(*m[3])
    batch.step(0.0, dt, warmup, stream=sh)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    l0 = og.kernel_launches()
    e0.record(stream)
    batch.step(0.0, dt, steps, stream=sh, check_status=False)
    e1.record(stream)
    torch.cuda.synchronize()
    batch.check(sh)
    ms = e0.elapsed_time(e1)
    launches = og.kernel_launches() - l0
    value = units_step * steps / (ms / 1e3)
    # the same members one at a time (single-instance fused path, graph)
    single_ms = 0.0
    for (mesh, params, model, ic), st in zip(members, states):
        stp = og.RK4Stepper(model)
        stp.step(st, 0.0, dt, 1, stream=sh)
        torch.cuda.synchronize()
        e0.record(stream)
        stp.step(st, 0.0, dt, steps, stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        single_ms += e0.elapsed_time(e1)
    single = units_step * steps / (single_ms / 1e3)
    big = max(range(len(wls)), key=lambda i: wls[i].ncells * wls[i].nlayers)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1,
            "steps": steps, "warmup": warmup,
            "ms_per_step": ms / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": "ensemble64", "members": len(wls),
                       "cell_levels": units_step // 4,
                       "nx": sorted({w.nx for w in wls}),
                       "levels": [min(w.nlayers for w in wls),
                                  max(w.nlayers for w in wls)],
                       "tracers": [min(w.ntracers for w in wls),
                                   max(w.ntracers for w in wls)],
                       "stepper": "rk4", "launch_config": cfg,
                       "largest_member": wls[big].name},
            "single_instance_sequential": {"value": single,
                                           "ms_per_step": single_ms / steps},
            "batch_over_single": value / single, "gpu_launches": launches}
    return line


def run_adjoint_ensemble(args):
    print(json.dumps(adjoint_ensemble_line(args.adjoint_steps,
                                           not args.no_comparisons)),
          flush=True)


def adjoint_ensemble_line(nsteps_override=0, comparisons=True):
    """Batched adjoints: 32 members (nx from {32, 64, 96, 128}, 16-64 levels,
    2 tracers, RK4, 300 steps, per-cell log-normal viscosity), gradient of
    the region loss w.r.t. the initial state and the viscosity field, each
    member with its own checkpoint budget, run as one batched ensemble
    (og.AdjointEnsemble: one launch per pass over the members of each
    lockstep group).  Timed against the batched plain forward of the same
    members; the stream-interleaved form (one stream per member) and the
    members' adjoints run one after another are reported beside it."""
    import torch
    import omega_playground_gb300 as og
    from omega_playground_gb300.workloads import (adjoint_ensemble,
                                                  initial_state,
                                                  lognormal_visc,
                                                  loss_and_grad, region_cells,
                                                  visc_scaling)
    torch.cuda.set_device(0)
    wls = (adjoint_ensemble(n=32, nsteps=nsteps_override) if nsteps_override
           else adjoint_ensemble(n=32))
    mem = []
    for wl in wls:
        visc = lognormal_visc(wl.nx * wl.ny, wl.seed + 5)
        probe = og.PlanarHexagonalMesh(wl.nx, wl.ny, wl.dc, wl.nlayers)
        mesh = og.PlanarHexagonalMesh(
            wl.nx, wl.ny, wl.dc, wl.nlayers,
            mesh_scaling_del2=visc_scaling(probe, visc, wl.visc_del2))
        params = wl.params()
        model = og.ShallowWaterModel(mesh, params)
        x0 = initial_state(mesh, wl)
        # checkpoint budget per member: 32 snapshots, 16 for the largest
        nsnap = 16 if wl.nx >= 128 else 32
        mem.append(dict(wl=wl, mesh=mesh, params=params, model=model, x0=x0,
                        region=region_cells(mesh, wl.seed + 99), nsnap=nsnap))
    dt, nsteps = wls[0].dt, wls[0].nsteps
    units = sum(w.ncells * w.nlayers * 4 for w in wls) * nsteps
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    cur = torch.cuda.current_stream()

    def timed(fn):
        torch.cuda.synchronize()
        ev[0].record(cur)
        fn()
        torch.cuda.synchronize()
        ev[1].record(cur)
        torch.cuda.synchronize()
        return ev[0].elapsed_time(ev[1])

    # plain batched forward of the members
    states = []
    for m in mem:
        st = og.ShallowWaterState(m["mesh"], m["params"])
        st.upload(*m["x0"])
        states.append(st)
    batch = og.Batch([m["model"] for m in mem], states, "rk4", 4)
    best_cfg, _ = batch.autotune(dt, 2)
    batch.step(0.0, dt, 2)
    for st, m in zip(states, mem):
        st.upload(*m["x0"])
    fwd_ms = timed(lambda: batch.step(0.0, dt, nsteps))
    # batched adjoint: forward sweep, loss gradients, backward sweep
    adjs = [og.Adjoint(m["model"], m["nsnap"]) for m in mem]
    X0 = []
    XN = []
    for m in mem:
        a = og.ShallowWaterState(m["mesh"], m["params"])
        a.upload(*m["x0"])
        X0.append(a)
        XN.append(og.ShallowWaterState(m["mesh"], m["params"]))
    # the batched ensemble: every schedule action one launch per pass over
    # the members of a lockstep group (one group per snapshot budget)
    ens = og.AdjointEnsemble(adjs)
    # warm-up: a full-length forward sweep plans the members' schedules
    # (host, once per step and snapshot count), a 2-step pair builds the
    # tables and captures the graphs
    ens.forward(X0, 0.0, dt, nsteps, XN)
    ens.forward(X0, 0.0, dt, 2, XN)
    Gw = []
    for m in mem:
        G = og.ShallowWaterState(m["mesh"], m["params"])
        G.fill(0.0)
        Gw.append(G)
    ens.backward(Gw)
    torch.cuda.synchronize()
    l0 = og.kernel_launches()
    f_ms = timed(lambda: ens.forward(X0, 0.0, dt, nsteps, XN))
    Gs, loss = [], 0.0
    for m, xn in zip(mem, XN):
        L, g = loss_and_grad(*xn.download(), m["region"])
        loss += L
        G = og.ShallowWaterState(m["mesh"], m["params"])
        G.upload(*g)
        Gs.append(G)
    grads = [g.download() for g in Gs]
    b_ms = timed(lambda: ens.backward(Gs))
    launches = og.kernel_launches() - l0
    gvisc = [a.grad_visc()[1] for a in adjs]
    # the same adjoints, one stream per member (stream-interleaved actions)
    s_ms = stream_launches = seq_ms = None
    if comparisons:
        for G, g in zip(Gs, grads):
            G.upload(*g)
        streams = [torch.cuda.Stream() for _ in mem]
        sh = [s.cuda_stream for s in streams]
        l1 = og.kernel_launches()
        s_ms = timed(lambda: og.adjoint_batch_forward(adjs, X0, 0.0, dt,
                                                      nsteps, XN, sh))
        s_ms += timed(lambda: og.adjoint_batch_backward(adjs, Gs, sh))
        stream_launches = og.kernel_launches() - l1
        seq_ms = 0.0
    # the same adjoints one member at a time (default stream)
    for m in (mem if comparisons else []):
        a = og.Adjoint(m["model"], m["nsnap"])
        x = og.ShallowWaterState(m["mesh"], m["params"])
        x.upload(*m["x0"])
        xn = og.ShallowWaterState(m["mesh"], m["params"])
        seq_ms += timed(lambda: a.forward(x, 0.0, dt, nsteps, xn))
        g = og.ShallowWaterState(m["mesh"], m["params"])
        g.upload(*loss_and_grad(*xn.download(), m["region"])[1])
        seq_ms += timed(lambda: a.backward(g))
    line = {"metric": METRIC, "value": (f_ms + b_ms) / fwd_ms,
            "unit": "adjoint/forward time ratio", "n_gpus": 1,
            "steps": nsteps, "warmup": 2, "ms_per_step": (f_ms + b_ms) / nsteps,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": "adjoint_ensemble32", "members": len(wls),
                       "nx": sorted({w.nx for w in wls}),
                       "levels": [min(w.nlayers for w in wls),
                                  max(w.nlayers for w in wls)],
                       "tracers": 2, "stepper": "rk4",
                       "snapshots": sorted({m["nsnap"] for m in mem})},
            "batched_forward_ms": fwd_ms, "batch_config": best_cfg,
            "adjoint_forward_sweep_ms": f_ms,
            "adjoint_backward_sweep_ms": b_ms,
            "groups": ens.groups()[0], "gpu_launches": launches,
            "stream_interleaved_ms": s_ms,
            "stream_interleaved_launches": stream_launches,
            "sequential_member_adjoints_ms": seq_ms,
            "batched_over_sequential_speedup":
                seq_ms / (f_ms + b_ms) if seq_ms else None,
            "forward_updates_per_s": units / (fwd_ms / 1e3), "loss": loss,
            "grad_visc_norm": float(np.sqrt(sum(float(np.sum(g * g))
                                                for g in gvisc)))}
    return line


def run_adjoint(args):
    """The checkpointed adjoint alone: the time ratio as the line's value."""
    import torch
    torch.cuda.set_device(0)
    a = adjoint_ratio(torch.cuda.current_stream(), args.adjoint_steps,
                      args.snapshots)
    line = {"metric": METRIC, "value": a["ratio"],
            "unit": "adjoint/forward time ratio", "n_gpus": 1,
            "steps": a["steps"], "warmup": 3,
            "ms_per_step": (a["checkpointed_forward_ms"] + a["backward_ms"])
            / a["steps"], "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": "rk4_128x128_adjoint", "nx": 128, "ny": 128,
                       "nlayers": 32, "ntracers": 2, "stepper": "rk4",
                       "snapshots": a["snapshots"]},
            "adjoint": a}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload == "ensemble64":
        run_ensemble(args)
        return
    if args.workload == "adjoint_ensemble32":
        run_adjoint_ensemble(args)
        return
    if args.workload == "rk4_128x128_adjoint":
        run_adjoint(args)
        return
    from omega_playground_gb300.workloads import WORKLOADS
    wl = WORKLOADS[args.workload]
    if args.nx:
        wl = wl.scaled(nx=args.nx, ny=args.nx, name=f"{wl.name}@nx{args.nx}")
    if args.impl == "reference":
        run_reference(args, wl)
    else:
        run_ours(args, wl)


if __name__ == "__main__":
    main()

"""The multi-process path of bench.py on CPU (world size 2, gloo, 127.0.0.1).

The shallow-water path does not shard with communication: each rank
advances its own replica and only the timing is reduced.  Each rank here
advances an oracle replica of a small mesh, then the test checks the
max-over-ranks time, the whole-job throughput and that the replicas are
bitwise identical (they exchanged no data), and that the reference arm's
non-zero ranks exit without work."""
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from omega_playground_gb300.workloads import WORKLOADS
    wl = WORKLOADS["lsrk5_512x512"].scaled(nx=12, ny=12, nlayers=4,
                                           ntracers=2)
    units, times, cores, w = bench.oracle_sample(wl, wl.nlayers, 2, 1)
    ms = 1e3 * sum(times)
    dist.barrier()
    ms_max = bench.max_over_ranks(ms, world)
    value = bench.replica_throughput(units * len(times), ms_max, world)
    all_ms = [None] * world
    dist.all_gather_object(all_ms, ms)
    # the replica's final state, for the bitwise comparison
    import pyoracle
    om = pyoracle.OracleMesh(w.nx, w.ny, w.dc, w.nlayers)
    m = type("M", (), {})()
    for k, v in om.tables.items():
        setattr(m, "m_" + k, v)
    m.m_period_x, m.m_period_y = om.period_x, om.period_y
    from omega_playground_gb300.workloads import initial_state
    h, vn, tr = (np.ascontiguousarray(a) for a in initial_state(m, w))
    pyoracle.OracleModel(om, **w.param_kwargs()).step(h, vn, tr, 0.0, w.dt, 3,
                                                      w.stepper, w.nstages)
    states = [None] * world
    dist.all_gather_object(states, (h.tobytes(), vn.tobytes(), tr.tobytes()))
    if rank == 0:
        out.put((ms_max, all_ms, value, units * len(times), states))
    dist.destroy_process_group()


def test_two_replicas_max_time_and_independence():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    mp.spawn(_worker, args=(2, port, q), nprocs=2, join=True)
    ms_max, all_ms, value, units, states = q.get(timeout=60)
    assert ms_max == max(all_ms)
    assert value == pytest.approx(2 * units / (ms_max / 1e3))
    assert states[0] == states[1]


def _ref_worker(rank, world, port, out):
    sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world))
    import io
    import contextlib
    import bench
    from omega_playground_gb300.workloads import WORKLOADS

    class A:
        steps, warmup, gpus = 1, 1, world
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(A, WORKLOADS["lsrk5_512x512"].scaled(
            nx=8, ny=8, nlayers=2, ntracers=1))
    out.put((rank, buf.getvalue()))


def test_reference_arm_runs_on_rank_zero_only():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    mp.spawn(_ref_worker, args=(2, _free_port(), q), nprocs=2, join=True)
    got = dict(q.get(timeout=60) for _ in range(2))
    assert got[1] == ""
    import json
    line = json.loads(got[0].strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_arm_json_line(capsys, monkeypatch):
    """The reference arm's single JSON line on a small workload: the keys
    the contract names, impl "reference", cpu_baseline and a zero-copy
    e2e with the line's own value and unit."""
    import json
    import types
    sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    import bench
    from omega_playground_gb300.workloads import WORKLOADS
    wl = WORKLOADS["lsrk5_512x512"].scaled(nx=8, ny=8, nlayers=4, ntracers=2)
    args = types.SimpleNamespace(gpus=1, steps=2, warmup=1)
    bench.run_reference(args, wl)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup",
                "ms_per_step", "higher_is_better", "scaling", "vs_baseline",
                "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["steps"] == 2 and line["warmup"] == 1
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"],
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert line["config"]["workload"] == wl.name
    # the same config keys as the GPU arm's line (the workload, stepper,
    # dt, parallelism, L2 note and the sampled level count)
    assert line["config"] == bench.workload_config(wl, 1, wl.nlayers)
    assert cb["cpu_model"]

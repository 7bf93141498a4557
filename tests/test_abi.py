"""The C-ABI library loads on a machine without a GPU, exports every entry
point include/swgpu.h declares, and rejects bad input on the host before any
CUDA call."""
import ctypes as C
import os
import re

import numpy as np

from omega_playground_gb300 import _build, _capi

HEADER = os.path.join(os.path.dirname(_build.PKG), "include", "swgpu.h")


def declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(swg_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = _capi.lib()
    names = declared()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_capi.exported_symbols())


def test_version_and_launch_counter():
    assert b"sm_103a" in _capi.lib().swg_version()
    assert _capi.lib().swg_kernel_launches() >= 0


def _desc_for(nx, ny, K):
    from test_mesh_builder import product_tables
    t, _, _ = product_tables(nx, ny, 1.0)
    d = _capi.MeshDesc()
    d.ncells, d.nedges, d.nvertices, d.nlayers = nx * ny, 3 * nx * ny, \
        2 * nx * ny, K
    for n in ("nedges_on_cell", "edges_on_cell", "nedges_on_edge",
              "edges_on_edge", "cells_on_edge", "vertices_on_edge",
              "edges_on_vertex", "cells_on_vertex"):
        setattr(d, n, t[n].ctypes.data_as(C.POINTER(C.c_int)))
    for n in ("area_cell", "edge_sign_on_cell", "dc_edge", "dv_edge",
              "weights_on_edge", "area_triangle", "kiteareas_on_vertex",
              "edge_sign_on_vertex"):
        setattr(d, n, t[n].ctypes.data_as(C.POINTER(C.c_double)))
    return d, t


def test_mesh_create_rejects_out_of_range_connectivity():
    d, t = _desc_for(4, 4, 2)
    t["cells_on_edge"][5, 1] = 16  # == ncells: out of range
    out = C.c_void_p()
    rc = _capi.lib().swg_mesh_create(C.byref(d), C.byref(out))
    assert rc == 1 and not out.value
    assert b"out of range" in _capi.lib().swg_last_error()


def test_mesh_create_rejects_bad_sizes_and_nulls():
    d, _ = _desc_for(4, 4, 2)
    d.nlayers = 0
    out = C.c_void_p()
    assert _capi.lib().swg_mesh_create(C.byref(d), C.byref(out)) == 1
    d, _ = _desc_for(4, 4, 2)
    d.dc_edge = None
    assert _capi.lib().swg_mesh_create(C.byref(d), C.byref(out)) == 1
    assert b"NULL" in _capi.lib().swg_last_error()
    d, t = _desc_for(4, 4, 2)
    t["nedges_on_cell"][3] = 7
    assert _capi.lib().swg_mesh_create(C.byref(d), C.byref(out)) == 1


def test_mesh_create_rejects_max_levels_out_of_range():
    d, t = _desc_for(4, 4, 2)
    ml = np.full(16, 2, np.int32)
    ml[7] = 3  # > nlayers
    d.max_level_cell = ml.ctypes.data_as(C.POINTER(C.c_int))
    out = C.c_void_p()
    assert _capi.lib().swg_mesh_create(C.byref(d), C.byref(out)) == 1
    assert b"max level" in _capi.lib().swg_last_error()
    d, t = _desc_for(4, 4, 2)
    mv = np.full(32, -1, np.int32)
    d.max_level_vertex_bot = mv.ctypes.data_as(C.POINTER(C.c_int))
    assert _capi.lib().swg_mesh_create(C.byref(d), C.byref(out)) == 1


def test_null_handles_are_errors_not_crashes():
    lib = _capi.lib()
    assert lib.swg_state_create(None, 0, C.byref(C.c_void_p())) == 1
    assert lib.swg_model_create(None, None, C.byref(C.c_void_p())) == 1
    assert lib.swg_stepper_create(None, 0, 4, C.byref(C.c_void_p())) == 1
    assert lib.swg_step(None, None, 0.0, 1.0, 1, 0, None) == 1
    assert lib.swg_compute_tendency(None, None, None, 0.0, 0, None) == 1
    assert lib.swg_mesh_destroy(None) == 0
    # host-resident states
    out = C.c_void_p()
    assert lib.swg_host_stepper_create(None, 1, 5, 16, C.byref(out)) == 1
    assert not out.value
    levels = (C.c_int * 2)(3, 4)
    assert lib.swg_host_stepper_create_levels(None, 1, 5, 2, levels,
                                              C.byref(out)) == 1
    assert lib.swg_host_step(None, None, None, None, 0.0, 1.0, 1, None) == 1
    n = C.c_int(0)
    assert lib.swg_host_stepper_chunks(None, None, C.byref(n)) == 1
    assert lib.swg_host_stepper_destroy(None) == 0
    assert lib.swg_host_alloc(8, None) == 1
    assert lib.swg_host_free(None) == 0


def test_checkpoint_cost_matches_binomial_formula():
    """Plain advances of the optimal schedule equal Griewank-Walther's
    t(n, s) = r n - C(s + r, s + 1) with C(s + r - 1, s) < n <= C(s + r, s)
    (host-only planner, no GPU)."""
    from math import comb
    lib = _capi.lib()
    for n, s in [(1000, 32), (100, 5), (50, 1), (7, 3), (20, 4), (12, 12),
                 (300, 10)]:
        r = 0
        while comb(s + r, s) < n:
            r += 1
        t = r * n - comb(s + r, s + 1) if r > 0 else 0
        assert lib.swg_checkpoint_cost(n, s) == t, (n, s)
    assert lib.swg_checkpoint_cost(1000, 32) == 2405
    # outside the planner's range
    assert lib.swg_checkpoint_cost(10001, 32) == -1
    assert lib.swg_checkpoint_cost(0, 32) == -1
    assert lib.swg_checkpoint_cost(10, 0) == -1


def _plan_restated(N, S, ns):
    """The adjoint planner's dynamic program, restated (costs in hundredths
    of a plain step): f(n, s) reverses n steps from an available state, h(n,
    s) also produces the final state; 0 = the taped pair, m > 0 = split."""
    S = max(0, min(S, N - 1))
    cA, cT, cP = 100, 104, (100 * (ns - 1) + 40) // ns
    f = [[0] * (S + 1) for _ in range(N + 1)]
    h = [[0] * (S + 1) for _ in range(N + 1)]
    fm = [[0] * (S + 1) for _ in range(N + 1)]
    hm = [[0] * (S + 1) for _ in range(N + 1)]
    for n in range(1, N + 1):
        for s in range(S + 1):
            if n == 1:
                f[n][s], h[n][s] = cP, cT
                continue
            rest = f[n - 2][s] + (n - 2) * cA + cT
            bf, bh, mf, mh = rest + cP, rest + cT, 0, 0
            if s > 0:
                for m in range(1, n):
                    base = m * cA + f[m][s]
                    if base + f[n - m][s - 1] < bf:
                        bf, mf = base + f[n - m][s - 1], m
                    if base + h[n - m][s - 1] < bh:
                        bh, mh = base + h[n - m][s - 1], m
            f[n][s], fm[n][s], h[n][s], hm[n][s] = bf, mf, bh, mh
    return f, h, fm, hm, S


def _schedule(N, nsnap, ns):
    lib = _capi.lib()
    count = C.c_int(0)
    assert lib.swg_adj_schedule(N, nsnap, ns, 0, None, C.byref(count)) == 0
    buf = (C.c_int * (3 * count.value))()
    assert lib.swg_adj_schedule(N, nsnap, ns, count.value, buf,
                                C.byref(count)) == 0
    return [tuple(buf[3 * i:3 * i + 3]) for i in range(count.value)]


def _simulate(acts, N, nsnap):
    """Runs a schedule on positions only: every step is reversed once, in
    order N-1 ... 0, from a tape of that step; a tape is never overwritten
    before its step is reversed; snapshots stay in range."""
    cur, snaps, tapes, ended, rev = 0, {}, {}, False, []
    plain = tadv = 0
    for t, a, b in acts:
        if t == 0:
            assert cur == a and b > 0 and not (ended and a + b > N)
            cur += b
            plain += b
        elif t == 1:
            assert 0 <= a < nsnap
            snaps[a] = cur
        elif t == 2:
            cur = snaps[a]
        elif t == 3:
            assert ended and cur == a and tapes.get(b) is None
            rev.append(a)
        elif t == 4:
            assert cur == a and tapes.get(b) is None
            tapes[b] = a
            cur += 1
            tadv += 1
        elif t == 5:
            assert ended and tapes.get(b) == a
            tapes[b] = None
            rev.append(a)
        else:
            assert t == 6 and not ended and cur == N and not rev
            ended = True
    assert rev == list(range(N - 1, -1, -1))
    return plain, tadv


def test_adjoint_schedule_is_valid_and_optimal():
    """The adjoint's checkpoint schedule (host-only planner, no GPU): it
    reverses every step exactly once from that step's own tape with the
    given snapshots, and its counts are the restated dynamic program's."""
    import omega_playground_gb300 as og
    for N in list(range(1, 26)) + [40, 77]:
        for nsnap in (1, 2, 3, 5, 9):
            for ns in (4, 5, 1):
                acts = _schedule(N, nsnap, ns)
                plain, tadv = _simulate(acts, N, nsnap)
                assert og.adjoint_plan(N, nsnap, ns) == (plain, tadv)
                f, h, fm, hm, S = _plan_restated(N, nsnap - 1, ns)
                cP = (100 * (ns - 1) + 40) // ns
                ntape = N - tadv
                assert 100 * plain + 104 * tadv + cP * ntape == h[N][S], \
                    (N, nsnap, ns)
    # the benchmarked adjoint: 1000 RK4 steps, 32 snapshots
    plain, tadv = og.adjoint_plan(1000, 32, 4)
    assert (plain, tadv) == (1932, 440)
    assert plain + tadv < og.checkpoint_cost(1000, 32) == 2405
    assert _simulate(_schedule(1000, 32, 4), 1000, 32) == (plain, tadv)
    lib = _capi.lib()
    n = C.c_int(0)
    assert lib.swg_adj_schedule(10001, 32, 4, 0, None, C.byref(n)) == 1
    assert lib.swg_adj_schedule(10, 32, 3, 0, None, C.byref(n)) == 1


def test_adjoint_schedule_alternates_tapes():
    """In the backward sweep a taped advance never writes the tape that the
    most recent reversal read (it runs on the advance stream while that
    reversal may still run), and a tape from a state always writes it (it
    runs on the reversals' stream, after that reversal)."""
    for N, nsnap in ((12, 3), (77, 5), (300, 16), (1000, 32)):
        acts = _schedule(N, nsnap, 4)
        end = [i for i, a in enumerate(acts) if a[0] == 6][0]
        recent, checked = None, 0
        for t, a, b in acts[end + 1:]:
            if t == 4:
                assert recent is None or b != recent, (N, nsnap)
                checked += 1
            elif t == 3:
                assert recent is None or b == recent, (N, nsnap)
                recent = b
            elif t == 5:
                recent = b
        assert checked > 0


def test_host_stepper_edge_layout():
    """Chunk layouts with small end chunks (host-state stepper autotuning)."""
    import omega_playground_gb300 as og
    assert og.HostStepper.edge_layout(64, 16, 8) == [8, 16, 16, 16, 8]
    assert og.HostStepper.edge_layout(64, 16, 4) == [4, 16, 16, 16, 8, 4]
    assert og.HostStepper.edge_layout(7, 3, 1) == [1, 3, 2, 1]
    assert og.HostStepper.edge_layout(6, 3, 3) == [6]


def test_adjoint_plans_from_concurrent_threads():
    """The planner's process-wide cache under concurrent callers (ctypes
    releases the GIL during the call): every thread gets the counts that a
    lone call gives, for fresh and cached plans alike."""
    import threading
    import omega_playground_gb300 as og
    cases = [(n, s, ns) for n in (37, 120, 301) for s in (3, 7)
             for ns in (4, 5)]
    want = {c: og.adjoint_plan(*c) for c in cases}
    got, errors = [], []

    def worker(seed):
        try:
            order = cases[seed % len(cases):] + cases[:seed % len(cases)]
            for c in order + [(400 + seed, 5, 4)]:
                got.append((c, og.adjoint_plan(*c)))
        except Exception as e:  # reported below, not lost in the thread
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(8)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors
    for c, r in got:
        if c in want:
            assert r == want[c], c
        else:
            assert r == og.adjoint_plan(*c), c
    assert len(got) == 8 * (len(cases) + 1)


_OOM_CHILD = r"""
import ctypes as C, resource, sys
lib = C.CDLL(sys.argv[1])
lib.swg_last_error.restype = C.c_char_p
lib.swg_checkpoint_cost.restype = C.c_longlong
vm = [int(l.split()[1]) * 1024 for l in open("/proc/self/status")
      if l.startswith("VmSize:")][0]
# room for ordinary work, not for the plans' tables (several GB)
resource.setrlimit(resource.RLIMIT_AS, (vm + (256 << 20), vm + (256 << 20)))
p, t = C.c_longlong(0), C.c_longlong(0)
rc = lib.swg_adj_plan(10000, 10000, 4, C.byref(p), C.byref(t))
print("plan", rc, lib.swg_last_error().decode())
print("cost", lib.swg_checkpoint_cost(10000, 10000),
      lib.swg_last_error().decode())
"""


def test_host_allocation_failure_is_a_status_not_an_exception():
    """A host allocation that fails inside an entry point (here the
    planner's tables under an address-space limit, in a child process)
    comes back as SWG_ERR_OOM with a message; nothing throws across the C
    ABI and the process does not abort."""
    import subprocess
    import sys
    r = subprocess.run([sys.executable, "-c", _OOM_CHILD, _build.LIB],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = dict(l.split(" ", 1) for l in r.stdout.splitlines())
    assert lines["plan"].startswith("2 swg_adj_plan: host allocation"), r.stdout
    assert lines["cost"].startswith("-1 swg_checkpoint_cost: host allocation"), \
        r.stdout

"""bench.py's host-side bookkeeping, on the CPU: the clock record that
decides whether a measurement stands (the median SM clock and every
throttle reason seen while the timed steps ran), the L2 note, the
whole-job throughput of replicas, and the `config` object both arms print."""
import subprocess
import sys

import bench
from omega_playground_gb300.workloads import WORKLOADS

# nvidia-smi --format=csv,noheader,nounits lines for bench.ClockSampler.FIELDS
# (sm MHz, max sm MHz, power W, active-reasons mask, then four reasons)
_QUIET = "2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"
_CAPPED = "1965, 2070, 1398.7, 0x0000000000000004, Not Active, Not Active, Not Active, Active"
_HOT = "1500, 2070, 1100.0, 0x0000000000000040, Not Active, Active, Not Active, Not Active"


def _sampler(lines):
    """A ClockSampler whose process printed `lines` (a stand-in for
    nvidia-smi, which this machine may not have)."""
    s = bench.ClockSampler.__new__(bench.ClockSampler)
    text = "".join(line + "\n" for line in lines)
    s.proc = subprocess.Popen(
        [sys.executable, "-c", "import sys; sys.stdout.write(%r)" % text],
        stdout=subprocess.PIPE, text=True)
    s.proc.wait(timeout=30)
    return s


def test_clock_record_median_and_reasons():
    rec = _sampler([_QUIET, _QUIET, _CAPPED, "garbled line", _QUIET]).stop()
    assert rec["sm_mhz"] == 2070.0 and rec["sm_max_mhz"] == 2070.0
    assert rec["reasons"] == ["sw_power_cap"] and rec["samples"] == 4
    rec = _sampler([_HOT, _HOT, _QUIET]).stop()
    assert rec["sm_mhz"] == 1500.0
    assert rec["reasons"] == ["hw_thermal_slowdown"]
    rec = _sampler([]).stop()
    assert rec["sm_mhz"] is None and rec["samples"] == 0


def test_clock_record_without_a_sampler():
    s = bench.ClockSampler.__new__(bench.ClockSampler)
    s.proc = None
    assert s.stop()["reasons"] == ["unsampled"]


def test_l2_note_and_replica_throughput():
    assert "larger than L2; no flush" in bench.l2_note(1.61e9)
    assert "fits in L2" in bench.l2_note(50e6)
    # 4 replicas of 1e6 updates, the slowest rank took 250 ms
    assert bench.replica_throughput(10**6, 250.0, 4) == 1.6e7
    assert bench.max_over_ranks(12.5, 1) == 12.5


def test_both_arms_share_the_config_keys():
    wl = WORKLOADS["lsrk5_512x512"]
    cfg = bench.workload_config(wl, 1, wl.nlayers)
    assert cfg["workload"] == "lsrk5_512x512"
    assert (cfg["nx"], cfg["ny"], cfg["nlayers"], cfg["ntracers"]) == \
        (512, 512, 64, 8)
    assert {"dt", "parallelism", "l2", "sample_nlayers"} <= set(cfg)
    assert bench.workload_config(wl, 2, 16)["parallelism"] == "replicas x2"

"""The bench's clock record: nvidia-smi rows are read with their timestamps,
only samples taken while the frames ran count, throttle reasons are
collected, and a timed region too short for the 200 ms sampling period is
followed by untimed frames until the sampler has seen the load.  Checked on
CPU with the sampler's output file written by the test."""
import datetime
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


class _Done:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def _row(t, sm, reasons=()):
    ts = datetime.datetime.fromtimestamp(t).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
    flags = ["Active" if n in reasons else "Not Active" for n in bench.ClockSampler.REASONS]
    return f"{ts}, 0, {sm}, 2070, 900.0, 0x0, " + ", ".join(flags) + "\n"


def _sampler(lines):
    s = bench.ClockSampler.__new__(bench.ClockSampler)
    s.index, s.t0, s.t1, s.hold_frames = 0, None, None, 0
    import tempfile
    s.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
    s.f.write("".join(lines))
    s.f.flush()
    s.p = _Done()
    return s


def test_samples_before_the_timed_region_are_ignored():
    now = time.time()
    s = _sampler([_row(now - 2.0, 345), _row(now - 1.5, 345)])
    s.t0 = now - 1.0
    s.t1 = now - 0.5
    with open(s.f.name, "a") as f:
        f.write(_row(now - 0.8, 1965))
        f.write(_row(now - 0.3, 1980, ("sw_power_cap",)))
    c = s.stop()
    assert c["samples"] == 2 and c["samples_in_timed_region"] == 1
    assert c["sm_mhz"] == (1965 + 1980) / 2 and c["sm_max_mhz"] == 2070
    assert c["reasons"] == ["sw_power_cap"]


def test_hold_runs_frames_until_enough_samples():
    s = _sampler([])
    s.begin()
    frames = []

    def step():
        frames.append(1)
        with open(s.f.name, "a") as f:   # one sample per step, as if 200 ms passed
            f.write(_row(time.time(), 1900))
    s.hold(step, min_samples=3)
    assert len(frames) == 3 and s.hold_frames == 3
    s.end()
    c = s.stop()
    assert c["samples"] == 3 and c["hold_frames"] == 3


def test_no_samples_gives_none():
    s = _sampler([])
    s.begin()
    s.end()
    assert s.stop() is None

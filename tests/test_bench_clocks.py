"""bench.py's clock sampler on CPU: nvidia-smi lines with their own
timestamps, the samples before a timed region left out, the ones inside it
counted, throttle reasons collected (no GPU and no nvidia-smi needed)."""
import datetime
import os
import sys
import time

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)


class _Done:
    """Stands in for the finished nvidia-smi process."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def kill(self):
        pass


def _line(t, sm_mhz, power_cap="Not Active", hw="Not Active"):
    stamp = datetime.datetime.fromtimestamp(t).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
    return (f"{stamp}, 0, {sm_mhz}, 2070, 900.00, 0x0000000000000000, {hw}, Not Active, Not Active, "
            f"{power_cap}")


def _sampler(lines, begin=None, end=None):
    import bench

    c = bench.ClockSampler(0)
    c.lines = list(lines)
    c.proc = _Done()
    c.t_begin, c.t_end = begin, end
    return c


def test_samples_before_the_region_are_left_out():
    now = time.time()
    lines = [_line(now - 1.0, 1000), _line(now + 0.05, 2070), _line(now + 0.3, 2040, power_cap="Active"),
             _line(now + 0.5, 2070)]
    c = _sampler(lines, begin=now, end=now + 0.1)
    assert c.since_begin() == 3
    info = c.stop()
    assert info["samples"] == 3
    assert info["in_region"] == 1
    assert info["sm_mhz"] == 2070.0  # the idle 1000 MHz sample taken before the region is not counted
    assert info["sm_max_mhz"] == 2070.0
    assert info["reasons"] == ["sw_power_cap"]


def test_hardware_slowdown_is_reported():
    now = time.time()
    c = _sampler([_line(now + 0.1, 1500, hw="Active")], begin=now, end=now + 1.0)
    info = c.stop()
    assert info["reasons"] == ["hw_slowdown"]
    assert info["in_region"] == 1


def test_no_region_keeps_every_sample_and_malformed_lines_are_skipped():
    now = time.time()
    c = _sampler([_line(now, 2000), "garbage", _line(now + 0.1, 2070)])
    info = c.stop()
    assert info["samples"] == 2
    assert "in_region" not in info


def test_no_sample_after_the_region_began_gives_none():
    now = time.time()
    c = _sampler([_line(now - 2.0, 2070)], begin=now, end=now + 0.1)
    assert c.since_begin() == 0
    assert c.stop() is None

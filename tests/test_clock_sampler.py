"""bench.py's clock sampler against a stand-in nvidia-smi (CPU only): the
sample taken before the timed region starts is left out, the samples during it
and the one after it are kept, and throttle reasons marked Active are reported."""
import importlib.util
import os
import stat
import sys
import textwrap
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

FAKE = textwrap.dedent("""\
    #!{python}
    import sys, time
    time.sleep(0.3)  # start-up delay
    print("0, 1000, 2070, 100.0, 0x0, Not Active, Not Active, Not Active, Not Active", flush=True)
    i = 0
    while True:
        time.sleep(0.05)
        cap = "Active" if i == 1 else "Not Active"
        print(f"0, 2070, 2070, 900.0, 0x4, Not Active, Not Active, Not Active, {{cap}}", flush=True)
        i += 1
""")


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_sampler_window(bench, tmp_path):
    exe = tmp_path / "fake-smi"
    exe.write_text(FAKE.format(python=sys.executable))
    exe.chmod(exe.stat().st_mode | stat.S_IXUSR)
    s = bench.ClockSampler(0, cmd=str(exe))
    t0 = time.monotonic()
    s.start()
    assert time.monotonic() - t0 >= 0.25  # returned only after the first sample
    time.sleep(0.2)  # the timed region
    c = s.stop()
    assert c["sm_mhz"] == 2070.0 and c["sm_max_mhz"] == 2070.0
    assert c["samples"] >= 2
    assert c["reasons"] == ["sw_power_cap"]
    assert s.proc.poll() is not None


def test_sampler_without_nvidia_smi(bench, tmp_path):
    s = bench.ClockSampler(0, cmd=str(tmp_path / "missing"))
    s.start()
    assert s.stop()["reasons"] == ["nvidia-smi unavailable"]

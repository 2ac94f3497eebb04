"""bench.py's reference arm, run on a small case of the same band without a GPU.

The reference arm times the CPU restatement of the reference path (oracle/)
and prints one JSON line: impl "reference", the metric, a value,
cpu_baseline and e2e.  Run here at n = 20,000 so it takes seconds.
"""
import json
import os
import subprocess
import sys

from tests.conftest import ROOT


def test_reference_arm_prints_its_line():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "20000", "--partitions",
           "8", "--steps", "1", "--warmup", "0"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "solves/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert "n=20,000" in line["config"]["workload"] and "partitions=8" in line["config"]["workload"]


def test_reference_arm_reports_the_counts_it_ran():
    """The line's steps and warmup are the solves actually timed and run
    before them (requests above the caps are cut, and the line says so), and
    steps x ms_per_step stays within the timed seconds it reports."""
    import bench

    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "20000", "--partitions",
           "8", "--steps", str(bench.REF_MAX_STEPS + 5), "--warmup", str(bench.REF_MAX_WARMUP + 2)]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["steps"] == bench.REF_MAX_STEPS and line["warmup"] == bench.REF_MAX_WARMUP
    assert line["steps_requested"] == bench.REF_MAX_STEPS + 5
    # the median step is at most the mean: K median steps fit in the timed total
    assert line["steps"] * line["ms_per_step"] / 1000.0 <= line["timed_s"] * 1.5


def _free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_under_two_ranks_prints_once():
    """Launched the way a multi-GPU run is (torch.distributed.run, 2 ranks):
    rank 0 alone times the CPU path and prints; rank 1 exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--rows", "20000",
           "--partitions", "8", "--steps", "1", "--warmup", "0"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0


def test_one_core_sample_runs_on_one_thread_and_restores_the_default():
    sys.path.insert(0, ROOT)
    import bench
    from oracle import oracle

    before = oracle.set_threads(0)
    line = bench.cpu_one_core(20000, 8, 2)
    assert line["cores"] == 1 and line["kind"] == "port" and line["value"] > 0
    assert "2 of the 8 partitions" in line["sample"]
    assert oracle.set_threads(0) == before


def test_clock_sampler_counts_only_the_timed_region(tmp_path):
    """The sampler against a stand-in for nvidia-smi that prints a row every
    20 ms: start() returns once rows flow, and stop() summarises the rows
    after begin() (clock median, max clock, throttle reasons seen)."""
    sys.path.insert(0, ROOT)
    import time

    import bench

    fake = tmp_path / "fake-smi"
    fake.write_text(f"#!{sys.executable}\n"
                    "import time\n"
                    "i = 0\n"
                    "while True:\n"
                    "    cap = 'Active' if i >= 8 else 'Not Active'\n"
                    "    print(f'{1800 + 100 * (i % 3)}, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, {cap}',"
                    " flush=True)\n"
                    "    i += 1\n"
                    "    time.sleep(0.02)\n")
    fake.chmod(0o755)
    s = bench.ClockSampler(0, interval_ms=20, cmd=str(fake))
    s.start()
    assert s.rows and s.mark == len(s.rows)
    s.begin()
    time.sleep(0.4)
    out = s.stop()
    assert out["samples"] >= 5 and out["interval_ms"] == 20
    assert out["sm_max_mhz"] == 2070.0 and 1800.0 <= out["sm_mhz"] <= 2000.0
    assert out["reasons"] == ["sw_power_cap"]
    missing = bench.ClockSampler(0, cmd=str(tmp_path / "absent"))
    missing.start()
    assert missing.stop()["reasons"] == ["nvidia-smi unavailable"]


def test_clock_sampler_falls_back_to_200_ms(tmp_path):
    """A tool that refuses the short interval (exits without output) is
    started again at 200 ms."""
    sys.path.insert(0, ROOT)
    import time

    import bench

    fake = tmp_path / "picky-smi"
    fake.write_text(f"#!{sys.executable}\n"
                    "import sys, time\n"
                    "if sys.argv[sys.argv.index('-lms') + 1] != '200':\n"
                    "    sys.exit(2)\n"
                    "while True:\n"
                    "    print('2070, 2070, 800.0, 0x0, Not Active, Not Active, Not Active, Not Active', flush=True)\n"
                    "    time.sleep(0.2)\n")
    fake.chmod(0o755)
    s = bench.ClockSampler(0, interval_ms=50, cmd=str(fake))
    s.start()
    s.begin()
    time.sleep(0.5)
    out = s.stop()
    assert out["interval_ms"] == 200 and out["samples"] >= 1 and out["sm_mhz"] == 2070.0 and out["reasons"] == []

"""bench.py's reference arm (`--impl reference`) on the CPU: the reference's algorithm as
the oracle port, timed on the host's cores, printing one JSON line with the same metric,
unit and workload as the GPU arm and its cpu_baseline / e2e objects. Runs at a tiny
sample so the check takes seconds; it needs no GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line(M, O):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                        "--warmup", "0", "--cpu-sample", "24"], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "photon_paths_per_s" and d["unit"] == "paths/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 2 and d["warmup"] == 0
    assert d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and "24 photons" in cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_gpu_arm_fails_loudly_without_a_device(M):
    """Without a CUDA device the GPU arm exits non-zero with the library's error and prints
    no number: there is no CPU fallback behind it."""
    if M.lib().mcrt_device_count() > 0:
        import pytest

        pytest.skip("a CUDA device is visible")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--steps", "1", "--warmup", "3",
                        "--no-extras"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode != 0
    assert r.stdout.strip() == ""
    assert "no CUDA device is visible" in r.stderr


def test_reference_arm_does_not_load_the_library():
    """The reference arm builds its workload from the oracle's own types and Mie tables:
    the process never imports the library's package nor maps libmcrt.so."""
    code = (
        "import sys, runpy\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', '--cpu-sample', '8']\n"
        "runpy.run_path('bench.py', run_name='__main__')\n"
        "maps = open('/proc/self/maps').read()\n"
        "assert 'mcrt_gb300' not in sys.modules, 'package imported'\n"
        "assert 'libmcrt.so' not in maps, 'libmcrt.so mapped'\n"
        "assert 'libmcrt_oracle.so' in maps\n"
        "print('checked')\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().endswith("checked")

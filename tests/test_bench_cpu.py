"""bench.py's reference arm runs on the host cores (the CPU FFT stand-in for
the reference's FFTW path), so its JSON line can be checked here: one line,
the contract keys, the reference's own metric and config."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def _run(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args],
                       capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


def test_reference_arm_line():
    d = _run("--impl", "reference", "--workload", "c2c3d_64x1", "--steps", "2",
             "--warmup", "1")
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["unit"] == "GB/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 2
    assert d["config"]["workload"] == "c2c3d_64x1"
    assert d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"]


def test_reference_arm_special_workloads():
    """The ragged batch and the Poisson step have CPU legs too: pocketfft
    over a sample of the ragged grids, and the whole loss + gradient step in
    complex64 numpy."""
    for w in ("ragged48", "poisson4x128"):
        d = _run("--impl", "reference", "--workload", w, "--steps", "1")
        assert d["impl"] == "reference" and d["value"] > 0, w
        assert d["cpu_baseline"]["kind"] == "port"


def test_gpus_n_starts_n_ranks():
    """`bench.py --gpus 2` started without torchrun starts two rank
    processes itself; rank 0 prints one line with n_gpus 2 and the max of
    the ranks' times (dry run: gloo, no GPU, made-up times 1 + rank ms)."""
    d = _run("--gpus", "2", "--dry-run")
    assert d["n_gpus"] == 2
    assert d["ms_per_step"] == 2.0
    assert d["dry_run"] is True


def test_reference_arm_reports_requested_gpus():
    d = _run("--impl", "reference", "--workload", "c2c3d_64x1", "--gpus", "2",
             "--steps", "1", "--warmup", "1")
    assert d["n_gpus"] == 2 and d["impl"] == "reference"

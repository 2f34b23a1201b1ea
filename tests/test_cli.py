"""The command-line driver (fft3d-fpga_gb300/cli/fft.c): the reference
example's options (examples/helper.cpp:44-57), its entry-point selection
(examples/fft.cpp:37-73), verification by the reference's SNR > 120 dB rule
against an FP64 host FFT, and the measurement report.

CPU tests cover option parsing and the initialisation failure without a
GPU; GPU tests run every entry-point path with verification on."""
import os
import subprocess

import pytest

from conftest import gpu_available


@pytest.fixture(scope="module")
def cli(libpath):
    exe = os.path.join(os.path.dirname(libpath), "fft")
    assert os.access(exe, os.X_OK)
    return exe


def _run(cli, *args, timeout=300):
    return subprocess.run([cli, *args], capture_output=True, text=True, timeout=timeout)


def test_help(cli):
    r = _run(cli, "-h")
    assert r.returncode == 0
    for flag in ("--num", "--dim", "--back", "--iter", "--path", "--noverify",
                 "--batch", "--burst", "--use_bram", "--use_usm", "--emulate"):
        assert flag in r.stdout


def test_missing_path_is_an_error(cli):
    r = _run(cli, "-n", "16")
    assert r.returncode == 1
    assert "path" in r.stderr


@pytest.mark.parametrize("args", [["-d", "4"], ["-n", "x"], ["-i", "0"], ["--bogus"],
                                  ["extra"]])
def test_bad_options(cli, tmp_path, args):
    f = tmp_path / "p.json"
    f.write_text("{}")
    r = _run(cli, "-p", str(f), *args)
    assert r.returncode == 1


def test_configuration_banner_and_init_failure_without_gpu(cli, tmp_path):
    if gpu_available():
        pytest.skip("a GPU is present")
    f = tmp_path / "p.json"
    f.write_text("{}")
    r = _run(cli, "-p", str(f), "-n", "32", "-d", "2", "-b", "-c", "3")
    assert "Points             : 32^2" in r.stdout
    assert "Direction          : Backward" in r.stdout
    assert "Batch              : 3" in r.stdout
    assert r.returncode == 1 and "initialization error" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("args", [
    ["-d", "1", "-n", "4096", "-c", "3"],
    ["-d", "1", "-n", "65536", "-c", "2", "-b"],
    ["-d", "1", "-n", "1024", "-s"],
    ["-d", "2", "-n", "256"],
    ["-d", "2", "-n", "128", "-m", "-c", "4", "-b"],
    ["-d", "2", "-n", "64", "-m", "-s", "-c", "2"],
    ["-d", "3", "-n", "64"],
    ["-d", "3", "-n", "32", "-m", "-b"],
    ["-d", "3", "-n", "64", "-c", "3", "-i", "3"],
    ["-d", "3", "-n", "32", "-s"],
    ["-d", "3", "-n", "32", "-s", "-c", "2", "-b"],
])
def test_cli_paths_verify(cli, cuda, tmp_path, args):
    f = tmp_path / "p.json"
    f.write_text("{}")
    r = _run(cli, "-p", str(f), *args)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Throughput" in r.stdout and "GB/s" in r.stdout
    assert "FAILED" not in r.stdout

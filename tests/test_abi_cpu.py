"""The drop-in boundary without a GPU: the library loads, exports every
symbol the public headers declare, keeps the reference's struct layout, and
rejects invalid arguments the way the reference's gtest suite expects
(tests/test_fft1d_fpga.cpp, test_fft2d_fpga.cpp, test_fft3d_fpga.cpp,
test_fft_setup.cpp)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, gpu_available

INCLUDE = os.path.join(ROOT, "include")


def declared_functions():
    names = set()
    for f in ("fftfpga.h", "fftfpga_ext.h"):
        text = open(os.path.join(INCLUDE, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
            name = m.group(1)
            if name.startswith(("fpga_", "fftfpga", "fftgb_")) and name != "fpga_timing":
                names.add(name)
    return sorted(names)


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert "fftfpgaf_c2c_3d_ddr_batch" in names and "fftgb_exec" in names
    assert len(names) >= 30
    for name in names:
        assert hasattr(lib, name), name


def test_reference_entry_points_present(lib):
    ref = ["fpga_initialize", "fpga_final", "fftfpga_complex_malloc",
           "fftfpgaf_complex_malloc", "fftfpga_c2c_1d", "fftfpgaf_c2c_1d",
           "fftfpgaf_c2c_1d_svm", "fftfpgaf_c2c_2d_bram",
           "fftfpgaf_c2c_2d_bram_svm", "fftfpgaf_c2c_2d_ddr",
           "fftfpgaf_c2c_3d_bram", "fftfpgaf_c2c_3d_ddr",
           "fftfpgaf_c2c_3d_ddr_batch", "fftfpgaf_c2c_3d_ddr_svm",
           "fftfpgaf_c2c_3d_ddr_svm_batch"]
    for name in ref:
        assert hasattr(lib, name), name


def test_struct_layout():
    from fftgb._lib import FpgaT, Float2, Double2
    assert ctypes.sizeof(FpgaT) == 48
    assert FpgaT.valid.offset == 40
    assert FpgaT.exec_t.offset == 16
    assert ctypes.sizeof(Float2) == 8
    assert ctypes.sizeof(Double2) == 16


@pytest.fixture(scope="module")
def validity_bin(libpath, tmp_path_factory):
    d = tmp_path_factory.mktemp("cbin")
    exe = str(d / "test_validity")
    libdir = os.path.dirname(libpath)
    src = os.path.join(ROOT, "tests", "c", "test_validity.c")
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I" + INCLUDE, src,
                    "-L" + libdir, "-lfftfpga", "-Wl,-rpath," + libdir, "-o", exe],
                   check=True)
    return exe


@pytest.mark.skipif(gpu_available(), reason="CPU-only variant (no device)")
def test_c_validity_suite_without_gpu(validity_bin):
    r = subprocess.run([validity_bin], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr


def test_python_validity(lib):
    buf = np.zeros(64 * 64 * 64 * 2, np.complex64)
    p = buf.ctypes.data
    assert not lib.fftfpgaf_c2c_1d(64, None, p, False, 1).valid
    assert not lib.fftfpgaf_c2c_1d(63, p, p, False, 1).valid
    assert not lib.fftfpgaf_c2c_1d(64, p, p, False, 0).valid
    assert not lib.fftfpgaf_c2c_2d_ddr(63, p, p, False).valid
    assert not lib.fftfpgaf_c2c_2d_bram(64, p, None, False, False, 1).valid
    assert not lib.fftfpgaf_c2c_3d_ddr(48, p, p, False).valid
    assert not lib.fftfpgaf_c2c_3d_ddr_batch(64, p, p, False, False, 1).valid
    assert not lib.fftfpgaf_c2c_3d_ddr_svm(64, p, p, False, False).valid
    assert not lib.fftfpgaf_c2c_2d_bram_svm(64, p, p, False, 1).valid
    assert not lib.fftfpga_c2c_1d(64, None, p, False, 1).valid


def test_malloc(lib):
    assert lib.fftfpgaf_complex_malloc(0) is None
    assert lib.fftfpga_complex_malloc(0) is None
    p = lib.fftfpgaf_complex_malloc(4096)
    assert p and p % 64 == 0
    ctypes.CDLL(None).free(ctypes.c_void_p(p))


@pytest.mark.skipif(gpu_available(), reason="CPU-only variant (no device)")
def test_init_codes_without_gpu(lib, tmp_path):
    f = tmp_path / "plans.cache"
    f.write_text("")
    assert lib.fpga_initialize(b"NVIDIA CUDA", b"", False) == -1
    assert lib.fpga_initialize(b"NVIDIA CUDA", None, False) == -1
    assert lib.fpga_initialize(b"TEST", str(f).encode(), False) == -2
    assert lib.fpga_initialize(b"cuda", str(f).encode(), False) == -3


@pytest.mark.skipif(gpu_available(), reason="CPU-only variant (no device)")
def test_ext_api_without_gpu(lib):
    h = ctypes.c_void_p()
    assert lib.fftgb_plan_3d(ctypes.byref(h), 8, 8, 8, 1, 0) == -2  # ENODEV
    assert lib.fftgb_plan_1d(None, 8, 1, 0) == -1
    assert lib.fftgb_exec(None, None, None, 0, 1.0, None) == -1
    assert lib.fftgb_version().startswith(b"fftgb")

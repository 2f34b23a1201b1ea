"""Build libfftfpga.so in-tree (fft3d-fpga_gb300/lib/) for sm_103a.

    python fft3d-fpga_gb300/build.py          # incremental
    python fft3d-fpga_gb300/build.py --clean  # from scratch

Also builds the command-line driver lib/fft (cli/fft.c) against the library.

CUDA sources are compiled with nvcc for sm_103a only, the C host library
with gcc; translation units compile in parallel and the shared library links
against the shared CUDA runtime.  No cmake, no network.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
INC = os.path.join(ROOT, "include")
OUT = os.path.join(HERE, "lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libfftfpga.so")
CLI_SRC = "cli/fft.c"
CLI = os.path.join(OUT, "fft")

NVCC = os.environ.get("NVCC", "nvcc")
CC = os.environ.get("CC", "gcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                  "-I" + INC, "--expt-relaxed-constexpr"]
CFLAGS = ["-O2", "-std=c11", "-fPIC", "-Wall", "-Wextra", "-Werror",
          "-I" + INC]

CU_SOURCES = [
    "kernels/fft_pass.cu",
    "kernels/fft_pass_tma.cu",
    "kernels/fft3d_fused.cu",
    "kernels/fft3d_fused_tma.cu",
    "kernels/fft1d_cluster.cu",
    "kernels/fft3d_cluster.cu",
    "kernels/spectral.cu",
    "kernels/tc_selftest.cu",
    "kernels/fft_tc.cu",
    "kernels/fft_ragged.cu",
    "kernels/fft_real.cu",
    "kernels/fft_blue.cu",
    "kernels/fft_mix.cu",
    "kernels/fft_mix_real.cu",
    "kernels/fft_mix_4s.cu",
    "kernels/fft_mix2_a.cu",
    "kernels/fft_mix2_b.cu",
    "kernels/fft_mix2_c.cu",
    "kernels/fft_mix3_d.cu",
    "kernels/fft_mix3_e.cu",
    "kernels/fft_mix3_f.cu",
    "kernels/fft_mix3_g.cu",
    "kernels/fft_mix3_h.cu",
    "kernels/fft_mix3_i.cu",
    "shim/shim.cu",
    "shim/ragged.cu",
    "shim/noalloc.cu",
    "shim/real.cu",
]
C_SOURCES = [
    "api/src/fftfpga.c",
    "api/src/fft1d.c",
    "api/src/fft2d.c",
    "api/src/fft3d.c",
]
HEADERS = [
    "kernels/fft_core.cuh",
    "kernels/fft_pass.cuh",
    "kernels/fft3d_fused.cuh",
    "kernels/fft3d_fused_cfg.cuh",
    "kernels/fft1d_cluster.cuh",
    "kernels/fft3d_cluster.cuh",
    "kernels/spectral.cuh",
    "kernels/filter.cuh",
    "kernels/fft_tc.cuh",
    "kernels/fft_ragged.cuh",
    "kernels/fft_real.cuh",
    "kernels/fft_blue.cuh",
    "kernels/fft_mix.cuh",
    "kernels/fft_mix_impl.cuh",
    "kernels/tc_core.cuh",
    "shim/shim.h",
    "shim/worklist.h",
    "shim/tables.h",
]


def _obj_name(src: str) -> str:
    return os.path.join(OBJ, src.replace("/", "_") + ".o")


def _stale(src: str, obj: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [os.path.join(HERE, src)] + [os.path.join(HERE, h) for h in HEADERS]
    deps += [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src: str) -> tuple[str, str]:
    obj = _obj_name(src)
    path = os.path.join(HERE, src)
    if src.endswith(".cu"):
        cmd = [NVCC] + NVFLAGS + ["-c", path, "-o", obj]
    else:
        cmd = [CC] + CFLAGS + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}{r.stderr}")
    return obj, r.stderr


def build(clean: bool = False, verbose: bool = False) -> str:
    if clean and os.path.isdir(OUT):
        shutil.rmtree(OUT)
    os.makedirs(OBJ, exist_ok=True)
    sources = CU_SOURCES + C_SOURCES
    todo = [s for s in sources if _stale(s, _obj_name(s))]
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(todo))) as ex:
            for obj, err in ex.map(_compile, todo):
                if verbose and err.strip():
                    print(err, file=sys.stderr)
    objs = [_obj_name(s) for s in sources]
    if todo or not os.path.exists(LIB):
        cmd = [NVCC] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}{r.stderr}")
    cli_src = os.path.join(HERE, CLI_SRC)
    if (not os.path.exists(CLI) or os.path.getmtime(CLI) < os.path.getmtime(LIB)
            or os.path.getmtime(CLI) < os.path.getmtime(cli_src)):
        cmd = [CC] + CFLAGS + [cli_src, "-o", CLI, "-L" + OUT, "-lfftfpga", "-lm",
                               "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed: {' '.join(cmd)}\n{r.stdout}{r.stderr}")
    return LIB


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--clean", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(clean=a.clean, verbose=a.verbose))


if __name__ == "__main__":
    main()

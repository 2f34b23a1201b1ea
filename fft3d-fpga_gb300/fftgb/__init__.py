"""fftgb - Python access to libfftfpga.so, the GB300 implementation of the
FFTFPGA C API (include/fftfpga.h) and its extensions (include/fftfpga_ext.h).

    import fftgb.api      # host numpy arrays through the reference's entry points
    import fftgb.plan     # torch CUDA tensors through device-pointer plans
    import fftgb.autograd # torch.autograd.Function over the adjoint kernels
"""
from ._lib import FFTGBError, lib, load, last_error  # noqa: F401

__all__ = ["FFTGBError", "lib", "load", "last_error"]

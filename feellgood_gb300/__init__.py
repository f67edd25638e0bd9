"""GB300 implementation of FeeLLGood's per-time-step LLG update.

The compute path is the C-ABI library ``_build/libfggpu.so`` (hand-written sm_103a CUDA
kernels plus C++ host code), declared in ``include/fggpu.h``. This package only binds it
with ctypes; there is no Python or CPU fallback for any compute call.
"""
from .api import (Context, load_msh, cuboid, rng_seed, rng_angle, run, settings_dump, checkpoint_peek, pinned_empty, measure_peaks, FgError, StepReport, fg_lib, lib_path, GAMMA0, MU0, FG_OK,  # noqa: F401
                  FG_SOLVER_ITER_OVERFLOW, FG_SOLVER_CANNOT_CONVERGE, FG_ETIMEDOUT, FG_PREC_FP64,
                  FG_PREC_FP32_REFINE, FG_DEMAG_AUTO, FG_DEMAG_DIRECT, FG_DEMAG_FMM)

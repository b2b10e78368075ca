"""GB300-native ABC simulation + rejection hot path of
pthomaslab/abc_inference_transcription: a C-ABI CUDA library (libabcgpu.so,
include/abcgpu.h) with a Python host mirror of the reference's interface."""
from .abi import FP32, FP64, AbcConfig, AbcError, AbcPrior, MODEL_NAMES, load_library, nstats, num_params  # noqa: F401
from .config import (CellTable, factor_prior, make_config, minute_prior, reference_prior,  # noqa: F401
                     synthetic_cells)

__all__ = ["FP32", "FP64", "AbcConfig", "AbcPrior", "AbcError", "MODEL_NAMES", "load_library", "nstats", "num_params",
           "CellTable", "make_config", "reference_prior", "factor_prior", "minute_prior", "synthetic_cells"]

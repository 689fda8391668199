"""GB300-native P3 microphysics (EAMxx ``p3_main``) behind the reference's call surface.

The compute lives in libp3x.so (CUDA for sm_103a, C ABI in include/p3x.h);
this package holds the Python-side mirror of the reference interface.
"""
from . import _lib
from ._lib import (P3X_FP64, P3X_FP32_BULK, P3X_STAGE_PART12, P3X_STAGE_SED, P3X_STAGE_PART3, P3Error, Runtime,
                   default_runtime, load, INPUT_FIELDS, OUTPUT_FIELDS, PROG_FIELDS, ALL_FIELDS)
from .p3 import P3Batch, P3Context, P3Fields, P3Microphysics, P3Server, generate_inputs

__all__ = ["P3X_FP64", "P3X_FP32_BULK", "P3X_STAGE_PART12", "P3X_STAGE_SED", "P3X_STAGE_PART3", "P3Error",
           "Runtime", "default_runtime", "load", "P3Batch", "P3Context", "P3Fields", "P3Microphysics", "P3Server", "generate_inputs", "INPUT_FIELDS",
           "OUTPUT_FIELDS", "PROG_FIELDS", "ALL_FIELDS"]

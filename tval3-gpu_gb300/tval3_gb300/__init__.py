"""tval3_gb300: GB300-native (sm_103a) TVAL3 reconstruction.

The computation lives in libtval3_gb300.so (hand-written CUDA kernels behind a
C ABI, include/tval3/tval3_c.h); this package is the Python view of that ABI
plus seeded synthetic workloads and the PyTorch autograd binding.
"""
from .capi import (PREC_BF16, PREC_BF16_DF64, PREC_FP16, PREC_FP16_DF64, PREC_FP32, PREC_FP32_DF64,
                   PREC_FP32_F64VEC, PREC_FP64, TRAV_BRESENHAM, TRAV_SIDDON, TV_ANISO, TV_ISO, Tval3Error,
                   default_options, load)
from .api import (Batch, D, DenseMatrix, Dt, Geometry, Operator, Solver, SparseMatrix, tval3_gpu, tval3_gpu_3d,
                  tval3_gpu_batched)

__all__ = ["PREC_BF16", "PREC_BF16_DF64", "PREC_FP16", "PREC_FP16_DF64", "PREC_FP32", "PREC_FP32_DF64",
           "PREC_FP32_F64VEC", "PREC_FP64",
           "TRAV_BRESENHAM", "TRAV_SIDDON",
           "TV_ANISO",
           "TV_ISO", "Tval3Error", "default_options", "load", "D", "DenseMatrix", "Dt", "Geometry", "Operator",
           "Solver", "SparseMatrix", "tval3_gpu", "tval3_gpu_3d", "Batch", "tval3_gpu_batched"]

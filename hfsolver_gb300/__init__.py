"""GB300-native (sm_103a) kernels for hfsolver's molecular Gaussian-orbital path.

The compute path is libhfgpu.so (hand-written CUDA for sm_103a, C ABI in
include/hfgpu.h); this package is its Python face, with the reference's
routine names (see hfsolver_gb300.api).
"""
from .api import (HFGPUError, RHFOptions, SCFNotConverged, autotune_clear, autotune_table, basis_size, boys,
                  doscf, eigh, find_pole_diag, formG, getints2, getInts, getS, getT, getV, jk, mbpt2, mbpt3, mp2_energy, packed_size, rhf, rhf_batch,
                  rhf_gauss, rhf_gradient, transform_int2, tridiag_eigen)
from ._lib import LIB_PATH

__all__ = ["HFGPUError", "RHFOptions", "SCFNotConverged", "autotune_clear", "autotune_table", "basis_size", "boys", "doscf",
           "eigh", "find_pole_diag", "formG", "getints2", "getInts", "getS",
           "getT", "getV", "jk", "mbpt2", "mbpt3", "mp2_energy", "packed_size", "rhf", "rhf_batch", "rhf_gauss",
           "rhf_gradient", "transform_int2", "tridiag_eigen", "LIB_PATH"]

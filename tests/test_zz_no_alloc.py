"""The allocation-free Fock build, hfgpu_formG_device_noalloc, through the C ABI.

Some callers cannot let a library allocate device memory: their memory is
owned by their own allocator or a fixed quota, or a cudaMalloc would stall a
latency-critical loop.  For them the library offers this variant of
hfgpu_formG, which works on device buffers the caller owns and keeps its
scratch in a fixed 2 MiB per-device array.  This test gives it device buffers
made by the caller (torch here), calls it twice in a row with different
densities (the shared scratch must be cleared between calls), and compares
each result with the allocating entry point hfgpu_formG within the tolerance
the other parity tests use.  It also checks that a basis larger than the
scratch limit is refused with a clear error.  The file sorts last so that a
run stopping at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from tests.golden_reference_answers import CASES
from tests.gpu_common import assert_close

pytestmark = pytest.mark.gpu


def test_noalloc_formG_matches_formG(oracle):
    import torch

    import hfsolver_gb300 as hf
    from hfsolver_gb300 import _lib

    L = _lib.lib()
    c = CASES["NH3"]
    ref = oracle.rhf_gauss(c["atno"], np.array(c["xyz"], float))
    int2 = ref["int2"]
    n = ref["P"].shape[0]
    dev = torch.device("cuda", 0)
    d_int2 = torch.from_numpy(int2.copy()).to(dev)
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(7)
    for call in range(2):
        if call == 0:
            P = ref["P"]
        else:
            P = rng.standard_normal((n, n))
            P = 0.5 * (P + P.T)
        expect = hf.formG(P, int2)
        d_P = torch.from_numpy(np.asfortranarray(P).ravel(order="F").copy()).to(dev)
        d_G = torch.full((n * n,), np.nan, dtype=torch.float64, device=dev)
        rc = L.hfgpu_formG_device_noalloc(n, ctypes.c_void_p(d_int2.data_ptr()), ctypes.c_void_p(d_P.data_ptr()),
                                          ctypes.c_void_p(d_G.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == _lib.OK, L.hfgpu_last_error()
        torch.cuda.synchronize(dev)
        G = d_G.cpu().numpy().reshape(n, n, order="F")
        assert_close(G, expect, 1e-11, 1e-11, f"call {call}")

    rc = L.hfgpu_formG_device_noalloc(513, ctypes.c_void_p(d_int2.data_ptr()), ctypes.c_void_p(d_P.data_ptr()),
                                      ctypes.c_void_p(d_G.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == _lib.ERR_INVALID
    assert b"512" in L.hfgpu_last_error()

"""The allocation-free Fock build, hfgpu_formG_device_noalloc, through the C ABI.

Some callers cannot let a library allocate device memory: their memory is
owned by their own allocator or a fixed quota, or a cudaMalloc would stall a
latency-critical loop.  For them the library offers this variant of
hfgpu_formG, which works on device buffers the caller owns and keeps its
scratch in a fixed 2 MiB per-device array.  This test gives it device buffers
made by the caller (torch here), calls it twice in a row with different
densities (the shared scratch must be cleared between calls), and compares
each result with the oracle's formG and with the allocating entry point
hfgpu_formG, within the tolerance the other parity tests use.  The device's
free memory must not change across the second call.  It also checks that a
basis larger than the scratch limit is refused with a clear error.  The file
sorts last so that a run stopping at the first failure has already run every
other test."""
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
    rng = np.random.default_rng(7)
    P1 = rng.standard_normal((n, n))
    densities = [ref["P"], 0.5 * (P1 + P1.T)]
    expect_oracle = [oracle.formG(P, int2) for P in densities]
    expect_lib = [hf.formG(P, int2) for P in densities]

    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    d_int2 = torch.from_numpy(int2.copy()).to(dev)
    d_Ps = [torch.from_numpy(np.asfortranarray(P).ravel(order="F").copy()).to(dev) for P in densities]
    d_Gs = [torch.full((n * n,), np.nan, dtype=torch.float64, device=dev) for _ in densities]
    torch.cuda.synchronize(dev)
    free = []
    for call, (d_P, d_G) in enumerate(zip(d_Ps, d_Gs)):
        free.append(torch.cuda.mem_get_info(dev)[0])
        rc = L.hfgpu_formG_device_noalloc(n, ctypes.c_void_p(d_int2.data_ptr()), ctypes.c_void_p(d_P.data_ptr()),
                                          ctypes.c_void_p(d_G.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == _lib.OK, L.hfgpu_last_error()
        torch.cuda.synchronize(dev)
    free.append(torch.cuda.mem_get_info(dev)[0])
    assert free[2] == free[1], f"the second call changed the device's free memory: {free[1]} -> {free[2]}"
    for call, d_G in enumerate(d_Gs):
        G = d_G.cpu().numpy().reshape(n, n, order="F")
        assert_close(G, expect_oracle[call], 1e-11, 1e-11, f"call {call} vs oracle formG")
        assert_close(G, expect_lib[call], 1e-11, 1e-11, f"call {call} vs hfgpu_formG")

    d_P, d_G = d_Ps[0], d_Gs[0]
    rc = L.hfgpu_formG_device_noalloc(513, ctypes.c_void_p(d_int2.data_ptr()), ctypes.c_void_p(d_P.data_ptr()),
                                      ctypes.c_void_p(d_G.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == _lib.ERR_INVALID
    assert b"512" in L.hfgpu_last_error()

"""The C ABI (include/hfgpu.h) without a GPU: the library loads, exports every
declared entry point, the ctypes table matches the header, and host-side
validation rejects bad input with a status code instead of aborting (the
reference's stop_error ends the process)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hfgpu.h")


@pytest.fixture(scope="module")
def L():
    from hfsolver_gb300 import _lib

    if not os.path.exists(_lib.LIB_PATH):
        from hfsolver_gb300.build import build

        build()
    return _lib.lib()


def declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(hfgpu_\w+)\s*\(", txt)))


def test_every_declared_symbol_is_exported(L):
    names = declared()
    assert len(names) >= 12
    for n in names:
        assert hasattr(L, n), n


def test_binding_table_covers_header(L):
    from hfsolver_gb300 import _lib

    assert set(_lib.SIGNATURES) == set(declared())


def test_struct_layouts(L):
    from hfsolver_gb300 import _lib

    o = _lib.Options()
    L.hfgpu_default_options(o)
    assert o.nscf == 40 and o.mix_alpha == 1.0 and o.tolE == 1e-10 and o.tolP == 1e-8
    assert ctypes.sizeof(_lib.Options) == 88  # int, 3 doubles, 2 ints, double, 2 ints, int[8]
    assert ctypes.sizeof(_lib.Result) == 216  # 6 doubles, 4 ints, 3 int64, 16 doubles


def test_basis_size(L):
    import hfsolver_gb300 as hf

    assert hf.basis_size([8, 1, 1]) == 25
    assert hf.basis_size([8, 1, 1] * 8) == 200
    assert hf.basis_size([99]) == 0


def test_invalid_input_is_a_status_not_an_abort(L):
    import hfsolver_gb300 as hf
    from hfsolver_gb300 import _lib

    with pytest.raises(hf.HFGPUError) as e:
        hf.rhf([99], [[0, 0, 0]])
    assert e.value.code == _lib.ERR_INVALID
    with pytest.raises(hf.HFGPUError) as e:
        hf.rhf([8, 1, 1], [[0, 0, 0], [np.nan, 0, 0], [0, 1, 0]])
    assert e.value.code == _lib.ERR_INVALID
    with pytest.raises(hf.HFGPUError) as e:  # f shells (Z >= 21) are not supported
        hf.rhf([26], [[0, 0, 0]])
    assert e.value.code == _lib.ERR_UNSUPPORTED
    # getInts with an istart outside coef/alpha
    with pytest.raises(hf.HFGPUError) as e:
        hf.getInts([3], [5], [0.0], [0.0], [0.0], [0], [0], [0], [1.0], [1.0])
    assert e.value.code == _lib.ERR_INVALID
    # getints2 with a wrong int2 length
    Lb = L
    n = 1
    arr_i = (ctypes.c_int * 1)(1)
    arr_d = (ctypes.c_double * 3)(0, 0, 0)
    arr_p = (ctypes.c_int * 3)(0, 0, 0)
    c1 = (ctypes.c_double * 1)(1.0)
    out = (ctypes.c_double * 1)(0.0)
    rc = Lb.hfgpu_getints2(n, arr_i, arr_i, arr_d, arr_p, 1, c1, c1, out, 7)
    assert rc == _lib.ERR_INVALID
    assert b"m(m+1)/2" in Lb.hfgpu_last_error()


def test_eigh_rejects_bad_arguments_before_the_gpu(L):
    """hfgpu_eigh validates sizes and pointers on the host (no device work)."""
    import hfsolver_gb300 as hf
    from hfsolver_gb300 import _lib

    buf = (ctypes.c_double * 4)()
    assert L.hfgpu_eigh(0, buf, buf, buf, buf) == _lib.ERR_INVALID
    assert L.hfgpu_eigh(2, None, buf, buf, buf) == _lib.ERR_INVALID
    assert L.hfgpu_eigh(2, buf, buf, buf, None) == _lib.ERR_INVALID
    with pytest.raises(ValueError):
        hf.eigh(np.eye(3), np.eye(2))
    # the host tridiagonal solver: sizes and non-finite input
    assert L.hfgpu_tridiag_eigen(0, buf, buf, buf, buf) == _lib.ERR_INVALID
    with pytest.raises(ValueError):
        hf.tridiag_eigen([1.0, 2.0], [])


def test_boys_rejects_bad_arguments_before_the_gpu(L):
    """hfgpu_boys checks its arguments on the host, as the reference's Fm stops
    on them (src/special_functions.f90:218-221)."""
    from hfsolver_gb300 import _lib

    T = (ctypes.c_double * 2)(1.0, -1.0)
    F = (ctypes.c_double * 40)()
    assert L.hfgpu_boys(13, 1, T, F) == _lib.ERR_INVALID
    assert L.hfgpu_boys(-1, 1, T, F) == _lib.ERR_INVALID
    assert L.hfgpu_boys(4, 2, T, F) == _lib.ERR_INVALID
    assert b"T must be" in L.hfgpu_last_error()
    T[1] = float("nan")
    assert L.hfgpu_boys(4, 2, T, F) == _lib.ERR_INVALID


def test_find_pole_diag_rejects_bad_arguments_before_the_gpu(L):
    from hfsolver_gb300 import _lib

    buf = (ctypes.c_double * 64)()
    it = ctypes.c_int(0)
    assert L.hfgpu_find_pole_diag(4, buf, buf, 2, 0, 10, 1e-10, buf, ctypes.byref(it)) == _lib.ERR_INVALID
    assert L.hfgpu_find_pole_diag(4, buf, buf, 2, 5, 10, 1e-10, buf, ctypes.byref(it)) == _lib.ERR_INVALID
    assert L.hfgpu_find_pole_diag(4, buf, buf, 4, 1, 10, 1e-10, buf, ctypes.byref(it)) == _lib.ERR_INVALID
    assert L.hfgpu_find_pole_diag(4, buf, buf, 2, 1, 0, 1e-10, buf, ctypes.byref(it)) == _lib.ERR_INVALID

"""The roofline work units (hfsolver_gb300/roofline.py) against the count the
library itself sums into eri_flops (hfgpu_md_flops), and a few fixed values.
Needs no GPU."""
import itertools

import pytest

from hfsolver_gb300 import roofline


@pytest.fixture(scope="module")
def L():
    from hfsolver_gb300 import _lib

    return _lib.lib()


def test_md_flops_matches_the_library(L):
    for la, lb, lc, ld in itertools.product(range(3), repeat=4):
        assert L.hfgpu_md_flops(la, lb, lc, ld) == roofline.md_flops(la, lb, lc, ld)


def test_md_flops_fixed_values():
    # (ss|ss): 30 + 0 + 2 C(4,4) + 2 + 2
    assert roofline.md_flops(0, 0, 0, 0) == 36
    # (dd|dd): L = 8, nH(4) = 35, 36 components per side
    assert roofline.md_flops(2, 2, 2, 2) == 30 + 24 + 2 * 495 + 2 * 36 * 35 * 35 + 2 * 36 * 36 * 35
    assert roofline.nherm(4) == 35 and roofline.ncart(2) == 6


def test_transform_and_tensor_counts():
    n, o, v = 400, 80, 320
    assert roofline.transform_flops(n, o, v) == 2 * o * n**4 + 2 * o * v * n**3 + 2 * o**2 * v * n**2 + \
        2 * o**2 * v**2 * n
    assert roofline.tensor_flops(128, 64, 32) == 2 * 21 * 128 * 64 * 32
    assert roofline.mp2_sum_bytes(40, 160) == 8 * 40**2 * 160**2
    assert roofline.fock_flops(1000) == 12000 and roofline.fock_bytes(1000) == 8000

"""Oracle C restatement against hfsolver's own src/cints.c + src/qc.c compiled
unmodified into oracle/_ref/libref.so (only where the reference sources were
present at build time; skipped elsewhere).  The restatement keeps the
reference's operation order, so agreement is bit-for-bit."""
import ctypes
import os

import numpy as np
import pytest

from tests.golden_reference_answers import CASES

REF = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                   "libref.so")
pytestmark = pytest.mark.skipif(not os.path.exists(REF), reason="reference build not present")


@pytest.fixture(scope="module")
def ref(oracle):
    L = ctypes.CDLL(REF)
    oracle._bind(L, prefix="")
    return L


@pytest.mark.parametrize("name", ["H2O", "CH4_1", "NH3", "Ne"])
def test_bit_exact_integrals(oracle, ref, name):
    c = CASES[name]
    b = oracle.Basis(c["atno"], np.array(c["xyz"], float))
    a = oracle.getInts(b)
    r = oracle.getInts(b, L=ref, prefix="")
    assert np.array_equal(a, r)
    for w in "STV":
        assert np.array_equal(oracle.one_electron(b, w), oracle.one_electron(b, w, L=ref, prefix=""))

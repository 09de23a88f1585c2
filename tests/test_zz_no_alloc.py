"""sesp_energies_static (fixed scratch, no device allocation) against
sesp_energies, through the C ABI, on consecutive calls.

The scratch array is shared by every call on a device and keeps the last
call's contents, so the checks run twice in a row, on a state whose energies
changed in between, and after a larger system has filled more of the array.
"""
import ctypes

import numpy as np
import pytest

from surfactant_enhanced_spreading_gb300 import engine as E
from surfactant_enhanced_spreading_gb300 import system as S

pytestmark = pytest.mark.gpu

TOL_PLAIN = 1e-10


def _static(eng):
    out = np.full(8, np.nan)
    E._check(E._lib.sesp_energies_static(eng._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    return out


def _close(a, b):
    scale = np.abs(b).sum()
    return np.abs(a - b).max() / scale < TOL_PLAIN


@pytest.mark.parametrize("precision", [E.PLAIN_FP64, E.MIXED])
def test_static_matches_allocating_on_two_calls(precision):
    big = E.Engine(S.droplet(2000, 20, cells=(12, 12, 8), seed=5), precision)
    big.force(True)
    assert _close(_static(big), big.energies())
    big.close()

    eng = E.Engine(S.droplet(600, 6, cells=(8, 8, 8), seed=21), precision)
    eng.force(True)
    ref = eng.energies()
    first = _static(eng)
    second = _static(eng)
    assert _close(first, ref), (first, ref)
    assert _close(second, ref), (second, ref)
    assert np.array_equal(first, second)
    # both entry points add the same per-site energies in the same order
    assert np.array_equal(first, ref)

    E.mybox_start(eng)
    eng.run(99101, 15)
    eng.force(False)
    ref2 = eng.energies()
    third = _static(eng)
    fourth = _static(eng)
    assert not np.array_equal(ref2, ref)
    assert _close(third, ref2), (third, ref2)
    assert _close(fourth, ref2), (fourth, ref2)
    assert np.array_equal(third, ref2)


def test_static_rejects_contexts_beyond_its_scratch():
    s = S.droplet(20000, 200, cells=(24, 24, 12), seed=2024, graphite_layers=0)
    eng = E.Engine([s, s], E.MIXED)
    assert eng.replica_count() == 2
    assert eng.state()[0].shape[0] > 131072
    out = np.zeros(8)
    with pytest.raises(E.SespError, match="EINVAL.*exceed its fixed scratch"):
        E._check(E._lib.sesp_energies_static(eng._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    assert np.all(out == 0.0)

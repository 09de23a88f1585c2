"""The pair field's launch shape (work-item tile, CTAs per SM) is picked by
the autotuner; no shape may change any result."""
import numpy as np
import pytest

from surfactant_enhanced_spreading_gb300 import engine as E
from surfactant_enhanced_spreading_gb300 import system as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sys_small():
    return S.droplet(600, 6, cells=(8, 8, 8), seed=21)


@pytest.mark.parametrize("precision", [E.PLAIN_FP64, E.MIXED])
def test_shapes_give_identical_forces(sys_small, precision):
    eng = E.Engine(sys_small, precision)
    f0 = eng.force(True)
    tile, cps, mx = eng.autotune()
    assert tile in (32, 64) and 1 <= cps <= mx
    assert eng.tuning() == (tile, cps, mx)
    assert np.array_equal(eng.force(True), f0)
    for shape in [(32, 1), (64, 1), (32, mx), (64, mx), (64, max(1, mx // 2))]:
        eng.set_tuning(*shape)
        assert eng.tuning()[:2] == shape
        assert np.array_equal(eng.force(True), f0), shape
        assert np.array_equal(eng.force(False), f0), shape


def test_shapes_give_identical_trajectories(sys_small):
    runs = []
    for shape in [(64, None), (32, 1)]:
        eng = E.Engine(sys_small, E.MIXED)
        eng.force(True)
        if shape[1] is None:
            eng.autotune()
        else:
            eng.set_tuning(*shape)
        eng.init_accel()
        eng.run(99101, 25)
        runs.append(eng.state())
    for a, b in zip(runs[0], runs[1]):
        assert np.array_equal(a, b)


def test_invalid_shapes_are_refused(sys_small):
    eng = E.Engine(sys_small, E.MIXED)
    with pytest.raises(E.SespError, match="EINVAL"):
        eng.set_tuning(48, 1)
    with pytest.raises(E.SespError, match="EINVAL"):
        eng.set_tuning(64, 0)
    with pytest.raises(E.SespError, match="ESTATE"):
        eng.autotune()   # no force call yet

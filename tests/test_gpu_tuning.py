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
    assert tile in ((32, 64, 128) if precision == E.MIXED else (32, 64)) and 1 <= cps <= mx
    assert eng.tuning() == (tile, cps, mx)
    assert np.array_equal(eng.force(True), f0)
    shapes = [(32, 1), (64, 1), (32, mx), (64, mx), (64, max(1, mx // 2))]
    if precision == E.MIXED:
        shapes += [(128, 1), (128, 4)]
    for shape in shapes:
        eng.set_tuning(*shape)
        assert eng.tuning()[:2] == shape
        assert np.array_equal(eng.force(True), f0), shape
        assert np.array_equal(eng.force(False), f0), shape


def test_shapes_give_identical_trajectories(sys_small):
    runs = []
    for shape in [(64, None), (32, 1), (128, 2)]:
        eng = E.Engine(sys_small, E.MIXED)
        eng.force(True)
        if shape[1] is None:
            eng.autotune()
        else:
            eng.set_tuning(*shape)
        eng.init_accel()
        eng.run(99101, 25)
        runs.append(eng.state())
    for other in runs[1:]:
        for a, b in zip(runs[0], other):
            assert np.array_equal(a, b)


def test_invalid_shapes_are_refused(sys_small):
    eng = E.Engine(sys_small, E.MIXED)
    with pytest.raises(E.SespError, match="EINVAL"):
        eng.set_tuning(48, 1)
    with pytest.raises(E.SespError, match="EINVAL"):
        eng.set_tuning(64, 0)
    plain = E.Engine(sys_small, E.PLAIN_FP64)
    with pytest.raises(E.SespError, match="EINVAL"):
        plain.set_tuning(128, 1)   # 4 targets per lane: the FP32 path only
    with pytest.raises(E.SespError, match="ESTATE"):
        eng.autotune()   # no force call yet


@pytest.mark.parametrize("precision", [E.MIXED, E.MIXED_FP32C])
def test_constraint_shapes_give_identical_trajectories(precision):
    """Surfactant warps per CTA of the constraint halves, and the water order
    that every rebuild derives from the previous sweeps, change no bit."""
    s = S.droplet(900, 30, cells=(8, 8, 8), seed=5)   # 30 surfactants: 4 groups of up to 8
    runs = []
    mx = 2 if precision == E.MIXED else 8
    for sw in ((1, 1), (2, mx), (4, 2), (3, 1), None):
        eng = E.Engine(s, precision)
        eng.force(True)
        if sw is None:
            eng.autotune()
            tun = eng.constraint_tuning()
            assert 1 <= tun[0] <= 4 and 1 <= tun[1] <= mx and tun[2:] == (4, mx)
        else:
            eng.set_constraint_tuning(*sw)
            assert eng.constraint_tuning() == sw + (4, mx)
        eng.init_accel()
        eng.run(99101, 25)
        runs.append(eng.state() + (eng.eta, eng.counters()[0]))
        eng.close()
    for r in runs[1:]:
        for a, b in zip(runs[0], r):
            assert np.array_equal(a, b)


def test_autotune_restores_the_state():
    s = S.droplet(700, 12, cells=(8, 8, 8), seed=6)
    eng = E.Engine(s, E.MIXED)
    E.mybox_start(eng)
    eng.run(99101, 7)
    before = eng.state() + (eng.eta,)
    eng.autotune()
    after = eng.state() + (eng.eta,)
    for a, b in zip(before, after):
        assert np.array_equal(a, b)
    with pytest.raises(E.SespError, match="EINVAL"):
        eng.set_constraint_tuning(0, 1)
    with pytest.raises(E.SespError, match="EINVAL"):
        eng.set_constraint_tuning(5, 1)
    with pytest.raises(E.SespError, match="EINVAL"):
        eng.set_constraint_tuning(1, 3)   # SESP_MIXED: at most 2 surfactants per warp
    eng.close()

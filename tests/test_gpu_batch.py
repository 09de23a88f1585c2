"""Several replica droplets of uneven size in one context (one launch per
kernel for all of them): every replica's result equals the same system run
alone, bit for bit, since each cell's arithmetic is independent of the rest."""
import numpy as np
import pytest

from surfactant_enhanced_spreading_gb300 import engine as E
from surfactant_enhanced_spreading_gb300 import system as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def systems():
    return [S.droplet(300, 2, cells=(8, 8, 4), seed=31), S.droplet(900, 8, cells=(8, 8, 8), seed=32),
            S.droplet(150, 0, cells=(4, 4, 4), seed=33)]


@pytest.mark.parametrize("precision", [E.PLAIN_FP64, E.MIXED])
def test_batch_forces_equal_alone(systems, precision):
    batch = E.Engine(systems, precision)
    assert batch.replica_count() == 3
    fb = batch.force(True)
    for q, s in enumerate(systems):
        alone = E.Engine(s, precision)
        fa = alone.force(True)
        assert np.array_equal(fb[batch.offsets[q]:batch.offsets[q + 1]], fa)


def test_batch_trajectory_equal_alone(systems):
    batch = E.Engine(systems, E.PLAIN_FP64)
    batch.force(True)
    batch.init_accel()
    batch.run(99101, 20)
    pb, vb, _ = batch.state()
    etas = batch.etas()
    for q, s in enumerate(systems):
        alone = E.Engine(s, E.PLAIN_FP64)
        alone.force(True)
        alone.init_accel()
        alone.run(99101, 20)
        pa, va, _ = alone.state()
        sl = slice(batch.offsets[q], batch.offsets[q + 1])
        assert np.array_equal(pb[sl], pa)
        assert np.array_equal(vb[sl], va)
        assert etas[q] == alone.eta


def test_per_replica_eta_and_failures(systems):
    """sesp_set_eta_batch sets each replica's thermostat variable (and
    sesp_set_state gives all replicas the same one); sesp_failures_batch
    splits the SHAKE / RATTLE failure count by replica."""
    batch = E.Engine(systems, E.MIXED)
    batch.force(True)
    batch.init_accel()
    batch.set_etas([0.5, -0.25, 0.125])
    assert list(batch.etas()) == [0.5, -0.25, 0.125]
    batch.set_state(None, None, None, 0.75)
    assert list(batch.etas()) == [0.75, 0.75, 0.75]
    with pytest.raises(ValueError):
        batch.set_etas([0.0, 0.0])
    batch.set_etas([0.0, 0.0, 0.0])
    batch.run(99101, 10)
    f = batch.failures()
    assert f.shape == (3,) and f.sum() == batch.counters()[0] == 0

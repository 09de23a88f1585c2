"""Diagnostics on the GPU: the reference's consistency checks (molecule
count, total charge, O and H counts) and its temperature-rescaling variant,
through the C ABI, against counts and sums taken on the host; and the state
transfers of the C ABI."""
import numpy as np
import pytest

from surfactant_enhanced_spreading_gb300 import engine as E
from surfactant_enhanced_spreading_gb300 import initial as I
from surfactant_enhanced_spreading_gb300 import system as S

pytestmark = pytest.mark.gpu


def _expected(s):
    return [s.n_water + s.n_surf, s.n_water + s.n_surf, None, s.n_water, 2 * s.n_water, s.n_water, 0, 0]


@pytest.mark.parametrize("precision", [E.PLAIN_FP64, E.MIXED])
def test_checks_on_a_droplet(precision):
    s = S.droplet(1500, 15, cells=(8, 8, 8), seed=12)
    eng = E.Engine(s, precision)
    with pytest.raises(E.SespError):
        eng.checks()                       # no cell lists before a force call
    eng.force(True)
    row = eng.checks()
    assert row.shape == (1, 8)
    exp = _expected(s)
    for k in (0, 1, 3, 4, 5, 6, 7):
        assert row[0, k] == exp[k], (k, row[0])
    # the model is neutral: water and surfactant charges sum to zero
    assert abs(row[0, 2]) < 1e-9
    E.mybox_start(eng)
    eng.run(99101, 20)
    eng.force(True)
    again = eng.checks()
    assert np.array_equal(again[:, [0, 1, 3, 4, 5, 6, 7]], row[:, [0, 1, 3, 4, 5, 6, 7]])
    eng.close()


def test_checks_per_replica():
    systems = [S.droplet(700, 5, cells=(8, 8, 8), seed=3), S.droplet(400, 0, cells=(8, 8, 8), seed=4)]
    eng = E.Engine(systems, E.MIXED)
    eng.force(True)
    rows = eng.checks()
    assert rows.shape == (2, 8)
    for s, r in zip(systems, rows):
        exp = _expected(s)
        for k in (0, 1, 3, 4, 5, 6, 7):
            assert r[k] == exp[k], (k, r)
    eng.close()


def test_rescale_temperature_with_reference_velocities():
    s = S.droplet(1200, 12, cells=(8, 8, 8), seed=8)
    s.vel = I.reference_velocities(s.pos, s.n_water, s.n_surf, s.cells)
    eng = E.Engine(s, E.PLAIN_FP64)
    t0 = eng.temperature()
    assert abs(t0 / S.TR - 1.0) < 1e-12
    before = eng.rescale_temperature()            # the reference's target, 3.9
    assert before == t0
    assert abs(eng.temperature() / E.RESCALE_TARGET - 1.0) < 1e-12
    _, vel, _ = eng.state()
    f = np.sqrt(E.RESCALE_TARGET / t0)
    assert np.array_equal(vel, f * s.vel)
    with pytest.raises(E.SespError):
        eng.rescale_temperature(0.0)
    eng.close()


def test_state_round_trip_through_the_staging_buffer():
    """sesp_set_state / sesp_download_state move (n, 3) arrays through one
    copy each and a transposing kernel: exact round trip, partial uploads
    leave the other arrays alone, and state(out=...) fills caller buffers."""
    s = S.droplet(300, 3, cells=(8, 8, 8), seed=9)
    eng = E.Engine(s, E.MIXED)
    rng = np.random.default_rng(1)
    p, v, a = (s.pos + 1e-3 * rng.normal(size=s.pos.shape) for _ in range(3))
    eng.set_state(p, v, a, eta=0.25)
    p2, v2, a2 = eng.state()
    assert np.array_equal(p2, p) and np.array_equal(v2, v) and np.array_equal(a2, a)
    assert eng.eta == 0.25
    v3 = v * 2.0
    eng.set_state(vel=v3, eta=0.5)
    out = tuple(np.empty_like(p) for _ in range(3))
    eng.state(out=out)
    assert np.array_equal(out[0], p) and np.array_equal(out[1], v3) and np.array_equal(out[2], a)

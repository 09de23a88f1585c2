"""The configuration preset on the GPU against its FP64 oracle (oracle/orc_cfg.c):
SPC water, 12-bead flexible chains, graphite, periodic in x and y.

Bars: plain FP64 forces and energies within 1e-10 (relative) of the oracle,
per force term and in total; 100-step plain trajectories within 1e-8 sigma;
mixed-precision force RMS relative error within 1e-5 of the oracle on the
20,000-water / 200-chain shape (also with compensated FP32 sums);
replicas bit-identical alone and batched."""
import numpy as np
import pytest

import oracle as O
from surfactant_enhanced_spreading_gb300 import config_preset as C
from surfactant_enhanced_spreading_gb300 import engine as E

pytestmark = pytest.mark.gpu

TERMS = [("near", E.T_NEAR), ("far", E.T_FAR), ("bond", E.T_BOND), ("angle", E.T_VALENCE),
         ("dihedral", E.T_DIHEDRAL), ("pairs", E.T_INTERNAL), ("subtract", E.T_SUBTRACT), ("wall", E.T_WALL),
         ("graphite", E.T_GRAPHITE)]


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a - b)


@pytest.fixture(scope="module")
def c1():
    """The 1,000-water, 2-layer graphite shape of the small plain configuration (96 A box),
    with 20 chains so every chain term is exercised."""
    return C.config_droplet(1000, 20, cells=(8, 8, 8), seed=5, graphite_layers=2)


@pytest.fixture(scope="module")
def c1p(c1):
    """The same state with every site displaced by ~0.01 sigma, so bond
    lengths and angles leave their minima (a force-field check on generic
    geometry; not integrated)."""
    s = c1.copy()
    s.pos = s.pos + np.random.default_rng(9).normal(scale=0.01, size=s.pos.shape)
    return s


@pytest.fixture(scope="module")
def straddling(c1p):
    """The perturbed droplet moved by half a box in x and y: it straddles both periodic faces."""
    s = c1p.copy()
    s.pos[:, 0] += c1p.cells[0] * C.RS / 2.0
    s.pos[:, 1] += c1p.cells[1] * C.RS / 2.0
    return s


@pytest.mark.parametrize("which", ["c1p", "straddling"])
def test_plain_forces_per_term_match_oracle(which, request):
    s = request.getfixturevalue(which)
    eng = E.Engine(s, E.PLAIN_FP64)
    orc = O.Oracle(s)
    assert isinstance(orc, O.ConfigOracle)
    eng.force(True)
    orc.force(True)
    for name, t in TERMS:
        fg = eng.force(False, t)
        fo = orc.force(False, t)
        err = rel(fg, fo)
        assert err < 1e-10, (name, err)
    fg = eng.force(True)
    fo = orc.force(True)
    assert rel(fg, fo) < 1e-10
    assert eng.pair_counts() == orc.pair_counts()


def test_plain_energies_match_oracle(c1p):
    eng = E.Engine(c1p, E.PLAIN_FP64)
    orc = O.Oracle(c1p)
    eng.force(True)
    orc.force(True)
    eg, eo = eng.energies(), orc.energies()
    scale = np.abs(eo).sum()
    for k in range(8):
        assert abs(eg[k] - eo[k]) <= 1e-10 * max(abs(eo[k]), 1e-3 * scale), (k, eg[k], eo[k])
    es = eng.energies_static()
    assert np.allclose(es, eg, rtol=1e-12, atol=0)


def test_temperature_on_the_device_matches_oracle(c1):
    eng = E.Engine(c1, E.PLAIN_FP64)
    orc = O.Oracle(c1)
    assert abs(eng.temperature() - orc.temperature()) < 1e-12 * orc.temperature()
    assert abs(eng.temperature() - C.TR) < 1e-9


def test_plain_trajectory_100_steps(c1):
    """100 steps (10 list / far-field rebuilds) of the plain path against the
    oracle: positions within 1e-8 sigma, velocities within 1e-8 of their
    scale, the thermostat variable within 1e-9 relative."""
    eng = E.Engine(c1, E.PLAIN_FP64)
    orc = O.Oracle(c1)
    eng.force(True)
    orc.force(True)
    eng.init_accel()
    orc.init_accel()
    eng.run(1, 100)
    orc.run(1, 100)
    pg, vg, _ = eng.state()
    po, vo = orc.get(0), orc.get(1)
    assert np.abs(pg - po).max() < 1e-8
    assert np.abs(vg - vo).max() < 1e-8 * np.abs(vo).max()
    assert abs(eng.eta - orc.eta) <= 1e-9 * max(abs(orc.eta), 1e-12)
    assert eng.counters()[0] == orc.fail_count() == 0


def test_mixed_force_error_c2_shape():
    """20,000 waters + 200 chains on 4-layer graphite (240 x 240 x 144 A):
    the mixed path's force RMS relative error against the FP64 oracle."""
    s = C.config_droplet(**C.C2, seed=2024)
    orc = O.Oracle(s)
    fo = orc.force(True)
    for prec in (E.MIXED, E.MIXED_FP32C, E.MIXED_COMP):
        fm = E.Engine(s, prec).force(True)
        assert rel(fm, fo) < 1e-5, (prec, rel(fm, fo))
    fp = E.Engine(s, E.PLAIN_FP64).force(True)
    assert rel(fp, fo) < 1e-10


@pytest.mark.parametrize("prec", [E.MIXED, E.MIXED_COMP])
def test_replicas_bit_identical_alone_and_batched(prec):
    systems = [C.config_droplet(400, 4, cells=(8, 8, 8), seed=31), C.config_droplet(900, 10, cells=(12, 8, 8), seed=32)]
    batch = E.Engine(systems, prec)
    batch.force(True)
    batch.init_accel()
    batch.run(1, 25)
    pb, vb, _ = batch.state()
    for k, s in enumerate(systems):
        e = E.Engine(s, prec)
        e.force(True)
        e.init_accel()
        e.run(1, 25)
        p, v, _ = e.state()
        sl = slice(batch.offsets[k], batch.offsets[k + 1])
        assert np.array_equal(p, pb[sl]) and np.array_equal(v, vb[sl])


def test_periodic_shift_changes_nothing(c1):
    """The droplet moved by one box length in x: every force term the same."""
    s = c1.copy()
    s.pos[:, 0] += c1.cells[0] * C.RS
    f0 = E.Engine(c1, E.PLAIN_FP64).force(True)
    f1 = E.Engine(s, E.PLAIN_FP64).force(True)
    assert rel(f1, f0) < 1e-10   # the shifted coordinates round differently


def test_mixed_water_constraints_matrix_form(c1):
    """The mixed path's matrix SHAKE / RATTLE of the waters against the plain
    path's Gauss-Seidel sweeps from identical inputs: both stop inside the
    1e-8 tolerance of the same constrained state, so positions agree to
    well below 1e-7 sigma, and every water bond meets the tolerance."""
    plain = E.Engine(c1, E.PLAIN_FP64)
    mixed = E.Engine(c1, E.MIXED)
    f = plain.force(True)
    mixed.force(True)
    plain.init_accel()
    p0, v0, a0 = plain.state()
    mixed.set_state(p0, v0, a0, 0.0)
    for e in (plain, mixed):
        e.move_a()
    pp, vp, _ = plain.state()
    pm, vm, _ = mixed.state()
    assert np.abs(pm - pp).max() < 1e-7
    assert np.abs(vm - vp).max() < 1e-7
    w = pm[:3 * c1.n_water].reshape(-1, 3, 3) * 3.166
    hh = 2 * np.sin(np.radians(109.47 / 2))
    for (i, j), dd in (((0, 1), 1.0), ((1, 2), hh), ((2, 0), 1.0)):
        d2 = ((w[:, i] - w[:, j]) ** 2).sum(1)
        assert np.abs(d2 - dd * dd).max() <= 2.0001e-8 * dd * dd
    # RATTLE: the mixed path's velocities meet RATTLE's own test, |R.V / dt| /
    # ((1/m_i + 1/m_j) d^2) <= tol, for every water bond
    mixed.force(True)
    mixed.move_b()
    pm2, vm2, _ = mixed.state()
    m = np.array([1.0, 1.00794 / 15.9994, 1.00794 / 15.9994])
    r = pm2[:3 * c1.n_water].reshape(-1, 3, 3)
    v = vm2[:3 * c1.n_water].reshape(-1, 3, 3)
    for (i, j), dd in (((0, 1), 1.0), ((1, 2), hh), ((2, 0), 1.0)):
        g = np.einsum("ij,ij->i", r[:, i] - r[:, j], v[:, i] - v[:, j]) / 0.00127362 / ((1 / m[i] + 1 / m[j]) * dd * dd / 3.166 ** 2)
        assert np.abs(g).max() <= 1.0001e-8
    assert mixed.counters()[0] == 0

"""The oracle against hand-computable known answers (tests/golden) and the
reference's constants.  CPU only."""
import math
import os

import numpy as np
import pytest

import oracle as O
from surfactant_enhanced_spreading_gb300 import system as S

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _sys_from(pos, nw, ns, cells):
    return S.System(n_water=nw, n_surf=ns, cells=tuple(int(c) for c in cells), pos=np.array(pos, dtype=np.float64),
                    vel=np.zeros_like(pos), carbons=np.zeros((0, 3)), graphite_on=False)


def test_constants():
    c = O.constants()
    assert c["xpi"] == float(np.float32(675.05))          # single-precision literal, src/mybox.cmns:41
    assert abs(c["rc"] - 10.0 / 3.166) < 1e-15
    assert abs(c["rs"] - (10.0 / 3.166 + 2.0 / 3.166)) < 1e-15
    assert c["dt"] == 0.00127362


def test_pair_waters_golden():
    g = np.load(os.path.join(GOLD, "pair_waters.npz"))
    o = O.Oracle(_sys_from(g["pos"], 2, 0, g["cells"]))
    f = o.force(True, O.TERM_NEAR)
    np.testing.assert_allclose(f, g["force"], rtol=1e-12, atol=1e-9)


def test_pair_water_surf_golden():
    g = np.load(os.path.join(GOLD, "pair_water_surf.npz"))
    o = O.Oracle(_sys_from(g["pos"], 1, 1, g["cells"]))
    f = o.force(True, O.TERM_NEAR)
    np.testing.assert_allclose(f, g["force"], rtol=1e-11, atol=1e-8)


def test_wall_golden():
    g = np.load(os.path.join(GOLD, "wall.npz"))
    # place 7 waters' O at the fixture points (rigid geometry irrelevant for the wall)
    pos = []
    for p in g["pos"]:
        pos += [p, p + [0.3, 0.0, 0.0], p + [0.0, 0.3, 0.0]]
    o = O.Oracle(_sys_from(np.array(pos), len(g["pos"]), 0, (4, 4, 4)))
    f = o.force(True, O.TERM_WALL)
    np.testing.assert_allclose(f[0::3], g["force"], rtol=1e-13)


def test_generator_constraints_exact():
    s = S.droplet(40, 2, cells=(8, 8, 4), seed=3)
    pos = s.pos * S.SIGMA
    w = pos[:120].reshape(40, 3, 3)
    assert np.allclose(np.linalg.norm(w[:, 1] - w[:, 0], axis=1), 1.0, atol=1e-12)
    assert np.allclose(np.linalg.norm(w[:, 2] - w[:, 0], axis=1), 1.0, atol=1e-12)
    assert np.allclose(np.linalg.norm(w[:, 2] - w[:, 1], axis=1), S.WATER_HH, atol=1e-12)
    sp = pos[120:].reshape(2, 29, 3)
    for b, (i, j) in enumerate(S.SURF_BONDS):
        assert np.allclose(np.linalg.norm(sp[:, i - 1] - sp[:, j - 1], axis=1), S.SURF_BOND_LEN[b], atol=1e-12)


def test_pair_surf_surf_golden():
    """Two surfactants: Coulomb for every site pair, LJ within rc with
    Lorentz-Berthelot parameters (hand-computed with numpy)."""
    g = np.load(os.path.join(GOLD, "pair_surf_surf.npz"))
    o = O.Oracle(_sys_from(g["pos"], 0, 2, g["cells"]))
    f = o.force(True, O.TERM_NEAR)
    np.testing.assert_allclose(f, g["force"], rtol=1e-11, atol=1e-8 * np.abs(g["force"]).max())


def test_graphite_site_golden():
    """One water in the bottom layer of cells over a patch of carbons: the
    O-carbon LJ within rc; hydrogens feel none."""
    g = np.load(os.path.join(GOLD, "graphite_site.npz"))
    s = S.System(n_water=1, n_surf=0, cells=tuple(int(c) for c in g["cells"]), pos=g["pos"].copy(),
                 vel=np.zeros((3, 3)), carbons=g["carbons"].copy(), graphite_on=True)
    f = O.Oracle(s).force(True, O.TERM_GRAPHITE)
    np.testing.assert_allclose(f[0], g["force_o"], rtol=1e-12, atol=1e-12 * np.abs(g["force_o"]).max())
    assert np.all(f[1:] == 0.0)


def test_far_field_two_waters_golden():
    """Two waters three cells apart meet only through the far field; the
    order-4 expansion reproduces their exact Coulomb force to the
    truncation bound ((a + b) / R)^5 < 5e-6."""
    g = np.load(os.path.join(GOLD, "far_pair.npz"))
    o = O.Oracle(_sys_from(g["pos"], 2, 0, g["cells"]))
    assert np.abs(o.force(True, O.TERM_NEAR)).max() == 0.0
    f = o.force(True, O.TERM_FAR)
    assert np.linalg.norm(f - g["force"]) / np.linalg.norm(g["force"]) < 5e-6


def test_shake_water_golden():
    """SHAKE of one water from a perturbed predictor (configuration preset,
    tolerance 1e-8) lands on the exact solution of the constraint equations."""
    from surfactant_enhanced_spreading_gb300 import config_preset as C
    g = np.load(os.path.join(GOLD, "shake_water.npz"))
    s = S.System(n_water=1, n_surf=0, cells=(8, 8, 8), pos=g["old"].copy(), vel=g["predictor"] - g["old"],
                 carbons=np.zeros((0, 3)), graphite_on=False, preset=C.PRESET_CONFIG)
    o = O.Oracle(s)
    o.set(2, np.zeros((3, 3)))
    o.eta = 0.0
    o.move_a()
    assert np.abs(o.get(0) - g["solved"]).max() < 1e-8
    assert o.fail_count() == 0

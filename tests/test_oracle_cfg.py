"""The oracle of the configuration preset (oracle/orc_cfg.c) checked on the CPU:
forces against finite differences of its energies, the far field against a
direct sum over the periodic image supercell, Newton's third law, periodic
invariance, and the generator's geometry."""
import numpy as np
import pytest

import oracle as O
from surfactant_enhanced_spreading_gb300 import config_preset as C


@pytest.fixture(scope="module")
def small():
    return C.config_droplet(300, 6, cells=(8, 8, 8), seed=11)


def test_legendre_closed_form_matches_recurrence():
    """The oracle's associated Legendre function (explicit polynomial from
    Rodrigues' formula) against scipy's recurrence, with the reference's edge
    conventions."""
    from scipy.special import lpmv
    for l in range(9):
        for m in range(l + 1):
            for x in np.linspace(-1.0, 1.0, 33):
                ref = lpmv(m, l, x)
                assert abs(O.legendre(l, m, x) - ref) <= 1e-13 * max(1.0, abs(ref))
    assert O.legendre(-1, 0, 0.3) == 1.0
    assert O.legendre(2, 3, 0.3) == 0.0


def test_generator_geometry(small):
    p = small.pos * 3.166
    ch = p[3 * small.n_water:].reshape(-1, 12, 3)
    b = np.linalg.norm(np.diff(ch, axis=1), axis=2)
    assert np.allclose(b, C.BOND, atol=1e-9)
    u, v = ch[:, :-2] - ch[:, 1:-1], ch[:, 2:] - ch[:, 1:-1]
    ang = np.degrees(np.arccos(np.einsum("ijk,ijk->ij", u, v) / np.linalg.norm(u, axis=2) / np.linalg.norm(v, axis=2)))
    assert np.allclose(ang, C.ANGLE, atol=1e-7)
    w = p[:3 * small.n_water].reshape(-1, 3, 3)
    assert np.allclose(np.linalg.norm(w[:, 1] - w[:, 0], axis=1), 1.0, atol=1e-12)
    # rigid water velocities: no relative velocity along any bond
    vv = small.vel[:3 * small.n_water].reshape(-1, 3, 3)
    for i, j in ((0, 1), (1, 2), (2, 0)):
        assert np.abs(np.einsum("ij,ij->i", w[:, i] - w[:, j], vv[:, i] - vv[:, j])).max() < 1e-12
    m = small.masses()
    t = (m[:, None] * (small.vel / 0.00127362) ** 2).sum() / (3 * small.n_sites - 3 * small.n_water)
    assert abs(t - C.TR) < 1e-9
    # the sheet tiles the periodic box: every carbon has three neighbours at
    # 1.42 A up to the strain that fits whole cells into the box
    from scipy.spatial import cKDTree
    cb = small.carbons * 3.166
    top = cb[cb[:, 2] == cb[:, 2].max()]
    L = np.array(small.cells[:2]) * 12.0
    tree = cKDTree(np.mod(top[:, :2] + L / 2, L), boxsize=L)
    d, _ = tree.query(np.mod(top[:, :2] + L / 2, L), k=4)
    nx = round(L[0] / (3 * C.CC))
    assert np.allclose(d[:, 1:], C.CC, rtol=1.0 / (2 * nx) + 1e-9)


def _fd(o, pos, g, a, which, h=1e-6):
    e = []
    for sgn in (1, -1):
        p = pos.copy()
        p[g, a] += sgn * h
        o.set(0, p)
        e.append(o.energies()[which].sum())
    o.set(0, pos)
    return -(e[0] - e[1]) / (2 * h)


@pytest.mark.parametrize("terms,which", [
    (O.TERM_NEAR, [0, 1]),
    (O.TERM_BOND | O.TERM_VALENCE | O.TERM_DIHEDRAL, [4]),
    (O.TERM_INTERNAL, [3]),
    (O.TERM_WALL, [5]),
    (O.TERM_GRAPHITE, [6]),
])
def test_forces_are_energy_gradients(small, terms, which):
    o = O.ConfigOracle(small)
    o.force(True)
    pos = o.get(0)
    f = o.force(False, terms)
    rng = np.random.default_rng(5)
    nw3 = 3 * small.n_water
    sites = list(rng.choice(nw3, 4, replace=False)) + list(nw3 + rng.choice(small.n_sites - nw3, 6, replace=False))
    if terms == O.TERM_GRAPHITE:   # sites near the sheet
        low = np.argsort(pos[:nw3:3, 2])[:6] * 3
        sites = list(low)
    for g in sites:
        for a in range(3):
            fd = _fd(o, pos, g, a, which)
            assert abs(fd - f[g, a]) <= 2e-5 * max(1.0, abs(f[g, a])), (g, a, fd, f[g, a])


def test_dihedral_gradient_random_conformations():
    """Dihedral forces (torsion-angle gradient form) against finite
    differences on chains in random conformations, trans and gauche."""
    s = C.config_droplet(60, 8, cells=(8, 8, 8), seed=21)
    o = O.ConfigOracle(s)
    o.force(True)
    pos = o.get(0)
    f = o.force(False, O.TERM_DIHEDRAL)
    nw3 = 3 * s.n_water
    for g in range(nw3, s.n_sites, 5):
        for a in range(3):
            fd = _fd(o, pos, g, a, [4])
            assert abs(fd - f[g, a]) <= 2e-5 * max(1.0, abs(f[g, a]))


def test_near_field_newton_third_law(small):
    o = O.ConfigOracle(small)
    f = o.force(True, O.TERM_NEAR)
    assert np.abs(f.sum(axis=0)).max() < 1e-9 * np.abs(f).max() * small.n_sites


def test_far_field_against_direct_image_sum(small):
    """Far field plus its intramolecular correction against the direct
    Coulomb sum over the 3 x 3 image supercell outside the 27-cell block:
    order-4 accuracy, a few per cent of the far-field force (a missing or
    doubled image box would show as O(1))."""
    o = O.ConfigOracle(small)
    ff = o.force(True, O.TERM_FAR | O.TERM_SUBTRACT)
    d = o.direct_far()
    assert np.linalg.norm(ff - d) / np.linalg.norm(d) < 0.04
    fn = o.force(True, O.TERM_NEAR)
    tot = fn + d
    assert np.linalg.norm(fn + ff - tot) / np.linalg.norm(tot) < 0.01


def test_periodic_invariance(small):
    """Moving the whole system by one box length in x or y changes no force."""
    o = O.ConfigOracle(small)
    f0 = o.force(True)
    for a in (0, 1):
        s2 = small.copy()
        s2.pos[:, a] += small.cells[a] * C.RS
        f1 = O.ConfigOracle(s2).force(True)
        assert np.linalg.norm(f1 - f0) / np.linalg.norm(f0) < 1e-12
    # and a droplet split by the periodic boundary: forces move with it
    s3 = small.copy()
    s3.pos[:, 0] += small.cells[0] * C.RS / 2.0
    s4 = small.copy()
    s4.pos[:, 0] -= small.cells[0] * C.RS / 2.0
    f3, f4 = O.ConfigOracle(s3).force(True), O.ConfigOracle(s4).force(True)
    assert np.linalg.norm(f3 - f4) / np.linalg.norm(f3) < 1e-12


def test_integrator_constraints_and_thermostat(small):
    o = O.ConfigOracle(small)
    o.force(True)
    o.init_accel()
    o.run(1, 20)
    assert o.fail_count() == 0
    p = o.get(0) * 3.166
    w = p[:3 * small.n_water].reshape(-1, 3, 3)
    d = np.linalg.norm(w[:, 1] - w[:, 0], axis=1)
    assert np.abs(d - 1.0).max() < 1e-7           # SHAKE tolerance 1e-8 on d^2
    assert np.isfinite(o.eta)
    assert 0.5 * C.TR < o.temperature() < 4.0 * C.TR   # the lattice start heats before the thermostat catches up

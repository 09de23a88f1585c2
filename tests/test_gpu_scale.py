"""Parity at scale and on the hand-computed fixtures, through the C ABI.

* The reference force field's benchmark-sized system (20,000 waters + 200
  surfactants, 65,800 sites): the plain FP64 path within 1e-10 of the oracle
  per force term, the mixed path within 1e-5 (force RMS) of the oracle.
* The large configuration (312,000 sites, periodic): plain within 1e-10 and
  mixed within 1e-5 of the oracle.
* The known answers of tests/golden on the GPU: surfactant-surfactant pairs,
  graphite on a site, two waters joined only by the far field, and SHAKE of
  one water (plain sweeps and the mixed path's matrix form).
"""
import os

import numpy as np
import pytest

import oracle as O
from surfactant_enhanced_spreading_gb300 import config_preset as C
from surfactant_enhanced_spreading_gb300 import engine as E
from surfactant_enhanced_spreading_gb300 import system as S

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TERMS = [E.T_NEAR, E.T_FAR, E.T_VALENCE, E.T_DIHEDRAL, E.T_BERENDSEN, E.T_INTERNAL, E.T_SUBTRACT, E.T_WALL,
         E.T_GRAPHITE]


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_reference_bench_system_per_term():
    s = S.droplet(20000, 200, cells=(24, 24, 12), seed=2024, graphite_layers=4)
    orc = O.Oracle(s)
    plain = E.Engine(s, E.PLAIN_FP64)
    fo = orc.force(True)
    assert rel(plain.force(True), fo) < 1e-10
    for t in TERMS:
        fot = orc.force(False, t)
        if np.linalg.norm(fot) == 0.0:
            continue
        assert rel(plain.force(False, t), fot) < 1e-10, t
    assert rel(E.Engine(s, E.MIXED).force(True), fo) < 1e-5


def test_large_configuration_against_oracle():
    s = C.config_droplet(**C.C3, seed=2024)
    fo = O.Oracle(s).force(True)
    assert rel(E.Engine(s, E.PLAIN_FP64).force(True), fo) < 1e-10
    assert rel(E.Engine(s, E.MIXED).force(True), fo) < 1e-5


def _sys(pos, nw, ns, cells, carbons=None, preset=0):
    carb = np.zeros((0, 3)) if carbons is None else carbons
    return S.System(n_water=nw, n_surf=ns, cells=tuple(int(c) for c in cells), pos=np.array(pos, dtype=np.float64),
                    vel=np.zeros_like(pos), carbons=carb, graphite_on=carbons is not None, preset=preset)


def test_golden_pairs_graphite_far_on_gpu():
    g = np.load(os.path.join(GOLD, "pair_surf_surf.npz"))
    f = E.Engine(_sys(g["pos"], 0, 2, g["cells"]), E.PLAIN_FP64).force(True, E.T_NEAR)
    np.testing.assert_allclose(f, g["force"], rtol=1e-11, atol=1e-8 * np.abs(g["force"]).max())
    g = np.load(os.path.join(GOLD, "graphite_site.npz"))
    f = E.Engine(_sys(g["pos"], 1, 0, g["cells"], g["carbons"]), E.PLAIN_FP64).force(True, E.T_GRAPHITE)
    np.testing.assert_allclose(f[0], g["force_o"], rtol=1e-12, atol=1e-12 * np.abs(g["force_o"]).max())
    assert np.all(f[1:] == 0.0)
    g = np.load(os.path.join(GOLD, "far_pair.npz"))
    f = E.Engine(_sys(g["pos"], 2, 0, g["cells"]), E.PLAIN_FP64).force(True, E.T_FAR)
    assert rel(f, g["force"]) < 5e-6


@pytest.mark.parametrize("precision", [E.PLAIN_FP64, E.MIXED])
def test_golden_shake_water_on_gpu(precision):
    g = np.load(os.path.join(GOLD, "shake_water.npz"))
    s = _sys(g["old"], 1, 0, (8, 8, 8), preset=C.PRESET_CONFIG)
    s.vel = g["predictor"] - g["old"]
    eng = E.Engine(s, precision)
    eng.set_state(None, None, np.zeros((3, 3)), 0.0)
    eng.move_a()
    pos, _, _ = eng.state()
    assert np.abs(pos - g["solved"]).max() < 1e-8
    assert eng.counters()[0] == 0

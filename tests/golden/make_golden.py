"""Generate the known-answer fixtures in this folder.

The reference ships no tests, fixtures or golden vectors, and it cannot be
compiled in this image, so these fixtures are hand-computable cases written
from the reference's force laws with numpy alone (no oracle code):

* ``pair_waters.npz``: two SPC/E waters in one cell, the nine site-pair
  Coulomb terms qq xpi d / r^3 and the O-O LJ term
  48 r^-6 (r^-6 - 1/2) d / r^2 (src/evalw1w1.f90:65-239);
* ``pair_water_surf.npz``: one water and one 29-site surfactant 5 A apart,
  Coulomb for all site pairs and LJ between the water O and every surfactant
  site with Lorentz-Berthelot parameters (src/evalw1s.f90:34-60,
  src/init_arrays.f90:476-502);
* ``wall.npz``: the wall force 48/d^13 from six faces (src/eval_wall.f90:17-23).

Run: python tests/golden/make_golden.py
"""
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SIGMA = 3.166
EPS = 650.2
XPI = float(np.float32(675.05))
RC = 10.0 / SIGMA
RS = 12.0 / SIGMA
QW = np.array([-0.8476, 0.4238, 0.4238])
QS = np.array([0.435, -0.700, 0.265, 0.29, -0.58, 0.29, 0.29, -0.58, 0.29, 0.29, -0.58, 0.29, 0.29, -0.58, 0.29,
               0.0, 0.0, 0.3, 0.0, -0.3, 0.15, 0.0, 0.0, 0.0, -0.3, 0.15, 0.0, 0.0, 0.0])
SGS = np.array([2.6, 3.07, 3.983, 3.983, 3.047, 3.983, 3.983, 3.047, 3.983, 3.983, 3.047, 3.983, 3.983, 3.047, 3.983,
                3.95, 3.95, 3.385, 3.786, 2.955, 3.385, 3.786, 3.786, 3.786, 2.955, 3.385, 3.786, 3.786, 3.786]) / SIGMA
EPSS = np.array([33.5, 711.76, 478.12, 478.12, 817.67, 478.12, 478.12, 817.67, 478.12, 478.12, 817.67, 478.12, 478.12,
                 817.67, 478.12, 382.47, 382.47, 2448.0, 753.2, 849.3, 2448.0, 753.2, 753.2, 753.2, 849.3, 2448.0, 753.2,
                 753.2, 753.2]) / EPS


def water(o, rng):
    half = math.radians(109.47) / 2
    t = np.array([[0, 0, 0], [math.sin(half), 0, math.cos(half)], [-math.sin(half), 0, math.cos(half)]])
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    return (t @ q.T + o) / SIGMA


def pair_force(xi, xj, qq, eps=None, sg6=None):
    d = xi - xj
    r2 = d @ d
    r = math.sqrt(r2)
    ft = qq / r ** 3
    if eps is not None and r <= RC:
        r6 = 1.0 / r2 ** 3
        ft += 48.0 * eps * sg6 * r6 * (sg6 * r6 - 0.5) / r2
    return d * ft


def main():
    rng = np.random.default_rng(7)
    # two waters near the centre of cell (0,0,0) of a 4^3-cell box
    c = -1.5 * RS * SIGMA
    w1 = water(np.array([c - 1.2, c - 0.5, c]), rng)
    w2 = water(np.array([c + 1.6, c + 0.7, c + 0.4]), rng)
    pos = np.concatenate([w1, w2])
    f = np.zeros_like(pos)
    for a in range(3):
        for b in range(3):
            qq = QW[a] * QW[b] * XPI
            lj = (a == 0 and b == 0)
            fij = pair_force(pos[a], pos[3 + b], qq, 1.0 if lj else None, 1.0)
            f[a] += fij
            f[3 + b] -= fij
    np.savez(os.path.join(HERE, "pair_waters.npz"), pos=pos, force=f, cells=np.array([4, 4, 4]))

    # one water and one surfactant (rigid template built along +x)
    ws = water(np.array([c, c, c]), rng)
    s = []
    p = np.array([c + 5.0, c - 3.0, c - 2.0])
    for k in range(29):
        s.append(p + np.array([0.0, 0.21 * k, 0.05 * (k % 3)]))
    s = np.array(s) / SIGMA
    pos = np.concatenate([ws, s])
    f = np.zeros_like(pos)
    for a in range(3):
        for k in range(29):
            qq = QW[a] * QS[k] * XPI
            if a == 0:
                eps = math.sqrt(1.0 * EPSS[k])
                sg6 = ((1.0 + SGS[k]) / 2.0) ** 6
                fij = pair_force(pos[a], pos[3 + k], qq, eps, sg6)
            else:
                fij = pair_force(pos[a], pos[3 + k], qq)
            f[a] += fij
            f[3 + k] -= fij
    np.savez(os.path.join(HERE, "pair_water_surf.npz"), pos=pos, force=f, cells=np.array([4, 4, 4]))

    # wall
    pts = rng.uniform(-0.45, 0.45, size=(7, 3)) * 4 * RS
    hb = 2 * RS
    fw = 48.0 / (pts - hb) ** 13 + 48.0 / (hb + pts) ** 13
    np.savez(os.path.join(HERE, "wall.npz"), pos=pts, force=fw, half_box=hb)


if __name__ == "__main__":
    main()

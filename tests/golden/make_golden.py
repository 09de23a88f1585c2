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
* ``wall.npz``: the wall force 48/d^13 from six faces (src/eval_wall.f90:17-23);
* ``pair_surf_surf.npz``: two 29-site surfactants 6 A apart, Coulomb for all
  site pairs and LJ within rc with Lorentz-Berthelot parameters
  (src/evalSS.f90:36-120, src/init_arrays.f90:476-502);
* ``graphite_site.npz``: one water on a patch of carbons in the bottom layer
  of cells, the O-carbon LJ 48 eps sg6 r^-6 (sg6 r^-6 - 1/2) d / r^2 within
  rc with sigma 3.19 A, epsilon 392 J/mol (src/eval_graphite.f90:10-11,
  104-126);
* ``far_pair.npz``: two waters three cells apart (only the far field joins
  them), with the exact Coulomb force between them; an order-4 expansion
  about cell centres 0.48 sigma or less from every site (R = 3 cells =
  11.4 sigma) must reproduce it to ((a + b) / R)^5 < 5e-6;
* ``shake_water.npz``: one SPC water, an old geometry and a predictor 0.02
  sigma off it, and the exact solution of the SHAKE equations (corrections
  along the old bond vectors, every constraint length met) by Newton's
  method to round-off (src/move_w1_a.f90:64-122).

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

    rng2 = np.random.default_rng(11)
    # two surfactants (rigid synthetic templates) 6 A apart in x
    sa = np.array([np.array([c - 3.0, c - 3.0, c]) + np.array([0.0, 0.21 * k, 0.05 * (k % 3)]) for k in range(29)])
    sb = sa + np.array([6.0, 0.3, -0.2])
    pos = np.concatenate([sa, sb]) / SIGMA
    f = np.zeros_like(pos)
    for a in range(29):
        for b in range(29):
            qq = QS[a] * QS[b] * XPI
            eps = math.sqrt(EPSS[a] * EPSS[b])
            sg6 = ((SGS[a] + SGS[b]) / 2.0) ** 6
            fij = pair_force(pos[a], pos[29 + b], qq, eps, sg6)
            f[a] += fij
            f[29 + b] -= fij
    np.savez(os.path.join(HERE, "pair_surf_surf.npz"), pos=pos, force=f, cells=np.array([4, 4, 4]))

    # one water above a patch of carbons in the bottom cell layer of a 4^3 box
    half = 2 * RS * SIGMA
    zc = -half + 4.0                                  # carbon plane 4 A above the lower wall
    cx, cy = -half + 1.5 * RS * SIGMA, -half + 1.5 * RS * SIGMA   # centre of column (1, 1)
    carb = []
    for i in range(-4, 5):
        for j in range(-4, 5):
            carb.append([cx + 1.42 * i + 0.3 * (j % 2), cy + 1.23 * j, zc])
    carb = np.array(carb)
    wg = water(np.array([cx + 0.4, cy - 0.3, zc + 3.1]), rng2)
    sg = (1.0 + 3.19 / SIGMA) / 2.0
    sgc6 = (3.19 / SIGMA) ** 6
    epc = 392.0 / EPS
    fo = np.zeros(3)
    for cpos in carb / SIGMA:
        d = wg[0] - cpos
        r2 = d @ d
        if r2 <= RC * RC:
            r6 = 1.0 / r2 ** 3
            fo += 48.0 * epc * sgc6 * r6 * (sgc6 * r6 - 0.5) / r2 * d
    np.savez(os.path.join(HERE, "graphite_site.npz"), pos=wg, carbons=carb / SIGMA, force_o=fo, cells=np.array([4, 4, 4]))

    # two waters three cells apart along x: exact Coulomb between them
    q = []
    for k, off in enumerate((0.0, 3.0)):
        centre = np.array([-half + (0.5 + off) * RS * SIGMA, -half + 1.5 * RS * SIGMA, -half + 1.5 * RS * SIGMA])
        q.append(water(centre + rng2.uniform(-0.3, 0.3, 3), rng2))
    pos = np.concatenate(q)
    f = np.zeros_like(pos)
    for a in range(3):
        for b in range(3):
            fij = pair_force(pos[a], pos[3 + b], QW[a] * QW[b] * XPI)
            f[a] += fij
            f[3 + b] -= fij
    np.savez(os.path.join(HERE, "far_pair.npz"), pos=pos, force=f, cells=np.array([4, 4, 4]))

    # SHAKE of one SPC water: exact solution of the constraint equations
    r0 = water(np.array([0.2, -0.1, 0.3]), rng2)
    p0 = r0 + rng2.normal(scale=0.02, size=(3, 3))
    m = np.array([15.9994, 1.00794, 1.00794]) / 15.9994
    hh = 2.0 * math.sin(math.radians(109.47) / 2.0)
    dsq = np.array([1.0, hh * hh, 1.0]) / SIGMA ** 2
    bonds = [(0, 1), (1, 2), (2, 0)]
    R = np.array([r0[i] - r0[j] for i, j in bonds])
    g = np.zeros(3)

    def moved(g):
        p = p0.copy()
        for b, (i, j) in enumerate(bonds):
            p[i] += g[b] * R[b] / m[i]
            p[j] -= g[b] * R[b] / m[j]
        return p

    for _ in range(60):
        p = moved(g)
        res = np.array([dsq[b] - (p[i] - p[j]) @ (p[i] - p[j]) for b, (i, j) in enumerate(bonds)])
        J = np.zeros((3, 3))
        for b, (i, j) in enumerate(bonds):
            for cb, (ci, cj) in enumerate(bonds):
                dp = (((i == ci) - (i == cj)) / m[i] - ((j == ci) - (j == cj)) / m[j]) * R[cb]
                J[b, cb] = -2.0 * (p[i] - p[j]) @ dp
        g = g - np.linalg.solve(J, res)
    np.savez(os.path.join(HERE, "shake_water.npz"), old=r0, predictor=p0, solved=moved(g))


if __name__ == "__main__":
    main()

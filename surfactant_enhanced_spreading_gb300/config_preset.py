"""Seeded synthetic systems of the configuration preset.

The benchmark configurations describe a different force field from the
reference's (which is SPC/E water with 29-site trisiloxane surfactants with
rigid bonds in a closed box): SPC water, 12-bead united-atom surfactant
chains with harmonic bonds, angles and dihedrals, graphite with
Lorentz-Berthelot carbon parameters, and a box periodic in x and y.  The
engine runs it as ``PRESET_CONFIG`` (``sesp_params.preset``).  Its
parameters, in the units the configurations quote:

* water: rigid, O-H 1.0 A, H-O-H 109.47 deg, charges O -0.82 / H +0.41, LJ on
  O only (sigma 3.166 A, epsilon 0.65 kJ/mol);
* chains: beads 1-4 form the head (charges +0.40, -0.60, +0.60, -0.40; LJ
  sigma / epsilon 3.75 A / 0.815, 2.80 / 0.457, 3.95 / 0.382, 2.80 / 0.457
  kJ/mol; masses 15.035, 15.999, 14.027, 15.999), beads 5-12 the CH2 tail
  (uncharged, sigma 3.9 A, epsilon 0.38 kJ/mol, mass 14.027); bonds harmonic
  at 1.53 A with k = 2000 kJ/mol/A^2 (U = k/2 (r - r0)^2), angles 112 deg
  with k = 519.7 kJ/mol/rad^2, triple-cosine (OPLS-style) dihedrals
  a (1 + cos phi) + b (1 - cos 2 phi) + c (1 + cos 3 phi) with a = 2.9517,
  b = -0.5669, c = 6.5790 kJ/mol (trans at 180 deg); LJ + Coulomb without
  cutoff between beads four or more bonds apart, none between closer ones;
* graphite: AB-stacked layers 3.35 A apart, C-C 1.42 A (the lattice is
  stretched or compressed along x and y so that a whole number of cells
  tiles the periodic box: by at most 1 / (2 n) for n cells, 2.2 % in a
  96 A box, 0.4 % in a 480 A box), carbon sigma 3.4 A, epsilon
  0.23 kJ/mol, acting on every LJ site of the bottom cell layers within
  rc = 10 A;
* Coulomb of other molecules uncut over the 27 cells (12 A) around a site,
  LJ truncated at 10 A, order-4 multipole far field over the 3 x 3
  supercell of periodic images, walls at the two z faces;
* SHAKE / RATTLE tolerance 1e-8, Nose-Hoover relaxation time 0.1 ps
  (50 steps of 2 fs), target 300 K.

Positions are in sigma = 3.166 A; velocities are displacements per step.
Sites are stored waters first (O, H, H), then chains (bead 1 .. 12).
"""
from __future__ import annotations

import math

import numpy as np

from .system import DT, RS, SIGMA, System, _rand_rots, water_template

PRESET_REFERENCE = 0
PRESET_CONFIG = 1
N_BEAD = 12
EPSILON = 650.2                      # J/mol, the reduced energy unit
R_GAS = 8.314462618                  # J/mol/K
T_KELVIN = 300.0
TR = R_GAS * T_KELVIN / EPSILON      # 300 K in reduced units
TAU_STEPS = 0.1e-12 / 2.0e-15        # Nose-Hoover relaxation time: 0.1 ps of 2 fs steps
SHAKE_TOL = 1e-8
BOND = 1.53                          # A
ANGLE = 112.0                        # deg
CC = 1.42                            # A, graphite C-C
LAYER = 3.35                         # A, graphite interlayer spacing
_O, _H = 15.9994, 1.00794
HEAD_MASS = [15.035, 15.9994, 14.027, 15.9994]
CHAIN_MASS = np.array(HEAD_MASS + [14.027] * 8) / _O
WATER_MASS = np.array([_O, _H, _H]) / _O
JITTER = 0.05    # lattice jitter, a fraction of the 3.10 A spacing
CLOSE = 1.8      # A: no two sites of different molecules closer in a generated state


def graphite_periodic(layers: int, half_x: float, half_y: float, z_top: float) -> np.ndarray:
    """AB-stacked graphite tiling the periodic box [-half_x, half_x) x
    [-half_y, half_y) (Angstrom in and out): the rectangular 4-atom cell of
    graphene (3 cc by sqrt(3) cc) repeated nx by ny times, stretched to the
    box; layer k at z_top - 3.35 k, odd layers shifted by one bond along x."""
    lx, ly = 2.0 * half_x, 2.0 * half_y
    nx = max(1, int(round(lx / (3.0 * CC))))
    ny = max(1, int(round(ly / (math.sqrt(3.0) * CC))))
    ax, ay = lx / nx, ly / ny           # strained cell edges
    cx, cy = ax / 3.0, ay / math.sqrt(3.0)
    basis = np.array([[0.0, 0.0], [cx, 0.0], [1.5 * cx, 0.5 * math.sqrt(3.0) * cy],
                      [2.5 * cx, 0.5 * math.sqrt(3.0) * cy]])
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    origin = np.stack([i.ravel() * ax, j.ravel() * ay], axis=1)
    sheet = (origin[:, None, :] + basis[None, :, :]).reshape(-1, 2)
    out = []
    for layer in range(layers):
        p = sheet + (np.array([cx, 0.0]) if layer % 2 else 0.0)
        p = np.mod(p, [lx, ly]) - [half_x, half_y]
        out.append(np.column_stack([p, np.full(len(p), z_top - LAYER * layer)]))
    return np.concatenate(out).astype(np.float64)


def chain_conformation(rng, tries: int = 200) -> np.ndarray:
    """12 beads in Angstrom from bead 1 at the origin along +z on average:
    bonds 1.53 A, angles 112 deg, dihedrals trans (60 %) or gauche +-65 deg
    with +-15 deg of jitter, beads four or more bonds apart kept 3.2 A
    apart."""
    th = math.radians(ANGLE)
    for _ in range(tries):
        b1 = np.array([0.0, 0.0, 1.0])
        d = rng.normal(size=3)
        d -= d.dot(b1) * b1
        d /= np.linalg.norm(d)
        p = [np.zeros(3), BOND * b1]
        # third bead: angle 112 deg at bead 2
        p.append(p[1] + BOND * (math.cos(math.pi - th) * b1 + math.sin(math.pi - th) * d))
        ok = True
        for k in range(3, N_BEAD):
            r = rng.uniform()
            phi = math.pi if r < 0.6 else (math.radians(65.0) if r < 0.8 else -math.radians(65.0))
            phi += math.radians(rng.uniform(-15.0, 15.0))
            a, b, c = p[k - 3], p[k - 2], p[k - 1]
            bc = (c - b) / np.linalg.norm(c - b)
            n = np.cross(b - a, bc)
            n /= np.linalg.norm(n)
            m = np.cross(n, bc)
            # new bond in the local frame: angle th at c, dihedral phi (trans at 180 deg)
            dvec = np.array([-math.cos(th), math.sin(th) * math.cos(phi), math.sin(th) * math.sin(phi)])
            new = c + BOND * (dvec[0] * bc + dvec[1] * m + dvec[2] * n)
            if any(np.linalg.norm(new - p[j]) < 3.2 for j in range(k - 3)):
                ok = False
                break
            p.append(new)
        if ok:
            return np.array(p)
    raise RuntimeError("could not build a clash-free chain")


def _rigid_project(vel, pos, mass):
    """Velocities of each water replaced by the rigid-body motion (centre-of-
    mass velocity plus rotation) that fits them in the mass-weighted least-
    squares sense, so they satisfy the three bond constraints."""
    m = mass[None, :, None]
    mt = mass.sum()
    vcm = (m * vel).sum(axis=1) / mt
    rcm = (m * pos).sum(axis=1) / mt
    r = pos - rcm[:, None, :]
    L = (m * np.cross(r, vel - vcm[:, None, :])).sum(axis=1)
    eye = np.eye(3)[None]
    inertia = (m[..., None] * ((r * r).sum(-1)[..., None, None] * eye - r[..., :, None] * r[..., None, :])).sum(axis=1)
    w = np.linalg.solve(inertia, L[..., None])[..., 0]
    return vcm[:, None, :] + np.cross(w[:, None, :], r)


def config_droplet(n_water: int, n_chain: int = 0, cells=(8, 8, 8), seed: int = 0, graphite_layers: int = 2,
                   temperature: float = TR) -> System:
    """Hemispherical droplet of ``n_water`` SPC waters with ``n_chain``
    12-bead chains at its surface, on ``graphite_layers`` layers of graphite
    covering the floor of a box of ``cells`` 12 A cells, periodic in x and
    y (cells in x and y at least 8, all multiples of 4).  Waters sit on a
    seed-jittered cubic lattice at 0.0334 per cubic A (1.0 g/cm^3; jitter
    +-5 % of the spacing) with random orientations, re-drawn until no two
    sites of different molecules are within 1.8 A; chains start with bead 1 just outside the water
    surface and extend outwards in random trans / gauche conformations;
    Maxwell velocities at ``temperature`` (300 K), waters moving rigidly,
    scaled to that temperature exactly."""
    rng = np.random.default_rng(seed)
    cells = tuple(int(c) for c in cells)
    if cells[0] < 8 or cells[1] < 8 or any(c % 4 for c in cells):
        raise ValueError("the periodic preset needs cells that are multiples of 4, at least 8 in x and y")
    half = np.array(cells, dtype=np.float64) * RS * SIGMA / 2.0          # Angstrom
    z_top = -half[2] + 2.0 + LAYER * max(graphite_layers - 1, 0)
    z_base = z_top + 3.2
    density = 0.0334
    radius = (3.0 * n_water / (2.0 * math.pi * density)) ** (1.0 / 3.0)
    a = density ** (-1.0 / 3.0)
    nlat = int(radius / a) + 3
    g = np.arange(-nlat, nlat + 1, dtype=np.float64)
    gx, gy, gz = np.meshgrid(g, g, np.arange(0, nlat + 1, dtype=np.float64), indexing="ij")
    pts = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1) * a
    pts = pts + rng.uniform(-JITTER, JITTER, size=pts.shape) * a
    pts[:, 2] = np.abs(pts[:, 2])
    pts = pts[np.linalg.norm(pts, axis=1) <= radius * 1.15]
    pts = pts[np.argsort(np.linalg.norm(pts, axis=1), kind="stable")]
    from scipy.spatial import cKDTree
    chains = []
    if n_chain:
        library = [chain_conformation(rng) for _ in range(min(n_chain, 64))]
        zax = np.array([0.0, 0.0, 1.0])
        cell = 3.5
        grid = {}   # spatial hash of placed beads (3.5 A cells) for the clash test

        def clashes(cand):
            for p in cand:
                k = np.floor(p / cell).astype(int)
                for dx in (-1, 0, 1):
                    for dy in (-1, 0, 1):
                        for dz in (-1, 0, 1):
                            for q in grid.get((k[0] + dx, k[1] + dy, k[2] + dz), ()):
                                if (p[0] - q[0]) ** 2 + (p[1] - q[1]) ** 2 + (p[2] - q[2]) ** 2 < cell * cell:
                                    return True
            return False

        for k in range(n_chain):
            for t in range(600):
                conf = library[int(rng.integers(len(library)))]
                u = rng.normal(size=3)
                u[2] = abs(u[2]) + 0.1
                u /= np.linalg.norm(u)
                shell = radius + 2.5 + rng.uniform(0.0, 2.0 + 0.002 * k + 0.02 * max(0, t - 100))
                # rotate the chain's +z axis onto u, then spin it about u
                v = np.cross(zax, u)
                s_, c_ = np.linalg.norm(v), zax.dot(u)
                if s_ < 1e-12:
                    rot = np.eye(3)
                else:
                    vx = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
                    rot = np.eye(3) + vx + vx @ vx * ((1 - c_) / s_ ** 2)
                spin = rng.uniform(0, 2 * math.pi)
                K = np.array([[0, -u[2], u[1]], [u[2], 0, -u[0]], [-u[1], u[0], 0]])
                rspin = np.eye(3) + math.sin(spin) * K + (1 - math.cos(spin)) * (K @ K)
                cand = conf @ (rspin @ rot).T + u * shell
                if cand[:, 2].min() < 2.5:
                    continue
                if np.min(np.linalg.norm(cand, axis=1)) < radius + 1.5:
                    continue
                if clashes(cand):
                    continue
                chains.append(cand)
                for p in cand:
                    kk = np.floor(p / cell).astype(int)
                    grid.setdefault((kk[0], kk[1], kk[2]), []).append(p)
                break
            else:
                raise RuntimeError("could not place chain %d" % k)
    if chains:
        dmin, _ = cKDTree(np.concatenate(chains)).query(pts, k=1)
        pts = pts[dmin > 3.0]
    if len(pts) < n_water:
        raise RuntimeError("lattice too small for the droplet")
    pts = pts[:n_water]
    wt = water_template()
    wat = np.einsum("ij,mkj->mik", wt, _rand_rots(rng, n_water)) + pts[:, None, :]
    chain_flat = np.concatenate(chains) if chains else np.zeros((0, 3))
    # re-draw the orientation of waters with a site closer than CLOSE to a
    # site of another molecule.  A water's sites stay within 1 A of its
    # (fixed) oxygen, so only waters whose oxygens are within CLOSE + 2 A can
    # clash: those pairs are found once and re-checked every pass.
    wp = cKDTree(pts).query_pairs(CLOSE + 2.0 + 1e-6, output_type="ndarray")
    ctree = cKDTree(chain_flat) if len(chain_flat) else None
    near_chain = np.zeros(n_water, dtype=bool)
    if ctree is not None:
        d, _ = ctree.query(pts, k=1)
        near_chain = d < CLOSE + 1.0 + 1e-6
    for _pass in range(400):
        a, b = wp[:, 0], wp[:, 1]
        d2 = ((wat[a][:, :, None, :] - wat[b][:, None, :, :]) ** 2).sum(-1).reshape(len(a), -1).min(axis=1)
        bad_pairs = wp[d2 < CLOSE * CLOSE]
        # one water of each clashing pair (the later one on even passes, the earlier on odd ones)
        bad = bad_pairs[:, 0] if _pass % 2 else bad_pairs[:, 1]
        if near_chain.any():
            idx = np.nonzero(near_chain)[0]
            dc, _ = ctree.query(wat[idx].reshape(-1, 3), k=1)
            bad = np.concatenate([bad, idx[(dc.reshape(-1, 3) < CLOSE).any(axis=1)]])
        bad = np.unique(bad)
        if not len(bad):
            break
        wat[bad] = np.einsum("ij,mkj->mik", wt, _rand_rots(rng, len(bad))) + pts[bad][:, None, :]
    else:
        raise RuntimeError("could not orient the waters without close contacts")
    pos = np.concatenate([wat.reshape(-1, 3), chain_flat])
    pos[:, 2] += z_base
    if np.any(np.abs(pos[:, :2]) > half[:2] - 1.0) or np.any(pos[:, 2] > half[2] - 2.0):
        raise RuntimeError("droplet does not fit the box; use more cells")
    carb = graphite_periodic(graphite_layers, half[0], half[1], z_top) if graphite_layers else np.zeros((0, 3))
    masses = np.concatenate([np.tile(WATER_MASS, n_water), np.tile(CHAIN_MASS, n_chain)])
    v = rng.normal(size=(masses.size, 3)) * np.sqrt(temperature / masses)[:, None]
    if n_water:
        v[:3 * n_water] = _rigid_project(v[:3 * n_water].reshape(n_water, 3, 3), wat, WATER_MASS).reshape(-1, 3)
    dof = 3 * masses.size - 3 * n_water
    t_now = float((masses[:, None] * v * v).sum()) / dof
    v *= math.sqrt(temperature / t_now)
    return System(n_water=n_water, n_surf=n_chain, cells=cells, pos=pos / SIGMA, vel=v * DT, carbons=carb / SIGMA,
                  graphite_on=bool(graphite_layers), preset=PRESET_CONFIG)


# the benchmark configurations' shapes in this preset (boxes rounded to
# whole 12 A cells, multiples of 4 per axis).  The large one gets 192 A in z
# instead of 150 A: its hemisphere of 100,000 waters at 1 g/cm^3 has a radius
# of 112.6 A, which with the chains on its surface and the 4-layer sheet
# under it does not fit 150 A.
C1 = dict(n_water=1000, n_chain=0, cells=(8, 8, 8), graphite_layers=2)        # 96 x 96 x 96 A
C2 = dict(n_water=20000, n_chain=200, cells=(20, 20, 12), graphite_layers=4)  # 240 x 240 x 144 A
C3 = dict(n_water=100000, n_chain=1000, cells=(40, 40, 16), graphite_layers=4)  # 480 x 480 x 192 A


def sheet_cells(n_water: int) -> int:
    """Cells per side of the periodic box whose graphite sheet spans 2.5 x
    the droplet diameter (rounded up to a multiple of 4, at least 8)."""
    radius = (3.0 * n_water / (2.0 * math.pi * 0.0334)) ** (1.0 / 3.0)
    n = int(math.ceil(2.5 * 2.0 * radius / (RS * SIGMA)))
    n = max(8, n + (-n) % 4)
    return n


def box_height_cells(n_water: int, n_chain: int) -> int:
    """Cells in z that hold the droplet and its chains above the sheet."""
    radius = (3.0 * n_water / (2.0 * math.pi * 0.0334)) ** (1.0 / 3.0)
    need = radius + (25.0 if n_chain else 8.0) + 2.0 + 4 * LAYER + 3.2
    n = int(math.ceil(need / (RS * SIGMA)))
    return max(4, n + (-n) % 4)

"""Seeded synthetic systems in the reference's reduced units.

The reference reads its initial state from ``data_cont2.dat`` (alternating
position / velocity lines, waters O,H,H first, then 29-site surfactants,
src/read_config.f90:16-38) and its carbons from ``graphite.dat``
(src/read_graphite.f90:19-33), neither of which ships with it.  This module
builds such states from a seed:

* a hemispherical droplet of rigid 3-site waters (O-H 1 A, H-O-H 109.47 deg,
  the constraint lengths of src/init_arrays.f90:566-574) on a seed-jittered
  cubic lattice at 0.0334 molecules per cubic Angstrom, random orientations
  (re-drawn until no site is within 1.5 A of another molecule's);
* 29-site trisiloxane surfactants built on the bond graph of
  src/init_arrays.f90:229-264 with the exact constraint lengths of
  src/init_arrays.f90:509-565, placed at the droplet surface;
* an AB-stacked graphite sheet (C-C 1.421 A, 3.41 A layer spacing, the
  lattice of src/make_graphite.f90:18-80) of any number of layers;
* Maxwell velocities at the reference's target temperature tr = 3.81087
  (src/mybox.f90:48), stored as displacements per step.

Positions are in sigma = 3.166 A, the box is centred on the origin and spans
``n_cells * rs`` per axis with ``rs = 12 A`` (src/mybox.cmns:38-40,
src/init_box_dimensions.f90:14-20).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

SIGMA = 3.166
EPSILON = 650.2
RC = 10.0 / SIGMA
RS = 10.0 / SIGMA + 2.0 / SIGMA
DT = 0.00127362
TR = 3.81087
N_SURF_SITE = 29

# bond graph of the 29-site surfactant (1-based), src/init_arrays.f90:229-264
SURF_BONDS = [(i, i + 1) for i in range(1, 19)] + [
    (18, 20), (20, 21), (21, 22), (21, 23), (21, 24), (18, 25), (25, 26), (26, 27), (26, 28), (26, 29)]
# constraint lengths in Angstrom by bond index, src/init_arrays.f90:509-565
SURF_BOND_LEN = [0.945, 1.430, 1.516, 1.410, 1.410, 1.516, 1.410, 1.410, 1.516, 1.410, 1.410, 1.516,
                 1.410, 1.410, 1.516, 1.540, 1.88, 1.88, 1.60, 1.60, 1.88, 1.88, 1.88, 1.60, 1.60,
                 1.88, 1.88, 1.88]
# masses relative to oxygen, src/init_arrays.f90:266-312
_HY, _C, _O, _SI = 1.00794, 12.011, 15.9994, 28.0855
_ME, _METHYL = _C + 2 * _HY, _C + 3 * _HY
SURF_MASS = np.array([_HY, _O, _ME, _ME, _O, _ME, _ME, _O, _ME, _ME, _O, _ME, _ME, _O, _ME, _ME, _ME,
                      _SI, _METHYL, _O, _SI, _METHYL, _METHYL, _METHYL, _O, _SI, _METHYL, _METHYL,
                      _METHYL]) / _O
WATER_MASS = np.array([_O, _HY, _HY]) / _O
WATER_HH = 2.0 * math.sin(109.47 * math.pi / 180.0 / 2.0)   # Angstrom
CLOSE = 1.5   # Angstrom: no two sites of different molecules closer in a generated state


@dataclasses.dataclass
class System:
    """A state in reference order: ``pos``/``vel`` are (n_sites, 3) float64."""

    n_water: int
    n_surf: int
    cells: tuple          # (ncx, ncy, ncz) L4 cells, multiples of 4
    pos: np.ndarray
    vel: np.ndarray
    carbons: np.ndarray   # (n_c, 3) float64
    graphite_on: bool = True
    preset: int = 0       # 0: the reference's force field; 1: the configuration preset (config_preset.py)

    @property
    def sites_per_surf(self) -> int:
        return N_SURF_SITE if self.preset == 0 else 12

    @property
    def n_sites(self) -> int:
        return 3 * self.n_water + self.sites_per_surf * self.n_surf

    @property
    def half_box(self) -> np.ndarray:
        return np.array(self.cells, dtype=np.float64) * RS / 2.0

    def masses(self) -> np.ndarray:
        if self.preset:
            from .config_preset import CHAIN_MASS
            return np.concatenate([np.tile(WATER_MASS, self.n_water), np.tile(CHAIN_MASS, self.n_surf)])
        return np.concatenate([np.tile(WATER_MASS, self.n_water), np.tile(SURF_MASS, self.n_surf)])

    def copy(self) -> "System":
        return dataclasses.replace(self, pos=self.pos.copy(), vel=self.vel.copy(), carbons=self.carbons.copy())


def _rand_rot(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def _rand_rots(rng, n):
    """n uniformly random rotation matrices (unit quaternions)."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    a, b, c, d = q.T
    return np.stack([np.stack([a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)], -1),
                     np.stack([2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)], -1),
                     np.stack([2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d], -1)], 1)


def water_template() -> np.ndarray:
    """O, H, H in Angstrom with O at the origin."""
    half = 109.47 * math.pi / 180.0 / 2.0
    return np.array([[0.0, 0.0, 0.0], [math.sin(half), 0.0, math.cos(half)],
                     [-math.sin(half), 0.0, math.cos(half)]])


def surfactant_template(rng, tries: int = 200) -> np.ndarray:
    """29 sites in Angstrom satisfying every constraint length exactly.

    Sites are placed along the bond tree from site 1 with near-tetrahedral
    bond angles (105-118 degrees to the parent bond); the children of one
    site are spread evenly in azimuth around the parent bond (random offset,
    +-15 degrees of jitter), so branch sites stay near-tetrahedral too.
    Placements closer than 2.6 A to a site three or more bonds away are
    rejected.
    """
    adj = {i: [] for i in range(1, 30)}
    blen = {}
    for b, (i, j) in enumerate(SURF_BONDS):
        adj[i].append(j)
        adj[j].append(i)
        blen[(i, j)] = blen[(j, i)] = SURF_BOND_LEN[b]
    # bond-graph distances for the clash test
    dist = np.full((30, 30), 99, dtype=int)
    for s in range(1, 30):
        dist[s, s] = 0
        frontier = [s]
        while frontier:
            nxt = []
            for u in frontier:
                for v in adj[u]:
                    if dist[s, v] > dist[s, u] + 1:
                        dist[s, v] = dist[s, u] + 1
                        nxt.append(v)
            frontier = nxt
    jit = math.radians(15.0)
    for _ in range(tries):
        pos = {1: np.zeros(3)}
        parent = {1: None}
        order = [1]
        ok = True
        k = 0
        while k < len(order) and ok:
            u = order[k]
            k += 1
            kids = [v for v in adj[u] if v not in pos]
            p = parent[u]
            if p is not None:
                b1 = pos[u] - pos[p]
                b1 /= np.linalg.norm(b1)
                e1 = np.cross(b1, rng.normal(size=3))
                e1 /= np.linalg.norm(e1)
                e2 = np.cross(b1, e1)
            for attempt in range(60):
                phi0 = rng.uniform(0.0, 2.0 * math.pi)
                cands = []
                for kc, v in enumerate(kids):
                    if p is None:
                        d = rng.normal(size=3)
                    else:
                        ang = math.radians(rng.uniform(105.0, 118.0))
                        phi = phi0 + 2.0 * math.pi * kc / len(kids) + rng.uniform(-jit, jit)
                        perp = math.cos(phi) * e1 + math.sin(phi) * e2
                        d = math.cos(math.pi - ang) * b1 + math.sin(math.pi - ang) * perp
                    d /= np.linalg.norm(d)
                    cands.append(pos[u] + blen[(u, v)] * d)
                clash = False
                for v, cand in zip(kids, cands):
                    if any(dist[v, w] >= 3 and np.linalg.norm(cand - pw) < 2.6 for w, pw in pos.items()):
                        clash = True
                        break
                if not clash:
                    break
            else:
                ok = False
                break
            for v, cand in zip(kids, cands):
                pos[v] = cand
                parent[v] = u
                order.append(v)
        if ok and len(pos) == 29:
            return np.array([pos[i] for i in range(1, 30)])
    raise RuntimeError("could not build a clash-free surfactant")


def graphite(layers: int, half_x: float, half_y: float, z_top: float) -> np.ndarray:
    """AB-stacked graphite (Angstrom in, Angstrom out) covering |x|<half_x, |y|<half_y."""
    cc = 1.421
    a1 = np.array([1.5 * cc, math.sqrt(3) / 2 * cc])
    a2 = np.array([1.5 * cc, -math.sqrt(3) / 2 * cc])
    n = int(2 * max(half_x, half_y) / cc) + 4
    i, j = np.meshgrid(np.arange(-n, n + 1), np.arange(-n, n + 1), indexing="ij")
    base = i.ravel()[:, None] * a1 + j.ravel()[:, None] * a2
    out = []
    for layer in range(layers):
        shift = np.array([cc, 0.0]) if layer % 2 else np.zeros(2)
        z = z_top - 3.41 * layer
        for b in (np.zeros(2), np.array([cc, 0.0])):
            p = base + b + shift
            keep = (np.abs(p[:, 0]) < half_x) & (np.abs(p[:, 1]) < half_y)
            out.append(np.column_stack([p[keep], np.full(keep.sum(), z)]))
    return np.concatenate(out).astype(np.float64)


def maxwell(masses: np.ndarray, rng, temperature: float = TR) -> np.ndarray:
    """Velocities as displacements per step at a reduced temperature."""
    v = rng.normal(size=(masses.size, 3)) * np.sqrt(temperature / masses)[:, None]
    return v * DT


def droplet(n_water: int, n_surf: int = 0, cells=(8, 8, 8), seed: int = 0, graphite_layers: int = 2,
            graphite_extent: float | None = None, temperature: float = TR) -> System:
    """Hemispherical droplet on graphite in a closed box of ``cells`` L4 cells.

    The top carbon layer sits 4 A above the lower wall, inside the bottom
    layer of cells, so the graphite term (bottom cells only,
    src/eval_graphite.f90:13-15) acts on the first water layer.  The sheet
    covers the whole floor unless ``graphite_extent`` (half-width, A) limits
    it: a molecule that leaves a smaller sheet sinks beside its edge, under
    the top carbon plane, and meets the carbons side-on.
    """
    rng = np.random.default_rng(seed)
    cells = tuple(int(c) for c in cells)
    half = np.array(cells, dtype=np.float64) * RS * SIGMA / 2.0          # Angstrom
    z_graph = -half[2] + 4.0
    z_base = z_graph + 3.2
    density = 0.0334
    radius = (3.0 * n_water / (2.0 * math.pi * density)) ** (1.0 / 3.0)
    a = density ** (-1.0 / 3.0)
    nlat = int(radius / a) + 3
    g = np.arange(-nlat, nlat + 1, dtype=np.float64)
    gx, gy, gz = np.meshgrid(g, g, np.arange(0, nlat + 1, dtype=np.float64), indexing="ij")
    pts = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1) * a
    pts = pts + rng.uniform(-0.15, 0.15, size=pts.shape) * a
    pts[:, 2] = np.abs(pts[:, 2])
    pts = pts[np.linalg.norm(pts, axis=1) <= radius * 1.15]
    pts = pts[np.argsort(np.linalg.norm(pts, axis=1), kind="stable")]
    surf_sites = []
    if n_surf:
        # a library of clash-free conformations, each placed with its own rotation
        library = [surfactant_template(rng) for _ in range(min(n_surf, 16))]
        library = [t - t.mean(axis=0) for t in library]
        centres = []
        for k in range(n_surf):
            tmpl = library[k % len(library)]
            for _t in range(400):
                rot = _rand_rot(rng)
                u = rng.normal(size=3)
                u[2] = abs(u[2]) + 0.15
                u /= np.linalg.norm(u)
                # a shell around the droplet surface, thicker as it fills
                # ... widened further after repeated clashes (crowded small droplets)
                widen = 0.1 * max(0, _t - 100)
                centre = u * (radius + 3.0 + rng.uniform(0.0, 4.0 + 0.05 * len(surf_sites) + widen))
                cand = tmpl @ rot.T + centre
                if cand[:, 2].min() < 2.0:
                    cand[:, 2] += 2.0 - cand[:, 2].min()
                cc = cand.mean(axis=0)
                clash = False
                if centres:
                    near = np.nonzero(np.linalg.norm(np.array(centres) - cc, axis=1) < 32.0)[0]
                    for q in near:
                        if np.min(np.linalg.norm(cand[:, None, :] - surf_sites[q][None, :, :], axis=2)) < 3.5:
                            clash = True
                            break
                if clash:
                    continue
                surf_sites.append(cand)
                centres.append(cc)
                break
            else:
                raise RuntimeError("could not place surfactant")
    # waters: keep lattice points clear of surfactant sites
    if surf_sites:
        from scipy.spatial import cKDTree
        dmin, _ = cKDTree(np.concatenate(surf_sites)).query(pts, k=1)
        pts = pts[dmin > 3.0]
    if len(pts) < n_water:
        raise RuntimeError("lattice too small for the droplet")
    pts = pts[:n_water]
    wt = water_template()
    rots = _rand_rots(rng, n_water)
    wat = np.einsum("ij,mkj->mik", wt, rots) + pts[:, None, :]
    # re-draw the orientation of waters with a site closer than CLOSE to a
    # site of another molecule (jittered lattice points can be ~2.2 A apart)
    from scipy.spatial import cKDTree
    surf_flat = np.concatenate(surf_sites) if surf_sites else np.zeros((0, 3))
    for _pass in range(200):
        flat = np.concatenate([wat.reshape(-1, 3), surf_flat])
        pairs = cKDTree(flat).query_pairs(CLOSE, output_type="ndarray")
        mol = np.concatenate([np.arange(3 * n_water) // 3, n_water + np.arange(len(surf_flat)) // N_SURF_SITE])
        if len(pairs):
            pairs = pairs[mol[pairs[:, 0]] != mol[pairs[:, 1]]]
        if not len(pairs):
            break
        # one water of each pair (the later one on even passes, the earlier on
        # odd ones, the water of a water-surfactant pair)
        first = pairs[:, 0] if _pass % 2 else pairs[:, 1]
        other = pairs[:, 1] if _pass % 2 else pairs[:, 0]
        bad = np.unique(np.where(mol[first] < n_water, first, other) // 3)
        wat[bad] = np.einsum("ij,mkj->mik", wt, _rand_rots(rng, len(bad))) + pts[bad][:, None, :]
    else:
        raise RuntimeError("could not orient the waters without close contacts")
    pos = [wat.reshape(-1, 3)]
    if surf_sites:
        pos.append(np.concatenate(surf_sites))
    pos = np.concatenate(pos)
    pos[:, 2] += z_base
    if np.any(np.abs(pos[:, :2]) > half[:2] - 1.0) or np.any(pos[:, 2] > half[2] - 1.0):
        raise RuntimeError("droplet does not fit the box; use more cells")
    ex = min(graphite_extent, half[0]) if graphite_extent is not None else half[0]
    ey = min(graphite_extent, half[1]) if graphite_extent is not None else half[1]
    carb = graphite(graphite_layers, ex, ey, z_graph) if graphite_layers else np.zeros((0, 3))
    masses = np.concatenate([np.tile(WATER_MASS, n_water), np.tile(SURF_MASS, n_surf)])
    vel = maxwell(masses, rng, temperature)
    return System(n_water=n_water, n_surf=n_surf, cells=cells, pos=pos / SIGMA, vel=vel,
                  carbons=carb / SIGMA, graphite_on=bool(graphite_layers))


def reference_box_system(seed: int = 0) -> System:
    """The reference's production size: 9,997 waters and 475 surfactants in the
    12 x 12 x 12-cell walled cube (src/mybox.cmns:55-60)."""
    return droplet(9997, 475, cells=(12, 12, 12), seed=seed)

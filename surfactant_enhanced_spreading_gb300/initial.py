"""Initial conditions the reference makes for itself: its start-up
velocities and its graphite sheet.

* ``lcg`` / ``lcg_draws``: the linear congruential generator of
  src/random.f90:1-9 (x -> ((3612 int(566927 x) + 5701) mod 566927 + 0.5) /
  566927), started from 0.378389247 (src/init_temp.f90:21-22).
* ``reference_velocities``: init_temp (src/init_temp.f90), which the
  reference calls after reading its restart file and which replaces the
  velocities read there (src/mybox.f90:57-60).  Every rank restarts the
  generator and walks its 64 cells; each site gets the unit vector of three
  draws mapped to [-1, 1); the mean velocity of each of five groups (O, H,
  CH2, Si, CH3) is removed per rank; one global factor then brings the
  temperature sum m v^2 / dt^2 / (3 N - constraints) to tr.
* ``graphite_sheet``: make_graphite (src/make_graphite.f90:18-101), the
  two-layer AB sheet of 22,956 carbons the reference reads from
  ``graphite.dat``; ``write_graphite_dat`` / ``read_graphite_dat`` and
  ``write_graphite_pdb`` are its two output files.

Sums follow the reference's loop order (sequential, cell by cell), so a start
made here is the one the reference would make from the same positions, up to
the order in which MPI adds the 27 ranks' kinetic sums.
"""
from __future__ import annotations

import math

import numpy as np

from .io import _fortran_a, _fortran_f, _fortran_i
from .system import DT, N_SURF_SITE, RS, SIGMA, SURF_MASS, TR, WATER_MASS

LCG_A, LCG_C, LCG_M = 3612, 5701, 566927
SEED = 0.378389247

# velocity groups of init_temp (src/init_temp.f90:124-448)
G_O, G_H, G_CH2, G_SI, G_CH3 = range(5)
WATER_GROUPS = (G_O, G_H, G_H)
SURF_GROUPS = (G_H, G_O, G_CH2, G_CH2, G_O, G_CH2, G_CH2, G_O, G_CH2, G_CH2, G_O, G_CH2, G_CH2, G_O, G_CH2,
               G_CH2, G_CH2, G_SI, G_CH3, G_O, G_SI, G_CH3, G_CH3, G_CH3, G_O, G_SI, G_CH3, G_CH3, G_CH3)
# the one mass the temperature sum takes per group (emw(1), emw(2), ems(3),
# ems(18), ems(19); src/init_temp.f90:782)
GROUP_MASS = (WATER_MASS[0], WATER_MASS[1], SURF_MASS[2], SURF_MASS[17], SURF_MASS[18])


def lcg(x: float) -> float:
    """One draw of src/random.f90:1-9."""
    ix = int(x * float(LCG_M))
    return (float((LCG_A * ix + LCG_C) % LCG_M) + 0.5) / float(LCG_M)


def lcg_draws(n: int, x0: float = SEED) -> np.ndarray:
    """n successive draws from x0.  After the first draw x = (i + 0.5) / m and
    int(x m) = i exactly, so the stream is the integer recurrence
    i -> (3612 i + 5701) mod 566927 (tests check this over the whole range)."""
    n = int(n)
    out = np.empty(n, dtype=np.float64)
    if n == 0:
        return out
    i = (LCG_A * int(x0 * float(LCG_M)) + LCG_C) % LCG_M
    ints = np.empty(n, dtype=np.int64)
    for k in range(n):
        ints[k] = i
        i = (LCG_A * i + LCG_C) % LCG_M
    return (ints.astype(np.float64) + 0.5) / float(LCG_M)


def site_groups(n_water: int, n_surf: int) -> np.ndarray:
    return np.concatenate([np.tile(np.array(WATER_GROUPS, dtype=np.int8), n_water),
                           np.tile(np.array(SURF_GROUPS, dtype=np.int8), n_surf)])


# ---------------------------------------------------------------- cell lists of read_config

def _rank_axis(v, nr, rhs, rsd):
    """ibox2 - 1 along one axis (src/ibox.f90:127-139), clamped to the box."""
    k = ((v + rhs) * nr / rsd).astype(np.int64)
    return np.clip(k, 0, nr - 1)


def _local_axis(v, rk, nr, rhs, rsd):
    """ibox64 - 1 along one axis relative to the rank centre of
    src/init_box_dimensions.f90:40-42 (src/ibox.f90:172-186)."""
    b = float(nr)
    c2 = rsd * (rk + 1) / b - rhs - rsd / b / 2.0
    return np.clip(((v - c2 + 2.0 * RS) / RS).astype(np.int64), 0, 3)


def rank_cell_lists(pos: np.ndarray, n_water: int, n_surf: int, cells) -> list:
    """The lists read_config builds (src/read_config.f90:44-175), in rank order
    (x fastest): per rank 64 cells (x fastest), each a triple of molecule
    lists (w1 waters, w2 waters, surfactants) in file order.  A water is w1
    when its three sites share the rank and the cell of its O; a molecule's
    cell is that of its O (water) or of site 14 (surfactant)."""
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    nc = np.array(cells, dtype=np.int64)
    if np.any(nc % 4):
        raise ValueError("cell counts must be multiples of 4")
    nr = nc // 4
    rsd = nc * RS
    rhs = rsd / 2.0
    key_site = np.concatenate([3 * np.arange(n_water), 3 * n_water + N_SURF_SITE * np.arange(n_surf) + 13])

    def locate(p):
        rk = np.stack([_rank_axis(p[:, a], nr[a], rhs[a], rsd[a]) for a in range(3)], axis=1)
        lc = np.stack([_local_axis(p[:, a], rk[:, a], nr[a], rhs[a], rsd[a]) for a in range(3)], axis=1)
        return rk, lc

    rk, lc = locate(pos[key_site])
    rank = rk[:, 0] + nr[0] * (rk[:, 1] + nr[1] * rk[:, 2])
    cell = lc[:, 0] + 4 * lc[:, 1] + 16 * lc[:, 2]
    w1 = np.zeros(n_water + n_surf, dtype=bool)
    if n_water:
        w1[:n_water] = True
        for t in (1, 2):
            rt, lt = locate(pos[3 * np.arange(n_water) + t])
            w1[:n_water] &= np.all(rt == rk[:n_water], axis=1) & np.all(lt == lc[:n_water], axis=1)
    nrank = int(np.prod(nr))
    lists = [[([], [], []) for _ in range(64)] for _ in range(nrank)]
    for m in range(n_water + n_surf):
        kind = 2 if m >= n_water else (0 if w1[m] else 1)
        lists[rank[m]][cell[m]][kind].append(m)
    return lists


# ---------------------------------------------------------------- init_temp

def _sum_seq(a: np.ndarray) -> np.ndarray:
    """Sequential sum along axis 0 (the reference's loop order)."""
    if a.shape[0] == 0:
        return np.zeros(a.shape[1:])
    return np.add.accumulate(a, axis=0)[-1]


def reference_velocities(pos: np.ndarray, n_water: int, n_surf: int, cells, temperature: float = TR) -> np.ndarray:
    """Start-up velocities of src/init_temp.f90 for these positions (sigma),
    as displacements per step, in the reference's site order.

    Per rank (src/init_temp.f90:21-122): the generator restarts at SEED;
    cell by cell, the w1 waters', w2 waters' and surfactants' sites draw
    three numbers each, mapped to 2 (x - 0.5) and scaled to unit length.
    Per rank, per group (src/init_temp.f90:124-780): the group's
    mean is removed (sum times 1 / count), then sum v^2 taken.  The ranks'
    m v^2 sums are added and every velocity is scaled by
    sqrt(tr / T) with T = sum / dt^2 / (3 N - (3 n_water + 28 n_surf))
    (src/init_temp.f90:782-823)."""
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    n = 3 * n_water + N_SURF_SITE * n_surf
    if pos.shape[0] != n:
        raise ValueError(f"{pos.shape[0]} positions for {n} sites")
    groups = site_groups(n_water, n_surf)
    vel = np.zeros((n, 3))
    v2_ranks = []
    for rank in rank_cell_lists(pos, n_water, n_surf, cells):
        # draw order: cells, then w1 / w2 / surfactant sites molecule by molecule
        draw = []
        # accumulation order of the group sums: cells, then per list each site
        # index across the list's molecules (the reference's strided loops)
        acc = []
        for w1, w2, sf in rank:
            for mols, first, ns in ((w1, 0, 3), (w2, 0, 3), (sf, 3 * n_water, N_SURF_SITE)):
                base = [first + ns * (m - (n_water if ns == N_SURF_SITE else 0)) for m in mols]
                draw.extend(b + t for b in base for t in range(ns))
                acc.extend(b + t for t in range(ns) for b in base)
        if not draw:
            v2_ranks.append(np.zeros(5))
            continue
        draw = np.array(draw, dtype=np.int64)
        acc = np.array(acc, dtype=np.int64)
        u = lcg_draws(3 * draw.size).reshape(-1, 3)
        d = 2.0 * (u - 0.5)
        inv = 1.0 / np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
        vel[draw] = d * inv[:, None]
        g_acc = groups[acc]
        for g in range(5):
            sel = acc[g_acc == g]
            if sel.size:
                vel[sel] -= _sum_seq(vel[sel]) * (1.0 / sel.size)
        # sum = sum + vx**2 + vy**2 + vz**2 adds the three squares one by one
        sq = vel[acc] ** 2
        v2_ranks.append(np.array([_sum_seq(sq[g_acc == g].ravel()) for g in range(5)]))
    v2sum = [GROUP_MASS[0] * s[0] + GROUP_MASS[1] * s[1] + GROUP_MASS[2] * s[2] + GROUP_MASS[3] * s[3]
             + GROUP_MASS[4] * s[4] for s in v2_ranks]
    v2total = 0.0
    for s in v2sum:
        v2total += s
    dof = 3 * n - (3 * n_water + 28 * n_surf)
    temp = v2total / (DT * DT) / dof
    return math.sqrt(temperature / temp) * vel


def temperature(vel: np.ndarray, n_water: int, n_surf: int) -> float:
    """sum m v^2 / dt^2 / (3 N - constraints) (src/compute_temperature.f90:240-242)."""
    vel = np.asarray(vel, dtype=np.float64).reshape(-1, 3)
    m = np.concatenate([np.tile(WATER_MASS, n_water), np.tile(SURF_MASS, n_surf)])
    n = vel.shape[0]
    return float((m * (vel * vel).sum(axis=1)).sum() / (DT * DT) / (3 * n - (3 * n_water + 28 * n_surf)))


# ---------------------------------------------------------------- make_graphite

GRAPHITE_IX = 81
GRAPHITE_Z = -16.0          # zcarbon, sigma


def graphite_sheet(ix: int = GRAPHITE_IX, z: float = GRAPHITE_Z) -> np.ndarray:
    """Carbons (sigma) of src/make_graphite.f90:18-101 in its order: the upper
    layer row by row (two atoms per lattice point), two edge rows, then the
    lower layer shifted by one bond in x and 3.41 A down; centred in x and y.
    ix = 81 gives iy = 70 rows and 22,956 carbons."""
    pi = 4.0 * math.atan(1.0)
    ccbond = 1.421 / SIGMA
    xshift = math.cos(60.0 * pi / 180.0) * ccbond
    yshift = math.sin(60.0 * pi / 180.0) * ccbond
    iy = int(math.sin(60.0 * pi / 180.0) * ix)
    ins = 2 * ix * iy + 2 * (iy - 1)
    x = np.empty(2 * ins)
    y = np.empty(2 * ins)
    zz = np.empty(2 * ins)
    k = 0
    for i in range(1, ix + 1):
        yup = yshift if i % 2 == 0 else 0.0
        for j in range(1, iy + 1):
            x[k] = i * (ccbond + xshift)
            y[k] = j * 2.0 * yshift + yup
            x[k + 1] = x[k] + ccbond
            y[k + 1] = y[k]
            k += 2
    for j in range(1, iy):
        x[k] = ccbond
        y[k] = j * 2.0 * yshift + yshift
        k += 1
    for j in range(1, iy):
        x[k] = (ix + 1) * (ccbond + xshift)
        y[k] = (j + 1) * 2.0 * yshift - yshift
        k += 1
    zz[:ins] = z
    x[ins:] = x[:ins] + ccbond
    y[ins:] = y[:ins]
    zz[ins:] = zz[:ins] - 3.41 / SIGMA
    xc = (x.max() + x.min()) / 2.0
    yc = (y.max() + y.min()) / 2.0
    return np.column_stack([x - xc, y - yc, zz])


def write_graphite_dat(path: str, carbons: np.ndarray) -> None:
    """graphite.dat, `(f10.4,f11.4,f11.4)` in sigma (src/make_graphite.f90:125-129)."""
    with open(path, "w") as f:
        for x, y, z in np.asarray(carbons, dtype=np.float64).reshape(-1, 3):
            f.write(_fortran_f(x, 10, 4) + _fortran_f(y, 11, 4) + _fortran_f(z, 11, 4) + "\n")


def read_graphite_dat(path: str, n: int | None = 22956) -> np.ndarray:
    """The first n carbons of a graphite.dat (all with n=None), as
    src/read_graphite.f90:19-22 reads them."""
    with open(path) as f:
        lines = [ln for ln in f.read().splitlines() if ln.strip()]
    if n is not None:
        if len(lines) < n:
            raise ValueError(f"{path}: {len(lines)} carbons, {n} needed")
        lines = lines[:n]
    return np.array([(float(s[0:10]), float(s[10:21]), float(s[21:32])) for s in lines], dtype=np.float64)


def write_graphite_pdb(path: str, carbons: np.ndarray) -> None:
    """graphite.pdb: HETATM records in Angstrom (src/make_graphite.f90:131-135)."""
    with open(path, "w") as f:
        for j, (x, y, z) in enumerate(np.asarray(carbons, dtype=np.float64).reshape(-1, 3) * SIGMA, start=1):
            f.write("HETATM" + _fortran_i(j, 5) + _fortran_a("C", 5) + _fortran_a("GPH", 4) + _fortran_i(j, 6)
                    + _fortran_f(x, 12, 3) + _fortran_f(y, 8, 3) + _fortran_f(z, 8, 3) + "\n")

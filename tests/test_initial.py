"""Initial-condition generators (the reference's LCG, init_temp and
make_graphite restated host side) and the warning rules of the consistency
checks.  CPU only."""
import math

import numpy as np
import pytest

from surfactant_enhanced_spreading_gb300 import initial as I
from surfactant_enhanced_spreading_gb300 import system as S


def test_lcg_stream_is_the_integer_recurrence():
    m = I.LCG_M
    i = np.arange(m, dtype=np.int64)
    x = (i.astype(np.float64) + 0.5) / float(m)
    assert np.array_equal((x * float(m)).astype(np.int64), i)
    x0 = I.SEED
    lit = []
    for _ in range(5000):
        x0 = I.lcg(x0)
        lit.append(x0)
    assert np.array_equal(I.lcg_draws(5000), np.array(lit))
    d = I.lcg_draws(200000)
    assert d.min() > 0.0 and d.max() < 1.0


def test_lcg_first_draws():
    # by hand: 0.378389247 * 566927 = 214519.07...
    assert int(I.SEED * I.LCG_M) == 214519
    i1 = (3612 * 214519 + 5701) % 566927
    assert I.lcg(I.SEED) == (i1 + 0.5) / 566927.0
    i2 = (3612 * i1 + 5701) % 566927
    assert I.lcg_draws(2)[1] == (i2 + 0.5) / 566927.0


def test_graphite_sheet_geometry():
    g = I.graphite_sheet()
    assert g.shape == (22956, 3)
    ins = 22956 // 2
    cc = 1.421 / S.SIGMA
    top, bot = g[:ins], g[ins:]
    assert np.all(top[:, 2] == -16.0)
    assert np.all(bot[:, 2] == -16.0 - 3.41 / S.SIGMA)
    assert np.allclose(bot[:, 0] - top[:, 0], cc, atol=1e-13)
    assert np.array_equal(bot[:, 1], top[:, 1])
    assert abs(g[:, 0].max() + g[:, 0].min()) < 1e-12
    assert abs(g[:, 1].max() + g[:, 1].min()) < 1e-12
    from scipy.spatial import cKDTree
    d, _ = cKDTree(top[:, :2]).query(top[:, :2], k=2)
    nn = d[:, 1]
    assert np.allclose(nn, cc, rtol=1e-12), (nn.min(), nn.max(), cc)


def test_graphite_files_round_trip(tmp_path):
    g = I.graphite_sheet()
    p = tmp_path / "graphite.dat"
    I.write_graphite_dat(str(p), g)
    lines = p.read_text().splitlines()
    assert len(lines) == 22956 and all(len(ln) == 32 for ln in lines[:50])
    back = I.read_graphite_dat(str(p))
    assert np.abs(back - g).max() <= 0.5e-4 + 1e-12
    with pytest.raises(ValueError):
        I.read_graphite_dat(str(p), n=22957)
    q = tmp_path / "graphite.pdb"
    I.write_graphite_pdb(str(q), g[:20])
    recs = q.read_text().splitlines()
    assert len(recs) == 20 and recs[0].startswith("HETATM    1    C GPH     1")
    assert abs(float(recs[3][26:38]) - g[3, 0] * S.SIGMA) <= 0.5e-3 + 1e-9


def _literal_init_temp(pos, n_water, n_surf, cells, temperature):
    """src/init_temp.f90 transcribed loop by loop, over the lists of
    rank_cell_lists (small systems only)."""
    lists = I.rank_cell_lists(pos, n_water, n_surf, cells)
    vel = np.zeros((3 * n_water + 29 * n_surf, 3))
    groups = I.site_groups(n_water, n_surf)
    v2sum_ranks = []

    def sites(kind, mols):
        if kind < 2:
            return [3 * m + t for m in mols for t in range(3)]
        return [3 * n_water + 29 * (m - n_water) + t for m in mols for t in range(29)]

    for rank in lists:
        x = I.SEED
        for cell in rank:
            for kind in range(3):
                for g in sites(kind, cell[kind]):
                    x = I.lcg(x); xx = 2.0 * (x - 0.5)
                    x = I.lcg(x); yy = 2.0 * (x - 0.5)
                    x = I.lcg(x); zz = 2.0 * (x - 0.5)
                    xyz = 1.0 / math.sqrt(xx * xx + yy * yy + zz * zz)
                    vel[g] = (xx * xyz, yy * xyz, zz * xyz)
        sums = np.zeros((5, 3))
        cnt = np.zeros(5, dtype=np.int64)

        def strided(cell):
            for kind in range(3):
                mols = cell[kind]
                ns = 3 if kind < 2 else 29
                for t in range(ns):
                    for m in mols:
                        yield (3 * m + t) if kind < 2 else (3 * n_water + 29 * (m - n_water) + t)

        for cell in rank:
            for g in strided(cell):
                k = groups[g]
                for a in range(3):
                    sums[k, a] = sums[k, a] + vel[g, a]
                cnt[k] += 1
        sv = np.zeros(5)
        for cell in rank:
            for g in strided(cell):
                k = groups[g]
                rn = 1.0 / cnt[k]
                for a in range(3):
                    vel[g, a] = vel[g, a] - sums[k, a] * rn
                sv[k] = sv[k] + vel[g, 0] ** 2 + vel[g, 1] ** 2 + vel[g, 2] ** 2
        m = I.GROUP_MASS
        v2sum_ranks.append(m[0] * sv[0] + m[1] * sv[1] + m[2] * sv[2] + m[3] * sv[3] + m[4] * sv[4])
    v2total = 0.0
    for s in v2sum_ranks:
        v2total += s
    n = vel.shape[0]
    temp = v2total / (S.DT * S.DT) / (3 * n - (3 * n_water + 28 * n_surf))
    return math.sqrt(temperature / temp) * vel


def test_reference_velocities_match_the_literal_loops():
    s = S.droplet(150, 3, cells=(8, 8, 8), seed=4)
    v = I.reference_velocities(s.pos, s.n_water, s.n_surf, s.cells)
    ref = _literal_init_temp(s.pos, s.n_water, s.n_surf, s.cells, S.TR)
    assert np.array_equal(v, ref)


def test_reference_velocities_properties():
    s = S.droplet(1200, 12, cells=(8, 8, 8), seed=9)
    v = I.reference_velocities(s.pos, s.n_water, s.n_surf, s.cells)
    assert abs(I.temperature(v, s.n_water, s.n_surf) / S.TR - 1.0) < 1e-12
    assert np.array_equal(v, I.reference_velocities(s.pos, s.n_water, s.n_surf, s.cells))
    groups = I.site_groups(s.n_water, s.n_surf)
    lists = I.rank_cell_lists(s.pos, s.n_water, s.n_surf, s.cells)
    for rank in lists:
        sites = []
        for w1, w2, sf in rank:
            sites += [3 * m + t for m in w1 + w2 for t in range(3)]
            sites += [3 * s.n_water + 29 * (m - s.n_water) + t for m in sf for t in range(29)]
        sites = np.array(sites, dtype=np.int64)
        for g in range(5):
            sel = sites[groups[sites] == g]
            if sel.size:
                assert np.abs(v[sel].sum(axis=0)).max() < 1e-12 * sel.size
    # every molecule sits in exactly one list
    seen = sorted(m for rank in lists for cell in rank for lst in cell for m in lst)
    assert seen == list(range(s.n_water + s.n_surf))
    # unit vectors before the mean removal and the common scale: speeds stay close
    speed = np.linalg.norm(v, axis=1)
    assert speed.std() / speed.mean() < 0.2


def test_rank_lists_split_waters():
    s = S.droplet(800, 0, cells=(8, 8, 8), seed=3, graphite_layers=0)
    lists = I.rank_cell_lists(s.pos, s.n_water, 0, s.cells)
    assert len(lists) == 8
    n_w1 = sum(len(c[0]) for r in lists for c in r)
    n_w2 = sum(len(c[1]) for r in lists for c in r)
    assert n_w1 + n_w2 == 800 and n_w2 > 0 and n_w1 > n_w2
    with pytest.raises(ValueError):
        I.rank_cell_lists(s.pos, s.n_water, 0, (6, 8, 8))

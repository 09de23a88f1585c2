"""The oracle's literal restatement of the reference's 39 list-based pair
kernels (src/eval[wS]*.f90 over the lists of src/build*.f90) equals the
located-cell rule the GPU kernel implements: every site gets the Coulomb force
of all sites of other molecules located in the 27 cells around its own cell,
plus truncated LJ by site kind.  CPU only."""
import numpy as np
import pytest

import oracle as O
from surfactant_enhanced_spreading_gb300 import system as S


@pytest.mark.parametrize("nw,ns,cells,seed", [(300, 0, (4, 4, 4), 0), (300, 4, (8, 8, 4), 1), (700, 10, (8, 8, 4), 2)])
def test_literal_lists_equal_located_rule(nw, ns, cells, seed):
    s = S.droplet(nw, ns, cells=cells, seed=seed)
    o = O.Oracle(s)
    f_lit = o.force(True, O.TERM_NEAR)
    f_gen, _ = o.near_generic()
    scale = np.sqrt((f_lit ** 2).mean())
    assert np.abs(f_lit - f_gen).max() / scale < 1e-12
    assert (o.located() >= 0).all()


def test_near_third_law():
    s = S.droplet(400, 5, cells=(8, 8, 4), seed=4)
    o = O.Oracle(s)
    f = o.force(True, O.TERM_NEAR)
    assert np.abs(f.sum(0)).max() / np.abs(f).max() < 1e-12


def test_w1_w2_split_and_keys():
    s = S.droplet(500, 3, cells=(8, 8, 4), seed=5)
    o = O.Oracle(s)
    o.force(True, O.TERM_NEAR)
    key, w1 = o.keys()
    # w1 waters sit wholly in their key cell; split waters have a site elsewhere
    loc = o.located()
    for m in range(s.n_water):
        cells = set(loc[3 * m:3 * m + 3])
        assert (len(cells) == 1 and key[m] in cells) == bool(w1[m]) or not w1[m]
        assert loc[3 * m] == key[m]  # the O is located in its key cell


def test_pair_counts_match_located_rule():
    s = S.droplet(300, 2, cells=(8, 8, 4), seed=6)
    o = O.Oracle(s)
    o.force(True, O.TERM_NEAR)
    ncoul, nlj = o.pair_counts()
    loc = o.located()
    mol = np.concatenate([np.repeat(np.arange(s.n_water), 3), s.n_water + np.repeat(np.arange(s.n_surf), 29)])
    ncx, ncy, ncz = s.cells
    cx, cy, cz = loc % ncx, (loc // ncx) % ncy, loc // (ncx * ncy)
    near = (np.abs(cx[:, None] - cx[None]) <= 1) & (np.abs(cy[:, None] - cy[None]) <= 1) & (np.abs(cz[:, None] - cz[None]) <= 1)
    near &= mol[:, None] != mol[None]
    assert ncoul == int(near.sum())

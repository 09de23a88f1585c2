"""The reference's restart and snapshot formats (src/read_config.f90,
src/write_pdb.f90): exact record layout and round trips."""
import math
import os

import numpy as np
import pytest

from surfactant_enhanced_spreading_gb300 import io as sio
from surfactant_enhanced_spreading_gb300 import system as S


def test_restart_line_layout(tmp_path):
    p = tmp_path / "cfg.dat"
    sio.write_config(str(p), np.array([[1.5, -2.25, 10.0]]), np.array([[0.002, -0.003, 0.0]]))
    lines = p.read_text().splitlines()
    assert lines[0] == "   1.500   -2.250   10.000"
    # velocity v / 0.01 + 0.5
    assert lines[1] == "   0.700    0.200    0.500"


def test_restart_round_trip(tmp_path):
    s = S.droplet(300, 3, cells=(8, 8, 4), seed=5)
    p = tmp_path / "data_cont2.dat"
    sio.write_config(str(p), s.pos, s.vel)
    pos, vel = sio.read_config(str(p), s.n_water, s.n_surf, box_half=s.half_box)
    assert pos.shape == s.pos.shape and vel.shape == s.vel.shape
    # 3 decimals: half a unit of the last place, plus the reader's exp(-9) shift
    assert np.abs(pos - math.exp(-9.0) - s.pos).max() <= 5e-4 + 1e-12
    assert np.abs(vel - s.vel).max() <= 5e-6 + 1e-12


def test_restart_checks(tmp_path):
    p = tmp_path / "short.dat"
    sio.write_config(str(p), np.zeros((3, 3)), np.zeros((3, 3)))
    with pytest.raises(ValueError, match="needed"):
        sio.read_config(str(p), 2, 0)
    q = tmp_path / "far.dat"
    sio.write_config(str(q), np.array([[50.0, 0.0, 0.0]] * 3), np.zeros((3, 3)))
    with pytest.raises(ValueError, match="out of bounds"):
        sio.read_config(str(q), 1, 0, box_half=np.array([10.0, 10.0, 10.0]))


def test_pdb_record_layout(tmp_path):
    pos = np.array([[1.0, 2.0, 3.0], [0.5, 0.25, -1.0], [0.0, 0.0, 0.0]]) / S.SIGMA
    paths = sio.write_pdb(str(tmp_path), 100, pos, 1, 0)
    assert [os.path.basename(x) for x in paths] == ["data0000100a.pdb", "data0000100s.pdb"]
    lines = open(paths[0]).read().splitlines()
    assert lines[0] == "HETATM    1    O WAT     1       1.000   2.000   3.000"
    assert lines[1] == "HETATM    2    H WAT     1       0.500   0.250  -1.000"
    assert open(paths[1]).read() == ""


def test_pdb_file_split_and_surfactants(tmp_path):
    nw, ns = 33334, 2
    pos = np.zeros((3 * nw + 29 * ns, 3))
    paths = sio.write_pdb(str(tmp_path), 7, pos, nw, ns)
    assert [os.path.basename(x) for x in paths] == ["data0000007a.pdb", "data0000007b.pdb", "data0000007s.pdb"]
    assert sum(1 for _ in open(paths[0])) == 3 * 33333
    assert sum(1 for _ in open(paths[1])) == 3
    srf = open(paths[2]).read().splitlines()
    assert len(srf) == 58
    assert srf[17][11:16] == "   Si" and srf[29][6:11] == "   30" and srf[29][20:26] == "     2"
    # exactly 33,333 waters fit one file
    assert len(sio.write_pdb(str(tmp_path), 8, np.zeros((3 * 33333, 3)), 33333, 0)) == 2

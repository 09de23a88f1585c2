"""The reference's file formats for this path: the restart file it starts
from and the PDB snapshots it writes.

Restart (src/read_config.f90:16-38): for every mobile site, in the
reference's order (waters O, H, H, then 29-site surfactants), one position
line and one velocity line, both Fortran `(f8.3,f9.3,f9.3)`.  Positions are
in sigma; on reading the reference adds exp(-9) to every coordinate (so no
site lies exactly on a cell face).  A velocity is stored as v / 0.01 + 0.5
(v in sigma per step) and read back as (stored - 0.5) * 0.01.

Snapshots (src/write_pdb.f90:19-169): HETATM records
`(a6,i5,a5,a4,i6,f12.3,f8.3,f8.3)` with coordinates in Angstrom; waters go
33,333 molecules per file named data<7-digit step><a, b, ...>.pdb, the
surfactants into data<7-digit step>s.pdb.
"""
from __future__ import annotations

import math
import os

import numpy as np

from .system import SIGMA

POS_OFFSET = math.exp(-9.0)          # added by the reference's reader
WATERS_PER_FILE = 33333
WATER_NAMES = ("O", "H", "H")
SURF_NAMES = ("H", "O", "C", "C", "O", "C", "C", "O", "C", "C", "O", "C", "C", "O", "C", "C", "C", "Si", "C",
              "O", "Si", "C", "C", "C", "O", "Si", "C", "C", "C")


def _fortran_f(v: float, w: int, d: int) -> str:
    """Fortran Fw.d output: right-justified in w columns, d decimals,
    asterisks when the number does not fit."""
    s = f"{v:{w}.{d}f}"
    if len(s) > w:
        return "*" * w
    return s


def _fortran_a(s: str, w: int) -> str:
    """Fortran Aw output: a shorter string is right-justified."""
    return s[-w:].rjust(w)


def _fortran_i(v: int, w: int) -> str:
    s = str(int(v)).rjust(w)
    return "*" * w if len(s) > w else s


def _line3(x: float, y: float, z: float) -> str:
    return _fortran_f(x, 8, 3) + _fortran_f(y, 9, 3) + _fortran_f(z, 9, 3)


def write_config(path: str, pos: np.ndarray, vel: np.ndarray) -> None:
    """Restart file of positions and velocities (reduced units), as
    src/read_config.f90 reads it."""
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    vel = np.asarray(vel, dtype=np.float64).reshape(-1, 3)
    if pos.shape != vel.shape:
        raise ValueError("positions and velocities differ in shape")
    enc = vel / 0.01 + 0.5
    with open(path, "w") as f:
        for p, v in zip(pos, enc):
            f.write(_line3(*p) + "\n")
            f.write(_line3(*v) + "\n")


def _parse3(line: str) -> tuple:
    # fixed columns 1-8, 9-17, 18-26
    return float(line[0:8]), float(line[8:17]), float(line[17:26])


def read_config(path: str, n_water: int, n_surf: int, box_half: np.ndarray | None = None):
    """Positions and velocities of a restart file, as the reference reads
    them: positions + exp(-9), velocities (stored - 0.5) * 0.01.  With
    box_half (sigma), coordinates outside [-half, half] raise ValueError (the
    reference prints "out of bounds")."""
    n = 3 * n_water + 29 * n_surf
    with open(path) as f:
        lines = [ln for ln in f.read().splitlines() if ln.strip()]
    if len(lines) < 2 * n:
        raise ValueError(f"{path}: {len(lines)} lines, {2 * n} needed for {n} sites")
    raw = np.array([_parse3(lines[k]) for k in range(2 * n)], dtype=np.float64)
    pos, vel = raw[0::2], raw[1::2]
    if box_half is not None:
        bh = np.asarray(box_half, dtype=np.float64)
        if np.any(np.abs(pos) > bh):
            raise ValueError(f"{path}: positions out of bounds")
    return pos + POS_OFFSET, (vel - 0.5) * 0.01


def pdb_stem(step: int) -> str:
    """data<step as 7 digits, zero padded> (src/write_pdb.f90:25-69)."""
    return "data" + str(int(step)).zfill(7)[-7:]


def _record(serial: int, name: str, res: str, resseq: int, x: float, y: float, z: float) -> str:
    return ("HETATM" + _fortran_i(serial, 5) + _fortran_a(name, 5) + _fortran_a(res, 4) + _fortran_i(resseq, 6)
            + _fortran_f(x, 12, 3) + _fortran_f(y, 8, 3) + _fortran_f(z, 8, 3))


def write_pdb(directory: str, step: int, pos: np.ndarray, n_water: int, n_surf: int) -> list:
    """Snapshot files of one step (positions in sigma, written in Angstrom);
    returns the paths written."""
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3) * SIGMA
    stem = os.path.join(directory, pdb_stem(step))
    paths = []
    n_files = int(n_water / (WATERS_PER_FILE + 0.0001)) + 1
    if n_files > 10:
        raise ValueError("the snapshot format names at most 10 water files (333,330 waters)")
    for k in range(n_files):
        m0 = k * WATERS_PER_FILE
        m1 = min(n_water, m0 + WATERS_PER_FILE)
        path = stem + "abcdefghij"[k] + ".pdb"
        with open(path, "w") as f:
            for i in range(m1 - m0):
                for t in range(3):
                    x, y, z = pos[3 * (m0 + i) + t]
                    f.write(_record(3 * i + t + 1, WATER_NAMES[t], "WAT", i + 1, x, y, z) + "\n")
        paths.append(path)
    path = stem + "s.pdb"
    base = 3 * n_water
    with open(path, "w") as f:
        serial = 0
        for i in range(n_surf):
            for t in range(29):
                serial += 1
                x, y, z = pos[base + 29 * i + t]
                f.write(_record(serial, SURF_NAMES[t], "SRF", i + 1, x, y, z) + "\n")
    paths.append(path)
    return paths

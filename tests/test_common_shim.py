"""The COMMON-block layer (include/sesp_common.h) through its C-level test
program (tests/cmn_shim_test.c), which fills every domain's COMMON arrays
by a transcription of src/read_config.f90:45-175 and calls the layer.

* layout (host only): the layer's map places every molecule in the slot the
  transcription chose, scatter reproduces read_config's arrays bit for bit,
  gather inverts scatter, re-assignment follows the reference's w1 / w2 /
  surfactant rule for moved molecules, and the error paths;
* steps (GPU): the step loop run through the gfortran-named subroutines on
  the reference's 27-domain box: the first forces read from the COMMON
  arrays within 1e-10 of the oracle; after 20 steps the mirror holds the
  device state bit for bit, molecules sit where read_config would put them,
  and the trajectory matches the same run through the Python binding
  (molecule order differs, so within 1e-8 sigma, not bit for bit).
"""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from surfactant_enhanced_spreading_gb300 import engine as E
from surfactant_enhanced_spreading_gb300 import system as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "surfactant_enhanced_spreading_gb300")


def _cuda_lib():
    for d in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib",
              "/usr/local/cuda/targets/x86_64-linux/lib"):
        if os.path.isdir(d):
            return d
    return "/usr/local/cuda/lib64"


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    from surfactant_enhanced_spreading_gb300.csrc import build
    build.build()
    exe = str(tmp_path_factory.mktemp("cmn") / "cmn_shim_test")
    cmd = ["gcc", "-O2", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cmn_shim_test.c"), "-o", exe, "-L", PKG, "-lsesp",
           "-Wl,-rpath," + PKG, "-Wl,-rpath," + _cuda_lib(), "-lm"]
    subprocess.run(cmd, check=True)
    return exe


@pytest.fixture(scope="module")
def state():
    """The reference's box (12 x 12 x 12 cells, 27 domains of 4^3 cells):
    2,000 waters and 12 surfactants on 2 graphite layers."""
    return S.droplet(2000, 12, cells=(12, 12, 12), seed=77, graphite_layers=2)


def _write(path, s, nsteps=0, precision=E.PLAIN_FP64):
    hdr = np.array([s.n_water, s.n_surf, *s.cells, len(s.carbons), nsteps, precision], dtype=np.int32)
    with open(path, "wb") as f:
        f.write(hdr.tobytes())
        f.write(np.ascontiguousarray(s.pos, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(s.vel, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(s.carbons, dtype=np.float64).tobytes())


def test_layout_round_trip(program, state, tmp_path):
    inp = str(tmp_path / "in.bin")
    _write(inp, state)
    r = subprocess.run([program, "0", inp], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK layout: 2000 waters, 12 surfactants, 27 domains" in r.stdout


@pytest.mark.gpu
def test_step_loop_through_common(program, state, tmp_path):
    inp, out = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    nsteps = 20
    _write(inp, state, nsteps)
    r = subprocess.run([program, "1", inp, out], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    n3 = 3 * state.n_sites
    raw = np.fromfile(out, dtype=np.float64)
    f0, pos, vel, eta = raw[:n3].reshape(-1, 3), raw[n3:2 * n3].reshape(-1, 3), raw[2 * n3:3 * n3].reshape(-1, 3), raw[-1]
    fo = O.Oracle(state).force(True)
    assert np.linalg.norm(f0 - fo) / np.linalg.norm(fo) < 1e-10
    eng = E.Engine(state, E.PLAIN_FP64)
    eng.force(True)
    eng.init_accel()
    eng.run(99101, nsteps)
    p, v, _ = eng.state()
    assert np.abs(pos - p).max() < 1e-8
    assert np.abs(vel - v).max() < 1e-8 * np.abs(v).max()
    assert abs(eta - eng.eta) <= 1e-8 * max(abs(eng.eta), 1e-12)

"""Build recipe of the engine library ``libsesp.so`` (sm_103a only).

Five translation units are compiled in parallel with nvcc and linked into a
shared library next to this file's package:

* ``k_exact.cu`` with ``-fmad=false``: cell assignment and the FP64
  SHAKE/RATTLE integrator, whose discrete decisions and iteration counts must
  round like the reference's separately rounded Fortran arithmetic;
* ``k_constraint.cu``: the mixed paths' constraint sweeps (FP64, or FP32);
* ``k_force.cu``: pair, multipole and intramolecular kernels;
* ``sesp_api.cu``: the C ABI (host code compiled without contraction so the
  force-field tables and translation operators are reproducible);
* ``sesp_common.cpp``: the COMMON-block layer over that ABI (host code).
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB = os.path.join(PKG, "libsesp.so")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr", "-diag-suppress", "1444"]
UNITS = [("k_exact.cu", ["-fmad=false"]), ("k_constraint.cu", []), ("k_force.cu", []), ("sesp_api.cu", []),
         ("sesp_common.cpp", [])]
HEADERS = ["sesp_internal.cuh", "k_launch.cuh", os.path.join("..", "..", "include", "sesp.h"),
           os.path.join("..", "..", "include", "sesp_common.h")]


def _nvcc():
    for cand in [os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"]:
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(HERE, h) for h in HEADERS]
    jobs = []
    objs = []
    for src, flags in UNITS:
        s = os.path.join(HERE, src)
        o = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs + [__file__]):
            jobs.append([nvcc, "-c", s, "-o", o] + ARCH + COMMON + list(flags) + list(extra))

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed for " + cmd[2])
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc, "-shared", "-o", LIB + ".tmp"] + objs + ARCH + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))

"""Build recipe for the CPU oracle (test infrastructure only).

Compiles the C restatement in this folder into ``oracle/liborc.so`` with gcc.
``-ffp-contract=off`` keeps every multiply and add separately rounded, as the
reference's Fortran arithmetic is, so the constraint iterations can be compared
bit for bit with the GPU engine's (which is compiled the same way for them).
With OpenMP (``-fopenmp``, used when gcc accepts it) the pair kernels and the
FMA passes run over cells in parallel; the pair forces are summed per thread
and added in thread order, so a run is deterministic for a given thread count.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["orc_setup.c", "orc_pair.c", "orc_fma.c", "orc_intra.c", "orc_move.c", "orc_api.c", "orc_cfg.c"]
LIB = os.path.join(HERE, "liborc.so")


def build(force=False, quiet=True):
    srcs = [os.path.join(HERE, s) for s in SOURCES] + [os.path.join(HERE, "orc.h")]
    if not force and os.path.exists(LIB):
        lib_t = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= lib_t for s in srcs):
            return LIB
    base = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
            "-Wall", "-Wno-unused-function", "-Wno-misleading-indentation", "-Wno-unknown-pragmas",
            "-o", LIB + ".tmp"] + [os.path.join(HERE, s) for s in SOURCES] + ["-lm"]
    # OpenMP over cells (pair kernels with per-thread force buffers, FMA
    # passes); without it the same code runs on one thread
    res = subprocess.run(base[:1] + ["-fopenmp"] + base[1:], capture_output=True, text=True)
    if res.returncode != 0:
        res = subprocess.run(base, capture_output=True, text=True)
    if res.returncode != 0:
        sys.stderr.write(res.stdout + res.stderr)
        raise RuntimeError("oracle build failed")
    if not quiet and (res.stdout or res.stderr):
        sys.stderr.write(res.stdout + res.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, quiet=False))

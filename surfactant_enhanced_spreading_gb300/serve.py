"""Request loop for spreading runs on one GPU, with continuous batching.

A request is one droplet run: its initial state (a seeded droplet of waters
and surfactants on graphite, built by the client), a step count and an arrival
time.  The server admits requests in arrival order as long as their device
memory fits the HBM budget, gives each its own engine context (own CUDA
stream, state resident on the device), and advances every admitted run by
chunks of `chunk` steps launched asynchronously: chunks of different runs
execute concurrently on the GPU, and a run that arrives while others are
running starts as soon as memory allows.  Finished runs are downloaded,
their memory is released and the next requests are admitted.

Every run is independent of the others (its own context; all kernels are
deterministic), so its result is bit-identical whether it runs alone or in
the mix - which tests/test_gpu_serve.py checks.

A run whose SHAKE/RATTLE failure count passes `max_failures` between chunks
has blown up (a state that has, collapses into a few cells and slows every
later step by orders of magnitude): it is stopped, reported as failed with
the steps it completed, and its memory goes to the next request.
"""
from __future__ import annotations

import dataclasses
import math
import time

import numpy as np

from . import config_preset as CP
from . import engine as E
from . import system as S


@dataclasses.dataclass
class Request:
    rid: int
    system: S.System
    steps: int
    arrival: float = 0.0        # seconds after the start of the run


@dataclasses.dataclass
class Result:
    rid: int
    n_sites: int
    steps: int
    arrival: float
    admitted: float
    finished: float
    pos: np.ndarray | None = None
    vel: np.ndarray | None = None
    eta: float = 0.0
    device_bytes: int = 0
    estimate_bytes: int = 0
    shake_failures: int = 0     # SHAKE/RATTLE molecule failures over the run (engine counter 0)
    steps_done: int = -1        # steps completed (-1: all of them)
    failed: bool = False        # stopped after its failures passed the server's limit

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def cells_for(n_water: int, n_surf: int) -> tuple:
    """A closed box (multiples of 4 cells of 12 A) that holds the droplet the
    generator builds for these counts."""
    radius = (3.0 * n_water / (2.0 * math.pi * 0.0334)) ** (1.0 / 3.0)
    shell = 14.0 if n_surf else 2.0
    half_xy = radius + shell + 0.02 * n_surf + 8.0
    height = 7.2 + radius + shell + 0.02 * n_surf + 8.0
    cx = 4 * math.ceil(2.0 * half_xy / 12.0 / 4.0)
    cz = 4 * math.ceil(2.0 * height / 12.0 / 4.0)
    return (max(cx, 4), max(cx, 4), max(cz, 4))


def make_request(rid: int, n_water: int, n_surf: int, steps: int, seed: int, arrival: float = 0.0,
                 preset: int = 0) -> Request:
    """One droplet run.  preset 0: the reference's force field in a closed
    box; preset 1: the configuration preset, 12-bead chains, on a periodic
    2-layer sheet 2.5 droplet diameters across."""
    if preset == CP.PRESET_CONFIG:
        n = CP.sheet_cells(n_water)
        cells = (n, n, CP.box_height_cells(n_water, n_surf))
        s = CP.config_droplet(n_water, n_surf, cells=cells, seed=seed, graphite_layers=2)
        return Request(rid=rid, system=s, steps=steps, arrival=arrival)
    cells = list(cells_for(n_water, n_surf))
    for _ in range(4):
        try:
            s = S.droplet(n_water, n_surf, cells=tuple(cells), seed=seed)
            return Request(rid=rid, system=s, steps=steps, arrival=arrival)
        except RuntimeError as e:
            if "does not fit" not in str(e):
                raise
            cells = [c + 4 for c in cells]
    raise RuntimeError(f"no box found for {n_water} waters and {n_surf} surfactants")


def estimate_bytes(system: S.System) -> int:
    """Upper estimate of an engine's device memory for this system, from the
    engine's allocation list: per-site, per-molecule and per-cell arrays, the
    multipole tables of the three levels, the translation operators and the
    per-column carbon lists (each carbon lies within reach of at most about
    8 bottom-layer columns) with their 8 groups of 33 y-bin starts and a z
    range, with a 10 % margin."""
    n = system.n_sites
    nmol = system.n_water + system.n_surf
    nc = np.array(system.cells, dtype=np.int64)
    ncell = int(np.prod(nc))
    n3, n2 = ncell // 8, ncell // 64
    per = getattr(system, "preset", 0) == CP.PRESET_CONFIG
    d2 = max(1, int((nc // 4).max()) - 1)
    w2 = 2 * d2 + 1
    per_site = 12 * 8 + 1 + 4 * 4 + 32 + 16 + 8 + 4 + 3 * 8 + 27 * 8 + 6 + 3 * 8 + 12 * 8
    per_mol = 5 * 4 + 2 * 8 + 4 + 4 + 2 * 4 + 2   # incl. the constraint halves' water lists and sweep counts
    cz = 25 * 16
    cells = ncell * (5 * 4 + 2 * cz + 4 + 9 * 20 + 25 * 8) + n3 * (4 + 2 * cz) + n2 * (4 + 2 * cz)
    ops = (w2 ** 3 + 4 * 8) * 15 * 25 * 16 + w2 ** 3 * 45 * 24
    # real-form M2L at L4 and L3: operators, class-packed multipoles, partial
    # sums of 21 offset groups (FP64 sizes: an upper bound)
    pad4 = int(np.prod(nc // 2 + 4)) * 200
    pad3 = int(np.prod(nc // 4 + 4)) * 200
    ops += 8 * (2 * 343 * 25 * 28 + pad4 + pad3 + 21 * 25 * (ncell + n3)) + 16 * 16 * (ncell // 1024 + 1) + 8 * 189 * 4
    ncarb = system.carbons.reshape(-1, 3).shape[0]
    ncol = int(nc[0] * nc[1])
    # each carbon lies within reach of about 8 bottom-layer columns (12 with
    # the periodic preset's wider reach)
    reach_cols = 12 if per else 8
    graphite = reach_cols * ncarb * 48 + (ncol + 1) * 4 + ncol * 8 * (33 * 4 + 8) + int(nc.sum()) * 8 + n * 4
    surf = system.sites_per_surf * system.n_surf * 4 + n * 4
    if per:   # the image-summed L2 M2L factors of the replica (FP64 and FP32)
        surf += int(np.prod(2 * (nc // 4) - 1)) * 45 * 24
    total = n * per_site + nmol * per_mol + cells + ops + graphite + surf + 4096
    return int(1.1 * total) + (1 << 20)


class Server:
    def __init__(self, budget_bytes: int, precision: int = E.MIXED, chunk: int = 100, max_active: int = 64,
                 device: int = 0, keep_state: bool = True, max_failures: int = 1000):
        self.budget = int(budget_bytes)
        self.precision = precision
        self.chunk = int(chunk)
        self.max_active = int(max_active)
        self.max_failures = int(max_failures)
        self.device = device
        self.keep_state = keep_state
        self.peak_used = 0          # largest admitted estimate total seen by the last run()

    def run(self, requests: list[Request], clock=time.perf_counter) -> list[Result]:
        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        for r in pending:
            if estimate_bytes(r.system) > self.budget:
                raise E.SespError(f"EBUDGET: request {r.rid} needs more than the whole budget")
        active = []
        results = []
        used = 0
        self.peak_used = 0
        t0 = clock()
        while pending or active:
            now = clock() - t0
            # admission in arrival order while the budget allows (no overtaking)
            while pending and pending[0].arrival <= now and len(active) < self.max_active:
                req = pending[0]
                est = estimate_bytes(req.system)
                if used + est > self.budget:
                    break
                pending.pop(0)
                eng = E.Engine(req.system, self.precision, device=self.device)
                eng.force(True)
                eng.init_accel()
                actual = eng.device_bytes()
                nbytes = max(est, actual)
                used += nbytes
                self.peak_used = max(self.peak_used, used)
                active.append({"req": req, "eng": eng, "done": 0, "kb": 99101, "bytes": nbytes, "actual": actual, "est": est,
                               "admitted": clock() - t0, "running": False})
            progressed = False
            for a in list(active):
                eng = a["eng"]
                if a["running"] and eng.busy():
                    continue
                a["running"] = False
                req = a["req"]
                failures = int(eng.counters()[0])
                failed = failures > self.max_failures
                if a["done"] < req.steps and not failed:
                    n = min(self.chunk, req.steps - a["done"])
                    eng.run_async(a["kb"], n)
                    a["kb"] += n
                    a["done"] += n
                    a["running"] = True
                    progressed = True
                    continue
                eng.sync()
                fin = clock() - t0
                res = Result(rid=req.rid, n_sites=req.system.n_sites, steps=req.steps, arrival=req.arrival,
                             admitted=a["admitted"], finished=fin, device_bytes=a["actual"],
                             estimate_bytes=a["est"], shake_failures=failures,
                             steps_done=a["done"] if failed else -1, failed=failed)
                if self.keep_state:
                    pos, vel, _ = eng.state()
                    res.pos, res.vel, res.eta = pos, vel, eng.eta
                eng.close()
                used -= a["bytes"]
                active.remove(a)
                results.append(res)
                progressed = True
            if not progressed:
                if pending and not active:
                    # idle until the next arrival
                    wait = pending[0].arrival - (clock() - t0)
                    if wait > 0:
                        time.sleep(min(wait, 0.01))
                else:
                    time.sleep(0.0002)
        return sorted(results, key=lambda r: r.rid)


class SlotServer:
    """The same request loop with the running requests as the replicas
    ("slots") of one batched context, so that every launch advances all of
    them.

    Requests join and leave at chunk boundaries.  A chunk is `chunk` steps, a
    multiple of the rebuild interval, so at a boundary every run has just
    done a rebuild step.  When the set of runs changes, the context is formed
    again from the runs' current states.  The old context's state is
    downloaded: positions, velocities, accelerations, eta and failure counts.
    The new context uploads it and calls force(rebuild).  The rebuild starts
    from the same positions the runs' last rebuild step used, so it builds
    the same lists and local expansions.  Each continuing run then gets back
    its accelerations and eta; a new run gets init_accel's.  A run's
    trajectory is therefore bit-identical to the same run alone;
    tests/test_gpu_serve.py checks it.  Request step counts must be multiples
    of the rebuild interval (10)."""

    def __init__(self, budget_bytes: int, precision: int = E.MIXED, chunk: int = 100, max_active: int = 64,
                 device: int = 0, keep_state: bool = True, max_failures: int = 1000, interval: int = 10):
        if chunk % interval:
            raise ValueError("the chunk must be a multiple of the rebuild interval")
        self.budget = int(budget_bytes)
        self.precision = precision
        self.chunk = int(chunk)
        self.interval = int(interval)
        self.max_active = int(max_active)
        self.max_failures = int(max_failures)
        self.device = device
        self.keep_state = keep_state
        self.peak_used = 0
        self.reforms = 0            # contexts formed by the last run()
        self.reform_s = 0.0         # host time spent forming them
        self.form_parts = {}        # ... split into upload, force and state

    def _form(self, runs):
        """A batched context over the runs, each at its current state."""
        t = time.perf_counter()
        mark = [t]

        def lap(name):
            now = time.perf_counter()
            self.form_parts[name] = self.form_parts.get(name, 0.0) + now - mark[0]
            mark[0] = now
        systems = []
        for a in runs:
            s = a["req"].system.copy() if a["pos"] is not None else a["req"].system
            if a["pos"] is not None:
                s.pos, s.vel = a["pos"], a["vel"]
            systems.append(s)
        eng = E.Engine(systems, self.precision, device=self.device)
        lap("upload")
        eng.force(True)
        lap("force")
        eng.init_accel()
        if any(a["pos"] is not None for a in runs):
            _, _, acc = eng.state()
            for k, a in enumerate(runs):
                if a["acc"] is not None:
                    acc[eng.offsets[k]:eng.offsets[k + 1]] = a["acc"]
            eng.set_state(None, None, acc, 0.0)
        eng.set_etas([a["eta"] for a in runs])
        lap("state")
        self.reforms += 1
        self.reform_s += time.perf_counter() - t
        return eng

    def run(self, requests: list[Request], clock=time.perf_counter) -> list[Result]:
        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        presets = {getattr(r.system, "preset", 0) for r in pending}
        if len(presets) > 1:
            raise ValueError("the requests of one batched context share one force field (preset)")
        for r in pending:
            if estimate_bytes(r.system) > self.budget:
                raise E.SespError(f"EBUDGET: request {r.rid} needs more than the whole budget")
            if r.steps % self.interval:
                raise ValueError(f"request {r.rid}: steps must be a multiple of {self.interval}")
        runs, results = [], []
        eng = None
        kb = 99101
        used = 0
        self.peak_used = 0
        self.reforms, self.reform_s, self.form_parts = 0, 0.0, {}
        t0 = clock()
        while pending or runs:
            if eng is not None:
                eng.sync()
                fails = eng.failures()
                for k, a in enumerate(runs):
                    a["fails"] = a["fails0"] + int(fails[k])
            now = clock() - t0
            leaving = [a for a in runs if a["done"] >= a["req"].steps or a["fails"] > self.max_failures]
            free = used - sum(a["est"] for a in leaving)
            joining = []
            for req in pending:
                if req.arrival > now or len(runs) - len(leaving) + len(joining) >= self.max_active:
                    break
                est = estimate_bytes(req.system)
                if free + est > self.budget:
                    break
                free += est
                joining.append(req)
            if eng is not None and (leaving or joining):
                # chunk boundary with a change: take the runs' states out of the context
                pos, vel, acc = eng.state()
                etas = eng.etas()
                for k, a in enumerate(runs):
                    sl = slice(eng.offsets[k], eng.offsets[k + 1])
                    a["pos"], a["vel"], a["acc"], a["eta"] = pos[sl], vel[sl], acc[sl], float(etas[k])
                eng.close()
                eng = None
            for a in leaving:
                req = a["req"]
                failed = a["done"] < req.steps
                res = Result(rid=req.rid, n_sites=req.system.n_sites, steps=req.steps, arrival=req.arrival,
                             admitted=a["admitted"], finished=now, device_bytes=a["est"], estimate_bytes=a["est"],
                             shake_failures=a["fails"], steps_done=a["done"] if failed else -1, failed=failed)
                if self.keep_state:
                    res.pos, res.vel, res.eta = a["pos"], a["vel"], a["eta"]
                results.append(res)
                runs.remove(a)
            used = free
            self.peak_used = max(self.peak_used, used)
            for req in joining:
                pending.remove(req)
                runs.append({"req": req, "done": 0, "est": estimate_bytes(req.system), "admitted": clock() - t0,
                             "pos": None, "vel": None, "acc": None, "eta": 0.0, "fails": 0, "fails0": 0})
            if not runs:
                if pending:
                    wait = pending[0].arrival - (clock() - t0)
                    if wait > 0:
                        time.sleep(min(wait, 0.01))
                continue
            if eng is None:
                eng = self._form(runs)
                for a in runs:
                    a["fails0"] = a["fails"]
            n = min(self.chunk, min(a["req"].steps - a["done"] for a in runs))
            eng.run_async(kb, n)
            kb += n
            for a in runs:
                a["done"] += n
        if eng is not None:
            eng.close()
        return sorted(results, key=lambda r: r.rid)


def summarize(results: list[Result], wall: float | None = None) -> dict:
    lat = np.array([r.latency for r in results])
    atom_steps = float(sum(r.n_sites * (r.steps if r.steps_done < 0 else r.steps_done) for r in results))
    span = wall if wall is not None else (max(r.finished for r in results) - min(r.arrival for r in results))
    return {"requests": len(results), "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)), "mean_latency_s": float(lat.mean()),
            "atom_steps_per_s": atom_steps / span if span > 0 else None, "span_s": span,
            "shake_failures": int(sum(r.shake_failures for r in results)),
            "failed_requests": [r.rid for r in results if r.failed]}


def poisson_requests(n: int, rate_per_s: float, seed: int, water=(1000, 50000), surf=(0, 500), steps=(500, 5000),
                     step_quantum: int = 100, preset: int = 0) -> list[Request]:
    """Seeded Poisson arrivals of seeded droplet runs."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(n):
        t += rng.exponential(1.0 / rate_per_s)
        nw = int(rng.integers(water[0], water[1] + 1))
        ns = int(rng.integers(surf[0], surf[1] + 1))
        st = int(rng.integers(steps[0] // step_quantum, steps[1] // step_quantum + 1)) * step_quantum
        out.append(make_request(k, nw, ns, st, seed=int(rng.integers(1 << 30)), arrival=t, preset=preset))
    return out


def run_one_at_a_time(requests: list[Request], precision: int, device: int = 0, chunk: int = 100) -> list[Result]:
    """The same requests served strictly one after another in arrival order
    (no overlap), for comparison with Server.run: a request starts at its
    arrival or when the previous one finished, whichever is later."""
    out = []
    t0 = time.perf_counter()
    for req in sorted(requests, key=lambda r: (r.arrival, r.rid)):
        wait = req.arrival - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        start = time.perf_counter() - t0
        eng = E.Engine(req.system, precision, device=device)
        E.mybox_start(eng)
        kb = 99101
        for k in range(0, req.steps, chunk):
            n = min(chunk, req.steps - k)
            eng.run(kb, n)
            kb += n
        eng.sync()
        pos, vel, _ = eng.state()
        out.append(Result(rid=req.rid, n_sites=req.system.n_sites, steps=req.steps, arrival=req.arrival,
                          admitted=start, finished=time.perf_counter() - t0, pos=pos, vel=vel, eta=eng.eta,
                          shake_failures=int(eng.counters()[0])))
        eng.close()
    return out


def main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser(description="Serve seeded droplet runs with Poisson arrivals on one GPU.")
    ap.add_argument("--requests", type=int, default=24)
    ap.add_argument("--rate", type=float, default=8.0, help="arrivals per second")
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--budget-gb", type=float, default=8.0)
    ap.add_argument("--chunk", type=int, default=100)
    ap.add_argument("--water", type=int, nargs=2, default=(1000, 20000))
    ap.add_argument("--surf", type=int, nargs=2, default=(0, 200))
    ap.add_argument("--steps", type=int, nargs=2, default=(500, 2000))
    ap.add_argument("--compare-plain", action="store_true",
                    help="also serve the same requests one at a time on the plain FP64 path")
    a = ap.parse_args(argv)
    reqs = poisson_requests(a.requests, a.rate, a.seed, water=tuple(a.water), surf=tuple(a.surf),
                            steps=tuple(a.steps))
    srv = Server(int(a.budget_gb * 2**30), precision=E.MIXED, chunk=a.chunk)
    # warm the library and the device once so the first request does not pay for it
    warm = make_request(-1, 300, 3, 100, seed=1)
    srv.run([warm])
    res = srv.run(reqs)
    out = {"mode": "continuous batching, mixed precision", "budget_bytes": srv.budget,
           "peak_admitted_bytes": srv.peak_used, **summarize(res)}
    if a.compare_plain:
        seq = run_one_at_a_time(reqs, E.PLAIN_FP64, chunk=a.chunk)
        out["one_at_a_time_plain_fp64"] = summarize(seq)
    print(json.dumps(out))


if __name__ == "__main__":
    main()

"""Benchmark of the per-timestep force-and-integrate path.

One step = move_a (Nose-Hoover predictor + SHAKE), the force section (near
field, local-expansion force, intramolecular, walls, graphite; every 10th step
also the cell sort, lists and far-field build) and move_b (RATTLE), exactly the
body of the reference's step loop (src/mybox.f90:136-227).

Workload (default): the single-system mixed-precision configuration with the
reference's force field: 20,000 SPC/E waters and 200 29-site trisiloxane
surfactants on 4-layer AB graphite, closed box of 24 x 24 x 12 cells of 12 A
(288 x 288 x 144 A), seeded synthetic droplet.  Metric: atom-steps/s (mobile
sites x steps / s), with ns/day at 2 fs; the plain FP64 GPU path is measured on
the same workload and reported beside it with the mixed path's force error.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun each rank runs its own replica on its GPU (no collective in the
data path; replicas only), timing is the max over ranks.
"""
from __future__ import annotations

import argparse
import math
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(n_water=20000, n_surf=200, cells=(24, 24, 12), graphite_layers=4, seed=2024)
DT_FS = 2.0
FLOPS_COUL = 18       # per ordered site pair, Coulomb only (sqrt and divide as 1 each)
FLOPS_LJ_EXTRA = 11   # added when the pair is LJ-active within rc
FLOPS_L2P = 25 * 40   # local-expansion force per site


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", action="store_true", help="small workload (tests / profiling)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plain-steps", type=int, default=20)
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-replica batched measurement")
    ap.add_argument("--no-served", action="store_true", help="skip the served-stream measurement")
    ap.add_argument("--replicas", type=int, default=64)
    ap.add_argument("--requests", type=int, default=12)
    return ap.parse_args()


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """torch.distributed only for the barrier and the max over ranks."""

    def __init__(self, ws):
        self.ws = ws
        self.dist = None
        if ws > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, v):
        if not self.dist:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


def make_system(small):
    from surfactant_enhanced_spreading_gb300 import system as S
    if small:
        return S.droplet(6000, 60, cells=(16, 16, 8), seed=7, graphite_layers=2)
    w = WORKLOAD
    return S.droplet(w["n_water"], w["n_surf"], cells=w["cells"], seed=w["seed"], graphite_layers=w["graphite_layers"])


def make_batch(n, seed, small=False):
    """Batched workload: n replicas, waters ~ logU[1k, 30k] (logU[300, 1k]
    for --small), surfactants per water ~ U[0, 2%], each droplet on its own
    2-layer sheet over the whole floor of the smallest closed box (multiples
    of 4 cells) that holds it."""
    from surfactant_enhanced_spreading_gb300 import serve
    rng = np.random.default_rng(seed)
    lo, hi = (300, 1000) if small else (1000, 30000)
    out = []
    for k in range(n):
        nw = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        ns = int(round(nw * rng.uniform(0.0, 0.02)))
        out.append(serve.make_request(k, nw, ns, 1, seed=int(rng.integers(1 << 30))).system)
    return out


def run_batched(args, local, E):
    systems = make_batch(args.replicas, 4242, args.small)
    n_sites = sum(s.n_sites for s in systems)
    res = {"replicas": len(systems), "sites": n_sites,
           "workload": f"{len(systems)} replicas, waters ~ logU[{'300, 1k' if args.small else '1k, 30k'}], "
                       "surfactants ~ U[0, 2%] of waters, 2-layer graphite over the box floor, seed 4242"}
    for name, prec, steps in (("mixed", E.MIXED, 20), ("plain_fp64", E.PLAIN_FP64, 3)):
        eng = E.Engine(systems, prec, device=local)
        eng.force(True)
        eng.autotune()
        eng.init_accel()
        eng.run(99101, 3)
        ms = eng.run_timed(99104, steps, flush_l2=True)
        res[name] = {"value": n_sites * steps / (ms.sum() / 1e3), "unit": "atom-steps/s", "steps": steps,
                     "ms_per_step": float(ms.mean()), "shake_failures": eng.counters()[0]}
        eng.close()
        del eng
    res["mixed_vs_plain_speedup"] = res["mixed"]["value"] / res["plain_fp64"]["value"]
    return res


def run_served(args, local):
    from surfactant_enhanced_spreading_gb300 import engine as E
    from surfactant_enhanced_spreading_gb300 import serve
    dist = (dict(water=(300, 1000), surf=(0, 10), steps=(100, 300)) if args.small else
            dict(water=(1000, 50000), surf=(0, 500), steps=(500, 5000)))
    reqs = serve.poisson_requests(args.requests, 2.0, 777, **dist)
    srv = serve.Server(64 << 30, precision=E.MIXED, chunk=100, device=local, keep_state=False)
    srv.run([serve.make_request(-1, 300, 3, 100, seed=1)])   # first use of the library
    t0 = time.perf_counter()
    results = srv.run(reqs)
    wall = time.perf_counter() - t0
    out = serve.summarize(results)
    out.update({"requests": len(results), "arrivals_per_s": 2.0, "wall_s": wall,
                "sample": f"{args.requests} seeded Poisson requests: waters ~ U{list(dist['water'])}, "
                          f"surfactants ~ U{list(dist['surf'])}, steps ~ U{list(dist['steps'])} in 100-step chunks, "
                          "mixed precision, HBM budget 64 GiB",
                "peak_admitted_bytes": srv.peak_used})
    return out


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        self.path = os.path.join("/tmp", f"sesp_clocks_{os.getpid()}.csv")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if not self.proc:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        if not rows:
            return out
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        out = {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
               "reasons": reasons, "samples": len(rows)}
        return out


def run_ours(args, ws, rank, local):
    import oracle as O  # the CPU-baseline leg only
    from surfactant_enhanced_spreading_gb300 import engine as E

    D = Dist(ws)
    s = make_system(args.small)
    n_sites = s.n_sites

    # --- mixed path: warm-up, then K steps with per-step CUDA events, cold L2
    eng = E.Engine(s, E.MIXED, device=local)
    eng.force(True)
    eng.init_accel()
    kb = 99101
    eng.run(kb, args.warmup)
    kb += args.warmup
    tile, ctas, ctas_max = eng.autotune()   # launch shapes (no effect on results)
    surf_warps, mols_per_warp = eng.constraint_tuning()[:2]
    eng.run(kb, 1)
    kb += 1
    D.barrier()
    clocks = Clocks(local)
    clocks.start()
    step_ms = eng.run_timed(kb, args.steps, flush_l2=True)
    clk = clocks.stop()
    kb += args.steps
    D.barrier()
    t_ms = D.max(float(step_ms.sum()))
    value = ws * n_sites * args.steps / (t_ms / 1e3)
    ms_per_step = t_ms / args.steps

    # kernel launches in the timed region for this workload (waters, surfactants
    # and graphite present): 9 per step (gather, graphite and intramolecular on
    # the side stream, pair field + finish, site forces, constraint half + eta
    # for move_a, the constraint half for move_b) and 22 more per rebuild step
    # (locate, sort 3, work items 5, isub, graphite list, water order 3, P2M,
    # 2 M2M, multipole packing, 2 M2L, 2 L2L)
    n_rebuild = sum(1 for k in range(kb - args.steps, kb) if k % 10 == 0)
    launches = 9 * args.steps + 22 * n_rebuild

    # --- per-kernel durations over a second pass (events around kernel families)
    eng.enable_timing(True)
    eng.kernel_times(reset=True)
    eng.run(kb, 20)
    kt = eng.kernel_times(reset=True)
    eng.enable_timing(False)
    kb += 20
    ncoul, nlj = eng.pair_counts()
    near_ms = kt[0]
    flops = ncoul * FLOPS_COUL + nlj * FLOPS_LJ_EXTRA + n_sites * FLOPS_L2P
    achieved = flops / (near_ms / 1e3) / 1e12 if near_ms > 0 else None
    peak = fp32_nominal_tflops(local)
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "near_field_traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get("bytes_per_launch")
        except Exception:
            traffic = None

    # --- the same mixed path with the constraint iterations in FP32 (a
    # separate precision mode, reported beside the headline)
    e32 = E.Engine(s, E.MIXED_FP32C, device=local)
    e32.force(True)
    e32.init_accel()
    e32.run(99101, args.warmup)
    c_ms = e32.run_timed(99101 + args.warmup, args.steps, flush_l2=True)
    fp32c = {"value": n_sites * args.steps / (c_ms.sum() / 1e3), "unit": "atom-steps/s",
             "ms_per_step": float(c_ms.mean()), "shake_failures": e32.counters()[0]}
    del e32

    # --- plain FP64 GPU path on the same workload, and the mixed force error
    plain = E.Engine(s, E.PLAIN_FP64, device=local)
    f64 = plain.force(True)
    mixed_ref = E.Engine(s, E.MIXED, device=local)
    f32 = mixed_ref.force(True)
    ferr = float(np.linalg.norm(f32 - f64) / np.linalg.norm(f64))
    del mixed_ref
    plain.init_accel()
    plain.run(99101, 5)
    p_ms = plain.run_timed(99106, args.plain_steps, flush_l2=True)
    plain_value = n_sites * args.plain_steps / (p_ms.sum() / 1e3)
    del plain

    # --- end to end through the C ABI with host buffers: each 10-step chunk
    # uploads the state from pinned host memory, runs, downloads the state
    pos, vel, acc = eng.state()
    try:
        import torch
        hp = torch.from_numpy(pos).pin_memory().numpy()
        hv = torch.from_numpy(vel).pin_memory().numpy()
        ha = torch.from_numpy(acc).pin_memory().numpy()
    except Exception:
        hp, hv, ha = pos, vel, acc
    eta = eng.eta
    chunks = max(1, args.steps // 10)
    D.barrier()
    t0 = time.perf_counter()
    for c in range(chunks):
        eng.set_state(hp, hv, ha, eta)
        eng.run(kb, 10)
        kb += 10
        eng.state(out=(hp, hv, ha))
        eta = eng.eta
    t_e2e = D.max(time.perf_counter() - t0)
    e2e_value = ws * n_sites * 10 * chunks / t_e2e
    state_bytes = 3 * 3 * 8 * n_sites
    e2e = {"value": e2e_value, "unit": "atom-steps/s", "h2d_bytes_per_step": state_bytes / 10,
           "d2h_bytes_per_step": state_bytes / 10,
           "how": "per 10-step chunk: sesp_set_state from pinned host pos/vel/acc, sesp_run(10), sesp_download_state"}

    # --- batched replicas and the served stream (single-GPU runs only)
    batched = run_batched(args, local, E) if (ws == 1 and not args.no_batched) else None
    served = run_served(args, local) if (ws == 1 and not args.no_served) else None

    # --- CPU baseline: the oracle on the same workload, bounded sample
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(s, O)

    T = eng.temperature()
    cnt = eng.counters()
    D.close()
    if rank != 0:
        return
    ns_day = value / n_sites * 86400 * DT_FS * 1e-6 if ws == 1 else value / ws / n_sites * 86400 * DT_FS * 1e-6
    line = {
        "metric": "atom-steps/s", "value": value, "unit": "atom-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 pair/multipole/bonded terms; f64 constraint iterations, thermostat, kinetic sums, positions",
        "data": "synthetic (seeded droplet; no dataset)",
        "config": {"workload": ("small droplet 6,000 waters + 60 surfactants, 16x16x8 cells" if args.small else
                                "single system, 20,000 SPC/E waters + 200 29-site trisiloxane surfactants on 4-layer "
                                "graphite, 24x24x12 cells (288x288x144 A), reference force field"),
                   "n_sites": n_sites, "precision": "mixed", "rebuild_interval": 10,
                   "l2": "flushed between timed steps (256 MB write outside the timed intervals)",
                   "pair_field_shape": {"tile": tile, "ctas_per_sm": ctas, "ctas_per_sm_max": ctas_max,
                                        "how": "sesp_autotune before the timed steps"},
                   "constraint_shape": {"surf_warps_per_cta": surf_warps, "surfactants_per_warp": mols_per_warp,
                                        "how": "sesp_autotune"},
                   "parallelism": f"replicas x{ws}"},
        "ns_per_day": ns_day,
        "plain_fp64": {"value": plain_value, "unit": "atom-steps/s", "steps": args.plain_steps,
                       "ms_per_step": float(p_ms.mean())},
        "mixed_vs_plain_speedup": value / ws / plain_value,
        "mixed_fp32_constraints": fp32c,
        "mixed_force_rms_rel_error": ferr,
        "batched": batched,
        "served": served,
        "roofline": {"bound": "fp32", "kernel": "k_near<mixed> (pair + fused local-expansion force)",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": (achieved / peak) if (achieved and peak) else None, "traffic": traffic,
                     "peak_source": "nominal FP32 FMA rate: SMs x 128 lanes x 2 x max SM clock (no FP32 figure "
                                    "in MEASURED_PEAKS.json)",
                     "algorithmic_flops_per_launch": flops, "pairs_coulomb": ncoul, "pairs_lj": nlj,
                     "near_ms_per_launch": near_ms},
        "kernel_ms": {"near": kt[0], "site_and_intra": kt[4], "move_a": kt[2], "move_b": kt[3],
                      "rebuild_sort": kt[5], "far_build": kt[6]},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
        "temperature": T,
        "shake_failures": cnt[0],
    }
    print(json.dumps(line))


def fp32_nominal_tflops(device):
    try:
        out = subprocess.run(["nvidia-smi", f"--id={device}", "--query-gpu=clocks.max.sm", "--format=csv,noheader,nounits"],
                             capture_output=True, text=True, timeout=20).stdout.strip()
        mhz = float(out.splitlines()[0])
    except Exception:
        mhz = 2070.0
    sms = 152
    try:
        import torch
        sms = torch.cuda.get_device_properties(device).multi_processor_count
    except Exception:
        pass
    return sms * 128 * 2 * mhz * 1e6 / 1e12


def oracle_step_rate(s, O):
    """The oracle (the FP64 C restatement of the reference, OpenMP over cells)
    on the same system: after the start-up force call, one rebuild step
    (kb = 99110) and one ordinary step (kb = 99111) are timed and combined on
    the reference's schedule of one rebuild every 10 steps
    (src/mybox.f90:24,140)."""
    o = O.Oracle(s)
    o.force(True)
    o.init_accel()
    t0 = time.perf_counter()
    o.step(99110)
    t_r = time.perf_counter() - t0
    t0 = time.perf_counter()
    o.step(99111)
    t_p = time.perf_counter() - t0
    per_step = (t_r + 9.0 * t_p) / 10.0
    return s.n_sites / per_step, per_step, t_r, t_p, o


def cpu_baseline(s, O):
    value, per_step, t_r, t_p, _ = oracle_step_rate(s, O)
    return {"value": value, "unit": "atom-steps/s", "cores": O.threads(), "kind": "port",
            "sample": f"1 rebuild step ({t_r:.2f} s) + 1 ordinary step ({t_p:.2f} s) of the full workload on "
                      f"{O.threads()} OpenMP threads, combined as (rebuild + 9 ordinary) / 10"}


def run_reference(args, ws, rank, local, budget_s=90.0):
    """The reference's own algorithm on the host cores: the oracle port on all
    OpenMP threads (the Fortran + MPI reference cannot be built here: no
    Fortran compiler or MPI).  K steps are timed when they fit the time
    budget, else the rebuild-weighted two-step sample stands for them."""
    if rank != 0:
        return
    import oracle as O
    s = make_system(args.small)
    value, per_step, t_r, t_p, o = oracle_step_rate(s, O)
    steps = max(1, args.steps)
    if steps * per_step <= budget_s:
        kb0 = 99112
        for k in range(min(args.warmup, 1)):
            o.step(kb0)
            kb0 += 1
        t0 = time.perf_counter()
        o.run(kb0, steps)
        elapsed = time.perf_counter() - t0
        value, per_step = s.n_sites * steps / elapsed, elapsed / steps
        sample = f"{steps} consecutive steps (rebuild every 10th) on {O.threads()} OpenMP threads"
        done = steps
    else:
        sample = (f"1 rebuild step ({t_r:.2f} s) + 1 ordinary step ({t_p:.2f} s) on {O.threads()} OpenMP threads, "
                  f"combined as (rebuild + 9 ordinary) / 10 ({steps} steps would exceed {budget_s:.0f} s)")
        done = 2
    line = {"metric": "atom-steps/s", "value": value, "unit": "atom-steps/s", "n_gpus": 0, "steps": done,
            "warmup": 1, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded droplet)", "impl": "reference",
            "config": {"workload": "same system as the GPU arm" + (" (small)" if args.small else ""),
                       "n_sites": s.n_sites},
            "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": O.threads(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    ws, rank, local = dist_info()
    if args.impl == "reference":
        run_reference(args, ws, rank, local)
    else:
        run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()

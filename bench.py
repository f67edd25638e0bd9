#!/usr/bin/env python3
"""Benchmark: LLG steps/s at 1.2M tets, FP32-body + FP64-refinement path vs plain FP64 GPU path.

Workload (the film configuration): permalloy film 400 x 400 x 10 nm on a 2 nm grid
(200 x 200 x 5 cells x 6 tetrahedra = 1,200,000 tets, 242,406 nodes, 168,000 boundary
triangles), Ms = 8e5 A/m, Ae = 1.3e-11 J/m, K = 0, alpha = 0.02; initial m = seeded
uniform random unit vectors smoothed by 3 Jacobi passes over the node graph; zero applied
field; fixed dt = 5e-14 s; BiCG tolerance 1e-6 (max 700 iterations); FMM demag (P = 9).
A step is one accepted time step of the reference loop: base_projection, element
integrals, solve, node update, demag of m and of v, energies, evolution
(src/time_integration.cpp:193-231). Synthetic data; no files are read.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

One JSON line on stdout (rank 0). For N > 1 every rank runs an independent replica on its
own GPU (the path does not shard); value is the sum over ranks of steps/s (max-over-ranks
time).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MS, AE, ALPHA, DT = 8.0e5, 1.3e-11, 0.02, 5e-14
TOL, MAXITER = 1e-6, 700
SEED = 12345
METRIC = "LLG steps/s @1.2M tets: learned-guess FP32+refine vs plain FP64 GPU, equal tol"


def film_mesh():
    import feellgood_gb300 as fg
    return fg.cuboid(200, 200, 5, 400.0, 400.0, 10.0, 1e-9, MS)


def initial_state(mesh, seed=SEED, passes=3):
    """Uniform unit vectors (seeded) smoothed by Jacobi passes m_i <- normalize(m_i + sum_j m_j)."""
    rng = np.random.default_rng(seed)
    n = len(mesh["xyz"])
    m = rng.normal(size=(n, 3))
    m /= np.linalg.norm(m, axis=1, keepdims=True)
    t = mesh["tets"]
    pairs = np.concatenate([t[:, [a, b]] for a in range(4) for b in range(a + 1, 4)])
    pairs = np.unique(np.sort(pairs, axis=1), axis=0)
    for _ in range(passes):
        acc = m.copy()
        np.add.at(acc, pairs[:, 0], m[pairs[:, 1]])
        np.add.at(acc, pairs[:, 1], m[pairs[:, 0]])
        m = acc / np.linalg.norm(acc, axis=1, keepdims=True)
    return m


def regions():
    return [dict(Ae=1e-11, Ms=795774.7, alpha=0.5), dict(Ae=AE, Ms=MS, alpha=ALPHA)]


def prefactor(dt, dtmax):
    tt = dt / (100.0 * dtmax)
    return 1.0 + tt * abs(math.log(tt))


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = str(gpu_index)
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", self.gpu], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return rank, world, dist
    return 0, 1, None


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_steps(ctx, n, H, dtmax, angles):
    """n accepted steps; returns (device ms per step list, reports)."""
    ms, reps = [], []
    for k in range(n):
        rep = ctx.step(DT, prefactor(DT, dtmax), H, angles())
        if rep["status"] != 0:
            raise RuntimeError(f"solver failed: {rep}")
        ctx.compute_all(H)
        t = ctx.timings()
        ms.append(float(np.sum(t)))
        reps.append(rep)
    return ms, reps


def cpu_leg(mesh, u0, steps, warmup, budget_s=25.0, levels=5):
    """The oracle (CPU restatement of the reference path, FP64, OpenMP over all host cores):
    full steps (base_projection, element integrals, 2x2-block CSR assembly, bicg_dir, update,
    demag of m and v with the CPU FMM at the reference's tree depth, energies, evolution)."""
    from oracle import fgo
    o = fgo.Oracle({k: mesh[k] for k in ("xyz", "tets", "tet_reg", "tris", "tri_reg", "dMs")},
                   [fgo.make_region(), fgo.make_region(A=AE, Ms=MS, alpha=ALPHA)])
    cores = fgo.lib().fgo_max_threads()
    o.set_solver(TOL, MAXITER)
    o.set_demag(levels)
    o.set_state(u0)
    H = np.zeros(3)
    o.compute_all(H)  # also builds the FMM tree (set-up, untimed)
    fgo.srand(SEED)
    times = []
    t_start = time.perf_counter()
    for k in range(warmup + steps):
        t0 = time.perf_counter()
        o.base_projection(fgo.draw_angle())
        r = o.step(DT, prefactor(DT, DT), H)
        if r["fail"]:
            raise RuntimeError(f"oracle solve failed: {r}")
        o.compute_all(H)
        t1 = time.perf_counter()
        if k >= warmup:
            times.append(t1 - t0)
        if time.perf_counter() - t_start > budget_s and times:
            break
    per = float(np.mean(times))
    return {"value": 1.0 / per, "unit": "steps/s", "cores": cores, "kind": "port",
            "sample": f"{len(times)} full oracle step(s) of the same film workload (1.2M tets) after {warmup} "
                      f"warm-up: element integrals + 2x2-block CSR assembly + bicg_dir + update + demag x2 "
                      f"(CPU FP64 FMM, P=9, 32^3-leaf tree as ScalFMM in the reference) + energies"}


def reference_arm(args):
    rank, world, dist = dist_setup(args.gpus)
    if rank != 0:
        return
    import feellgood_gb300 as fg  # mesh set-up only (host C++), the compute is the oracle's
    mesh = film_mesh()
    u0 = initial_state(mesh)
    steps = max(1, min(args.steps, 3))
    c = cpu_leg(mesh, u0, steps, 1, budget_s=120.0)
    line = {"metric": METRIC, "value": c["value"], "unit": "steps/s", "n_gpus": args.gpus, "steps": steps,
            "warmup": 1, "ms_per_step": 1e3 / c["value"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "film 400x400x10 nm, 2 nm grid, 1.2M tets, alpha 0.02, dt 5e-14, tol 1e-6",
                       "global_batch": 1, "seq_len": 0, "parallelism": "replicas"},
            "impl": "reference", "cpu_baseline": c,
            "e2e": {"value": c["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=5)
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        reference_arm(args)
        return
    rank, world, dist = dist_setup(args.gpus)
    import __graft_entry__
    __graft_entry__.build_product()
    import feellgood_gb300 as fg

    mesh = film_mesh()
    u0 = initial_state(mesh)
    H = np.zeros(3)
    fg.rng_seed(SEED)
    angles = fg.rng_angle

    # FP32 body + FP64 refinement (headline)
    ctx = fg.Context(mesh, regions(), tol=TOL, max_iter=MAXITER, precision=fg.FG_PREC_FP32_REFINE,
                     demag=fg.FG_DEMAG_FMM, profile=0)
    ctx.set_state(u0)
    ctx.compute_all(H)  # initial compute_all of the reference loop (time_integration.cpp:140)
    run_steps(ctx, args.warmup, H, DT, angles)
    launches0 = ctx.counters()[0]
    clk = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")) if world > 1 else 0)
    clk.start()
    t_wall0 = time.perf_counter()
    ms, reps = run_steps(ctx, args.steps, H, DT, angles)
    t_wall = time.perf_counter() - t_wall0
    clocks = clk.stop()
    launches = (ctx.counters()[0] - launches0) // args.steps
    dev_s = max_over_ranks(dist, float(np.sum(ms)) / 1e3)
    value = world * args.steps / dev_s
    iters = [r["iters"] for r in reps]
    refs = [r["refinements"] for r in reps]

    # stage breakdown (separate, profiled evaluations; not part of the timed region)
    prof = fg.Context(mesh, regions(), tol=TOL, max_iter=MAXITER, precision=fg.FG_PREC_FP32_REFINE,
                      demag=fg.FG_DEMAG_FMM, profile=1)
    st = ctx.get_state(0)
    prof.set_state(st["u"], st["v"], st["phi"], st["phiv"])
    prof.demag(0)
    fmm_stage = prof.fmm_timings()
    cnt = prof.counters()
    prof.step(DT, prefactor(DT, DT), H, 0.3)
    phase = prof.timings()
    prof.close()

    # end to end through the C ABI with host buffers: state in, step, compute_all, state out
    nn = len(mesh["xyz"])
    st = ctx.get_state(0)
    h_u, h_v, h_phi, h_phiv = st["u"].copy(), st["v"].copy(), st["phi"].copy(), st["phiv"].copy()
    e2e_t = []
    for k in range(args.e2e_steps + 1):
        t0 = time.perf_counter()
        ctx.set_state(h_u, h_v, h_phi, h_phiv)
        ctx.step(DT, prefactor(DT, DT), H, angles())
        ctx.compute_all(H)
        out = ctx.get_state(0)
        h_u, h_v, h_phi, h_phiv = out["u"], out["v"], out["phi"], out["phiv"]
        if k:
            e2e_t.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(dist, float(np.sum(e2e_t)))
    e2e_value = world * len(e2e_t) / e2e_s
    state_bytes = nn * 8 * 8

    # plain FP64 GPU path, same workload and tolerance
    plain_value = None
    plain_iters = None
    if args.plain_steps > 0:
        cp = fg.Context(mesh, regions(), tol=TOL, max_iter=MAXITER, precision=fg.FG_PREC_FP64, demag=fg.FG_DEMAG_FMM)
        cp.set_state(u0)
        cp.compute_all(H)
        fg.rng_seed(SEED)
        run_steps(cp, 1, H, DT, angles)
        pms, preps = run_steps(cp, args.plain_steps, H, DT, angles)
        plain_value = args.plain_steps / (float(np.sum(pms)) / 1e3)
        plain_iters = float(np.mean([r["iters"] for r in preps]))
        pu = cp.get_state(0)["u"]
        cp.close()

    # roofline of the dominant kernel of the step
    ms_step = float(np.mean(ms))
    L, n_m2l, n_p2p = cnt[1], cnt[2], cnt[3]
    stage_names = ["p2m", "m2m", "m2l", "l2l", "l2p_p2p"]
    dom = int(np.argmax(fmm_stage))
    share = 2 * fmm_stage[dom] / ms_step
    roof = None
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    if stage_names[dom] == "m2l":
        flops = 2.0 * 100 * 100 * n_m2l
        ach = flops / (fmm_stage[dom] * 1e-3) / 1e12
        pk = peaks.get("bf16_tflops", 1900.0)
        roof = {"kernel": "k_translate (M2L, FP32 CUDA cores)", "bound": "tensor", "achieved": ach, "peak": pk,
                "unit": "TFLOP/s", "frac": ach / pk, "traffic": None,
                "note": "M2L is a batched 100x100 GEMM run on FP32 CUDA cores; peak is the measured bf16 tensor peak"}
    else:
        # near field: pairs; bytes = leaf-local source reads (16 B per source per target leaf)
        ach_pairs = n_p2p / (fmm_stage[dom] * 1e-3)
        roof = {"kernel": f"{stage_names[dom]}", "bound": "hbm", "achieved": None, "peak": peaks.get("hbm_gbs"),
                "unit": "GB/s", "frac": None, "traffic": None, "pairs_per_s": ach_pairs}
    roof["share_of_step"] = share
    roof["peak_source"] = "measured" if peaks else "fallback"

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_leg(mesh, u0, 1, 1)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_s * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded smoothed random film state)",
            "config": {"workload": "film 400x400x10 nm, 2 nm grid: 1,200,000 tets, 242,406 nodes; alpha 0.02; "
                                   "dt 5e-14; BiCG tol 1e-6; FMM P=9",
                       "global_batch": 1, "seq_len": 0, "parallelism": "replicas" if world > 1 else "single",
                       "guess": "previous-step v (learned guess not in this line)",
                       "l2": "working set per step > L2 (tets 163 MB + sources 107 MB + FMM operators 15 MB)"},
            "plain_fp64_steps_per_s": plain_value,
            "speedup_vs_plain_fp64": (value / world) / plain_value if plain_value else None,
            "iters_per_step": float(np.mean(iters)), "refinements_per_step": float(np.mean(refs)),
            "plain_iters_per_step": plain_iters,
            "phase_ms": {"elements": phase[0], "solve": phase[1], "demag_x2": float(2 * np.sum(fmm_stage))},
            "fmm": {"L": L, "m2l_pairs": n_m2l, "p2p_pairs": n_p2p,
                    "stage_ms": dict(zip(stage_names, [float(x) for x in fmm_stage]))},
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": state_bytes,
                    "d2h_bytes_per_step": state_bytes},
            "gpu_launches": int(launches),
            "clocks": clocks,
            "wall_s_timed": t_wall,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()


if __name__ == "__main__":
    main()

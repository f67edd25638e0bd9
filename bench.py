#!/usr/bin/env python3
"""Benchmark: LLG steps/s at 1.2M tets, learned-guess FP32-body + FP64-refinement path vs the
plain FP64 GPU path at the same BiCG tolerance.

Workload (the film configuration): permalloy film 400 x 400 x 10 nm on a 2 nm grid
(200 x 200 x 5 cells x 6 tetrahedra = 1,200,000 tets, 242,406 nodes, 168,000 boundary
triangles), Ms = 8e5 A/m, Ae = 1.3e-11 J/m, K = 0, alpha = 0.02; initial m = seeded
uniform random unit vectors smoothed by 3 Jacobi passes over the node graph; zero applied
field; fixed dt = 5e-14 s; BiCG tolerance 1e-6 (max 700 iterations); FMM demag (P = 9).
A step is one accepted time step of the reference loop: base_projection, element
integrals, solve, node update, demag of m and of v, energies, evolution
(src/time_integration.cpp:193-231). The learned initial guess is trained online on the
solver's own solutions for --train-steps untimed solves first and keeps training (timed)
afterwards. Synthetic data; no files are read.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
  python bench.py --workload batch64     # 64 independent cubes, batched (its own line)
  python bench.py --workload wire        # nanowire domain wall, learned guess (its own line)
  python bench.py --workload platelet    # 3.84M-tet vortex platelet, learned guess at scale
  python bench.py --workload spin        # the film with the spin-accumulation coupling

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


def replicas_value(dist, world, steps, seconds):
    """Whole-job throughput of N independent replicas: all ranks' steps over the slowest rank's time."""
    slowest = max_over_ranks(dist, seconds)
    return world * steps / slowest, slowest


def run_steps(ctx, n, H, dtmax, angles):
    """n accepted steps (angles: a callable or a sequence); returns (per-step device ms of the
    phases [elements, solve, demag x2, energy + evolution, whole step], reports)."""
    ms, reps = [], []
    for k in range(n):
        ang = angles() if callable(angles) else angles[k]
        rep = ctx.step(DT, prefactor(DT, dtmax), H, ang)
        if rep["status"] != 0:
            raise RuntimeError(f"solver failed: {rep}")
        ctx.compute_all(H)
        ms.append([float(x) for x in ctx.timings()])
        reps.append(rep)
    return np.array(ms).reshape(-1, 5), reps


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




def ncu_traffic(kernel):
    """DRAM bytes (read + write) of one launch of `kernel` on the film workload, from the ncu
    capture summarised in profiles/<kernel>_film_1.2M.md (None if there is no capture)."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_film_1.2M.md")
    scale = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9}
    try:
        tot, seen = 0.0, 0
        for line in open(path):
            for key in ("dram__bytes_read.sum", "dram__bytes_write.sum"):
                if f"`{key}`" in line:
                    val, unit = line.split("|")[2].split()
                    tot += float(val.replace(",", "")) * scale[unit]
                    seen += 1
        return tot if seen == 2 else None
    except (OSError, ValueError, KeyError):
        return None


# FP32 lane operations of the near field per (target, source) pair, both charge sets (count
# of the f32x2 pass: 3 subtractions, 1 multiply and 2 fused multiply-adds for r^2, one fused
# multiply-add per set; packed instructions do two of them), and SFU reciprocal square
# roots per pair (shared by the sets)
P2P_FMA_LANE_OPS_PER_PAIR = 8
P2P_RSQRT_PER_PAIR = 1


def compute_roofs(compute, sm_mhz):
    """Measured compute roofs (fg_measure_peaks, per SM and clock) at the sampled SM clock."""
    if not compute:
        return None
    hz = (sm_mhz or compute["sm_mhz"]) * 1e6
    n = compute["n_sm"]
    return {"fma_lane_ops_per_s": compute["ffma_per_clk_sm"] * n * hz,
            "rsqrt_per_s": compute["rsqrt_per_clk_sm"] * n * hz,
            "tf32_tflops": compute["tf32_n128_flops_per_clk_sm"] * n * hz / 1e12,
            "sm_mhz": hz / 1e6, "per_clk_per_sm": {k: compute[k] for k in (
                "ffma_per_clk_sm", "ffma2_per_clk_sm", "rsqrt_per_clk_sm", "tf32_n128_flops_per_clk_sm")}}


def roofline_of(kernel, ms, units, peaks, roofs=None):
    """Roofline entry of one kernel from its live per-launch device time (CUDA events)."""
    hbm = peaks.get("hbm_gbs", 6800.0)
    src = "measured" if peaks else "fallback"
    if kernel.startswith("k_m2l_tc"):
        # useful flops: 2 x 100 x 100 per (cell, source cell) pair and charge set; the roof is
        # the measured tcgen05 kind::tf32 rate at the sampled clock (the kernel's instruction)
        fl = 2.0 * 100 * 100 * units["m2l_pairs"]
        ach = fl / (ms * 1e-3) / 1e12
        peak = roofs["tf32_tflops"] if roofs else peaks.get("bf16_tflops", 1900.0) / 2
        # issued: three TF32 products per useful one, M padded 100 -> 128 rows, K 100 -> 104
        issued = ach * 3 * 1.28 * 1.04
        return {"kernel": kernel, "bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                "frac": ach / peak, "issued_tflops": issued, "issued_frac": issued / peak, "traffic": None,
                "algorithmic_per_launch": fl,
                "peak_source": "measured tcgen05.mma kind::tf32 throughput (fg_measure_peaks) at the sampled SM clock"
                if roofs else "fallback: half the measured BF16 rate"}
    by = units["bytes"]
    ach = by / (ms * 1e-3) / 1e9
    e = {"kernel": kernel, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
         "traffic": units.get("traffic"), "algorithmic_per_launch": by, "peak_source": src}
    return e


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="film", choices=["film", "batch64", "wire", "platelet", "spin"])
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--fp64-batch-steps", type=int, default=10,
                    help="batch64: timed steps of the FP64 batch (at most --steps)")
    ap.add_argument("--train-steps", type=int, default=None,
                    help="untimed solves that train the learned guess (default 40; 0 with --quick)")
    ap.add_argument("--train-every", type=int, default=4,
                    help="after those, the guess keeps training (timed) on every n-th solve")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--compare-steps", type=int, default=0,
                    help="wire / platelet: steps of the plain FP64 comparison run (default: all timed steps)")
    ap.add_argument("--drift", type=int, default=0,
                    help="accuracy study: N steps of the precision paths and of the plain FP64 path from the same "
                         "state and angles on --workload film, wire or platelet (JSON lines of max |dm|)")
    ap.add_argument("--drift-tol", default="1e-6",
                    help="accuracy study: comma-separated BiCG tolerances, one JSON line each")
    ap.add_argument("--drift-split", action="store_true",
                    help="accuracy study: add the FP32 + refinement path with a full FP64 demag and with a full "
                         "FP32 demag every step (what the solver and the demag each contribute)")
    ap.add_argument("--quick", action="store_true",
                    help="timed steps only (no training, comparisons, end-to-end or CPU legs): for profiling")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.quick:
        args.plain_steps, args.e2e_steps, args.no_cpu = 0, 0, True
    if args.train_steps is None:
        args.train_steps = 0 if args.quick else 40
    if args.impl == "reference":
        reference_arm(args)
        return
    if args.drift > 0:
        drift_study(args)
        return
    if args.workload == "batch64":
        bench_batch(args)
        return
    if args.workload in ("wire", "platelet"):
        bench_learned_workload(args)
        return
    if args.workload == "spin":
        bench_spin(args)
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
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    compute = fg.measure_peaks()  # measured FP32 / SFU / TF32 roofs, per SM and clock

    # learned guess + FP32 body + FP64 refinement (headline). The guess is trained online
    # on the solver's own solutions; those solves are not timed.
    ctx = fg.Context(mesh, regions(), tol=TOL, max_iter=MAXITER, precision=fg.FG_PREC_FP32_REFINE,
                     demag=fg.FG_DEMAG_FMM, learned_guess=1, mlp_train_every=args.train_every, profile=1)
    ctx.set_state(u0)
    ctx.compute_all(H)  # initial compute_all of the reference loop (time_integration.cpp:140)
    train_ms, _ = run_steps(ctx, args.train_steps, H, DT, angles)
    run_steps(ctx, args.warmup, H, DT, angles)
    start = ctx.get_state(0)
    ctx.fmm_timings()  # resets the stage accumulators: the stage times below are the timed region's
    step_angles = [angles() for _ in range(args.steps)]
    launches0 = ctx.counters()[0]
    clk = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")) if world > 1 else 0)
    clk.start()
    if dist is not None:
        dist.barrier()
    t_wall0 = time.perf_counter()
    ms, reps = run_steps(ctx, args.steps, H, DT, step_angles)
    t_wall = time.perf_counter() - t_wall0
    clocks = clk.stop()
    fmm_stage = ctx.fmm_timings()
    cnt = ctx.counters()
    lanes_per_row, solver_blocks = ctx.solver_lanes_per_row(), ctx.solver_blocks()
    launches = (cnt[0] - launches0) // args.steps
    value, dev_s = replicas_value(dist, world, args.steps, float(ms[:, 4].sum()) / 1e3)
    iters = [r["iters"] for r in reps]
    refs = [r["refinements"] for r in reps]
    acc = [r["guess_accepted"] for r in reps]
    r0_ratio = [r["res0"] / r["res0_fallback"] for r in reps if r["res0_fallback"] > 0]

    # end to end through the C ABI with pinned host buffers: state in, step, compute_all,
    # state out (into the same buffers)
    nn = len(mesh["xyz"])
    host = {"u": fg.pinned_empty((nn, 3)), "v": fg.pinned_empty((nn, 3)), "phi": fg.pinned_empty(nn),
            "phiv": fg.pinned_empty(nn)}
    ctx.get_state(0, out=host)
    e2e_t = []
    for k in range(args.e2e_steps + 1):
        t0 = time.perf_counter()
        ctx.set_state(host["u"], host["v"], host["phi"], host["phiv"])
        ctx.step(DT, prefactor(DT, DT), H, angles())
        ctx.compute_all(H)
        ctx.get_state(0, out=host)
        if k:
            e2e_t.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(dist, float(np.sum(e2e_t))) if e2e_t else None
    e2e_value = world * len(e2e_t) / e2e_s if e2e_t else None
    state_bytes = nn * 8 * 8
    ctx.close()

    # the same steps (state and angles) with the previous-step guess: what the learned guess gains
    prev_value = prev_iters = prev_phase = None
    cp = None if args.quick else fg.Context(mesh, regions(), tol=TOL, max_iter=MAXITER, precision=fg.FG_PREC_FP32_REFINE,
                    demag=fg.FG_DEMAG_FMM)
    if cp is not None:
        cp.set_state(start["u"], start["v"], start["phi"], start["phiv"])
        pms, preps = run_steps(cp, args.steps, H, DT, step_angles)
        prev_value = args.steps / (float(pms[:, 4].sum()) / 1e3)
        prev_iters = float(np.mean([r["iters"] for r in preps]))
        prev_phase = dict(zip(["elements", "solve", "demag_x2", "energy_evolution", "step"],
                              [float(x) for x in pms.mean(axis=0)]))
        cp.close()

    # plain FP64 GPU path, same state, angles and tolerance
    plain_value = plain_iters = plain_detail = None
    if args.plain_steps > 0:
        cp = fg.Context(mesh, regions(), tol=TOL, max_iter=MAXITER, precision=fg.FG_PREC_FP64, demag=fg.FG_DEMAG_FMM,
                        profile=1)
        cp.set_state(start["u"], start["v"], start["phi"], start["phiv"])
        n = min(args.plain_steps, args.steps)
        pms, preps = run_steps(cp, n, H, DT, step_angles)
        plain_value = n / (float(pms[:, 4].sum()) / 1e3)
        plain_iters = float(np.mean([r["iters"] for r in preps]))
        pc = cp.counters()
        plain_detail = {"phase_ms": dict(zip(["elements", "solve", "demag_x2", "energy_evolution", "step"],
                                             [float(x) for x in pms.mean(axis=0)])),
                        "fmm": {"L": int(pc[1]), "m2l_pairs": float(pc[2]), "p2p_pairs": float(pc[3]),
                                "stage_ms": dict(zip(["p2m", "m2m", "m2l", "l2l", "l2p_p2p"],
                                                     [float(x) for x in cp.fmm_timings()]))}}
        cp.close()

    # roofline of the dominant kernel: per-launch device times from CUDA events in the timed region
    ph = ms.mean(axis=0)
    L, n_m2l, n_p2p = int(cnt[1]), float(cnt[2]), float(cnt[3])
    stage_names = ["p2m", "m2m", "m2l", "l2l", "l2p_p2p"]
    nsrc = 5 * 1200000 + 4 * 168000
    kernels = {
        # per step: (device ms per launch, launches per step, algorithmic units). One FMM
        # evaluation per step covers both charge sets (m and v): the near field reads each
        # source's (x, y, z, q_m) and q_v once (20 B) and each target's coordinates and node
        # index once and writes two potentials (36 B); M2L does both sets' products.
        "k_l2p_p2p (near field + L2P)": (fmm_stage[4], 1, {"bytes": 20.0 * nsrc + 36.0 * nn}),
        "k_m2l_tc (M2L, tcgen05 3xTF32)": (fmm_stage[2], 1, {"m2l_pairs": 2 * n_m2l}),
        "k_tet_ds + k_node64 (elements)": (ph[0], 1, {"bytes": 1200000 * (4 * 4 + 12 * 8 + 8 + 4 + 4 * 40 + 4 * 32) +
                                                       nn * (3 * 8 + 2 * 8 + 8 * 8)}),
    }
    dom = max(kernels, key=lambda k: kernels[k][0] * kernels[k][1])
    kernels[dom][2]["traffic"] = ncu_traffic(dom.split()[0])
    roofs = compute_roofs(compute, clocks.get("sm_mhz"))
    roof = roofline_of(dom, kernels[dom][0], kernels[dom][2], peaks, roofs)
    roof["traffic_source"] = f"profiles/{dom.split()[0]}_film_1.2M.md (one ncu launch)"
    roof["share_of_step"] = kernels[dom][0] * kernels[dom][1] / float(ms[:, 4].mean())
    if dom.startswith("k_l2p_p2p"):
        # the near field's binding roofs are its compute pipes, measured by fg_measure_peaks:
        # one SFU reciprocal square root and 8 FP32 lane operations per (target, source) pair
        pairs_s = n_p2p / (fmm_stage[4] * 1e-3)
        roof["pairs_per_s"] = pairs_s
        roof["compute"] = {
            "sfu_rsqrt": {"achieved_per_s": pairs_s * P2P_RSQRT_PER_PAIR, "peak_per_s": roofs["rsqrt_per_s"],
                          "frac": pairs_s * P2P_RSQRT_PER_PAIR / roofs["rsqrt_per_s"]},
            "fp32_fma_pipe": {"achieved_lane_ops_per_s": pairs_s * P2P_FMA_LANE_OPS_PER_PAIR,
                              "peak_lane_ops_per_s": roofs["fma_lane_ops_per_s"],
                              "frac": pairs_s * P2P_FMA_LANE_OPS_PER_PAIR / roofs["fma_lane_ops_per_s"]},
            "peak_source": "fg_measure_peaks microbenchmarks (per SM and clock) at the sampled SM clock",
            "sm_mhz": roofs["sm_mhz"]}
    m2l_roof = roofline_of("k_m2l_tc (M2L, tcgen05 3xTF32)", fmm_stage[2], {"m2l_pairs": 2 * n_m2l}, peaks, roofs)

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
                                   "dt 5e-14; BiCG tol 1e-6; FMM P=9; learned guess trained online for "
                                   f"{args.train_steps} untimed solves, then on every {args.train_every}th",
                       "global_batch": 1, "seq_len": 0, "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (tets 163 MB + sources 107 MB + FMM operators 15 MB per step)"},
            "plain_fp64_steps_per_s": plain_value,
            "speedup_vs_plain_fp64": (value / world) / plain_value if plain_value else None,
            "prev_guess_fp32_refine_steps_per_s": prev_value,
            "iters_per_step": float(np.mean(iters)), "refinements_per_step": float(np.mean(refs)),
            "solver_lanes_per_row": lanes_per_row, "solver_blocks": solver_blocks,
            "prev_guess_iters_per_step": prev_iters, "prev_guess_phase_ms": prev_phase, "plain_iters_per_step": plain_iters,
            "plain_fp64_detail": plain_detail,
            "learned_guess": {"accepted_frac": float(np.mean(acc)),
                              "res0_over_fallback_median": float(np.median(r0_ratio)) if r0_ratio else None,
                              "train_solves": args.train_steps},
            "phase_ms": dict(zip(["elements", "solve", "demag_x2", "energy_evolution", "step"],
                                 [float(x) for x in ph])),
            "fmm": {"L": L, "m2l_pairs": n_m2l, "p2p_pairs": n_p2p,
                    "stage_ms": dict(zip(stage_names, [float(x) for x in fmm_stage]))},
            "roofline": roof,
            "m2l_roofline": m2l_roof,
            "measured_compute_roofs": roofs,
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


def drift_study(args):
    """Trajectory accuracy: N steps of the FP32 + refinement path (with and without the learned
    guess) and of a control (the plain FP64 path with the learned guess: the same arithmetic,
    another valid initial guess) against the plain FP64 path, from the same state with the same
    basis angles, at each BiCG tolerance of --drift-tol, all with the FMM at the same depth.
    Prints one JSON line per tolerance: max |dm| per pair at the checkpoints, iterations and
    refinements per step, device ms per step."""
    import __graft_entry__
    __graft_entry__.build_product()
    import feellgood_gb300 as fg
    if args.workload in ("wire", "platelet"):
        mesh, u0, H, alpha, _ = (wire_workload if args.workload == "wire" else platelet_workload)(fg)
        regs = [dict(Ae=1e-11, Ms=795774.7, alpha=0.5), dict(Ae=AE, Ms=MS, alpha=alpha)]
        desc = " ".join((wire_workload if args.workload == "wire" else platelet_workload).__doc__.split())
    else:
        mesh = film_mesh()
        u0, H, regs = initial_state(mesh), np.zeros(3), regions()
        desc = "film 400x400x10 nm, 2 nm grid, 1.2M tets, alpha 0.02, dt 5e-14, zero field, seeded smoothed random m"
    fg.rng_seed(SEED)
    angles = [fg.rng_angle() for _ in range(args.drift)]
    marks = sorted({k for k in (10, 100, 300, 1000, 2000, 5000) if k < args.drift} | {args.drift})
    variants = {"plain": dict(precision=fg.FG_PREC_FP64),
                "control_plain_learned": dict(precision=fg.FG_PREC_FP64, learned_guess=1),
                "fp32_refine": dict(precision=fg.FG_PREC_FP32_REFINE),
                "fp32_refine_learned": dict(precision=fg.FG_PREC_FP32_REFINE, learned_guess=1)}
    if args.drift_split:
        variants["fp32_refine_fp64_demag"] = dict(precision=fg.FG_PREC_FP32_REFINE, demag_increment=2)
        variants["fp32_refine_full_fp32_demag"] = dict(precision=fg.FG_PREC_FP32_REFINE, demag_increment=0)
    depth = None
    for tol in [float(t) for t in args.drift_tol.split(",")]:
        snaps, info = {}, {}
        for name, opts in variants.items():
            c = fg.Context(mesh, regs, tol=tol, max_iter=MAXITER, demag=fg.FG_DEMAG_FMM,
                           mlp_train_every=args.train_every, fmm_leaf=-depth if depth else 0, **opts)
            depth = depth or int(c.counters()[1])  # every run at the first run's FMM depth
            c.set_state(u0)
            c.compute_all(H)
            snaps[name], its, refs, ms = {}, [], [], []
            for k in range(args.drift):
                rep = c.step(DT, prefactor(DT, DT), H, angles[k])
                if rep["status"] != 0:
                    raise RuntimeError(f"{name}: solver failed at step {k}: {rep}")
                its.append(rep["iters"])
                refs.append(rep["refinements"])
                c.compute_all(H)
                ms.append(float(c.timings()[4]))
                if k + 1 in marks:
                    snaps[name][k + 1] = c.get_state(0)["u"].copy()
            info[name] = {"iters_per_step": float(np.mean(its)), "refinements_per_step": float(np.mean(refs)),
                          "device_ms_per_step_median": float(np.median(ms))}
            c.close()
        for name in variants:
            if name != "plain":
                info[name]["max_abs_dm_vs_plain"] = {
                    str(k): float(np.linalg.norm(snaps[name][k] - snaps["plain"][k], axis=1).max()) for k in marks}
        ctrl = info["control_plain_learned"]["max_abs_dm_vs_plain"][str(args.drift)]
        line = {"metric": f"max |dm| after {args.drift} steps vs the plain FP64 path, tol {tol:g} ({args.workload})",
                "value": info["fp32_refine_learned"]["max_abs_dm_vs_plain"][str(args.drift)], "unit": "1",
                "higher_is_better": False, "steps": args.drift, "tol": tol, "fmm_depth": depth,
                "control_spread": ctrl, "runs": info, "config": {"workload": desc}}
        print(json.dumps(line), flush=True)


def wire_workload(fg, seed=SEED):
    """Nanowire 40 x 40 x 1000 nm on a 2.5 nm grid (16 x 16 x 400 cells x 6 = 614,400 tets),
    head-to-head domain wall at z = 500 nm (m_z = tanh((500 - z) / 20 nm), transverse
    component through the wall) with a seeded +-0.02 transverse perturbation; 5 mT along +z;
    alpha 0.05."""
    mesh = fg.cuboid(16, 16, 400, 40.0, 40.0, 1000.0, 1e-9, MS)
    rng = np.random.default_rng(seed)
    z = mesh["xyz"][:, 2] / 1e-9
    mz = np.tanh((500.0 - z) / 20.0)
    u = np.stack([np.sqrt(np.clip(1 - mz * mz, 0, 1)), np.zeros_like(mz), mz], axis=1)
    u[:, :2] += rng.uniform(-0.02, 0.02, size=(len(z), 2))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    return mesh, u, np.array([0.0, 0.0, 0.005 / fg.MU0]), 0.05, 200


def platelet_workload(fg, seed=SEED):
    """Platelet 1000 x 1000 x 10 nm on a 2.5 nm grid (400 x 400 x 4 cells x 6 = 3,840,000 tets),
    in-plane vortex m = (-y, x, 0) / r about the centre with m_z = 1 within r < 10 nm, seeded
    Gaussian noise sigma 0.02; zero field; alpha 0.01."""
    mesh = fg.cuboid(400, 400, 4, 1000.0, 1000.0, 10.0, 1e-9, MS)
    rng = np.random.default_rng(seed)
    xy = mesh["xyz"][:, :2] / 1e-9 - 500.0
    r = np.hypot(xy[:, 0], xy[:, 1])
    u = np.zeros((len(r), 3))
    core = r < 10.0
    u[~core, 0] = -xy[~core, 1] / r[~core]
    u[~core, 1] = xy[~core, 0] / r[~core]
    u[core, 2] = 1.0
    u += rng.normal(0, 0.02, size=u.shape)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    return mesh, u, np.zeros(3), 0.01, 300


def bench_learned_workload(args):
    """The learned guess where it is meant to be used: trained online on the first steps of the
    run (200 for the wire, 300 for the platelet; not timed), then the timed steps (--steps:
    2000 and 5000 are the configurations' lengths), compared on the same state and angles with
    the previous-step guess (same precision) and with the plain FP64 path (its first
    --compare-steps steps, default all): steps/s, BiCG iterations per step and max |dm| of the
    learned-guess path against the plain FP64 path after those steps."""
    import __graft_entry__
    __graft_entry__.build_product()
    import feellgood_gb300 as fg
    mesh, u0, H, alpha, ntrain = (wire_workload if args.workload == "wire" else platelet_workload)(fg)
    regs = [dict(Ae=1e-11, Ms=795774.7, alpha=0.5), dict(Ae=AE, Ms=MS, alpha=alpha)]
    ncmp = min(args.steps, args.compare_steps or args.steps)
    fg.rng_seed(SEED)
    angles = fg.rng_angle
    ctx = fg.Context(mesh, regs, tol=TOL, max_iter=MAXITER, precision=fg.FG_PREC_FP32_REFINE, demag=fg.FG_DEMAG_FMM,
                     learned_guess=1, mlp_train_steps=ntrain, mlp_train_every=args.train_every, profile=1)
    depth = int(ctx.counters()[1])
    ctx.set_state(u0)
    ctx.compute_all(H)
    run_steps(ctx, ntrain + args.warmup, H, DT, angles)
    start = ctx.get_state(0)
    ctx.fmm_timings()
    step_angles = [angles() for _ in range(args.steps)]
    clk = ClockSampler(0)
    clk.start()
    ms1, reps1 = run_steps(ctx, ncmp, H, DT, step_angles[:ncmp])
    learned_cmp = ctx.get_state(0)
    ms2, reps2 = run_steps(ctx, args.steps - ncmp, H, DT, step_angles[ncmp:])
    clocks = clk.stop()
    ms = np.concatenate([ms1, ms2]) if len(ms2) else ms1
    reps = reps1 + reps2
    fmm_stage = ctx.fmm_timings()
    cnt = ctx.counters()
    learned = ctx.get_state(0)
    recenter_ms = None
    if args.workload == "wire":
        # Fem::recenter on the wire's state (threshold 0: it always translates), wall clock of
        # the call (average, nearest-node search and copy, synchronised); on a copy of the state
        rc = fg.Context(mesh, regs, tol=TOL, max_iter=MAXITER, precision=fg.FG_PREC_FP32_REFINE,
                        demag=fg.FG_DEMAG_FMM)
        rc.set_state(learned["u"], learned["v"], learned["phi"], learned["phiv"])
        rc.recenter("Z", 0.0)  # first call builds the nearest-node grid
        t0 = time.perf_counter()
        for _ in range(5):
            rc.recenter("Z", 0.0)
        recenter_ms = (time.perf_counter() - t0) / 5 * 1e3
        rc.close()
    ctx.close()
    out = {"learned": (args.steps / (ms[:, 4].sum() / 1e3), float(np.mean([r["iters"] for r in reps])),
                       float(np.mean([r["refinements"] for r in reps])))}
    acc = float(np.mean([r["guess_accepted"] for r in reps]))
    r0 = float(np.median([r["res0"] / r["res0_fallback"] for r in reps if r["res0_fallback"] > 0]))
    finals = {}
    for name, opts, n in (("previous_step_guess", dict(precision=fg.FG_PREC_FP32_REFINE), args.steps),
                          ("plain_fp64", dict(precision=fg.FG_PREC_FP64), ncmp)):
        c = fg.Context(mesh, regs, tol=TOL, max_iter=MAXITER, demag=fg.FG_DEMAG_FMM, fmm_leaf=-depth, **opts)
        c.set_state(start["u"], start["v"], start["phi"], start["phiv"])
        pms, preps = run_steps(c, n, H, DT, step_angles[:n])
        out[name] = (n / (pms[:, 4].sum() / 1e3), float(np.mean([r["iters"] for r in preps])),
                     float(np.mean([r["refinements"] for r in preps])))
        finals[name] = c.get_state(0)
        c.close()
    dm = np.linalg.norm(learned_cmp["u"] - finals["plain_fp64"]["u"], axis=1).max()
    ntets = len(mesh["tets"])
    line = {
        "metric": f"LLG steps/s, {args.workload} ({ntets} tets), learned guess + FP32 body + FP64 refinement",
        "value": out["learned"][0], "unit": "steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 / out["learned"][0], "higher_is_better": True, "dtype": "f32+f64",
        "data": "synthetic (seeded)",
        "config": {"workload": " ".join((wire_workload if args.workload == "wire" else platelet_workload).__doc__.split()),
                   "train_solves_untimed": ntrain, "dt": DT, "tol": TOL, "fmm_depth": depth},
        "iters_per_step": {k: v[1] for k, v in out.items()},
        "refinements_per_step": {k: v[2] for k, v in out.items()},
        "steps_per_s": {k: v[0] for k, v in out.items()},
        "learned_guess": {"accepted_frac": acc, "res0_over_fallback_median": r0},
        "speedup_vs_plain_fp64": out["learned"][0] / out["plain_fp64"][0],
        "speedup_vs_previous_step_guess": out["learned"][0] / out["previous_step_guess"][0],
        "max_abs_dm_vs_plain_fp64": {"after_steps": ncmp, "value": float(dm)},
        "fmm": {"L": int(cnt[1]), "m2l_pairs": float(cnt[2]), "p2p_pairs": float(cnt[3]),
                "stage_ms": dict(zip(["p2m", "m2m", "m2l", "l2l", "l2p_p2p"], [float(x) for x in fmm_stage]))},
        "clocks": clocks,
    }
    if recenter_ms is not None:
        line["recenter_ms_per_call"] = recenter_ms
    print(json.dumps(line), flush=True)


def bench_spin(args):
    """The film with the spin-accumulation coupling: current injected through the x = 400 nm
    face (jn = 1e3 A/m^2, polarisation along y; the spin field enters the next step's element
    integrals explicitly, and at the fixed dt = 5e-14 s a current of 1e5 A/m^2 made the
    velocity grow tenfold per step, while 1e3 keeps the run stable), the x = 0 face grounded
    (V = 0, s = 0);
    permalloy-like transport parameters (sigma 5e6 S/m, N0 1e47, P 0.5, l_sd 1 nm, l_sf 5 nm).
    FP32 body + FP64 refinement with the previous-step guess, with and without the coupling,
    same state and angles; the spin solve (FP32 BiCGSTAB body with FP64 refinement over
    3 x 242k unknowns) runs in every compute_all."""
    import __graft_entry__
    __graft_entry__.build_product()
    import feellgood_gb300 as fg
    mesh = film_mesh()
    x = mesh["xyz"][:, 0]
    reg = np.ones(len(mesh["tris"]), np.int32)
    tx = x[mesh["tris"]]
    reg[np.all(np.abs(tx - x.min()) < 1e-15, axis=1)] = 2
    reg[np.all(np.abs(tx - x.max()) < 1e-15, axis=1)] = 3
    mesh = dict(mesh, tri_reg=reg)
    sp = dict(sigma=5e6, dens_state=1e47, P=0.5, lsd=1e-9, lsf=5e-9)
    regs = [dict(Ae=1e-11, Ms=795774.7, alpha=0.5, **sp), dict(Ae=AE, Ms=MS, alpha=ALPHA, **sp)]
    bc = [dict(), dict(), dict(V=0.0, s=(0, 0, 0)), dict(jn=1e3, uP=(0, 1, 0))]
    u0 = initial_state(mesh)
    H = np.zeros(3)
    fg.rng_seed(SEED)
    angles = [fg.rng_angle() for _ in range(args.warmup + args.steps)]
    out = {}
    for name, spin in (("spin", 1), ("no_spin", 0)):
        c = fg.Context(mesh, regs, bc, tol=TOL, max_iter=MAXITER, precision=fg.FG_PREC_FP32_REFINE,
                       demag=fg.FG_DEMAG_FMM, spin_acc=spin)
        c.set_state(u0)
        c.compute_all(H)
        run_steps(c, args.warmup, H, DT, angles[:args.warmup])
        clk = ClockSampler(0)
        clk.start()
        if spin:  # the spin solve's own device time and iterations, step by step
            ms_l, reps = [], []
            spin_ms, spin_it = [], []
            for k in range(args.steps):
                m1, r1 = run_steps(c, 1, H, DT, angles[args.warmup + k:args.warmup + k + 1])
                ms_l.append(m1[0])
                reps += r1
                inf = c.spin_info()
                spin_ms.append(inf["ms"])
                spin_it.append(inf["iters"])
            ms = np.array(ms_l)
        else:
            ms, reps = run_steps(c, args.steps, H, DT, angles[args.warmup:])
        clocks = clk.stop()
        info = c.spin_info() if spin else {}
        out[name] = {"steps_per_s": args.steps / (ms[:, 4].sum() / 1e3), "ms_per_step": float(ms[:, 4].mean()),
                     "phase_ms": dict(zip(["elements", "solve", "demag_x2_and_spin", "energy_evolution", "step"],
                                          [float(v) for v in ms.mean(axis=0)])),
                     "iters_per_step": float(np.mean([r["iters"] for r in reps])), "clocks": clocks}
        if spin:
            out[name]["spin_solve"] = {"status": info["status"], "iters_per_solve": float(np.mean(spin_it)),
                                       "ms_per_solve": float(np.mean(spin_ms)),
                                       "us_per_iteration": 1e3 * float(np.sum(spin_ms)) / max(1, int(np.sum(spin_it))),
                                       "potential_cg_iters": info["V_iters"]}
            out[name]["max_abs_s"] = float(np.abs(c.get_spin()).max())
        c.close()
    line = {"metric": "LLG steps/s, film 1.2M tets with spin accumulation (FP32 body + FP64 refinement)",
            "value": out["spin"]["steps_per_s"], "unit": "steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": out["spin"]["ms_per_step"], "higher_is_better": True,
            "dtype": "f32+f64", "data": "synthetic (seeded smoothed random film state)",
            "config": {"workload": " ".join(bench_spin.__doc__.split())}, "detail": out,
            "clocks": out["spin"]["clocks"],
            "spin_cost_ms_per_step": out["spin"]["ms_per_step"] - out["no_spin"]["ms_per_step"]}
    print(json.dumps(line), flush=True)


BATCH_N, BATCH_H = 64, 2.5


def batch_workload(fg, seed=SEED):
    """64 cubes, edges uniform(20, 80) nm rounded to the 2.5 nm grid, seeded applied fields of
    magnitude uniform(0, 100) mT in random directions, uniform random initial m."""
    rng = np.random.default_rng(seed)
    n = np.clip(np.rint(rng.uniform(20, 80, BATCH_N) / BATCH_H), 1, None).astype(int)
    meshes = [fg.cuboid(int(k), int(k), int(k), k * BATCH_H, k * BATCH_H, k * BATCH_H, 1e-9, MS) for k in n]
    dirs = rng.normal(size=(BATCH_N, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    Hext = dirs * (rng.uniform(0, 0.1, BATCH_N) / fg.MU0)[:, None]
    us = []
    for m in meshes:
        u = rng.normal(size=(len(m["xyz"]), 3))
        us.append(u / np.linalg.norm(u, axis=1, keepdims=True))
    return n, meshes, Hext, us


def bench_batch(args):
    """Batched samples: steps*samples/s of one batch context (one persistent solve per step,
    graph-replayed) against looping single contexts over the samples."""
    rank, world, dist = dist_setup(args.gpus)
    import __graft_entry__
    __graft_entry__.build_product()
    import feellgood_gb300 as fg
    dt, alpha = 1e-14, 0.1
    regs = [dict(Ae=1e-11, Ms=795774.7, alpha=0.5), dict(Ae=AE, Ms=MS, alpha=alpha)]
    n, meshes, Hext, us = batch_workload(fg)
    ntets = int(sum(6 * k ** 3 for k in n))
    t_setup = time.perf_counter()
    b = fg.Context(meshes, regs, tol=TOL, max_iter=MAXITER, precision=fg.FG_PREC_FP32_REFINE,
                   demag=fg.FG_DEMAG_FMM)
    setup_s = time.perf_counter() - t_setup  # fg_batch_create: packing, forest of octrees, autotuning
    b.set_state(np.concatenate(us))
    b.batch_compute_all(Hext, energies=False)
    fg.rng_seed(SEED)
    ang = np.array([[fg.rng_angle() for _ in range(BATCH_N)] for _ in range(args.warmup + args.steps)])
    s, _ = b.batch_run(dt, prefactor(dt, dt), Hext, ang[:args.warmup])
    launches0 = b.counters()[0]
    clk = ClockSampler(0)
    clk.start()
    s, reps = b.batch_run(dt, prefactor(dt, dt), Hext, ang[args.warmup:])
    clocks = clk.stop()
    graph, dev_ms = b.batch_run_info()
    launches = (b.counters()[0] - launches0) // args.steps
    value = args.steps * BATCH_N / (dev_ms * 1e-3)
    fails = int(sum(r["fails"] for r in reps))
    iters = float(np.mean([r["iters"] / args.steps for r in reps]))
    E = b.batch_compute_all(Hext)
    tree = b.fmm_tree_info()
    b.close()
    # the octree built with the host's comparison sort instead, for its set-up time
    t_setup = time.perf_counter()
    bh = fg.Context(meshes, regs, tol=TOL, max_iter=MAXITER, precision=fg.FG_PREC_FP32_REFINE,
                    demag=fg.FG_DEMAG_FMM, fmm_tree_host=1)
    setup_host_s = time.perf_counter() - t_setup
    tree_host = bh.fmm_tree_info()
    bh.close()

    # the same batch with the plain FP64 solver and FP64 forest FMM (graph-replayed): the
    # like-for-like of looping the plain FP64 path over the samples
    b64 = fg.Context(meshes, regs, tol=TOL, max_iter=MAXITER, precision=fg.FG_PREC_FP64, demag=fg.FG_DEMAG_FMM)
    b64.set_state(np.concatenate(us))
    b64.batch_compute_all(Hext, energies=False)
    k64 = max(1, min(args.steps, args.fp64_batch_steps))
    b64.batch_run(dt, prefactor(dt, dt), Hext, ang[:1])
    s64, reps64 = b64.batch_run(dt, prefactor(dt, dt), Hext, ang[args.warmup:args.warmup + k64])
    ms64 = b64.batch_run_info()[1]
    fp64_batch = {"value": k64 * BATCH_N / (ms64 * 1e-3), "steps": k64, "ms_per_step": ms64 / k64,
                  "failed_solves": int(sum(r["fails"] for r in reps64)),
                  "iters_per_step_mean": float(np.mean([r["iters"] / k64 for r in reps64]))}
    b64.close()

    # the same batch with the learned guess (one network for all samples): trained on the first
    # steps by fg_batch_step, then graph-replayed with the network frozen
    bl = fg.Context(meshes, regs, tol=TOL, max_iter=MAXITER, precision=fg.FG_PREC_FP32_REFINE,
                    demag=fg.FG_DEMAG_FMM, learned_guess=1, mlp_train_steps=30, mlp_train_every=1)
    bl.set_state(np.concatenate(us))
    bl.batch_compute_all(Hext, energies=False)
    acc = []
    for k in range(30 + 2):
        _, rr = bl.batch_step(dt, prefactor(dt, dt), Hext, ang[k % len(ang)])
        if k >= 30:
            acc += [r["guess_accepted"] for r in rr]
        bl.batch_compute_all(Hext, energies=False)
    kl = max(1, min(args.steps, 100))
    bl.batch_run(dt, prefactor(dt, dt), Hext, ang[:1])
    sl, repl = bl.batch_run(dt, prefactor(dt, dt), Hext, ang[args.warmup:args.warmup + kl])
    msl = bl.batch_run_info()[1]
    learned_batch = {"value": kl * BATCH_N / (msl * 1e-3), "steps": kl, "ms_per_step": msl / kl,
                     "train_steps": 30, "accepted_frac_after_training": float(np.mean(acc)) if acc else None,
                     "failed_solves": int(sum(r["fails"] for r in repl)),
                     "iters_per_step_mean": float(np.mean([r["iters"] / kl for r in repl]))}
    bl.close()

    # looping single contexts over the samples, the same steps: plain FP64 and FP32 + refinement
    loops = {}
    for name, prec in (("plain_fp64", fg.FG_PREC_FP64), ("fp32_refine", fg.FG_PREC_FP32_REFINE)):
        tot = 0.0
        for g, m in enumerate(meshes):
            c = fg.Context(m, regs, tol=TOL, max_iter=MAXITER, precision=prec, demag=fg.FG_DEMAG_FMM)
            c.set_state(us[g])
            c.compute_all(Hext[g])
            c.step(dt, prefactor(dt, dt), Hext[g], ang[0, g])
            c.compute_all(Hext[g])
            k = min(2, args.steps)
            for j in range(k):
                r = c.step(dt, prefactor(dt, dt), Hext[g], ang[args.warmup + j, g])
                c.compute_all(Hext[g])
                tot += float(c.timings()[4]) / k
            c.close()
        loops[name] = BATCH_N / (tot * 1e-3)
    if rank == 0:
        line = {
            "metric": "LLG steps*samples/s, 64 independent cubes (batched, one persistent solve per step)",
            "value": value, "unit": "steps*samples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded)",
            "config": {"workload": f"64 cubes, edges uniform(20,80) nm on a 2.5 nm grid ({n.min()}..{n.max()} "
                                   f"cells per edge, {ntets} tets), alpha 0.1, dt 1e-14, random fields "
                                   "0-100 mT, FP32 + FP64 refinement, forest FMM",
                       "global_batch": BATCH_N, "seq_len": 0, "parallelism": "single"},
            "graph_replay": bool(graph), "failed_solves": fails, "iters_per_step_mean": iters,
            "loop_single_contexts_steps_samples_per_s": loops,
            "speedup_vs_loop_plain_fp64": value / loops["plain_fp64"],
            "speedup_vs_loop_fp32_refine": value / loops["fp32_refine"],
            "gpu_launches": int(launches), "clocks": clocks,
            "batch_create_wall_s": setup_s,
            "fmm_setup": {"device_sort": tree, "host_sort": tree_host, "batch_create_wall_s_host_sort": setup_host_s},
            "fp64_batch_steps_samples_per_s": fp64_batch,
            "learned_guess_batch_steps_samples_per_s": learned_batch,
            "speedup_fp64_batch_vs_loop_plain_fp64": fp64_batch["value"] / loops["plain_fp64"],
            "energy_sample0": [float(x) for x in E[0]],
        }
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()

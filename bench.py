"""Throughput of the GB300 WCSPH-DEM step (particle-steps/s) -- one JSON line.

Workload (default): the 800k-fluid variant of the large dam break -- tank
4 x 0.8 x 1.5 m, fluid block 0.167 x 0.8 x 0.75 m at dx = 0.005 (792,000
fluid, 2,157,576 dummy wall particles), 2,000 DEM spheres R ~ U[0.01, 0.03]
rejection-sampled above the water, 178,528 DEM wall spheres, dt = 2.5e-5 --
generated from seeded rules (synthetic data).  ``--workload scaled`` runs the
dx = 0.01 dam break (100,000 fluid, 160 DEM); ``--workload batch64`` advances
64 seeded dx = 0.02 dam breaks of different sizes as one batched state.

A step is one loop body of run_forward: moving grids re-binned + one coupled
SPHDEM step, replayed from CUDA graphs.  value = (fluid + DEM) particles x
steps / device time (CUDA events on the launch stream, barrier + synchronize
on both sides, max over ranks).  The state (~200 MB at 800k) is larger than
the 129 MB L2, so no flush is needed between steps.  e2e: the same metric
through the public API (SPHDEM_OneStep) with the state copied from pinned host
memory before and back after every step.  N > 1: independent replicas, one per
GPU (the path does not shard), value = sum over ranks.

``--impl reference`` times the reference algorithm on the host cores instead:
the CPU oracle (a restatement of the reference's Warp kernels) with all
threads; the first timed step runs in full, the others on a bounded sample
(every S-th subject particle) scaled by the measured full/sample ratio.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0
PROFILE_DIR = ROOT / "profiles"

# Algorithmic bytes per unit of each phase's kernel: every input field read
# once, every output field written once (FP32).  Units: fluid particles unless
# stated.
PHASE_BYTES = {
    "force": ("fluid", 36 + 24),          # pos, vel, m, rho, pres in; acc, pgf out
    "density": ("fluid", 20 + 8),         # pos, m, flt in; rho, pres out
    "wall_density": ("wall", 16 + 8),     # pos, m in; rho, pres out (per wall particle)
    "porosity": ("fluid", 20 + 4),        # pos, m, rho in; porosity out
    "grid_sph": ("fluid", 12 + 8 + 32 + 36),  # bin pos; key+order; gather in; sorted out
    "react_integrate": ("fluid", 44 + 48),
    "exchange": ("dem", 176),
    "contacts": ("dem", 176),
    "grid_dem": ("dem", 20),
    "dem_step": ("dem", 72 + 48),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
WORKLOADS = ("large800k", "scaled", "small", "batch64", "learned")
BATCH_MEMBERS = 64


def _case_spec(workload: str):
    from warp_sph_gpt_gb300.generate import config_large, config_scaled

    if workload == "large800k":
        gen, pos, rad = config_large(fluid_width=0.167, seed=0, n_dem=2000)
        desc = ("large dam break, 800k variant: tank 4x0.8x1.5 m, fluid 0.167x0.8x0.75 m at dx=0.005, "
                "2,000 DEM R~U[0.01,0.03], dt=2.5e-5")
    elif workload == "scaled":
        gen, pos, rad = config_scaled(seed=0)
        desc = "scaled dam break: tank 2x0.4x1 m, fluid 0.5x0.4x0.5 m at dx=0.01, 160 DEM R=0.025, dt=5e-5"
    elif workload == "small":
        from warp_sph_gpt_gb300.generate import config_small

        gen, pos, rad = config_small(), None, None
        desc = "config-1 dam break: the reference's input files (12,500 fluid, 48,336 wall, 20 DEM), dt=1e-4"
    else:
        raise SystemExit(f"unknown workload {workload}")
    return gen, pos, rad, desc


def make_case(workload: str, device):
    """One case as host/device structs (the reference arm uses member 0 of a batch)."""
    from warp_sph_gpt_gb300.generate import build_case, config_batch_member, solver_config

    if workload == "batch64":
        gen, pos, rad = config_batch_member(0)
        desc = f"batch member 0 of {BATCH_MEMBERS}"
    elif workload == "learned":
        from warp_sph_gpt_gb300.generate import config_small

        gen, pos, rad = config_small(), None, None
        desc = "config-1 dam break (12,500 fluid, 20 DEM), plain method"
    else:
        gen, pos, rad, desc = _case_spec(workload)
    P, B, D, W = build_case(gen, pos, rad, device=device)
    solv = solver_config(gen)
    return gen, solv, (P, B, D, W), desc


def default_lanes(n_fluid: int) -> int:
    """One warp per particle for small systems (one thread each leaves most
    SMs idle), one thread per particle otherwise."""
    return 32 if n_fluid <= 50_000 else 1


def make_runner(workload: str, device, cell_factor: float = 1.0):
    """GPU state of a workload: a Case, or an Ensemble of 64 seeded dam breaks."""
    from warp_sph_gpt_gb300.batch import Case, Ensemble
    from warp_sph_gpt_gb300.generate import config_batch_member

    if workload == "batch64":
        members = [config_batch_member(i) for i in range(BATCH_MEMBERS)]
        r = Ensemble(members, device=device, cell_factor=cell_factor)
        r.gen = members[0][0]
        r.desc = (f"ensemble of {BATCH_MEMBERS} dam breaks (tank 2x0.4x1 m, dx=0.02, fluid block "
                  "U[0.3,0.7] x 0.4 x U[0.3,0.6] m, 0-40 DEM R=0.025, dt=1e-4), one batched step")
    else:
        gen, pos, rad, desc = _case_spec(workload)
        r = Case(gen, pos, rad, device=device, cell_factor=cell_factor)
        r.gen, r.desc = gen, desc
    return r


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        self.gpu = gpu_index
        # raw samples (summarised into the JSON line); SPHDEM_CLOCKS_DIR keeps them elsewhere
        out = Path(os.environ.get("SPHDEM_CLOCKS_DIR", tempfile.gettempdir()))
        self.path = out / f"sphdem_clocks_{os.getpid()}_{id(self):x}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return None
        rows = []
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def peak_hbm():
    try:
        peaks = json.loads(PEAKS_FILE.read_text())
        return float(peaks["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(kernel: str, workload: str):
    """Per-launch DRAM bytes from the committed ncu summary, if present."""
    for p in PROFILE_DIR.glob(f"*{kernel}*{workload}*.txt"):
        for line in p.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                try:
                    return float(line.split(":", 1)[1])
                except ValueError:
                    pass
    return None


def reduce_max(value: float, world: int, device=None) -> float:
    """Max of a per-rank float over all ranks (the timing rule: the slowest
    replica sets the job time).  Identity for world == 1."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# Square roots per SM per clock of the MUFU pipe (sqrt.approx): the tensor-core
# porosity pass evaluates one per subject-candidate pair of every 128 x 128 chunk.
MUFU_SQRT_PER_SM_CLK = 16


def porosity_compute_roofline(ctx, D, scales, porosity_ms: float, device):
    """The porosity normaliser is bound by the pair evaluations, not HBM: the
    tensor cores give each pair's squared distance and the MUFU pipe its
    square root, so pairs per second are compared with 152 SMs x 16 square
    roots per clock.  'evaluated' counts every pair of the evaluated chunks
    (the tiles' windows), 'in_ball' the pairs inside the coupling support
    (exact count around 256 sampled listed particles)."""
    import torch

    if D.n == 0 or porosity_ms <= 0 or scales[3] <= 0:
        return None
    n_near = int(ctx.ctl[6].item())
    chunks = int(ctx.ctl[10].item())
    if n_near <= 0:
        return None
    w = ctx.work
    g = torch.Generator(device="cpu").manual_seed(0)
    pick = torch.randperm(n_near, generator=g)[:256].to(device)
    subj = w["f_posv"][w["near_list"][:n_near][pick].long(), :3]
    fluid = w["f_posv"][:, :3]
    support = 2.0 * float(scales[3])
    counts = torch.cat([(torch.cdist(subj[i:i + 32], fluid) < support).sum(1) for i in range(0, len(subj), 32)])
    pairs = float(counts.float().mean().item()) * n_near
    evaluated = float(chunks) * 128 * 128
    props = torch.cuda.get_device_properties(device)
    peaks = json.loads(PEAKS_FILE.read_text()) if PEAKS_FILE.exists() else {}
    mhz = float(peaks.get("sm_max_mhz", 2070.0))
    peak = props.multi_processor_count * MUFU_SQRT_PER_SM_CLK * mhz * 1e6
    secs = porosity_ms * 1e-3
    return {"bound": "mufu", "kernel": "k_porosity_mma", "listed_particles": n_near,
            "in_ball_pairs_per_step": pairs, "evaluated_pairs_per_step": evaluated,
            "achieved_pairs_per_s": evaluated / secs, "in_ball_pairs_per_s": pairs / secs,
            "peak_pairs_per_s": peak, "frac": evaluated / secs / peak, "in_ball_frac": pairs / secs / peak,
            "peak_basis": f"{props.multi_processor_count} SMs x {MUFU_SQRT_PER_SM_CLK} square roots per clock x "
                          f"{mhz:.0f} MHz (one per evaluated pair; the squared distances come from tcgen05 MMAs)"}


def output_run(args, solv, P, B, D, W, grids, scales, n_units, first_step):
    """The same steps with a VTP frame (fluid + wall, DEM) every output_step
    steps through the asynchronous FrameWriter; wall time includes writing every
    file and the collections."""
    import shutil
    import tempfile

    import torch

    from warp_sph_gpt_gb300 import run_steps
    from warp_sph_gpt_gb300.output import FrameWriter

    out_dir = tempfile.mkdtemp(prefix="sphdem_frames_")
    try:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        writer = FrameWriter(solv, P, B, D, W, out_dir=out_dir)
        step = first_step
        for _ in range(max(1, args.steps // args.output_step)):
            run_steps(solv, P, B, grids[0], grids[1], D, W, grids[2], grids[3], first_step=step,
                      n_steps=args.output_step, search_scales=scales)
            step += args.output_step
            writer.write_frame(step)
        writer.finalize()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        files = os.listdir(out_dir)
        size = sum(os.path.getsize(os.path.join(out_dir, f)) for f in files)
        steps = step - first_step
        return {"value": n_units * steps / wall, "unit": "particle-steps/s", "steps": steps,
                "frames": len(writer.frames), "bytes_written": size, "wall_s": round(wall, 3),
                "note": "wall clock incl. formatting and writing every VTP/PVD file (asynchronous writer thread)"}
    finally:
        shutil.rmtree(out_dir, ignore_errors=True)


def job_throughput(units_per_replica: int, steps: int, world: int, ms_max: float) -> float:
    """Whole-job particle-steps/s of `world` replicas timed by the slowest."""
    return world * units_per_replica * steps / (ms_max * 1e-3)


def gpu_arm(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist
    import ctypes as C

    from warp_sph_gpt_gb300 import SPHDEM_OneStep, dem_search_scales, run_steps
    from warp_sph_gpt_gb300 import _lib
    from warp_sph_gpt_gb300.engine import context_for

    torch.cuda.set_device(local_rank)
    device = torch.device("cuda", local_rank)
    tuning = {}
    if args.autotune:
        from warp_sph_gpt_gb300.autotune import autotune, case_key

        probe = make_runner(args.workload, device)
        key = case_key(probe.P, probe.B, probe.D, probe.W, probe.ninst)
        n_fluid = probe.P.n
        del probe
        tuning = autotune(lambda cf: make_runner(args.workload, device, cf), key,
                          ninst=BATCH_MEMBERS if args.workload == "batch64" else 1, log=log, n_fluid=n_fluid)
        args.cell_factor = tuning["cell_factor"]
        log(f"[rank {rank}] autotuned: {tuning}")
        torch.cuda.empty_cache()
    runner = make_runner(args.workload, device, args.cell_factor)
    if not tuning:
        tuning = {"lanes_sph": args.lanes_sph or default_lanes(runner.P.n)}
        if args.porosity_variant >= 0:
            tuning["porosity_variant"] = args.porosity_variant
        if args.nbr_cap >= 0:
            tuning["nbr_cap"] = args.nbr_cap
        if args.nbr_format >= 0:
            tuning["nbr_format"] = args.nbr_format
    runner.tune(tuning)
    gen, solv, desc = runner.gen, runner.solv, runner.desc
    P, B, D, W = runner.P, runner.B, runner.D, runner.W
    scales, grids = runner.scales, runner.grids
    n_units = P.n + D.n
    log(f"[rank {rank}] {desc}: fluid {P.n}, wall {B.n}, DEM {D.n}, DEM wall {W.n}")

    # warm-up (also captures the graphs)
    run_steps(solv, P, B, grids[0], grids[1], D, W, grids[2], grids[3], first_step=0, n_steps=args.warmup,
              search_scales=scales)
    torch.cuda.synchronize()
    ctx = context_for(P, B, D, W, tuple(grids))

    def barrier():
        if world > 1:
            dist.barrier()

    stream = torch.cuda.current_stream()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clocks:
        start.record(stream)
        run_steps(solv, P, B, grids[0], grids[1], D, W, grids[2], grids[3], first_step=args.warmup,
                  n_steps=args.steps, search_scales=scales)
        end.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = start.elapsed_time(end)
    first = args.warmup
    shep = sum(1 for s in range(first, first + args.steps) if s == 0 or s % solv.shepard_step == 0)
    k1 = ctx.lib.sphdem_graph_kernels(C.byref(ctx.ctx), 1)
    k0 = ctx.lib.sphdem_graph_kernels(C.byref(ctx.ctx), 0)
    launches = shep * max(k1, 0) + (args.steps - shep) * max(k0, 0)
    ms_max = reduce_max(ms, world, device)
    ctx.check_status()

    # per-phase device times (CUDA events between phases, same stream)
    phase_ms = np.zeros(len(_lib.PHASES))
    reps = 5
    buf = (C.c_float * len(_lib.PHASES))()
    for r in range(reps):
        ctx.prepare(rebuild_moving=False)
        _lib.check(ctx.lib.sphdem_profile_step(C.byref(ctx.ctx), C.byref(ctx.params), first + args.steps + r, 1,
                                               buf, ctx.stream), "profile")
        D._flip("dem")  # the profiled step swapped both contact CSRs on the device
        D._flip("bnd")
        phase_ms += np.array(buf[:])
    phase_ms /= reps
    phases = {name: round(float(v), 4) for name, v in zip(_lib.PHASES, phase_ms)}
    dom = max(phases, key=phases.get)
    unit, per = PHASE_BYTES.get(dom, ("fluid", 0))
    units = {"fluid": P.n, "wall": B.n, "dem": D.n}[unit]
    alg_bytes = per * units
    peak, peak_kind = peak_hbm()
    achieved = alg_bytes / (phases[dom] * 1e-3) / 1e9 if phases[dom] > 0 else 0.0

    compute = porosity_compute_roofline(ctx, D, scales, phases.get("porosity", 0.0), device)
    output = output_run(args, solv, P, B, D, W, grids, scales, n_units, first + args.steps + reps) \
        if args.output_step > 0 else None

    # e2e through the public API with host buffers
    e2e_steps = min(args.steps, args.e2e_steps)
    host = {k: torch.empty_like(t, device="cpu").pin_memory() for k, t in
            (("pos", P.pos), ("vel", P.vel), ("dpos", D.pos), ("dvel", D.vel), ("domega", D.omega))}
    for k, t in (("pos", P.pos), ("vel", P.vel), ("dpos", D.pos), ("dvel", D.vel), ("domega", D.omega)):
        host[k].copy_(t)
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    d2h = h2d
    torch.cuda.synchronize()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for s in range(e2e_steps):
        P.pos.copy_(host["pos"], non_blocking=True)
        P.vel.copy_(host["vel"], non_blocking=True)
        D.pos.copy_(host["dpos"], non_blocking=True)
        D.vel.copy_(host["dvel"], non_blocking=True)
        D.omega.copy_(host["domega"], non_blocking=True)
        SPHDEM_OneStep(solv, P, B, D, W, *grids, first + args.steps + reps + s, scales)
        host["pos"].copy_(P.pos, non_blocking=True)
        host["vel"].copy_(P.vel, non_blocking=True)
        host["dpos"].copy_(D.pos, non_blocking=True)
        host["dvel"].copy_(D.vel, non_blocking=True)
        host["domega"].copy_(D.omega, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = reduce_max(e0.elapsed_time(e1), world, device)

    result = {
        "metric": "particle-steps/s",
        "value": job_throughput(n_units, args.steps, world, ms_max),
        "unit": "particle-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded generator rules of the reference's input_gen)",
        "config": {"workload": desc, "fluid": P.n, "wall": B.n, "dem": D.n, "dem_wall": W.n,
                   "particles_counted": "fluid + moving DEM", "parallelism": f"replicas x{world}",
                   "cell_factor": args.cell_factor, "members": getattr(runner, "ninst", 1),
                   "tuning": {k: v for k, v in tuning.items() if k != "ms_per_step"},
                   "l2": "state > 129 MB L2 (no flush)" if args.workload == "large800k"
                   else "state < L2 (resident between steps, as in a run)"},
        "e2e": {"value": job_throughput(n_units, e2e_steps, world, e2e_ms), "unit": "particle-steps/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": e2e_steps,
                "api": "SPHDEM_OneStep per step, state copied from / to pinned host memory"},
        "roofline": {"bound": "hbm", "kernel_phase": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "traffic": profile_traffic(dom, args.workload)},
        "compute_roofline": compute,
        "with_output": output,
        "phases_ms": phases,
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        if args.workload == "batch64":
            # members are independent: the oracle times member 0 (same particle-steps/s per core)
            g0, s0, parts0, _ = make_case("batch64", "cpu")
            result["cpu_baseline"] = cpu_baseline(g0, s0, parts0, dem_search_scales(parts0[2], parts0[3]),
                                                  args.cpu_budget_s)
            result["cpu_baseline"]["sample"] += " (ensemble member 0; members are independent)"
        else:
            result["cpu_baseline"] = cpu_baseline(gen, solv, (P, B, D, W), scales, args.cpu_budget_s)
    return result


# ---------------------------------------------------------------------------
# learned surrogate vs plain on the config-1 dam break
# ---------------------------------------------------------------------------
def _fluid_density(case):
    from warp_sph_gpt_gb300.kernels import Kernel_density_sph

    Kernel_density_sph(case.P, case.B, case.grids[0], case.grids[1], case.solv.support, case.solv.h)
    return case.P.rho.clone()


def _edge_flops(E, nn, nr):
    """Tensor-core FLOPs of one forward pass: two edge passes (16->128->128 per
    edge) and the node layers (16->128, 128->128 on all nodes, 128->16 on
    receivers)."""
    return 2 * E * 2 * (16 * 128 + 128 * 128) + nn * 2 * (16 * 128 + 128 * 128) + nr * 2 * 128 * 16


def learned_arm(args, rank, world, local_rank):
    import ctypes as C

    import torch

    from warp_sph_gpt_gb300 import surrogate as S
    from warp_sph_gpt_gb300.batch import Case, Ensemble
    from warp_sph_gpt_gb300.generate import config_batch_member, config_small

    torch.cuda.set_device(local_rank)
    device = torch.device("cuda", local_rank)
    t_start = time.perf_counter()
    # training data: trajectories of the batched plain solver (seeded dx = 0.02 dam breaks)
    members = [config_batch_member(1000 + i) for i in range(args.train_members)]
    ens = Ensemble(members, device=device)
    s = ens.solv
    cfg = S.SurrogateConfig(radius=float(args.graph_radius or s.support), dt=float(s.dt), rho0=float(s.rho0),
                            tol=args.judge_tol, judge=args.judge, pos_tol=args.pos_tol_dx * 0.02)
    t0 = time.perf_counter()
    ts = S.generate(ens, args.train_steps, cfg, log=log)
    t_gen = time.perf_counter() - t0
    n_val = max(1, len(members) // 8)
    train_ids = list(range(len(members) - n_val))
    val_ids = list(range(len(members) - n_val, len(members)))
    S.fit_scales(ts, cfg, train_ids[:16], device)
    net = S.Network(cfg, device, seed=args.seed)
    prior = S.evaluate(net, ts, val_ids, zero=True)
    t0 = time.perf_counter()
    hist = S.train(net, ts, train_ids, iters=args.train_iters, lr=2e-3, log=log, log_every=500,
                   seed=100 * args.seed, edge_weight=args.edge_weight, noise=(args.noise_x, args.noise_v),
                   ema=args.ema)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    on_policy = []
    if args.dagger_rounds > 0:
        cases = []
        for i in [i for i in train_ids if len(members[i][1])][: args.dagger_cases]:  # members with DEM
            gen_i, pos_i, rad_i = members[i]
            c = Case(gen_i, pos_i, rad_i, device=device)
            c.tune({"lanes_sph": default_lanes(c.P.n)})
            cases.append(c)
        for rnd in range(args.dagger_rounds):
            snaps0 = [c.snapshot() for c in cases]
            on_policy += S.collect_on_policy(net, cases, args.train_steps, log=log)
            for c, s0 in zip(cases, snaps0):
                c.restore(s0)
            hist += S.train(net, ts, train_ids, iters=args.dagger_iters, lr=1e-3, log=log, log_every=1000,
                            edge_weight=args.edge_weight, extra=on_policy, seed=100 * args.seed + rnd + 1,
                            ema=args.ema)
        t_train = time.perf_counter() - t0
    if args.ema > 0.0:
        net.use_ema()
    val = S.evaluate(net, ts, val_ids)
    log(f"held-out one-jump loss: prior {prior:.4f} -> trained {val:.4f}")
    del ts, ens
    torch.cuda.empty_cache()

    n = args.rollout_steps
    K = cfg.substeps + 1
    dx = 0.02
    # plain: graph replay of the coupled step
    plain = Case(config_small(), device=device)
    plain.tune({"lanes_sph": default_lanes(plain.P.n)})
    snap0 = plain.snapshot()
    plain.run(0, 3 * K)
    torch.cuda.synchronize()
    plain.restore(snap0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clocks_plain:
        e0.record()
        plain.run(0, n)
        e1.record()
        torch.cuda.synchronize()
    t_plain = e0.elapsed_time(e1) * 1e-3
    pos_p, vel_p = plain.P.pos.clone(), plain.P.vel.clone()
    dpos_p = plain.D.pos.clone()
    rho_p = _fluid_density(plain)
    # the plain method's own density deviation at every jump boundary (untimed re-run)
    plain_final = plain.snapshot()
    plain.restore(snap0)
    plain_dev, plain_change = [], []
    rho_prev = None
    for s0 in range(0, n, K):
        plain.run(s0, min(K, n - s0))
        plain_dev.append((plain.P.rho - cfg.rho0).abs().max().item() / cfg.rho0)
        if rho_prev is not None:
            plain_change.append((plain.P.rho - rho_prev).abs().max().item() / cfg.rho0)
        rho_prev = plain.P.rho.clone()
    plain.restore(plain_final)
    # the plain method against itself in another FP32 summation order (one
    # thread per particle instead of one warp): the trajectory's own noise floor
    alt = Case(config_small(), device=device)
    alt.tune({"lanes_sph": 1 if default_lanes(alt.P.n) == 32 else 32})
    alt.run(0, n)
    alt_err = (alt.P.pos - pos_p).norm(dim=1) / dx
    plain_reordered = {"pos_max_dx": alt_err.max().item(), "pos_rms_dx": alt_err.pow(2).mean().sqrt().item(),
                       "order": "same plain step, thread instead of warp per particle"}
    del alt
    # learned: one plain step + m learned substeps per jump, density judge, plain fallback
    learned = Case(config_small(), device=device)
    learned.tune({"lanes_sph": default_lanes(learned.P.n)})
    snapL = learned.snapshot()
    ro = S.LearnedRollout(learned, net)
    ro.native = not args.rollout_hosted
    ro.run(0, 6 * K)  # both Shepard variants run eagerly once, then are captured
    torch.cuda.synchronize()
    learned.restore(snapL)
    ro.stats = dict(jumps=0, fallbacks=0, plain_steps=0, learned_steps=0, max_dev_accepted=0.0, max_pos_accepted=0.0,
                    jump_kernels=0)
    # e2e: initial state from pinned host memory, final state back to the host
    host_in = {k: t.detach().cpu().pin_memory() for k, t in (("pos", learned.P.pos), ("vel", learned.P.vel),
                                                              ("dpos", learned.D.pos), ("dvel", learned.D.vel))}
    host_out = {k: torch.empty_like(v).pin_memory() for k, v in host_in.items()}
    h2d = sum(v.numel() * v.element_size() for v in host_in.values())
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clocks_learned:
        torch.cuda.nvtx.range_push("learned_rollout")
        t0 = time.perf_counter()
        learned.P.pos.copy_(host_in["pos"], non_blocking=True)
        learned.P.vel.copy_(host_in["vel"], non_blocking=True)
        learned.D.pos.copy_(host_in["dpos"], non_blocking=True)
        learned.D.vel.copy_(host_in["dvel"], non_blocking=True)
        stats = ro.run(0, n)
        host_out["pos"].copy_(learned.P.pos, non_blocking=True)
        host_out["vel"].copy_(learned.P.vel, non_blocking=True)
        host_out["dpos"].copy_(learned.D.pos, non_blocking=True)
        host_out["dvel"].copy_(learned.D.vel, non_blocking=True)
        torch.cuda.synchronize()
        t_learned = time.perf_counter() - t0
        torch.cuda.nvtx.range_pop()
    err = (learned.P.pos - pos_p).norm(dim=1) / dx
    q = torch.quantile(err.float(), torch.tensor([0.99, 0.999], device=device)).tolist()
    worst = int(err.argmax().item())
    nd = (pos_p[worst] - dpos_p).norm(dim=1).min().item() / dx if learned.D.n else float("nan")
    where = {"z_m": pos_p[worst, 2].item(), "speed_mps": vel_p[worst].norm().item(), "nearest_dem_dx": nd,
             "rho_plain": rho_p[worst].item()}
    derr = (learned.D.pos - dpos_p).norm(dim=1) / dx if learned.D.n else torch.zeros(1, device=device)
    rho_l = _fluid_density(learned)
    rho_dev = ((rho_l - rho_p).abs().max() / cfg.rho0).item()
    rho_rms = ((rho_l - rho_p).pow(2).mean().sqrt() / cfg.rho0).item()
    # tensor-core roofline of the network's forward pass on the final state
    g = ro.g
    g.set_nodes(S.Sets(learned.P, learned.B, learned.D, learned.W))
    g.build()
    E = g.n_edges()
    g.forward(net)
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 20
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("mpnn_forward")
    f0.record()
    for _ in range(reps):
        g.forward(net)
    f1.record()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    fwd_ms = f0.elapsed_time(f1) / reps
    flops = _edge_flops(E, g.n_nodes, g.n_recv)
    peaks = json.loads(PEAKS_FILE.read_text()) if PEAKS_FILE.exists() else {}
    peak_tf = float(peaks.get("bf16_tflops", 1900.0))
    achieved_tf = flops / (fwd_ms * 1e-3) / 1e12
    units = learned.P.n + learned.D.n
    value = units * n / t_learned
    return {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": n, "warmup": 6 * K, "ms_per_step": t_learned * 1e3 / n, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16 network (fp32 accumulate) + f32 plain steps",
        "data": "synthetic (seeded generator rules; training trajectories from the batched plain solver)",
        "config": {"workload": "learned K-step surrogate vs plain on the config-1 dam break "
                               "(12,500 fluid, 20 DEM, dt=1e-4)", "K": K, "judge_tol": cfg.tol, "judge": cfg.judge,
                   "pos_tol_dx": args.pos_tol_dx, "seed": args.seed,
                   "graph_radius": cfg.radius, "edge_weight": args.edge_weight,
                   "train_noise": [args.noise_x, args.noise_v], "dagger_rounds": args.dagger_rounds, "ema": args.ema,
                   "rollout": "host-judged" if args.rollout_hosted else "device-judged",
                   "rollout_steps": n, "fluid": learned.P.n, "dem": learned.D.n,
                   "l2": "state < L2 (resident between steps, as in a run)"},
        "plain": {"value": units * n / t_plain, "ms_per_step": t_plain * 1e3 / n, "clocks": clocks_plain.summary()},
        "speedup_vs_plain": t_plain / t_learned,
        "error_vs_plain": {"pos_max_dx": err.max().item(), "pos_rms_dx": err.pow(2).mean().sqrt().item(),
                           "pos_p99_dx": q[0], "pos_p999_dx": q[1], "worst_particle": where,
                           "dem_pos_max_dx": derr.max().item(), "rho_max_diff": rho_dev, "rho_rms_diff": rho_rms,
                           "learned_final_density_deviation": ((rho_l - cfg.rho0).abs().max() / cfg.rho0).item(),
                           "plain_final_density_deviation": ((rho_p - cfg.rho0).abs().max() / cfg.rho0).item(),
                           "judge_max_dev_accepted": stats["max_dev_accepted"]},
        "plain_reordered_vs_plain": plain_reordered,
        "plain_density_deviation": {"max": max(plain_dev), "mean": sum(plain_dev) / len(plain_dev),
                                    "fraction_above_tol": sum(d > cfg.tol for d in plain_dev) / len(plain_dev)},
        "plain_density_change_per_jump": {"max": max(plain_change), "mean": sum(plain_change) / len(plain_change),
                                          "fraction_above_tol": sum(d > cfg.tol for d in plain_change)
                                          / len(plain_change)},
        "rollout": stats,
        "training": {"members": len(members), "train_members": len(train_ids), "val_members": len(val_ids),
                     "trajectory_steps": args.train_steps, "iterations": args.train_iters,
                     "generate_s": round(t_gen, 2), "train_s": round(t_train, 2),
                     "val_loss_prior": prior, "val_loss_trained": val, "loss_history": hist[-3:],
                     "output_scales": list(cfg.scale)},
        "roofline": {"bound": "tensor", "kernel_phase": "mpnn forward (k_rows, k_edges)", "achieved": achieved_tf,
                     "peak": peak_tf, "unit": "TFLOP/s", "frac": achieved_tf / peak_tf,
                     "peak_source": "measured" if peaks else "fallback", "flops_per_launch": flops,
                     "edges": E, "forward_ms": fwd_ms, "traffic": None},
        "e2e": {"value": units * n / t_learned, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d / n,
                "d2h_bytes_per_step": h2d / n,
                "api": "LearnedRollout.run over the whole rollout; initial state from pinned host memory, final "
                       "state back"},
        "gpu_launches": stats["jump_kernels"] + (stats["plain_steps"] - stats["jumps"])
        * max(0, int(ro.lib.sphdem_graph_kernels(C.byref(ro.ctx.ctx), 0))),
        "clocks": clocks_learned.summary(),
        "wall_s": round(time.perf_counter() - t_start, 1),
    }


# ---------------------------------------------------------------------------
# CPU (reference algorithm) timing
# ---------------------------------------------------------------------------
def _oracle_state(parts):
    from oracle.oracle import HostState

    return HostState(*parts)


def cpu_sample(host, solv, scales, stride: int, step: int) -> float:
    """Seconds of one oracle step over every stride-th subject, run on a fresh
    copy of the state (a sampled step leaves the unsampled subjects stale, so
    samples must not run on each other's results)."""
    import copy

    from oracle import oracle as O

    state = copy.deepcopy(host)
    O.set_subject_stride(stride)
    t0 = time.perf_counter()
    state.sphdem_onestep(solv, step, scales, p="f32")
    dt = time.perf_counter() - t0
    O.set_subject_stride(1)
    return dt


def _prime_at_least(k: int) -> int:
    """Smallest prime >= k: prime strides do not alias with the particle
    lattice's dimensions (every layer of the lattice is sampled alike)."""
    k = max(2, int(k))
    while any(k % d == 0 for d in range(2, int(k ** 0.5) + 1)):
        k += 1
    return k


def cpu_fit(host, solv, scales, budget_s: float):
    """Choose a prime subject stride S so one sample fits the budget, then fit
    the full-step time F + V from samples at S and at a prime near 2S."""
    n = len(host.sph["pos"])
    stride = _prime_at_least(max(2, n // 2048))
    t = cpu_sample(host, solv, scales, stride, 1)
    # aim one sample at ~budget/4
    while t < budget_s / 8 and stride > 2:
        stride = _prime_at_least(max(2, stride // 2))
        t = cpu_sample(host, solv, scales, stride, 1)
        if stride == 2:
            break
    s2 = _prime_at_least(2 * stride)
    t1 = cpu_sample(host, solv, scales, stride, 1)
    t2 = cpu_sample(host, solv, scales, s2, 1) if s2 <= n else t1
    inv1, inv2 = 1.0 / stride, 1.0 / s2
    V = max(0.0, (t1 - t2) / (inv1 - inv2)) if t1 > t2 else t1 * stride
    F = max(0.0, t1 - V * inv1)
    return stride, t1, t2, F + V


def cpu_full_step(host, solv, scales, step: int) -> float:
    """Seconds of one complete oracle step (every subject) on a fresh copy."""
    return cpu_sample(host, solv, scales, 1, step)


def cpu_single_thread(host, solv, scales, stride: int, cores: int, t_full: float):
    """Single-thread figure: one sampled step on 1 thread and on all cores at
    the same stride; the full single-thread step is the measured full step
    scaled by their ratio (the reference's Warp CPU launches are serial)."""
    from oracle import oracle as O

    O.set_threads(1)
    t1 = cpu_sample(host, solv, scales, stride, 1)
    O.set_threads(cores)
    tm = cpu_sample(host, solv, scales, stride, 1)
    return t1, tm, t_full * t1 / tm if tm > 0 else float("nan")


def cpu_baseline(gen, solv, parts, scales, budget_s):
    """The FP32 oracle on the host cores: one complete step timed (measured),
    the two-point stride fit kept as a cross-check (extrapolated), and the
    single-thread figure (sample ratio)."""
    from oracle import oracle as O

    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    O.set_threads(cores)
    host = _oracle_state(parts)
    n_units = len(host.sph["pos"]) + len(host.dem["pos"])
    t_full = cpu_full_step(host, solv, scales, 1)
    stride, t1, t2, fit = cpu_fit(host, solv, scales, budget_s)
    s1 = _prime_at_least(4 * stride)
    st1, stm, t_single = cpu_single_thread(host, solv, scales, s1, cores, t_full)
    return {"value": n_units / t_full, "unit": "particle-steps/s", "cores": cores, "kind": "port",
            "measured": {"full_step_s": round(t_full, 3), "steps_timed_in_full": 1, "threads": cores},
            "extrapolated": {"full_step_s": round(fit, 3), "value": n_units / fit,
                             "method": f"t(S) = F + V/S from one step on every {stride}-th and every "
                                       f"{_prime_at_least(2 * stride)}-th subject ({t1:.2f} s, {t2:.2f} s)"},
            "single_thread": {"value": n_units / t_single, "full_step_s": round(t_single, 2),
                              "method": f"measured full step x (1-thread / {cores}-thread time of one step on "
                                        f"every {s1}-th subject: {st1:.2f} s / {stm:.2f} s)"},
            "sample": f"CPU oracle (restatement of the reference Warp kernels, FP32) on {cores} threads: one "
                      f"complete coupled step of the workload timed ({t_full:.2f} s, fresh copy of the state)"}


def reference_arm(args):
    """--impl reference: the reference algorithm on the host cores.  The first
    timed step runs every subject (measured); the others run a bounded sample
    (every S-th subject) scaled by the measured full/sample ratio, so the
    whole run stays within a few minutes."""
    from oracle import oracle as O

    gen, solv, parts, desc = make_case(args.workload, "cpu")
    from warp_sph_gpt_gb300 import dem_search_scales

    scales = dem_search_scales(parts[2], parts[3])
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    O.set_threads(cores)
    host = _oracle_state(parts)
    n_units = parts[0].n + parts[2].n
    stride, t1, t2, fit = cpu_fit(host, solv, scales, args.cpu_budget_s)
    for s in range(args.warmup):  # warm-up samples (caches, thread pool)
        cpu_sample(host, solv, scales, stride, 1 + s)
    t_full = cpu_full_step(host, solv, scales, 1 + args.warmup)
    t_sample0 = cpu_sample(host, solv, scales, stride, 1 + args.warmup)
    scale = t_full / t_sample0 if t_sample0 > 0 else 1.0
    steps = [t_full]
    for s in range(1, args.steps):
        steps.append(cpu_sample(host, solv, scales, stride, 1 + args.warmup + s) * scale)
    step_s = statistics.mean(steps)
    value = n_units / step_s
    timing = f"step 1 of {args.steps} timed in full ({t_full:.2f} s, every subject)"
    if args.steps > 1:
        timing += (f"; steps 2-{args.steps} on every {stride}-th subject, scaled by the measured full/sample "
                   f"ratio {scale:.2f}")
    return {"impl": "reference", "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
            "n_gpus": 0, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator rules of the reference's input_gen)",
            "config": {"workload": desc, "fluid": parts[0].n, "wall": parts[1].n, "dem": parts[2].n,
                       "dem_wall": parts[3].n},
            "timing": timing,
            "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                             "measured": {"full_step_s": round(t_full, 3), "steps_timed_in_full": 1},
                             "extrapolated": {"full_step_s": round(fit, 3),
                                              "method": f"two-point stride fit (strides {stride}, "
                                                        f"{_prime_at_least(2 * stride)})"},
                             "sample": timing},
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def extra_workloads(args) -> dict:
    """The batched ensemble and the learned surrogate, each run by this script
    in a child process (their own CUDA state) after the headline measurement,
    summarised into the headline line so one default run records them."""
    out = {}
    for wl, extra in (("batch64", ["--no-cpu-baseline"]), ("learned", [])):
        cmd = [sys.executable, str(Path(__file__).resolve()), "--workload", wl, "--steps", str(args.steps),
               "--warmup", str(args.warmup), "--no-extras", *extra]
        t0 = time.perf_counter()
        proc = subprocess.run(cmd, capture_output=True, text=True)
        wall = time.perf_counter() - t0
        line = next((x for x in proc.stdout.splitlines()[::-1] if x.startswith("{")), None)
        if proc.returncode != 0 or line is None:
            out[wl] = {"error": f"exit {proc.returncode}: {proc.stderr.strip().splitlines()[-1:] or ''}"}
            continue
        r = json.loads(line)
        keep = ("value", "unit", "ms_per_step", "steps", "warmup", "e2e", "gpu_launches", "clocks")
        d = {k: r[k] for k in keep if k in r}
        d["config"] = r.get("config", {}).get("workload")
        d["wall_s"] = round(wall, 1)
        if wl == "batch64":
            d["members"] = r.get("config", {}).get("members")
            d["fluid"] = r.get("config", {}).get("fluid")
        else:
            for k in ("speedup_vs_plain", "plain", "error_vs_plain", "rollout", "plain_reordered_vs_plain"):
                d[k] = r.get(k)
            t = r.get("training", {})
            d["training"] = {k: t.get(k) for k in ("members", "iterations", "train_s", "val_loss_prior",
                                                   "val_loss_trained")}
            d["judge"] = {k: r.get("config", {}).get(k) for k in ("judge", "judge_tol", "pos_tol_dx")}
        out[wl] = d
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=("gb300", "reference"))
    ap.add_argument("--workload", default="large800k", choices=WORKLOADS)
    ap.add_argument("--train-members", type=int, default=64, help="learned: ensemble members of training data")
    ap.add_argument("--train-steps", type=int, default=1000, help="learned: plain steps per training trajectory")
    ap.add_argument("--train-iters", type=int, default=10000, help="learned: Adam iterations")
    ap.add_argument("--rollout-steps", type=int, default=1000, help="learned: steps of the compared rollouts")
    ap.add_argument("--judge-tol", type=float, default=0.01, help="learned: density judge tolerance / rho0")
    ap.add_argument("--seed", type=int, default=0, help="learned: seed of the network's initial weights and sampling")
    ap.add_argument("--pos-tol-dx", type=float, default=0.0045,
                    help="learned: position judge -- fall back when the network's correction would move a particle "
                         "more than this many dx beyond the constant-acceleration prior within one jump (0 = off)")
    ap.add_argument("--ema", type=float, default=0.0, help="learned: parameter moving-average decay (0 = off)")
    ap.add_argument("--rollout-hosted", action="store_true",
                    help="learned: judge every jump on the host (one graph launch and read-back per jump) instead "
                         "of on the device; its kernels are visible to a launch-list profiler")
    ap.add_argument("--dagger-rounds", type=int, default=2,
                    help="learned: rounds of on-policy data (states of judged learned rollouts + plain targets)")
    ap.add_argument("--dagger-cases", type=int, default=16, help="learned: training members rolled out per round")
    ap.add_argument("--dagger-iters", type=int, default=4000, help="learned: Adam iterations per on-policy round")
    ap.add_argument("--noise-x", type=float, default=0.0, help="learned: training input noise on positions [m]")
    ap.add_argument("--noise-v", type=float, default=0.0, help="learned: training input noise on velocities [m/s]")
    ap.add_argument("--edge-weight", type=float, default=0.0,
                    help="learned: weight of the neighbour relative-displacement term of the training loss")
    ap.add_argument("--judge", type=int, default=0, choices=(0, 1),
                    help="learned: 0 = density change over the jump, 1 = density deviation |rho - rho0| / rho0")
    ap.add_argument("--graph-radius", type=float, default=0.04,
                    help="learned: edge radius in m (0 = the SPH support 2h); 0.04 = 2 dx at config 1")
    ap.add_argument("--autotune", action="store_true",
                    help="time the launch candidates first (cached per case and GPU) and run the fastest")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-budget-s", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="large800k: skip the batch64 and learned runs that the default line also reports")
    ap.add_argument("--output-step", type=int, default=0,
                    help="also time the run with a VTP frame every N steps (asynchronous writer)")
    ap.add_argument("--porosity-variant", type=int, default=-1, choices=(-1, 0, 1, 2),
                    help="porosity normaliser implementation (-1 = library default)")
    ap.add_argument("--lanes-sph", type=int, default=0, choices=(0, 1, 32),
                    help="threads per particle of the SPH loops (0 = by system size)")
    ap.add_argument("--nbr-cap", type=int, default=-1,
                    help="neighbour-record capacity between the density and force passes (-1 = sized by the "
                         "library, 0 = none)")
    ap.add_argument("--nbr-format", type=int, default=-1, choices=(-1, 0, 1),
                    help="neighbour records: 0 = member slots, 1 = walk masks (-1 = library default, slots)")
    ap.add_argument("--cell-factor", type=float, default=1.0,
                    help="fluid/wall cell width as a fraction of the SPH support")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(reference_arm(args)), flush=True)
        return

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", init_method="env://")
    result = (learned_arm if args.workload == "learned" else gpu_arm)(args, rank, world, local_rank)
    if rank == 0 and world == 1 and args.workload == "large800k" and not args.no_extras:
        result["extras"] = extra_workloads(args)
    if rank == 0:
        print(json.dumps(result), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()

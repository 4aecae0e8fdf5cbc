"""Benchmark of the COLA particle-mesh step on GB300.

Workload (default): nDGP, rc*H0 = 1, density screening on (Gaussian filter,
Rsmooth 1 Mpc/h), 512^3 particles on a 1024^3 mesh, Box 1024 Mpc/h, 50
linear-in-a steps from z = 19 to z = 0, seed 5003, amplitude-fixed 2LPT
initial conditions, P(k) every step in 512 linear bins over [2 pi/Box,
k_Nyquist], RSD multipoles at z = 0.

One bench step is one whole run of the workload's schedule: fresh 2LPT
initial conditions (generated on the device, not timed), then all of its KDK
steps (50 for the default), so the throughput covers the run from z = 19 to
z = 0, where clustering slows the particle kernels.  A KDK step is the CIC
deposit, R2C, P(k) binning, fifth force (smoothing C2R, screening, R2C),
force k-space pass, three C2R and the fused interpolation + kick + drift.
Inputs are synthetic; the working set (~50 GB) is far larger than L2, so no
L2 flush is needed.

value: Mparticle-steps/s with the particle state resident in HBM (CUDA
       events on the context stream around each run's KDK steps).
e2e:   the same metric through the host-buffer C-ABI call mgp_step_host
       (pinned host particle arrays copied in and out every KDK step) over
       one whole run.
--impl reference: the FP64 CPU oracle (restatement of the reference's C
       code, particle loops parallel over x slabs as the reference's MPI
       tasks) timed on the host cores on a bounded sample of the workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "mg-picola-public_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "Mparticle-steps/s at 512^3 / 1024^3 mesh; P(k) rel. err vs FP64 oracle"
UNIT = "Mparticle-steps/s"

CONFIGS = {
    # name: (Ns, N, Box, model, nsteps_total, seed)
    "ndgp_512_1024": dict(Ns=512, N=1024, Box=1024.0, model="dgp", nsteps=50, seed=5003, fixed=1, nbins=512),
    "ndgp_256_512": dict(Ns=256, N=512, Box=512.0, model="dgp", nsteps=50, seed=5003, fixed=1, nbins=256),
    "lcdm_64_128": dict(Ns=64, N=128, Box=256.0, model="lcdm", nsteps=10, seed=5001, fixed=0, nbins=64),
    # 64 independent f(R) boxes (seeds 6001-6032, each normal + inverted,
    # |fR0| log-uniform in [1e-6, 1e-4]) in one batch, one graph launch per run
    "fofr_batch_64x64_128": dict(Ns=64, N=128, Box=256.0, model="fofr", nsteps=20, seed=6001, fixed=0, nbins=64,
                                 batch=64),
    # c1 with the whole 10-step run captured into one CUDA graph (the batch
    # engine with a single box): at this size the step is launch-bound
    "lcdm_64_128_graph": dict(Ns=64, N=128, Box=256.0, model="lcdm", nsteps=10, seed=5001, fixed=0, nbins=64,
                              batch=1),
    # COLA step with the learned force closure applied every step (256^3
    # particles on the 256^3 mesh, Box 256 Mpc/h, 30 steps)
    "closure_lcdm_256": dict(Ns=256, N=256, Box=256.0, model="lcdm", nsteps=30, seed=7017, fixed=0, nbins=128,
                             closure=True),
    # f(R) Hu-Sawicki n=1, |fR0|=1e-5, screening, scale-dependent growth on
    # 512 log-spaced k in [1e-4, 10] h/Mpc (256^3 particles, 512^3 mesh)
    "fofr_sd_256_512": dict(Ns=256, N=512, Box=512.0, model="fofr", nsteps=30, seed=5002, fixed=0, nbins=256,
                            sd=True),
    # the same with massive neutrinos (0.4 eV, synthetic CAMB tables)
    "fofr_nu_256_512": dict(Ns=256, N=512, Box=512.0, model="fofr", nsteps=30, seed=5002, fixed=0, nbins=256,
                            sd=True, nu=True),
}

# the closure network alone (random features on a 192^3 mesh): one forward
# or one Adam step per bench step; the convolution kernels' profiling workload
CONFIGS["closure_fwd_192"] = dict(N=192, probe=True)
CONFIGS["closure_train_192"] = dict(N=192, probe=True, train=True)

SD_GRID = dict(sd_nk=512, sd_kmin=1e-4, sd_kmax=10.0)
_NU_INFO = []


def nu_info():
    """Synthetic CAMB transfer tables (0.4 eV) in a temporary directory,
    written once per process."""
    if not _NU_INFO:
        import tempfile
        from tests.golden import camb_tables
        _NU_INFO.append(camb_tables.write_tables(tempfile.mkdtemp(prefix="mgp_camb_")))
    return _NU_INFO[0]


def model_name(cfg):
    if cfg["model"] == "dgp":
        name = "nDGP rcH0=1 screening (Gaussian, Rsmooth=1)"
    elif cfg["model"] == "fofr":
        name = "f(R) HS n=1 |fR0|=1e-5 screening"
    else:
        name = "LCDM"
    if cfg.get("sd"):
        name += ", scale-dependent growth (512 log k in [1e-4, 10] h/Mpc)"
    if cfg.get("nu"):
        name += " + massive neutrinos 0.4 eV (synthetic CAMB tables)"
    return name


def closure_flops(N):
    """Algorithmic FLOPs of one closure forward: 2 x 27 x C_in x C_out per
    voxel and layer over the live channels (3->16, 16->16, 16->16, 16->3)."""
    return 2 * 27 * (3 * 16 + 16 * 16 + 16 * 16 + 16 * 3) * N ** 3

# |fR0| of the batch: one value per seed pair, drawn log-uniform in [1e-6, 1e-4]
# by numpy's PCG64 with this seed.
BATCH_FR0_SEED = 20260604


def batch_boxes(cfg):
    if cfg["batch"] == 1:  # one box: the whole run as one graph launch
        return [dict(Seed=cfg["seed"], inverted=0, fofr0=1e-5)]
    rng = np.random.default_rng(BATCH_FR0_SEED)
    f0 = 10 ** rng.uniform(-6.0, -4.0, cfg["batch"] // 2)
    return [dict(Seed=cfg["seed"] + i, inverted=inv, fofr0=float(f0[i])) for i in range(cfg["batch"] // 2)
            for inv in (0, 1)]


def make_params(M, cfg):
    kw = dict(Nmesh=cfg["N"], Nsample=cfg["Ns"], Box=cfg["Box"], Seed=cfg["seed"], Init_Redshift=19.0,
              amplitude_fixed_initial_condition=cfg["fixed"], pofk_compute_every_step=1, pofk_nbins=cfg["nbins"],
              pofk_bintype=0, pofk_kmin=2 * np.pi / cfg["Box"], pofk_kmax=np.pi * cfg["N"] / cfg["Box"],
              pofk_subtract_shotnoise=1, Omega=0.267, OmegaBaryon=0.049, HubbleParam=0.71, Sigma8=0.8,
              PrimordialIndex=0.96, WhichSpectrum=2, UseCOLA=1)
    if cfg["model"] == "dgp":
        kw.update(model=M.MODEL_DGP, modified_gravity_active=1, include_screening=1, rcH0_DGP=1.0, Rsmooth=1.0,
                  smoothing_filter=M.FILTER_GAUSSIAN, input_pofk_is_for_lcdm=1, input_sigma8_is_for_lcdm=1)
    elif cfg["model"] == "fofr":
        kw.update(model=M.MODEL_FOFR, modified_gravity_active=1, include_screening=1, fofr0=1e-5, nfofr=1.0,
                  input_pofk_is_for_lcdm=1, input_sigma8_is_for_lcdm=1)
    if cfg.get("sd"):
        kw.update(scaledependent=1, **SD_GRID)
    if cfg.get("nu"):
        kw.update(massive_neutrinos=1, nu_include_massive_neutrinos=1, nu_SumMassNuEV=0.4,
                  nu_FilenameTransferInfofile=nu_info())
    return M.default_params(**kw)


def rank_seed(cfg, rank):
    """Replicas are independent boxes: rank r runs seed + r."""
    return cfg["seed"] + rank


def reduce_max(value, dist):
    """The job's time is the slowest rank's (max over ranks); identity on one
    process."""
    if dist is None:
        return value
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world, Np, steps, elapsed):
    """Whole-job throughput: the particle-steps of all ranks over the slowest
    rank's time (Mparticle-steps/s)."""
    return world * Np * steps / elapsed / 1e6


def shard(items, rank, world):
    """The boxes of rank r: r, r + world, r + 2 world, ... (independent
    boxes need no collective; each rank runs its share as one batch)."""
    return items[rank::world]


def run_batch(args, cfg, rank=0, world=1, dist=None):
    """A batch of independent boxes: each timed step is one graph launch that
    runs the whole KDK loop of every box; value counts particle-steps of all
    boxes (drift steps; the final output kick is included in the time).
    With several ranks the boxes are split across them (shard) and the job's
    time is the slowest rank's."""
    import mgpicola as M

    p = make_params(M, cfg)
    all_boxes = batch_boxes(cfg)
    boxes = shard(all_boxes, rank, world)
    B, Np, nst = len(boxes), cfg["Ns"] ** 3, cfg["nsteps"]
    batch = M.Batch(p, boxes)
    default_tuning = batch.tuning()
    batch.run(nst)
    default_ms = batch.ms(0)
    tune_t0 = time.perf_counter()
    tuned_ms = batch.autotune(nst)  # launch budgets picked by timing, before the timed region
    tune_s = time.perf_counter() - tune_t0
    tuning = batch.tuning()
    deposit_tiles = batch.deposit_tiles()
    for _ in range(args.warmup):
        batch.run(nst)
    launches = batch.graph_kernels()
    times, walls = [], []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            batch.run(nst)
            pk = [batch.pofk(b, nst)[1] for b in range(B)]  # the per-box results, read back every run
            walls.append(time.perf_counter() - t0)
            times.append(batch.ms(0))
    ic_ms = batch.ms(1)
    nodes = batch.graph_nodes()
    batch.close()
    ms = reduce_max(float(np.mean(times)), dist)
    wall = reduce_max(float(np.mean(walls)), dist)
    B_job = len(all_boxes)
    value = B_job * Np * nst / (ms * 1e-3) / 1e6
    N = cfg["N"]
    Nc = N ** 3
    # minimum HBM bytes per box-step (FP32): 84 Np particle traffic + the grid
    # traffic incl. the FFTs, 92 Nc with MG screening (six FFTs), 52 Nc for
    # LCDM (four FFTs and the P(k) pass)
    abytes = (84 * Np + (92 if cfg["model"] in ("fofr", "dgp") else 52) * Nc) * B
    achieved = abytes / (ms * 1e-3 / nst) / 1e9
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"hbm_gbs": 6800.0}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    out = {
        "metric": "Mparticle-steps/s of a batch of independent boxes", "value": round(value, 3), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": ("synthetic (2LPT ICs generated on the device, seeds %d-%d normal + inverted)"
                 % (cfg["seed"], cfg["seed"] + B // 2 - 1) if B > 1 else
                 "synthetic (2LPT IC generated on the device, seed %d)" % cfg["seed"]),
        "config": {"workload": args.config, "boxes": B_job, "boxes_per_rank": B, "particles_per_box": Np, "mesh": N,
                   "box_mpc_h": cfg["Box"], "step": "one graph launch: all %d KDK steps of every box" % nst,
                   "model": ("f(R) Hu-Sawicki n=1, screening, |fR0| log-uniform [1e-6, 1e-4] (seed %d)" % BATCH_FR0_SEED
                             if B > 1 else model_name(cfg)),
                   "steps_per_run": nst, "pofk_every_step": True, "pofk_bins": cfg["nbins"],
                   "launch_budgets": {"tuned": tuning, "default": default_tuning,
                                      "order": "blocks/SM: CIC deposit, grid passes, kick, P(k) binning",
                                      "deposit_tiles": deposit_tiles,
                                      "deposit_tiles_meaning": "0 lattice-order deposit, 8/16 tile side in cells",
                                      "autotune_s": round(tune_s, 2), "graph_ms_default": round(default_ms, 3),
                                      "graph_ms_tuned": round(tuned_ms, 3)},
                   "l2": "working set %.1f GB > L2" % (B * (6 * 4 * N * N * 2 * (N // 2 + 1) + 48 * Np) / 1e9)},
        "e2e": {"value": round(B_job * Np * nst / wall / 1e6, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(B * cfg["nbins"] * 8), "api": "mgp_batch_run + mgp_batch_pofk",
                "includes": "2LPT ICs of all boxes, graph launch, per-box P(k) read-back"},
        "gpu_launches": int(launches * args.steps),
        "graph": {"launches_per_run": 1, "nodes": nodes, "own_kernels": launches, "ic_ms": round(ic_ms, 3)},
        "per_box_completion_ms": {"p50": round(float(np.percentile(times, 50)), 3),
                                  "p99": round(float(np.percentile(times, 99)), 3),
                                  "min": round(float(np.min(times)), 3), "max": round(float(np.max(times)), 3),
                                  "note": "the boxes advance in lock step, so every box of a run completes "
                                          "with that run's graph: percentiles over the %d timed runs of %d boxes"
                                          % (len(times), B)},
        "roofline": {"bound": "hbm", "kernel": "whole step (FFTs included)", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": None,
                     "algorithmic_bytes_per_step": abytes, "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args)
        out["pofk_check"] = pofk_check(args.config)
    if rank == 0:
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                f = [x.strip() for x in out.stdout.strip().split(",")]
                if len(f) == 7:
                    self.samples.append(f)
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def algorithmic_bytes(N, Np, kernel):
    """Minimum HBM bytes per launch of each stage (FP32)."""
    NH = N // 2 + 1
    nreal = N * N * 2 * NH
    ncomplex = N * N * NH
    return {
        "cic": 12 * Np + 4 * N ** 3,                 # read s, write the mesh once
        "pofk": 8 * ncomplex,                         # read delta(k)
        "forces": 2 * 8 * ncomplex + 3 * 8 * ncomplex,  # read delta, MG source; write 3 complex grids
        # force grids once; s,v,D1,D2 in, s,v out (the tile kick also reads the order and each
        # slot's lattice point, and D1, D2 as a 32-byte record: 88 Np by design, the extra
        # counted as overhead, not as work)
        "interp_kick_drift": 12 * N ** 3 + 72 * Np,
        "mg": 8 * ncomplex + 4 * nreal + 8 * nreal,   # smoothing pass + screening pass (excl. FFTs)
    }[kernel]


# DRAM bytes per launch measured by ncu (dram__bytes.sum.per_second x gpu__time_duration.sum)
# on the nDGP step at 256^3 particles / 512^3 mesh, one launch each at step 46 of the 50-step
# run (profiles/deposit_and_kick_late_ndgp_256_512.md; tile deposit and tile kick over
# 8 x 8 x 64-cell tiles, the kick reading each slot's lattice point from the sort; the
# deposit's figure is its two passes, tile sums with owner writes and the halo pass).  Every term of these kernels scales with the particle count or the
# cell count, which grow together between the configurations (Nmesh = 2 Nsample), so the
# figure is scaled by the cell count.
TRAFFIC_256_512 = {"interp_kick_drift": 4.154e9, "cic": 1.420e9}


def measured_traffic(cfg, N, Np, kernel):
    # captured on the nDGP step's tile path only (scale-dependent growth and
    # the closure workloads run other kick or deposit forms)
    if kernel not in TRAFFIC_256_512 or Np * 8 != N ** 3 or cfg.get("model") != "dgp" or cfg.get("sd"):
        return None
    return int(TRAFFIC_256_512[kernel] * (N / 512.0) ** 3)


STAGES = ["sort", "fill", "cic", "r2c", "pofk", "mg", "forces", "c2r", "interp_kick_drift", "lpt_fields", "closure",
          "closure_conv"]


def run_gpu(args):
    import mgpicola as M

    # flush dirty pages left by earlier work on this host (snapshot files)
    # before the timed regions: their write-back competes with the
    # host-buffer copies of the e2e leg
    os.sync()

    cfg = CONFIGS[args.config]
    if cfg.get("probe"):
        return run_closure_probe(args, cfg)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    if cfg.get("batch"):
        return run_batch(args, cfg, rank, world, dist)
    p = make_params(M, cfg)
    p.Seed = rank_seed(cfg, rank)
    Np = cfg["Ns"] ** 3
    N = cfg["N"]
    nst = cfg["nsteps"]
    ctx = M.Context(p, device=local if world > 1 else 0)
    closure = None
    if cfg.get("closure"):
        closure = M.Closure(N, seed=cfg["seed"], device=local if world > 1 else 0)  # He-normal init weights
        closure.attach(ctx)
    A0 = 1.0 / (1.0 + p.Init_Redshift)
    da = (1.0 - A0) / nst

    def schedule():
        """(A, AI, AF, AFF) of the nst linear-in-a KDK steps (src/main.c:394-611)."""
        A, AI = A0, A0
        for _ in range(nst):
            AF, AFF = A + 0.5 * da, A + da
            yield A, AI, AF, AFF
            A, AI = AFF, AF

    def run(timed=False):
        """One bench step: the IC (not timed), then the whole schedule
        bracketed by events on the context stream.  Returns the device ms,
        this library's launches of the KDK steps and, when timed, the stage
        ms of every KDK step."""
        ctx.displacement_fields()
        if timed:
            ctx.set_timing(True, history=nst)
        l0 = ctx.launches()
        ctx.mark(0)
        for a in schedule():
            ctx.step(*a)
        ctx.mark(1)
        ms = ctx.mark_ms(0, 1)
        launches = ctx.launches() - l0
        stages = None
        if timed:
            stages = [{k: max(0.0, ctx.kernel_ms_step(k, i)) for k in STAGES + ["step"]} for i in range(nst)]
            ctx.set_timing(False)
        return ms, launches, stages

    def barrier():
        if dist is not None:
            dist.barrier()

    warm_ms = 0.0
    for _ in range(args.warmup):
        warm_ms = run()[0]
    # e2e through the host-buffer C-ABI entry point, pinned host memory: one
    # whole run from the IC state, after the warm-up runs and before the
    # timed device runs (on a host that ran GPU work before this process,
    # one host-buffer step in every 5-6 was seen to stall for 50-75 ms in its
    # copies; every step time is reported in e2e.step_ms)
    ctx.displacement_fields()
    arrs = ctx.get_particles()
    # the P[]-style arrays in page-locked host memory (mgp_host_alloc): on a
    # busy host, copies from registered pageable arrays slowed down several-fold
    pos, vel, d1, d2 = (M.host_array(a.shape) for a in arrs)
    for dst, src in zip((pos, vel, d1, d2), arrs):
        dst[...] = src
    del arrs

    def host_step(a, first):
        # the LPT displacements D1, D2 (P[].D, P[].D2) are fixed after the IC:
        # they travel with the first step of the run, later steps pass NULL
        # and the step keeps the device copy (mgp_step_host)
        t0 = time.perf_counter()
        ctx.step_host(*a, pos, vel, d1 if first else None, d2 if first else None)
        return time.perf_counter() - t0

    barrier()
    e2e_ms = [host_step(a, i == 0) * 1e3 for i, a in enumerate(schedule())]
    e2e_t = reduce_max(sum(e2e_ms) * 1e-3, dist)
    e2e_val = job_value(world, Np, nst, e2e_t)
    # per-stage events cost ~50 event records per KDK step on the host: with
    # steps of a few ms that is noise, but a launch-bound step of ~0.3 ms
    # would be slowed by them, so short steps take their stage times from one
    # extra run after the timed region instead
    stages_in_timed = warm_ms / nst >= 2.0
    barrier()
    run_ms, launches, per_step = [], 0, []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            ms, nl, st = run(timed=stages_in_timed)
            run_ms.append(ms)
            launches += nl
            if st is not None:
                per_step.append(st)
    barrier()
    if not per_step:
        per_step.append(run(timed=True)[2])
    elapsed = reduce_max(sum(run_ms) * 1e-3, dist)
    ms_per_run = elapsed / args.steps * 1e3
    value = job_value(world, Np, args.steps * nst, elapsed)
    # stage ms per KDK step, averaged over the timed runs, overall and per
    # decile of the schedule
    stage_ms = {k: float(np.mean([[st[i][k] for i in range(nst)] for st in per_step])) for k in STAGES}
    deciles = []
    for d in range(10):
        lo, hi = d * nst // 10, (d + 1) * nst // 10
        if hi > lo:
            row = {k: round(float(np.mean([[st[i][k] for i in range(lo, hi)] for st in per_step])), 4)
                   for k in STAGES + ["step"] if any(st[i][k] > 0 for st in per_step for i in range(lo, hi))}
            row["steps"] = [lo, hi - 1]
            deciles.append(row)

    # RSD multipoles P0/P2/P4 at z = 0 of that run's final state
    # (compute_RSD_powerspectrum, src/compute_pofk.c:403-512: y and z lines
    # of sight, averaged), timed end to end on the host (two
    # redshift-space deposits, two R2C, binning)
    ctx.kernel_ms("interp_kick_drift")  # synchronise before timing
    t0 = time.perf_counter()
    rsd = ctx.pofk_rsd(1.0)
    rsd_ms = (time.perf_counter() - t0) * 1e3
    for a in (pos, vel, d1, d2):
        M.host_free(a)
    full_check = None
    if rank == 0 and not args.no_cpu_baseline:
        full_check = fullsize_check(ctx, cfg, args.config, schedule)
    ctx.close()
    if closure is not None:
        closure.close()

    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"hbm_gbs": 6800.0}
    # stages that are one own kernel (the "mg" stage wraps two cuFFT calls)
    own = {k: v for k, v in stage_ms.items() if k in ("cic", "pofk", "forces", "interp_kick_drift") and v > 0}
    dom = max(own, key=own.get)
    abytes = algorithmic_bytes(N, Np, dom)
    achieved = abytes / (own[dom] * 1e-3) / 1e9
    peak = float(peaks.get("hbm_gbs", 6800.0))
    traffic = measured_traffic(cfg, N, Np, dom)
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic,
            "traffic_source": ("ncu DRAM bytes of one launch at step 46 of the 50-step nDGP run at 256^3 particles / "
                               "512^3 mesh (rate x duration), scaled by particles and cells") if traffic else
                              "no ncu capture of this kernel for this workload",
            "algorithmic_bytes_per_launch": abytes, "mean_launch_ms": round(own[dom], 4),
            "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback 6800 GB/s"}
    if closure is not None:
        conv_ms = stage_ms["closure_conv"]
        fl = closure_flops(N)
        tf = fl / (conv_ms * 1e-3) / 1e12
        bpeak = float(peaks.get("bf16_tflops_sustained", 1700.0))
        roof = {"bound": "tensor", "kernel": "closure_conv (4 conv launches of one forward)", "achieved": round(tf, 2),
                "peak": bpeak, "unit": "TFLOP/s", "frac": round(tf / bpeak, 4), "traffic": None,
                "algorithmic_flops_per_forward": fl, "conv_ms_per_step": round(conv_ms, 4),
                "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (kernel timed inside the step)"}
    # per KDK step positions and velocities in; D1, D2 with the first step of
    # the run only (scale-dependent growth: the step assigns its own fields)
    h2d = 2 * 12 * Np
    h2d_run = h2d * nst + (0 if cfg.get("sd") else 2 * 12 * Np)
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_run, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (2LPT IC generated on the device, seed %d)" % cfg["seed"],
        "config": {"workload": args.config, "particles": Np, "mesh": N, "box_mpc_h": cfg["Box"],
                   "model": model_name(cfg)
                   + (" + learned force closure (4x 3^3 conv, 16 ch, BF16/FP32 acc)" if closure is not None else ""),
                   "step": "one whole run: IC (untimed) + %d KDK steps z = 19 -> 0" % nst,
                   "kdk_steps_per_step": nst, "ms_per_kdk_step": round(ms_per_run / nst, 4),
                   "pofk_every_step": True, "pofk_bins": cfg["nbins"], "l2": "inputs larger than L2",
                   "parallelism": "replicas (one box per rank)" if world > 1 else "single GPU"},
        "e2e": {"value": round(e2e_val, 3), "unit": UNIT,
                "h2d_bytes_per_step": h2d_run, "d2h_bytes_per_step": 2 * 12 * Np * nst,
                "h2d_bytes_per_kdk_step": h2d, "d2h_bytes_per_kdk_step": 2 * 12 * Np,
                "h2d_once_per_run": "D1, D2 (the LPT displacements, fixed after the IC) with the first KDK step"
                                    if not cfg.get("sd") else None,
                "api": "mgp_step_host", "runs": 1,
                "kdk_step_ms": {"mean": round(float(np.mean(e2e_ms)), 2), "max": round(float(np.max(e2e_ms)), 2),
                                "min": round(float(np.min(e2e_ms)), 2)},
                "step_ms": [round(float(x), 1) for x in e2e_ms]},
        "gpu_launches": int(launches),
        "stage_ms_per_kdk_step": {k: round(v, 4) for k, v in stage_ms.items()},
        "stage_timing": "per-step CUDA events in the timed runs" if stages_in_timed else
                        "per-step CUDA events in one extra run after the timed region (steps < 2 ms)",
        "stage_ms_by_decile": deciles,
        "run_ms": [round(x, 2) for x in run_ms],
        "rsd_multipoles": {"ms": round(rsd_ms, 3), "bins": int(len(rsd[0])), "a": 1.0,
                           "los": "y and z, averaged (compute_RSD_powerspectrum)"},
        "roofline": roof,
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args)
        out["pofk_check"] = pofk_check(args.config)
        if full_check is not None:
            out["pofk_check_fullsize"] = full_check
    if rank == 0:
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


def run_closure_probe(args, cfg):
    """The closure network alone on an N^3 mesh (random features): each step
    is one forward (4 convolution layers) or, with train, one Adam step on
    N^3 random particles.  Used for the convolution kernels' profiles."""
    import mgpicola as M

    N = cfg["N"]
    rng = np.random.default_rng(1)
    x = rng.normal(0, 1, (N ** 3, 3)).astype(np.float32)
    with M.Closure(N, seed=3) as cl:
        cl.set_sample(x, None)
        if cfg.get("train"):
            cells = np.minimum(rng.uniform(0, N, (N ** 3, 3)).astype(np.float32), np.float32(N - 1e-3))
            cl.set_particle_sample(cells, rng.normal(0, 1, (N ** 3, 3)).astype(np.float32))
            work = lambda: cl.train_step(1e-4)  # noqa: E731
        else:
            work = cl.forward
        for _ in range(args.warmup):
            work()
        with ClockSampler(0) as clk:
            t0 = time.perf_counter()
            for _ in range(args.steps):
                work()
            wall = time.perf_counter() - t0
    fl = closure_flops(N) * (3 if cfg.get("train") else 1)
    print(json.dumps({"metric": "closure %s TFLOP/s" % ("training step" if cfg.get("train") else "forward"),
                      "value": round(fl * args.steps / wall / 1e12, 3), "unit": "TFLOP/s", "n_gpus": 1,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(wall / args.steps * 1e3, 3),
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
                      "data": "synthetic (random features)", "config": {"workload": args.config, "mesh": N},
                      "note": "host wall clock per call (each call synchronises); a profiling workload",
                      "clocks": clk.summary()}))


_KEEP = []


def oracle_params(O, cfg):
    rp = O.RunParams()
    sdkw = dict(scaledependent=1, **SD_GRID) if cfg.get("sd") else {}
    nu = None
    if cfg.get("nu"):
        nu = O.Neutrinos(nu_info(), 0.267, 0.049, 0.71, 0.96, 0.4, 1)
        _KEEP.append(nu)  # the oracle structs point at its tables
        sdkw["nu"] = nu
    if cfg["model"] == "dgp":
        rp.mg = O.make_mg(O.DGP, 0.267, rcH0=1.0, rsmooth=1.0)
    elif cfg["model"] == "fofr":
        rp.mg = O.make_mg(O.FOFR, 0.267, fofr0=1e-5, nfofr=1.0, **sdkw)
    else:
        rp.mg = O.make_mg(O.LCDM, 0.267, **sdkw)
    rp.pw = O.make_power(omega=0.267, omega_b=0.049, h=0.71, ns=0.96, sigma8=0.8, nu=nu)
    rp.ic = O.ICParams(cfg["N"], cfg["Ns"], cfg["Box"], cfg["seed"], 0, cfg["fixed"], 0, 1.0)
    rp.init_redshift = 19.0
    rp.nsteps = cfg["nsteps"]
    rp.final_redshift = 0.0
    rp.pofk_nbins, rp.pofk_bintype, rp.pofk_subtract_shotnoise = cfg["nbins"], 0, 1
    rp.pofk_kmin, rp.pofk_kmax = 2 * np.pi / cfg["Box"], np.pi * cfg["N"] / cfg["Box"]
    rp.usecola = 1
    return rp


SAMPLE = {"ndgp_512_1024": "ndgp_128_256", "ndgp_256_512": "ndgp_128_256", "lcdm_64_128": "lcdm_64_128",
          "lcdm_64_128_graph": "lcdm_64_128",
          "fofr_batch_64x64_128": "fofr_64_128", "closure_lcdm_256": "lcdm_128_128",
          "fofr_sd_256_512": "fofr_sd_64_128", "fofr_nu_256_512": "fofr_nu_64_128"}
CONFIGS["fofr_sd_64_128"] = dict(Ns=64, N=128, Box=128.0, model="fofr", nsteps=30, seed=5002, fixed=0, nbins=64,
                                 sd=True)
CONFIGS["fofr_nu_64_128"] = dict(Ns=64, N=128, Box=128.0, model="fofr", nsteps=30, seed=5002, fixed=0, nbins=64,
                                 sd=True, nu=True)
CONFIGS["fofr_64_128"] = dict(Ns=64, N=128, Box=256.0, model="fofr", nsteps=20, seed=6001, fixed=0, nbins=64)
CONFIGS["lcdm_128_128"] = dict(Ns=128, N=128, Box=128.0, model="lcdm", nsteps=30, seed=7017, fixed=0, nbins=64)
CONFIGS["ndgp_128_256"] = dict(Ns=128, N=256, Box=256.0, model="dgp", nsteps=50, seed=5003, fixed=1, nbins=128)


FIXTURE_CHECK = {"ndgp_512_1024": "ndgp_256_512_50", "ndgp_256_512": "ndgp_256_512_50"}


def pofk_check(config):
    """P(k) relative error against the FP64 oracle, stated with the throughput.
    For the nDGP workloads: the same model, seed and IC type at the workload's
    cell size (256^3 particles / 512^3 mesh, Box 512, the full 50-step
    schedule to z = 0) against the stored FP64 oracle run of that case
    (tests/golden/orc_ndgp_256_512_50.npz); for the others the same model at
    64^3 particles / 128^3 mesh, run to z = 0 on the GPU and through the
    oracle's KDK loop in this job.  The maximum |P_gpu / P_oracle - 1| over
    the bins with k <= 0.5 h/Mpc."""
    import mgpicola as M
    from oracle import oracle as O
    from tests.golden import oracle_runs as R

    fx = FIXTURE_CHECK.get(config)
    ref = R.load(fx) if fx else None
    if ref is not None:
        c = R.CASES[fx]
        with M.Context(R.gpu_params(M, c)) as ctx:
            k, pk, pos = R.gpu_run(ctx, c)
        out = R.compare(ref, k, pk, pos)
        out["case"] = ("%s at 256^3 particles / 512^3 mesh, Box 512, %d steps z = 19 -> 0, seed %d, vs the stored "
                       "FP64 oracle run (tests/golden/orc_%s.npz)" % (model_name(CONFIGS[config]), c["nsteps"],
                                                                     c["seed"], fx))
        out["max_rel_err"] = float("%.3g" % out["max_rel_err"])
        return out

    cfg = dict(CONFIGS[config], Ns=64, N=128, Box=256.0, nsteps=10, nbins=64)
    cfg.pop("closure", None)
    cfg.pop("batch", None)
    p = make_params(M, cfg)
    note = ""
    if cfg.get("sd"):
        # the oracle's IC rescaling is one number; with scale-dependent growth
        # mg_pofk_ratio depends on k, so both sides take P(k) as quoted
        p.input_pofk_is_for_lcdm = 0
        note = ", input P(k) quoted for the model"
    A0 = 1.0 / (1.0 + p.Init_Redshift)
    da = (1.0 - A0) / cfg["nsteps"]
    with M.Context(p) as ctx:
        ctx.displacement_fields()
        A, AI = A0, A0
        for _ in range(cfg["nsteps"]):
            ctx.step(A, AI, A + 0.5 * da, A + da)  # assigns the scale-dependent fields where needed
            A, AI = A + da, A + 0.5 * da
        ctx.get_displacements(A)
        k, pk, _, n = ctx.pofk(total=bool(cfg.get("nu")))
    rp = oracle_params(O, cfg)
    if p.modified_gravity_active and p.input_pofk_is_for_lcdm and not cfg.get("sd"):
        # the IC is rescaled by mg_pofk_ratio(k, 1), k-independent without
        # scale-dependent growth (2LPT.c:392-407)
        rp.ic.pofk_rescale = O.Cosmo(rp.mg, p.Init_Redshift).mg_pofk_ratio(0.1, 1.0)
    nb = p.pofk_nbins
    kb, po, km, nm = (np.zeros(max(nb, p.Nmesh)) for _ in range(4))
    n_o = O.lib().orc_run(rp, np.zeros((p.Nsample ** 3, 3)), np.zeros((p.Nsample ** 3, 3)), kb, po, km, nm)
    m = (nm[:n_o] > 0) & (kb[:n_o] <= 0.5) & (kb[:n_o] > 0)
    err = float(np.max(np.abs(pk[:n_o][m] / po[:n_o][m] - 1.0)))
    return {"max_rel_err": float("%.3g" % err), "k_max_h_mpc": 0.5, "bins": int(m.sum()),
            "case": "%s at 64^3 particles / 128^3 mesh, Box 256, 10 steps to z = 0, seed %d%s, vs the FP64 oracle"
                    % (model_name(cfg), cfg["seed"], note)}


def fullsize_check(ctx, cfg, config, schedule):
    """The 512^3 / 1024^3 workload itself against the stored FP64 oracle run
    of its first steps (tests/golden/orc_ndgp_512_1024_3.npz): the bench's
    own context redoes the IC and those steps."""
    from tests.golden import oracle_runs as R

    if config != "ndgp_512_1024":
        return None
    ref = R.load("ndgp_512_1024_3")
    if ref is None:
        return None
    c = R.CASES["ndgp_512_1024_3"]
    k, pk, pos = R.gpu_run(ctx, c)
    out = R.compare(ref, k, pk, pos)
    out["max_rel_err"] = float("%.3g" % out["max_rel_err"])
    out["case"] = ("the workload itself (512^3 / 1024^3, seed %d) at the start of step %d of its %d-step schedule vs "
                   "the stored FP64 oracle run (tests/golden/orc_ndgp_512_1024_3.npz)" % (c["seed"], c["stop"],
                                                                                         c["nsteps"]))
    return out


def cpu_baseline(args, nsteps=1):
    from oracle import oracle as O

    name = SAMPLE[args.config]
    cfg = CONFIGS[name]
    dt = O.lib().orc_time_steps(oracle_params(O, cfg), nsteps)
    Np = cfg["Ns"] ** 3
    return {"value": round(Np / dt / 1e6, 4), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": "%d full FP64 KDK step(s) of the same model at %d^3 particles / %d^3 mesh (Box %g) on %d "
                      "threads: OpenMP FFTs, CIC over x slabs with per-thread ghost slices and the other particle "
                      "and grid loops parallel, the reference's MPI-task shape; per-particle cost at 512^3/1024^3 "
                      "is higher (FFT ~ N^3 log N)" % (nsteps, cfg["Ns"], cfg["N"], cfg["Box"], os.cpu_count())}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O

    name = SAMPLE[args.config]
    cfg = CONFIGS[name]
    rp = oracle_params(O, cfg)
    if args.warmup > 0:
        O.lib().orc_time_steps(rp, 1)
    dt = O.lib().orc_time_steps(rp, max(1, args.steps))
    Np = cfg["Ns"] ** 3
    v = Np / dt / 1e6
    cb = {"value": round(v, 4), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
          "sample": "FP64 oracle KDK steps at %d^3 particles / %d^3 mesh, same model, %d threads (OpenMP FFTs, "
                    "CIC over x slabs with per-thread ghost slices, parallel particle and grid loops)"
                    % (cfg["Ns"], cfg["N"], os.cpu_count())}
    print(json.dumps({"metric": METRIC, "value": round(v, 4), "unit": UNIT, "n_gpus": 0, "steps": args.steps,
                      "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                      "config": {"workload": args.config, "sample": name}, "impl": "reference",
                      "cpu_baseline": cb,
                      "e2e": {"value": round(v, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="ndgp_512_1024", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one rank per GPU: start them under torch's launcher on this node
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(args.gpus),
               "--master-addr", "127.0.0.1", "--master-port", os.environ.get("MGP_BENCH_PORT", "29533"),
               os.path.abspath(__file__)] + sys.argv[1:]
        sys.exit(subprocess.call(cmd))
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

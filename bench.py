"""Benchmark of the COLA particle-mesh step on GB300.

Workload (default): nDGP, rc*H0 = 1, density screening on (Gaussian filter,
Rsmooth 1 Mpc/h), 512^3 particles on a 1024^3 mesh, Box 1024 Mpc/h, 50
linear-in-a steps from z = 19, seed 5003, amplitude-fixed 2LPT initial
conditions, P(k) every step in 512 linear bins over [2 pi/Box, k_Nyquist].
A step is one KDK step: CIC deposit, R2C, P(k) binning, fifth force (smoothing
C2R, screening, R2C), force k-space pass, three C2R, fused interpolation +
kick + drift.  Inputs are synthetic (generated by the IC on the device);
the working set (~50 GB) is far larger than L2, so no L2 flush is needed.

value: Mparticle-steps/s with the particle state resident in HBM.
e2e:   the same metric through the host-buffer C-ABI call mgp_step_host
       (pinned host particle arrays copied in and out every step).
--impl reference: the FP64 CPU oracle (restatement of the reference's C
       code) timed on the host cores on a bounded sample of the workload.
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


def run_batch(args, cfg):
    """A batch of independent boxes: each timed step is one graph launch that
    runs the whole KDK loop of every box; value counts particle-steps of all
    boxes (drift steps; the final output kick is included in the time)."""
    import mgpicola as M

    p = make_params(M, cfg)
    boxes = batch_boxes(cfg)
    B, Np, nst = len(boxes), cfg["Ns"] ** 3, cfg["nsteps"]
    batch = M.Batch(p, boxes)
    default_tuning = batch.tuning()
    batch.run(nst)
    default_ms = batch.ms(0)
    tune_t0 = time.perf_counter()
    tuned_ms = batch.autotune(nst)  # launch budgets picked by timing, before the timed region
    tune_s = time.perf_counter() - tune_t0
    tuning = batch.tuning()
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
    ms = float(np.mean(times))
    value = B * Np * nst / (ms * 1e-3) / 1e6
    wall = float(np.mean(walls))
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
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / nst, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": ("synthetic (2LPT ICs generated on the device, seeds %d-%d normal + inverted)"
                 % (cfg["seed"], cfg["seed"] + B // 2 - 1) if B > 1 else
                 "synthetic (2LPT IC generated on the device, seed %d)" % cfg["seed"]),
        "config": {"workload": args.config, "boxes": B, "particles_per_box": Np, "mesh": N, "box_mpc_h": cfg["Box"],
                   "model": ("f(R) Hu-Sawicki n=1, screening, |fR0| log-uniform [1e-6, 1e-4] (seed %d)" % BATCH_FR0_SEED
                             if B > 1 else model_name(cfg)),
                   "steps_per_run": nst, "pofk_every_step": True, "pofk_bins": cfg["nbins"],
                   "launch_budgets": {"tuned": tuning, "default": default_tuning,
                                      "order": "blocks/SM: CIC deposit, grid passes, kick, P(k) binning",
                                      "autotune_s": round(tune_s, 2), "graph_ms_default": round(default_ms, 3),
                                      "graph_ms_tuned": round(tuned_ms, 3)},
                   "l2": "working set %.1f GB > L2" % (B * (6 * 4 * N * N * 2 * (N // 2 + 1) + 48 * Np) / 1e9)},
        "e2e": {"value": round(B * Np * nst / wall / 1e6, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(B * cfg["nbins"] * 8 / nst), "api": "mgp_batch_run + mgp_batch_pofk",
                "includes": "2LPT ICs of all boxes, graph launch, per-box P(k) read-back"},
        "gpu_launches": int(launches * args.steps),
        "graph": {"launches_per_run": 1, "nodes": nodes, "own_kernels": launches, "ic_ms": round(ic_ms, 3)},
        "per_box_completion_ms": {"p50": round(ms, 3), "p99": round(ms, 3),
                                  "note": "lock step: every box finishes with the graph"},
        "roofline": {"bound": "hbm", "kernel": "whole step (FFTs included)", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": None,
                     "algorithmic_bytes_per_step": abytes, "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args)
        out["pofk_check"] = pofk_check(args.config)
    print(json.dumps(out))


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
        "interp_kick_drift": 12 * N ** 3 + 72 * Np,   # force grids once; s,v,D1,D2 in, s,v out
        "mg": 8 * ncomplex + 4 * nreal + 8 * nreal,   # smoothing pass + screening pass (excl. FFTs)
    }[kernel]


# DRAM bytes per launch measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum) on the
# nDGP step at 256^3 particles / 512^3 mesh, one launch each from a steady step.  Every term of
# these kernels scales with the particle count or the cell count, which grow together between
# the configurations (Nmesh = 2 Nsample), so the figure is scaled by the cell count.
TRAFFIC_256_512 = {"interp_kick_drift": 3.404e9, "forces": 2.655e9, "cic": 1.466e9, "pofk": 1.040e9}


def measured_traffic(N, Np, kernel):
    if kernel not in TRAFFIC_256_512 or Np * 8 != N ** 3:
        return None
    return int(TRAFFIC_256_512[kernel] * (N / 512.0) ** 3)


def run_gpu(args):
    import mgpicola as M

    # flush dirty pages left by earlier work on this host (snapshot files)
    # before the timed regions: their write-back competes with the
    # host-buffer copies of the e2e leg
    os.sync()

    cfg = CONFIGS[args.config]
    if cfg.get("batch"):
        return run_batch(args, cfg)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    p = make_params(M, cfg)
    p.Seed = rank_seed(cfg, rank)
    Np = cfg["Ns"] ** 3
    N = cfg["N"]
    ctx = M.Context(p, device=local if world > 1 else 0)
    closure = None
    if cfg.get("closure"):
        closure = M.Closure(N, seed=cfg["seed"], device=local if world > 1 else 0)  # He-normal init weights
        closure.attach(ctx)
    ctx.displacement_fields()
    A0 = 1.0 / (1.0 + p.Init_Redshift)
    da = (1.0 - A0) / cfg["nsteps"]
    state = {"A": A0, "AI": A0}

    def step():
        A, AI = state["A"], state["AI"]
        AF, AFF = A + 0.5 * da, A + da
        ctx.step(A, AI, AF, AFF)
        state["A"], state["AI"] = AFF, AF

    def sync():
        # mgp_kernel_ms synchronises the context stream on its last event
        ctx.kernel_ms("interp_kick_drift")

    def barrier():
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        step()
    ctx.set_timing(True)
    sync()
    barrier()
    launches0 = ctx.launches()
    stage_ms = {k: 0.0 for k in ["fill", "cic", "r2c", "pofk", "mg", "forces", "c2r", "interp_kick_drift", "lpt_fields",
                                 "closure", "closure_conv"]}
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        dev_ms = 0.0
        for _ in range(args.steps):
            step()
            dev_ms += ctx.kernel_ms("step")  # CUDA events around the whole step
            for k in stage_ms:
                v = ctx.kernel_ms(k)
                if v > 0:
                    stage_ms[k] += v
        wall = time.perf_counter() - t0
    elapsed = dev_ms * 1e-3
    launches = ctx.launches() - launches0
    barrier()
    elapsed = reduce_max(elapsed, dist)
    ms_per_step = elapsed / args.steps * 1e3
    value = job_value(world, Np, args.steps, elapsed)

    # e2e through the host-buffer C-ABI entry point, pinned host memory
    ctx.set_timing(False)
    pos, vel, d1, d2 = ctx.get_particles()
    for a in (pos, vel, d1, d2):
        M.pin(a)
    e2e_steps = max(1, min(args.steps, 10))

    def host_step():
        A, AI = state["A"], state["AI"]
        AF, AFF = A + 0.5 * da, A + da
        t0 = time.perf_counter()
        ctx.step_host(A, AI, AF, AFF, pos, vel, d1, d2)
        state["A"], state["AI"] = AFF, AF
        return time.perf_counter() - t0

    host_step()  # untimed: allocates the staging buffers and the copy stream
    barrier()
    e2e_ms = [host_step() * 1e3 for _ in range(e2e_steps)]
    e2e_t = reduce_max(sum(e2e_ms) * 1e-3, dist)
    for a in (pos, vel, d1, d2):
        M.unpin(a)
    e2e_val = job_value(world, Np, e2e_steps, e2e_t)
    # RSD multipoles P0/P2/P4 of the final state (compute_RSD_powerspectrum,
    # src/compute_pofk.c:403-512: y and z lines of sight, averaged), timed
    # end to end on the host (two redshift-space deposits, two R2C, binning)
    ctx.kernel_ms("interp_kick_drift")  # synchronise before timing
    t0 = time.perf_counter()
    rsd = ctx.pofk_rsd(state["A"])
    rsd_ms = (time.perf_counter() - t0) * 1e3
    ctx.close()
    if closure is not None:
        closure.close()

    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"hbm_gbs": 6800.0}
    # stages that are one own kernel (the "mg" stage wraps two cuFFT calls)
    own = {k: v / args.steps for k, v in stage_ms.items() if k in ("cic", "pofk", "forces", "interp_kick_drift")}
    dom = max(own, key=own.get)
    abytes = algorithmic_bytes(N, Np, dom)
    achieved = abytes / (own[dom] * 1e-3) / 1e9
    peak = float(peaks.get("hbm_gbs", 6800.0))
    traffic = measured_traffic(N, Np, dom)
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum at 256^3 particles / "
                              "512^3 mesh, scaled by particles and cells",
            "algorithmic_bytes_per_launch": abytes, "peak_source": "MEASURED_PEAKS.json hbm_gbs"}
    if closure is not None:
        conv_ms = stage_ms["closure_conv"] / args.steps
        fl = closure_flops(N)
        tf = fl / (conv_ms * 1e-3) / 1e12
        bpeak = float(peaks.get("bf16_tflops_sustained", 1700.0))
        roof = {"bound": "tensor", "kernel": "closure_conv (4 conv launches of one forward)", "achieved": round(tf, 2),
                "peak": bpeak, "unit": "TFLOP/s", "frac": round(tf / bpeak, 4), "traffic": None,
                "algorithmic_flops_per_forward": fl, "conv_ms_per_step": round(conv_ms, 4),
                "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (kernel timed inside the step)"}
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (2LPT IC generated on the device, seed 5003)",
        "config": {"workload": args.config, "particles": Np, "mesh": N, "box_mpc_h": cfg["Box"],
                   "model": model_name(cfg)
                   + (" + learned force closure (4x 3^3 conv, 16 ch, BF16/FP32 acc)" if closure is not None else ""),
                   "pofk_every_step": True, "pofk_bins": cfg["nbins"], "l2": "inputs larger than L2",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": round(e2e_val, 3), "unit": UNIT,
                # scale-dependent growth: the step assigns its own D1/D2, only pos/vel go up
                "h2d_bytes_per_step": (2 if cfg.get("sd") else 4) * 12 * Np,
                "d2h_bytes_per_step": 2 * 12 * Np, "api": "mgp_step_host",
                "step_ms": [round(x, 2) for x in e2e_ms]},
        "gpu_launches": int(launches),
        "stage_ms_per_step": {k: round(v / args.steps, 4) for k, v in stage_ms.items()},
        "rsd_multipoles": {"ms": round(rsd_ms, 3), "bins": int(len(rsd[0])), "a": round(state["A"], 5),
                           "los": "y and z, averaged (compute_RSD_powerspectrum)"},
        "roofline": roof,
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args)
        out["pofk_check"] = pofk_check(args.config)
    if rank == 0:
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


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


def pofk_check(config):
    """P(k) relative error against the FP64 oracle, stated with the throughput:
    the same model, seed and IC type at 64^3 particles / 128^3 mesh (the
    512^3/1024^3 run is far beyond what the FP64 oracle can redo on the host),
    run to z = 0 on the GPU and through the oracle's KDK loop; the maximum
    |P_gpu / P_oracle - 1| over the bins with k <= 0.5 h/Mpc."""
    import mgpicola as M
    from oracle import oracle as O

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


def cpu_baseline(args, nsteps=1):
    from oracle import oracle as O

    name = SAMPLE[args.config]
    cfg = CONFIGS[name]
    dt = O.lib().orc_time_steps(oracle_params(O, cfg), nsteps)
    Np = cfg["Ns"] ** 3
    return {"value": round(Np / dt / 1e6, 4), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": "%d full FP64 KDK step(s) of the same model at %d^3 particles / %d^3 mesh (Box %g), "
                      "OpenMP FFTs on all host cores, serial CIC/interp as the reference; per-particle cost at "
                      "512^3/1024^3 is higher (FFT ~ N^3 log N)" % (nsteps, cfg["Ns"], cfg["N"], cfg["Box"])}


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
          "sample": "FP64 oracle KDK steps at %d^3 particles / %d^3 mesh, same model" % (cfg["Ns"], cfg["N"])}
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
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

"""FP64 oracle runs at the benchmark workloads' sizes, stored as fixtures.

The GPU tests and bench.py's P(k) check compare the CUDA path against these
files, so the long FP64 runs are made once (on a host with the memory for
them) instead of in every test session.  Cases:

  ndgp_256_512_50   nDGP rcH0 = 1 with density screening (Gaussian filter,
                    Rsmooth 1 Mpc/h), 256^3 particles / 512^3 mesh, Box 512
                    Mpc/h (the 512^3/1024^3 workload's cell size and model),
                    the full 50-step schedule from z = 19 to z = 0, seed 5003,
                    amplitude-fixed 2LPT ICs, P(k) at z = 0 in 256 linear bins
                    [2 pi/Box, k_Nyquist], shot noise subtracted.
  ndgp_512_1024_3   the 512^3 particle / 1024^3 mesh workload itself (Box
                    1024, 512 bins, its 50-step schedule), stopped at the
                    start of step 3 after that step's density and P(k).
                    Needs ~80 GB of host memory.

Each file holds the P(k) table (bin k, P, mean k, modes), a subsample of
the particle positions (every `stride`-th particle in lattice order) and
the case parameters.  Run from the repository root:

    python tests/golden/oracle_runs.py ndgp_256_512_50 [ndgp_512_1024_3]
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# name: (Ns, N, Box, nsteps of the schedule, stop_step (0 = run to z = 0), bins, seed, particle stride)
CASES = {
    "ndgp_256_512_50": dict(Ns=256, N=512, Box=512.0, nsteps=50, stop=0, nbins=256, seed=5003, stride=509),
    "ndgp_512_1024_3": dict(Ns=512, N=1024, Box=1024.0, nsteps=50, stop=3, nbins=512, seed=5003, stride=4093),
}
# the nDGP model and cosmology of the workloads
COSMO = dict(Omega=0.267, OmegaBaryon=0.049, HubbleParam=0.71, Sigma8=0.8, PrimordialIndex=0.96)
INIT_REDSHIFT = 19.0


def path(name):
    return os.path.join(ROOT, "tests", "golden", "orc_%s.npz" % name)


def oracle_params(O, c):
    rp = O.RunParams()
    rp.mg = O.make_mg(O.DGP, COSMO["Omega"], rcH0=1.0, rsmooth=1.0)
    rp.pw = O.make_power(omega=COSMO["Omega"], omega_b=COSMO["OmegaBaryon"], h=COSMO["HubbleParam"],
                         ns=COSMO["PrimordialIndex"], sigma8=COSMO["Sigma8"])
    # amplitude-fixed IC; the P(k) is quoted for LCDM and rescaled by
    # mg_pofk_ratio(k, 1), k-independent without scale-dependent growth
    # (2LPT.c:392-407)
    rp.ic = O.ICParams(c["N"], c["Ns"], c["Box"], c["seed"], 0, 1, 0, 1.0)
    rp.ic.pofk_rescale = O.Cosmo(rp.mg, INIT_REDSHIFT).mg_pofk_ratio(0.1, 1.0)
    rp.init_redshift = INIT_REDSHIFT
    rp.nsteps = c["nsteps"]
    rp.final_redshift = 0.0
    rp.pofk_nbins, rp.pofk_bintype, rp.pofk_subtract_shotnoise = c["nbins"], 0, 1
    rp.pofk_kmin, rp.pofk_kmax = 2 * np.pi / c["Box"], np.pi * c["N"] / c["Box"]
    rp.usecola = 1
    rp.stop_step = c["stop"]
    return rp


def run(name):
    from oracle import oracle as O

    c = CASES[name]
    rp = oracle_params(O, c)
    n = c["Ns"] ** 3
    pos, vel = np.zeros((n, 3)), np.zeros((n, 3))
    cap = max(c["nbins"], c["N"])
    kb, pk, km, nm = (np.zeros(cap) for _ in range(4))
    t0 = time.time()
    nb = O.lib().orc_run(rp, pos, vel, kb, pk, km, nm)
    dt = time.time() - t0
    idx = np.arange(0, n, c["stride"])
    np.savez(path(name), k=kb[:nb], pk=pk[:nb], kmean=km[:nb], nmodes=nm[:nb], idx=idx, pos=pos[idx],
             oracle_seconds=dt, threads=os.cpu_count(), **c)
    print(name, "bins", nb, "oracle %.1f s" % dt)


def gpu_params(M, c):
    """mgp_params of the same case (the nDGP workload's parameter keys)."""
    return M.default_params(
        Nmesh=c["N"], Nsample=c["Ns"], Box=c["Box"], Seed=c["seed"], Init_Redshift=INIT_REDSHIFT,
        amplitude_fixed_initial_condition=1, pofk_compute_every_step=1, pofk_nbins=c["nbins"], pofk_bintype=0,
        pofk_kmin=2 * np.pi / c["Box"], pofk_kmax=np.pi * c["N"] / c["Box"], pofk_subtract_shotnoise=1,
        WhichSpectrum=2, UseCOLA=1, model=M.MODEL_DGP, modified_gravity_active=1, include_screening=1,
        rcH0_DGP=1.0, Rsmooth=1.0, smoothing_filter=M.FILTER_GAUSSIAN, input_pofk_is_for_lcdm=1,
        input_sigma8_is_for_lcdm=1, **COSMO)


def gpu_run(ctx, c):
    """The case on a context made from gpu_params: IC, the steps of the
    schedule up to the stop, the density and P(k) there.  Returns (k, P,
    positions of the stored subsample)."""
    A0 = 1.0 / (1.0 + INIT_REDSHIFT)
    da = (1.0 - A0) / c["nsteps"]
    ctx.displacement_fields()
    A, AI = A0, A0
    for _ in range(c["stop"] or c["nsteps"]):
        ctx.step(A, AI, A + 0.5 * da, A + da)
        A, AI = A + da, A + 0.5 * da
    ctx.get_displacements(A)
    k, pk, _, _ = ctx.pofk()
    pos = ctx.get_particles()[0]
    return k, pk, pos[np.arange(0, c["Ns"] ** 3, c["stride"])]


def compare(ref, k, pk, pos, kmax=0.5):
    """Largest |P/P_oracle - 1| over the bins with modes and 0 < k <= kmax,
    and the rms position difference (periodic) in units of the particle
    spacing."""
    n = len(ref["pk"])
    m = (ref["nmodes"] > 0) & (ref["k"] > 0) & (ref["k"] <= kmax)
    err = float(np.max(np.abs(pk[:n][m] / ref["pk"][m] - 1.0)))
    box = float(ref["Box"])
    dx = np.abs(pos.astype(np.float64) - ref["pos"])
    dx = np.minimum(dx, box - dx)
    rms = float(np.sqrt(np.mean(dx ** 2)) / (box / int(ref["Ns"])))
    return {"max_rel_err": err, "bins": int(m.sum()), "k_max_h_mpc": kmax, "pos_rms_over_spacing": rms,
            "particles_compared": int(len(ref["pos"]))}


def load(name):
    """The stored run as a dict, or None when the file has not been made."""
    if not os.path.exists(path(name)):
        return None
    f = np.load(path(name))
    return {k: f[k] for k in f.files}


if __name__ == "__main__":
    for name in sys.argv[1:] or ["ndgp_256_512_50"]:
        run(name)

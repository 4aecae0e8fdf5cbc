"""Training and evaluation driver of the learned force closure.

Training data come from the method itself: for each training seed the same
2LPT initial conditions are run with a mesh r times finer than the target
mesh; at chosen steps the fine run's particles are also put on the coarse
mesh, and the sample is (coarse-mesh features, per-particle fine force minus
coarse force); the loss compares that residual with the network output
interpolated to the particles, i.e. as the kick uses it.  The network is trained on those
samples with Adam on the GPU (mgp_closure_train_step); it is evaluated by
running held-out seeds on the coarse mesh with and without the closure and
comparing their final P(k), measured on the coarse mesh, with the fine run's
particles measured on the same mesh.
"""
import time

import numpy as np

import mgpicola as M


def run_params(N, Ns, box, seed, model, nbins, fofr0=1e-5, zi=19.0):
    kw = dict(Nmesh=N, Nsample=Ns, Box=box, Seed=seed, Init_Redshift=zi, pofk_compute_every_step=0,
              pofk_nbins=nbins, pofk_bintype=0, pofk_kmin=2 * np.pi / box, pofk_kmax=np.pi * N / box,
              pofk_subtract_shotnoise=1, Omega=0.267, OmegaBaryon=0.049, HubbleParam=0.71, Sigma8=0.8,
              PrimordialIndex=0.96, WhichSpectrum=2, UseCOLA=1)
    if model == "fofr":
        kw.update(model=M.MODEL_FOFR, modified_gravity_active=1, include_screening=1, fofr0=fofr0, nfofr=1.0,
                  input_pofk_is_for_lcdm=1, input_sigma8_is_for_lcdm=1)
    return M.default_params(**kw)


def schedule(nsteps, zi=19.0, zf=0.0):
    """(A, AI, AF, AFF) of each KDK step of main.c:394-611 for one output."""
    A0, ao = 1.0 / (1.0 + zi), 1.0 / (1.0 + zf)
    da = (ao - A0) / nsteps
    A, AI, out = A0, A0, []
    for _ in range(nsteps):
        out.append((A, AI, A + 0.5 * da, A + da))
        A, AI = A + da, A + 0.5 * da
    return out, A, AI


def collect(cl, seed, model, Nc, r, Ns, box, nsteps, snaps, slot, band=True):
    """Run the fine mesh for one seed and store a sample at each step in
    `snaps`; returns the next free slot, the targets' rms values and the
    samples' scale factors."""
    rms, avals = [], []
    with M.Context(run_params(Nc * r, Ns, box, seed, model, 64)) as fine, \
            M.Context(run_params(Nc, Ns, box, seed, model, 64)) as coarse:
        fine.displacement_fields()
        steps, _, _ = schedule(nsteps)
        for ts, (A, AI, AF, AFF) in enumerate(steps):
            fine.get_displacements(A)
            if ts in snaps:
                pos, vel, _, _ = fine.get_particles()
                coarse.set_particles(pos, vel)
                coarse.get_displacements(A)
                cl.features(coarse, A)
                rms.append(cl.target_particles(fine, coarse, band=band))
                avals.append(A)
                cl.store(slot)
                slot += 1
            fine.kick_drift(AI, AF, A, AFF, drift=True)
    return slot, rms, avals


def scale_table(rms, avals):
    """Residual rms per snapshot scale factor (rms over the seeds)."""
    a = np.asarray(avals)
    r = np.asarray(rms)
    ua = np.unique(a)
    return ua, np.array([np.sqrt(np.mean(r[a == u] ** 2)) for u in ua])


def train(cl, nsamples, epochs, lr0, seed=0, log=None):
    rng = np.random.default_rng(seed)
    hist = []
    it, total = 0, epochs * nsamples
    for ep in range(epochs):
        losses = []
        for s in rng.permutation(nsamples):
            lr = lr0 * 0.5 * (1.0 + np.cos(np.pi * it / total))  # cosine decay
            cl.load(int(s))
            losses.append(cl.train_step(lr))
            it += 1
        hist.append(float(np.mean(losses)))
        if log:
            log("epoch %d loss %.4e" % (ep, hist[-1]))
    return hist


def final_particles(p, nsteps, closure=None):
    """Run IC + nsteps KDK steps + the output kick; returns pos, vel and the
    wall time of the steps (IC excluded)."""
    with M.Context(p) as ctx:
        if closure is not None:
            closure.attach(ctx)
        ctx.displacement_fields()
        steps, A, AI = schedule(nsteps)
        t0 = time.perf_counter()
        for (A_, AI_, AF, AFF) in steps:
            ctx.get_displacements(A_)
            ctx.kick_drift(AI_, AF, A_, AFF, drift=True)
        ctx.get_displacements(A)
        ctx.kick_drift(AI, A, A, A, drift=False)
        pos, vel, _, _ = ctx.get_particles()
        dt = time.perf_counter() - t0
        if closure is not None:
            M.Closure.detach(ctx)
    return pos, vel, dt


def pofk_on_mesh(p, pos, vel):
    """P(k) of the given particles deposited on p's mesh at a = 1."""
    with M.Context(p) as ctx:
        ctx.set_particles(pos, vel)
        ctx.get_displacements(1.0)
        return ctx.pofk()


def k_within(k, ratio, tol):
    """Largest k up to which every bin's |P/P_fine - 1| stays <= tol."""
    ok = np.abs(ratio - 1.0) <= tol
    bad = np.nonzero(~ok)[0]
    if len(bad) == 0:
        return float(k[-1]) if len(k) else 0.0
    return float(k[bad[0] - 1]) if bad[0] > 0 else 0.0


def evaluate(cl, seed, model, Nc, r, Ns, box, nsteps, kmax=1.0):
    pc = run_params(Nc, Ns, box, seed, model, Nc // 2)
    pf = run_params(Nc * r, Ns, box, seed, model, Nc // 2)
    posf, velf, tf = final_particles(pf, nsteps)
    posc, velc, tc = final_particles(pc, nsteps)
    posn, veln, tn = final_particles(pc, nsteps, closure=cl)
    k, pkf, _, nf = pofk_on_mesh(pc, posf, velf)
    _, pkc, _, _ = pofk_on_mesh(pc, posc, velc)
    _, pkn, _, _ = pofk_on_mesh(pc, posn, veln)
    m = (nf > 0) & (k <= kmax) & (k > 0)
    return dict(k=k[m], fine=pkf[m], plain=pkc[m], closure=pkn[m],
                err_plain=float(np.max(np.abs(pkc[m] / pkf[m] - 1))),
                err_closure=float(np.max(np.abs(pkn[m] / pkf[m] - 1))),
                t_fine=tf, t_plain=tc, t_closure=tn)


def run_c5(model, Nc=256, r=3, box=256.0, nsteps=30, train_seeds=range(7001, 7017), test_seeds=range(7017, 7021),
           every=3, epochs=16, lr=2e-3, kmax=1.0, tol=0.01, band=True, net_seed=5, log=print, weights_out=None,
           highpass=None):
    """Learned-closure workload: collect training samples from the fine and
    coarse meshes of `train_seeds`, train, and evaluate on `test_seeds` by the
    final P(k) against the fine mesh.  The closure is accepted up to the k
    where its error stays within `tol`; beyond that the plain force is the
    result."""
    Ns = Nc
    snaps = set(range(0, nsteps, every)) | {nsteps - 1}
    out = dict(model=model, Nmesh=Nc, Nmesh_fine=r * Nc, Nsample=Ns, Box=box, nsteps=nsteps, epochs=epochs, lr=lr,
               band_limited_target=band, train_seeds=list(train_seeds), test_seeds=list(test_seeds), tol=tol, kmax=kmax)
    with M.Closure(Nc, seed=net_seed) as cl:
        if highpass is not None:
            cl.set_highpass(highpass)
        cl.reserve(len(train_seeds) * len(snaps), Ns ** 3)
        t0 = time.perf_counter()
        slot, rms, avals = 0, [], []
        for sd in train_seeds:
            slot, rr, aa = collect(cl, sd, model, Nc, r, Ns, box, nsteps, snaps, slot, band=band)
            rms += rr
            avals += aa
        out["collect_s"] = time.perf_counter() - t0
        out["samples"] = slot
        ta, ts = scale_table(rms, avals)
        cl.set_scale_table(ta, ts)  # the step scales the output by the residual rms at its a
        out["scale_table"] = [ta.tolist(), ts.tolist()]
        t0 = time.perf_counter()
        hist = train(cl, slot, epochs, lr, log=log)
        out["train_s"] = time.perf_counter() - t0
        out["train_steps"] = epochs * slot
        out["loss_over_var"] = hist  # each sample's loss is relative to its own mean square target
        out["highpass_lambda_cells"] = cl.highpass()
        if weights_out:
            w, b, sc = cl.weights()
            np.savez(weights_out, w=w, b=b, scale_a=ta, scale_s=ts, highpass_lambda_cells=cl.highpass())
        evs = []
        for sd in test_seeds:
            ev = evaluate(cl, sd, model, Nc, r, Ns, box, nsteps, kmax=kmax)
            rp, rc = ev["plain"] / ev["fine"], ev["closure"] / ev["fine"]
            evs.append(dict(seed=sd, err_plain=ev["err_plain"], err_closure=ev["err_closure"],
                            k_within_tol_plain=k_within(ev["k"], rp, tol), k_within_tol_closure=k_within(ev["k"], rc, tol),
                            t_fine_s=ev["t_fine"], t_plain_s=ev["t_plain"], t_closure_s=ev["t_closure"],
                            k=ev["k"].tolist(), ratio_plain=rp.tolist(), ratio_closure=rc.tolist()))
            log("seed %d: max |P/P_fine-1| to k=%.1f plain %.4f closure %.4f; within %.0f%% to k=%.3f (plain %.3f)"
                % (sd, kmax, ev["err_plain"], ev["err_closure"], 100 * tol, evs[-1]["k_within_tol_closure"],
                   evs[-1]["k_within_tol_plain"]))
        out["eval"] = evs
        out["accepted_to_kmax"] = all(e["err_closure"] <= tol for e in evs)
    return out


def main(argv=None):
    import argparse
    import json

    ap = argparse.ArgumentParser(description="train and evaluate the learned force closure")
    ap.add_argument("--model", default="lcdm", choices=["lcdm", "fofr"])
    ap.add_argument("--nmesh", type=int, default=256)
    ap.add_argument("--ntrain", type=int, default=16)
    ap.add_argument("--ntest", type=int, default=4)
    ap.add_argument("--epochs", type=int, default=16)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--every", type=int, default=3)
    ap.add_argument("--full-target", action="store_true", help="do not band-limit the fine force")
    ap.add_argument("--highpass", type=float, default=None,
                    help="cutoff wavelength (cells) of the closure output's high-pass")
    ap.add_argument("--out", default=None, help="JSON report")
    ap.add_argument("--weights", default=None, help=".npz for the trained weights")
    a = ap.parse_args(argv)
    rep = run_c5(a.model, Nc=a.nmesh, box=float(a.nmesh), train_seeds=range(7001, 7001 + a.ntrain),
                 test_seeds=range(7017, 7017 + a.ntest), every=a.every, epochs=a.epochs, lr=a.lr,
                 band=not a.full_target, weights_out=a.weights, highpass=a.highpass)
    if a.out:
        with open(a.out, "w") as f:
            json.dump(rep, f, indent=1)
    return rep


if __name__ == "__main__":
    main()

"""Generate golden fixtures from MG-PICOLA's own code (run here).

Builds the reference's unmodified C sources against the single-rank shims
(oracle/ref_build.py), runs small COLA simulations for each model and stores
the final P(k) table and a subsample of the final GADGET snapshot in
tests/golden/ref_<case>.npz.  tests/test_golden.py checks the FP64 oracle
against these files.  The white-noise stream in both is the project's Philox
stand-in for GSL's ranlxd1 (the shim's gsl_rng_uniform), so the runs share
identical initial conditions.

Run from the repository root, with MGP_REFERENCE_SRC set to the reference's
src/ directory:  MGP_REFERENCE_SRC=<reference>/src python tests/golden/make_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import ref_build  # noqa: E402
from tests.golden import camb_tables, particle_files, spectrum_table  # noqa: E402

BASE = dict(Nmesh=32, Nsample=16, Box=128.0, Init_Redshift=19.0, Seed=4242, nsteps=5, rsd=0, nbins=16, bintype=0,
            shotnoise=0, kmin=0.0, kmax=0.0, cola=1, z1steps=0, sphere=0, pofk_lcdm=0, s8_lcdm=1, lcdm_growth=0,
            which_spectrum=2, which_transfer=0, unit_length=3.085678e24, input_unit_length=3.085678e24)
COSMO = dict(Omega=0.267, OmegaBaryon=0.049, HubbleParam=0.71, Sigma8=0.8, PrimordialIndex=0.96)

CASES = {
    # case: (binary model, MG keys)
    "lcdm": ("FOFR_LCDM", dict(modified_gravity_active=0, fofr0=1e-5, nfofr=1.0, include_screening=1)),
    "fofr": ("FOFR_LCDM", dict(modified_gravity_active=1, fofr0=1e-5, nfofr=1.0, include_screening=1)),
    "fofr_nosc": ("FOFR_LCDM", dict(modified_gravity_active=1, fofr0=1e-5, nfofr=1.0, include_screening=0)),
    "dgp": ("DGP", dict(modified_gravity_active=1, rcH0_DGP=1.0, Rsmooth=1.0, include_screening=1)),
    "jbd": ("BRANSDICKE", dict(modified_gravity_active=1, wBD=100.0, Omegah2=0.14, Omegar2=4e-5, Omegav2=0.36,
                               include_screening=1)),
    "mbeta": ("MBETA_LCDM", dict(modified_gravity_active=1, range_symm=1.0, assb_symm=0.5, beta_symm=1.0,
                                 include_screening=1)),
    "lcdm_fixed_inv": ("FOFR_LCDM", dict(modified_gravity_active=0, fofr0=1e-5, nfofr=1.0, include_screening=1,
                                         amplitude_fixed_initial_condition=1, inverted_initial_condition=1)),
    # SCALEDEPENDENT builds: growth factors D(k, a) from 2D tables
    "fofr_sd": ("FOFR", dict(modified_gravity_active=1, fofr0=1e-5, nfofr=1.0, include_screening=1)),
    "mbeta_sd": ("MBETA", dict(modified_gravity_active=1, range_symm=1.0, assb_symm=0.5, beta_symm=1.0,
                               include_screening=1)),
    # MASSIVE_NEUTRINOS build (scale dependent) on the synthetic CAMB tables
    # of camb_tables.py: P(k) of CDM+baryons and of the total matter field
    "lcdm_nu": ("FOFRNU", dict(modified_gravity_active=0, fofr0=1e-5, nfofr=1.0, include_screening=1,
                               nu_include_massive_neutrinos=1, nu_SumMassNuEV=camb_tables.SUM_MNU_EV)),
    "fofr_nu": ("FOFRNU", dict(modified_gravity_active=1, fofr0=1e-5, nfofr=1.0, include_screening=1,
                               nu_include_massive_neutrinos=1, nu_SumMassNuEV=camb_tables.SUM_MNU_EV)),
    # redshift-space multipoles (compute_RSD_powerspectrum): at the output
    # (pofk_compute_rsd_pofk 2), and every step plus the output (1)
    # initial conditions from two GADGET-1 files of a displaced 20^3 lattice
    # (particle_files.py), READICFROMFILE build
    "lcdm_icfile": ("FOFR_LCDM_IC", dict(modified_gravity_active=0, fofr0=1e-5, nfofr=1.0, include_screening=1,
                                         ReadParticlesFromFile=1, TypeInputParticleFiles=3, NumInputParticleFiles=2,
                                         RamsesOutputNumber=0)),
    "lcdm_rsd": ("FOFR_LCDM", dict(modified_gravity_active=0, fofr0=1e-5, nfofr=1.0, include_screening=1), dict(rsd=2)),
    # standard PM instead of COLA (UseCOLA 0): 2LPT velocities at the IC
    "lcdm_pm": ("FOFR_LCDM", dict(modified_gravity_active=0, fofr0=1e-5, nfofr=1.0, include_screening=1),
                dict(cola=0)),
    # logarithmic bins in [0.1, 1] h/Mpc, shot noise subtracted
    "fofr_logbins": ("FOFR_LCDM", dict(modified_gravity_active=1, fofr0=1e-5, nfofr=1.0, include_screening=1),
                     dict(nbins=10, bintype=1, shotnoise=1, kmin=0.1, kmax=1.0)),
    # two outputs: z = 1 after 3 steps, z = 0 after 4 more (the output steps'
    # half kicks, src/main.c:394-611)
    "dgp_2out": ("DGP", dict(modified_gravity_active=1, rcH0_DGP=1.0, Rsmooth=1.0, include_screening=1),
                 dict(z1steps=3, nsteps=4)),
    # w(a) = w0 + wa (1 - a) background (EQUATIONOFSTATE_PARAMETRIZATION)
    "lcdm_w0wa": ("FOFR_LCDM_W0WA", dict(modified_gravity_active=0, fofr0=1e-5, nfofr=1.0, include_screening=1,
                                         w_0=-0.9, w_a=0.2)),
    # nDGP: top-hat and sharp-k smoothing, and no screening
    "dgp_tophat": ("DGP_TOPHAT", dict(modified_gravity_active=1, rcH0_DGP=1.0, Rsmooth=1.0, include_screening=1)),
    "dgp_sharpk": ("DGP_SHARPK", dict(modified_gravity_active=1, rcH0_DGP=1.0, Rsmooth=1.0, include_screening=1)),
    "dgp_nosc": ("DGP", dict(modified_gravity_active=1, rcH0_DGP=1.0, Rsmooth=1.0, include_screening=0)),
    # ASCII snapshot output (a build without GADGET_STYLE)
    "lcdm_ascii": ("FOFR_LCDM_ASCII", dict(modified_gravity_active=0, fofr0=1e-5, nfofr=1.0, include_screening=1)),
    # spherical mode cut of the IC (SphereMode 1)
    "lcdm_sphere": ("FOFR_LCDM", dict(modified_gravity_active=0, fofr0=1e-5, nfofr=1.0, include_screening=1),
                    dict(sphere=1)),
    # the input P(k) and sigma8 quoted for LCDM: the IC rescaled by
    # mg_pofk_ratio and the sigma8 enhancement (2LPT.c:392-407)
    "fofr_lcdmic": ("FOFR_LCDM", dict(modified_gravity_active=1, fofr0=1e-5, nfofr=1.0, include_screening=1),
                    dict(pofk_lcdm=1, s8_lcdm=0)),
    # LCDM growth factors in an f(R) run (use_lcdm_growth_factors 1)
    "fofr_lcdmgrowth": ("FOFR_LCDM", dict(modified_gravity_active=1, fofr0=1e-5, nfofr=1.0, include_screening=1),
                        dict(lcdm_growth=1)),
    # tabulated transfer function (WhichSpectrum 0, WhichTransfer 1)
    "lcdm_transfer": ("FOFR_LCDM", dict(modified_gravity_active=0, fofr0=1e-5, nfofr=1.0, include_screening=1),
                      dict(which_spectrum=0, which_transfer=1)),
    # lengths in kpc/h (UnitLength_in_cm 3.085678e21, Box 128000 kpc/h)
    "lcdm_kpc": ("FOFR_LCDM", dict(modified_gravity_active=0, fofr0=1e-5, nfofr=1.0, include_screening=1),
                 dict(unit_length=3.085678e21, Box=128000.0)),
    # tabulated input spectrum (WhichSpectrum 1, spectrum_table.py)
    "lcdm_table": ("FOFR_LCDM", dict(modified_gravity_active=0, fofr0=1e-5, nfofr=1.0, include_screening=1),
                   dict(which_spectrum=1)),
    "fofr_rsd": ("FOFR_LCDM", dict(modified_gravity_active=1, fofr0=1e-5, nfofr=1.0, include_screening=1), dict(rsd=1)),
}

STD = """use_lcdm_growth_factors  {lcdm_growth}
input_pofk_is_for_lcdm   {pofk_lcdm}
input_sigma8_is_for_lcdm {s8_lcdm}
pofk_compute_every_step   1
pofk_compute_rsd_pofk     {rsd}
pofk_nbins                {nbins}
pofk_bintype              {bintype}
pofk_subtract_shotnoise   {shotnoise}
pofk_kmin                 {kmin}
pofk_kmax                 {kmax}
OutputDir                   {out}
FileBase                    run
OutputRedshiftFile          {out}/outputs.txt
NumFilesWrittenInParallel   1
UseCOLA          {cola}
Buffer           1.5
Nmesh            {Nmesh}
Nsample          {Nsample}
Box              {Box}
Init_Redshift    {Init_Redshift}
Seed             {Seed}
SphereMode       {sphere}
WhichSpectrum    {which_spectrum}
WhichTransfer    {which_transfer}
FileWithInputSpectrum  {spectrum_file}
FileWithInputTransfer  {transfer_file}
Omega            {Omega}
OmegaBaryon      {OmegaBaryon}
HubbleParam      {HubbleParam}
Sigma8           {Sigma8}
PrimordialIndex  {PrimordialIndex}
UnitLength_in_cm                {unit_length}
UnitMass_in_g                   1.989e43
UnitVelocity_in_cm_per_s        1e5
InputSpectrum_UnitLength_in_cm  {input_unit_length}
"""


def run_reference(model, mg, base=None, cosmo=None, nu_info=None):
    """Run the reference binary of `model` on one small case; returns the
    final CDM P(k) table, the total one (neutrino builds) and the snapshot's
    positions and velocities.  nu_info: the CAMB info file of a neutrino
    build (default: the synthetic tables of camb_tables.py)."""
    base = dict(BASE, **(base or {}))
    cosmo = dict(COSMO, **(cosmo or {}))
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "outputs.txt"), "w") as f:
            if base["z1steps"]:
                f.write("1, %d\n" % base["z1steps"])
            f.write("0, %d\n" % base["nsteps"])
        spectrum = spectrum_table.write_pk_table(os.path.join(d, "pk_table.dat")) if base["which_spectrum"] == 1 else "none"
        transfer = (spectrum_table.write_transfer_table(os.path.join(d, "t_table.dat")) if base["which_transfer"] == 1
                    else "none")
        txt = STD.format(out=d, spectrum_file=spectrum, transfer_file=transfer, **base, **cosmo) + "".join(
            "%s %s\n" % kv for kv in mg.items())
        if "nu_SumMassNuEV" in mg:
            info = nu_info or camb_tables.write_tables(os.path.join(d, "camb"))
            txt += "nu_FilenameTransferInfofile %s\n" % info
        if mg.get("ReadParticlesFromFile"):
            icdir = particle_files.write_ic_files(os.path.join(d, "ic"), base["Box"])
            txt += "InputParticleFileDir %s\nInputParticleFilePrefix ics\n" % icdir
        pf = os.path.join(d, "params.txt")
        with open(pf, "w") as f:
            f.write(txt)
        log = subprocess.run([ref_build.binary(model), pf], capture_output=True, text=True)
        if log.returncode != 0:
            raise RuntimeError(model + ": " + log.stdout[-2000:] + log.stderr[-2000:])
        out = dict(pk=np.loadtxt(os.path.join(d, "pofk_run_z0.000_CDM.txt")))
        for f in sorted(os.listdir(d)):
            if f.startswith("pofk_RSD_run_z"):
                out["rsd_" + f[len("pofk_RSD_run_z"):-4]] = np.loadtxt(os.path.join(d, f))
        if "nu_SumMassNuEV" in mg:
            out["pk_total"] = np.loadtxt(os.path.join(d, "pofk_run_z0.000_total.txt"))
        n = base["Nsample"] ** 3
        out["info_txt"] = np.array(open(os.path.join(d, "info_run_z0p000.txt")).read())
        if model in ref_build.NO_GADGET_STYLE:
            # ASCII: the particle count, then x y z vx vy vz per line (%12.6f)
            lines = open(os.path.join(d, "run_z0p000.0")).read().splitlines()
            out["ascii_first_line"] = np.array(lines[0])
            rows = np.array([[float(v) for v in l.split()] for l in lines[1:]])
            out["pos"], out["vel"] = rows[:, :3].copy(), rows[:, 3:].copy()
        else:
            raw = open(os.path.join(d, "run_z0p000.0"), "rb").read()
            out["gadget_header"] = np.frombuffer(raw[:264], dtype=np.uint8).copy()
            out["pos"] = np.frombuffer(raw[268:268 + 12 * n], dtype="<f4").reshape(n, 3).copy()
            out["vel"] = np.frombuffer(raw[268 + 12 * n + 8:268 + 24 * n + 8], dtype="<f4").reshape(n, 3).copy()
        if base["z1steps"]:
            raw = open(os.path.join(d, "run_z1p000.0"), "rb").read()
            out["pos_z1"] = np.frombuffer(raw[268:268 + 12 * n], dtype="<f4").reshape(n, 3).copy()
            out["vel_z1"] = np.frombuffer(raw[268 + 12 * n + 8:268 + 24 * n + 8], dtype="<f4").reshape(n, 3).copy()
            out["pk_z1"] = np.loadtxt(os.path.join(d, "pofk_run_z1.000_CDM.txt"))
    return out


def run_case(name, model, mg, base=None):
    mgd = dict(inverted_initial_condition=0, amplitude_fixed_initial_condition=0)
    mgd.update(mg)
    r = run_reference(model, mgd, base=base)
    n = BASE["Nsample"] ** 3
    idx = np.arange(0, n, 8)
    extra = {k: v for k, v in r.items()
             if k in ("pk_total", "pk_z1", "info_txt", "ascii_first_line", "gadget_header") or k.startswith("rsd_")}
    extra.update({k: r[k][idx] for k in ("pos_z1", "vel_z1") if k in r})
    np.savez(os.path.join(ROOT, "tests", "golden", "ref_%s.npz" % name), pk=r["pk"], idx=idx, pos=r["pos"][idx],
             vel=r["vel"][idx], model=model, **{k: float(v) for k, v in mgd.items()}, **dict(BASE, **(base or {})),
             **extra)
    print(name, "bins", r["pk"].shape[0])

if __name__ == "__main__":
    ref_build.build()
    # optional case names on the command line regenerate only those
    for name, case in CASES.items():
        if len(sys.argv) > 1 and name not in sys.argv[1:]:
            continue
        run_case(name, *case)

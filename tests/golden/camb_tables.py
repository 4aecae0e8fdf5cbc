"""Synthetic CAMB transfer-function tables for the massive-neutrino build.

The build reads an info file "<dir> <nfiles>" followed by one line
"<file> <z>" per redshift, each file a header line and rows of 13 columns
(src/read_CAMB_data.h:1-30): k/h, T_cdm, T_b, T_photon, T_nu (massless),
T_massive-nu, T_total, T_no-nu, T_total-de, T_Weyl, and three velocity
columns.  The tables here are closed-form stand-ins with the physical
traits that matter to the code paths (a BBKS-shaped CDM transfer function
growing with a, a baryon suppression, neutrino free-streaming below a
scale that grows with a), written with fixed precision so the reference
run, the oracle and the CUDA path read identical numbers.  Redshifts
increase down the info file, as the 2D spline needs.
"""
import os

import numpy as np

REDSHIFTS = [0.0, 0.5, 1.0, 2.0, 4.0, 9.0, 19.0, 49.0, 99.0, 199.0, 300.0]
SUM_MNU_EV = 0.4


def transfer_columns(k, z, omega=0.267, omega_b=0.049, h=0.71, sum_mnu_ev=SUM_MNU_EV):
    """The 13 columns at wavenumbers k (h/Mpc) and redshift z."""
    q = k / (omega * h)
    t0 = np.log(1.0 + 2.34 * q) / (2.34 * q) * (1.0 + 3.89 * q + (16.1 * q) ** 2 + (5.46 * q) ** 3 +
                                                (6.71 * q) ** 4) ** -0.25
    g = 1.0 / (1.0 + z) * (1.0 + 0.1 / (1.0 + z))
    tc = t0 * g
    x = (k / 0.2) ** 2
    tb = tc * (1.0 - 0.25 * x / (1.0 + x))
    kfs = 0.05 / np.sqrt(1.0 + z)
    tnu = tc / (1.0 + (k / kfs) ** 2)
    onu = sum_mnu_ev / (93.14 * h * h)
    ocdm = omega - omega_b - onu
    tcb = (omega_b * tb + ocdm * tc) / (omega_b + ocdm)
    ttot = ((omega - onu) * tcb + onu * tnu) / omega
    zero = np.zeros_like(k)
    return np.stack([k, tc, tb, zero, tnu, tnu, ttot, tcb, ttot, ttot, zero, zero, zero], axis=1)


def write_tables(directory, nk=150, kmin=1e-4, kmax=100.0, **kw):
    """Write the per-redshift files and the info file into `directory`;
    returns the info file's path."""
    os.makedirs(directory, exist_ok=True)
    k = np.exp(np.linspace(np.log(kmin), np.log(kmax), nk))
    lines = ["%s %d" % (directory, len(REDSHIFTS))]
    for i, z in enumerate(REDSHIFTS):
        name = "transfer_%02d.dat" % i
        cols = transfer_columns(k, z, **kw)
        with open(os.path.join(directory, name), "w") as f:
            f.write("# k/h CDM baryon photon nu mass_nu total no_nu total_de Weyl v_CDM v_b v_b-v_c\n")
            for row in cols:
                f.write(" ".join("%.8e" % v for v in row) + "\n")
        lines.append("%s %.4f" % (name, z))
    info = os.path.join(directory, "transfer_info.txt")
    with open(info, "w") as f:
        f.write("\n".join(lines) + "\n")
    return info

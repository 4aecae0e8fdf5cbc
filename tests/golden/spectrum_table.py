"""A tabulated linear power spectrum for WhichSpectrum = 1 (read_power_table,
src/power.c): two columns k (h/Mpc) and P(k) ((Mpc/h)^3), log-spaced k in
[1e-4, 100] h/Mpc; a BBKS-shaped spectrum with n_s = 0.96 (its amplitude is
reset by the sigma8 normalisation).  Fixed-precision text, so the reference
run and the CUDA path read identical numbers."""
import numpy as np


def write_pk_table(path, omega=0.267, h=0.71, ns=0.96, n=300):
    k = np.exp(np.linspace(np.log(1e-4), np.log(100.0), n))
    q = k / (omega * h)
    t = np.log(1.0 + 2.34 * q) / (2.34 * q) * (1.0 + 3.89 * q + (16.1 * q) ** 2 + (5.46 * q) ** 3 +
                                               (6.71 * q) ** 4) ** -0.25
    p = 2.0e4 * k ** ns * t * t
    with open(path, "w") as f:
        for a, b in zip(k, p):
            f.write("%.8e %.8e\n" % (a, b))
    return path


def write_transfer_table(path, omega=0.267, h=0.71, n=300):
    """A tabulated transfer function for WhichSpectrum = 0, WhichTransfer = 1
    (read_transfer_table, src/power.c): k (h/Mpc) and T(k), BBKS-shaped."""
    k = np.exp(np.linspace(np.log(1e-4), np.log(100.0), n))
    q = k / (omega * h)
    t = np.log(1.0 + 2.34 * q) / (2.34 * q) * (1.0 + 3.89 * q + (16.1 * q) ** 2 + (5.46 * q) ** 3 +
                                               (6.71 * q) ** 4) ** -0.25
    with open(path, "w") as f:
        for a, b in zip(k, t):
            f.write("%.8e %.8e\n" % (a, b))
    return path

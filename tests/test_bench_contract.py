"""bench.py's roofline bookkeeping on CPU: the algorithmic bytes of the
dominant kernels and which workloads carry an ncu traffic figure."""
import importlib.util
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_contract", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    argv, sys.argv = sys.argv, ["bench.py"]
    try:
        spec.loader.exec_module(mod)
    finally:
        sys.argv = argv
    return mod


def test_kick_and_deposit_bytes_at_the_default_workload():
    b = _bench()
    N, Np = 1024, 512 ** 3
    assert b.algorithmic_bytes(N, Np, "interp_kick_drift") == 12 * N ** 3 + 72 * Np == 22548578304
    assert b.algorithmic_bytes(N, Np, "cic") == 12 * Np + 4 * N ** 3


def test_ncu_traffic_only_where_it_was_captured():
    b = _bench()
    c3, c3s = b.CONFIGS["ndgp_512_1024"], b.CONFIGS["ndgp_256_512"]
    # captured at 256^3 / 512^3, scaled by the cell count to 512^3 / 1024^3
    small = b.measured_traffic(c3s, 512, 256 ** 3, "interp_kick_drift")
    assert small == int(b.TRAFFIC_256_512["interp_kick_drift"])
    assert b.measured_traffic(c3, 1024, 512 ** 3, "interp_kick_drift") == 8 * small
    # other kick and deposit forms (scale-dependent growth, closure, LCDM) have none
    for name in ("fofr_sd_256_512", "fofr_nu_256_512", "closure_lcdm_256", "lcdm_64_128"):
        cfg = b.CONFIGS[name]
        assert b.measured_traffic(cfg, cfg["N"], cfg["Ns"] ** 3, "interp_kick_drift") is None
    # a mesh that is not twice the particle lattice has no scaled figure either
    assert b.measured_traffic(c3, 1024, 256 ** 3, "interp_kick_drift") is None


def test_job_value_counts_all_ranks_over_the_slowest():
    b = _bench()
    assert abs(b.job_value(4, 1000, 10, 2.0) - 4 * 1000 * 10 / 2.0 / 1e6) < 1e-12

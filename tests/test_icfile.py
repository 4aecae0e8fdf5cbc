"""Initial conditions from particle files (src/readICfromfile.c): the host
readers of the three formats (GADGET-1, ASCII, RAMSES) against the positions
written into them, and the READICFROMFILE parameter keys."""
import os
import struct

import numpy as np
import pytest

import mgpicola as M
from golden.particle_files import gadget_file  # noqa: F401  (also imported by test_gpu_icfile)
from test_host import write_param


def ascii_file(path, pos01):
    with open(path, "w") as f:
        f.write("%d\n" % len(pos01))
        for x, y, z in pos01:
            f.write("%.17g %.17g %.17g 1.0\n" % (x, y, z))


def ramses_file(path, pos01):
    def rec(b):
        return struct.pack("<i", len(b)) + b + struct.pack("<i", len(b))

    n = len(pos01)
    with open(path, "wb") as f:
        for v in (1, 3, n):
            f.write(rec(struct.pack("<i", v)))
        f.write(rec(struct.pack("<4i", 1, 2, 3, 4)))
        f.write(rec(struct.pack("<i", 0)))
        f.write(rec(struct.pack("<2i", 0, 0)))
        f.write(rec(struct.pack("<2i", 0, 0)))
        f.write(rec(struct.pack("<i", 0)))
        for a in range(3):
            f.write(rec(np.ascontiguousarray(pos01[:, a], "<f8").tobytes()))


def params_for(tmp_path, ftype, nfiles, prefix="part", outnum=7):
    p = M.default_params(ReadParticlesFromFile=1, TypeInputParticleFiles=ftype, NumInputParticleFiles=nfiles,
                         InputParticleFileDir=str(tmp_path), InputParticleFilePrefix=prefix, RamsesOutputNumber=outnum)
    return p


def two_sets(seed):
    rng = np.random.default_rng(seed)
    a = rng.uniform(0, 1, (50, 3))
    b = rng.uniform(0, 1, (37, 3))
    a[0] = [1.0, 0.25, 0.999999999]  # the reader wraps x >= 1 to x - 1
    return a, b


def test_read_gadget_files(tmp_path):
    box = 256.0
    a, b = two_sets(1)
    gadget_file(os.path.join(tmp_path, "part.0"), a * box, box)
    gadget_file(os.path.join(tmp_path, "part.1"), b * box, box)
    got = M.read_particle_files(params_for(tmp_path, 3, 2))
    # the reference divides the float positions by BoxSize and keeps floats
    want = np.vstack([a, b]) * box
    want = (want.astype(np.float32).astype(np.float64) * (1.0 / box)).astype(np.float32)
    want = np.where(want >= 1.0, (want - 1.0).astype(np.float32), want).astype(np.float64)
    np.testing.assert_array_equal(got, want)


def test_read_ascii_files(tmp_path):
    a, b = two_sets(2)
    ascii_file(os.path.join(tmp_path, "part.1"), a)
    ascii_file(os.path.join(tmp_path, "part.2"), b)
    got = M.read_particle_files(params_for(tmp_path, 2, 2))
    want = np.vstack([a, b])
    want = np.where(want >= 1.0, want - 1.0, want)
    np.testing.assert_array_equal(got, want)


def test_read_ramses_files(tmp_path):
    a, b = two_sets(3)
    ramses_file(os.path.join(tmp_path, "part_00007.out00001"), a)
    ramses_file(os.path.join(tmp_path, "part_00007.out00002"), b)
    got = M.read_particle_files(params_for(tmp_path, 1, 2))
    want = np.vstack([a, b])
    want = np.where(want >= 1.0, want - 1.0, want)
    np.testing.assert_array_equal(got, want)


def test_read_particle_file_errors(tmp_path):
    with pytest.raises(M.MGPError, match="cannot open file"):
        M.read_particle_files(params_for(tmp_path, 3, 1))
    with pytest.raises(M.MGPError, match="unknown file-format"):
        M.read_particle_files(params_for(tmp_path, 4, 1))
    with open(os.path.join(tmp_path, "bad.0"), "wb") as f:
        f.write(struct.pack("<i", 100) + bytes(100))
    with pytest.raises(M.MGPError):
        M.read_particle_files(params_for(tmp_path, 3, 1, prefix="bad"))


def test_parameter_file_readic_keys(tmp_path):
    keys = ("ReadParticlesFromFile 1\nInputParticleFileDir /data/ic\nInputParticleFilePrefix snap\n"
            "TypeInputParticleFiles 3\nNumInputParticleFiles 4\nRamsesOutputNumber 1\n")
    p = M.read_parameterfile(write_param(tmp_path, M.MODEL_LCDM, extra=keys), M.MODEL_LCDM, read_ic_from_file=True)
    assert p.ReadParticlesFromFile == 1 and p.TypeInputParticleFiles == 3 and p.NumInputParticleFiles == 4
    assert p.InputParticleFileDir == b"/data/ic" and p.InputParticleFilePrefix == b"snap"
    # the keys are required in that build, and not allowed without it
    with pytest.raises(M.MGPError, match="miss a value for tag 'RamsesOutputNumber'"):
        M.read_parameterfile(write_param(tmp_path, M.MODEL_LCDM, extra=keys.replace("RamsesOutputNumber 1\n", "")),
                             M.MODEL_LCDM, read_ic_from_file=True)
    with pytest.raises(M.MGPError, match="not allowed or multiple"):
        M.read_parameterfile(write_param(tmp_path, M.MODEL_LCDM, extra=keys), M.MODEL_LCDM)

"""Particle files for the initial-conditions-from-files path
(src/readICfromfile.c): a GADGET-1 writer (type-1 positions in Box units,
zero velocities; the reader uses npart[1] and BoxSize of the header) and a
deterministic displaced lattice, so the reference run, the oracle and the
CUDA path read identical float32 positions."""
import os
import struct

import numpy as np


def gadget_file(path, pos_box, box):
    """GADGET-1 file with type-1 positions (Box units) and zero velocities."""
    n = len(pos_box)
    hdr = struct.pack("<6I6dddii6Iiiddddii6Ii", 0, n, 0, 0, 0, 0, *([0.0] * 6), 0.1, 9.0, 0, 0, 0, n, 0, 0, 0, 0, 0, 1,
                      box, 0.267, 0.733, 0.71, 0, 0, 0, 0, 0, 0, 0, 0, 0)
    hdr += b"\0" * (256 - len(hdr))
    blk = np.ascontiguousarray(pos_box, "<f4").tobytes()
    with open(path, "wb") as f:
        f.write(struct.pack("<i", 256) + hdr + struct.pack("<i", 256))
        f.write(struct.pack("<i", len(blk)) + blk + struct.pack("<i", len(blk)))
        f.write(struct.pack("<i", len(blk)) + bytes(len(blk)) + struct.pack("<i", len(blk)))


def displaced_lattice(n1d, box, amp=0.25):
    """n1d^3 particles: a lattice displaced by three plane waves (amplitude
    `amp` of the spacing each), wrapped into [0, box); closed form, no RNG."""
    q = np.stack(np.meshgrid(*(np.arange(n1d),) * 3, indexing="ij"), -1).reshape(-1, 3) * (box / n1d)
    waves = [((1, 0, 0), 0.3), ((0, 2, 1), 1.1), ((1, 1, 3), 2.0)]
    d = np.zeros_like(q)
    for (kx, ky, kz), ph in waves:
        arg = 2 * np.pi * (kx * q[:, 0] + ky * q[:, 1] + kz * q[:, 2]) / box + ph
        d += amp * (box / n1d) * np.stack([np.sin(arg), np.cos(arg + 0.5), np.sin(2 * arg + 1.0)], 1)
    return np.mod(q + d, box).astype(np.float32)


def write_ic_files(directory, box, prefix="ics", nfiles=2, n1d=20):
    """The displaced lattice split over `nfiles` GADGET-1 files
    <directory>/<prefix>.<i>; returns the directory."""
    os.makedirs(directory, exist_ok=True)
    pos = displaced_lattice(n1d, box)
    for i, part in enumerate(np.array_split(pos, nfiles)):
        gadget_file(os.path.join(directory, "%s.%d" % (prefix, i)), part, box)
    return directory

"""Small Gadget binary snapshots and what the reference's reader returns.

Run here, where the reference sources are readable:
    python tests/golden/make_snapshot_golden.py

Writes tests/golden/snapshots/:
  f2_snap.0, f2_snap.1   format II, two files, little-endian, types 1 and 2
                         with masses in the header's table, redshift 0.5
  f1_snap                format I, one file, big-endian, types 0 (gas, masses
                         in a MASS block) and 1, redshift 0
and tests/golden/snapshot_golden.npz: the header fields and the POS, VEL,
ID and MASS blocks as library/readsnap.py (read_block, snapshot_header)
returns them, per particle type.  The reference's readgadget.py imports h5py
(not installed), so its binary path -- readsnap.read_block per type, in the
order of the type list -- is called directly.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "snapshots")
# the reference tree: $PYLIANS3_REFERENCE (default /root/reference)
REF = os.path.join(os.environ.get("PYLIANS3_REFERENCE", "/root/reference"), "library")


def write_snapshot(path, end, fmt, npart, nall, massarr, time, redshift, filenum, box,
                   blocks):
    """One Gadget binary file; blocks: list of (name, ndarray) after HEAD."""
    def rec(f, name, payload):
        n = np.array([len(payload)], end + "u4").tobytes()
        if fmt == 2:
            f.write(np.array([8], end + "u4").tobytes())
            f.write(name.encode("latin-1"))
            f.write(np.array([len(payload) + 8], end + "u4").tobytes())
            f.write(np.array([8], end + "u4").tobytes())
        f.write(n)
        f.write(payload)
        f.write(n)

    h = b"".join([
        np.asarray(npart, end + "i4").tobytes(), np.asarray(massarr, end + "f8").tobytes(),
        np.array([time, redshift], end + "f8").tobytes(), np.array([0, 0], end + "i4").tobytes(),
        np.asarray(nall, end + "u4").tobytes(), np.array([0, filenum], end + "i4").tobytes(),
        np.array([box, 0.3, 0.7, 0.7], end + "f8").tobytes()])
    h += b"\0" * (256 - len(h))
    with open(path, "wb") as f:
        rec(f, "HEAD", h)
        for name, arr in blocks:
            rec(f, name, np.ascontiguousarray(arr).astype(arr.dtype.newbyteorder(end)).tobytes())


def main():
    os.makedirs(OUT, exist_ok=True)
    rng = np.random.default_rng(77)
    box = 100000.0    # kpc/h
    # ---- format II, 2 files, types 1 and 2 (masses in the table)
    per_file = [np.array([0, 1500, 700, 0, 0, 0]), np.array([0, 1200, 600, 0, 0, 0])]
    nall = per_file[0] + per_file[1]
    massarr = [0.0, 0.05, 0.003, 0.0, 0.0, 0.0]
    next_id = 1
    for i, npart in enumerate(per_file):
        n = int(npart.sum())
        pos = (rng.random((n, 3)) * box).astype(np.float32)
        vel = (rng.standard_normal((n, 3)) * 300).astype(np.float32)
        ids = np.arange(next_id, next_id + n, dtype=np.uint32)
        next_id += n
        write_snapshot(os.path.join(OUT, "f2_snap.%d" % i), "<", 2, npart, nall, massarr,
                       1 / 1.5, 0.5, 2, box, [("POS ", pos), ("VEL ", vel), ("ID  ", ids)])
    # ---- format I, 1 file, big-endian, gas with a MASS block + type 1
    npart = np.array([900, 1100, 0, 0, 0, 0])
    n = int(npart.sum())
    pos = (rng.random((n, 3)) * box).astype(np.float32)
    vel = (rng.standard_normal((n, 3)) * 300).astype(np.float32)
    ids = np.arange(1, n + 1, dtype=np.uint32)
    mass = rng.uniform(0.001, 0.002, 900).astype(np.float32)
    write_snapshot(os.path.join(OUT, "f1_snap"), ">", 1, npart, npart, [0.0, 0.04, 0, 0, 0, 0],
                   1.0, 0.0, 1, box,
                   [("POS ", pos), ("VEL ", vel), ("ID  ", ids), ("MASS", mass)])

    sys.path.insert(0, REF)
    import readsnap
    out = {}
    for tag, snap, types in (("f2", "f2_snap", (1, 2)), ("f1", "f1_snap", (0, 1))):
        path = os.path.join(OUT, snap)
        h = readsnap.snapshot_header(path)
        for key in ("npart", "massarr", "time", "redshift", "nall", "filenum", "boxsize",
                    "omega_m", "omega_l", "hubble", "format"):
            out["%s_head_%s" % (tag, key)] = np.asarray(getattr(h, key))
        for t in types:
            for block in ("POS ", "VEL ", "ID  ", "MASS"):
                out["%s_%s_%d" % (tag, block.strip(), t)] = readsnap.read_block(path, block, t)
    np.savez_compressed(os.path.join(HERE, "snapshot_golden.npz"), **out)
    print(sorted(out)[:6], len(out))


if __name__ == "__main__":
    main()

"""The Gadget binary reader against what the reference's readsnap returned
for the committed fixtures (format II two-file little-endian, format I
big-endian with a MASS block).  CPU only."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SNAP = os.path.join(HERE, "golden", "snapshots")


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(HERE, "golden", "snapshot_golden.npz"))


@pytest.fixture(scope="module")
def rg():
    from pylians3_gb300 import readgadget
    return readgadget


CASES = (("f2", "f2_snap", (1, 2)), ("f1", "f1_snap", (0, 1)))


@pytest.mark.parametrize("tag,snap,types", CASES)
def test_header(gold, rg, tag, snap, types):
    h = rg.header(os.path.join(SNAP, snap))
    for key in ("npart", "massarr", "nall"):
        np.testing.assert_array_equal(getattr(h, key), gold["%s_head_%s" % (tag, key)])
    for key in ("time", "redshift", "filenum", "boxsize", "omega_m", "omega_l", "hubble",
                "format"):
        assert getattr(h, key) == gold["%s_head_%s" % (tag, key)][()], key


@pytest.mark.parametrize("tag,snap,types", CASES)
@pytest.mark.parametrize("block", ["POS ", "VEL ", "ID  ", "MASS"])
def test_blocks(gold, rg, tag, snap, types, block):
    path = os.path.join(SNAP, snap)
    for t in types:
        got = rg.read_block(path, block, [t])
        want = gold["%s_%s_%d" % (tag, block.strip(), t)]
        if block == "MASS":
            assert got.dtype == np.float32
            np.testing.assert_array_equal(got, want.astype(np.float32))
        else:
            np.testing.assert_array_equal(got, want)
    both = rg.read_block(path, block, list(types))
    want = np.concatenate([gold["%s_%s_%d" % (tag, block.strip(), t)] for t in types])
    np.testing.assert_array_equal(both, want.astype(both.dtype))


def test_hdf5_and_missing(rg, tmp_path):
    p = tmp_path / "snap.hdf5"
    p.write_bytes(b"\x89HDF")
    with pytest.raises(ImportError):
        rg.header(str(p))
    with pytest.raises(Exception):
        rg.header(str(tmp_path / "nothing"))


def test_rsd_oracle_wraps(oracle):
    pos = np.array([[1.0, 2.0, 999.0], [1.0, 2.0, 1.0], [5.0, 5.0, 5.0]], np.float32)
    vel = np.array([[0, 0, 300.0], [0, 0, -2.5e5], [0, 0, 0]], np.float32)
    oracle.pos_redshift_space(pos, vel, 1000.0, 100.0, 0.0, 2)
    assert 0.0 <= pos[:, 2].min() and pos[:, 2].max() <= 1000.0
    assert pos[2, 2] == np.float32(5.0)

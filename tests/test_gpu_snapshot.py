"""Snapshot -> spectrum driver on the GPU: streamed block reads, the
redshift-space shift, and Pk_comp against the oracle pipeline of
Pk_snapshot.py:34-91 on the committed Gadget fixtures."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
SNAP = os.path.join(HERE, "golden", "snapshots")
TOL_PK = 1e-4


@pytest.fixture(scope="module")
def gpu():
    import torch
    assert torch.cuda.is_available()
    from pylians3_gb300 import build_native
    build_native.build()
    import pylians3_gb300 as P
    return P


@pytest.mark.parametrize("snap,types", [("f2_snap", [1, 2]), ("f1_snap", [0, 1])])
@pytest.mark.parametrize("block", ["POS ", "VEL ", "MASS"])
def test_streamed_block_equals_host_read(gpu, snap, types, block):
    from pylians3_gb300 import readgadget as rg
    path = os.path.join(SNAP, snap)
    want = rg.read_block(path, block, types)
    # a 4 KB chunk forces many slabs through the two pinned buffers
    got = rg.read_block_to_device(path, block, types, chunk_bytes=4096)
    assert got.is_cuda
    np.testing.assert_array_equal(got.cpu().numpy(), want.astype(np.float32))


def test_rsd_matches_restatement(gpu, oracle):
    import torch
    from pylians3_gb300.redshift_space_library import pos_redshift_space
    rng = np.random.default_rng(8)
    n = 200000
    pos = (rng.random((n, 3)) * 1000).astype(np.float32)
    vel = (rng.standard_normal((n, 3)) * 800).astype(np.float32)
    vel[:100, 2] = -3.0e6          # crosses the box several times
    vel[100:200, 2] = 3.0e6
    for axis in (0, 2):
        want = pos.copy()
        oracle.pos_redshift_space(want, vel, 1000.0, 150.0, 0.7, axis)
        got = pos.copy()
        pos_redshift_space(got, vel, 1000.0, 150.0, 0.7, axis)
        np.testing.assert_array_equal(got, want)
        t = torch.from_numpy(pos.copy()).cuda()
        pos_redshift_space(t, torch.from_numpy(vel).cuda(), 1000.0, 150.0, 0.7, axis)
        np.testing.assert_array_equal(t.cpu().numpy(), want)


def _oracle_pk(oracle, pos, dims, box, axis, W=None):
    delta = np.zeros((dims,) * 3, np.float32)
    oracle.MA(pos, delta, box, "CIC", W=W)
    mean = (np.sum(W, dtype=np.float64) if W is not None else len(pos) * 1.0) / dims ** 3
    delta /= mean
    delta -= 1.0
    return oracle.Pk(delta, box, axis=axis, MAS="CIC", threads=4)


@pytest.mark.parametrize("do_RSD,axis", [(False, 0), (True, 2)])
def test_pk_comp_single_type(gpu, oracle, tmp_path, do_RSD, axis):
    from pylians3_gb300 import Pk_snapshot, readgadget as rg
    path = os.path.join(SNAP, "f2_snap")
    h = rg.header(path)
    box = h.boxsize / 1e3
    pos = rg.read_block(path, "POS ", [1]) / 1e3
    if do_RSD:
        vel = rg.read_block(path, "VEL ", [1])
        Hub = 100.0 * np.sqrt(h.omega_m * (1.0 + h.redshift) ** 3 + h.omega_l)
        oracle.pos_redshift_space(pos, vel, box, Hub, h.redshift, axis)
    ref = _oracle_pk(oracle, pos, 16, box, axis)
    fout = Pk_snapshot.Pk_comp(path, 1, 16, do_RSD, axis, 1, str(tmp_path))
    got = np.loadtxt(fout)
    np.testing.assert_allclose(got[:, 0], ref.k3D, rtol=1e-12)
    np.testing.assert_array_equal(got[:, 4], ref.Nmodes3D)
    err = np.abs(got[:, 1:4] - ref.Pk).max(axis=1) / np.abs(ref.Pk[:, 0])
    assert err.max() <= TOL_PK
    assert os.path.basename(fout) == ("Pk_CDM_RS_axis=2_z=0.500.dat" if do_RSD
                                      else "Pk_CDM_z=0.500.dat")


def test_pk_comp_all_types_mass_weighted(gpu, oracle, tmp_path):
    """ptype = -1 on a snapshot with gas: masses from the MASS block and the
    header's table, deposited as weights."""
    from pylians3_gb300 import Pk_snapshot, readgadget as rg
    path = os.path.join(SNAP, "f1_snap")
    box = rg.header(path).boxsize / 1e3
    types = [0, 1, 2, 3, 4, 5]
    pos = rg.read_block(path, "POS ", types) / 1e3
    M = rg.read_block(path, "MASS", types) * 1e10
    ref = _oracle_pk(oracle, pos, 16, box, 0, W=M.astype(np.float32))
    spec, _ = Pk_snapshot.Pk_comp_spectrum(path, -1, 16, False, 0)
    err = np.abs(spec.Pk - ref.Pk).max(axis=1) / np.abs(ref.Pk[:, 0])
    assert err.max() <= TOL_PK

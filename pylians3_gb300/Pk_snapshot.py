"""Snapshot -> power spectrum driver on the GPU.

``Pk_comp(snapshot_fname, ptype, dims, do_RSD, axis, cpus, folder_out)`` as
Pylians3's library/Pk_library/Pk_snapshot.py:34-91: reads the particles of
one type (or all types, ptype = -1, weighted by mass) of a Gadget binary
snapshot, optionally moves them to redshift space along ``axis``, deposits
them with CIC on a dims^3 grid and writes k, P0, P2, P4, Nmodes to
folder_out/Pk_<type>[_RS_axis=<axis>]_z=<z>.dat.  Every step after the
disk read runs on the device: the blocks are streamed into HBM through
pinned buffers (readgadget.read_block_to_device), the positions are
converted to Mpc/h, displaced (pos_redshift_space) and handed to the fused
particles -> spectrum call (pyl_pk_particles), so the grid never leaves the
device.  ``Pk_comp_spectrum`` returns the spectrum instead of writing it.
"""
from __future__ import annotations

import numpy as np

from . import readgadget
from .pipeline import power_spectrum
from .redshift_space_library import pos_redshift_space

name_dict = {"0": "GAS", "01": "GCDM", "02": "GNU", "04": "Gstars",
             "1": "CDM", "12": "CDMNU", "14": "CDMStars",
             "2": "NU", "24": "NUStars",
             "4": "Stars",
             "-1": "matter"}


def Pk_comp_spectrum(snapshot_fname, ptype, dims, do_RSD, axis, device="cuda"):
    """(spectrum, header) of one particle type (or -1: all, mass-weighted)."""
    import torch
    head = readgadget.header(snapshot_fname)
    BoxSize = head.boxsize / 1e3                     # Mpc/h
    Nall = head.nall.astype(np.int64)
    redshift = head.redshift
    Hubble = 100.0 * np.sqrt(head.omega_m * (1.0 + redshift) ** 3 + head.omega_l)
    types = [0, 1, 2, 3, 4, 5] if ptype == -1 else [ptype]
    pos = readgadget.read_block_to_device(snapshot_fname, "POS ", types, device)
    pos.div_(1e3)                                    # kpc/h -> Mpc/h
    if do_RSD:
        vel = readgadget.read_block_to_device(snapshot_fname, "VEL ", types, device)
        pos_redshift_space(pos, vel, BoxSize, Hubble, redshift, axis)
        del vel
    W = None
    if ptype == -1:
        if Nall[0] == 0:          # no gas: masses from the header's table
            W = torch.empty(int(Nall.sum()), dtype=torch.float32, device=device)
            off = 0
            for t in range(6):
                W[off:off + int(Nall[t])] = float(head.massarr[t] * 1e10)
                off += int(Nall[t])
        else:
            W = readgadget.read_block_to_device(snapshot_fname, "MASS", types, device)
            W.mul_(1e10)
    spec = power_spectrum(pos, dims, float(BoxSize), "CIC", axis=axis, W=W)
    return spec, head


def Pk_comp(snapshot_fname, ptype, dims, do_RSD, axis, cpus, folder_out):
    print("Computing power spectrum...")
    spec, head = Pk_comp_spectrum(snapshot_fname, ptype, dims, do_RSD, axis)
    z = "%.3f" % head.redshift
    fout = folder_out + "/Pk_" + name_dict[str(ptype)]
    if do_RSD:
        fout += "_RS_axis=" + str(axis) + "_z=" + z + ".dat"
    else:
        fout += "_z=" + z + ".dat"
    np.savetxt(fout, np.transpose([spec.k3D, spec.Pk[:, 0], spec.Pk[:, 1], spec.Pk[:, 2],
                                   spec.Nmodes3D]))
    return fout

"""Gadget snapshot reader for the snapshot -> spectrum driver.

Reads Gadget format I and II binary snapshots (single or multi-file, either
byte order) with the interface of Pylians3's library/readgadget.py:
``header(snapshot)`` (:23-84), ``read_block(snapshot, block, ptype)``
(:117-170) for the POS/VEL/MASS/ID blocks, ``read_field``; the block layout
follows library/readsnap.py:97-380 (block numbers POS 2, VEL 3, ID 4, MASS 5
in format I; named blocks in format II; velocities times sqrt(a) when the
redshift is not 0; MASS filled from the header's mass table where it is
set).  HDF5 snapshots need h5py, which is not installed here: they raise.

``read_block_to_device`` streams a block straight into a CUDA tensor: each
(particle type, file) slab is read into one of two pinned host buffers and
copied to the device on a side stream while the next slab is read.
"""
from __future__ import annotations

import math
import os

import numpy as np

_BLOCK_NUM = {"POS ": 2, "VEL ": 3, "ID  ": 4, "MASS": 5}


def fname_format(snapshot):
    """(first file, 'binary' | 'hdf5') as readgadget.fname_format (:6-19)."""
    if os.path.exists(snapshot):
        return snapshot, ("hdf5" if snapshot[-4:] == "hdf5" else "binary")
    if os.path.exists(snapshot + ".0"):
        return snapshot + ".0", "binary"
    if os.path.exists(snapshot + ".hdf5"):
        return snapshot + ".hdf5", "hdf5"
    if os.path.exists(snapshot + ".0.hdf5"):
        return snapshot + ".0.hdf5", "hdf5"
    raise Exception("File not found!")


def _no_hdf5():
    raise ImportError("HDF5 snapshots need h5py, which is not available; "
                      "Gadget format I/II binary snapshots are supported")


class _Layout:
    """Format, byte order and block table of one binary file."""

    def __init__(self, filename):
        with open(filename, "rb") as f:
            b = f.read(4)
        little, big = int.from_bytes(b, "little"), int.from_bytes(b, "big")
        if little in (8, 256):
            self.end, size0 = "<", little
        elif big in (8, 256):
            self.end, size0 = ">", big
        else:
            raise ValueError("not a Gadget binary file: %s" % filename)
        self.format = 2 if size0 == 8 else 1
        self.blocks = {}      # name or number -> (offset of the data, size in bytes)
        size = os.path.getsize(filename)
        u4 = np.dtype(self.end + "u4")
        with open(filename, "rb") as f:
            num = 1
            while f.tell() < size:
                name = None
                if self.format == 2:
                    f.seek(4, os.SEEK_CUR)
                    name = f.read(4).decode("latin-1")
                    f.seek(8, os.SEEK_CUR)
                bs = int(np.frombuffer(f.read(4), u4)[0])
                off = f.tell()
                f.seek(bs, os.SEEK_CUR)
                check = int(np.frombuffer(f.read(4), u4)[0])
                if check != bs:
                    raise ValueError("corrupt block %s in %s" % (name or num, filename))
                self.blocks[name if name is not None else num] = (off, bs)
                num += 1

    def find(self, block):
        key = block if self.format == 2 else _BLOCK_NUM[block]
        if key not in self.blocks:
            raise KeyError("block %r not found" % block)
        return self.blocks[key]


class header:
    """Snapshot header (readgadget.header, :23-84; readsnap.py:26-94)."""

    def __init__(self, snapshot):
        filename, fformat = fname_format(snapshot)
        if fformat == "hdf5":
            _no_hdf5()
        lay = _Layout(filename)
        e = lay.end
        with open(filename, "rb") as f:
            f.seek(4 + (16 if lay.format == 2 else 0))
            self.npart = np.fromfile(f, dtype=e + "i4", count=6).astype(np.int32)
            self.massarr = np.fromfile(f, dtype=e + "f8", count=6).astype(np.float64)
            self.time = float(np.fromfile(f, dtype=e + "f8", count=1)[0])
            self.redshift = float(np.fromfile(f, dtype=e + "f8", count=1)[0])
            self.sfr = int(np.fromfile(f, dtype=e + "i4", count=1)[0])
            self.feedback = int(np.fromfile(f, dtype=e + "i4", count=1)[0])
            self.nall = np.fromfile(f, dtype=e + "u4", count=6).astype(np.uint32)
            self.cooling = int(np.fromfile(f, dtype=e + "i4", count=1)[0])
            self.filenum = int(np.fromfile(f, dtype=e + "i4", count=1)[0])
            self.boxsize = float(np.fromfile(f, dtype=e + "f8", count=1)[0])
            self.omega_m = float(np.fromfile(f, dtype=e + "f8", count=1)[0])
            self.omega_l = float(np.fromfile(f, dtype=e + "f8", count=1)[0])
            self.hubble = float(np.fromfile(f, dtype=e + "f8", count=1)[0])
        self.format = lay.format
        # km/s/(Mpc/h)
        self.Hubble = 100.0 * np.sqrt(self.omega_m * (1.0 + self.redshift) ** 3 + self.omega_l)


def _files(snapshot, filenum):
    if os.path.exists(snapshot):
        return [snapshot]
    return ["%s.%d" % (snapshot, i) for i in range(filenum)]


def _item(block):
    if block in ("POS ", "VEL "):
        return np.dtype((np.float32, 3))
    if block == "MASS":
        return np.dtype(np.float32)
    if block == "ID  ":
        return None   # uint32 or uint64, from the block size
    raise Exception("block not implemented in readgadget!")


def _slabs(snapshot, block, ptype):
    """(file, byte offset, count, dtype, constant) for every (ptype, file) in
    the reference's order; constant is set for MASS taken from the table."""
    head = header(snapshot)
    out = []
    for pt in ptype:
        for fn in _files(snapshot, head.filenum):
            h = header(fn) if fn != snapshot else head
            lay = _Layout(fn)
            e = lay.end
            npart = h.npart.astype(np.int64)
            if block == "MASS":
                if h.massarr[pt] > 0:
                    out.append((fn, 0, int(npart[pt]), np.dtype(np.float32), h.massarr[pt]))
                    continue
                has = h.massarr == 0
            else:
                has = np.ones(6, bool)
            off, bs = lay.find(block)
            before = int(npart[:pt][has[:pt]].sum())
            total = int(npart[has].sum())
            dt = _item(block)
            if dt is None:
                dt = np.dtype(np.uint64 if total and bs == 8 * total else np.uint32)
            if dt.itemsize * total != bs:
                raise ValueError("block size of %s in %s: expected %d, found %d"
                                 % (block, fn, dt.itemsize * total, bs))
            out.append((fn, off + before * dt.itemsize, int(npart[pt]),
                        dt.newbyteorder(e) if dt.shape == () else np.dtype((e + "f4", 3)), None))
    return head, out


def read_block(snapshot, block, ptype, verbose=False):
    """Block of the whole snapshot for the listed particle types
    (readgadget.read_block, :117-170); positions in the snapshot's units."""
    if fname_format(snapshot)[1] == "hdf5":
        _no_hdf5()
    head, slabs = _slabs(snapshot, block, ptype)
    parts = []
    for fn, off, cnt, dt, const in slabs:
        if const is not None:
            parts.append(np.full(cnt, const, np.float32))
            continue
        with open(fn, "rb") as f:
            f.seek(off)
            a = np.fromfile(f, dtype=dt, count=cnt)
        parts.append(a.astype(a.dtype.newbyteorder("=")))
    data = np.concatenate(parts) if parts else np.zeros(0, np.float32)
    if block == "VEL " and head.redshift != 0:
        data *= math.sqrt(head.time)
    return data


def read_field(snapshot, block, ptype):
    """One particle type of one file (readgadget.read_field, :87-113)."""
    return read_block(snapshot, block, [ptype])


def read_block_to_device(snapshot, block, ptype, device="cuda", chunk_bytes=64 << 20):
    """POS/VEL/MASS block of the listed types as a CUDA float32 tensor,
    streamed through two pinned buffers (disk reads overlap the copies)."""
    import torch
    if fname_format(snapshot)[1] == "hdf5":
        _no_hdf5()
    head, slabs = _slabs(snapshot, block, ptype)
    width = 3 if block in ("POS ", "VEL ") else 1
    n = sum(s[2] for s in slabs)
    out = torch.empty((n, width) if width == 3 else (n,), dtype=torch.float32, device=device)
    if n == 0:
        return out
    flat = out.view(-1)
    cap = max(1, chunk_bytes // 4)
    bufs = [torch.empty(cap, dtype=torch.float32, pin_memory=True) for _ in range(2)]
    done = [None, None]
    stream = torch.cuda.Stream(device=device)
    pos = 0
    k = 0
    for fn, off, cnt, dt, const in slabs:
        left = cnt * width
        src_off = off
        with open(fn, "rb") if const is None else open(os.devnull, "rb") as f:
            while left > 0:
                m = min(left, cap)
                b = k % 2
                if done[b] is not None:
                    done[b].synchronize()          # its previous copy has landed
                view = bufs[b][:m].numpy()
                if const is not None:
                    view[:] = np.float32(const)
                else:
                    f.seek(src_off)
                    raw = f.read(4 * m)
                    a = np.frombuffer(raw, dtype=np.dtype(dt.base if dt.shape else dt))
                    view[:] = a if a.dtype.isnative else a.astype(np.float32)
                    src_off += 4 * m
                with torch.cuda.stream(stream):
                    flat[pos:pos + m].copy_(bufs[b][:m], non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record(stream)
                done[b] = ev
                pos += m
                left -= m
                k += 1
    stream.synchronize()
    if block == "VEL " and head.redshift != 0:
        out.mul_(math.sqrt(head.time))
    return out

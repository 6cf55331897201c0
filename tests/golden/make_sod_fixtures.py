"""Golden fixtures from the reference's Sod run (test data, not product).

The reference ships FP64 restart files of a 2-D Sod shock-tube run in
devel-izem/testcases/sod/restarts/restart_000NN.h5, written by
save_restart_hdf5 (devel-izem/src/module_io.f90:56-103): the interior
conserved variables /consvar/{rho,rhoU,rhoV,rhoW,rhoE,<species>} (ntx x nty
x ntz, FP64, code units) and /simulation/time (code units).  No HDF5 library
is installed here, so `read_h5` follows the few structures these files use:
a version-0 superblock, symbol-table groups (B-tree nodes 'TREE', local
heaps 'HEAP', symbol nodes 'SNOD'), version-1 object headers and contiguous
datasets (HDF5 File Format Specification, version 0 superblock).

Run from the repository root, where the reference tree is readable:

    python tests/golden/make_sod_fixtures.py /path/to/devel-izem/testcases/sod

It writes tests/golden/sod_restart_000NN.npz (arrays rho, rhoU, rhoV, rhoW,
rhoE, O2, N2 with shape (ntx, nty, ntz) in Fortran index order, and time)
and tests/golden/sod_grid.npz (the x, y, z coordinates of grid.dat, in
metres, parsed as the reference's list-directed read parses them).
"""
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
RESTARTS = (1, 2, 3)


def _u(d, off, n):
    return int.from_bytes(d[off:off + n], "little")


def _heap_name(d, heap, off):
    assert d[heap:heap + 4] == b"HEAP"
    data = _u(d, heap + 24, 8)
    end = d.index(b"\0", data + off)
    return d[data + off:end].decode()


def _group(d, btree, heap):
    """name -> (object header address, scratch) for a symbol-table group."""
    out = {}
    assert d[btree:btree + 4] == b"TREE", hex(btree)
    level, used = d[btree + 5], _u(d, btree + 6, 2)
    # keys and children follow the two sibling addresses: key0 child0 key1 child1 ...
    p = btree + 8 + 16 + 8
    for _ in range(used):
        child = _u(d, p, 8)
        p += 16
        if level > 0:
            out.update(_group(d, child, heap))
            continue
        assert d[child:child + 4] == b"SNOD"
        nsym = _u(d, child + 6, 2)
        q = child + 8
        for _ in range(nsym):
            name = _heap_name(d, heap, _u(d, q, 8))
            out[name] = (_u(d, q + 8, 8), _u(d, q + 16, 4), d[q + 24:q + 40])
            q += 40
    return out


def _messages(d, oh):
    assert d[oh] == 1, "object header version"
    nmsg = _u(d, oh + 2, 2)
    p = oh + 16
    for _ in range(nmsg):
        mtype, msize = _u(d, p, 2), _u(d, p + 2, 2)
        yield mtype, p + 8, msize
        p += 8 + msize


def _dataset(d, oh):
    dims, dtype, addr, size = None, None, None, None
    for mtype, p, _ in _messages(d, oh):
        if mtype == 1:      # dataspace
            ver, rank = d[p], d[p + 1]
            base = p + 8 if ver == 1 else p + 4
            dims = [_u(d, base + 8 * r, 8) for r in range(rank)]
        elif mtype == 3:    # datatype: floating point, byte order in bit 0 of the first bit field
            cls = d[p] & 0x0F
            size_b = _u(d, p + 4, 4)
            assert cls == 1 and size_b == 8, "FP64 expected"
            dtype = ">f8" if d[p + 1] & 1 else "<f8"
        elif mtype == 8:    # data layout, version 3: class 1 = contiguous
            assert d[p] == 3 and d[p + 1] == 1, "contiguous layout expected"
            addr, size = _u(d, p + 2, 8), _u(d, p + 10, 8)
    arr = np.frombuffer(d[addr:addr + size], dtype=dtype).astype(np.float64)
    # HDF5 stores the C-order extent of a Fortran array reversed: (ntz, nty, ntx)
    return arr.reshape(dims).transpose(tuple(range(len(dims) - 1, -1, -1)))


def read_h5(path):
    d = open(path, "rb").read()
    assert d[:8] == b"\x89HDF\r\n\x1a\n" and d[8] == 0, "version-0 superblock expected"
    root = 8 + 16 + 32          # root group symbol-table entry
    btree, heap = _u(d, root + 24, 8), _u(d, root + 32, 8)
    out = {}
    for gname, (_, cache, scratch) in _group(d, btree, heap).items():
        assert cache == 1
        gb, gh = struct.unpack("<QQ", scratch)
        for name, (oh, _, _) in _group(d, gb, gh).items():
            out["%s/%s" % (gname, name)] = _dataset(d, oh)
    return out


def read_grid(path):
    """The X-, Y- and Z-DIRECTION coordinate lists of a grid.dat file."""
    out, cur = {}, None
    for line in open(path):
        t = line.strip()
        if t.endswith("-DIRECTION"):
            cur = t[0].lower()
            out[cur] = []
        elif t == "END":
            break
        elif t and cur:
            out[cur].append(float(t))
    return {k: np.array(v, dtype=np.float64) for k, v in out.items()}


def main(sod_dir):
    np.savez_compressed(os.path.join(HERE, "sod_grid.npz"), **read_grid(os.path.join(sod_dir, "grid.dat")))
    for n in RESTARTS:
        f = read_h5(os.path.join(sod_dir, "restarts", "restart_%05d.h5" % n))
        arrays = {k.split("/")[1]: v for k, v in f.items() if k.startswith("consvar/")}
        arrays["time"] = np.asarray(f["simulation/time"]).reshape(-1)[:1]
        np.savez_compressed(os.path.join(HERE, "sod_restart_%05d.npz" % n), **arrays)
        print(n, {k: v.shape for k, v in arrays.items()}, float(arrays["time"][0]))


if __name__ == "__main__":
    main(sys.argv[1])

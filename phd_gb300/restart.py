"""Restart files in the reference's HDF5 layout (save_restart_hdf5 and
read_restart_hdf5, devel-izem/src/module_io.f90:56-197), so that a GPU run
can resume a reference restart and write one back.

A restart holds the interior conserved variables as 3-D FP64 datasets
/consvar/<name> of extent (ntx, nty, ntz) in Fortran index order (HDF5 stores
the reversed C-order extent), names rho, rhoU, rhoV, rhoW, rhoE and then the
species names, and the time (code units) as the 1-element dataset
/simulation/time.

No HDF5 library is installed on the machines this package runs on, so the
file structures are written and read here from the HDF5 File Format
Specification, version-0 superblock: symbol-table groups (a version-1 B-tree
of group nodes 'TREE', symbol nodes 'SNOD' and a local heap 'HEAP'),
version-1 object headers, and contiguous little-endian FP64 datasets whose
headers carry the same messages as the reference's files (dataspace with
maximum dimensions, IEEE double datatype, fill value, contiguous layout).
"""
import struct

import numpy as np

NIV_NAMES = ("rho", "rhoU", "rhoV", "rhoW", "rhoE")
SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
LEAF_K, INTERNAL_K = 4, 16      # group leaf / internal node K of the superblock


# ------------------------------------------------------------------ reading --
def _u(d, off, n):
    return int.from_bytes(d[off:off + n], "little")


def _heap_name(d, heap, off):
    if d[heap:heap + 4] != b"HEAP":
        raise ValueError("local heap expected at %#x" % heap)
    data = _u(d, heap + 24, 8)
    end = d.index(b"\0", data + off)
    return d[data + off:end].decode()


def _group(d, btree, heap):
    """name -> (object header address, cache type, scratch pad) of a group."""
    out = {}
    if d[btree:btree + 4] != b"TREE":
        raise ValueError("group B-tree expected at %#x" % btree)
    level, used = d[btree + 5], _u(d, btree + 6, 2)
    p = btree + 24 + 8          # after the header and key 0: child0 key1 child1 ...
    for _ in range(used):
        child = _u(d, p, 8)
        p += 16
        if level > 0:
            out.update(_group(d, child, heap))
            continue
        if d[child:child + 4] != b"SNOD":
            raise ValueError("symbol node expected at %#x" % child)
        q = child + 8
        for _ in range(_u(d, child + 6, 2)):
            out[_heap_name(d, heap, _u(d, q, 8))] = (_u(d, q + 8, 8), _u(d, q + 16, 4), d[q + 24:q + 40])
            q += 40
    return out


def _messages(d, oh):
    """(type, data address, size) of every message of a version-1 object
    header.  The header's first chunk follows its 16-byte prefix; an object
    header continuation message (type 0x10: address and length of a further
    block of messages) adds a chunk, and the prefix's message count covers
    the messages of every chunk, continuation and NIL messages included."""
    if d[oh] != 1:
        raise ValueError("version-1 object header expected at %#x" % oh)
    left = _u(d, oh + 2, 2)
    chunks = [(oh + 16, _u(d, oh + 8, 4))]
    while chunks and left > 0:
        p, n = chunks.pop(0)
        end = p + n
        while left > 0 and p + 8 <= end:
            mtype, msize = _u(d, p, 2), _u(d, p + 2, 2)
            left -= 1
            if mtype == 0x10:
                chunks.append((_u(d, p + 8, 8), _u(d, p + 16, 8)))
            else:
                yield mtype, p + 8, msize
            p += 8 + msize
    if left > 0:
        raise ValueError("object header at %#x: %d of its messages lie outside its chunks" % (oh, left))


def _dataset(d, oh):
    dims = dtype = addr = size = None
    for mtype, p, _ in _messages(d, oh):
        if mtype == 1:      # dataspace
            ver, rank = d[p], d[p + 1]
            base = p + 8 if ver == 1 else p + 4
            dims = [_u(d, base + 8 * r, 8) for r in range(rank)]
        elif mtype == 3:    # datatype: IEEE float, byte order in bit 0 of the first bit field
            if d[p] & 0x0F != 1 or _u(d, p + 4, 4) != 8:
                raise ValueError("FP64 dataset expected")
            dtype = ">f8" if d[p + 1] & 1 else "<f8"
        elif mtype == 8:    # data layout version 3, class 1 = contiguous
            if d[p] != 3 or d[p + 1] != 1:
                raise ValueError("contiguous layout expected")
            addr, size = _u(d, p + 2, 8), _u(d, p + 10, 8)
    arr = np.frombuffer(d[addr:addr + size], dtype=dtype).astype(np.float64)
    return arr.reshape(dims).transpose(tuple(range(len(dims) - 1, -1, -1)))


def read_h5(path):
    """Every dataset of a two-level file as {"group/name": array}, arrays in
    Fortran index order."""
    with open(path, "rb") as f:
        d = f.read()
    if d[:8] != SIG or d[8] != 0:
        raise ValueError("%s: HDF5 file with a version-0 superblock expected" % path)
    root = 8 + 16 + 32
    out = {}
    for gname, (_, cache, scratch) in _group(d, _u(d, root + 24, 8), _u(d, root + 32, 8)).items():
        if cache != 1:
            raise ValueError("group %s without a cached symbol table" % gname)
        gb, gh = struct.unpack("<QQ", scratch)
        for name, (oh, _, _) in _group(d, gb, gh).items():
            out["%s/%s" % (gname, name)] = _dataset(d, oh)
    return out


def read_restart(path):
    """(names, arrays, time): the /consvar datasets, rho, rhoU, rhoV, rhoW,
    rhoE first and then the species sorted by name (a group stores its
    members by name, not in the writer's order; state_from_restart takes the
    species order), and /simulation/time."""
    f = read_h5(path)
    cons = {k.split("/", 1)[1]: v for k, v in f.items() if k.startswith("consvar/")}
    species = sorted(n for n in cons if n not in NIV_NAMES)
    names = [n for n in NIV_NAMES if n in cons] + species
    return names, [cons[n] for n in names], float(np.asarray(f["simulation/time"]).reshape(-1)[0])


# ------------------------------------------------------------------ writing --
class _File:
    def __init__(self):
        self.buf = bytearray(96)        # superblock, filled last

    def alloc(self, n, align=8):
        pad = (-len(self.buf)) % align
        self.buf += b"\0" * pad
        at = len(self.buf)
        self.buf += b"\0" * n
        return at

    def put(self, at, data):
        self.buf[at:at + len(data)] = data


def _msg(mtype, body):
    body = bytes(body) + b"\0" * ((-len(body)) % 8)
    return struct.pack("<HHB3x", mtype, len(body), 0) + body


def _object_header(f, messages):
    body = b"".join(messages)
    at = f.alloc(16 + len(body))
    f.put(at, struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(body)) + body)
    return at


def _write_dataset(f, arr):
    a = np.asarray(arr, dtype="<f8")
    cdims = a.shape[::-1]                               # HDF5 extent of a Fortran-ordered array
    data = np.asfortranarray(a).tobytes(order="F")
    daddr = f.alloc(len(data))
    f.put(daddr, data)
    space = struct.pack("<BBBx4x", 1, len(cdims), 1) + b"".join(struct.pack("<Q", n) for n in cdims) * 2
    dtype = bytes([0x11, 0x20, 63, 0]) + struct.pack("<I", 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
    fill = bytes([2, 1, 2, 1])
    layout = struct.pack("<BBQQ", 3, 1, daddr, len(data))
    return _object_header(f, [_msg(1, space), _msg(3, dtype), _msg(5, fill), _msg(8, layout)])


def _write_group(f, entries):
    """entries: [(name, object header address, cache type, scratch)] ->
    (B-tree address, local heap address); names sorted as the format
    requires, at most 2 LEAF_K per symbol node."""
    entries = sorted(entries, key=lambda e: e[0].encode())
    heap_data = bytearray(8)                            # offset 0: the empty name
    offs = {}
    for name, *_ in entries:
        offs[name] = len(heap_data)
        s = name.encode() + b"\0"
        heap_data += s + b"\0" * ((-len(s)) % 8)
    heap = f.alloc(32)
    hdata = f.alloc(len(heap_data))
    f.put(hdata, heap_data)
    f.put(heap, b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap_data), UNDEF, hdata))   # no free block
    chunks = [entries[i:i + 2 * LEAF_K] for i in range(0, len(entries), 2 * LEAF_K)] or [[]]
    snods = []
    for ch in chunks:
        at = f.alloc(8 + 40 * 2 * LEAF_K)
        body = b"SNOD" + struct.pack("<BxH", 1, len(ch))
        for name, oh, cache, scratch in ch:
            body += struct.pack("<QQI4x", offs[name], oh, cache) + scratch.ljust(16, b"\0")
        f.put(at, body)
        snods.append((at, offs[ch[-1][0]] if ch else 0))
    bt = f.alloc(24 + (2 * INTERNAL_K + 1) * 8 + 2 * INTERNAL_K * 8)
    body = b"TREE" + struct.pack("<BBHQQ", 0, 0, len(snods), UNDEF, UNDEF) + struct.pack("<Q", 0)
    for at, key in snods:
        body += struct.pack("<QQ", at, key)
    f.put(bt, body)
    return bt, heap


def write_restart(path, names, arrays, time):
    """A restart file as save_restart_hdf5 writes it: /consvar/<names[i]> =
    arrays[i] (interior, Fortran index order) and /simulation/time."""
    if len(names) != len(arrays):
        raise ValueError("one array per name")
    f = _File()
    cons = [(n, _write_dataset(f, a), 0, b"") for n, a in zip(names, arrays)]
    cb, ch = _write_group(f, cons)
    cons_oh = _object_header(f, [_msg(0x11, struct.pack("<QQ", cb, ch))])
    t_oh = _write_dataset(f, np.array([float(time)]))
    sb, sh = _write_group(f, [("time", t_oh, 0, b"")])
    sim_oh = _object_header(f, [_msg(0x11, struct.pack("<QQ", sb, sh))])
    rb, rh = _write_group(f, [("consvar", cons_oh, 1, struct.pack("<QQ", cb, ch)),
                              ("simulation", sim_oh, 1, struct.pack("<QQ", sb, sh))])
    root_oh = _object_header(f, [_msg(0x11, struct.pack("<QQ", rb, rh))])
    eof = len(f.buf)
    sb_bytes = SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", LEAF_K, INTERNAL_K, 0)
    sb_bytes += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
    sb_bytes += struct.pack("<QQI4xQQ", 0, root_oh, 1, rb, rh)
    f.put(0, sb_bytes)
    with open(path, "wb") as out:
        out.write(bytes(f.buf))


# ------------------------------------------------- state <-> restart arrays --
def state_from_restart(names, arrays, ng, species=None):
    """Ghosted conserved variables (Fortran order, ghosts 0) from restart
    arrays, as read_restart_hdf5 fills v(sx:ex, sy:ey, sz:ez, :) before its
    closure (comm_cons, prim_inv_var_err_mach, upd_extrapolation and the
    ghost faces: izem_gpu_finalize_ic); species orders the species
    variables (default: the file's).  T starts at 0 as in the reference."""
    order = list(NIV_NAMES) + list(species if species is not None else [n for n in names if n not in NIV_NAMES])
    idx = {n: q for q, n in enumerate(names)}
    missing = [n for n in order if n not in idx]
    if missing:
        raise KeyError("restart lacks %s" % missing)
    nx, ny, nz = arrays[0].shape
    shp = (nx + 2 * ng, ny + 2 * ng, nz + 2 * ng)
    v = np.zeros(shp + (len(order),), order="F")
    for q, n in enumerate(order):
        v[ng:ng + nx, ng:ng + ny, ng:ng + nz, q] = arrays[idx[n]]
    nrv = len(order) - 5
    return {"v": v, "T": np.zeros(shp, order="F"), "W_i": np.zeros(shp, order="F"), "cp": np.zeros(shp, order="F"),
            "ha": np.zeros(shp + (nrv,), order="F"), "shock_sensor": np.zeros(shp, dtype=np.uint8, order="F")}


def restart_from_state(v, ng, species):
    """(names, arrays) of save_restart_hdf5 from the ghosted conserved
    variables: the interior of each variable."""
    names = list(NIV_NAMES) + list(species)
    sl = (slice(ng, v.shape[0] - ng), slice(ng, v.shape[1] - ng), slice(ng, v.shape[2] - ng))
    return names, [np.asfortranarray(v[sl + (q,)]) for q in range(len(names))]

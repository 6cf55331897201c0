"""Golden fixtures from the reference's Sod run (test data, not product).

The reference ships FP64 restart files of a 2-D Sod shock-tube run in
devel-izem/testcases/sod/restarts/restart_000NN.h5, written by
save_restart_hdf5 (devel-izem/src/module_io.f90:56-103): the interior
conserved variables /consvar/{rho,rhoU,rhoV,rhoW,rhoE,<species>} (ntx x nty
x ntz, FP64, code units) and /simulation/time (code units).  No HDF5 library
is installed here; phd_gb300.restart.read_h5 reads the few structures these
files use (version-0 superblock, symbol-table groups, version-1 object
headers, contiguous datasets).

Run from the repository root, where the reference tree is readable:

    python tests/golden/make_sod_fixtures.py /path/to/devel-izem/testcases/sod

It writes tests/golden/sod_restart_000NN.npz (arrays rho, rhoU, rhoV, rhoW,
rhoE, O2, N2 with shape (ntx, nty, ntz) in Fortran index order, and time)
tests/golden/sod_grid.npz (the x, y, z coordinates of grid.dat, in
metres, parsed as the reference's list-directed read parses them) and
tests/golden/sod_plot_000NN.npz (temperature, pressure, density and x
velocity of the post-processor's FP32 plot files, dimensional) and
tests/golden/sod_weno5_plot_000NN.npz (the same fields of
testcases/sod/weno5_400, the run repeated with ORDER_WENO = 5; its 400 x 11
plot files are the only output of that run the reference ships).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from phd_gb300.restart import read_h5  # noqa: E402
RESTARTS = (1, 2, 3, 10)
PLOTS = (1, 3)
WENO5_PLOTS = (1, 3)   # testcases/sod/weno5_400: the same run with ORDER_WENO = 5


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


def read_vtr(path):
    """(piece extent, {name: FP64 array}) of a VTK RectilinearGrid piece in
    raw appended big-endian FP32 (each block prefixed by its byte count), as
    the reference's post-processor writes plots/plotNNNNN_BBBBB.vtr."""
    import re
    d = open(path, "rb").read()
    head = d[:d.index(b"<AppendedData")].decode()
    arrs = re.findall(r'Name="([^"]+)" NumberOfComponents="1" format="appended" offset="(\d+)"', head)
    ext = [int(x) for x in re.search(r'Piece Extent="([^"]+)"', head).group(1).split()]
    start = d.index(b"_", d.index(b"<AppendedData")) + 1
    out = {}
    for name, off in arrs:
        o = start + int(off)
        n = int.from_bytes(d[o:o + 4], "big")
        out[name] = np.frombuffer(d[o + 4:o + 4 + n], dtype=">f4").astype(np.float64)
    return ext, out


def plot_fields(sod_dir, n, sub="plots"):
    """The two x-blocks of plot n of the directory `sub` merged on the
    400 x 11 grid (the blocks share the point at x index 200)."""
    fields = {}
    for piece in (0, 1):
        ext, d = read_vtr(os.path.join(sod_dir, sub, "plot%05d_%05d.vtr" % (n, piece)))
        nxp, nyp = ext[1] - ext[0] + 1, ext[3] - ext[2] + 1
        for name, key in (("Temperature", "T"), ("Pressure", "P"), ("Density", "rho"), ("Velocity-X", "u")):
            a = d[name].reshape(nyp, nxp).T
            f = fields.setdefault(key, np.zeros((400, nyp)))
            f[ext[0] - 1:ext[1]] = a
    return fields


def main(sod_dir):
    np.savez_compressed(os.path.join(HERE, "sod_grid.npz"), **read_grid(os.path.join(sod_dir, "grid.dat")))
    for n in RESTARTS:
        f = read_h5(os.path.join(sod_dir, "restarts", "restart_%05d.h5" % n))
        arrays = {k.split("/")[1]: v for k, v in f.items() if k.startswith("consvar/")}
        arrays["time"] = np.asarray(f["simulation/time"]).reshape(-1)[:1]
        np.savez_compressed(os.path.join(HERE, "sod_restart_%05d.npz" % n), **arrays)
        if n in PLOTS:
            np.savez_compressed(os.path.join(HERE, "sod_plot_%05d.npz" % n), **plot_fields(sod_dir, n))
        print(n, {k: v.shape for k, v in arrays.items()}, float(arrays["time"][0]))
    for n in WENO5_PLOTS:
        np.savez_compressed(os.path.join(HERE, "sod_weno5_plot_%05d.npz" % n),
                            **plot_fields(sod_dir, n, sub="weno5_400"))


if __name__ == "__main__":
    main(sys.argv[1])

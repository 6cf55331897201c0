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
and tests/golden/sod_grid.npz (the x, y, z coordinates of grid.dat, in
metres, parsed as the reference's list-directed read parses them).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from phd_gb300.restart import read_h5  # noqa: E402
RESTARTS = (1, 2, 3, 10)


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

"""Host-side set-up of the reference's thermodynamic and reference data.

Restates, in Python, the initialisation chain the Fortran host runs before the
hot path and passes to the GPU library through izem_gpu_init:

* ``constants``   -- module_tools.f90:453-571 (hard-coded non-dimensional
  references) with ``suth`` (module_tools.f90:582-591);
* ``read_therm``  -- thd_file_read_therm, thd/thd_tools_perfectgas.f90:367-458
  (CHEMKIN THERMO records: name in columns 1-18, T ranges in columns 46-75,
  then 5E15 / 5E15 / 4E15 coefficient lines);
* ``read_tranfit``-- thd_cofd_read, thd/thd_tools_perfectgas.f90:478-639
  (list-directed tranfit.out: diffusion, conductivity, viscosity fits,
  molar masses);
* ``thd_init``    -- thd/thd_tools_perfectgas.f90:12-229 (code units).

The species sets used by the workloads are shipped as JSON under
``phd_gb300/data`` (extracted from the reference's testcase files by
``phd_gb300/data/make_species_data.py``) because the reference tree is not
present where the library runs.
"""
import json
import math
import os

from .capi import IzemAdi, IzemThd, NSMAX, NPOLY

DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")


def suth(T):
    """Sutherland viscosity (module_tools.f90:582-591)."""
    return 1.4580e-6 * T ** 1.5 / (T + 110.4)


def vand(T):
    return 0.6938730e-6 * T


def constants():
    """Non-dimensional references, in the reference's operation order."""
    a = {}
    a["gamma_inf"] = 1.40
    gamma = a["gamma_inf"]
    gm1 = gamma - 1.0
    gm1_i = 1.0 / gm1
    a["re"] = 65000.0
    a["pr"] = 0.72
    a["le"] = 1.0
    a["ma"] = 2.25
    a["ggmopr"] = gamma * gm1_i / a["pr"]
    a["sqgmr"] = math.sqrt(gamma) * a["ma"] / a["re"]
    a["sc"] = a["le"] * a["pr"]
    a["t_ref"] = 169.44
    a["l_ref"] = 0.00004839025546795050
    a["r_ref"] = 8.31451
    r_m_ref = 287.15
    a["w_ref"] = a["r_ref"] / r_m_ref
    a["cp_ref"] = a["gamma_inf"] * (a["r_ref"] / a["w_ref"]) / (a["gamma_inf"] - 1.0)
    a["mu_ref"] = vand(a["t_ref"]) if a["t_ref"] < 110.4 else suth(a["t_ref"])
    a["c_inf"] = math.sqrt(a["gamma_inf"] * (a["r_ref"] / a["w_ref"]) * a["t_ref"])
    a["u_ref"] = a["c_inf"] / math.sqrt(a["gamma_inf"])
    u_inf = a["c_inf"] * a["ma"]
    a["time_ref"] = a["l_ref"] / a["u_ref"]
    a["rho_ref"] = a["re"] * a["mu_ref"] / (a["l_ref"] * u_inf)
    a["p_ref"] = a["rho_ref"] * (a["u_ref"] * a["u_ref"])
    a["lbda_ref"] = a["cp_ref"] * a["mu_ref"] / a["pr"]
    a["d_ref"] = a["lbda_ref"] / (a["rho_ref"] * a["cp_ref"] * a["le"])
    return a


def adi_struct(a=None):
    a = a or constants()
    s = IzemAdi()
    for name, _ in IzemAdi._fields_:
        setattr(s, name, a[name])
    return s


def _fortran_float(tok):
    return float(tok.replace("D", "E").replace("d", "e"))


def read_therm(path, names):
    """Parse a CHEMKIN THERMO file for the given species names.

    Returns {name: {"tmin", "tmax", "tlim", "high": [a1..a7], "low": [a1..a7]}}.
    The first record whose leading token equals the name wins, as in the
    reference reader's top-to-bottom search.
    """
    with open(path) as f:
        lines = f.read().splitlines()
    if lines[0].strip() not in ("THERMO", "THERMO ALL"):
        raise ValueError("not a THERMO file: %s" % path)
    out = {}
    for name in names:
        ln = 2
        found = None
        while ln < len(lines):
            rec = lines[ln]
            spec = rec[0:18]
            if spec.strip() == "END":
                break
            tok = spec.split()[0] if spec.split() else ""
            if tok == name:
                found = ln
                break
            ln += 4
        if found is None:
            raise KeyError("species %s not in %s" % (name, path))
        rec = lines[found].ljust(80)
        tmin = _fortran_float(rec[45:55])
        tmax = _fortran_float(rec[55:65])
        tlim = _fortran_float(rec[65:75])
        def fields(s, n):
            s = s.ljust(15 * n)
            return [_fortran_float(s[15 * q:15 * (q + 1)]) for q in range(n)]
        l2 = fields(lines[found + 1], 5)
        l3 = fields(lines[found + 2], 5)
        l4 = fields(lines[found + 3], 4)
        high = l2 + l3[0:2]
        low = l3[2:5] + l4
        out[name] = {"tmin": tmin, "tmax": tmax, "tlim": tlim, "high": high, "low": low}
    return out


def read_tranfit(path):
    """Parse tranfit.out (list-directed records, one value per record)."""
    with open(path) as f:
        recs = [r.strip() for r in f.read().splitlines() if r.strip() != ""]
    pos = [0]

    def nxt():
        r = recs[pos[0]]
        pos[0] += 1
        return r

    nreac = int(nxt().split()[0])
    nspec = int(nxt().split()[0])
    npoly = int(nxt().split()[0])
    nele = int(nxt().split()[0])
    names = [None] * nspec
    cofd = [[[0.0] * npoly for _ in range(nspec)] for _ in range(nspec)]
    for j in range(nspec):
        if int(nxt().split()[0]) != j + 1:
            raise ValueError("tranfit format")
        names[j] = nxt().split()[0]
        for k in range(j + 1):
            nxt()
            vals = [_fortran_float(nxt().split()[0]) for _ in range(npoly)]
            cofd[j][k] = vals
            cofd[k][j] = vals
    if int(nxt().split()[0]) != -2:
        raise ValueError("tranfit format")
    coflam = []
    for k in range(nspec):
        nxt()
        coflam.append([_fortran_float(nxt().split()[0]) for _ in range(npoly)])
    if int(nxt().split()[0]) != -2:
        raise ValueError("tranfit format")
    cofeta = []
    for k in range(nspec):
        nxt()
        cofeta.append([_fortran_float(nxt().split()[0]) for _ in range(npoly)])
    if int(nxt().split()[0]) != -2:
        raise ValueError("tranfit format")
    wmol = []
    for k in range(nspec):
        nxt()
        wmol.append(_fortran_float(nxt().split()[0]))
    nxt()
    awt = [_fortran_float(nxt().split()[0]) for _ in range(nele)]
    if int(nxt().split()[0]) != -2:
        raise ValueError("tranfit format")
    kncf = [[int(nxt().split()[0]) for _ in range(nele)] for _ in range(nspec)]
    if int(nxt().split()[0]) != -1:
        raise ValueError("tranfit format")
    return {"nreac": nreac, "names": names, "npoly": npoly, "cofd": cofd, "coflam": coflam,
            "cofeta": cofeta, "W_gmol": wmol, "awt_gmol": awt, "kncf": kncf}


def load_species(setname):
    """Load a shipped species set (thermo + transport fits) by name."""
    with open(os.path.join(DATA_DIR, "species_%s.json" % setname)) as f:
        return json.load(f)


def thd_init(species, a=None):
    """Build the izem_thd structure in code units (thd_tools_perfectgas.f90:12-229)."""
    a = a or constants()
    names = species["names"]
    ns = len(names)
    if ns > NSMAX:
        raise ValueError("too many species")
    t = IzemThd()
    t.nspc = ns
    gamma = a["gamma_inf"]
    gam_m1 = gamma - 1.0
    t.gam2 = gam_m1 / gamma
    t.tinf = a["t_ref"]
    t.pinf = a["p_ref"]
    t.p0 = 101325.0
    t.muinf = a["mu_ref"]
    t.laminf = a["lbda_ref"]
    winf = a["w_ref"]
    for k, nm in enumerate(names):
        W = species["W_gmol"][k] / 1000.0
        t.W[k] = W
        t.Wc[k] = W / winf
        t.Wc_i[k] = 1.0 / t.Wc[k]
        t.dinf[k] = a["d_ref"]
        th = species["therm"][nm]
        t.tpolymin[k] = th["tmin"]
        t.tpolymax[k] = th["tmax"]
        t.tpolylim[k] = th["tlim"]
        for c in range(7):
            t.heatcap[k][0][c] = th["low"][c]
            t.heatcap[k][1][c] = th["high"][c]
        for l in range(ns):
            for n in range(NPOLY):
                t.cofd[k][l][n] = species["cofd"][k][l][n]
        for n in range(NPOLY):
            t.coflam[k][n] = species["coflam"][k][n]
            t.cofeta[k][n] = species["cofeta"][k][n]
    return t


def eglib_link(sp):
    """EGLIB linking data (what the Linkeg file would hold) for a species
    set: molar masses, the molecular parameters of tran.dat, and the ln(eta)
    and ln(D_kl at 1 atm) fits of tranfit.out (CGS, cubic in ln T)."""
    from .capi import IzemEglib
    names = sp["names"]
    n = len(names)
    if "molecular" not in sp:
        raise ValueError("species set has no molecular parameters for EGLIB")
    L = IzemEglib()
    L.ns = n
    for k in range(n):
        lin, eps, sig, dip, pol, zrot = sp["molecular"][k]
        L.lin[k] = int(lin)
        L.wt[k] = sp["W_gmol"][k]
        L.eps[k], L.sig[k], L.dip[k], L.pol[k], L.zrot[k] = eps, sig, dip, pol, zrot
        for q in range(4):
            L.cofe[k][q] = sp["cofeta"][k][q]
            for l in range(n):
                L.cofd[k][l][q] = sp["cofd"][k][l][q]
    return L

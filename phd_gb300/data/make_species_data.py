"""Regenerate the species data files shipped with the package.

Reads the reference's own testcase data (CHEMKIN THERMO file and tranfit.out
transport fits) and writes them as JSON for the library and its tests:

  species_h2air9.json : H H2 O O2 OH H2O HO2 H2O2 N2
                        (testcases/shockedshearlayer/tranfit.out + testcases/sod/therm.dat,
                         molecular parameters from testcases/sod/tran.dat)
  species_o2n2.json   : O2 N2  (testcases/sod/tranfit.out + testcases/sod/therm.dat + tran.dat)
  species_air2.json   : two identical calorically perfect pseudo-species of air
                        (cp/R = 3.5 exactly, so gamma = 1.4), with power-law
                        transport fits giving Pr = 0.71; written from formulas,
                        not from the reference.

Usage:  python phd_gb300/data/make_species_data.py [REFERENCE_ROOT]
"""
import json
import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from phd_gb300.thd import read_therm, read_tranfit  # noqa: E402


def read_tran_dat(path, names):
    """Molecular parameters of the CHEMKIN transport database (tran.dat):
    geometry (0 atom, 1 linear, 2 nonlinear), Lennard-Jones well depth eps/k
    [K], collision diameter [Angstrom], dipole moment [Debye],
    polarizability [Angstrom^3], rotational relaxation number at 298 K."""
    out = {}
    with open(path) as f:
        for line in f:
            tok = line.split("!")[0].split()
            if len(tok) >= 7 and tok[0] in names and tok[0] not in out:
                out[tok[0]] = [int(tok[1])] + [float(x) for x in tok[2:7]]
    missing = [n for n in names if n not in out]
    if missing:
        raise ValueError("no transport data for %s in %s" % (missing, path))
    return out


def build(tranfit_path, therm_path, tran_path=None):
    tf = read_tranfit(tranfit_path)
    th = read_therm(therm_path, tf["names"])
    d = {"names": tf["names"], "W_gmol": tf["W_gmol"], "cofd": tf["cofd"], "coflam": tf["coflam"],
            "cofeta": tf["cofeta"], "awt_gmol": tf["awt_gmol"], "kncf": tf["kncf"], "therm": th,
            "source": [os.path.relpath(tranfit_path, REF), os.path.relpath(therm_path, REF)]}
    if tran_path:
        lj = read_tran_dat(tran_path, tf["names"])
        d["molecular"] = [lj[n] for n in tf["names"]]   # lin, eps/k, sigma, dipole, polarizability, zrot
        d["source"].append(os.path.relpath(tran_path, REF))
    return d


def air2():
    # mu(T) = mu0 (T/300)^0.7 [kg/m/s]; lambda = mu cp / Pr; D = mu / (rho Sc) at 1 atm.
    W = 28.9647          # g/mol
    R = 8.31451
    cp = 3.5 * R / (W * 1e-3)
    mu0, n, Pr, Sc = 1.846e-5, 0.7, 0.71, 0.71
    # ln(q_cgs) = c0 + c1 ln T
    eta_c1 = n
    eta_c0 = math.log(mu0 * 10.0) - n * math.log(300.0)          # g/cm/s
    lam0 = mu0 * cp / Pr                                            # W/m/K
    lam_c0 = math.log(lam0 * 1e5) - n * math.log(300.0)            # erg/cm/K/s
    rho0 = 101325.0 / (R / (W * 1e-3) * 300.0)
    d0 = mu0 / (rho0 * Sc) * 1e4                                    # cm^2/s at 1 atm
    d_c1 = 1.0 + n
    d_c0 = math.log(d0) - d_c1 * math.log(300.0)
    a6 = -3.5 * 298.15
    coef = [3.5, 0.0, 0.0, 0.0, 0.0, a6, 0.0]
    therm = {nm: {"tmin": 200.0, "tmax": 6000.0, "tlim": 1000.0, "high": list(coef), "low": list(coef)}
             for nm in ("AIRA", "AIRB")}
    cofd = [[[d_c0, d_c1, 0.0, 0.0] for _ in range(2)] for _ in range(2)]
    return {"names": ["AIRA", "AIRB"], "W_gmol": [W, W], "cofd": cofd,
            "coflam": [[lam_c0, n, 0.0, 0.0]] * 2, "cofeta": [[eta_c0, eta_c1, 0.0, 0.0]] * 2,
            "awt_gmol": [], "kncf": [[], []], "therm": therm,
            "source": ["formula: cp/R=3.5, mu=1.846e-5 (T/300)^0.7 kg/m/s, Pr=Sc=0.71"]}


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_species_data.py <root of the reference checkout (holds devel-izem/)>")
    REF = sys.argv[1]
    tc = os.path.join(REF, "devel-izem", "testcases")
    sets = {
        "h2air9": build(os.path.join(tc, "shockedshearlayer", "tranfit.out"), os.path.join(tc, "sod", "therm.dat"),
                        os.path.join(tc, "sod", "tran.dat")),
        "o2n2": build(os.path.join(tc, "sod", "tranfit.out"), os.path.join(tc, "sod", "therm.dat"),
                      os.path.join(tc, "sod", "tran.dat")),
        "air2": air2(),
    }
    for name, data in sets.items():
        with open(os.path.join(HERE, "species_%s.json" % name), "w") as f:
            json.dump(data, f, indent=1)
        print("wrote species_%s.json (%s)" % (name, " ".join(data["names"])))

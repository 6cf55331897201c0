"""CHEMKIN-II mechanism reader (the subset of ckinterp the H2/air set uses).

Builds the izem_mech structure (the information ckinterp writes to chem.bin
and CKINIT loads, devel-izem/src/chemkin/vode.f:391): species, NASA-7 thermo
(taken from the shipped THERMO data, CHEMKIN mid-temperature switch),
reactions with Arrhenius parameters converted to E/R, explicit reverse
parameters (REV), third-body efficiencies, LOW fall-off and TROE.

Supported syntax: ELEMENTS/SPECIES/REACTIONS/END blocks, '!' comments, the
REACTIONS units keywords CAL/MOLE KCAL/MOLE JOULES/MOLE KJOULES/MOLE
KELVINS, '=', '<=>', '=>', '+M', '(+M)', a species as the fall-off collider
'(+K)', integer stoichiometric prefixes, auxiliary keywords REV, LOW, TROE,
SRI (3 or 5 parameters; d = 1, e = 0 when 3 are given), LT and RLT
(Landau-Teller B, C; RLT with REV) and species efficiencies 'S/val/'.
"""
import os
import re

from .capi import IzemMech, MAXREAC, NSMAX
from .thd import DATA_DIR, load_species

RU = 8.314510e7           # erg/mol/K  (CHEMKIN-II CKRP)
RUC = RU / 4.184e7        # cal/mol/K
PATM = 1.01325e6          # dyn/cm^2

_E_UNITS = {"CAL/MOLE": 1.0 / RUC, "KCAL/MOLE": 1000.0 / RUC, "JOULES/MOLE": 1.0 / (RU * 1e-7),
            "KJOULES/MOLE": 1000.0 / (RU * 1e-7), "KELVINS": 1.0}


def _strip(line):
    return line.split("!")[0].rstrip()


def _side(txt, species):
    """Parse one side of a reaction equation -> list of (species index, coeff),
    whether it carries +M, whether it carries a fall-off collider (+M) or
    (+K), and the collider as izem_mech's kfal (0: (+M), k+1: species k)."""
    txt = txt.replace(" ", "")
    fall, kfal = False, 0
    col = re.search(r"\(\+([^()]+)\)", txt)
    if col:
        fall = True
        nm = col.group(1)
        if nm.upper() != "M":
            if nm not in species:
                raise ValueError("unknown fall-off collider %s" % nm)
            kfal = species.index(nm) + 1
        txt = txt.replace(col.group(0), "")
    parts = [p for p in txt.split("+") if p]
    thb = False
    out = {}
    for p in parts:
        if p == "M":
            thb = True
            continue
        m = re.match(r"^(\d*)(.+)$", p)
        n = int(m.group(1)) if m.group(1) else 1
        nm = m.group(2)
        if nm not in species:
            raise ValueError("unknown species %s" % nm)
        k = species.index(nm)
        out[k] = out.get(k, 0) + n
    return sorted(out.items()), thb, fall, kfal


def read_mechanism(path, thermo_set="h2air9"):
    with open(path) as f:
        lines = [_strip(l) for l in f]
    lines = [l for l in lines if l.strip()]
    species = []
    q = 0
    escale = 1.0 / RUC
    reactions = []
    while q < len(lines):
        key = lines[q].split()[0].upper()
        if key.startswith("ELEM"):
            q += 1
            while lines[q].strip().upper() != "END":
                q += 1
            q += 1
        elif key.startswith("SPEC"):
            q += 1
            while lines[q].strip().upper() != "END":
                species += lines[q].split()
                q += 1
            q += 1
        elif key.startswith("REAC"):
            for tok in lines[q].split()[1:]:
                if tok.upper() in _E_UNITS:
                    escale = _E_UNITS[tok.upper()]
            q += 1
            while lines[q].strip().upper() != "END":
                l = lines[q]
                up = l.strip().upper()
                if "=" in l and not up.startswith(("REV", "LOW", "TROE", "SRI")):
                    toks = l.split()
                    A, b, E = float(toks[-3]), float(toks[-2]), float(toks[-1])
                    eq = "".join(toks[:-3])
                    if "<=>" in eq:
                        lhs, rhs = eq.split("<=>"); rev = 1
                    elif "=>" in eq:
                        lhs, rhs = eq.split("=>"); rev = 0
                    else:
                        lhs, rhs = eq.split("="); rev = 1
                    r, thb1, fall1, kfal1 = _side(lhs, species)
                    p, thb2, fall2, kfal2 = _side(rhs, species)
                    if fall1 != fall2 or kfal1 != kfal2:
                        raise ValueError("fall-off collider differs between the sides: %s" % eq)
                    reactions.append({"eq": eq, "reac": r, "prod": p, "par": (A, b, E * escale), "rev": rev,
                                      "rpar": None, "thb": thb1 or (fall1 and not kfal1), "fall": 1 if fall1 else 0,
                                      "kfal": kfal1, "low": None, "troe": None, "sri": None, "lt": None,
                                      "rlt": None, "eff": {}})
                else:
                    rx = reactions[-1]
                    for kw, body in re.findall(r"([A-Za-z0-9()]+)\s*/([^/]*)/", l):
                        kwu = kw.upper()
                        vals = [float(x) for x in body.split()]
                        if kwu == "REV":
                            rx["rev"] = 2
                            rx["rpar"] = (vals[0], vals[1], vals[2] * escale)
                        elif kwu == "LOW":
                            rx["low"] = (vals[0], vals[1], vals[2] * escale)
                        elif kwu == "TROE":
                            rx["troe"] = vals
                        elif kwu in ("LT", "RLT"):
                            if len(vals) != 2:
                                raise ValueError("%s takes 2 parameters: %s" % (kwu, rx["eq"]))
                            rx[kwu.lower()] = vals
                        elif kwu == "SRI":
                            if len(vals) not in (3, 5):
                                raise ValueError("SRI takes 3 or 5 parameters: %s" % rx["eq"])
                            rx["sri"] = vals + [1.0, 0.0][len(vals) - 3:]
                        elif kw in species:
                            rx["eff"][species.index(kw)] = vals[0]
                        else:
                            raise ValueError("unsupported auxiliary keyword %s" % kw)
                q += 1
            q += 1
        else:
            q += 1
    return build_struct(species, reactions, thermo_set)


def build_struct(species, reactions, thermo_set):
    sp = load_species(thermo_set)
    if sp["names"] != species:
        raise ValueError("mechanism species %s differ from thermo set %s" % (species, sp["names"]))
    if len(reactions) > MAXREAC or len(species) > NSMAX:
        raise ValueError("mechanism too large")
    m = IzemMech()
    m.kk, m.ii = len(species), len(reactions)
    m.ru, m.patm = RU, PATM
    for k, nm in enumerate(species):
        m.wt[k] = sp["W_gmol"][k]
        th = sp["therm"][nm]
        m.tmid[k] = th["tlim"]
        for c in range(7):
            m.a[k][0][c] = th["low"][c]
            m.a[k][1][c] = th["high"][c]
    for i, rx in enumerate(reactions):
        for s in range(6):
            m.nuk[i][s] = -1
            m.nu[i][s] = 0
        if len(rx["reac"]) > 3 or len(rx["prod"]) > 3:
            raise ValueError("more than 3 species on a side: %s" % rx["eq"])
        for s, (k, n) in enumerate(rx["reac"]):
            m.nuk[i][s] = k
            m.nu[i][s] = -n
        for s, (k, n) in enumerate(rx["prod"]):
            m.nuk[i][3 + s] = k
            m.nu[i][3 + s] = n
        for c in range(3):
            m.par[i][c] = rx["par"][c]
        m.rev[i] = rx["rev"]
        if rx["rpar"]:
            for c in range(3):
                m.rpar[i][c] = rx["rpar"][c]
        m.thb[i] = 1 if rx["thb"] else 0
        if rx["rlt"] and rx["rev"] != 2:
            raise ValueError("RLT without REV: %s" % rx["eq"])
        for key in ("lt", "rlt"):
            if rx[key]:
                for c in range(2):
                    getattr(m, key)[i][c] = rx[key][c]
        for k in range(len(species)):
            m.eff[i][k] = rx["eff"].get(k, 1.0)
        if rx["fall"]:
            if rx["low"] is None:
                raise ValueError("fall-off reaction without LOW: %s" % rx["eq"])
            if rx["troe"] and rx["sri"]:
                raise ValueError("both TROE and SRI: %s" % rx["eq"])
            if rx["troe"] and len(rx["troe"]) not in (3, 4):
                raise ValueError("TROE takes 3 or 4 parameters: %s" % rx["eq"])
            m.fall[i] = len(rx["troe"]) if rx["troe"] else (2 if rx["sri"] else 1)
            m.kfal[i] = rx["kfal"]
            for c in range(3):
                m.low[i][c] = rx["low"][c]
            if rx["troe"]:
                for c, val in enumerate(rx["troe"]):
                    m.troe[i][c] = val
            if rx["sri"]:
                for c, val in enumerate(rx["sri"]):
                    m.sri[i][c] = val
    return m


def h2_mechanism():
    """The shipped 9-species H2/air mechanism (CHEMKIN input written from the
    reference's hard-coded San Diego / Boivin rate data)."""
    return read_mechanism(os.path.join(DATA_DIR, "h2_sandiego12.inp"), "h2air9")

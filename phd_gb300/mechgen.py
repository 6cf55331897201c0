"""Mechanism compiler: the constant-volume reactor right-hand side of one
CHEMKIN mechanism as straight-line CUDA code.

The chemistry kernels evaluate CHEMKIN's rate expressions (CKCVBS, CKHMS,
CKRATT, CKRATX, CKWYR; chemkin/vode.f) for whatever mechanism the caller
uploads, walking its reaction tables at run time.  Species concentrations,
rates of progress and production rates are then indexed by table entries,
so they live in local memory, and every term costs a table load and a
branch.  For a mechanism known when the library is built this module writes
the same expressions, in the same operation order, with the table entries
as literals: reaction loops unrolled, indices fixed, absent terms dropped.
The arithmetic is the generic form's (fun_tpart / fun_cpart in chem.cu),
operation for operation, so a host build of the two gives identical bits.

Supported: irreversible reactions, reverse rates from the equilibrium
constant (CKSMH's entropy-enthalpy difference) or from explicit parameters
(REV), +M third bodies with efficiencies, Lindemann, SRI and Troe (3 or 4
parameter) fall-off with the (+M) collider or one species (+K), and
Landau-Teller factors on forward (LT) and explicit reverse (RLT) rates.

``python -m phd_gb300.mechgen`` rewrites ``csrc/chem_gen.cuh`` from the
shipped mechanism; a test checks that the committed file is what this
module writes.
"""
import os
import struct

HERE = os.path.dirname(os.path.abspath(__file__))
LT_P1 = 1.0 / 3.0        # the Landau-Teller exponents of chem.cu (kLtP1, kLtP2)
LT_P2 = 2.0 * LT_P1
OUT = os.path.join(HERE, "csrc", "chem_gen.cuh")


def lit(x):
    """A double literal that reads back to exactly x (C99/C++17 hex float)."""
    x = float(x)
    if x == 0.0:
        return "-0.0" if struct.pack(">d", x)[0] & 0x80 else "0.0"
    return "(%s)" % x.hex() if x < 0 else x.hex()


def bits(x):
    return "0x%016xULL" % struct.unpack("<Q", struct.pack("<d", float(x)))[0]


def powi_expr(x, m):
    """powi(x, m) of chem.cu for m > 0, unrolled: the same products in the
    same order (y = 1.0 * x^2 is x^2 exactly)."""
    assert m > 0
    n = m
    y = x if n % 2 else None
    xx = x
    n >>= 1
    while n:
        xx = "(%s * %s)" % (xx, xx)
        if n % 2:
            y = xx if y is None else "(%s * %s)" % (y, xx)
        n >>= 1
    return y


def _reactions(m):
    out = []
    for i in range(m.ii):
        r = {"i": i, "nuk": list(m.nuk[i]), "nu": list(m.nu[i]), "par": list(m.par[i]), "rev": m.rev[i],
             "rpar": list(m.rpar[i]), "thb": m.thb[i], "fall": m.fall[i], "low": list(m.low[i]),
             "troe": list(m.troe[i]), "sri": list(m.sri[i]), "kfal": m.kfal[i],
             "lt": list(m.lt[i]), "rlt": list(m.rlt[i]),
             "eff": [m.eff[i][k] for k in range(m.kk)]}
        if r["fall"] not in (0, 1, 2, 3, 4):
            raise NotImplementedError("reaction %d: fall-off form %d" % (i, r["fall"]))
        if r["nu"][0] == 0:
            raise NotImplementedError("reaction %d: no reactant" % i)
        out.append(r)
    return out


def generate(m, name="h2air9", source="phd_gb300/data/h2_sandiego12.inp"):
    kk = m.kk
    R = _reactions(m)
    rev = [r["i"] for r in R if r["rev"] != 0]
    eqk = any(r["rev"] == 1 for r in R)
    fall = [r["i"] for r in R if r["fall"]]
    troe = [r["i"] for r in R if r["fall"] > 1]
    kr_slot = {i: q for q, i in enumerate(rev)}
    lo_slot = {i: q for q, i in enumerate(fall)}
    tr_slot = {i: q for q, i in enumerate(troe)}
    wt_inv = [1.0 / m.wt[k] for k in range(kk)]
    ru_wt = [m.ru / m.wt[k] for k in range(kk)]
    L = []
    w = L.append
    w("// Generated by phd_gb300/mechgen.py from %s -- do not edit." % source)
    w("// The constant-volume reactor right-hand side of this mechanism (%d species," % kk)
    w("// %d reactions) as straight-line code: the expressions and operation order of" % m.ii)
    w("// fun_tpart / fun_cpart in chem.cu with the mechanism's tables as literals.")
    w("#pragma once")
    w("")
    w("namespace chem_gen {")
    w("")
    w("constexpr int KK = %d;" % kk)
    w("")
    w("// temperature terms of one right-hand side; the finite-difference Jacobian's")
    w("// species columns reuse them (rc_drive)")
    w("struct FunT {")
    w("  double T;")
    w("  double rut;")
    w("  double cvk[%d], h[%d];" % (kk, kk))
    w("  double kf[%d];" % m.ii)
    if rev:
        w("  double kr[%d];   // reactions %s" % (len(rev), ", ".join(map(str, rev))))
    if fall:
        w("  double klow[%d];   // reactions %s" % (len(fall), ", ".join(map(str, fall))))
    if troe:
        w("  double fclog[%d];   // reactions %s" % (len(troe), ", ".join(map(str, troe))))
    w("};")
    w("")
    # ---------------------------------------------------------------- tpart
    w("HD __forceinline__ void tpart(double T, FunT& t) {")
    w("  const double Tinv = 1.0 / T;")
    w("  const double alogt = log(T);")
    w("  const double T2 = T * T, T3 = T * T2, T4 = T2 * T2;")
    w("  t.T = T;")
    w("  t.rut = T * %s;" % lit(m.ru))
    if eqk:
        w("  double %s;   // S/R - H/RT (CKSMH)" % ", ".join("smh%d" % k for k in range(kk)))
    for k in range(kk):
        lo, hi = list(m.a[k][0]), list(m.a[k][1])
        w("  {   // species %d" % k)
        w("    const bool hi = T > %s;" % lit(m.tmid[k]))
        for j in range(7 if eqk else 6):
            w("    const double a%d = hi ? %s : %s;" % (j, lit(hi[j]), lit(lo[j])))
        w("    const double cps = a0 + T * a1 + T2 * a2 + T3 * a3 + T4 * a4;")
        w("    t.cvk[%d] = %s * (cps - 1.0);" % (k, lit(ru_wt[k])))
        w("    const double hs = a0 + (0.5 * T) * a1 + (T2 * (1.0 / 3.0)) * a2 + (0.25 * T3) * a3 + (0.2 * T4) * a4;")
        w("    t.h[%d] = t.rut * (hs + a5 * Tinv) * %s;" % (k, lit(wt_inv[k])))
        if eqk:
            w("    const double sv = (alogt - 1.0) * a0 + (0.5 * T) * a1 + (T2 * (1.0 / 6.0)) * a2 +")
            w("                      (T3 * (1.0 / 12.0)) * a3 + (T4 * 0.05) * a4;")
            w("    smh%d = sv + a6 - a5 * Tinv;" % k)
        w("  }")
    for r in R:
        i = r["i"]
        p = r["par"]
        w("  t.kf[%d] = %s * exp(%s * alogt - %s * Tinv);" % (i, lit(p[0]), lit(p[1]), lit(p[2])))
        if any(r["lt"]):   # Landau-Teller: the expression of fun_tpart
            w("  t.kf[%d] = t.kf[%d] * exp(%s / pow(T, %s) + %s / pow(T, %s));"
              % (i, i, lit(r["lt"][0]), lit(LT_P1), lit(r["lt"][1]), lit(LT_P2)))
        if r["rev"] == 2:
            q = r["rpar"]
            w("  t.kr[%d] = %s * exp(%s * alogt - %s * Tinv);" % (kr_slot[i], lit(q[0]), lit(q[1]), lit(q[2])))
        elif r["rev"] == 1:   # k_f / K_c, K_c from the species' S/R - H/RT
            w("  {")
            w("    double sumsmh = 0.0;")
            for n in range(6):
                if r["nuk"][n] >= 0:
                    w("    sumsmh = sumsmh + %s * smh%d;" % (lit(float(r["nu"][n])), r["nuk"][n]))
            w("    double eqk = sumsmh != 0.0 ? exp(fmin(sumsmh, 690.77552789821368)) : 1.0;")
            w("    eqk = eqk * powi(%s * Tinv / %s, %d);" % (lit(m.patm), lit(m.ru), sum(r["nu"])))
            w("    t.kr[%d] = t.kf[%d] / fmax(eqk, 1.0e-300);" % (kr_slot[i], i))
            w("  }")
        if any(r["rlt"]):
            w("  t.kr[%d] = t.kr[%d] * exp(%s / pow(T, %s) + %s / pow(T, %s));"
              % (kr_slot[i], kr_slot[i], lit(r["rlt"][0]), lit(LT_P1), lit(r["rlt"][1]), lit(LT_P2)))
        if r["fall"]:
            q = r["low"]
            w("  t.klow[%d] = %s * exp(%s * alogt - %s * Tinv);" % (lo_slot[i], lit(q[0]), lit(q[1]), lit(q[2])))
            if r["fall"] == 2:   # SRI: ln(a exp(-b/T) + exp(-T/c)) in the fclog slot
                sr = r["sri"]
                cinv = 1.0 / sr[2] if sr[2] != 0.0 else 0.0
                w("  t.fclog[%d] = log(%s * exp(-%s * Tinv) + exp(-T * %s));" % (tr_slot[i], lit(sr[0]), lit(sr[1]),
                                                                                  lit(cinv)))
            elif r["fall"] > 1:
                ta = r["troe"][0]
                ti0 = 1.0 / r["troe"][1] if r["troe"][1] != 0.0 else 0.0
                ti1 = 1.0 / r["troe"][2] if r["troe"][2] != 0.0 else 0.0
                w("  {")
                w("    const double ta = %s;" % lit(ta))
                w("    double fcent = (1.0 - ta) * exp(-T * %s) + ta * exp(-T * %s);" % (lit(ti0), lit(ti1)))
                if r["fall"] == 4:
                    w("    fcent = fcent + exp(-%s * Tinv);" % lit(r["troe"][3]))
                w("    t.fclog[%d] = log(fmax(fcent, 1.0e-300)) * 0.4342944819032518277;" % tr_slot[i])
                w("  }")
    w("}")
    w("")
    # ---------------------------------------------------------------- cpart
    w("HD __forceinline__ void cpart(double rho, const double* z, const FunT& t, double* zp) {")
    w("  const double* Y = z + 1;")
    w("  double cv = 0.0, ctot = 0.0;")
    for k in range(kk):
        w("  cv = cv + Y[%d] * t.cvk[%d];" % (k, k))
        w("  const double C%d = rho * Y[%d] * %s;" % (k, k, lit(wt_inv[k])))
        w("  ctot = ctot + C%d;" % k)
    for r in R:
        i = r["i"]
        nuk, nu = r["nuk"], r["nu"]
        w("  double rop%d;" % i)
        w("  {   // reaction %d" % i)
        w("    double rkft = t.kf[%d];" % i)
        isrev = r["rev"] != 0
        if isrev:
            w("    double rkrt = t.kr[%d];" % kr_slot[i])
        ctb = None
        if r["thb"]:
            w("    double ctb = ctot;")
            for k in range(kk):
                if r["eff"][k] != 1.0:
                    w("    ctb = ctb + %s * C%d;" % (lit(r["eff"][k] - 1.0), k))
            ctb = "ctb"
        if r["fall"]:
            f = lo_slot[i]
            if r["kfal"]:   # one species is the collider; a third-body factor stays
                w("    const double pr = t.klow[%d] * C%d / rkft;" % (f, r["kfal"] - 1))
            else:
                w("    const double pr = t.klow[%d] * %s / rkft;" % (f, ctb if ctb else "1.0"))
                ctb = None
            w("    double pcor = pr / (1.0 + pr);")
            if r["fall"] == 2:
                w("    {")
                w("      const double prlog = log(fmax(pr, 1.0e-300)) * 0.4342944819032518277;")
                w("      const double xp = 1.0 / (1.0 + prlog * prlog);")
                w("      pcor = exp(xp * t.fclog[%d]) * %s * pow(t.T, %s) * pcor;" % (tr_slot[i], lit(r["sri"][3]),
                                                                                   lit(r["sri"][4])))
                w("    }")
            elif r["fall"] > 1:
                w("    {")
                w("      const double prlog = log(fmax(pr, 1.0e-300)) * 0.4342944819032518277;")
                w("      const double fclog = t.fclog[%d];" % tr_slot[i])
                w("      const double xn = 0.75 - 1.27 * fclog;")
                w("      const double cprlog = prlog - (0.4 + 0.67 * fclog);")
                w("      const double q = cprlog / (xn - 0.14 * cprlog);")
                w("      const double flog = fclog / (1.0 + q * q);")
                w("      pcor = exp(flog * 2.302585092994045684) * pcor;")
                w("    }")
            w("    rkft = rkft * pcor;")
            if isrev:
                w("    rkrt = rkrt * pcor;")
        if ctb:
            w("    rkft = rkft * ctb;")
            if isrev:
                w("    rkrt = rkrt * ctb;")
        w("    double rkf = rkft * %s;" % powi_expr("C%d" % nuk[0], -nu[0]))
        if isrev:
            w("    double rkr = rkrt * %s;" % powi_expr("C%d" % nuk[3], nu[3]))
        if nuk[1] >= 0:
            w("    rkf = rkf * %s;" % powi_expr("C%d" % nuk[1], -nu[1]))
            if nuk[2] >= 0:
                w("    rkf = rkf * %s;" % powi_expr("C%d" % nuk[2], -nu[2]))
        if isrev and nuk[4] >= 0:
            w("    rkr = rkr * %s;" % powi_expr("C%d" % nuk[4], nu[4]))
            if nuk[5] >= 0:
                w("    rkr = rkr * %s;" % powi_expr("C%d" % nuk[5], nu[5]))
        w("    rop%d = %s;" % (i, "rkf - rkr" if isrev else "rkf"))
        w("  }")
    # production rates, in the generic accumulation order (slot outer, reaction inner)
    acc = {k: [] for k in range(kk)}
    for n in range(6):
        for r in R:
            k = r["nuk"][n]
            if k >= 0:
                acc[k].append("rop%d * %s" % (r["i"], lit(float(r["nu"][n]))))
    for k in range(kk):
        expr = "0.0"
        for t in acc[k]:
            expr = "(%s + %s)" % (expr, t)
        w("  const double wdot%d = %s;" % (k, expr))
    w("  const double rho_i = 1.0 / rho;")
    w("  double sum = 0.0;")
    for k in range(kk):
        w("  zp[%d] = wdot%d * %s * rho_i;" % (k + 1, k, lit(m.wt[k])))
        w("  sum = sum + t.h[%d] * wdot%d * %s + (-t.rut) * wdot%d;" % (k, k, lit(m.wt[k]), k))
    w("  zp[0] = -sum / (rho * cv);")
    w("}")
    w("")
    # ------------------------------------------------------- host check
    w("// True when m is the mechanism this file was generated from (every table")
    w("// entry the right-hand side reads, bit for bit).")
    w("inline bool matches(const izem_mech& m) {")
    w("  auto b = [](double x) { unsigned long long u; memcpy(&u, &x, sizeof(u)); return u; };")
    w("  if (m.kk != %d || m.ii != %d || b(m.ru) != %s) return false;" % (kk, m.ii, bits(m.ru)))
    conds = []
    for k in range(kk):
        conds.append("b(m.wt[%d]) == %s" % (k, bits(m.wt[k])))
        conds.append("b(m.tmid[%d]) == %s" % (k, bits(m.tmid[k])))
        for s_ in range(2):
            for j in range(7):
                conds.append("b(m.a[%d][%d][%d]) == %s" % (k, s_, j, bits(m.a[k][s_][j])))
    for r in R:
        i = r["i"]
        for n in range(6):
            conds.append("m.nuk[%d][%d] == %d && m.nu[%d][%d] == %d" % (i, n, r["nuk"][n], i, n, r["nu"][n]))
        for j in range(3):
            conds.append("b(m.par[%d][%d]) == %s" % (i, j, bits(r["par"][j])))
        conds.append("m.rev[%d] == %d && m.thb[%d] == %d && m.fall[%d] == %d" % (i, r["rev"], i, r["thb"], i, r["fall"]))
        for j in range(2):
            conds.append("b(m.lt[%d][%d]) == %s && b(m.rlt[%d][%d]) == %s" % (i, j, bits(r["lt"][j]), i, j,
                                                                          bits(r["rlt"][j])))
        if r["rev"] == 2:
            for j in range(3):
                conds.append("b(m.rpar[%d][%d]) == %s" % (i, j, bits(r["rpar"][j])))
        if r["thb"]:
            for k in range(kk):
                conds.append("b(m.eff[%d][%d]) == %s" % (i, k, bits(r["eff"][k])))
        if r["fall"]:
            conds.append("m.kfal[%d] == %d" % (i, r["kfal"]))
            for j in range(3):
                conds.append("b(m.low[%d][%d]) == %s" % (i, j, bits(r["low"][j])))
            if r["fall"] == 2:
                for j in range(5):
                    conds.append("b(m.sri[%d][%d]) == %s" % (i, j, bits(r["sri"][j])))
            elif r["fall"] > 1:
                for j in range(4 if r["fall"] == 4 else 3):
                    conds.append("b(m.troe[%d][%d]) == %s" % (i, j, bits(r["troe"][j])))
    for q in range(0, len(conds), 4):
        w("  if (!(%s)) return false;" % " && ".join(conds[q:q + 4]))
    w("  return true;")
    w("}")
    w("")
    w("}  // namespace chem_gen")
    return "\n".join(L) + "\n"


def main():
    from .mech import h2_mechanism
    text = generate(h2_mechanism())
    with open(OUT, "w") as f:
        f.write(text)
    print("wrote %s (%d lines)" % (OUT, text.count("\n")))


if __name__ == "__main__":
    main()

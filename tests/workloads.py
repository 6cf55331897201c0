"""Small seeded cases shared by the parity tests (sizes the oracle finishes
in well under a second)."""
import numpy as np

from phd_gb300.thd import eglib_link, load_species

import oracle
from phd_gb300 import ics


def _copy(state):
    return {k: np.array(v, order="F", copy=True) for k, v in state.items()}


def case(name, n=12, seed=ics.SEED, eglib=False, vis_dt=False, ng=3):
    """Returns cfg, thd, adi, dxi, finalized state (oracle-closed), info.
    eglib: EGLIB precision-1 transport (cfg.eglib = 1, linking data set on
    the oracle; the caller sets it on the GPU context).  vis_dt: the Fourier
    criteria of the time step (cfg.vis_dt = 1).  ng = 4: WENO7 (mixing
    layer only)."""
    if name == "tgv":
        cfg, thd, adi, dxi, st, info = ics.tgv(n, lib_dscalar=oracle.metrics_dscalar)
    elif name == "mix":
        nz = max(n // 2, 8, 2 * ng + 1)
        cfg, thd, adi, dxi, st, info = ics.mixing_layer(n, n, nz, Lx=n * 47e-6, Ly=n * 47e-6, Lz=nz * 47e-6,
                                                         seed=seed, lib_dscalar=oracle.metrics_dscalar, ng=ng)
    else:
        raise KeyError(name)
    if eglib:
        cfg.eglib = 1
    if vis_dt:
        cfg.vis_dt = 1
    orc = oracle.Oracle(cfg, thd, adi, *dxi)
    if eglib:
        orc.set_eglib(eglib_link(load_species("h2air9" if name == "mix" else "o2n2")))
    orc.finalize_ic(st)
    return cfg, thd, adi, dxi, st, info, orc


def perturb(state, amp, seed=7):
    """Add seeded relative noise to the interior conserved variables (for
    sensor and nonlinear-WENO coverage)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    v = state["v"]
    noise = 1.0 + amp * rng.standard_normal(v.shape[:3])
    for q in range(v.shape[3]):
        v[..., q] *= noise
    return state


def copy(state):
    return _copy(state)


def normwise(a, b, floor=1e-6):
    """max |a-b| / max |b| per trailing component.

    A component whose reference values are pure rounding noise (e.g. the
    diffusive flux of a uniform mixture) is scaled by ``floor`` times the
    largest component instead of by its own size."""
    a = np.asarray(a); b = np.asarray(b)
    num = np.abs(a - b).reshape(-1, a.shape[-1]).max(axis=0)
    den = np.abs(b).reshape(-1, b.shape[-1]).max(axis=0)
    den = np.maximum(den, floor * den.max())
    den = np.where(den == 0, 1.0, den)
    return num / den


def mixing_layer_with_streams(nx=12, ny=24, nz=8):
    """A mixing layer whose y extent (12 mm, 24 points) reaches the pure fuel
    and oxidiser streams: the chemistry window holds cells that the
    dvodesimp skip test leaves alone.  Returns cfg, thd, adi, dxi, state,
    oracle and the skip data (pure-stream mass fractions, H2 and N2
    indices)."""
    cfg, thd, adi, dxi, st, info = ics.mixing_layer(nx, ny, nz, Lx=nx * 47e-6, Ly=12e-3, Lz=nz * 47e-6,
                                                     lib_dscalar=oracle.metrics_dscalar)
    cfg.reaction = 1
    orc = oracle.Oracle(cfg, thd, adi, *dxi)
    orc.finalize_ic(st)
    names = load_species("h2air9")["names"]
    ih2, in2 = names.index("H2"), names.index("N2")
    yf = np.zeros(9); yf[ih2] = 0.5; yf[in2] = 0.5
    yo = np.zeros(9); yo[names.index("O2")] = 0.233; yo[in2] = 0.767
    return cfg, thd, adi, dxi, st, orc, (yf, yo, ih2, in2)


RTOL, ATOL = 1e-6, 1e-10   # the reference's DVODE tolerances (module_reaction.f90, ITOL = 1)


def tol_units(got, ref):
    """|got - ref| in units of the integrator's tolerance RTOL |ref| + ATOL."""
    return np.abs(np.asarray(got) - np.asarray(ref)) / (RTOL * np.abs(np.asarray(ref)) + ATOL)


def chem_error_stats(got, ref, ng=3, nrv=9):
    """Per-cell error of a chemistry-carrying state against the oracle's, in
    units of the integrator's tolerance: temperature and every species mass
    fraction (the DVODE unknowns z = [T, Y_1..Y_K], chemkin reaction_v.f),
    summarised as median, 99th percentile and max over the interior."""
    i = (slice(ng, -ng),) * 3
    rT = tol_units(got["T"][i], ref["T"][i]).ravel()
    vg, vr = got["v"][i], ref["v"][i]
    rY = np.stack([tol_units(vg[..., 5 + q] / vg[..., 0], vr[..., 5 + q] / vr[..., 0]).ravel()
                   for q in range(nrv)], axis=1).max(axis=1)
    out = {}
    for nm, r in (("T", rT), ("Y", rY)):
        out[nm] = {"median": float(np.median(r)), "p99": float(np.percentile(r, 99)), "max": float(r.max())}
    return out


def oracle_step(orc, st, mech, loop):
    """The reference driver's step (izem.f90:252-281) on the oracle, in the
    order of phd_gb300.izem.TimeLoop: timestep with the previous dtmin and
    DTmax, then chem(dt/2), rk3(dt), chem(dt/2) when mech is given.
    loop: dict with dtmin, DTmax and time, updated in place.  Returns dt."""
    _, dt = orc.timestep(st, DTmax=loop["DTmax"], dtmin=loop["dtmin"])
    if mech is not None:
        orc.chem_step(st, mech, 0.5 * dt, loop["time"])
    orc.rk3(st, dt, loop["time"])
    loop["time"] += dt
    if mech is not None:
        loop["DTmax"] = orc.chem_step(st, mech, 0.5 * dt, loop["time"])
    loop["dtmin"] = dt
    return dt


# Bounds that any last-bit perturbation of the right-hand side meets on the
# batched ignition reactors (the reciprocal form alone, on the host, reaches
# T max 97 and species p99 74).
BATCH_LIMITS = {"T_median": 1e-3, "T_p99": 10.0, "T_max": 200.0, "Y_median": 1e-2, "Y_p90": 10.0, "Y_rel": 1e-3}
# On the window reactors of the 20^3 reacting field over 1e-6 s, where
# ignition fronts cross many cells within the step, the reciprocal form
# alone reaches T median 0.0016, p99 8.8, max 209; species median 0.081,
# p90 29; species relative to their largest value 1.33e-3.  These bounds
# are twice that.
FIELD_LIMITS = {"T_median": 1e-2, "T_p99": 20.0, "T_max": 400.0, "Y_median": 0.2, "Y_p90": 60.0, "Y_rel": 3e-3}


def reactor_error_bounds(Tg, Yg, To, Yo, limits=None):
    """Errors of an integrated reactor batch against the oracle's, in the
    integrator's tolerance units per cell (T, and the largest over the
    species), plus the species error relative to each species' largest
    value.  Returns (stats dict, message, ok) for the given limits
    (BATCH_LIMITS by default): T median, p99 and max; species median and
    p90; species relative to their largest value plus ATOL (a species that
    stays below ATOL everywhere is rounding noise to the integrator)."""
    lim = BATCH_LIMITS if limits is None else limits
    rT = tol_units(Tg, To).ravel()
    rY = tol_units(Yg, Yo).reshape(len(rT), -1).max(axis=1)
    yn = float((np.abs(Yg - Yo) / (np.abs(Yo).max(axis=0) + ATOL)).max())
    st = {"T": {"median": float(np.median(rT)), "p99": float(np.percentile(rT, 99)), "max": float(rT.max())},
          "Y": {"median": float(np.median(rY)), "p90": float(np.percentile(rY, 90)), "p99": float(np.percentile(rY, 99)),
                "max": float(rY.max())},
          "Y_rel_to_max": yn}
    ok = (st["T"]["median"] < lim["T_median"] and st["T"]["p99"] <= lim["T_p99"] and st["T"]["max"] <= lim["T_max"]
          and st["Y"]["median"] < lim["Y_median"] and st["Y"]["p90"] <= lim["Y_p90"] and yn <= lim["Y_rel"])
    return st, "tol units: %s" % st, ok


# The shipped mechanism with its first fall-off reaction in the SRI form and
# its second with one species, H2O, as the collider: the CKRATX branches
# (vode.f:1185-1236) the H2/air set does not use.  The parameters exercise
# those branches; they are not fitted to any data.
SRI_PARAMS = (0.45, 797.0, 979.0, 1.2, 0.1)


def variant_mechanism(tmp_path):
    """Write the variant mechanism under tmp_path (a pathlib.Path) and read
    it with phd_gb300.mech.read_mechanism."""
    import os
    from phd_gb300.mech import read_mechanism
    from phd_gb300.thd import DATA_DIR
    with open(os.path.join(DATA_DIR, "h2_sandiego12.inp")) as f:
        text = f.read()
    text = text.replace("   TROE / 0.5  1.0E-30  1.0E30 /\n",
                        "   SRI / %s /\n" % "  ".join(repr(x) for x in SRI_PARAMS))
    text = text.replace("H2O2(+M)=>OH+OH(+M)", "H2O2(+H2O)=>OH+OH(+H2O)")
    text = text.replace("   TROE / 0.735  94.0  1756.0  5182.0 /\n   H2/2.5/ H2O/6.0/\n",
                        "   TROE / 0.735  94.0  1756.0  5182.0 /\n")
    path = tmp_path / "h2_sri_collider.inp"
    path.write_text(text)
    return read_mechanism(str(path), "h2air9")


def equilibrium_variant_mechanism(tmp_path):
    """The shipped mechanism with the explicit reverse parameters (REV) of
    its first three reactions and of H+OH+M=H2O+M removed: those reverse
    rates then come from the equilibrium constant (CKRATT's
    RKRT = RKFT / EQK, vode.f:1015-1022), the path that the shipped set,
    whose reverse rates are all explicit, does not take."""
    import os
    from phd_gb300.mech import read_mechanism
    from phd_gb300.thd import DATA_DIR
    with open(os.path.join(DATA_DIR, "h2_sandiego12.inp")) as f:
        text = f.read()
    for rev in ("   REV / 7.04E13  -0.26   0.143 /\n", "   REV / 3.03E04   2.63   4.840 /\n",
                "   REV / 1.28E10   1.19  18.700 /\n", "   REV / 1.03E23  -1.75 118.580 /\n"):
        assert rev in text
        text = text.replace(rev, "")
    path = tmp_path / "h2_equilibrium.inp"
    path.write_text(text)
    return read_mechanism(str(path), "h2air9")


# Landau-Teller parameters (B, C) put on the forward and the explicit reverse
# rate of H2+O<=>OH+H: exercise the factors, not fitted to any data.
LT_PARAMS, RLT_PARAMS = (-25.0, 10.0), (5.0, -2.0)


def landau_teller_variant_mechanism(tmp_path):
    """The shipped mechanism with Landau-Teller factors (LT, RLT; CKRATT,
    vode.f:973-981, 1032-1041) on H2+O<=>OH+H (reaction 1)."""
    import os
    from phd_gb300.mech import read_mechanism
    from phd_gb300.thd import DATA_DIR
    with open(os.path.join(DATA_DIR, "h2_sandiego12.inp")) as f:
        text = f.read()
    rev = "   REV / 3.03E04   2.63   4.840 /\n"
    assert rev in text
    text = text.replace(rev, rev + "   LT / %r %r /\n   RLT / %r %r /\n" % (LT_PARAMS + RLT_PARAMS))
    path = tmp_path / "h2_landau_teller.inp"
    path.write_text(text)
    return read_mechanism(str(path), "h2air9")


VARIANTS = {"sri_collider": variant_mechanism, "equilibrium": equilibrium_variant_mechanism,
            "landau_teller": landau_teller_variant_mechanism}

"""Seeded synthetic workloads (initial conditions, grids, switches).

The reference hard-codes every initial condition in module_ICs.f90 and has no
Taylor-Green or temporal mixing-layer case that matches the benchmark
configurations, so these generators build them.  Each returns the raw state
(interior filled, ghosts extrapolated, temperature guess everywhere) in code
units; the caller closes it with ``finalize_ic`` (module_ICs.f90:2874-2879),
on the GPU (IzemGPU.finalize_ic) or on the oracle, exactly as the reference's
init routines end.

Workloads:
* ``tgv``           Taylor-Green vortex, periodic n^3 box of side 2*pi*L0,
                    Mach 0.1, Re = 1600, calorically perfect air (gamma 1.4).
* ``mixing_layer``  temporal H2/air mixing layer, 9 species, x/z periodic,
                    y zero-gradient; tanh profile of thickness 0.5 mm,
                    dU = 100 m/s, 1% seeded white-noise velocity.
* ``jet_les``       reacting planar H2/air jet with the jet faces.
* ``batched_reactors`` independent reactors of the batched-chemistry
                    distribution; ``reacting_field`` the same distribution as
                    smooth fields on a grid, for the learned chemistry.
"""
import math

import numpy as np

from .capi import BC_EXTRAPOLATION, BC_PERIODIC, IzemCfg
from .thd import adi_struct, constants, load_species, thd_init

SEED = 20261203


def make_cfg(nx, ny, nz, nrv, bc=(BC_PERIODIC,) * 6, vis=1, weno_avg=1, max_rel_weight=0.15, forcesum=1,
             reaction=0, eglib=0, cfl=0.5, cflmin=0.1, cpr=20.0, fo=0.1, vis_dt=0, linfix=0):
    c = IzemCfg()
    c.nx, c.ny, c.nz, c.ng, c.ndim, c.nrv = nx, ny, nz, 3, 3, nrv
    for f in range(6):
        c.bc[f] = bc[f]
    c.weno_avg = weno_avg
    c.max_rel_weight = max_rel_weight
    c.vis, c.eglib, c.forcesum, c.reaction, c.vis_dt = vis, eglib, forcesum, reaction, vis_dt
    c.cfl, c.cflmin, c.cpr, c.fo = cfl, cflmin, cpr, fo
    c.weno5_linear_fix = linfix
    return c


def ha_code(thd, T):
    """Species enthalpies in code units at code temperature T (array), the
    NASA-7 evaluation of ha_scalar (module_thermodynamics.f90:873-978)."""
    T = np.asarray(T, dtype=np.float64)
    ns = thd.nspc
    out = np.empty(T.shape + (ns,))
    for k in range(ns):
        tk = T * thd.tinf
        res = np.empty_like(tk)
        for rng, mask in ((0, tk < thd.tpolylim[k]), (1, tk >= thd.tpolylim[k])):
            a = [thd.heatcap[k][rng][c] for c in range(7)]
            t = np.clip(tk, thd.tpolymin[k], thd.tpolymax[k])
            h = a[0] * t + a[1] * t ** 2 * 0.5 + a[2] * t ** 3 / 3.0 + a[3] * t ** 4 * 0.25 + a[4] * t ** 5 * 0.2 + a[5]
            cp = a[0] + a[1] * t + a[2] * t ** 2 + a[3] * t ** 3 + a[4] * t ** 4
            h = h + cp * (tk - t)
            res = np.where(mask, h, res)
        out[..., k] = thd.Wc_i[k] / thd.tinf * res
    return out


def grid_dxi(coord_m, ng, adi, lib_dscalar):
    """dx_i over (1-ng .. n+ng) in code units: dscalar on the global
    coordinates, inverted, times L_ref; ghost entries stay 1*L_ref
    (module_tools.f90:374-432, 185-187)."""
    n = len(coord_m)
    inner = lib_dscalar(np.asarray(coord_m, dtype=np.float64), ng)
    out = np.full(n + 2 * ng, 1.0)
    out[ng:ng + n] = inner
    return out * adi["l_ref"]


def _state_from_primitives(thd, a, rho_d, u_d, v_d, w_d, T_d, Y, ng):
    """Fill a ghosted state from dimensional interior primitives (interior
    arrays of shape (nx,ny,nz)), ghosts by zero-gradient extension."""
    nx, ny, nz = rho_d.shape
    nrv = thd.nspc
    cons, T = _cons_from_primitives(thd, a, rho_d, u_d, v_d, w_d, T_d, Y)
    pad = ((ng, ng), (ng, ng), (ng, ng))
    vg = np.empty((nx + 2 * ng, ny + 2 * ng, nz + 2 * ng, 5 + nrv), order="F")
    for q in range(5 + nrv):
        vg[..., q] = np.pad(cons[..., q], pad, mode="edge")
    Tg = np.asfortranarray(np.pad(T, pad, mode="edge"))
    return _state_dict(vg, Tg, nrv)


def _state_dict(vg, Tg, nrv):
    shp = vg.shape[:3]
    return {"v": vg, "T": Tg, "W_i": np.zeros(shp, order="F"), "cp": np.zeros(shp, order="F"),
            "ha": np.zeros(shp + (nrv,), order="F"), "shock_sensor": np.zeros(shp, dtype=np.uint8, order="F")}


def _cons_from_primitives(thd, a, rho_d, u_d, v_d, w_d, T_d, Y):
    """Conserved variables (..., 5 + nrv) and the code-unit temperature of
    dimensional primitives (arrays of one shape; Y with a trailing species
    axis)."""
    nrv = thd.nspc
    rho = rho_d / a["rho_ref"]
    u, v, w = u_d / a["u_ref"], v_d / a["u_ref"], w_d / a["u_ref"]
    T = T_d / a["t_ref"]
    W_i = np.zeros_like(T)
    for k in range(nrv):
        W_i += Y[..., k] * thd.Wc_i[k]
    P = rho * T * W_i
    ha = ha_code(thd, T)
    hm = np.einsum("...k,...k->...", ha, Y)
    cons = np.empty(rho.shape + (5 + nrv,))
    cons[..., 0] = rho
    cons[..., 1] = rho * u
    cons[..., 2] = rho * v
    cons[..., 3] = rho * w
    cons[..., 4] = rho * hm - P + 0.5 * rho * (u * u + v * v + w * w)
    for k in range(nrv):
        cons[..., 5 + k] = rho * Y[..., k]
    return cons, T


def tgv(n=64, lib_dscalar=None):
    """Taylor-Green vortex: periodic n^3, box 2*pi*L0, Mach 0.1, Re 1600."""
    a = constants()
    sp = load_species("air2")
    thd = thd_init(sp, a)
    W = sp["W_gmol"][0] * 1e-3
    Rm = a["r_ref"] / W
    T0, p0 = 300.0, 101325.0
    c0 = math.sqrt(1.4 * Rm * T0)
    U0 = 0.1 * c0
    rho0 = p0 / (Rm * T0)
    ce = sp["cofeta"][0]
    mu0 = math.exp(ce[0] + ce[1] * math.log(T0)) * 0.1
    L0 = 1600.0 * mu0 / (rho0 * U0)
    h = 2.0 * math.pi * L0 / n
    x = np.arange(n) * h
    X, Y_, Z = np.meshgrid(x / L0, x / L0, x / L0, indexing="ij")
    u = U0 * np.sin(X) * np.cos(Y_) * np.cos(Z)
    v = -U0 * np.cos(X) * np.sin(Y_) * np.cos(Z)
    w = np.zeros_like(u)
    p = p0 + rho0 * U0 * U0 / 16.0 * (np.cos(2 * X) + np.cos(2 * Y_)) * (np.cos(2 * Z) + 2.0)
    T = np.full_like(u, T0)
    rho = p / (Rm * T)
    Ys = np.zeros(u.shape + (2,))
    Ys[..., 0] = 0.5
    Ys[..., 1] = 0.5
    state = _state_from_primitives(thd, a, rho, u, v, w, T, Ys, 3)
    cfg = make_cfg(n, n, n, 2)
    dxi = [grid_dxi(x, 3, a, lib_dscalar) for _ in range(3)]
    info = {"L0": L0, "U0": U0, "rho0": rho0, "T0": T0, "p0": p0, "mu0": mu0,
            "t_conv": L0 / U0, "name": "TGV %d^3 Ma 0.1 Re 1600" % n}
    return cfg, thd, adi_struct(a), dxi, state, info


def mixing_layer(nx=256, ny=256, nz=128, Lx=12e-3, Ly=12e-3, Lz=6e-3, seed=SEED, lib_dscalar=None, ng=3):
    """Temporal H2/air mixing layer (9 species), x and z periodic, y
    extrapolation; ng = 3 (WENO5) or 4 (WENO7)."""
    a = constants()
    sp = load_species("h2air9")
    thd = thd_init(sp, a)
    names = sp["names"]
    ix = {nm: q for q, nm in enumerate(names)}
    delta, dU, p0 = 0.5e-3, 100.0, 101325.0
    x = np.arange(nx) * (Lx / nx)
    z = np.arange(nz) * (Lz / nz)
    y = -0.5 * Ly + np.arange(ny) * (Ly / (ny - 1))
    Xg, Yg, Zg = np.meshgrid(x, y, z, indexing="ij")
    f = 0.5 * (1.0 + np.tanh(Yg / delta))
    Yf = np.zeros(len(names)); Yf[ix["H2"]] = 0.5; Yf[ix["N2"]] = 0.5
    Yo = np.zeros(len(names)); Yo[ix["O2"]] = 0.233; Yo[ix["N2"]] = 0.767
    Ys = (1.0 - f)[..., None] * Yf + f[..., None] * Yo
    T = (1.0 - f) * 1000.0 + f * 1200.0
    rng = np.random.Generator(np.random.PCG64(seed))
    u = 0.5 * dU * np.tanh(Yg / delta) + 0.01 * dU * rng.standard_normal(Xg.shape)
    v = 0.01 * dU * rng.standard_normal(Xg.shape)
    w = 0.01 * dU * rng.standard_normal(Xg.shape)
    Wmix_i = np.einsum("...k,k->...", Ys, 1.0 / (np.array(sp["W_gmol"]) * 1e-3))
    rho = p0 / (a["r_ref"] * Wmix_i * T)
    state = _state_from_primitives(thd, a, rho, u, v, w, T, Ys, ng)
    bc = (BC_PERIODIC, BC_PERIODIC, BC_EXTRAPOLATION, BC_EXTRAPOLATION, BC_PERIODIC, BC_PERIODIC)
    cfg = make_cfg(nx, ny, nz, 9, bc=bc)
    cfg.ng = ng
    dxi = [grid_dxi(x, ng, a, lib_dscalar), grid_dxi(y, ng, a, lib_dscalar), grid_dxi(z, ng, a, lib_dscalar)]
    info = {"name": "H2/air temporal mixing layer %dx%dx%d" % (nx, ny, nz), "delta": delta, "dU": dU, "seed": seed}
    return cfg, thd, adi_struct(a), dxi, state, info


def mixing_layer_block(nx=64, ny=64, nz=32, seed=SEED, lib_dscalar=None):
    """A smaller block of the 256 x 256 x 128 mixing layer with its grid
    spacing (12 mm / 256 in x, 12 mm / 255 in y, 6 mm / 128 in z), centred
    on the layer in y, with the same faces, profiles and seeded noise law."""
    return mixing_layer(nx, ny, nz, Lx=nx * 12e-3 / 256, Ly=(ny - 1) * 12e-3 / 255, Lz=nz * 6e-3 / 128, seed=seed,
                        lib_dscalar=lib_dscalar)


def jet_les(nx=512, ny=512, nz=256, dx=47e-6, width=2e-3, u_jet=300.0, u_co=10.0, T_jet=1000.0, T_co=1200.0,
            y_fuel=0.5, turb=0.02, seed=SEED, lib_dscalar=None):
    """Reacting planar H2/air jet: a slot of `width` (2 mm) in y issuing
    H2/N2 (y_fuel H2 by mass, the rest N2) at u_jet (300 m/s) and T_jet into
    air (O2/N2 0.233/0.767) at T_co (1200 K) and u_co (10 m/s), 1 atm; the
    9-species set.  Uniform spacing dx; x from the nozzle plane, y centred
    on the slot, z periodic.  Faces: the jet inflow on W (planar profile,
    no ramp, seeded fluctuations of relative amplitude turb), the
    characteristic outflow on E, extrapolation in y, periodic in z.  The
    initial field carries the inflow profile through the domain (the tanh
    profile of the inflow in |y|) with seeded velocity fluctuations of the
    same amplitude (numpy PCG64(seed)).  Returns cfg, thd, adi, dxi, state,
    info; info["coords"], info["lx"] and info["jet"] (capi.IzemJet) set up
    the jet faces."""
    from .capi import BC_INFLOWJET, BC_NSCBC_OUT, IzemJet
    a = constants()
    sp = load_species("h2air9")
    thd = thd_init(sp, a)
    names = sp["names"]
    ih2, io2, in2 = names.index("H2"), names.index("O2"), names.index("N2")
    x = np.arange(nx) * dx
    y = (np.arange(ny) - 0.5 * (ny - 1)) * dx
    z = np.arange(nz) * dx
    ng = 3
    # profiles across the slot (they depend on y only)
    th = np.tanh((np.abs(y) - 0.5 * width) / (0.04 * width))
    Ys = np.zeros((ny, len(names)))
    Ys[:, ih2] = 0.5 * (y_fuel - y_fuel * th)
    Ys[:, io2] = 0.5 * (0.233 + 0.233 * th)
    Ys[:, in2] = 0.5 * ((1.0 - y_fuel + 0.767) - (1.0 - y_fuel - 0.767) * th)
    T_y = 0.5 * ((T_jet + T_co) - (T_jet - T_co) * th)
    u_y = 0.5 * ((u_jet + u_co) - (u_jet - u_co) * th)
    Wmix_i = np.einsum("yk,k->y", Ys, 1.0 / (np.array(sp["W_gmol"]) * 1e-3))
    rho_y = 101325.0 / (a["r_ref"] * Wmix_i * T_y)
    # code units (as _state_from_primitives converts them)
    rho_c = rho_y / a["rho_ref"]
    T_c = T_y / a["t_ref"]
    W_i = np.zeros_like(T_c)
    for k in range(len(names)):
        W_i += Ys[:, k] * thd.Wc_i[k]
    P_c = rho_c * T_c * W_i
    hm = np.einsum("yk,yk->y", ha_code(thd, T_c), Ys)
    # seeded velocity fluctuations in the jet, drawn over the interior
    rng = np.random.Generator(np.random.PCG64(seed))
    amp = (turb * u_jet * 0.5 * (1.0 - th))[None, :, None]
    shp = (nx, ny, nz)
    u = (u_y[None, :, None] + amp * rng.uniform(-1.0, 1.0, shp)) / a["u_ref"]
    v = (amp * rng.uniform(-1.0, 1.0, shp)) / a["u_ref"]
    w = (amp * rng.uniform(-1.0, 1.0, shp)) / a["u_ref"]
    # ghosted state, ghosts by zero-gradient extension of the interior
    gsh = (nx + 2 * ng, ny + 2 * ng, nz + 2 * ng)
    jy = np.clip(np.arange(ny + 2 * ng) - ng, 0, ny - 1)   # ghosted y -> interior y

    def ext(a3):
        out = np.empty(gsh, order="F")
        out[ng:ng + nx, ng:ng + ny, ng:ng + nz] = a3
        out[:ng] = out[ng:ng + 1]
        out[ng + nx:] = out[ng + nx - 1:ng + nx]
        out[:, :ng] = out[:, ng:ng + 1]
        out[:, ng + ny:] = out[:, ng + ny - 1:ng + ny]
        out[:, :, :ng] = out[:, :, ng:ng + 1]
        out[:, :, ng + nz:] = out[:, :, ng + nz - 1:ng + nz]
        return out

    vg = np.empty(gsh + (5 + len(names),), order="F")
    rho3 = rho_c[None, :, None]
    vg[..., 0] = rho_c[jy][None, :, None]
    vg[..., 1] = ext(rho3 * u)
    vg[..., 2] = ext(rho3 * v)
    vg[..., 3] = ext(rho3 * w)
    vg[..., 4] = ext(rho3 * hm[None, :, None] - P_c[None, :, None] + 0.5 * rho3 * (u * u + v * v + w * w))
    for k in range(len(names)):
        vg[..., 5 + k] = (rho_c * Ys[:, k])[jy][None, :, None]
    del u, v, w
    Tg = np.empty(gsh, order="F")
    Tg[...] = T_c[jy][None, :, None]
    state = {"v": vg, "T": Tg, "W_i": np.zeros(gsh, order="F"), "cp": np.zeros(gsh, order="F"),
             "ha": np.zeros(gsh + (len(names),), order="F"), "shock_sensor": np.zeros(gsh, dtype=np.uint8, order="F")}
    bc = (BC_INFLOWJET, BC_NSCBC_OUT, BC_EXTRAPOLATION, BC_EXTRAPOLATION, BC_PERIODIC, BC_PERIODIC)
    cfg = make_cfg(nx, ny, nz, len(names), bc=bc)
    dxi = [grid_dxi(c, 3, a, lib_dscalar) for c in (x, y, z)]
    L = a["l_ref"]
    jet = IzemJet(width=width, ramp=0.0, T_jet=T_jet, T_co=T_co, p_jet=101325.0, p_co=101325.0, u_jet=u_jet,
                  u_co=u_co, y_fuel=y_fuel, p_far=101325.0, turb=turb, planar=1, reserved=0, seed=seed)
    info = {"name": "reacting planar H2/air jet %dx%dx%d" % (nx, ny, nz), "seed": seed,
            "coords": (x / L, y / L, z / L), "lx": (x[-1] - x[0]) / L, "time_ref": a["time_ref"], "jet": jet,
            "width_m": width, "dx_m": dx}
    return cfg, thd, adi_struct(a), dxi, state, info


def batched_reactors(n, seed=SEED):
    """Independent H2/air reactors: T ~ U[800, 2400] K, p ~ U[1, 10] atm,
    equivalence ratio ~ U[0.3, 3], progress c ~ U[0, 1] blending the unburnt
    mixture linearly toward the complete-combustion major products (H2O, N2
    and the excess O2 or H2), dt log-uniform in [1e-8, 1e-6] s.  Returns
    T [K], rho [g/cm^3], Y (n, 9) in the h2air9 species order, dt [s]."""
    sp = load_species("h2air9")
    W = np.array(sp["W_gmol"])
    rng = np.random.Generator(np.random.PCG64(seed))
    T = rng.uniform(800.0, 2400.0, n)
    p = rng.uniform(1.0, 10.0, n) * 101325.0
    phi = rng.uniform(0.3, 3.0, n)
    c = rng.uniform(0.0, 1.0, n)
    dt = 10.0 ** rng.uniform(-8.0, -6.0, n)
    Y = _blend_composition(phi, c, sp["names"], W)
    Wmix = 1.0 / (Y / W).sum(axis=1)
    rho = p * Wmix * 1e-3 / (8.314510 * T) * 1e-3    # kg/m^3 -> g/cm^3
    return np.ascontiguousarray(T), np.ascontiguousarray(rho), np.ascontiguousarray(Y), np.ascontiguousarray(dt)


def _blend_composition(phi, c, names, W):
    """Mass fractions (n, 9) of H2/air at equivalence ratio phi, blended
    linearly (weight c) from the unburnt mixture toward the complete-combustion
    major products: H2O, N2 and the excess O2 (lean) or H2 (rich)."""
    ix = {nm: q for q, nm in enumerate(names)}
    n = len(phi)
    Xu = np.zeros((n, 9)); Xb = np.zeros((n, 9))
    Xu[:, ix["H2"]] = 2.0 * phi; Xu[:, ix["O2"]] = 1.0; Xu[:, ix["N2"]] = 3.76
    lean = phi <= 1.0
    Xb[:, ix["H2O"]] = np.where(lean, 2.0 * phi, 2.0)
    Xb[:, ix["O2"]] = np.where(lean, 1.0 - phi, 0.0)
    Xb[:, ix["H2"]] = np.where(lean, 0.0, 2.0 * phi - 2.0)
    Xb[:, ix["N2"]] = 3.76
    Yu = Xu * W; Yu /= Yu.sum(axis=1, keepdims=True)
    Yb = Xb * W; Yb /= Yb.sum(axis=1, keepdims=True)
    return (1.0 - c)[:, None] * Yu + c[:, None] * Yb


def smooth_uniform(shape, corr, rng):
    """A seeded 3-D field whose value at every point is distributed
    uniformly on (0, 1) and which varies smoothly over about `corr` cells:
    independent standard normals on a lattice of spacing `corr`,
    interpolated trilinearly, divided at each point by the standard
    deviation of that interpolation (the square root of the sum of the
    squared corner weights, a product over the axes of (1-t)^2 + t^2), so
    that every point is exactly N(0, 1), then mapped through the normal
    distribution function."""
    lat = rng.standard_normal(tuple(n // corr + 2 for n in shape))
    return _smooth_eval(lat, corr, shape, 0, shape[2])


def _smooth_eval(lat, corr, shape, k0, k1):
    """smooth_uniform's field on the planes k0 <= k < k1 of the last axis,
    from its lattice `lat`."""
    from scipy.special import ndtr
    out, sd2 = lat, 1.0
    for ax, idx in enumerate((np.arange(shape[0]), np.arange(shape[1]), np.arange(k0, k1))):
        s = idx / corr
        i0 = np.floor(s).astype(np.int64)
        t = s - i0
        bshape = [1, 1, 1]
        bshape[ax] = len(idx)
        t = t.reshape(bshape)
        out = (1.0 - t) * np.take(out, i0, axis=ax) + t * np.take(out, i0 + 1, axis=ax)
        sd2 = sd2 * ((1.0 - t) ** 2 + t ** 2)
    return ndtr(out / np.sqrt(sd2))


def reacting_field(nx=512, ny=256, nz=256, dt_s=3e-7, corr=16, dx=47e-6, seed=SEED, lib_dscalar=None,
                   threads=None):
    """A reacting H2/air field at rest for the learned-chemistry workload:
    at every point T, p, the equivalence ratio and the progress variable
    follow the batched-reactor distribution (T ~ U[800, 2400] K,
    p ~ U[1, 10] atm, phi ~ U[0.3, 3], c ~ U[0, 1], the composition blended as
    in batched_reactors), but each of the four is a smooth seeded field
    (smooth_uniform, correlation length `corr` cells), so neighbouring cells
    hold neighbouring reactors.  Every face periodic, uniform spacing dx;
    the chemistry step is dt_s seconds (info["dt_s"]; the code-unit step is
    dt_s / info["time_ref"]), by default 3e-7 s, inside the batched
    distribution's [1e-8, 1e-6] s: over it a few per cent of the cells heat
    by more than 1 K and the hottest by some 200 K.  The interior is built in z slabs on
    `threads` host threads (numpy releases the interpreter lock in its
    array operations); ghosts by zero-gradient extension.  Returns cfg, thd,
    adi, dxi, state, info."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    a = constants()
    sp = load_species("h2air9")
    thd = thd_init(sp, a)
    W = np.array(sp["W_gmol"])
    nrv, ng = 9, 3
    rng = np.random.Generator(np.random.PCG64(seed))
    shp = (nx, ny, nz)
    lats = [rng.standard_normal(tuple(n // corr + 2 for n in shp)) for _ in range(4)]
    gsh = (nx + 2 * ng, ny + 2 * ng, nz + 2 * ng)
    vg = np.empty(gsh + (5 + nrv,), order="F")
    Tg = np.empty(gsh, order="F")

    def fill(k0):
        k1 = min(nz, k0 + 4)
        sub = (k1 - k0,)
        T = 800.0 + 1600.0 * _smooth_eval(lats[0], corr, shp, k0, k1)
        p = (1.0 + 9.0 * _smooth_eval(lats[1], corr, shp, k0, k1)) * 101325.0
        phi = 0.3 + 2.7 * _smooth_eval(lats[2], corr, shp, k0, k1)
        c = _smooth_eval(lats[3], corr, shp, k0, k1)
        Y = _blend_composition(phi.ravel(), c.ravel(), sp["names"], W).reshape(T.shape + (nrv,))
        Wmix_i = np.einsum("...k,k->...", Y, 1.0 / (W * 1e-3))
        rho = p / (a["r_ref"] * Wmix_i * T)
        zero = np.zeros(T.shape)
        cons, Tc = _cons_from_primitives(thd, a, rho, zero, zero, zero, T, Y)
        zs = slice(ng + k0, ng + k1)
        for q in range(5 + nrv):
            vg[ng:ng + nx, ng:ng + ny, zs, q] = cons[..., q]
        Tg[ng:ng + nx, ng:ng + ny, zs] = Tc
        return sub

    with ThreadPoolExecutor(threads or os.cpu_count() or 1) as ex:
        list(ex.map(fill, range(0, nz, 4)))
    for arr in [vg[..., q] for q in range(5 + nrv)] + [Tg]:
        arr[:ng] = arr[ng:ng + 1]
        arr[ng + nx:] = arr[ng + nx - 1:ng + nx]
        arr[:, :ng] = arr[:, ng:ng + 1]
        arr[:, ng + ny:] = arr[:, ng + ny - 1:ng + ny]
        arr[:, :, :ng] = arr[:, :, ng:ng + 1]
        arr[:, :, ng + nz:] = arr[:, :, ng + nz - 1:ng + nz]
    state = _state_dict(vg, Tg, nrv)
    cfg = make_cfg(nx, ny, nz, nrv)
    cfg.reaction = 1
    dxi = [grid_dxi(np.arange(n) * dx, ng, a, lib_dscalar) for n in shp]
    info = {"name": "reacting H2/air field %dx%dx%d at rest (batched-reactor distribution as smooth fields, "
                    "correlation length %d cells)" % (nx, ny, nz, corr),
            "seed": seed, "dt_s": dt_s, "time_ref": a["time_ref"], "corr": corr, "dx_m": dx}
    return cfg, thd, adi_struct(a), dxi, state, info


def jet(nx=24, ny=16, nz=16, species="o2n2", Lx=4e-3, Lr=1.5e-3, uco=20.0, lib_dscalar=None):
    """Box for the reference's jet boundaries: bc_inflowjet on the W face
    (the 1 mm nozzle centred on y = z = 0), bc_nscbc_out on the E face,
    y and z extrapolation; initially air (O2/N2 mass fractions 0.233/0.767,
    the other species 0) at 300 K and 1 atm, moving at uco in x.  Returns cfg, thd, adi, dxi, state, info; info["coords"]
    holds the interior coordinates in code units and info["lx"] the domain
    length Lx = (x_last - x_first) / L_ref (module_tools.f90:319,489)."""
    from .capi import BC_INFLOWJET, BC_NSCBC_OUT
    a = constants()
    sp = load_species(species)
    thd = thd_init(sp, a)
    names = sp["names"]
    x = np.arange(nx) * (Lx / (nx - 1))
    y = -Lr + np.arange(ny) * (2 * Lr / (ny - 1))
    z = -Lr + np.arange(nz) * (2 * Lr / (nz - 1))
    Xg, Yg, Zg = np.meshgrid(x, y, z, indexing="ij")
    Ya = np.zeros(len(names))
    Ya[names.index("O2")] = 0.233
    Ya[names.index("N2")] = 0.767
    Ys = np.broadcast_to(Ya, Xg.shape + (len(names),)).copy()
    T = np.full(Xg.shape, 300.0)
    Wmix_i = np.einsum("...k,k->...", Ys, 1.0 / (np.array(sp["W_gmol"]) * 1e-3))
    rho = 101325.0 / (a["r_ref"] * Wmix_i * T)
    u = np.full(Xg.shape, uco)
    zero = np.zeros(Xg.shape)
    state = _state_from_primitives(thd, a, rho, u, zero, zero, T, Ys, 3)
    bc = (BC_INFLOWJET, BC_NSCBC_OUT, BC_EXTRAPOLATION, BC_EXTRAPOLATION, BC_EXTRAPOLATION, BC_EXTRAPOLATION)
    cfg = make_cfg(nx, ny, nz, len(names), bc=bc)
    dxi = [grid_dxi(c, 3, a, lib_dscalar) for c in (x, y, z)]
    L = a["l_ref"]
    info = {"name": "jet box %dx%dx%d (%s)" % (nx, ny, nz, species),
            "coords": (x / L, y / L, z / L), "lx": (x[-1] - x[0]) / L, "time_ref": a["time_ref"]}
    return cfg, thd, adi_struct(a), dxi, state, info


def acoustic_pulse(nx=16, ny=12, nz=8, species="o2n2", L=1e-3, amp=0.05, u0=30.0, w0=10.0, blob=0.0, faces="xy",
                   ng=3, lib_dscalar=None):
    """Box with non-reflecting faces (NOREFLECTION: bc_noreflection and
    bc_noreflectionweno) for the waves that leave it: air (O2/N2 mass
    fractions 0.233/0.767) at 300 K and 1 atm moving at u0 in x and w0 in z, with a
    Gaussian pressure pulse of relative amplitude amp and width L/6 at the
    centre of the x-y section (isothermal: the density follows the
    pressure).  blob > 0 (nine-species sets) adds an H2 mass fraction
    blob * exp(-r^2/s^2) at the same place, taken from N2.  faces: the
    axes whose two faces are non-reflecting ("x", "xy" or "xyz"); the
    others are periodic.  Grid spacing L/(n-1) on every axis; ng = 3
    (WENO5) or 4 (WENO7, two-species sets).  Returns cfg, thd, adi, dxi,
    state, info."""
    from .capi import BC_NOREFLECTION
    a = constants()
    sp = load_species(species)
    thd = thd_init(sp, a)
    names = sp["names"]
    h = L / (nx - 1)
    x = np.arange(nx) * h
    y = np.arange(ny) * h
    z = np.arange(nz) * h
    Xg, Yg, Zg = np.meshgrid(x, y, z, indexing="ij")
    r2 = (Xg - x[-1] / 2) ** 2 + (Yg - y[-1] / 2) ** 2
    s2 = (L / 6.0) ** 2
    g = np.exp(-r2 / s2)
    Ya = np.zeros(len(names))
    Ya[names.index("O2")] = 0.233
    Ya[names.index("N2")] = 0.767
    Ys = np.broadcast_to(Ya, Xg.shape + (len(names),)).copy()
    if blob > 0.0:
        Ys[..., names.index("H2")] = blob * g
        Ys[..., names.index("N2")] -= blob * g
    T = np.full(Xg.shape, 300.0)
    Wmix_i = np.einsum("...k,k->...", Ys, 1.0 / (np.array(sp["W_gmol"]) * 1e-3))
    P = 101325.0 * (1.0 + amp * g)
    rho = P / (a["r_ref"] * Wmix_i * T)
    u = np.full(Xg.shape, u0)
    w = np.full(Xg.shape, w0)
    zero = np.zeros(Xg.shape)
    state = _state_from_primitives(thd, a, rho, u, zero, w, T, Ys, ng)
    bc = [BC_PERIODIC] * 6
    for d, ax in enumerate("xyz"):
        if ax in faces:
            bc[2 * d] = bc[2 * d + 1] = BC_NOREFLECTION
    cfg = make_cfg(nx, ny, nz, len(names), bc=tuple(bc))
    cfg.ng = ng
    dxi = [grid_dxi(c, ng, a, lib_dscalar) for c in (x, y, z)]
    info = {"name": "acoustic pulse %dx%dx%d (%s, non-reflecting %s faces)" % (nx, ny, nz, species, faces),
            "time_ref": a["time_ref"]}
    return cfg, thd, adi_struct(a), dxi, state, info


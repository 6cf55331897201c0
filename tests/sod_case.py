"""The reference's own Sod run, restated for the oracle (test infrastructure).

testcases/sod of the reference is a 2-D (DIM = 2) shock tube of O2/N2 air on
the 400 x 11 x 1 grid of its grid.dat, WENO7 (ORDER_WENO = 7, ng = 4) with
nonlinear weights where the Adams-Shariff sensor fires (PERCENT_WEIGHT
0.15), fitted viscous fluxes (VIS = T, EGLIB = F), no chemistry, CFL 0.5,
x extrapolation and y/z periodic boundaries, run on two x-blocks
(NUMPROCX = 2) from the SOD initial condition, with statistics and restart
files every DTIME = 7.0968962141250196e-6 s from TIME_OFFSET =
7.0968962141250196e-5 s (testcases/sod/output.cfg, sod.inp).

`sod_case` builds that configuration and the initial state of ini_sod
(module_ICs.f90:2715-2881); `run_to_stats` advances it with the main loop of
izem.f90:240-330 (timestep, the last step clipped onto the next statistics
time, rk3) and returns the state at each statistics time.
"""
import os

import numpy as np

import oracle
from phd_gb300.capi import BC_EXTRAPOLATION, BC_PERIODIC
from phd_gb300.ics import make_cfg
from phd_gb300.thd import adi_struct, constants, load_species, thd_init

HERE = os.path.dirname(os.path.abspath(__file__))
NG = 4
TIME_OFFSET_S = 7.0968962141250196e-05
DTIME_S = 7.0968962141250196e-06
NX_BLOCKS = 2


def golden(n):
    return np.load(os.path.join(HERE, "golden", "sod_restart_%05d.npz" % n))


def golden_plot(n, weno5=False):
    """Temperature [K], pressure [Pa], density [kg/m^3] and x velocity [m/s]
    of the reference's plot file n (FP32), shape (ntx, nty); weno5: of the
    run repeated with ORDER_WENO = 5 (testcases/sod/weno5_400)."""
    name = "sod_weno5_plot_%05d.npz" if weno5 else "sod_plot_%05d.npz"
    return np.load(os.path.join(HERE, "golden", name % n))


def sod_case(xblocks=NX_BLOCKS, ng=NG):
    """Configuration, species data, references, oracle, the ghosted initial
    state (closed by finalize_ic) and the metrics (dx_i, dy_i, dz_i) of the
    reference's Sod run.  xblocks: the MPI x-blocks of the reference's run,
    whose effects on the shock sensor and on the Newton stopping test the
    oracle emulates (1 for a single block).  ng = 3: the same run with
    ORDER_WENO = 5 (testcases/sod/weno5_400)."""
    NG = ng
    a = constants()
    sp = load_species("o2n2")
    thd = thd_init(sp, a)
    g = np.load(os.path.join(HERE, "golden", "sod_grid.npz"))
    xm, ym = g["x"], g["y"]
    nx, ny, nz, nrv = len(xm), len(ym), 1, 2
    bc = (BC_EXTRAPOLATION, BC_EXTRAPOLATION, BC_PERIODIC, BC_PERIODIC, BC_PERIODIC, BC_PERIODIC)
    cfg = make_cfg(nx, ny, nz, nrv, bc=bc, vis=1, weno_avg=1, max_rel_weight=0.15, forcesum=1, reaction=0, cfl=0.5)
    cfg.ng, cfg.ndim = NG, 2
    L = a["l_ref"]

    def dxi(coord):
        # metrics (module_tools.f90:374-432): dscalar on the global
        # coordinates in metres, inverted; ghost entries 1; times L_ref
        out = np.full(len(coord) + 2 * NG, 1.0)
        out[NG:NG + len(coord)] = oracle.metrics_dscalar(coord, NG)
        return out * L
    dz = np.full(nz + 2 * NG, 1.0) * L      # no z metric in 2-D: dz_i = 1 * L_ref
    grid = (dxi(xm), dxi(ym), dz)
    orc = oracle.Oracle(cfg, thd, adi_struct(a), *grid)
    orc.set_sensor_xblocks(xblocks)
    orc.set_newton_xblocks(xblocks)

    # ini_sod: mole fractions 0.233 / 0.767 turned into mass fractions by
    # X_to_Y (module_thermodynamics.f90:45-68); (P, rho) = (1, 1) left of
    # x = 0.5 m and (0.1, 0.125) right of it, code units
    Wc, Wc_i = np.array(thd.Wc[:nrv]), np.array(thd.Wc_i[:nrv])
    Xa = [0.233, 0.767]
    wrk = 0.0
    for l in range(nrv):
        wrk = wrk + Xa[l] * Wc[l]
    wrk = 1.0 / wrk
    Ya = [Xa[l] * Wc[l] * wrk for l in range(nrv)]
    Ws_i = 0.0
    for l in range(nrv):
        Ws_i = Ws_i + Ya[l] * Wc_i[l]
    shp = (nx + 2 * NG, ny + 2 * NG, nz + 2 * NG)
    v = np.zeros(shp + (5 + nrv,), order="F")
    T = np.zeros(shp, order="F")
    states = {}
    for side, (P, rho) in (("left", (1.0, 1.0)), ("right", (0.1, 0.125))):
        Temp = P / (rho * Ws_i)
        has = orc.ha_scalar(Temp)
        hm = 0.0
        for l in range(nrv):
            hm = hm + has[l] * Ya[l]
        if side == "right":
            rho = P / (Temp * Ws_i)
        states[side] = (Temp, rho, rho * hm - P + 0.5 * rho * 0.0)
    x_code = xm * (1.0 / L)
    for i in range(nx):
        Temp, rho, rhoE = states["left" if x_code[i] * L < 0.5 else "right"]
        I = NG + i
        T[I, NG:NG + ny, NG:NG + nz] = Temp
        v[I, NG:NG + ny, NG:NG + nz, 0] = rho
        v[I, NG:NG + ny, NG:NG + nz, 4] = rhoE
        for l in range(nrv):
            v[I, NG:NG + ny, NG:NG + nz, 5 + l] = rho * Ya[l]
    # temperature guess in the ghosts (the reference starts them at 0; the
    # error-to-machine-precision Newton of the closure converges either way)
    T = np.asfortranarray(np.pad(T[NG:-NG, NG:-NG, NG:-NG], NG, mode="edge"))
    st = {"v": v, "T": T, "W_i": np.zeros(shp, order="F"), "cp": np.zeros(shp, order="F"),
          "ha": np.zeros(shp + (nrv,), order="F"), "shock_sensor": np.zeros(shp, dtype=np.uint8, order="F")}
    orc.finalize_ic(st)
    return cfg, thd, a, orc, st, grid


def stat_times(a, n):
    """inp%timing(1:n) of a run without restart read (module_input.f90:724-727),
    in code units (adimensionalize, module_tools.f90:176)."""
    t = [TIME_OFFSET_S]
    for _ in range(n - 1):
        t.append(t[-1] + DTIME_S)
    return [x / a["time_ref"] for x in t]


def run_to_stats(orc, st, a, nstats, extra=False):
    """The main loop of izem.f90:240-330 without chemistry: timestep, the
    step that would pass the next statistics time clipped onto it, rk3.
    Returns [(time, steps, copy of v)] at each of the first nstats
    statistics times; with extra, copies of T and W_i follow v."""
    timing = stat_times(a, nstats)
    time, nb, ite, out = 0.0, 0, 0, []
    while nb < nstats:
        ite += 1
        _, dtmin = orc.timestep(st)
        write = False
        if time + dtmin > timing[nb] and time - dtmin < timing[nb]:
            dtmin = timing[nb] - time
            write = True
        orc.rk3(st, dtmin)
        time = time + dtmin
        if write:
            nb += 1
            keep = (st["v"].copy(), st["T"].copy(), st["W_i"].copy()) if extra else (st["v"].copy(),)
            out.append((time, ite) + keep)
    return out

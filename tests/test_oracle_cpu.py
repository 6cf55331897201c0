"""CPU checks of the oracle and of the host-side data chain (no GPU)."""
import json
import os

import numpy as np
import pytest

import oracle
import workloads as W
from phd_gb300 import thd as T
from phd_gb300.capi import IzemCfg, IzemThd, IzemAdi

import refdata


@refdata.needs_reference
@pytest.mark.parametrize("setname,tranfit", [("h2air9", "shockedshearlayer/tranfit.out"), ("o2n2", "sod/tranfit.out")])
def test_shipped_species_match_reference_files(setname, tranfit):
    tf = T.read_tranfit(refdata.path(tranfit))
    th = T.read_therm(refdata.path("sod", "therm.dat"), tf["names"])
    sp = T.load_species(setname)
    assert sp["names"] == tf["names"]
    assert sp["cofd"] == tf["cofd"] and sp["coflam"] == tf["coflam"] and sp["cofeta"] == tf["cofeta"]
    assert sp["therm"] == json.loads(json.dumps(th))


def test_constants_reference_values():
    a = T.constants()
    assert a["w_ref"] == 8.31451 / 287.15
    assert abs(a["mu_ref"] - 1.458e-6 * 169.44 ** 1.5 / (169.44 + 110.4)) == 0.0
    assert a["sqgmr"] == np.sqrt(1.4) * 2.25 / 65000.0


def test_thermo_continuity_and_cp():
    sp = T.load_species("h2air9")
    thd = T.thd_init(sp)
    cfg, _, adi, dxi, st, info, orc = W.case("mix", 12)
    # cp_scalar agrees with d(ha)/dT numerically, and h is continuous at T_lim
    Y = np.full(9, 1.0 / 9)
    # inside every species' [Tpolymin, Tpolymax]; outside, the reference
    # extrapolates h with constant cp but cp with its slope (not consistent)
    for Tk in (500.0, 999.9, 1000.1, 2500.0, 3400.0):
        Tc = Tk / thd.tinf
        h1 = orc.ha_scalar(Tc * (1 + 1e-6))
        h0 = orc.ha_scalar(Tc * (1 - 1e-6))
        dh = (h1 - h0) / (2e-6 * Tc)
        cp = orc.cp_scalar(Tc, Y)
        # cp_scalar carries gam2: cp = gam2 * sum Y dh/dT
        assert abs(cp - thd.gam2 * np.dot(Y, dh)) < 1e-6 * abs(cp)
    for k in range(9):
        tl = thd.tpolylim[k] / thd.tinf
        a = orc.ha_scalar(tl * (1 - 1e-13))[k]
        b = orc.ha_scalar(tl * (1 + 1e-13))[k]
        assert abs(a - b) < 1e-5 * abs(a) + 1e-6


@pytest.mark.parametrize("name", ["tgv", "mix"])
def test_free_stream_and_conservation(name):
    cfg, thd, adi, dxi, st, info, orc = W.case(name, 12)
    nv = 5 + cfg.nrv
    fl = np.zeros((cfg.nx, cfg.ny, cfg.nz, nv), order="F")
    if name == "tgv":
        # initial conditions extrapolate even periodic ghosts (upd_extrapolation,
        # module_BCs.f90:161-179); the first halo exchange restores periodicity
        orc.update_primitives(st)
        # periodic: sum of (fhat_i - fhat_{i-1}) telescopes to zero
        for d in range(3):
            fl[...] = 0
            orc.euler_flux(st, d, fl)
            dxi_d = dxi[d][3:-3]
            shape = [1, 1, 1]
            shape[d] = -1
            tel = (fl / dxi_d.reshape(shape + [1])).sum(axis=(0, 1, 2))
            assert np.all(np.abs(tel) <= 1e-12 * np.abs(fl / dxi_d.reshape(shape + [1])).sum(axis=(0, 1, 2)).max())


def test_uniform_state_has_zero_flux():
    cfg, thd, adi, dxi, st, info, orc = W.case("tgv", 12)
    v = st["v"]
    for q in range(v.shape[3]):
        v[..., q] = v[3, 3, 3, q]
    st["T"][...] = st["T"][3, 3, 3]
    orc.update_primitives(st)
    fl = np.zeros((cfg.nx, cfg.ny, cfg.nz, 7), order="F")
    for d in range(3):
        orc.euler_flux(st, d, fl)
    orc.visc_flux(st, fl)
    assert np.max(np.abs(fl)) < 1e-13


def test_rk3_sumY_and_positivity():
    cfg, thd, adi, dxi, st, info, orc = W.case("mix", 12)
    dt4, dt = orc.timestep(st)
    orc.rk3(st, dt)
    v = st["v"][3:-3, 3:-3, 3:-3]
    ysum = v[..., 5:].sum(axis=-1) / v[..., 0]
    assert np.max(np.abs(ysum - 1.0)) <= 1e-13
    assert np.all(v[..., 5:] >= 0)


def test_metrics_uniform_grid():
    x = np.arange(64) * 0.1
    d = oracle.metrics_dscalar(x)
    assert np.allclose(d, 10.0, rtol=1e-12)


def _fourier_restated(cfg, thd, adi, dxi, st):
    """The Fourier criteria of timestep (module_solver.f90:294-367) restated
    in numpy from the reference's array formulas: molefrac, the D_k and
    lambda of prim_vis_vars_wo_mu (module_thermodynamics.f90:1243-1420),
    filter_width (module_tools.f90:2328-2378) and the (l, k, j, i) scan for
    the species of the largest D_k."""
    ng, nrv = cfg.ng, cfg.nrv
    sl = (slice(ng, ng + cfg.nx), slice(ng, ng + cfg.ny), slice(ng, ng + cfg.nz))
    v, T, Wi, cp = st["v"][sl], st["T"][sl], st["W_i"][sl], st["cp"][sl]
    rho = v[..., 0]
    Wc = np.array(thd.Wc[:nrv])
    X = np.stack([v[..., 5 + l] / (rho * Wi * Wc[l]) for l in range(nrv)])
    lt = np.log(T * thd.tinf)
    lts = [np.ones_like(lt), lt, lt * lt, lt * lt * lt]
    cofd, coflam = np.array(thd.cofd), np.array(thd.coflam)
    P = rho * T * Wi
    dm = np.empty_like(X)
    for m in range(nrv):
        w1 = np.zeros_like(lt)
        ds = np.zeros_like(lt)
        for l in range(nrv):
            if l != m:
                dkj = sum(cofd[m][l][n] * lts[n] for n in range(4))
                w1 = w1 + (X[l] + 1e-12) * Wc[l] * Wi
                ds = ds + (X[l] + 1e-12) * (1.0 / np.exp(dkj))
        Kd = 1.0e-4 * thd.p0 / (thd.pinf * thd.dinf[m])
        dm[m] = w1 * Kd / (ds * P)
    ct = np.zeros_like(lt)
    w1 = np.zeros_like(lt)
    for l in range(nrv):
        c1 = np.exp(sum(coflam[l][n] * lts[n] for n in range(4)))
        ct = ct + X[l] / c1
        w1 = w1 + X[l] * c1
    ct = 0.5 * 1.0e-5 / thd.laminf * (1.0 / ct + w1)
    dx, dy, dz = (d[ng:-ng] for d in dxi)
    delta = 1.0 / np.cbrt(dx[:, None, None] * dy[None, :, None] * dz[None, None, :])
    d2 = delta * delta
    ldmax = int(np.argmax([dm[l].max() for l in range(nrv)]))   # first species reaching the maximum
    dt2 = adi.sc / adi.sqgmr * cfg.fo * np.min(d2 / dm[ldmax])
    dt3 = adi.pr / adi.sqgmr * cfg.fo * np.min(d2 * rho / (ct / cp))
    return ldmax, dt2, dt3


@pytest.mark.parametrize("name", ["mix", "tgv"])
def test_fourier_timestep_matches_restatement(name):
    """With VIS_DT the oracle's dt_4(2) and dt_4(3) equal the numpy
    restatement up to the rounding of exp and of the cube root; without it
    they stay 1, and dt_4(1) is the same either way."""
    cfg, thd, adi, dxi, st, info, orc = W.case(name, 12, vis_dt=True)
    dt4, dtmin = orc.timestep(st)
    _, dt2, dt3 = _fourier_restated(cfg, thd, adi, dxi, st)
    assert abs(dt4[1] - dt2) <= 1e-13 * dt2 and abs(dt4[2] - dt3) <= 1e-13 * dt3, (dt4, dt2, dt3)
    assert dtmin == min(dt4)
    cfg0, _, _, _, st0, _, orc0 = W.case(name, 12)
    dt40, _ = orc0.timestep(st0)
    assert dt40[0] == dt4[0] and dt40[1] == 1.0 and dt40[2] == 1.0


def test_fourier_timestep_binds_on_a_fine_grid():
    """On cells 20 times finer the diffusive limits (~dx^2) fall below the
    convective one (~dx), so dtmin is a Fourier criterion."""
    from phd_gb300 import ics
    cfg, thd, adi, dxi, st, info = ics.mixing_layer(12, 12, 8, Lx=12 * 2.35e-6, Ly=12 * 2.35e-6, Lz=8 * 2.35e-6,
                                                    lib_dscalar=oracle.metrics_dscalar)
    cfg.vis_dt = 1
    orc = oracle.Oracle(cfg, thd, adi, *dxi)
    orc.finalize_ic(st)
    dt4, dtmin = orc.timestep(st)
    _, dt2, dt3 = _fourier_restated(cfg, thd, adi, dxi, st)
    assert min(dt4[1], dt4[2]) < dt4[0] and dtmin == min(dt4[1], dt4[2])
    assert abs(dt4[1] - dt2) <= 1e-13 * dt2 and abs(dt4[2] - dt3) <= 1e-13 * dt3

"""The jet faces of the oracle (module_BCs.f90): bc_inflowjet on the W face
and bc_nscbc_out on the E face, closed by upd_prim_var_dirichlet, in the
stage update of rk3 (upd_boundaries with the stage time)."""
import numpy as np
import pytest

import oracle
from phd_gb300 import ics


def _jet(species="o2n2"):
    cfg, thd, adi, dxi, st, info = ics.jet(species=species, lib_dscalar=oracle.metrics_dscalar)
    orc = oracle.Oracle(cfg, thd, adi, *dxi)
    orc.finalize_ic(st)
    orc.set_coords(*info["coords"], info["lx"])
    return cfg, thd, adi, orc, st, info


@pytest.mark.parametrize("species", ["o2n2", "h2air9"])
def test_inflow_ghosts_hold_the_nozzle_profile(species):
    """After a step that ends past the 0.1 ms ramp, the W ghost points and
    the first plane hold bc_inflowjet's profile, restated here in numpy:
    tanh profiles of u, T and p in the radius, the exit at Mach 1.01 of the
    nozzle state, rho = p / (T W_i), rho E = rho h - p + rho u^2 / 2."""
    cfg, thd, adi, orc, st, info = _jet(species)
    t0 = 2e-4 / info["time_ref"]
    _, dt = orc.timestep(st)
    orc.rk3(st, 0.01 * dt, t0)     # a short step: the jet enters a field still at rest
    ng, nrv = cfg.ng, cfg.nrv
    y, z = info["coords"][1], info["coords"][2]
    hb = 0.0010 / adi.l_ref
    delt, y0 = 1.0 / (0.04 * hb), hb / 2.0
    T1, T2 = 1000.0 / adi.t_ref, 300.0 / adi.t_ref
    P1, P2 = 101325.0 * 15.0 / adi.p_ref, 101325.0 / adi.p_ref
    Wc_i = np.array(thd.Wc_i[:nrv])
    Ya = np.zeros(nrv)
    if nrv == 2:
        Ya[:] = (0.233, 0.767)
    else:
        Ya[1], Ya[8] = 1.0, 0.0
    Ws = Ya @ Wc_i
    cps = orc.cp_scalar(T1, Ya)
    gam = 1.0 / (1.0 - thd.gam2 * Ws / cps)
    u1, u2 = 1.01 * np.sqrt(gam * Ws * T1), 20.0 / adi.u_ref
    for j in (0, len(y) // 2, len(y) - 1):
        for k in (0, len(z) // 2):
            th = np.tanh((np.sqrt(y[j] ** 2 + z[k] ** 2) - y0) * delt)
            ux = 0.5 * ((u1 + u2) - (u1 - u2) * th)
            T = 0.5 * ((T1 + T2) - (T1 - T2) * th)
            P = 0.5 * ((P1 + P2) - (P1 - P2) * th)
            Y = np.zeros(nrv)
            if nrv == 2:
                Y[:] = (0.233, 0.767)
            else:
                Y[1] = 0.5 * (1.0 - th)
                Y[3] = 0.5 * (0.233 + 0.233 * th)
                Y[8] = 0.5 * ((0.767) - (-0.767) * th)
            rho = P / (T * (Y @ Wc_i))
            rhoE = rho * (orc.ha_scalar(T) @ Y) - P + 0.5 * rho * ux * ux
            for i in range(ng + 1):      # the ghost points and the first interior plane
                got = st["v"][i, ng + j, ng + k]
                want = np.concatenate([[rho, rho * ux, 0.0, 0.0, rhoE], rho * Y])
                assert np.allclose(got, want, rtol=1e-12, atol=1e-14 * rho), (i, j, k, got - want)


def test_nscbc_outflow_writes_one_state_and_steps_stay_finite():
    """bc_nscbc_out writes one advanced state at the last plane and every E
    ghost point; three steps of the jet box, the nozzle ramping in from
    t = 0, stay finite and positive."""
    cfg, thd, adi, orc, st, info = _jet()
    t0 = 0.0
    for _ in range(3):
        _, dt = orc.timestep(st)
        orc.rk3(st, dt, t0)
        t0 = t0 + dt
    ng, nx = cfg.ng, cfg.nx
    e = st["v"][ng + nx - 1:ng + nx + ng, ng:-ng, ng:-ng]
    assert np.array_equal(e, np.broadcast_to(e[:1], e.shape))
    assert np.isfinite(st["v"]).all() and (st["T"][ng:-ng, ng:-ng, ng:-ng] > 0).all()


def test_jet_faces_reject_chemistry_and_need_coordinates():
    cfg, thd, adi, dxi, st, info = ics.jet(lib_dscalar=oracle.metrics_dscalar)
    orc = oracle.Oracle(cfg, thd, adi, *dxi)
    orc.finalize_ic(st)
    with pytest.raises(oracle.OracleError):
        orc.rk3(st, 0.1, 0.0)

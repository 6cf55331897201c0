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


def test_jet_faces_need_coordinates():
    """rk3 and the chemistry step refuse a block with jet faces until the
    coordinates are set."""
    from phd_gb300.mech import h2_mechanism
    cfg, thd, adi, dxi, st, info = ics.jet(species="h2air9", lib_dscalar=oracle.metrics_dscalar)
    orc = oracle.Oracle(cfg, thd, adi, *dxi)
    orc.finalize_ic(st)
    with pytest.raises(oracle.OracleError):
        orc.rk3(st, 0.1, 0.0)
    with pytest.raises(oracle.OracleError):
        orc.chem_step(st, h2_mechanism(), 0.1, 0.0)


def test_planar_jet_inflow_with_the_workload_parameters():
    """With the reacting-jet workload's parameters (planar 2 mm slot, H2/N2
    0.5/0.5 at 300 m/s and 1000 K into air at 1200 K and 10 m/s, 1 atm, no
    ramp) and no fluctuations, the W ghosts hold the tanh profiles in |y|,
    restated here; with 2 % fluctuations the velocities move by at most 2 %
    of the jet velocity times the core weight, and two runs draw the same
    values."""
    from phd_gb300 import capi
    cfg, thd, adi, dxi, st0, info = ics.jet_les(12, 64, 8, lib_dscalar=oracle.metrics_dscalar)
    ng, nrv = cfg.ng, cfg.nrv
    y = info["coords"][1]
    jet = info["jet"]
    runs = []
    for turb in (0.0, 0.02, 0.02):
        orc = oracle.Oracle(cfg, thd, adi, *dxi)
        orc.set_coords(*info["coords"], info["lx"])
        j = capi.IzemJet(**{f: getattr(jet, f) for f, _ in capi.IzemJet._fields_})
        j.turb = turb
        orc.set_jet(j)
        st = {k: v.copy(order="F") for k, v in st0.items()}
        orc.finalize_ic(st)
        _, dt = orc.timestep(st)
        orc.rk3(st, 0.01 * dt, 0.0)
        runs.append(st["v"][:ng + 1, ng:-ng, ng:-ng].copy())
    hb = 2e-3 / adi.l_ref
    delt, y0 = 1.0 / (0.04 * hb), hb / 2.0
    T1, T2 = 1000.0 / adi.t_ref, 1200.0 / adi.t_ref
    P = 101325.0 / adi.p_ref
    u1, u2 = 300.0 / adi.u_ref, 10.0 / adi.u_ref
    Wc_i = np.array(thd.Wc_i[:nrv])
    for jj in (0, 20, 32, 63):
        th = np.tanh((abs(y[jj]) - y0) * delt)
        ux = 0.5 * ((u1 + u2) - (u1 - u2) * th)
        T = 0.5 * ((T1 + T2) - (T1 - T2) * th)
        Y = np.zeros(nrv)
        Y[1] = 0.5 * (0.5 - 0.5 * th)
        Y[3] = 0.5 * (0.233 + 0.233 * th)
        Y[8] = 0.5 * ((0.5 + 0.767) - (0.5 - 0.767) * th)
        rho = P / (T * (Y @ Wc_i))
        want = np.concatenate([[rho, rho * ux, 0.0, 0.0], rho * Y])
        got = runs[0][:, jj, :][..., [0, 1, 2, 3] + list(range(5, 5 + nrv))]
        assert np.allclose(got, np.broadcast_to(want, got.shape), rtol=1e-12, atol=1e-14 * rho), (jj, got[0, 0] - want)
        amp = 0.02 * u1 * 0.5 * (1.0 - th)
        for c in (1, 2, 3):
            d = runs[1][:, jj, :, c] / runs[1][:, jj, :, 0] - runs[0][:, jj, :, c] / runs[0][:, jj, :, 0]
            assert np.all(np.abs(d) <= amp * (1 + 1e-9) + 1e-15)
    assert np.array_equal(runs[1], runs[2])
    assert not np.array_equal(runs[0], runs[1])

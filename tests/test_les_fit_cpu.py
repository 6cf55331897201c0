"""LES with the fitted transport in the oracle (viscflux_LES_xyz,
module_viscflux.f90:2200-2977, with mu_SGS_smagorinsky and the criterion of
shock_det_ducros_slv, module_tools.f90:2099-2181), on the CPU."""
import numpy as np

import workloads as W


def _flux(orc, st, cfg):
    fl = np.zeros((cfg.nx, cfg.ny, cfg.nz, 5 + cfg.nrv), order="F")
    orc.visc_flux(st, fl)
    return fl


def test_zero_factor_reduces_to_the_laminar_flux():
    """MU_SGS_FACTOR = 0: mu_SGS = 0 and every SGS term vanishes; the
    species enthalpy flux is summed in the LES routine's order
    ((h rvd)(...) instead of h (rvd ...)), so the flux equals the laminar
    one to rounding."""
    cfg, thd, adi, dxi, st, info, orc = W.case("mix", 12)
    W.perturb(st, 0.02, seed=3)
    orc.update_primitives(st)
    lam = _flux(orc, st, cfg)
    orc.set_les(mu_sgs_factor=0.0, percent_weight_sgs=0.5)
    les = _flux(orc, st, cfg)
    err = W.normwise(les, lam)
    assert np.all(err <= 1e-13), err


def test_smagorinsky_terms_and_fourier_time_step():
    """MU_SGS_FACTOR 0.17: the flux changes, and the Fourier criteria of
    the next time step see the subgrid diffusivity and conductivity
    (module_solver.f90:294-367), so dt_4(2) and dt_4(3) can only shrink."""
    cfg, thd, adi, dxi, st, info, orc = W.case("mix", 12, vis_dt=True)
    W.perturb(st, 0.02, seed=3)
    orc.update_primitives(st)
    lam = _flux(orc, st, cfg)
    dt4_lam, _ = orc.timestep(W.copy(st))
    orc.set_les(mu_sgs_factor=0.17, percent_weight_sgs=0.5)
    les = _flux(orc, st, cfg)
    assert np.abs(les - lam).max() > 1e-6 * np.abs(lam).max()
    dt4_les, _ = orc.timestep(W.copy(st))
    assert dt4_les[0] == dt4_lam[0]
    assert dt4_les[1] < dt4_lam[1] and dt4_les[2] < dt4_lam[2]
    # switching LES off forgets mu_SGS
    orc.set_les(enable=False)
    dt4_off, _ = orc.timestep(W.copy(st))
    assert np.array_equal(dt4_off, dt4_lam)


def test_fitted_les_rk3_steps_stay_finite():
    """Two RK3 steps of the nine-species layer with the fitted-transport LES
    and the Fourier criteria."""
    cfg, thd, adi, dxi, st, info, orc = W.case("mix", 12, vis_dt=True)
    W.perturb(st, 0.02, seed=3)
    orc.update_primitives(st)
    orc.set_les(mu_sgs_factor=0.05, percent_weight_sgs=0.5)
    for _ in range(2):
        dt4, dt = orc.timestep(st)
        orc.rk3(st, dt)
    v = st["v"][3:-3, 3:-3, 3:-3]
    assert np.all(np.isfinite(v)) and v[..., 0].min() > 0

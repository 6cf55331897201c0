"""The GPU path on the reference's own Sod configuration (2-D, WENO7,
fitted viscous fluxes, extrapolation and periodic boundaries; the case of
tests/sod_case.py) against the oracle on one block.  The oracle with the
reference's two-block sensor reproduces the reference's restart files
(tests/test_sod_pin.py); here the GPU's WENO7 fluxes, 2-D viscous terms,
Newton, boundaries, time step and RK3 must agree with the oracle to 1e-12
relative per conserved variable, as the WENO5 3-D path does
(tests/test_gpu_parity.py)."""
import numpy as np
import pytest

import sod_case as S
import workloads as W
from phd_gb300.izem import IzemGPU
from phd_gb300.thd import adi_struct

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _gpu(cfg, thd, a, grid, st):
    g = IzemGPU(cfg, thd, adi_struct(a))
    g.set_grid(*grid)
    g.upload(**st)
    return g


def _interior(x):
    ng = S.NG
    return x[ng:-ng, ng:-ng, ng:-ng]


def test_sod_fluxes_match_oracle():
    """x and y WENO7 fluxes (with the sensor set by one sensor pass, so both
    the nonlinear and the linear reconstructions occur) and the 2-D viscous
    fluxes at the initial discontinuity."""
    cfg, thd, a, orc, st, grid = S.sod_case(xblocks=1)
    g = _gpu(cfg, thd, a, grid, st)
    orc.shock_sensor(st)
    g.shock_sensor()
    got_s = g.download()["shock_sensor"]
    assert np.array_equal(_interior(got_s), _interior(st["shock_sensor"]))
    assert _interior(st["shock_sensor"]).any()
    nv = 5 + cfg.nrv
    fl = np.zeros((cfg.nx, cfg.ny, cfg.nz, nv), order="F")
    orc.euler_flux(st, 0, fl)
    orc.euler_flux(st, 1, fl)
    orc.visc_flux(st, fl)
    g.zero_flux()
    g.euler_LLF_x()
    g.euler_LLF_y()
    g.viscflux_xyz()
    err = W.normwise(g.flux(), fl)
    g.close()
    assert np.all(err <= TOL), err


def test_sod_steps_match_oracle():
    """Full time steps (time step, RK3 with the sticky sensor, primitives,
    extrapolation and periodic halos) from the initial discontinuity: one
    step within TOL (the x momentum, created by cancellation, within 1e-10);
    after twenty steps the rounding differences of the two
    machines have grown at the discontinuity, and the state agrees within
    1e-10 (the y and z momenta, rounding noise of the 2-D run, absolutely
    within 1e-10 of the largest density)."""
    cfg, thd, a, orc, st, grid = S.sod_case(xblocks=1)
    g = _gpu(cfg, thd, a, grid, st)
    for step in range(20):
        _, dt_o = orc.timestep(st)
        _, dt_g = g.timestep()
        assert abs(dt_g - dt_o) <= 1e-14 * dt_o
        orc.rk3(st, dt_o)
        g.rk3(dt_o)
        if step == 0:
            # after one step the x momentum is small, made from the pressure
            # jump across the discontinuity: its rounding is relative to that
            # cancellation, not to its own size
            err = W.normwise(_interior(g.download()["v"]), _interior(st["v"]))
            assert np.all(err[[0, 4, 5, 6]] <= TOL) and err[1] <= 1e-10, err
    got = _interior(g.download()["v"])
    g.close()
    ref = _interior(st["v"])
    rho_max = np.abs(ref[..., 0]).max()
    for q in range(ref.shape[-1]):
        d = np.abs(got[..., q] - ref[..., q]).max()
        if q in (2, 3):
            assert d <= 1e-10 * rho_max, (q, d)
        else:
            assert d <= 1e-10 * np.abs(ref[..., q]).max(), (q, d / np.abs(ref[..., q]).max())


def test_gpu_reproduces_reference_restarts():
    """The GPU path, told that the reference ran on two x-blocks
    (set_sensor_xblocks), runs the reference's Sod case from its initial
    condition through the main loop's time stepping and reproduces the
    reference's own FP64 restart files at the first three statistics
    times, within the bounds of the oracle's pin (tests/test_sod_pin.py):
    density, energy, species and x momentum within 2e-9 of their largest
    magnitude, y and z momenta within 1e-10 of the largest density.  The
    x-blocks also stop their Newton loops on their own tests, as the
    reference's ranks do."""
    cfg, thd, a, orc, st, grid = S.sod_case(xblocks=S.NX_BLOCKS)
    g = _gpu(cfg, thd, a, grid, st)
    g.set_sensor_xblocks(S.NX_BLOCKS)
    timing = S.stat_times(a, 3)
    time, nb, out = 0.0, 0, []
    while nb < 3:
        _, dtmin = g.timestep()
        write = False
        if time + dtmin > timing[nb] and time - dtmin < timing[nb]:
            dtmin = timing[nb] - time
            write = True
        g.rk3(dtmin)
        time = time + dtmin
        if write:
            nb += 1
            out.append((time, g.download()["v"]))
    g.close()
    names = ["rho", "rhoU", "rhoV", "rhoW", "rhoE", "O2", "N2"]
    for n, (t, v) in enumerate(out, 1):
        ref = S.golden(n)
        assert abs(t - float(ref["time"][0])) <= 1e-12 * float(ref["time"][0])
        vi = _interior(v)
        rho_max = np.abs(ref["rho"]).max()
        for q, name in enumerate(names):
            err = np.abs(vi[..., q] - ref[name]).max()
            if name in ("rhoV", "rhoW"):
                assert err <= 1e-10 * rho_max, (n, name, err)
            else:
                assert err <= 2e-9 * np.abs(ref[name]).max(), (n, name, err / np.abs(ref[name]).max())


def test_gpu_resumes_reference_restart(tmp_path):
    """Restart 1 of the reference's Sod run written in its HDF5 layout, read
    back (phd_gb300/restart.py), uploaded with a cleared temperature and
    closed on the device (izem_gpu_finalize_ic, the closure of
    read_restart_hdf5):
    * with the Adams-Shariff flags of the run that wrote it (the reference
      never clears a flag and does not store them), the resumed GPU run
      reproduces restart 2 within 5e-10 of each field's largest magnitude;
    * with cleared flags, as the reference's own resume starts, it agrees
      with the oracle resumed the same way, within the same bound."""
    from phd_gb300 import restart as R
    names7 = ["rho", "rhoU", "rhoV", "rhoW", "rhoE", "O2", "N2"]
    cfg, thd, a, orc, st, grid = S.sod_case(xblocks=S.NX_BLOCKS)
    S.run_to_stats(orc, st, a, 1)
    flags = st["shock_sensor"].copy()
    g1 = S.golden(1)
    p = str(tmp_path / "restart_00001.h5")
    R.write_restart(p, names7, [g1[n] for n in names7], float(g1["time"][0]))
    names, arrs, t1 = R.read_restart(p)
    ref = S.golden(2)
    t2 = float(ref["time"][0])
    out = []
    for carried in (True, False):
        st2 = R.state_from_restart(names, arrs, S.NG, species=["O2", "N2"])
        if carried:
            st2["shock_sensor"][...] = flags
        g = _gpu(cfg, thd, a, grid, st2)
        g.set_sensor_xblocks(S.NX_BLOCKS)
        g.finalize_ic()
        time = t1
        while True:
            _, dt = g.timestep()
            last = time + dt > t2 and time - dt < t2
            if last:
                dt = t2 - time
            g.rk3(dt)
            time = time + dt
            if last:
                break
        out.append(_interior(g.download()["v"]))
        g.close()
    rho_max = np.abs(ref["rho"]).max()
    for q, name in enumerate(names7):
        err = np.abs(out[0][..., q] - ref[name]).max()
        if name in ("rhoV", "rhoW"):
            assert err <= 1e-10 * rho_max, (name, err)
        else:
            assert err <= 5e-10 * np.abs(ref[name]).max(), (name, err / np.abs(ref[name]).max())
    _, _, _, orc2, _, _ = S.sod_case(xblocks=S.NX_BLOCKS)
    st3 = R.state_from_restart(names, arrs, S.NG, species=["O2", "N2"])
    orc2.finalize_ic(st3)
    time = t1
    while True:
        _, dt = orc2.timestep(st3)
        last = time + dt > t2 and time - dt < t2
        if last:
            dt = t2 - time
        orc2.rk3(st3, dt)
        time = time + dt
        if last:
            break
    vo = _interior(st3["v"])
    for q, name in enumerate(names7):
        err = np.abs(out[1][..., q] - vo[..., q]).max()
        if name in ("rhoV", "rhoW"):
            assert err <= 1e-10 * rho_max, (name, err)
        else:
            assert err <= 5e-10 * np.abs(vo[..., q]).max(), (name, err / np.abs(vo[..., q]).max())


def test_gpu_reproduces_reference_weno5_plots():
    """The Sod run with ORDER_WENO = 5 on the GPU (two emulated x-blocks, as
    the reference ran it) against the FP32 plot files of the reference's
    WENO5 run (testcases/sod/weno5_400) at statistics times 1 and 3: the
    temperature, pressure, density and x velocity within the oracle's bound
    (tests/test_sod_pin.py, WENO5_PLOT_TOL)."""
    from test_sod_pin import WENO5_PLOT_TOL, plot_fields
    cfg, thd, a, orc, st, grid = S.sod_case(xblocks=S.NX_BLOCKS, ng=3)
    g = _gpu(cfg, thd, a, grid, st)
    g.set_sensor_xblocks(S.NX_BLOCKS)
    timing = S.stat_times(a, 3)
    time, nb, out = 0.0, 0, []
    while nb < 3:
        _, dtmin = g.timestep()
        write = False
        if time + dtmin > timing[nb] and time - dtmin < timing[nb]:
            dtmin = timing[nb] - time
            write = True
        g.rk3(dtmin)
        time = time + dtmin
        if write:
            nb += 1
            out.append(g.download())
    g.close()
    for n in (1, 3):
        d = out[n - 1]
        ref = S.golden_plot(n, weno5=True)
        for k, x in plot_fields(a, d["v"], d["T"], d["W_i"], 3).items():
            err = np.abs(x - ref[k]).max() / np.abs(ref[k]).max()
            assert err <= WENO5_PLOT_TOL, (n, k, err)

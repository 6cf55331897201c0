"""CPU checks of the oracle and of the host-side data chain (no GPU)."""
import json
import os

import numpy as np
import pytest

import oracle
import workloads as W
from phd_gb300 import thd as T
from phd_gb300.capi import IzemCfg, IzemThd, IzemAdi

# the reference tree, where it is mounted (IZEM_REFERENCE_TESTCASES overrides)
REF = os.environ.get("IZEM_REFERENCE_TESTCASES", "/root/reference/devel-izem/testcases")


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference tree not mounted")
@pytest.mark.parametrize("setname,tranfit", [("h2air9", "shockedshearlayer/tranfit.out"), ("o2n2", "sod/tranfit.out")])
def test_shipped_species_match_reference_files(setname, tranfit):
    tf = T.read_tranfit(os.path.join(REF, tranfit))
    th = T.read_therm(os.path.join(REF, "sod/therm.dat"), tf["names"])
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

"""The benchmark's own step under parity: one pass of the reference
driver's main loop (izem.f90:252-281) -- timestep, then the Strang sequence
reaction_selec(dt/2), rk3(dt), reaction_selec(dt/2) -- on a 64 x 64 x 32
block of the 256 x 256 x 128 H2/air mixing layer with its grid spacing,
y-extrapolation faces, EGLIB precision-1 transport and the 9-species
mechanism, through the library's TimeLoop on the GPU and the oracle's
restatement of the same sequence.

Bounds, written here:
  * without chemistry: every conserved variable within 1e-12 of the
    oracle's, relative to that variable's maximum; T likewise; the time step
    bit for bit; sum_k Y_k = 1 within 1e-13 in every cell.  The species
    absent from the initial streams (the radicals and H2O) hold only the
    rounding noise of the diffusion fluxes when chemistry is off; they are
    scaled by 1e-6 of the largest variable instead of their own maximum,
    as in the other parity tests;
  * with chemistry, in units of the integrator's tolerance
    tol(y) = RTOL |y| + ATOL (RTOL = 1e-6, ATOL = 1e-10) per cell, for T and
    for every species mass fraction: max <= 1e-4.  In this pre-ignition
    window every reactor takes the same three BDF steps on both sides, no
    adaptive step decision differs, and the two DVODE runs agree to
    rounding (measured: T 1.2e-9, species 4e-7 tol units, i.e. about 1e-15
    relative in T); a changed step decision would show as about one tol
    unit.  sum_k Y_k = 1 within 1e-13.
"""
import numpy as np
import pytest

import oracle
import workloads as W
from phd_gb300 import ics
from phd_gb300.izem import IzemGPU, TimeLoop
from phd_gb300.mech import h2_mechanism
from phd_gb300.thd import eglib_link, load_species

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _block(chem):
    cfg, thd, adi, dxi, st, info = ics.mixing_layer_block(64, 64, 32, lib_dscalar=oracle.metrics_dscalar)
    cfg.eglib = 1
    cfg.reaction = 1 if chem else 0
    link = eglib_link(load_species("h2air9"))
    orc = oracle.Oracle(cfg, thd, adi, *dxi)
    orc.set_eglib(link)
    orc.finalize_ic(st)
    g = IzemGPU(cfg, thd, adi)
    g.set_eglib(link)
    g.set_grid(*dxi)
    g.upload(**st)
    return cfg, g, orc, st


def _sum_y_err(state, nrv=9):
    v = state["v"][3:-3, 3:-3, 3:-3]
    return np.abs(v[..., 5:5 + nrv].sum(axis=-1) / v[..., 0] - 1.0).max()


@pytest.mark.parametrize("chem", [False, True])
def test_driver_step_on_the_mixing_layer_block(chem):
    cfg, g, orc, st = _block(chem)
    mech = h2_mechanism() if chem else None
    if chem:
        g.set_mechanism(mech)
    loop = TimeLoop(g, reaction=chem)
    ref = {"dtmin": 1.0, "DTmax": 0.0, "time": 0.0}
    for _ in range(2):   # the second step's dt reads the first step's dtmin and DTmax
        dt_g = loop.step()
        dt_o = W.oracle_step(orc, st, mech, ref)
        if not chem:
            assert dt_g == dt_o, (dt_g, dt_o)
        else:
            assert abs(dt_g - dt_o) <= 1e-9 * dt_o, (dt_g, dt_o)
    got = g.download()
    it_max, unconverged = g.newton_stats()
    g.close()
    assert unconverged == 0 and it_max >= 1
    assert _sum_y_err(got) <= 1e-13 and _sum_y_err(st) <= 1e-13
    if not chem:
        i = (slice(3, -3),) * 3
        err = W.normwise(got["v"][i], st["v"][i])
        assert np.all(err <= TOL), err
        errT = np.abs(got["T"][i] - st["T"][i]).max() / np.abs(st["T"][i]).max()
        assert errT <= TOL, errT
        return
    assert abs(loop.DTmax - ref["DTmax"]) <= 100 * (W.RTOL * 3000.0 + W.ATOL)
    s = W.chem_error_stats(got, st)
    msg = "tol units: T %s, Y %s" % (s["T"], s["Y"])
    print(msg)
    for k in ("T", "Y"):
        assert s[k]["max"] <= 1e-4, msg

"""The reacting LES jet (the 512 x 512 x 256 planar H2/air jet workload) on a
16 x 64 x 8 block of the same grid spacing: the jet faces (planar inflow
with the workload's parameters and seeded fluctuations, characteristic
outflow), the Smagorinsky closure under EGLIB (MU_SGS_FACTOR 0.17) and the
Strang chemistry, stepped by the reference main loop's sequence (phd_gb300.izem.TimeLoop)
on the GPU and by the oracle's restatement of the same sequence.

Bounds, written here:
  * without chemistry: every conserved variable within 1e-12 of the
    oracle's, relative to that variable's maximum (noise-level species
    scaled by 1e-6 of the largest variable, as in the other parity tests);
    T likewise; the first time step bit for bit, the later ones within
    1e-14 (maxima over states that agree to rounding; the inflow
    fluctuations draw per 1 ns time interval, so a last-bit difference in
    the time does not change them);
  * with chemistry, in units of the integrator's tolerance RTOL |y| + ATOL
    per cell, for T and every species mass fraction: max <= 1e-4 (the
    window is pre-ignition: every reactor takes the same BDF steps on both
    sides, so they agree to rounding); sum_k Y_k = 1 within 1e-13.
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


def _jet(chem):
    cfg, thd, adi, dxi, st, info = ics.jet_les(16, 64, 8, lib_dscalar=oracle.metrics_dscalar)
    cfg.eglib = 1
    cfg.reaction = 1 if chem else 0
    link = eglib_link(load_species("h2air9"))
    orc = oracle.Oracle(cfg, thd, adi, *dxi)
    orc.set_eglib(link)
    orc.set_coords(*info["coords"], info["lx"])
    orc.set_jet(info["jet"])
    orc.set_les(mu_sgs_factor=0.17)
    orc.finalize_ic(st)
    g = IzemGPU(cfg, thd, adi)
    g.set_eglib(link)
    g.set_grid(*dxi)
    g.upload(**st)
    g.set_coords(*info["coords"], info["lx"])
    g.set_jet(info["jet"])
    g.set_les(mu_sgs_factor=0.17)
    return cfg, g, orc, st


@pytest.mark.parametrize("chem", [False, True])
def test_jet_driver_steps(chem):
    cfg, g, orc, st = _jet(chem)
    mech = h2_mechanism() if chem else None
    if chem:
        g.set_mechanism(mech)
    loop = TimeLoop(g, reaction=chem)
    ref = {"dtmin": 1.0, "DTmax": 0.0, "time": 0.0}
    for q in range(3):
        dt_g = loop.step()
        dt_o = W.oracle_step(orc, st, mech, ref)
        # the first step from the same state is bit for bit; later ones are
        # maxima over states that agree to rounding
        assert dt_g == dt_o if q == 0 else abs(dt_g - dt_o) <= 1e-14 * dt_o, (q, dt_g, dt_o)
    got = g.download()
    g.close()
    i = (slice(3, -3),) * 3
    v = got["v"][i]
    assert np.abs(v[..., 5:].sum(axis=-1) / v[..., 0] - 1.0).max() <= 1e-13
    if not chem:
        err = W.normwise(v, st["v"][i])
        assert np.all(err <= TOL), err
        errT = np.abs(got["T"][i] - st["T"][i]).max() / np.abs(st["T"][i]).max()
        assert errT <= TOL, errT
        return
    s = W.chem_error_stats(got, st)
    msg = "tol units: T %s, Y %s" % (s["T"], s["Y"])
    for k in ("T", "Y"):
        assert s[k]["max"] <= 1e-4, msg

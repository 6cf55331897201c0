"""The benchmark's step at its full size: one pass of the reference driver's
main loop (izem.f90:252-281) -- timestep, reaction_selec(dt/2), rk3(dt),
reaction_selec(dt/2) -- on the whole 256 x 256 x 128 H2/air mixing layer
with EGLIB precision-1 transport and the 9-species mechanism, through the
library's TimeLoop on the GPU and the oracle's restatement of the same
sequence (OpenMP on the host cores; about half a minute).

Bounds, as for the 64 x 64 x 32 block (tests/test_gpu_strang.py): the time
step within 1e-9; T and every species mass fraction within 1e-4 of the
integrator's tolerance tol(y) = RTOL |y| + ATOL per cell; DTmax within 100
tolerance units of 3000 K; sum_k Y_k = 1 within 1e-13; and the density,
momentum and energy, which chemistry does not touch but the flow step
carries, within 1e-12 of each variable's maximum."""
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


def test_driver_step_on_the_full_mixing_layer():
    cfg, thd, adi, dxi, st, info = ics.mixing_layer(lib_dscalar=oracle.metrics_dscalar)
    assert (cfg.nx, cfg.ny, cfg.nz) == (256, 256, 128)
    cfg.eglib, cfg.reaction = 1, 1
    link = eglib_link(load_species("h2air9"))
    mech = h2_mechanism()
    orc = oracle.Oracle(cfg, thd, adi, *dxi)
    orc.set_eglib(link)
    orc.finalize_ic(st)
    g = IzemGPU(cfg, thd, adi)
    g.set_eglib(link)
    g.set_grid(*dxi)
    g.upload(**st)
    g.set_mechanism(mech)
    loop = TimeLoop(g, reaction=True)
    ref = {"dtmin": 1.0, "DTmax": 0.0, "time": 0.0}
    dt_g = loop.step()
    dt_o = W.oracle_step(orc, st, mech, ref)
    assert abs(dt_g - dt_o) <= 1e-9 * dt_o, (dt_g, dt_o)
    got = g.download()
    g.close()
    assert abs(loop.DTmax - ref["DTmax"]) <= 100 * (W.RTOL * 3000.0 + W.ATOL)
    i = (slice(3, -3),) * 3
    for s_ in (got, st):
        v = s_["v"][i]
        assert np.abs(v[..., 5:].sum(axis=-1) / v[..., 0] - 1.0).max() <= 1e-13
    err = W.normwise(got["v"][i][..., :5], st["v"][i][..., :5])
    s = W.chem_error_stats(got, st)
    msg = "flow %s; tol units: T %s, Y %s" % (err, s["T"], s["Y"])
    print(msg)
    assert np.all(err <= TOL), msg
    for k in ("T", "Y"):
        assert s[k]["max"] <= 1e-4, msg

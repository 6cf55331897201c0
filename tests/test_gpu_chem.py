"""Parity of the GPU stiff-chemistry kernels with the oracle.

Both integrate the same reactor with the same adaptive BDF method; FMA
contraction on the GPU perturbs rounding, which the adaptive step control
can amplify, so agreement is required within ten times the integrator's own
tolerance per component (10 * (RTOL |y| + ATOL), RTOL = 1e-6, ATOL = 1e-10),
and for most cells it is at rounding level."""
import numpy as np
import pytest

import oracle
import workloads as W
from phd_gb300 import ics
from phd_gb300.izem import IzemGPU, psr_batch
from phd_gb300.mech import h2_mechanism

pytestmark = pytest.mark.gpu
RTOL, ATOL = 1e-6, 1e-10


def test_psr_batch_matches_oracle():
    m = h2_mechanism()
    T, rho, Y, dt = ics.batched_reactors(2048, seed=21)
    To, Yo = T.copy(), Y.copy()
    ist_o, ns_o = oracle.psr_cells(m, To, rho.copy(), Yo, dt.copy())
    Tg, Yg = T.copy(), Y.copy()
    ist_g, ns_g, ms = psr_batch(m, Tg, rho.copy(), Yg, dt.copy())
    assert np.all(ist_g == 2) and np.all(ist_o == 2)
    assert np.all(np.abs(Tg - To) <= 10 * (RTOL * np.abs(To) + ATOL))
    assert np.all(np.abs(Yg - Yo) <= 10 * (RTOL * np.abs(Yo) + ATOL))
    # most cells agree to rounding
    assert np.median(np.abs(Tg - To) / To) < 1e-12


def test_field_chem_step_matches_oracle():
    cfg, thd, adi, dxi, st, info, orc = W.case("mix", 16)
    m = h2_mechanism()
    g = IzemGPU(cfg, thd, adi)
    g.set_grid(*dxi)
    g.upload(**st)
    g.set_mechanism(m)
    dt = 0.5
    dtm_o = orc.chem_step(st, m, dt)
    dtm_g = g.reaction_selec(dt)
    got = g.download()
    i = (slice(3, -3),) * 3
    T_o, T_g = st["T"][i], got["T"][i]
    assert np.all(np.abs(T_g - T_o) <= 10 * (RTOL * np.abs(T_o) + ATOL))
    v_o, v_g = st["v"][i], got["v"][i]
    for q in range(5, 14):
        yo = v_o[..., q] / v_o[..., 0]
        yg = v_g[..., q] / v_g[..., 0]
        assert np.all(np.abs(yg - yo) <= 10 * (RTOL * np.abs(yo) + ATOL))
    assert abs(dtm_g - dtm_o) <= 10 * (RTOL * 3000 + ATOL)
    st_ = g.chem_stats()
    assert st_["failed"] == 0

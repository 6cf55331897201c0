"""Parity of the GPU stiff-chemistry kernels with the oracle.

The device integrator is the oracle's algorithm in the oracle's operation
order: compiled for the host it reproduces the oracle bit for bit
(tests/test_chem_cpu.py::test_device_integrator_reproduces_oracle_bitwise).
On the GPU, fused multiply-adds and CUDA's exp/log perturb the last bits;
for ignition-delay cells the radical pool starts below ATOL = 1e-10 and
grows exponentially, so those perturbations change the adaptive step
sequence and the two results differ by the integrator's own global error.
Bounds (workloads.reactor_error_bounds), with tol(y) = RTOL |y| + ATOL
(RTOL = 1e-6) per cell:
  * temperature: median < 1e-3, 99th percentile <= 10, max <= 200 tol(T)
  * species (largest over k per cell): median < 1e-2, 90th percentile
    <= 10 tol(Y_k); every cell |dY_k| <= 1e-3 max_cells |Y_k|
  * batch median cell: relative T difference below 1e-10 (rounding level)
The same bounds hold for the device right-hand side compiled for the host
without FMA and with the host's libm (tests/test_chem_cpu.py): the
reciprocal form alone produces differences of this size."""
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
    st, msg, ok = W.reactor_error_bounds(Tg, Yg, To, Yo)
    print(msg)
    assert ok, msg
    assert np.median(np.abs(Tg - To) / To) < 1e-10, msg


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
    v_o, v_g = st["v"][i], got["v"][i]
    Yo = np.stack([v_o[..., q] / v_o[..., 0] for q in range(5, 14)], axis=-1).reshape(-1, 9)
    Yg = np.stack([v_g[..., q] / v_g[..., 0] for q in range(5, 14)], axis=-1).reshape(-1, 9)
    s_, msg, ok = W.reactor_error_bounds(got["T"][i].ravel(), Yg, st["T"][i].ravel(), Yo)
    print(msg)
    assert ok, msg
    assert abs(dtm_g - dtm_o) <= 100 * (RTOL * 3000 + ATOL)
    st_ = g.chem_stats()
    assert st_["failed"] == 0


def test_reacting_field_chem_step_matches_oracle():
    """The field chemistry step on the learned-chemistry workload's reacting
    field (ics.reacting_field: the batched-reactor distribution as smooth
    fields) over 1e-6 s, the longest step of the training range, in which
    ignition fronts cross many cells: within workloads.FIELD_LIMITS, twice
    what the rounding of the reciprocal form alone gives on the same
    reactors on the host (tests/test_chem_cpu.py), and DTmax alike."""
    cfg, thd, adi, dxi, st, info = ics.reacting_field(20, 20, 20, dt_s=1e-6, corr=4,
                                                      lib_dscalar=oracle.metrics_dscalar)
    m = h2_mechanism()
    orc = oracle.Oracle(cfg, thd, adi, *dxi)
    orc.finalize_ic(st)
    g = IzemGPU(cfg, thd, adi)
    g.set_grid(*dxi)
    g.upload(**st)
    g.set_mechanism(m)
    dt = info["dt_s"] / info["time_ref"]
    T0 = st["T"].copy()
    dtm_o = orc.chem_step(st, m, dt)
    dtm_g = g.reaction_selec(dt)
    got = g.download()
    g.close()
    i = (slice(3, -3),) * 3
    v_o, v_g = st["v"][i], got["v"][i]
    Yo = np.stack([v_o[..., q] / v_o[..., 0] for q in range(5, 14)], axis=-1).reshape(-1, 9)
    Yg = np.stack([v_g[..., q] / v_g[..., 0] for q in range(5, 14)], axis=-1).reshape(-1, 9)
    s_, msg, ok = W.reactor_error_bounds(got["T"][i].ravel(), Yg, st["T"][i].ravel(), Yo, W.FIELD_LIMITS)
    print(msg, "max window dT %.1f K" % (np.abs(st["T"][i] - T0[i]).max() * adi.t_ref))
    assert ok, msg
    assert np.abs(st["T"][i] - T0[i]).max() * adi.t_ref > 100.0     # the field reacts
    assert abs(dtm_g - dtm_o) <= 100 * (RTOL * abs(dtm_o) + ATOL)


@pytest.mark.parametrize("variant", ["sri_collider", "equilibrium", "landau_teller"])
def test_psr_batch_with_variant_mechanisms(tmp_path, variant):
    """The persistent BDF kernels with a mechanism that uses the SRI fall-off
    form and a single-species collider, reverse rates from the equilibrium
    constant, or Landau-Teller factors (workloads.VARIANTS; no generated
    right-hand side matches them, so the kernels walk the tables): within
    the bounds above against the oracle."""
    m = W.VARIANTS[variant](tmp_path)
    T, rho, Y, dt = ics.batched_reactors(2048, seed=51)
    To, Yo = T.copy(), Y.copy()
    ist_o, _ = oracle.psr_cells(m, To, rho.copy(), Yo, dt.copy())
    Tg, Yg = T.copy(), Y.copy()
    ist_g, _, _ = psr_batch(m, Tg, rho.copy(), Yg, dt.copy())
    assert np.all(ist_g == 2) and np.all(ist_o == 2)
    st, msg, ok = W.reactor_error_bounds(Tg, Yg, To, Yo)
    print(msg)
    assert ok, msg


def test_chem_autotune_batch_leaves_inputs_and_keeps_results():
    """The batch autotuner times the register-budget variants on copies of a
    sample: the caller's arrays are unchanged, it reports every variant and
    its choice, and a batch integrated afterwards stays within the bounds
    above against the oracle."""
    import torch
    from phd_gb300.izem import chem_autotune_device
    m = h2_mechanism()
    T, rho, Y, dt = ics.batched_reactors(4096, seed=23)
    dev = [torch.from_numpy(a).to("cuda:0") for a in (T, rho, Y, dt)]
    rep = chem_autotune_device(m, len(T), *dev)
    assert rep["sample"] == len(T) and rep["chosen"].startswith("128x")
    timed = {k: v for k, v in rep.items() if k.startswith("128x") and "(" in k}
    assert len(timed) == 5 and rep["chosen"] == min(timed, key=timed.get)
    assert np.array_equal(dev[0].cpu().numpy(), T) and np.array_equal(dev[2].cpu().numpy(), Y)
    To, Yo = T.copy(), Y.copy()
    oracle.psr_cells(m, To, rho.copy(), Yo, dt.copy())
    Tg, Yg = T.copy(), Y.copy()
    psr_batch(m, Tg, rho.copy(), Yg, dt.copy())
    rT = np.abs(Tg - To) / (RTOL * np.abs(To) + ATOL)
    assert rT.max() <= 100 and np.percentile(rT, 99) <= 10
    assert (np.abs(Yg - Yo) / np.abs(Yo).max(axis=0)).max() <= 1e-3


def test_dvodesimp_matches_oracle():
    """dvodesimp (module_reaction.f90:173-251) on the device: the same cells
    are left alone as by the oracle (v and T unchanged to the bit), the
    integrated ones agree within the bounds above, and max |dT| comes from
    them; disabling the skip restores the integration of every cell."""
    m = h2_mechanism()
    cfg, thd, adi, dxi, st, orc, (yf, yo, ih2, in2) = W.mixing_layer_with_streams()
    st0 = W.copy(st)
    orc.set_chem_skip(yf, yo, ih2, in2)
    dtm_o = orc.chem_step(st, m, 0.5)
    g = IzemGPU(cfg, thd, adi)
    g.set_grid(*dxi)
    g.upload(**st0)
    g.set_mechanism(m)
    g.set_chem_skip(yf, yo, ih2, in2)
    dtm_g = g.reaction_selec(0.5)
    got = g.download()
    i = (slice(3, -3),) * 3
    same_o = np.all(st["v"][i] == st0["v"][i], axis=-1) & (st["T"][i] == st0["T"][i])
    same_g = np.all(got["v"][i] == st0["v"][i], axis=-1) & (got["T"][i] == st0["T"][i])
    assert np.array_equal(same_g, same_o) and 0 < same_o.sum() < same_o.size
    T_o, T_g = st["T"][i], got["T"][i]
    assert np.all(np.abs(T_g - T_o) <= 100 * (RTOL * np.abs(T_o) + ATOL))
    for q in range(5, 14):
        yo_, yg_ = st["v"][i][..., q] / st["v"][i][..., 0], got["v"][i][..., q] / got["v"][i][..., 0]
        assert np.all(np.abs(yg_ - yo_) <= 1e-3 * np.abs(yo_).max() + ATOL)
    assert abs(dtm_g - dtm_o) <= 100 * (RTOL * 3000 + ATOL)
    assert g.chem_stats()["failed"] == 0
    g.set_chem_skip(enable=False)
    g.upload(**st0)
    g.reaction_selec(0.5)
    allc = g.download()
    g.close()
    assert np.sum(~(np.all(allc["v"][i] == st0["v"][i], axis=-1) & (allc["T"][i] == st0["T"][i]))) >= \
        np.sum(~same_o)


def test_generated_and_table_forms_agree():
    """The shipped mechanism runs on the right-hand side generated for it
    (phd_gb300/mechgen.py); the table-walking form gives the same results
    within the bounds above (the two compilations may fuse multiply-adds
    differently; on the host they agree bit for bit), and takes over when
    the generated form is not allowed."""
    from phd_gb300.izem import load_library
    lib = load_library()
    m = h2_mechanism()
    T, rho, Y, dt = ics.batched_reactors(2048, seed=21)
    out = []
    try:
        for allow in (1, 0):
            lib.izem_gpu_allow_chem_generated(allow)
            Tg, Yg = T.copy(), Y.copy()
            ist, ns, ms = psr_batch(m, Tg, rho.copy(), Yg, dt.copy())
            assert lib.izem_gpu_chem_generated() == allow and np.all(ist == 2)
            out.append((Tg, Yg))
    finally:
        lib.izem_gpu_allow_chem_generated(1)
    st, msg, ok = W.reactor_error_bounds(out[0][0], out[0][1], out[1][0], out[1][1])
    assert ok, msg
    To, Yo = T.copy(), Y.copy()
    oracle.psr_cells(m, To, rho.copy(), Yo, dt.copy())
    st, msg, ok = W.reactor_error_bounds(out[0][0], out[0][1], To, Yo)
    assert ok, msg

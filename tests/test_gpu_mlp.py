"""Surrogate MLP on the GPU: tensor-core forward and backward against the
FP64 oracle, training, and the gated surrogate chemistry step against the
FP64 BDF integrator.

Tolerances: inputs, weights and hidden activations are BF16 on both sides;
the device accumulates in FP32, so outputs agree to 1e-2 relative (norm-wise)
and parameter gradients to 3e-2 relative with cosine similarity >= 0.999."""
import time

import numpy as np
import pytest

from oracle import mlp_oracle as mo
from phd_gb300 import ics
from phd_gb300.izem import psr_batch
from phd_gb300.mech import h2_mechanism
from phd_gb300.surrogate import DEFAULT_GATE, Surrogate, calibrate_cap, features, train_ensemble, training_set

pytestmark = pytest.mark.gpu


def _data(M, seed=1):
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.standard_normal((M, 12)).astype(np.float32), rng.standard_normal((M, 10)).astype(np.float32)


def test_forward_matches_fp64_oracle():
    s = Surrogate(seed=11)
    W, b = s.get_params()
    x, _ = _data(1000)
    y = s.forward(x)
    ref, _ = mo.forward(W, b, x)
    err = np.abs(y - ref).max() / np.abs(ref).max()
    assert err < 1e-2, err


def test_gradients_match_fp64_oracle():
    s = Surrogate(seed=12)
    W, b = s.get_params()
    x, t = _data(512, seed=2)
    loss, gW, gb = s.grads(x, t)
    lref, rW, rb = mo.loss_and_grads(W, b, x, t)
    assert abs(loss - lref) <= 1e-2 * lref
    for l in range(5):
        for g, r in ((gW[l], rW[l]), (gb[l], rb[l])):
            g = g.astype(np.float64).ravel(); r = r.ravel()
            rel = np.linalg.norm(g - r) / np.linalg.norm(r)
            cos = g @ r / (np.linalg.norm(g) * np.linalg.norm(r))
            assert rel < 3e-2 and cos > 0.999, (l, rel, cos)


def test_training_reduces_loss():
    s = Surrogate(seed=13)
    rng = np.random.Generator(np.random.PCG64(4))
    x = rng.standard_normal((65536, 12)).astype(np.float32)
    t = np.stack([np.sin(x[:, k]) * np.cos(x[:, (k + 3) % 12]) for k in range(10)], axis=1).astype(np.float32)
    losses = s.train(x, t, epochs=6, batch=4096, lr=2e-3)
    assert losses[-1] < 0.2 * losses[0], losses


def test_device_features_match_host_features():
    """The gated step featurises the reactors on the device (FP32 logarithms,
    normalisation, BF16 rows for the tensor-core network).  Its raw
    temperature prediction equals izem_mlp_forward on the host's FP64
    features normalised the same way, up to BF16 rounding of the inputs."""
    mech = h2_mechanism()
    X, Yt = training_set(mech, 1 << 12, seed=5)
    s = Surrogate(seed=3)
    s.fit_norm(X, Yt)
    T, rho, Y, dt = ics.batched_reactors(4096, seed=41)
    wt = np.array([mech.wt[k] for k in range(mech.kk)])
    yh = s.forward(s.normalise(features(T, rho, Y, dt, wt)))
    dT_host = yh[:, 9].astype(np.float64) * s.norm[2 * 12 + 10 + 9] + s.norm[2 * 12 + 9]
    r = s.chem_step(mech, T.copy(), rho.copy(), Y.copy(), dt.copy(), DEFAULT_GATE)
    d = np.abs(r["dT_pred"] - dT_host)
    spread = np.std(dT_host)
    assert np.median(d) <= 1e-3 * spread and d.max() <= 0.1 * spread, (np.median(d), d.max(), spread)


def test_surrogate_gains_over_bdf_with_gate():
    """What the trained network gains over the method without it: on 2^20
    reactors the gated surrogate step, with its |dT| cap calibrated on other
    held-out reactors, is faster than BDF on every cell, and with the
    fallback active its
    temperature increments stay within 1 % of the largest FP64 increment.
    Without the cap, the same step accepts more cells: with it, the cells
    predicted above the cap go to the BDF integrator, and the others get the
    same surrogate result."""
    mech = h2_mechanism()
    s, s2 = train_ensemble(mech, n=1 << 19, seed=31, epochs=24)
    gcap, cal = calibrate_cap([s, s2], mech, DEFAULT_GATE, n=1 << 18)
    # 2^20 reactors: the fallback launch waits for its stiffest cell (a fixed
    # tail of about 0.1 s), so the gain shows once BDF on every cell costs more
    T, rho, Y, dt = ics.batched_reactors(1 << 20, seed=77)
    Tb, Yb = T.copy(), Y.copy()
    _, _, ms_bdf = psr_batch(mech, Tb, rho.copy(), Yb, dt.copy())
    dT_ref = Tb - T
    scale = np.abs(dT_ref).max()
    Tc, Yc = T.copy(), Y.copy()
    rc = s.chem_step(mech, Tc, rho.copy(), Yc, dt.copy(), gcap, partner=s2)
    errc = np.abs((Tc - T) - dT_ref)
    frac_fb = rc["fallback"] / len(T)
    assert rc["failed"] == 0
    assert errc.max() <= 0.01 * scale, (errc.max(), scale, frac_fb, gcap[9], cal["table"])
    assert frac_fb < 1.0
    assert rc["ms"] < ms_bdf, (rc["ms"], ms_bdf)   # the gated step is faster than BDF on every cell
    print("surrogate: dT cap %.0f K, fallback %.3f, max err %.3g K (scale %.3g K), BDF %.1f ms, surrogate %.1f ms "
          "(MLP %.1f ms)" % (gcap[9], frac_fb, errc.max(), scale, ms_bdf, rc["ms"], rc["ms_mlp"]))
    fb_c = s.fallback_cells()
    Ts, Ys = T.copy(), Y.copy()
    r = s.chem_step(mech, Ts, rho.copy(), Ys, dt.copy(), DEFAULT_GATE, partner=s2)
    err = np.abs((Ts - T) - dT_ref)
    fb_u = s.fallback_cells()
    assert r["failed"] == 0 and len(fb_c) == rc["fallback"] and len(fb_u) == r["fallback"]
    # the cap only adds rejections: the cells predicted above it fall back,
    # and the cells accepted with the cap get the same result without it
    over = np.flatnonzero(np.abs(rc["dT_pred"]) > gcap[9])
    assert np.all(np.isin(over, fb_c)) and np.all(np.isin(fb_u, fb_c))
    acc_c = np.setdiff1d(np.arange(len(T)), fb_c)
    assert np.array_equal(Tc[acc_c], Ts[acc_c]) and np.array_equal(Yc[acc_c], Ys[acc_c])
    # fallback cells are integrated by the BDF kernel for rejected cells: the
    # same integrator as BDF on every cell, within its tolerance (the
    # bounds of tests/test_gpu_chem.py)
    rT = np.abs(Tc[fb_c] - Tb[fb_c]) / (1e-6 * np.abs(Tb[fb_c]) + 1e-10)
    assert rT.max() <= 100, rT.max()
    print("without the cap: fallback %.3f, max err %.3g K" % (r["fallback"] / len(T), err.max()))


def _small_flow():
    from phd_gb300.izem import IzemGPU, metrics_dscalar
    cfg, thd, adi, dxi, st, info = ics.mixing_layer(32, 32, 16, Lx=32 * 47e-6, Ly=32 * 47e-6, Lz=16 * 47e-6,
                                                    lib_dscalar=metrics_dscalar)
    cfg.reaction = 1
    g = IzemGPU(cfg, thd, adi)
    g.set_grid(*dxi)
    g.upload(**st)
    g.finalize_ic()
    g.set_mechanism(h2_mechanism())
    _, dt = g.timestep(DTmax=0.0, dtmin=1.0)
    return g, dt


def test_flow_surrogate_with_every_cell_rejected_equals_bdf():
    """Chemistry mode CHEM_MLP with a gate that accepts nothing sends every
    window cell through the gather, the BDF kernel for rejected cells and
    the scatter: the flow state must equal that of the BDF mode.  The two
    modes run the same integrator in two kernels, which the compiler may
    contract differently, so temperatures and species agree within the
    integrator's tolerance (the bounds of tests/test_gpu_chem.py) and the
    density, momentum and energy, which chemistry does not touch, exactly."""
    g, dt = _small_flow()
    st0 = g.download()
    chem_dt = 2000.0 * dt   # long enough for visible chemistry in the mixing region
    d0 = g.reaction_selec(chem_dt, mode=0)
    ref = g.download()
    g.upload(**st0)
    s = Surrogate(seed=3)
    g.set_surrogate(s, gate=(1e9, -1e9, 1.0, -1.0, 2e-3, 1.0, 0.02, 1.0, 0.005))
    d1 = g.reaction_selec(chem_dt, mode=1)
    got = g.download()
    st = g.surrogate_stats()
    assert st["fallback"] == st["cells"] > 0
    assert abs(d1 - d0) <= 100 * (1e-6 * abs(d0) + 1e-10)
    assert np.array_equal(got["v"][..., :5], ref["v"][..., :5])
    assert np.all(np.abs(got["T"] - ref["T"]) <= 100 * (1e-6 * np.abs(ref["T"]) + 1e-10))
    for q in range(5, got["v"].shape[-1]):
        yg, yr = got["v"][..., q] / got["v"][..., 0], ref["v"][..., q] / ref["v"][..., 0]
        assert np.abs(yg - yr).max() <= 1e-3 * max(np.abs(yr).max(), 1e-30)


def test_flow_surrogate_error_within_gate():
    """A surrogate trained on the block's own reactors (labelled by the BDF
    integrator) replaces the chemistry of the accepted cells, the rest are
    integrated by BDF.  This block has only 5,625 window cells to train on,
    so the bound here is 5 % of the largest BDF increment over the block
    (ghost cells included); the full-size flow in bench.py trains on 2^19
    cells and reports its own error."""
    from phd_gb300.surrogate import flow_gate, flow_training_set, train_on
    g, dt = _small_flow()
    chem_dt = 2000.0 * dt
    mech = h2_mechanism()
    X, Yt = flow_training_set(g, mech, chem_dt, spread=0.05)
    s, s2 = train_on(X, Yt, epochs=900, batch=512)
    gate = flow_gate(X, Yt)
    st0 = g.download()
    t0 = st0["T"].copy()
    g.reaction_selec(chem_dt, mode=0)
    dT_ref = (g.download()["T"] - t0) * g.adi.t_ref
    g.upload(**st0)
    g.set_surrogate(s, s2, gate=gate)
    g.reaction_selec(chem_dt, mode=1)
    dT = (g.download()["T"] - t0) * g.adi.t_ref
    st = g.surrogate_stats()
    err = np.abs(dT - dT_ref).max()
    scale = np.abs(dT_ref).max()
    print("flow surrogate: cells %d fallback %d, max |dT err| %.3g K of max |dT| %.3g K"
          % (st["cells"], st["fallback"], err, scale))
    assert st["fallback"] < st["cells"]
    assert err <= 0.05 * scale


def test_bounded_wait_gives_up_and_the_device_stays_usable():
    """Failure detection without a fault: a kernel polls an mbarrier that
    nothing arrives on, in the way the tensor-core kernels poll theirs, and
    stops after a bounded number of polls with its error flag set; the
    context then runs the tensor-core forward normally."""
    from phd_gb300.izem import wait_selftest
    assert wait_selftest(4096) == 1
    s = Surrogate(seed=3)
    x = np.random.default_rng(0).standard_normal((512, 12)).astype(np.float32)
    y = s.forward(x)
    assert np.all(np.isfinite(y))

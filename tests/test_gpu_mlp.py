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
from phd_gb300.surrogate import DEFAULT_GATE, Surrogate, features, train_ensemble, training_set

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


def test_surrogate_gains_over_bdf_with_gate():
    """What the trained network gains over the method without it: the gated
    surrogate step is faster than BDF on every cell, and with the fallback
    active its temperature increments stay within 1 % of the largest FP64
    increment."""
    mech = h2_mechanism()
    s, s2 = train_ensemble(mech, n=1 << 19, seed=31, epochs=24)
    T, rho, Y, dt = ics.batched_reactors(1 << 17, seed=77)
    Tb, Yb = T.copy(), Y.copy()
    t0 = time.perf_counter()
    _, _, ms_bdf = psr_batch(mech, Tb, rho.copy(), Yb, dt.copy())
    Ts, Ys = T.copy(), Y.copy()
    r = s.chem_step(mech, Ts, rho.copy(), Ys, dt.copy(), DEFAULT_GATE, partner=s2)
    dT_ref = Tb - T
    err = np.abs((Ts - T) - dT_ref)
    scale = np.abs(dT_ref).max()
    frac_fb = r["fallback"] / len(T)
    assert r["failed"] == 0
    assert err.max() <= 0.01 * scale, (err.max(), scale, frac_fb)
    assert frac_fb < 1.0
    print("surrogate: fallback %.3f, max err %.3g K (scale %.3g K), BDF %.1f ms, surrogate %.1f ms (MLP %.1f ms)"
          % (frac_fb, err.max(), scale, ms_bdf, r["ms"], r["ms_mlp"]))

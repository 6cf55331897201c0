"""The reacting field of the learned-chemistry workload (ics.reacting_field):
the batched-reactor distribution laid out as smooth seeded fields, closed by
the oracle's finalize_ic."""
import numpy as np

import oracle
from phd_gb300 import ics


def test_smooth_uniform_marginal_and_smoothness():
    """Each point is uniform on (0, 1): over a field with many correlation
    cells the decile counts are near 10 %; neighbours are strongly
    correlated, points two correlation lengths apart hardly at all; the
    same seed gives the same field."""
    shape, corr = (160, 128, 96), 8
    u = ics.smooth_uniform(shape, corr, np.random.Generator(np.random.PCG64(4)))
    assert u.shape == shape and np.all((u > 0.0) & (u < 1.0))
    dec = np.histogram(u, bins=10, range=(0.0, 1.0))[0] / u.size
    assert np.all(np.abs(dec - 0.1) < 0.015), dec
    near = np.corrcoef(u[:-1].ravel(), u[1:].ravel())[0, 1]
    far = np.corrcoef(u[:-2 * corr].ravel(), u[2 * corr:].ravel())[0, 1]
    assert near > 0.95 and abs(far) < 0.1, (near, far)
    again = ics.smooth_uniform(shape, corr, np.random.Generator(np.random.PCG64(4)))
    assert np.array_equal(u, again)


def test_smooth_uniform_slabs_equal_the_whole_field():
    """The field evaluated plane range by plane range (as the threaded
    builder does) equals the field evaluated at once."""
    shape, corr = (40, 30, 21), 8
    u = ics.smooth_uniform(shape, corr, np.random.Generator(np.random.PCG64(3)))
    lat = np.random.Generator(np.random.PCG64(3)).standard_normal(tuple(n // corr + 2 for n in shape))
    parts = [ics._smooth_eval(lat, corr, shape, k, min(shape[2], k + 4)) for k in range(0, shape[2], 4)]
    assert np.array_equal(u, np.concatenate(parts, axis=2))


def test_reacting_field_state():
    """Mass fractions sum to 1, T and p lie in the distribution's ranges,
    the velocity is zero, the ghosts extend the interior, and the state is
    closed: the oracle's finalize_ic recovers the generator's temperature
    from the energy.  The build does not depend on the thread count."""
    cfg, thd, adi, dxi, st, info = ics.reacting_field(40, 32, 24, lib_dscalar=oracle.metrics_dscalar, threads=3)
    _, _, _, _, st1, _ = ics.reacting_field(40, 32, 24, lib_dscalar=oracle.metrics_dscalar, threads=1)
    for k in st:
        assert np.array_equal(st[k], st1[k]), k
    ng, nrv = cfg.ng, cfg.nrv
    v, T = st["v"], st["T"]
    rho = v[..., 0]
    Y = v[..., 5:] / rho[..., None]
    assert np.abs(Y.sum(axis=-1) - 1.0).max() < 1e-14 and Y.min() >= 0.0
    TK = T * adi.t_ref
    assert TK.min() >= 800.0 and TK.max() <= 2400.0
    W_i = np.einsum("...k,k->...", Y, np.array(thd.Wc_i[:nrv]))
    p_atm = rho * T * W_i * adi.p_ref / 101325.0
    assert p_atm.min() >= 1.0 - 1e-9 and p_atm.max() <= 10.0 + 1e-9
    assert np.all(v[..., 1:4] == 0.0)
    assert np.array_equal(v[:ng], np.broadcast_to(v[ng:ng + 1], v[:ng].shape))
    assert np.array_equal(T[:, :, -ng:], np.broadcast_to(T[:, :, -ng - 1:-ng], T[:, :, -ng:].shape))
    assert info["dt_s"] == 3e-7 and cfg.reaction == 1
    orc = oracle.Oracle(cfg, thd, adi, *dxi)
    T_gen = T.copy()
    orc.finalize_ic(st)
    assert np.abs(st["T"] - T_gen).max() <= 1e-9 * np.abs(T_gen).max()


def test_reaction_window_is_where_the_oracle_reacts():
    """surrogate.reaction_window, which the learned-chemistry bench uses to
    compare increments, covers exactly the cells the oracle's chemistry
    step changes on a reacting field with unequal extents."""
    from phd_gb300.mech import h2_mechanism
    from phd_gb300.surrogate import reaction_window
    cfg, thd, adi, dxi, st, info = ics.reacting_field(14, 12, 10, dt_s=1e-6, corr=4,
                                                      lib_dscalar=oracle.metrics_dscalar)
    orc = oracle.Oracle(cfg, thd, adi, *dxi)
    orc.finalize_ic(st)
    v0 = st["v"].copy()
    orc.chem_step(st, h2_mechanism(), info["dt_s"] / info["time_ref"])
    ng = cfg.ng
    inner = (slice(ng, -ng),) * 3
    changed = np.any(st["v"][inner][..., 5:] != v0[inner][..., 5:], axis=-1)
    mask = np.zeros(st["T"].shape, dtype=bool)
    mask[reaction_window(cfg)] = True
    assert np.array_equal(changed, mask[inner]) and changed.sum() == 7 * 5 * 3

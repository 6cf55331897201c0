"""The Ducros shock sensor (SHOCK_SENSOR_TYPE = DUCROS) of the oracle
against a numpy restatement of compute_duixj + shock_sensor_ducros
(module_tools.f90:2521-2719): velocity gradients by the 6th-order central
first derivative of dx_fixed1 (module_deriv.f90:926-1171), in the
reference's summation order, and the flag where
(div u)^2 / ((div u)^2 + |curl u|^2 + 1e-30) > DUCROS_TREDUC."""
import numpy as np
import pytest

import workloads as W

A6 = [-1.0 / 60.0, 9.0 / 60.0, -45.0 / 60.0, 0.0, 45.0 / 60.0, -9.0 / 60.0, 1.0 / 60.0]


def shake_velocity(st, amp=0.3, seed=11):
    """Seeded relative noise on each momentum component of the interior (a
    velocity field with divergence as well as rotation)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    v = st["v"]
    for a in range(1, 4):
        v[3:-3, 3:-3, 3:-3, a] *= 1.0 + amp * rng.standard_normal(v[3:-3, 3:-3, 3:-3, a].shape)
    return st


def _ducloc(st, dxi, ng=3):
    """ducloc at the interior points (numpy, periodic central stencils)."""
    v = st["v"]
    rho_i = 1.0 / np.where(v[..., 0] == 0.0, 1.0, v[..., 0])
    u = [v[..., 1 + a] * rho_i for a in range(3)]
    n = [s - 2 * ng for s in v.shape[:3]]
    du = {}
    for a in range(3):
        for d in range(3):
            dd = np.zeros(n)
            for l in range(-3, 4):
                sl = [slice(ng, ng + n[0]), slice(ng, ng + n[1]), slice(ng, ng + n[2])]
                sl[d] = slice(ng + l, ng + l + n[d])
                dd = dd + A6[l + 3] * u[a][tuple(sl)]
            shape = [1, 1, 1]
            shape[d] = n[d]
            du[(a, d)] = dd * dxi[d][ng:ng + n[d]].reshape(shape)
    div = du[(0, 0)] + du[(1, 1)] + du[(2, 2)]
    div = div * div
    wrk = du[(2, 1)] - du[(1, 2)]
    vort = wrk * wrk
    wrk = du[(0, 2)] - du[(2, 0)]
    vort = vort + wrk * wrk
    wrk = du[(1, 0)] - du[(0, 1)]
    vort = vort + wrk * wrk
    return div / (div + vort + 1e-30)


@pytest.mark.parametrize("treduc", [0.05, 0.2, 0.6])
def test_oracle_ducros_matches_numpy(treduc):
    """A perturbed Taylor-Green box (periodic: central stencils everywhere):
    the oracle's flags are the numpy restatement's, bit for bit."""
    cfg, thd, adi, dxi, st, info, orc = W.case("tgv", 12)
    shake_velocity(st)
    orc.update_primitives(st)
    orc.set_shock_sensor("DUCROS", treduc)
    st["shock_sensor"][...] = 0
    orc.shock_sensor(st)
    got = st["shock_sensor"][3:-3, 3:-3, 3:-3]
    ref = _ducloc(st, dxi) > treduc
    assert 0 < ref.sum() < ref.size
    assert np.array_equal(got.astype(bool), ref)


def test_ducros_flags_are_sticky():
    """A flag once set stays set: a second evaluation on a divergence-free
    field clears nothing."""
    cfg, thd, adi, dxi, st, info, orc = W.case("tgv", 12)
    orc.set_shock_sensor("DUCROS", 0.2)
    st["shock_sensor"][...] = 0
    st["shock_sensor"][5, 5, 5] = 1
    orc.shock_sensor(st)
    assert st["shock_sensor"][5, 5, 5] == 1


def test_set_shock_sensor_rejects_bad_arguments():
    cfg, thd, adi, dxi, st, info, orc = W.case("tgv", 12)
    import oracle
    with pytest.raises(oracle.OracleError):
        orc.set_shock_sensor("DUCROS", 1.5)

"""Non-reflecting faces (NOREFLECTION) in the oracle, on the CPU.

The oracle's bc_noreflectionweno (module_weno.f90:2129-4498) is checked
against a numpy restatement written from the same text with dense matrices:
at every boundary point of a non-reflecting face, the characteristic vectors
of the flux Jacobian at the point's own state, the eigenvalues of the waves
leaving the domain, and the one-sided derivative with wenopar's cnr weights
(module_weno.f90:199-217).  Also checked: the ghost fill of bc_noreflection
(module_BCs.f90:426-512) and the dropped flux difference of the Euler sweep
at the boundary points (module_weno.f90:620-623, 1002, 1018).
"""
import numpy as np
import pytest

import oracle
import workloads as W
from phd_gb300 import ics
from phd_gb300.capi import BC_NOREFLECTION

NG = 3
CNR = np.array([-49.0 / 20.0, 6.0, -15.0 / 2.0, 20.0 / 3.0, -15.0 / 4.0, 6.0 / 5.0, -1.0 / 6.0])


def _case(species="o2n2", faces="xy", blob=0.0, ng=NG):
    cfg, thd, adi, dxi, st, info = ics.acoustic_pulse(species=species, faces=faces, blob=blob, ng=ng,
                                                      lib_dscalar=oracle.metrics_dscalar)
    orc = oracle.Oracle(cfg, thd, adi, *dxi)
    orc.finalize_ic(st)
    orc.update_primitives(st)   # the ghosts of the non-reflecting faces as a stage leaves them
    return cfg, thd, dxi, st, orc


def char_matrices(d, uc, Y, psi, ht, q, cs, b1, b2, xi):
    """Dense left and right characteristic vectors along axis d for one
    state, row by row as module_weno.f90:2224-2418 writes them for the W face
    (the normal velocity and the tangential pair permuted for the others)."""
    nrv = len(Y)
    nv = 5 + nrv
    t1, t2 = (1, 2) if d == 0 else ((0, 2) if d == 1 else (0, 1))
    un = uc[d]
    el = np.zeros((nv, nv))
    er = np.zeros((nv, nv))
    csi = 1.0 / cs
    el[0, 0] = 0.5 * (b1 + un * csi)
    el[2, 0] = 0.5 * (b1 - un * csi)
    for a in range(3):
        el[0, 1 + a] = -0.5 * (b2 * un + csi) if a == d else -0.5 * (b2 * uc[a])
        el[2, 1 + a] = -0.5 * (b2 * un - csi) if a == d else -0.5 * (b2 * uc[a])
        el[1, 1 + a] = b2 * uc[a]
    el[0, 4] = el[2, 4] = 0.5 * b2
    el[1, 0] = 1.0 - b1
    el[1, 4] = -b2
    el[3, 0], el[3, 1 + t1] = -uc[t1], 1.0
    el[4, 0], el[4, 1 + t2] = -uc[t2], 1.0
    el[0, 5:] = 0.5 * b2 * psi
    el[1, 5:] = -2.0 * el[0, 5:]
    el[2, 5:] = el[0, 5:]
    el[5, 0] = (1 + xi) * q
    el[5, 1:4] = -(1 + xi) * np.asarray(uc)
    el[5, 4] = 1 + xi
    el[5, 5:] = xi * psi
    for s in range(nrv - 1):
        el[6 + s, 0] = -b1 * Y[s]
        el[6 + s, 1:4] = b2 * np.asarray(uc) * Y[s]
        el[6 + s, 4] = -b2 * Y[s]
        el[6 + s, 5:] = -b2 * Y[s] * psi
        el[6 + s, 5 + s] += 1.0
    er[0, 0:3] = 1.0
    er[1 + d, 0:3] = (un - cs, un, un + cs)
    er[1 + t1, 0:3] = uc[t1]
    er[1 + t1, 3] = 1.0
    er[1 + t2, 0:3] = uc[t2]
    er[1 + t2, 4] = 1.0
    er[4, 0:5] = (ht - un * cs, q, ht + un * cs, uc[t1], uc[t2])
    er[5:, 0] = Y
    er[5:, 2] = Y
    for l in range(5, nv - 1):
        er[l - 1, l] = 1.0
    er[nv - 2, nv - 1] = 1.0
    er[nv - 1, 5] = -1.0 / psi[-1]
    er[nv - 1, 6:] = -psi[:-1] / psi[-1]
    return el, er


def nr_term(st, thd, dxi, cfg, face):
    """numpy restatement of one face of bc_noreflectionweno; returns the
    interior-shaped array it adds to fl."""
    v, T, Wi, cp, ha = st["v"], st["T"], st["W_i"], st["cp"], st["ha"]
    nrv = cfg.nrv
    nv = 5 + nrv
    ng = cfg.ng
    n = (cfg.nx, cfg.ny, cfg.nz)
    d, hi = face // 2, face % 2
    sc = ng + (n[d] - 1 if hi else 0)
    gam2 = thd.gam2
    Wc_i = np.array([thd.Wc_i[k] for k in range(nrv)])
    out = np.zeros(n + (nv,))
    others = [a for a in range(3) if a != d]
    for q1 in range(n[others[0]]):
        for q2 in range(n[others[1]]):
            idx = [0, 0, 0]
            idx[d] = sc
            idx[others[0]] = ng + q1
            idx[others[1]] = ng + q2
            p = tuple(idx)
            rho_i = 1.0 / v[p + (0,)]
            uc = [v[p + (1 + a,)] * rho_i for a in range(3)]
            P = v[p + (0,)] * T[p] * Wi[p]
            gam = 1.0 / (1.0 - gam2 * Wi[p] / cp[p])
            cs = np.sqrt(gam * P * rho_i)
            Y = v[p][5:] * rho_i
            psi = -ha[p] + (gam / (gam - 1.0)) * T[p] * Wc_i
            q = 0.5 * sum(u * u for u in uc)
            ht = float(np.dot(ha[p], Y)) + q
            b2 = (gam - 1.0) / cs ** 2
            b1 = b2 * q
            xi = b1 - b2 * ht
            el, er = char_matrices(d, uc, Y, psi, ht, q, cs, b1, b2, xi)
            un = uc[d]
            lam = np.array([un - cs, un, un + cs] + [un] * (nv - 3))
            Ls = np.maximum(lam, 0.0) if hi else np.minimum(lam, 0.0)
            dw = np.zeros(nv)
            for st_ in range(2 * ng - 1):
                j = list(p)
                j[d] = sc - st_ if hi else sc + st_
                dw += (-CNR[st_] if hi else CNR[st_]) * v[tuple(j)]
            df = er @ (Ls * (el @ dw)) * dxi[d][sc]
            o = [0, 0, 0]
            o[d] = sc - ng
            o[others[0]] = q1
            o[others[1]] = q2
            out[tuple(o)] = df
    return out


@pytest.mark.parametrize("species,blob", [("o2n2", 0.0), ("h2air9", 0.02)])
def test_characteristic_vectors_are_inverse(species, blob):
    """The dense characteristic vectors of the restatement satisfy L R = I
    at every boundary state (the property the projection relies on)."""
    cfg, thd, dxi, st, orc = _case(species, blob=blob)
    v, T, Wi, cp, ha = st["v"], st["T"], st["W_i"], st["cp"], st["ha"]
    nrv = cfg.nrv
    Wc_i = np.array([thd.Wc_i[k] for k in range(nrv)])
    p = (NG, NG + 4, NG + 3)
    for d in range(3):
        rho_i = 1.0 / v[p + (0,)]
        uc = [v[p + (1 + a,)] * rho_i + 0.1 * (a + 1) for a in range(3)]
        gam = 1.0 / (1.0 - thd.gam2 * Wi[p] / cp[p])
        cs = np.sqrt(gam * v[p + (0,)] * T[p] * Wi[p] * rho_i)
        Y = v[p][5:] * rho_i
        psi = -ha[p] + (gam / (gam - 1.0)) * T[p] * Wc_i
        q = 0.5 * sum(u * u for u in uc)
        ht = float(np.dot(ha[p], Y)) + q
        b2 = (gam - 1.0) / cs ** 2
        el, er = char_matrices(d, uc, Y, psi, ht, q, cs, b2 * q, b2, b2 * q - b2 * ht)
        assert np.abs(el @ er - np.eye(5 + nrv)).max() < 1e-9


@pytest.mark.parametrize("species,blob,faces,ng", [("o2n2", 0.0, "xy", 3), ("h2air9", 0.02, "xyz", 3),
                                                    ("o2n2", 0.0, "xyz", 4)])
def test_oracle_nr_term_matches_numpy(species, blob, faces, ng):
    """NR_boundaries of the oracle = the numpy restatement, summed over the
    non-reflecting faces in the order W..F, to 1e-13 of each variable; ng = 3
    and 4 (five and seven cnr weights)."""
    cfg, thd, dxi, st, orc = _case(species, faces, blob, ng)
    nv = 5 + cfg.nrv
    fl = np.zeros((cfg.nx, cfg.ny, cfg.nz, nv), order="F")
    orc.nr_flux(st, fl)
    ref = np.zeros_like(fl)
    for f in range(6):
        if cfg.bc[f] == BC_NOREFLECTION:
            ref += nr_term(st, thd, dxi, cfg, f)
    assert np.abs(ref).max() > 0
    err = W.normwise(fl, ref)
    assert np.all(err <= 1e-13), err


def test_ghosts_hold_ten_times_the_boundary_state():
    """bc_noreflection: each ghost layer of a non-reflecting face holds the
    boundary point's conserved variables times 10 (interior face range):
    density, momentum and energy exactly; the partial densities after the
    ghost's force_sumY, to rounding."""
    cfg, thd, dxi, st, orc = _case("o2n2", "xy")
    v = st["v"]
    ng = NG
    inner = slice(ng, -ng)

    def same(ghost, bnd):
        assert np.array_equal(ghost[..., :5], 10.0 * bnd[..., :5])
        assert np.allclose(ghost[..., 5:], 10.0 * bnd[..., 5:], rtol=1e-14, atol=0.0)

    for g in range(1, ng + 1):
        same(v[ng - g, inner, inner], v[ng, inner, inner])
        same(v[-ng - 1 + g, inner, inner], v[-ng - 1, inner, inner])
        same(v[inner, ng - g, inner], v[inner, ng, inner])
        same(v[inner, -ng - 1 + g, inner], v[inner, -ng - 1, inner])
    # temperature and composition of the ghost are the boundary point's
    assert np.allclose(st["T"][0, inner, inner], st["T"][ng, inner, inner], rtol=1e-10)


def test_euler_sweep_drops_the_boundary_points():
    """fl_W = fl_E = 0: the x sweep writes 0 at i = 1 and i = nx of a box
    with non-reflecting x faces; interior points keep their difference."""
    cfg, thd, dxi, st, orc = _case("o2n2", "x")
    nv = 5 + cfg.nrv
    fl = np.zeros((cfg.nx, cfg.ny, cfg.nz, nv), order="F")
    orc.euler_flux(st, 0, fl)
    assert np.all(fl[0] == 0.0) and np.all(fl[-1] == 0.0)
    assert np.abs(fl[1:-1]).max() > 0
    fy = np.zeros_like(fl)
    orc.euler_flux(st, 1, fy)   # y is periodic here: nothing dropped
    assert np.abs(fy[:, 0]).max() > 0


def test_rk3_with_non_reflecting_faces_stays_finite():
    """Three RK3 steps of the pulse with non-reflecting x and y faces run on
    the oracle (the full stage: sweeps, viscous fluxes, NR_boundaries,
    update, ghost closure) and keep a positive density."""
    cfg, thd, dxi, st, orc = _case("o2n2", "xy")
    for _ in range(3):
        dt4, dt = orc.timestep(st)
        orc.rk3(st, dt, 0.0)
    v = st["v"][NG:-NG, NG:-NG, NG:-NG]
    assert np.all(np.isfinite(v)) and v[..., 0].min() > 0


def test_cnr_weights_of_the_reference():
    """wenopar's cnr: the seven weights (ng = 4) are the 6th-order one-sided
    first derivative and sum to 0; for ng = 3 the reference keeps the first
    five, which sum to -31/30, so the term it adds is not zero on a uniform
    state.  Both are kept."""
    assert abs(CNR.sum()) < 1e-14
    assert abs(CNR[:5].sum() + 31.0 / 30.0) < 1e-14
    x = np.arange(7.0)
    assert abs(np.dot(CNR, x) - 1.0) < 1e-13 and abs(np.dot(CNR, x ** 6) - 0.0) < 1e-9


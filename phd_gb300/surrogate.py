"""Learned chemistry surrogate (host side).

A 12 -> 4 x 256 (GELU) -> 10 MLP replaces, per cell, the chemistry increment
that reaction_dvode (module_reaction.f90:102-321) computes with DVODE.  It
runs in BF16 with FP32 accumulation on the tensor cores (libizem_gpu.so,
izem_mlp_*), is trained on the GPU by the library's forward, backward and
Adam kernels on samples labelled by the library's own FP64 BDF integrator
(izem_gpu_psr_batch), and is used behind an error gate that sends rejected
cells back to that integrator (izem_gpu_psr_batch_mlp).

Features (same formula as the device featurisation kernel):
    T [K], ln p [atm], ln(max(Y_k, 0) + 1e-10) for the 9 species, ln dt [s]
Targets: dY_k (9 species) and dT [K] over dt.
"""
import ctypes as C

import numpy as np

from .capi import IzemMech
from .izem import IzemError, load_library, psr_batch
from .thd import load_species

IN, OUT, H = 12, 10, 256
LIN = [16, H, H, H, H]
LOUT = [H, H, H, H, 16]
NL = 5

RU = 8.314510e7
PATM = 1.01325e6


def _bind(lib):
    if getattr(lib, "_mlp_bound", False):
        return lib
    P = C.c_void_p
    fpp = C.POINTER(C.POINTER(C.c_float))
    sig = {
        "izem_mlp_create": (C.c_int, [C.POINTER(P)]),
        "izem_mlp_destroy": (None, [P]),
        "izem_mlp_set_params": (C.c_int, [P, fpp, fpp]),
        "izem_mlp_get_params": (C.c_int, [P, fpp, fpp]),
        "izem_mlp_set_norm": (C.c_int, [P, C.POINTER(C.c_float)]),
        "izem_mlp_set_residual": (C.c_int, [P, C.c_int]),
        "izem_gpu_reactor_rhs": (C.c_int, [C.POINTER(IzemMech), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_int]),
        "izem_mlp_forward": (C.c_int, [P, C.c_int, C.c_void_p, C.c_void_p]),
        "izem_mlp_fallback_cells": (C.c_int, [P, C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
        "izem_mlp_grads": (C.c_int, [P, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(C.c_double), fpp, fpp]),
        "izem_mlp_train": (C.c_int, [P, C.c_longlong, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float,
                                     C.c_uint, C.c_void_p]),
        "izem_gpu_psr_batch_mlp": (C.c_int, [P, P, C.POINTER(IzemMech), C.c_int, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                             C.c_void_p, C.c_void_p, C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    lib._mlp_bound = True
    return lib


def features(T, rho, Y, dt, wt):
    """Raw (un-normalised) surrogate inputs, shape (n, 12)."""
    Yc = np.maximum(Y, 0.0)
    p_atm = rho * RU * T * (Yc / wt).sum(axis=1) / PATM
    f = np.empty((len(T), IN))
    f[:, 0] = T
    f[:, 1] = np.log(p_atm)
    f[:, 2:11] = np.log(Yc + 1e-10)
    f[:, 11] = np.log(dt)
    return f


def he_init(seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    W, b = [], []
    for l in range(NL):
        fan_in = IN if l == 0 else H
        w = np.zeros((LIN[l], LOUT[l]), dtype=np.float32)
        rows = IN if l == 0 else LIN[l]
        cols = OUT if l == NL - 1 else LOUT[l]
        w[:rows, :cols] = rng.standard_normal((rows, cols)) * np.sqrt(2.0 / fan_in)
        W.append(w)
        b.append(np.zeros(LOUT[l], dtype=np.float32))
    return W, b


class Surrogate:
    """Device MLP handle (izem_mlp) with its normalisation."""

    def __init__(self, seed=20261203):
        self.lib = _bind(load_library())
        h = C.c_void_p()
        rc = self.lib.izem_mlp_create(C.byref(h))
        if rc:
            raise IzemError(rc, "izem_mlp_create")
        self.h = h
        self.residual = False
        W, b = he_init(seed)
        self.set_params(W, b)
        self.norm = np.concatenate([np.zeros(IN), np.ones(IN), np.zeros(OUT), np.ones(OUT)]).astype(np.float32)
        self.set_norm(self.norm)

    def close(self):
        if getattr(self, "h", None):
            self.lib.izem_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    @staticmethod
    def _pp(arrs):
        t = (C.POINTER(C.c_float) * len(arrs))(*[a.ctypes.data_as(C.POINTER(C.c_float)) for a in arrs])
        return t

    def set_params(self, W, b):
        self._W = [np.ascontiguousarray(w, dtype=np.float32) for w in W]
        self._b = [np.ascontiguousarray(x, dtype=np.float32) for x in b]
        rc = self.lib.izem_mlp_set_params(self.h, self._pp(self._W), self._pp(self._b))
        if rc:
            raise IzemError(rc, "izem_mlp_set_params")

    def get_params(self):
        W = [np.zeros((LIN[l], LOUT[l]), dtype=np.float32) for l in range(NL)]
        b = [np.zeros(LOUT[l], dtype=np.float32) for l in range(NL)]
        rc = self.lib.izem_mlp_get_params(self.h, self._pp(W), self._pp(b))
        if rc:
            raise IzemError(rc, "izem_mlp_get_params")
        return W, b

    def set_residual(self, residual):
        """The network predicts the increment minus dt f(y0) (see
        explicit_increment); the gated step adds dt f(y0) back."""
        self.residual = bool(residual)
        rc = self.lib.izem_mlp_set_residual(self.h, int(self.residual))
        if rc:
            raise IzemError(rc, "izem_mlp_set_residual")

    def set_norm(self, norm):
        self.norm = np.ascontiguousarray(norm, dtype=np.float32)
        self.lib.izem_mlp_set_norm(self.h, self.norm.ctypes.data_as(C.POINTER(C.c_float)))

    def fit_norm(self, X, Yt):
        n = np.concatenate([X.mean(0), X.std(0) + 1e-6, Yt.mean(0), Yt.std(0) + 1e-12]).astype(np.float32)
        self.set_norm(n)
        return n

    def normalise(self, X, Yt=None):
        nx = ((X - self.norm[:IN]) / self.norm[IN:2 * IN]).astype(np.float32)
        if Yt is None:
            return np.ascontiguousarray(nx)
        ny = ((Yt - self.norm[2 * IN:2 * IN + OUT]) / self.norm[2 * IN + OUT:]).astype(np.float32)
        return np.ascontiguousarray(nx), np.ascontiguousarray(ny)

    def forward(self, xn):
        xn = np.ascontiguousarray(xn, dtype=np.float32)
        y = np.zeros((len(xn), OUT), dtype=np.float32)
        rc = self.lib.izem_mlp_forward(self.h, len(xn), xn.ctypes.data, y.ctypes.data)
        if rc:
            raise IzemError(rc, "izem_mlp_forward")
        return y

    def grads(self, xn, tn):
        xn = np.ascontiguousarray(xn, dtype=np.float32)
        tn = np.ascontiguousarray(tn, dtype=np.float32)
        gW = [np.zeros((LIN[l], LOUT[l]), dtype=np.float32) for l in range(NL)]
        gb = [np.zeros(LOUT[l], dtype=np.float32) for l in range(NL)]
        loss = C.c_double()
        rc = self.lib.izem_mlp_grads(self.h, len(xn), xn.ctypes.data, tn.ctypes.data, C.byref(loss),
                                     self._pp(gW), self._pp(gb))
        if rc:
            raise IzemError(rc, "izem_mlp_grads")
        return loss.value, gW, gb

    def train(self, xn, tn, epochs=20, batch=4096, lr=1e-3, seed=7):
        xn = np.ascontiguousarray(xn, dtype=np.float32)
        tn = np.ascontiguousarray(tn, dtype=np.float32)
        losses = np.zeros(epochs)
        rc = self.lib.izem_mlp_train(self.h, len(xn), xn.ctypes.data, tn.ctypes.data, 0, epochs, batch, lr, seed,
                                     losses.ctypes.data)
        if rc:
            raise IzemError(rc, "izem_mlp_train")
        return losses

    def chem_step(self, mech, T, rho, Y, dt, gate, partner=None):
        """Surrogate + gate + BDF fallback on independent reactors (host
        arrays updated in place).  partner: a second Surrogate; the
        prediction is the mean of the two and cells where their dT disagree
        are rejected.  Returns dict with fallback count, times and the raw
        predicted dT."""
        kncf = np.ascontiguousarray(np.array(load_species("h2air9")["kncf"], dtype=np.int32))
        g10 = gate10(gate)
        dTp = np.zeros(len(T))
        st3 = np.zeros(3, dtype=np.int32)
        ms2 = np.zeros(2, dtype=np.float32)
        rc = self.lib.izem_gpu_psr_batch_mlp(self.h, partner.h if partner is not None else None, C.byref(mech),
                                             len(T), T.ctypes.data, rho.ctypes.data,
                                             Y.ctypes.data, dt.ctypes.data, 0, g10.ctypes.data, kncf.ctypes.data,
                                             kncf.shape[1], dTp.ctypes.data, st3.ctypes.data, ms2.ctypes.data)
        if rc:
            raise IzemError(rc, "izem_gpu_psr_batch_mlp")
        return {"fallback": int(st3[0]), "max_steps": int(st3[1]), "failed": int(st3[2]), "ms": float(ms2[0]),
                "ms_mlp": float(ms2[1]), "dT_pred": dTp}

    def fallback_cells(self):
        """Sorted indices of the cells the last chem_step / chem_step_device
        on this network sent to the BDF integrator."""
        cnt = C.c_int()
        rc = self.lib.izem_mlp_fallback_cells(self.h, None, 0, C.byref(cnt))
        if rc:
            raise IzemError(rc, "izem_mlp_fallback_cells")
        out = np.zeros(max(cnt.value, 1), dtype=np.int32)
        rc = self.lib.izem_mlp_fallback_cells(self.h, out.ctypes.data, cnt.value, C.byref(cnt))
        if rc:
            raise IzemError(rc, "izem_mlp_fallback_cells")
        return np.sort(out[:cnt.value])

    def chem_step_device(self, mech, n, T, rho, Y, dt, gate, partner=None):
        """chem_step on arrays already on the device (torch CUDA tensors:
        T, rho, dt (n), Y (n, 9) row-major), updated in place; the caller's
        work on them must be complete.  Returns the same dictionary without
        dT_pred."""
        kncf = np.ascontiguousarray(np.array(load_species("h2air9")["kncf"], dtype=np.int32))
        g10 = gate10(gate)
        st3 = np.zeros(3, dtype=np.int32)
        ms2 = np.zeros(2, dtype=np.float32)
        rc = self.lib.izem_gpu_psr_batch_mlp(self.h, partner.h if partner is not None else None, C.byref(mech), n,
                                             T.data_ptr(), rho.data_ptr(), Y.data_ptr(), dt.data_ptr(), 1,
                                             g10.ctypes.data, kncf.ctypes.data, kncf.shape[1], None,
                                             st3.ctypes.data, ms2.ctypes.data)
        if rc:
            raise IzemError(rc, "izem_gpu_psr_batch_mlp")
        return {"fallback": int(st3[0]), "max_steps": int(st3[1]), "failed": int(st3[2]), "ms": float(ms2[0]),
                "ms_mlp": float(ms2[1])}


# Tmin, Tmax, dtmin, dtmax, tol_el, tol_T_abs [K], tol_T_rel, tol_ens_abs [K], tol_ens_rel,
# dT_cap [K] (largest predicted |dT| accepted)
DEFAULT_GATE = (800.0, 2400.0, 1e-8, 1e-6, 2e-3, 2.0, 0.003, 1.0, 0.002, float("inf"))
# tighter energy-consistency and agreement tolerances: more cells go to BDF
STRICT_GATE = (800.0, 2400.0, 1e-8, 1e-6, 2e-3, 0.5, 0.001, 0.2, 0.0003, float("inf"))


def gate10(gate):
    """The error gate as the 10 doubles the library reads; a 9-value gate
    (without the dT cap) is accepted and gets no cap."""
    g = [float(x) for x in gate]
    if len(g) == 9:
        g.append(float("inf"))
    if len(g) != 10:
        raise ValueError("the error gate has 10 values (Tmin, Tmax, dtmin, dtmax, tol_el, tol_T_abs, tol_T_rel, "
                         "tol_ens_abs, tol_ens_rel, dT_cap)")
    return np.ascontiguousarray(np.array(g, dtype=np.float64))


CAP_LADDER = (10.0, 20.0, 30.0, 50.0, 75.0, 100.0, 150.0, 200.0, 300.0, 400.0, 800.0)
# with a fixed, short step the increments are small and so is the cap
CAP_LADDER_FINE = (0.5, 1.0, 2.0, 3.0, 5.0, 7.5) + CAP_LADDER
ABS_SCALE_LADDER = (1.0, 0.5, 0.25, 0.1, 0.05)


def calibrate_cap(nets, mech, gate=DEFAULT_GATE, n=1 << 20, seed=977, target=0.005, caps=CAP_LADDER, dt_s=None,
                  abs_scales=(1.0,)):
    """Choose the gate's cap on the predicted |dT| on held-out reactors: n
    reactors of the batched-chemistry distribution (another seed than the
    training and test sets; with dt_s, all of them over that one step, the
    step of the field the gate will serve) are labelled by the FP64 BDF
    integrator and run through the gated step without a cap; the cap is the
    largest value of `caps` for which every accepted cell whose predicted
    |dT| is at most the cap has an error within target x the largest |dT|
    of the set.  With several abs_scales (descending), the gate's absolute
    tolerances -- the energy-consistency one on dT and the two networks'
    agreement on dT -- are scaled by each in turn until a cap meets the
    target: over a short step the increments, and the error that these
    tolerances let through, are small.  Returns (gate, per-cap table)."""
    from .ics import batched_reactors
    T, rho, Y, dt = batched_reactors(n, seed=seed)
    if dt_s is not None:
        dt[:] = dt_s
    Tb, Yb = T.copy(), Y.copy()
    psr_batch(mech, Tb, rho.copy(), Yb, dt.copy())
    ref = Tb - T
    scale = float(np.abs(ref).max())
    g0 = list(gate10(gate))
    table, best, g = [], None, None
    for f in abs_scales:
        g = list(g0)
        g[5], g[7], g[9] = g0[5] * f, g0[7] * f, float("inf")
        Ts, Ys = T.copy(), Y.copy()
        r = nets[0].chem_step(mech, Ts, rho.copy(), Ys, dt.copy(), g, partner=nets[1] if len(nets) > 1 else None)
        err = np.abs((Ts - T) - ref)
        acc = np.ones(n, dtype=bool)
        acc[nets[0].fallback_cells()] = False
        pred = np.abs(r["dT_pred"])
        for cap in sorted(caps):
            keep = acc & (pred <= cap)
            worst = float(err[keep].max()) if keep.any() else 0.0
            table.append({"abs_scale": f, "cap_K": cap, "max_err_K": worst,
                          "rejected_frac": float((~keep).sum()) / n})
            if worst <= target * scale and (best is None or cap > best):
                best = cap
            elif worst > target * scale:
                break
        if best is not None:
            break
    g[9] = float(best if best is not None else min(caps))
    return tuple(g), {"cells": n, "seed": seed, "target_frac": target, "scale_K": scale, "table": table,
                      "dt_s": dt_s}


def train_ensemble(mech, n=1 << 22, seed=31, epochs=30, batch=4096, lr=1e-3, members=2, log=None):
    """Train `members` networks on n reactors labelled by the GPU BDF
    integrator (same samples, different initialisations and shuffles), with
    a step-decayed learning rate.  Returns the list of Surrogates."""
    X, Yt = training_set(mech, n, seed)
    nets = []
    for q in range(members):
        s = Surrogate(seed=seed + 1000 * (q + 1))
        s.fit_norm(X, Yt)
        xn, tn = s.normalise(X, Yt)
        hist = []
        for stage, f in enumerate((1.0, 0.3, 0.1)):
            ep = max(1, epochs // 3)
            hist += list(s.train(xn, tn, epochs=ep, batch=batch, lr=lr * f, seed=seed + 17 * q + stage))
        if log is not None:
            log.append({"member": q, "loss": hist})
        nets.append(s)
    return nets


def training_set(mech, n, seed):
    """n reactors from the batched-chemistry distribution labelled by the
    FP64 BDF integrator on the GPU: returns raw features and targets."""
    from .ics import batched_reactors
    T, rho, Y, dt = batched_reactors(n, seed=seed)
    wt = np.array([mech.wt[k] for k in range(mech.kk)])
    X = features(T, rho, Y, dt, wt)
    T1, Y1 = T.copy(), Y.copy()
    psr_batch(mech, T1, rho.copy(), Y1, dt.copy())
    Yt = np.concatenate([Y1 - Y, (T1 - T)[:, None]], axis=1)
    return X, Yt


def reaction_window(cfg):
    """The reaction_dvode window (module_reaction.f90:155-171) as slices of
    the ghosted arrays: interior indices ng+1 .. n-ng-1 on every axis, the
    z bound taken with min(ny, ...) as the reference writes it."""
    ng = cfg.ng
    fx, fy = min(cfg.nx, cfg.nx - ng - 1), min(cfg.ny, cfg.ny - ng - 1)
    fz = min(cfg.ny, cfg.nz - ng - 1)
    return (slice(2 * ng, fx + ng), slice(2 * ng, fy + ng), slice(2 * ng, fz + ng))


def window_reactors(g, dt):
    """The reactors of one chemistry half step of an IzemGPU block: the
    reaction window (reaction_window) in physical units, i fastest.
    Returns T [K], rho [g/cm^3], Y (n, nrv), dt [s] (n values)."""
    cfg, adi = g.cfg, g.adi
    st = g.download()
    sl = reaction_window(cfg)
    v = st["v"][sl]
    rho = v[..., 0]
    n = rho.size
    Y = (v[..., 5:5 + cfg.nrv] / rho[..., None]).reshape(n, cfg.nrv, order="F")
    T = (st["T"][sl] * adi.t_ref).reshape(n, order="F")
    rho_c = (rho * adi.rho_ref * 1e-3).reshape(n, order="F")
    return (np.ascontiguousarray(T), np.ascontiguousarray(rho_c), np.ascontiguousarray(Y),
            np.full(n, dt * adi.time_ref))


def flow_reactors(g, mech, dt, n_max=1 << 20, spread=0.5, seed=5, age=0.0):
    """Reactors drawn from a flow block as the surrogate will meet them: its
    window reactors with the half step scaled by 10**U[-spread, spread].
    With age > 0, three quarters of them are first advanced by the FP64 BDF
    integrator over U[0, age] half steps, so that the set also holds the
    compositions the window reaches in later steps (the radical pool grows
    during the induction).  Returns T [K], rho [g/cm^3], Y (n, 9), dt [s]."""
    T, rho, Y, dtp = window_reactors(g, dt)
    rng = np.random.Generator(np.random.PCG64(seed))
    idx = rng.choice(len(T), size=min(n_max, len(T)), replace=False) if len(T) > n_max else np.arange(len(T))
    T, rho, Y, dtp = T[idx].copy(), rho[idx].copy(), np.ascontiguousarray(Y[idx]), dtp[idx].copy()
    if age > 0.0:
        a = rng.uniform(0.0, age, len(T))
        old = np.flatnonzero(rng.uniform(size=len(T)) >= 0.25)
        if len(old):
            Ta, Ya = T[old].copy(), np.ascontiguousarray(Y[old])
            psr_batch(mech, Ta, rho[old].copy(), Ya, dtp[old] * a[old])
            T[old], Y[old] = Ta, Ya
    dtp = dtp * 10.0 ** rng.uniform(-spread, spread, len(T))
    return T, rho, Y, dtp


def explicit_increment(mech, T, rho, Y, dt):
    """dt f(y0) in the target order (dY_1..dY_9, dT): the reactor
    right-hand side at the start state (izem_gpu_reactor_rhs) times dt."""
    lib = _bind(load_library())
    T = np.ascontiguousarray(T, dtype=np.float64)
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    z = np.zeros((len(T), mech.kk + 1))
    rc = lib.izem_gpu_reactor_rhs(C.byref(mech), len(T), T.ctypes.data, rho.ctypes.data, Y.ctypes.data, z.ctypes.data, 0)
    if rc:
        raise IzemError(rc, "izem_gpu_reactor_rhs")
    return np.concatenate([z[:, 1:], z[:, :1]], axis=1) * np.asarray(dt)[:, None]


def label(mech, T, rho, Y, dt, explicit=False):
    """FP64 BDF labels of reactors: raw features and targets (dY_k, dT);
    with explicit, also dt f(y0) (explicit_increment)."""
    wt = np.array([mech.wt[k] for k in range(mech.kk)])
    X = features(T, rho, Y, dt, wt)
    E = explicit_increment(mech, T, rho, Y, dt) if explicit else None
    T1, Y1 = T.copy(), Y.copy()
    psr_batch(mech, T1, rho.copy(), Y1, dt.copy())
    Yt = np.concatenate([Y1 - Y, (T1 - T)[:, None]], axis=1)
    return (X, Yt, E) if explicit else (X, Yt)


def flow_training_set(g, mech, dt, n_max=1 << 20, spread=0.5, seed=5, age=0.0):
    """flow_reactors labelled by the FP64 BDF integrator: raw features and
    targets."""
    return label(mech, *flow_reactors(g, mech, dt, n_max=n_max, spread=spread, seed=seed, age=age))


def train_on(X, Yt, members=2, seed=31, epochs=24, batch=4096, lr=1e-3, E=None):
    """Train `members` networks on raw features/targets (different
    initialisations and shuffles, step-decayed learning rate).  With E (the
    explicit increments dt f(y0)), the networks learn Yt - E and are marked
    residual: the gated step adds dt f(y0) back."""
    nets = []
    tgt = Yt if E is None else Yt - E
    for q in range(members):
        s = Surrogate(seed=seed + 1000 * (q + 1))
        s.set_residual(E is not None)
        s.fit_norm(X, tgt)
        xn, tn = s.normalise(X, tgt)
        for stage, f in enumerate((1.0, 0.3, 0.1)):
            s.train(xn, tn, epochs=max(1, epochs // 3), batch=batch, lr=lr * f, seed=seed + 17 * q + stage)
        nets.append(s)
    return nets


def flow_gate(X, Yt, dT_tol_frac=0.002):
    """Gate for a flow-trained surrogate: the envelope of its training
    temperatures and steps, element tolerance 2e-3, and temperature
    tolerances scaled by f = dT_tol_frac: energy consistency within
    f x (largest trained increment) + 5 f |dT|, agreement of the two
    networks within f/2 x that increment + 2.5 f |dT|."""
    scale = float(np.abs(Yt[:, -1]).max())
    dt = np.exp(X[:, 11])
    f = dT_tol_frac
    a = f * scale
    return (float(X[:, 0].min()), float(X[:, 0].max()), float(dt.min()), float(dt.max()), 2e-3, a, 5.0 * f, 0.5 * a,
            2.5 * f, float("inf"))


FLOW_TOL_LADDER = (0.00025, 0.0005, 0.00075, 0.001, 0.0015, 0.002, 0.003, 0.004, 0.008)


def calibrate_flow_gate(nets, mech, X, Yt, held, target=0.005, ladder=FLOW_TOL_LADDER):
    """Choose the flow gate's tolerance scale on held-out reactors (another
    draw from the same block, labelled by BDF): the largest f of `ladder`
    for which every accepted held-out cell's |dT| error is within
    target x the largest held-out |dT|.  held: (T, rho, Y, dt) raw
    reactors.  Returns (gate, table)."""
    T, rho, Y, dt = held
    Tb, Yb = T.copy(), Y.copy()
    psr_batch(mech, Tb, rho.copy(), Yb, dt.copy())
    ref = Tb - T
    scale = float(np.abs(ref).max())
    table, best = [], None
    for f in ladder:
        gate = flow_gate(X, Yt, f)
        Ts, Ys = T.copy(), Y.copy()
        r = nets[0].chem_step(mech, Ts, rho.copy(), Ys, dt.copy(), gate, partner=nets[1] if len(nets) > 1 else None)
        err = float(np.abs((Ts - T) - ref).max())
        table.append({"f": f, "max_err_frac": err / scale if scale > 0 else None,
                      "fallback_frac": r["fallback"] / len(T)})
        if err <= target * scale:
            best = f
        else:
            break
    return flow_gate(X, Yt, best if best is not None else ladder[0]), {"cells": len(T), "scale_K": scale,
                                                                        "target_frac": target, "table": table}

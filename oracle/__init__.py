"""CPU oracle of the IZEM hot path -- TEST INFRASTRUCTURE ONLY.

A ctypes wrapper over oracle/_build/libizem_oracle.so, the C++ restatement of
the reference Fortran routines (see izem_oracle.cpp).  Only the tests, the
smoke check and the CPU-baseline leg of bench.py may import this package; the
product library never calls it.
"""
import ctypes as C
import os

import numpy as np

from phd_gb300.capi import IzemAdi, IzemCfg, IzemEglib, IzemMech, IzemThd

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libizem_oracle.so")
_LIB = None
_dp = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)


def load():
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        from phd_gb300.build import build_oracle
        build_oracle()
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    sig = {
        "or_create": (P, [C.POINTER(IzemCfg), C.POINTER(IzemThd), C.POINTER(IzemAdi), _dp, _dp, _dp]),
        "or_destroy": (None, [P]),
        "or_set_sensor_xblocks": (C.c_int, [P, C.c_int]),
        "or_set_newton_xblocks": (C.c_int, [P, C.c_int]),
        "or_set_chem_skip": (C.c_int, [P, C.c_int, _dp, _dp, C.c_int, C.c_int]),
        "or_set_les": (C.c_int, [P, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]),
        "or_last_error": (C.c_int, [P, C.c_char_p, C.c_int]),
        "or_newton_it_max": (C.c_int, [P]),
        "or_cp_scalar": (None, [P, C.c_double, _dp, _dp]),
        "or_ha_scalar": (None, [P, C.c_double, _dp]),
        "or_shock_sensor": (C.c_int, [P, _dp, _dp, _dp, _u8p]),
        "or_euler_flux": (C.c_int, [P, C.c_int, _dp, _dp, _dp, _dp, _dp, _u8p, _dp]),
        "or_visc_flux": (C.c_int, [P, _dp, _dp, _dp, _dp, _dp, _dp]),
        "or_nr_flux": (C.c_int, [P, _dp, _dp, _dp, _dp, _dp, _dp]),
        "or_set_shock_sensor": (C.c_int, [P, C.c_int, C.c_double]),
        "or_prim_inv_var": (C.c_int, [P, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp]),
        "or_force_sumY": (C.c_int, [P, C.c_int, _dp]),
        "or_update_primitives": (C.c_int, [P, _dp, _dp, _dp, _dp, _dp]),
        "or_finalize_ic": (C.c_int, [P, _dp, _dp, _dp, _dp, _dp]),
        "or_rk3": (C.c_int, [P, C.c_double, C.c_double, _dp, _dp, _dp, _dp, _dp, _u8p]),
        "or_set_coords": (C.c_int, [P, _dp, _dp, _dp, C.c_double]),
        "or_set_jet": (C.c_int, [P, C.c_void_p]),
        "or_timestep": (C.c_int, [P, C.c_double, _dp, _dp, _dp, _dp, _dp, _dp]),
        "or_metrics_dscalar": (None, [C.c_int, C.c_int, _dp, _dp]),
        "or_chem_step": (C.c_int, [P, C.POINTER(IzemMech), C.c_double, C.c_double, _dp, _dp, _dp, _dp, _dp, _dp,
                                   C.POINTER(C.c_int)]),
        "or_psr_cells": (None, [C.POINTER(IzemMech), C.c_int, _dp, _dp, _dp, _dp, C.POINTER(C.c_int),
                                C.POINTER(C.c_int)]),
        "or_ck_fun": (None, [C.POINTER(IzemMech), C.c_double, _dp, _dp]),
        "or_set_eglib": (C.c_int, [P, C.POINTER(IzemEglib)]),
        "or_eg_point": (None, [C.POINTER(IzemEglib), C.c_double, _dp, _dp, _dp, C.c_double, _dp, _dp, _dp, _dp]),
        "or_ck_wdot": (None, [C.POINTER(IzemMech), C.c_double, C.c_double, _dp, _dp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def _p(a, kind=_dp):
    if a.ndim > 1 and not a.flags.f_contiguous:
        raise ValueError("oracle arrays must be Fortran-ordered")
    if (kind is _dp and a.dtype != np.float64) or (kind is _u8p and a.dtype != np.uint8):
        raise ValueError("oracle array has dtype %s" % a.dtype)
    return a.ctypes.data_as(kind)


class OracleError(RuntimeError):
    pass


def metrics_dscalar(coord, ng=3):
    lib = load()
    coord = np.ascontiguousarray(coord, dtype=np.float64)
    out = np.empty_like(coord)
    lib.or_metrics_dscalar(len(coord), ng, _p(coord), _p(out))
    return out


def psr_cells(mech, T, rho, Y, dt):
    """Independent constant-volume reactors (PSR per cell, DVODE restated),
    arrays updated in place; returns (istate, nsteps)."""
    lib = load()
    n = len(T)
    istate = np.zeros(n, dtype=np.int32)
    nsteps = np.zeros(n, dtype=np.int32)
    for a in (T, rho, dt):
        assert a.dtype == np.float64 and a.flags.c_contiguous
    assert Y.shape == (n, mech.kk) and Y.flags.c_contiguous
    lib.or_psr_cells(C.byref(mech), n, T.ctypes.data_as(_dp), rho.ctypes.data_as(_dp), Y.ctypes.data_as(_dp),
                     dt.ctypes.data_as(_dp), istate.ctypes.data_as(C.POINTER(C.c_int)),
                     nsteps.ctypes.data_as(C.POINTER(C.c_int)))
    return istate, nsteps


def eg_point(link, T, X, Y, cp, ww):
    """EGLIB precision 1 at one point (EGSPAR, EGSE2, EGSLCT2, EGSDR1):
    T [K], mole and mass fractions, species cp [erg/g/K], mean molar mass
    [g/mol] -> (eta [g/cm/s], lambda [erg/cm/s/K], chi, rho*D [l][m])."""
    lib = load()
    n = link.ns
    X, Y, cp = (np.ascontiguousarray(a, dtype=np.float64) for a in (X, Y, cp))
    eta, tc = C.c_double(), C.c_double()
    chit = np.zeros(n)
    D = np.zeros((n, n))
    lib.or_eg_point(C.byref(link), float(T), _p(X), _p(Y), _p(cp), float(ww), C.byref(eta), C.byref(tc), _p(chit),
                    D.ctypes.data_as(_dp))   # row-major [l][m]
    return eta.value, tc.value, chit, D


def ck_fun(mech, rho, z):
    lib = load()
    z = np.ascontiguousarray(z, dtype=np.float64)
    zp = np.zeros_like(z)
    lib.or_ck_fun(C.byref(mech), float(rho), z.ctypes.data_as(_dp), zp.ctypes.data_as(_dp))
    return zp


def ck_wdot(mech, rho, T, Y):
    lib = load()
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    w = np.zeros(mech.kk)
    lib.or_ck_wdot(C.byref(mech), float(rho), float(T), Y.ctypes.data_as(_dp), w.ctypes.data_as(_dp))
    return w


class Oracle:
    """Reference restatement operating in place on a host state dictionary
    {"v", "T", "W_i", "cp", "ha", "shock_sensor"} (Fortran-ordered arrays)."""

    def __init__(self, cfg, thd, adi, dx_i, dy_i, dz_i):
        self.lib = load()
        self.cfg = cfg
        self.nv = 5 + cfg.nrv
        self._grid = [np.ascontiguousarray(a, dtype=np.float64) for a in (dx_i, dy_i, dz_i)]
        self.h = self.lib.or_create(C.byref(cfg), C.byref(thd), C.byref(adi), *[_p(a) for a in self._grid])
        if not self.h:
            raise OracleError("unsupported configuration")

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.or_destroy(self.h)
            self.h = None

    def _rc(self, rc, what):
        if rc:
            buf = C.create_string_buffer(256)
            self.lib.or_last_error(self.h, buf, 256)
            raise OracleError("%s failed (%d): %s" % (what, rc, buf.value.decode()))

    def set_eglib(self, link):
        self._eglib = link
        self._rc(self.lib.or_set_eglib(self.h, C.byref(link)), "set_eglib")

    def set_newton_xblocks(self, nblk):
        """Test-only: each of nblk x-blocks runs its own Newton loop and
        stopping test (prim_inv_var per rank of an x-decomposition)."""
        self._rc(self.lib.or_set_newton_xblocks(self.h, int(nblk)), "set_newton_xblocks")

    def set_sensor_xblocks(self, nblk):
        """Emulate a run whose x direction was split into nblk MPI blocks:
        the shock sensor does not compare points across block edges."""
        self._rc(self.lib.or_set_sensor_xblocks(self.h, int(nblk)), "set_sensor_xblocks")

    def set_les(self, mu_sgs_factor=0.18, sc_sgs=0.7, pr_sgs=0.7, percent_weight_sgs=70.0, enable=True):
        """LES with the Smagorinsky closure: viscflux_eg_LES_xyz under EGLIB,
        viscflux_LES_xyz with the fitted transport."""
        self._rc(self.lib.or_set_les(self.h, int(bool(enable)), float(mu_sgs_factor), float(sc_sgs), float(pr_sgs),
                                     float(percent_weight_sgs)), "set_les")

    def set_chem_skip(self, y_fuel=None, y_oxidizer=None, index_h2=0, index_n2=0, enable=True):
        """dvodesimp: integrate only the cells that the skip test selects
        (pure fuel / oxidiser compositions, 0-based H2 and N2 indices)."""
        if not enable:
            self._rc(self.lib.or_set_chem_skip(self.h, 0, None, None, 0, 0), "set_chem_skip")
            return
        yf = np.ascontiguousarray(y_fuel, dtype=np.float64)
        yo = np.ascontiguousarray(y_oxidizer, dtype=np.float64)
        self._rc(self.lib.or_set_chem_skip(self.h, 1, _p(yf), _p(yo), int(index_h2), int(index_n2)), "set_chem_skip")

    def newton_warnings(self):
        return self.lib.or_last_error(self.h, None, 0)

    def newton_it_max(self):
        """Most Newton iterations any prim_inv_var call of this context ran."""
        return self.lib.or_newton_it_max(self.h)

    def cp_scalar(self, T, Y):
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        out = C.c_double()
        self.lib.or_cp_scalar(self.h, float(T), _p(Y), C.byref(out))
        return out.value

    def ha_scalar(self, T):
        out = np.zeros(self.cfg.nrv)
        self.lib.or_ha_scalar(self.h, float(T), _p(out))
        return out

    @staticmethod
    def _arrs(s):
        return s["v"], s["T"], s["W_i"], s["cp"], s["ha"]

    def shock_sensor(self, s):
        self._rc(self.lib.or_shock_sensor(self.h, _p(s["v"]), _p(s["T"]), _p(s["W_i"]), _p(s["shock_sensor"], _u8p)),
                 "shock_sensor")

    def euler_flux(self, s, direction, fl):
        v, T, W_i, cp, ha = self._arrs(s)
        self._rc(self.lib.or_euler_flux(self.h, direction, _p(v), _p(T), _p(W_i), _p(cp), _p(ha),
                                        _p(s["shock_sensor"], _u8p), _p(fl)), "euler_flux")

    def visc_flux(self, s, fl):
        v, T, W_i, cp, ha = self._arrs(s)
        self._rc(self.lib.or_visc_flux(self.h, _p(v), _p(T), _p(W_i), _p(cp), _p(ha), _p(fl)), "visc_flux")

    def set_shock_sensor(self, kind="ADAMSSHARIFF", ducros_treduc=0.2):
        """SHOCK_SENSOR_TYPE ("ADAMSSHARIFF" or "DUCROS") and DUCROS_TREDUC."""
        t = {"ADAMSSHARIFF": 0, "DUCROS": 1}[kind]
        self._rc(self.lib.or_set_shock_sensor(self.h, t, float(ducros_treduc)), "set_shock_sensor")

    def nr_flux(self, s, fl):
        """NR_boundaries: adds bc_noreflectionweno's term of every
        non-reflecting face to fl."""
        v, T, W_i, cp, ha = self._arrs(s)
        self._rc(self.lib.or_nr_flux(self.h, _p(v), _p(T), _p(W_i), _p(cp), _p(ha), _p(fl)), "nr_flux")

    def prim_inv_var(self, s, domain_id, err_mach=False):
        v, T, W_i, cp, ha = self._arrs(s)
        self._rc(self.lib.or_prim_inv_var(self.h, domain_id, int(err_mach), _p(v), _p(W_i), _p(T), _p(cp), _p(ha)),
                 "prim_inv_var")

    def update_primitives(self, s):
        v, T, W_i, cp, ha = self._arrs(s)
        self._rc(self.lib.or_update_primitives(self.h, _p(v), _p(T), _p(W_i), _p(cp), _p(ha)), "update_primitives")

    def finalize_ic(self, s):
        v, T, W_i, cp, ha = self._arrs(s)
        self._rc(self.lib.or_finalize_ic(self.h, _p(v), _p(T), _p(W_i), _p(cp), _p(ha)), "finalize_ic")

    def rk3(self, s, dt, time0=0.0):
        v, T, W_i, cp, ha = self._arrs(s)
        self._rc(self.lib.or_rk3(self.h, float(dt), float(time0), _p(v), _p(T), _p(W_i), _p(cp), _p(ha),
                                 _p(s["shock_sensor"], _u8p)), "rk3")

    def set_coords(self, x, y, z, lx):
        """Coordinates of the interior points (code units) and the domain
        length in x, for the jet boundaries."""
        xs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z)]
        self._keep_coords = xs
        self._rc(self.lib.or_set_coords(self.h, *[_p(a) for a in xs], float(lx)), "set_coords")

    def set_jet(self, jet):
        """Jet-face parameters (phd_gb300.capi.IzemJet)."""
        self._jet = jet
        self._rc(self.lib.or_set_jet(self.h, C.addressof(jet)), "set_jet")

    def chem_step(self, s, mech, dt, time=0.0):
        """reaction_selec over a half step dt at the given time (the jet
        faces' boundary closure reads both); returns DTmax [K]."""
        v, T, W_i, cp, ha = self._arrs(s)
        dtm = C.c_double()
        mx = C.c_int()
        self._rc(self.lib.or_chem_step(self.h, C.byref(mech), float(dt), float(time), _p(v), _p(T), _p(W_i), _p(cp),
                                       _p(ha), C.byref(dtm), C.byref(mx)), "chem_step")
        return dtm.value

    def timestep(self, s, DTmax=0.0, dtmin=1.0):
        v, T, W_i, cp, _ = self._arrs(s)
        dt4 = np.zeros(4)
        dtm = C.c_double(dtmin)
        self.lib.or_timestep(self.h, float(DTmax), _p(v), _p(T), _p(W_i), _p(cp), _p(dt4), C.byref(dtm))
        return dt4, dtm.value

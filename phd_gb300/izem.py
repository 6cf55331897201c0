"""Python host mirror of the IZEM hot-path interface over the C ABI.

The reference's Fortran driver calls, per time step (izem.f90:242-389):
``timestep`` (module_solver.f90:202), then ``rk3`` (module_solver.f90:694),
whose stages call the shock sensor, ``euler_LLF_x/_y/_z``
(module_weno.f90:537/1055/1595) and ``viscflux_xyz`` (module_viscflux.f90:
1660).  ``IzemGPU`` exposes the same operations, with the same argument
meaning and error behaviour (a non-zero status raises ``IzemError``; the
reference aborts through abort_mpi), on a device-resident state held by the
``libizem_gpu.so`` C library.  Arrays are numpy arrays in the reference's
Fortran layout: ``v`` has shape (nx+2ng, ny+2ng, nz+2ng, nv), order='F'.

There is no CPU fallback: if the CUDA library cannot be loaded this module
raises at import of the library.
"""
import ctypes as C
import os

import numpy as np

from . import capi
from .capi import IzemAdi, IzemCfg, IzemEglib, IzemJet, IzemMech, IzemThd

_LIB = None
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libizem_gpu.so")

_dp = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)


class IzemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (capi.ERR_NAMES.get(code, "error"), code, msg))
        self.code = code


def load_library(path=None):
    """Load the CUDA library (built by phd_gb300.build.build_gpu)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError("libizem_gpu.so is not built (%s); run __graft_entry__.build()" % path)
    lib = C.CDLL(path)
    P = C.c_void_p
    sig = {
        "izem_gpu_init": (C.c_int, [C.POINTER(IzemCfg), C.POINTER(IzemThd), C.POINTER(IzemAdi), C.POINTER(P)]),
        "izem_gpu_destroy": (None, [P]),
        "izem_gpu_last_error": (C.c_int, [P, C.c_char_p, C.c_int]),
        "izem_gpu_newton_stats": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int]),
        "izem_gpu_set_grid": (C.c_int, [P, _dp, _dp, _dp]),
        "izem_gpu_upload_state": (C.c_int, [P, _dp, _dp, _dp, _dp, _dp, _u8p]),
        "izem_gpu_download_state": (C.c_int, [P, _dp, _dp, _dp, _dp, _dp, _u8p]),
        "izem_gpu_download_flux": (C.c_int, [P, _dp]),
        "izem_gpu_zero_flux": (C.c_int, [P]),
        "izem_gpu_shock_sensor": (C.c_int, [P]),
        "izem_gpu_euler_flux": (C.c_int, [P, C.c_int]),
        "izem_gpu_visc_flux": (C.c_int, [P]),
        "izem_gpu_nr_flux": (C.c_int, [P]),
        "izem_gpu_set_shock_sensor": (C.c_int, [P, C.c_int, C.c_double]),
        "izem_gpu_update_primitives": (C.c_int, [P]),
        "izem_gpu_finalize_ic": (C.c_int, [P]),
        "izem_gpu_rk3": (C.c_int, [P, C.c_double, C.c_double]),
        "izem_gpu_timestep": (C.c_int, [P, C.c_double, _dp, _dp]),
        "izem_gpu_timer_start": (C.c_int, [P]),
        "izem_gpu_timer_stop": (C.c_int, [P, C.POINTER(C.c_float)]),
        "izem_gpu_set_kernel_timing": (C.c_int, [P, C.c_int]),
        "izem_gpu_kernel_times": (C.c_int, [P, C.c_int, C.c_char_p, C.c_int, C.POINTER(C.c_int), _dp,
                                            C.POINTER(C.c_int)]),
        "izem_gpu_synchronize": (C.c_int, [P]),
        "izem_metrics_dscalar": (C.c_int, [C.c_int, C.c_int, _dp, _dp]),
        "izem_gpu_set_mechanism": (C.c_int, [P, C.POINTER(IzemMech)]),
        "izem_gpu_chem_step": (C.c_int, [P, C.c_double, C.c_double, C.c_int, _dp]),
        "izem_gpu_chem_stats": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_ulonglong)]),
        "izem_gpu_psr_batch": (C.c_int, [C.POINTER(IzemMech), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_float)]),
        "izem_gpu_set_surrogate": (C.c_int, [P, P, P, _dp, C.POINTER(C.c_int), C.c_int]),
        "izem_gpu_set_eglib": (C.c_int, [P, C.POINTER(IzemEglib)]),
        "izem_gpu_autotune": (C.c_int, [P, C.c_double, C.c_char_p, C.c_int]),
        "izem_gpu_set_chem_variant": (C.c_int, [C.c_int]),
        "izem_gpu_chem_generated": (C.c_int, []),
        "izem_gpu_fp64_rate": (C.c_int, [_dp]),
        "izem_gpu_wait_selftest": (C.c_int, [C.c_int, C.POINTER(C.c_int)]),
        "izem_gpu_allow_chem_generated": (C.c_int, [C.c_int]),
        "izem_gpu_set_sensor_xblocks": (C.c_int, [P, C.c_int]),
        "izem_gpu_set_chem_skip": (C.c_int, [P, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
        "izem_gpu_set_les": (C.c_int, [P, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]),
        "izem_gpu_set_coords": (C.c_int, [P, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]),
        "izem_gpu_set_jet": (C.c_int, [P, C.POINTER(IzemJet)]),
        "izem_jet_reference": (None, [C.POINTER(IzemJet)]),
        "izem_gpu_chem_autotune": (C.c_int, [C.POINTER(IzemMech), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_int, C.c_char_p, C.c_int]),
        "izem_gpu_chem_surrogate_stats": (C.c_int, [P, C.POINTER(C.c_longlong), C.POINTER(C.c_int),
                                                    C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def _ptr(a, kind=_dp):
    return None if a is None else a.ctypes.data_as(kind)


def metrics_dscalar(coord, ng=3):
    """dscalar + inversion of the reference's metrics for one direction."""
    lib = load_library()
    coord = np.ascontiguousarray(coord, dtype=np.float64)
    out = np.empty_like(coord)
    rc = lib.izem_metrics_dscalar(len(coord), ng, _ptr(coord), _ptr(out))
    if rc:
        raise IzemError(rc, "izem_metrics_dscalar")
    return out


def psr_batch(mech, T, rho, Y, dt, device_ptrs=False):
    """Independent constant-volume reactors on the GPU (PSR_CHEMKIN per
    cell).  Host numpy arrays (T [K], rho [g/cm^3], Y (n, kk), dt [s]) are
    updated in place; returns (istate, nsteps, kernel_ms).  With
    device_ptrs the arguments are raw device addresses (ints) and the
    istate/nsteps outputs are not returned."""
    lib = load_library()
    ms = C.c_float()
    if device_ptrs:
        n = int(device_ptrs)
        rc = lib.izem_gpu_psr_batch(C.byref(mech), n, T, rho, Y, dt, None, None, 1, C.byref(ms))
        if rc:
            raise IzemError(rc, "izem_gpu_psr_batch")
        return None, None, ms.value
    n = len(T)
    for a in (T, rho, dt):
        if a.dtype != np.float64 or not a.flags.c_contiguous:
            raise ValueError("psr_batch arrays must be contiguous float64")
    if Y.shape != (n, mech.kk) or not Y.flags.c_contiguous:
        raise ValueError("Y must be a C-ordered (n, kk) array")
    istate = np.zeros(n, dtype=np.int32)
    nsteps = np.zeros(n, dtype=np.int32)
    rc = lib.izem_gpu_psr_batch(C.byref(mech), n, T.ctypes.data, rho.ctypes.data, Y.ctypes.data, dt.ctypes.data,
                                istate.ctypes.data, nsteps.ctypes.data, 0, C.byref(ms))
    if rc:
        raise IzemError(rc, "izem_gpu_psr_batch")
    return istate, nsteps, ms.value


def chem_autotune_device(mech, n, T, rho, Y, dt):
    """Choose the register-budget variant of the persistent chemistry
    kernels for independent reactors by timing each on the first
    min(n, 2^20) of them (device arrays as for psr_batch_device, left
    unchanged).  Returns the timings [ms] and the choice."""
    import json
    lib = load_library()
    buf = C.create_string_buffer(1024)
    rc = lib.izem_gpu_chem_autotune(C.byref(mech), n, T.data_ptr(), rho.data_ptr(), Y.data_ptr(), dt.data_ptr(), 1,
                                    buf, 1024)
    if rc:
        raise IzemError(rc, "izem_gpu_chem_autotune")
    return json.loads(buf.value.decode())


def psr_batch_device(mech, n, T, rho, Y, dt, istate=None, nsteps=None):
    """psr_batch on arrays already on the device: torch CUDA tensors (or raw
    device addresses) T (n), rho (n), Y (n, kk) row-major, dt (n); istate and
    nsteps (int32, n) are optional outputs.  The caller's work on these arrays
    must be complete (the library runs on its own stream and waits for it).
    Returns the kernel time in ms."""
    lib = load_library()

    def ptr(a):
        return None if a is None else (a if isinstance(a, int) else a.data_ptr())

    ms = C.c_float()
    rc = lib.izem_gpu_psr_batch(C.byref(mech), n, ptr(T), ptr(rho), ptr(Y), ptr(dt), ptr(istate), ptr(nsteps), 1,
                                C.byref(ms))
    if rc:
        raise IzemError(rc, "izem_gpu_psr_batch")
    return ms.value


class IzemGPU:
    """One device-resident block of the IZEM state (one GPU, one process)."""

    def __init__(self, cfg, thd, adi):
        self.lib = load_library()
        self.cfg, self.thd, self.adi = cfg, thd, adi
        self.nv = 5 + cfg.nrv
        self.ng = cfg.ng
        self.shape = (cfg.nx + 2 * cfg.ng, cfg.ny + 2 * cfg.ng, cfg.nz + 2 * cfg.ng)
        h = C.c_void_p()
        rc = self.lib.izem_gpu_init(C.byref(cfg), C.byref(thd), C.byref(adi), C.byref(h))
        if rc:
            raise IzemError(rc, "izem_gpu_init")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.izem_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc, what):
        if rc:
            buf = C.create_string_buffer(512)
            self.lib.izem_gpu_last_error(self.h, buf, 512)
            raise IzemError(rc, "%s: %s" % (what, buf.value.decode()))

    def newton_warnings(self):
        return self.lib.izem_gpu_last_error(self.h, None, 0)

    def newton_stats(self, reset=False):
        """(most Newton iterations of any sub-domain, solves that reached itmax)
        since the context was made or since the last reset."""
        it, unc = C.c_int(0), C.c_int(0)
        self._check(self.lib.izem_gpu_newton_stats(self.h, C.byref(it), C.byref(unc), int(bool(reset))),
                    "newton_stats")
        return it.value, unc.value

    # ---- state ----------------------------------------------------------
    def set_grid(self, dx_i, dy_i, dz_i):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (dx_i, dy_i, dz_i)]
        for a, n in zip(arrs, self.shape):
            if a.shape != (n,):
                raise ValueError("metric array has %s entries, expected %d" % (a.shape, n))
        self._grid = arrs
        self._check(self.lib.izem_gpu_set_grid(self.h, *[_ptr(a) for a in arrs]), "set_grid")

    def upload(self, v=None, T=None, W_i=None, cp=None, ha=None, shock_sensor=None):
        def prep(a, dt=np.float64):
            return None if a is None else np.asfortranarray(a, dtype=dt)
        v, T, W_i, cp, ha = (prep(a) for a in (v, T, W_i, cp, ha))
        ss = prep(shock_sensor, np.uint8)
        self._check(self.lib.izem_gpu_upload_state(self.h, _ptr(v), _ptr(T), _ptr(W_i), _ptr(cp), _ptr(ha),
                                                   _ptr(ss, _u8p)), "upload_state")

    def download(self, out=None):
        """The ghosted state as Fortran-ordered host arrays.  `out` (a dict
        like the one returned, e.g. in pinned memory) is filled in place
        instead of allocating new arrays."""
        gx, gy, gz = self.shape
        shapes = {"v": ((gx, gy, gz, self.nv), np.float64), "T": ((gx, gy, gz), np.float64),
                  "W_i": ((gx, gy, gz), np.float64), "cp": ((gx, gy, gz), np.float64),
                  "ha": ((gx, gy, gz, self.cfg.nrv), np.float64), "shock_sensor": ((gx, gy, gz), np.uint8)}
        arr = {}
        for k, (shp, dt) in shapes.items():
            a = None if out is None else out.get(k)
            if a is None:
                a = np.empty(shp, dtype=dt, order="F")
            elif a.shape != shp or a.dtype != dt or not a.flags.f_contiguous:
                raise ValueError("download: out[%r] must be a Fortran-ordered %s array of shape %s" % (k, dt, shp))
            arr[k] = a
        v, T, W_i, cp, ha, ss = (arr[k] for k in ("v", "T", "W_i", "cp", "ha", "shock_sensor"))
        self._check(self.lib.izem_gpu_download_state(self.h, _ptr(v), _ptr(T), _ptr(W_i), _ptr(cp), _ptr(ha),
                                                     _ptr(ss, _u8p)), "download_state")
        return {"v": v, "T": T, "W_i": W_i, "cp": cp, "ha": ha, "shock_sensor": ss}

    def flux(self):
        fl = np.empty((self.cfg.nx, self.cfg.ny, self.cfg.nz, self.nv), order="F")
        self._check(self.lib.izem_gpu_download_flux(self.h, _ptr(fl)), "download_flux")
        return fl

    def zero_flux(self):
        self._check(self.lib.izem_gpu_zero_flux(self.h), "zero_flux")

    # ---- reference operations ---------------------------------------------
    def shock_sensor(self):
        self._check(self.lib.izem_gpu_shock_sensor(self.h), "shock_sensor")

    def euler_LLF(self, direction):
        self._check(self.lib.izem_gpu_euler_flux(self.h, int(direction)), "euler_LLF")

    def euler_LLF_x(self):
        self.euler_LLF(0)

    def euler_LLF_y(self):
        self.euler_LLF(1)

    def euler_LLF_z(self):
        self.euler_LLF(2)

    def viscflux_xyz(self):
        self._check(self.lib.izem_gpu_visc_flux(self.h), "viscflux_xyz")

    def set_shock_sensor(self, kind="ADAMSSHARIFF", ducros_treduc=0.2):
        """SHOCK_SENSOR_TYPE ("ADAMSSHARIFF" or "DUCROS") and DUCROS_TREDUC
        (izem_gpu_set_shock_sensor)."""
        t = {"ADAMSSHARIFF": 0, "DUCROS": 1}[kind]
        self._check(self.lib.izem_gpu_set_shock_sensor(self.h, t, float(ducros_treduc)), "set_shock_sensor")

    def NR_boundaries(self):
        """bc_noreflectionweno on every non-reflecting face (adds to f)."""
        self._check(self.lib.izem_gpu_nr_flux(self.h), "NR_boundaries")

    def update_primitives(self):
        self._check(self.lib.izem_gpu_update_primitives(self.h), "update_primitives")

    def finalize_ic(self):
        self._check(self.lib.izem_gpu_finalize_ic(self.h), "finalize_ic")

    def rk3(self, dt, time0=0.0):
        self._check(self.lib.izem_gpu_rk3(self.h, float(dt), float(time0)), "rk3")

    def timestep(self, DTmax=0.0, dtmin=1.0):
        dt4 = np.zeros(4)
        dtm = C.c_double(dtmin)
        self._check(self.lib.izem_gpu_timestep(self.h, float(DTmax), _ptr(dt4), C.byref(dtm)), "timestep")
        return dt4, dtm.value

    def autotune(self, chem_dt=0.0):
        """Choose the thread blocks of the face-flux and viscous point kernels
        and (with chem_dt > 0 and a mechanism set) the register-budget
        variant of the persistent chemistry kernels by timing the candidates
        on the current state; returns the timings [ms] and choices."""
        import json
        buf = C.create_string_buffer(2048)
        self._check(self.lib.izem_gpu_autotune(self.h, float(chem_dt), buf, 2048), "autotune")
        return json.loads(buf.value.decode())

    def set_sensor_xblocks(self, nblk):
        """Reproduce a reference run decomposed into nblk MPI blocks along x:
        the shock sensor is not shared between blocks (izem_gpu_set_sensor_xblocks)."""
        self._check(self.lib.izem_gpu_set_sensor_xblocks(self.h, int(nblk)), "set_sensor_xblocks")

    def set_coords(self, x, y, z, lx):
        """Interior coordinates (code units) and Lx for the jet faces
        (izem_gpu_set_coords)."""
        xs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z)]
        self._check(self.lib.izem_gpu_set_coords(self.h, *[a.ctypes.data for a in xs], float(lx)), "set_coords")

    def set_jet(self, jet):
        """Jet-face parameters (capi.IzemJet; after set_coords)."""
        self._jet = jet
        self._check(self.lib.izem_gpu_set_jet(self.h, C.byref(jet)), "set_jet")

    def set_les(self, mu_sgs_factor=0.18, sc_sgs=0.7, pr_sgs=0.7, percent_weight_sgs=70.0, enable=True):
        """[IFLES] LES = T, MU_SGS_MODEL = SMAGORINSKY (izem_gpu_set_les):
        viscflux_eg_LES_xyz under EGLIB, viscflux_LES_xyz with the fitted
        transport; the deck defaults are the keyword defaults."""
        self._check(self.lib.izem_gpu_set_les(self.h, int(bool(enable)), float(mu_sgs_factor), float(sc_sgs),
                                              float(pr_sgs), float(percent_weight_sgs)), "set_les")

    def set_chem_skip(self, y_fuel=None, y_oxidizer=None, index_h2=0, index_n2=0, enable=True):
        """[REACTING] DVODESIMP (izem_gpu_set_chem_skip): chemistry mode 0
        integrates only the cells the skip test selects; y_fuel and
        y_oxidizer are the pure-stream mass fractions, index_h2 and index_n2
        0-based species indices.  enable=False integrates every cell again."""
        if not enable:
            self._check(self.lib.izem_gpu_set_chem_skip(self.h, 0, None, None, 0, 0), "set_chem_skip")
            return
        yf = np.ascontiguousarray(y_fuel, dtype=np.float64)
        yo = np.ascontiguousarray(y_oxidizer, dtype=np.float64)
        self._check(self.lib.izem_gpu_set_chem_skip(self.h, 1, yf.ctypes.data, yo.ctypes.data, int(index_h2),
                                                    int(index_n2)), "set_chem_skip")

    def set_chem_variant(self, v):
        """Pin the register-budget variant (0..4) of the persistent chemistry
        kernels, process-wide, without timing."""
        self._check(self.lib.izem_gpu_set_chem_variant(int(v)), "set_chem_variant")

    def set_eglib(self, link):
        """EGLIB linking data (phd_gb300.thd.eglib_link) for cfg.eglib = 1."""
        self._eglib = link
        self._check(self.lib.izem_gpu_set_eglib(self.h, C.byref(link)), "set_eglib")

    # ---- chemistry ----------------------------------------------------------
    def set_mechanism(self, mech):
        self._mech = mech
        self._check(self.lib.izem_gpu_set_mechanism(self.h, C.byref(mech)), "set_mechanism")

    def set_surrogate(self, net, partner=None, gate=None, kncf=None):
        """Learned chemistry for reaction_selec(mode=CHEM_MLP): a
        phd_gb300.surrogate.Surrogate (and optional partner network), the
        error gate (10 numbers, see surrogate.DEFAULT_GATE; 9 without the dT
        cap) and the element counts kncf[nrv][nele]."""
        from .surrogate import DEFAULT_GATE, gate10
        from .thd import load_species
        if kncf is None:
            kncf = load_species("h2air9")["kncf"]
        self._sur = (net, partner)
        self._gate = gate10(DEFAULT_GATE if gate is None else gate)
        self._kncf = np.ascontiguousarray(np.array(kncf, dtype=np.int32))
        self._check(self.lib.izem_gpu_set_surrogate(self.h, net.h, partner.h if partner is not None else None,
                                                    _ptr(self._gate), _ptr(self._kncf, C.POINTER(C.c_int)),
                                                    self._kncf.shape[1]), "set_surrogate")

    def surrogate_stats(self):
        """Last surrogate chemistry step: window cells, BDF fallback cells,
        total and network-only milliseconds."""
        n, fb, a, b = C.c_longlong(), C.c_int(), C.c_float(), C.c_float()
        self._check(self.lib.izem_gpu_chem_surrogate_stats(self.h, C.byref(n), C.byref(fb), C.byref(a), C.byref(b)),
                    "chem_surrogate_stats")
        return {"cells": n.value, "fallback": fb.value, "ms": a.value, "ms_network": b.value}

    def reaction_selec(self, dt, mode=0, time=0.0):
        """One Strang chemistry half step of length dt (code units) at the
        given time (the jet faces' boundary closure reads both); returns
        DTmax [K] (module_reaction.f90:47-100).  mode CHEM_BDF (0) integrates
        every cell with the BDF method, CHEM_MLP (1) uses the surrogate set by
        set_surrogate with BDF fallback."""
        d = C.c_double()
        self._check(self.lib.izem_gpu_chem_step(self.h, float(dt), float(time), int(mode), C.byref(d)),
                    "chem_step")
        return d.value

    def chem_stats(self):
        f, m, t = C.c_int(), C.c_int(), C.c_ulonglong()
        self._check(self.lib.izem_gpu_chem_stats(self.h, C.byref(f), C.byref(m), C.byref(t)), "chem_stats")
        return {"failed": f.value, "max_steps": m.value, "total_steps": t.value}

    # ---- timing -----------------------------------------------------------
    def timer_start(self):
        self._check(self.lib.izem_gpu_timer_start(self.h), "timer_start")

    def timer_stop(self):
        ms = C.c_float()
        self._check(self.lib.izem_gpu_timer_stop(self.h, C.byref(ms)), "timer_stop")
        return ms.value

    def set_kernel_timing(self, enable):
        self._check(self.lib.izem_gpu_set_kernel_timing(self.h, int(bool(enable))), "set_kernel_timing")

    def kernel_times(self):
        n = C.c_int()
        cap, nl = 64, 48
        names = C.create_string_buffer(cap * nl)
        launches = (C.c_int * cap)()
        ms = (C.c_double * cap)()
        self._check(self.lib.izem_gpu_kernel_times(self.h, cap, names, nl, launches, ms, C.byref(n)), "kernel_times")
        out = {}
        for q in range(min(n.value, cap)):
            nm = names.raw[q * nl:(q + 1) * nl].split(b"\0")[0].decode()
            out[nm] = (launches[q], ms[q])
        return out

    def synchronize(self):
        self._check(self.lib.izem_gpu_synchronize(self.h), "synchronize")


CHEM_BDF, CHEM_MLP = 0, 1


def fp64_rate():
    """FP64 FMA throughput of the current device in GFLOP/s
    (izem_gpu_fp64_rate)."""
    lib = load_library()
    out = np.zeros(1)
    rc = lib.izem_gpu_fp64_rate(out.ctypes.data_as(_dp))
    if rc:
        raise IzemError(rc, "izem_gpu_fp64_rate")
    return float(out[0])


def wait_selftest(polls=4096):
    """1 when a kernel polling an mbarrier that nothing arrives on gave up
    after `polls` polls (izem_gpu_wait_selftest)."""
    lib = load_library()
    out = C.c_int(-1)
    rc = lib.izem_gpu_wait_selftest(int(polls), C.byref(out))
    if rc:
        raise IzemError(rc, "izem_gpu_wait_selftest")
    return out.value


class TimeLoop:
    """One pass of the reference driver's main loop (izem.f90:252-281) over
    a device context:

    * ``timestep`` with the previous step's dtmin and the chemistry's DTmax
      (the CPR criterion dt_4(4) reads both);
    * with chemistry, the Strang sequence ``reaction_selec(dtmin/2)``,
      ``rk3(dtmin)`` from the current time, time += dtmin,
      ``reaction_selec(dtmin/2)``, whose DTmax feeds the next time step;
    * without chemistry, ``rk3(dtmin)`` and time += dtmin.

    The clipping of dtmin onto statistics times (:256-263) belongs to the
    caller, who may pass ``dt`` to impose a step.  ``fixed_dt`` (seconds) is
    the deck's FIXEDDT / DT: timestep then returns DT / time_ref for all
    four criteria without evaluating them (module_solver.f90:240-244).
    ``chem`` is the hook that runs a chemistry half step and returns DTmax;
    subclasses wrap it to log per-half-step statistics."""

    def __init__(self, solver, reaction, chem_mode=CHEM_BDF, time=0.0, fixed_dt=None):
        self.s = solver
        self.reaction = bool(reaction)
        self.mode = chem_mode
        self.time = float(time)
        self.dtmin = 1.0
        self.DTmax = 0.0
        self.dt4 = None
        self.fixed_dt = fixed_dt

    def chem(self, dt):
        return self.s.reaction_selec(dt, mode=self.mode, time=self.time)

    def timestep(self):
        if self.fixed_dt is not None:
            dtmin = float(self.fixed_dt) / self.s.adi.time_ref
            return np.full(4, dtmin), dtmin
        return self.s.timestep(DTmax=self.DTmax, dtmin=self.dtmin)

    def step(self, dt=None):
        self.dt4, dtmin = self.timestep()
        if dt is not None:
            dtmin = float(dt)
        if self.reaction:
            self.chem(0.5 * dtmin)
        self.s.rk3(dtmin, self.time)
        self.time += dtmin
        if self.reaction:
            self.DTmax = self.chem(0.5 * dtmin)
        self.dtmin = dtmin
        return dtmin

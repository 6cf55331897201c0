"""ctypes mirror of include/izem_gpu.h (structures and status codes).

The layout of every structure here must match the C header field for field;
tests/test_capi_layout.py checks the sizes against the compiled library.
"""
import ctypes as C

NSMAX = 10
NPOLY = 4

BC_PERIODIC = 0
BC_EXTRAPOLATION = 1
BC_INFLOWJET = 2
BC_NSCBC_OUT = 3
BC_NOREFLECTION = 4

OK = 0
ERR_ARG = 1
ERR_CUDA = 2
ERR_NEG_PRESSURE = 3
ERR_NEG_TEMPERATURE = 4
ERR_NAN = 5
ERR_CHEM = 6
ERR_TIMEOUT = 7
ERR_NOMEM = 8
ERR_STATE = 9
ERR_TOO_LARGE = 10

CHEM_BDF = 0
CHEM_MLP = 1

ERR_NAMES = {
    OK: "ok", ERR_ARG: "bad argument", ERR_CUDA: "CUDA error",
    ERR_NEG_PRESSURE: "negative pressure", ERR_NEG_TEMPERATURE: "negative temperature",
    ERR_NAN: "NaN in Newton temperature", ERR_CHEM: "stiff integrator failure",
    ERR_TIMEOUT: "device wait timed out", ERR_NOMEM: "out of device memory",
    ERR_STATE: "call out of order", ERR_TOO_LARGE: "above a fixed capacity",
}


class IzemCfg(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("ng", C.c_int), ("ndim", C.c_int), ("nrv", C.c_int),
        ("bc", C.c_int * 6),
        ("weno_avg", C.c_int),
        ("max_rel_weight", C.c_double),
        ("vis", C.c_int), ("eglib", C.c_int), ("forcesum", C.c_int),
        ("reaction", C.c_int), ("vis_dt", C.c_int),
        ("cfl", C.c_double), ("cflmin", C.c_double), ("cpr", C.c_double), ("fo", C.c_double),
        ("weno5_linear_fix", C.c_int),
    ]


class IzemThd(C.Structure):
    _fields_ = [
        ("nspc", C.c_int),
        ("gam2", C.c_double), ("tinf", C.c_double),
        ("pinf", C.c_double), ("p0", C.c_double),
        ("muinf", C.c_double), ("laminf", C.c_double),
        ("dinf", C.c_double * NSMAX),
        ("W", C.c_double * NSMAX), ("Wc", C.c_double * NSMAX), ("Wc_i", C.c_double * NSMAX),
        ("tpolymin", C.c_double * NSMAX), ("tpolymax", C.c_double * NSMAX),
        ("tpolylim", C.c_double * NSMAX),
        ("heatcap", ((C.c_double * 7) * 2) * NSMAX),
        ("cofd", ((C.c_double * NPOLY) * NSMAX) * NSMAX),
        ("coflam", (C.c_double * NPOLY) * NSMAX),
        ("cofeta", (C.c_double * NPOLY) * NSMAX),
    ]


MAXREAC = 32


class IzemMech(C.Structure):
    _fields_ = [
        ("kk", C.c_int), ("ii", C.c_int),
        ("ru", C.c_double), ("patm", C.c_double),
        ("wt", C.c_double * NSMAX), ("tmid", C.c_double * NSMAX),
        ("a", ((C.c_double * 7) * 2) * NSMAX),
        ("nuk", (C.c_int * 6) * MAXREAC), ("nu", (C.c_int * 6) * MAXREAC),
        ("par", (C.c_double * 3) * MAXREAC),
        ("rev", C.c_int * MAXREAC), ("rpar", (C.c_double * 3) * MAXREAC),
        ("thb", C.c_int * MAXREAC), ("eff", (C.c_double * NSMAX) * MAXREAC),
        ("fall", C.c_int * MAXREAC), ("low", (C.c_double * 3) * MAXREAC),
        ("troe", (C.c_double * 4) * MAXREAC),
        ("sri", (C.c_double * 5) * MAXREAC), ("kfal", C.c_int * MAXREAC),
        ("lt", (C.c_double * 2) * MAXREAC), ("rlt", (C.c_double * 2) * MAXREAC),
    ]


class IzemEglib(C.Structure):
    _fields_ = [
        ("ns", C.c_int), ("lin", C.c_int * NSMAX),
        ("wt", C.c_double * NSMAX), ("eps", C.c_double * NSMAX), ("sig", C.c_double * NSMAX),
        ("dip", C.c_double * NSMAX), ("pol", C.c_double * NSMAX), ("zrot", C.c_double * NSMAX),
        ("cofe", (C.c_double * 4) * NSMAX),
        ("cofd", ((C.c_double * 4) * NSMAX) * NSMAX),
    ]


class IzemAdi(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "gamma_inf", "re", "pr", "le", "ma", "sc", "sqgmr", "ggmopr",
        "t_ref", "l_ref", "r_ref", "w_ref", "cp_ref", "mu_ref", "c_inf", "u_ref", "time_ref",
        "rho_ref", "p_ref", "lbda_ref", "d_ref")]


class IzemJet(C.Structure):
    """izem_jet: parameters of the jet faces (SI units)."""
    _fields_ = [(n, C.c_double) for n in ("width", "ramp", "T_jet", "T_co", "p_jet", "p_co", "u_jet", "u_co",
                                          "y_fuel", "p_far", "turb")] + \
               [("planar", C.c_int), ("reserved", C.c_int), ("seed", C.c_ulonglong)]


def jet_reference():
    """The constants that bc_inflowjet and bc_nscbc_out hard-code
    (module_BCs.f90:1680-1700, 2390)."""
    return IzemJet(width=1e-3, ramp=1e-4, T_jet=1000.0, T_co=300.0, p_jet=101325.0 * 15.0, p_co=101325.0,
                   u_jet=0.0, u_co=20.0, y_fuel=1.0, p_far=94232.25, turb=0.0, planar=0, reserved=0, seed=0)

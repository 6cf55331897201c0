"""The C-ABI library loads and exports every entry point of include/*.h
(no device call is made: this runs without a GPU)."""
import ctypes as C
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:int|void|double|float|size_t)\s*\*?\s*(izem_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "izem_gpu_init" in names and "izem_gpu_rk3" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    from phd_gb300.build import build_gpu
    lib_path = build_gpu()
    lib = C.CDLL(lib_path)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layout_matches_header():
    from phd_gb300.build import build_gpu
    from phd_gb300.capi import IzemAdi, IzemCfg, IzemThd
    lib = C.CDLL(build_gpu())
    fn = lib.izem_abi_sizes
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(C.c_size_t)] * 3
    s = [C.c_size_t() for _ in range(3)]
    assert fn(*[C.byref(x) for x in s]) == 0
    assert [x.value for x in s] == [C.sizeof(IzemCfg), C.sizeof(IzemThd), C.sizeof(IzemAdi)]


@pytest.mark.parametrize("ng", [3, 4])
def test_host_metrics_match_oracle(ng):
    import numpy as np
    import oracle
    from phd_gb300.izem import metrics_dscalar
    from phd_gb300.build import build_gpu
    build_gpu()
    rng = np.random.Generator(np.random.PCG64(1))
    x = np.cumsum(0.5 + rng.random(40))
    assert np.array_equal(metrics_dscalar(x, ng), oracle.metrics_dscalar(x, ng))


def test_entry_points_reject_bad_arguments_before_any_device_call():
    """Argument checks come before any CUDA call, so they hold on a machine
    without a GPU: unsupported configurations, empty batches, unknown
    chemistry variants and missing pointers return IZEM_ERR_ARG (1)."""
    import numpy as np
    import oracle
    from phd_gb300 import ics
    from phd_gb300.capi import IzemMech
    from phd_gb300.izem import load_library
    lib = load_library()
    cfg, thd, adi, dxi, st, info = ics.tgv(8, lib_dscalar=oracle.metrics_dscalar)
    h = C.c_void_p()
    for field, bad in (("ng", 5), ("ndim", 2), ("nrv", 3)):
        good = getattr(cfg, field)
        setattr(cfg, field, bad)
        assert lib.izem_gpu_init(C.byref(cfg), C.byref(thd), C.byref(adi), C.byref(h)) == 1, field
        setattr(cfg, field, good)
    mech = IzemMech()
    mech.kk = 9
    one = np.zeros(9)
    p = one.ctypes.data_as(C.c_void_p)
    assert lib.izem_gpu_psr_batch(C.byref(mech), 0, p, p, p, p, None, None, 0, None) == 1
    mech.kk = 8
    assert lib.izem_gpu_psr_batch(C.byref(mech), 1, p, p, p, p, None, None, 0, None) == 1
    assert lib.izem_gpu_set_chem_variant(5) == 1 and lib.izem_gpu_set_chem_variant(-1) == 1
    assert lib.izem_gpu_chem_autotune(C.byref(mech), 0, p, p, p, p, 0, None, 0) == 1
    cnt = C.c_int()
    assert lib.izem_mlp_fallback_cells(None, None, 0, C.byref(cnt)) == 1
    assert lib.izem_gpu_set_chem_skip(None, 1, p, p, 0, 8) == 1
    lib.izem_gpu_set_les.argtypes = [C.c_void_p, C.c_int] + [C.c_double] * 4
    assert lib.izem_gpu_set_les(None, 1, 0.18, 0.7, 0.7, 70.0) == 1


def test_struct_layout_matches_a_c_compiler(tmp_path):
    """The ctypes mirrors of the header's structs have the sizes and member
    offsets a C compiler gives them (gcc on include/izem_gpu.h), including
    the mechanism's SRI and collider tables at its end."""
    import shutil
    import subprocess
    from phd_gb300.capi import IzemAdi, IzemCfg, IzemEglib, IzemMech, IzemThd
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    here = os.path.dirname(os.path.abspath(__file__))
    inc = os.path.join(os.path.dirname(here), "include")
    checks = [("izem_cfg", IzemCfg, ["ng", "bc", "cfl", "weno5_linear_fix"]),
              ("izem_thd", IzemThd, ["heatcap", "cofd", "cofeta"]),
              ("izem_adi", IzemAdi, ["time_ref", "d_ref"]),
              ("izem_eglib", IzemEglib, ["cofe", "cofd"]),
              ("izem_mech", IzemMech, ["a", "eff", "troe", "sri", "kfal", "lt", "rlt"])]
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "izem_gpu.h"', "int main(void) {"]
    for name, _, members in checks:
        lines.append('  printf("%%zu\\n", sizeof(%s));' % name)
        for mem in members:
            lines.append('  printf("%%zu\\n", offsetof(%s, %s));' % (name, mem))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    subprocess.check_call([gcc, "-std=c11", "-I", inc, "-o", exe, str(src)])
    got = [int(x) for x in subprocess.check_output([exe]).split()]
    want = []
    for _, cls, members in checks:
        want.append(C.sizeof(cls))
        want += [getattr(cls, mem).offset for mem in members]
    assert got == want


def test_chemistry_entry_points_refuse_bad_mechanism_tables():
    """A mechanism whose tables the kernels cannot evaluate is refused with
    IZEM_ERR_ARG before any device work: an unknown fall-off kind, a
    collider out of range, a zero SRI temperature.  The shipped mechanism
    passes the same check (the call then fails only for want of a device or
    succeeds on one)."""
    import numpy as np
    from phd_gb300.build import build_gpu
    from phd_gb300.capi import IzemMech
    from phd_gb300.mech import h2_mechanism
    lib = C.CDLL(build_gpu())
    fn = lib.izem_gpu_psr_batch
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(IzemMech), C.c_int] + [C.c_void_p] * 6 + [C.c_int, C.c_void_p]
    T, rho, dt = np.full(4, 1500.0), np.full(4, 1e-4), np.full(4, 1e-7)
    Y = np.zeros((4, 9))
    Y[:, 8] = 1.0

    def call(m):
        return fn(C.byref(m), 4, T.ctypes.data, rho.ctypes.data, Y.ctypes.data, dt.ctypes.data, None, None, 0, None)

    for edit in ("fall", "kfal", "sri", "nuk"):
        m = h2_mechanism()
        if edit == "fall":
            m.fall[3] = 5
        elif edit == "kfal":
            m.kfal[3] = 10
        elif edit == "sri":
            m.fall[3] = 2
            m.sri[3][2] = 0.0
        else:
            m.nuk[0][0] = 9
        assert call(m) == 1, edit   # IZEM_ERR_ARG
    assert call(h2_mechanism()) != 1

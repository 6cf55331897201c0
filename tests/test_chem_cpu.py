"""Chemistry oracle checks on the CPU: the CHEMKIN-format mechanism, the
restated DVODE against the real DVODE shipped in scipy (same algorithm,
MF = 22, same tolerances), element conservation of the reactor."""
import os

import numpy as np
import pytest

import oracle
import refdata
from phd_gb300 import ics
from phd_gb300.mech import h2_mechanism
from phd_gb300.thd import load_species


def test_mechanism_structure():
    m = h2_mechanism()
    assert (m.kk, m.ii) == (9, 12)
    assert sum(m.fall[i] > 1 for i in range(m.ii)) == 2          # two Troe fall-off reactions
    assert sum(m.rev[i] == 2 for i in range(m.ii)) == 6           # explicit reverse rates
    assert sum(m.thb[i] for i in range(m.ii)) == 4


def _elements(Y):
    sp = load_species("h2air9")
    W = np.array(sp["W_gmol"])
    kn = np.array(sp["kncf"], dtype=float)     # species x elements
    return (Y / W) @ kn


def test_reactor_conserves_elements_and_energy():
    m = h2_mechanism()
    T, rho, Y, dt = ics.batched_reactors(256, seed=11)
    e0 = _elements(Y)
    Y1 = Y.copy(); T1 = T.copy()
    ist, ns = oracle.psr_cells(m, T1, rho, Y1, dt)
    assert np.all(ist == 2)
    # BDF local errors are controlled at RTOL = 1e-6, ATOL = 1e-10 per species
    assert np.all(np.abs(_elements(Y1) - e0) <= 1e-6 * e0 + 1e-10)
    assert np.max(np.abs(Y1.sum(axis=1) - 1.0)) < 1e-6


def test_oracle_dvode_matches_scipy_dvode():
    scipy_integrate = pytest.importorskip("scipy.integrate")
    m = h2_mechanism()
    T, rho, Y, dt = ics.batched_reactors(24, seed=5)
    for q in range(len(T)):
        z0 = np.concatenate([[T[q]], Y[q]])
        r = scipy_integrate.ode(lambda t, z: oracle.ck_fun(m, rho[q], z))
        r.set_integrator("vode", method="bdf", with_jacobian=True, rtol=1e-6, atol=1e-10, nsteps=500, order=5)
        r.set_initial_value(z0, 0.0)
        zs = r.integrate(dt[q])
        if not r.successful():
            continue
        T1 = T[q:q + 1].copy(); Y1 = Y[q:q + 1].copy()
        oracle.psr_cells(m, T1, rho[q:q + 1].copy(), Y1, dt[q:q + 1].copy())
        # same algorithm: agreement far inside the integration tolerance
        assert abs(T1[0] - zs[0]) <= 1e-6 * zs[0] + 1e-9, (q, T1[0], zs[0])
        assert np.max(np.abs(Y1[0] - zs[1:]) - (1e-6 * np.abs(zs[1:]) + 1e-10)) <= 0.0


def test_chem_step_field_on_cpu():
    import workloads as W
    cfg, thd, adi, dxi, st, info, orc = W.case("mix", 16)
    m = h2_mechanism()
    dtm = orc.chem_step(st, m, 0.5)
    v = st["v"][3:-3, 3:-3, 3:-3]
    assert np.max(np.abs(v[..., 5:].sum(axis=-1) / v[..., 0] - 1.0)) < 1e-12
    assert dtm >= 0.0


@pytest.fixture(scope="module")
def host_chem(tmp_path_factory):
    """The GPU chemistry source (chem.cu) compiled for the host with FMA
    contraction off (tests/harness/chem_host_harness.cu)."""
    import ctypes as C
    import shutil
    import subprocess
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    here = os.path.dirname(os.path.abspath(__file__))
    so = str(tmp_path_factory.mktemp("chemhost") / "libchemhost.so")
    subprocess.check_call([nvcc, "-std=c++17", "-O2", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                           "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", so,
                           os.path.join(here, "harness", "chem_host_harness.cu")])
    return C.CDLL(so)


def _P(a):
    import ctypes as C
    return a.ctypes.data_as(C.c_void_p)


def test_device_integrator_reproduces_oracle_bitwise(host_chem):
    """The GPU BDF code, compiled for the host without FMA contraction, gives
    the oracle's results bit for bit: the device port is the same algorithm
    in the same operation order."""
    import ctypes as C
    m = h2_mechanism()
    T, rho, Y, dt = ics.batched_reactors(512, seed=21)
    To, Yo = T.copy(), Y.copy()
    oracle.psr_cells(m, To, rho.copy(), Yo, dt.copy())
    Th, Yh = T.copy(), Y.copy()
    ns = np.zeros(len(T), np.int32)
    host_chem.host_psr(C.byref(m), len(T), _P(Th), _P(rho), _P(Yh), _P(dt), _P(ns))
    assert np.array_equal(Th, To) and np.array_equal(Yh, Yo)


def test_device_rhs_with_reciprocals_matches_reference_order(host_chem):
    """The BDF kernels evaluate the reactor right-hand side with the
    divisions replaced by reciprocal multiplications (ck_fun_fast); on the
    host it agrees with the reference-order form to a few ulp of each
    term: 1e-12 relative to the largest rate of each component."""
    import ctypes as C
    m = h2_mechanism()
    T, rho, Y, dt = ics.batched_reactors(4096, seed=23)
    z = np.ascontiguousarray(np.concatenate([T[:, None], Y], axis=1))
    zr, zf = np.zeros_like(z), np.zeros_like(z)
    host_chem.host_fun_pair(C.byref(m), len(T), _P(rho), _P(z), _P(zr), _P(zf))
    scale = np.abs(zr).max(axis=0)
    assert np.array_equal(zf[:, scale == 0], zr[:, scale == 0])   # components that stay exactly zero
    err = (np.abs(zf - zr) / np.where(scale == 0, 1.0, scale)).max(axis=0)
    assert np.all(err < 1e-12), err


def test_generated_rhs_is_the_table_form_bit_for_bit(host_chem):
    """The right-hand side generated for the shipped mechanism
    (phd_gb300/csrc/chem_gen.cuh) performs the generic device form's
    operations in the same order with the tables as literals: on the host,
    without FMA contraction, every component is bit-identical on the 4096
    batched reactors and on states with negative mass fractions and
    temperatures on both sides of the NASA-7 switch.  The header recognises
    its own mechanism and no other."""
    import ctypes as C
    m = h2_mechanism()
    T, rho, Y, dt = ics.batched_reactors(4096, seed=29)
    rng = np.random.Generator(np.random.PCG64(3))
    Y2 = Y + 1e-9 * rng.standard_normal(Y.shape)          # DVODE iterates can go slightly negative
    T2 = rng.uniform(300.0, 3500.0, len(T))
    zs = [np.concatenate([T[:, None], Y], axis=1), np.concatenate([T2[:, None], Y2], axis=1)]
    for z in zs:
        z = np.ascontiguousarray(z)
        zt, zg = np.zeros_like(z), np.zeros_like(z)
        ok = C.c_int()
        host_chem.host_fun_gen_pair(C.byref(m), len(T), _P(rho), _P(z), _P(zt), _P(zg), C.byref(ok))
        assert ok.value == 1
        assert np.array_equal(zt, zg), np.abs(zt - zg).max(axis=0)
    m.par[0][0] *= 1.0 + 2.0 ** -52   # one table entry one ulp off: not the generated mechanism
    z = np.ascontiguousarray(zs[0][:4])
    host_chem.host_fun_gen_pair(C.byref(m), 4, _P(rho), _P(z), _P(np.zeros_like(z)), _P(np.zeros_like(z)), C.byref(ok))
    assert ok.value == 0


def test_generated_header_is_current():
    """csrc/chem_gen.cuh is what phd_gb300/mechgen.py writes for the shipped
    mechanism (regenerate with python -m phd_gb300.mechgen)."""
    from phd_gb300 import mechgen
    with open(mechgen.OUT) as f:
        assert f.read() == mechgen.generate(h2_mechanism())


def test_reciprocal_form_alone_against_the_oracle(host_chem):
    """The integrator with the device right-hand side (ck_fun_fast), on the
    host with the host's libm and no FMA contraction, against the oracle on
    the 2048 batched reactors of the GPU batch test.  The reciprocal form
    alone perturbs the last bits of the rates; in igniting cells that
    changes adaptive step decisions (about 6 % of the cells take another
    number of steps), and those cells differ by the integrator's own global
    error.  The bounds are those of workloads.reactor_error_bounds, which
    the GPU batch meets as well: the GPU's remaining difference from the
    oracle is of this kind, not an error of CUDA's exp/log or of FMA
    contraction."""
    import ctypes as C
    import workloads as W
    m = h2_mechanism()
    T, rho, Y, dt = ics.batched_reactors(2048, seed=21)
    To, Yo = T.copy(), Y.copy()
    oracle.psr_cells(m, To, rho.copy(), Yo, dt.copy())
    Th, Yh = T.copy(), Y.copy()
    ns = np.zeros(len(T), np.int32)
    host_chem.host_psr_fast(C.byref(m), len(T), _P(Th), _P(rho), _P(Yh), _P(dt), _P(ns))
    st, msg, ok = W.reactor_error_bounds(Th, Yh, To, Yo)
    print(msg)
    assert ok, msg
    assert st["T"]["max"] > 0   # the reciprocal form does change results


def _window(cfg):
    """reaction_dvode's window (module_reaction.f90:155-159) as slices of the
    ghosted arrays; its z bound uses ey."""
    ng = cfg.ng
    hi = (min(cfg.nx, cfg.nx - ng - 1), min(cfg.ny, cfg.ny - ng - 1), min(cfg.ny, cfg.nz - ng - 1))
    return tuple(slice(2 * ng, ng + h) for h in hi)


def test_dvodesimp_skips_pure_streams_and_keeps_the_rest():
    """dvodesimp (module_reaction.f90:173-251): window cells in the pure fuel
    or oxidiser streams (H2 or N2 within 1e-6 of the stream's) keep v and T
    to the bit; the others get the full path's result, with the closing
    species clipped; max |dT| comes from the integrated cells only."""
    import workloads as W
    m = h2_mechanism()
    cfg, thd, adi, dxi, st, orc, (yf, yo, ih2, in2) = W.mixing_layer_with_streams()
    st0 = W.copy(st)
    full = W.copy(st)
    dtm_full = orc.chem_step(full, m, 0.5)
    orc.set_chem_skip(yf, yo, ih2, in2)
    skip = W.copy(st)
    dtm_skip = orc.chem_step(skip, m, 0.5)
    w = _window(cfg)
    v0 = st0["v"][w]
    Y = v0[..., 5:] / v0[..., :1]
    pure = ~((np.abs(Y[..., ih2] - yf[ih2]) > 1e-6) & (np.abs(Y[..., in2] - yf[in2]) > 1e-6)
             & (np.abs(Y[..., ih2] - yo[ih2]) > 1e-6) & (np.abs(Y[..., in2] - yo[in2]) > 1e-6))
    moved = np.any(skip["v"][w] != v0, axis=-1) | (skip["T"][w] != st0["T"][w])
    assert 0 < pure.sum() < pure.size and not np.any(moved & pure)
    called = ~np.all(skip["v"][w][..., 5:] == v0[..., 5:], axis=-1) | (skip["T"][w] != st0["T"][w])
    assert called.sum() > 0
    assert np.array_equal(skip["T"][w][called], full["T"][w][called])
    assert np.array_equal(skip["v"][w][called][:, :13], full["v"][w][called][:, :13])
    assert np.allclose(skip["v"][w][called][:, 13], full["v"][w][called][:, 13], rtol=1e-15, atol=0)
    T_ref = adi.t_ref
    dT = np.abs(skip["T"][w] - st0["T"][w]) * T_ref
    assert dtm_skip <= dtm_full and abs(dtm_skip - dT.max()) <= 1e-9 * max(dT.max(), 1e-30)
    orc.set_chem_skip(enable=False)
    again = W.copy(st)
    assert orc.chem_step(again, m, 0.5) == dtm_full and np.array_equal(again["v"], full["v"])


@refdata.needs_reference
def test_mechanism_species_match_reference_interpreter_output():
    """The species, their order and molecular weights of the shipped
    mechanism are those of the reference's CHEMKIN interpreter listing for
    the 9-species case (testcases/shockedshearlayer/chem.out)."""
    rows = []
    for line in open(refdata.path("shockedshearlayer", "chem.out")):
        t = line.split()
        if len(t) >= 8 and t[0].endswith(".") and t[0][:-1].isdigit() and t[2] == "G":
            rows.append((t[1], float(t[4])))
    m = h2_mechanism()
    names = load_species("h2air9")["names"]
    assert [n for n, _ in rows] == names
    for k, (_, w) in enumerate(rows):
        assert abs(m.wt[k] - w) <= 5e-6 * w, (names[k], m.wt[k], w)


def _field_reactors(dt_s):
    """The window reactors of a 20^3 reacting field (ics.reacting_field) as
    independent reactors: T [K], rho [g/cm^3], Y (n, 9), dt [s]."""
    cfg, thd, adi, dxi, st, info = ics.reacting_field(20, 20, 20, dt_s=dt_s, corr=4,
                                                      lib_dscalar=oracle.metrics_dscalar)
    w = _window(cfg)
    v = st["v"][w]
    rho = np.ascontiguousarray(v[..., 0].ravel()) * adi.rho_ref * 1e-3
    Y = np.ascontiguousarray(np.stack([v[..., 5 + k].ravel() / v[..., 0].ravel() for k in range(9)], axis=1))
    T = np.ascontiguousarray(st["T"][w].ravel()) * adi.t_ref
    return T, rho, Y, np.full(len(T), dt_s)


def test_reciprocal_form_alone_on_the_reacting_field(host_chem):
    """As above, on the window reactors of the reacting field over 1e-6 s,
    where ignition fronts cross many cells within the step and the
    rounding of the reciprocal form alone moves them further than in the
    batch: held to workloads.FIELD_LIMITS, which the GPU field step meets
    against the oracle as well (tests/test_gpu_chem.py)."""
    import ctypes as C
    import workloads as W
    m = h2_mechanism()
    T, rho, Y, dt = _field_reactors(1e-6)
    To, Yo = T.copy(), Y.copy()
    oracle.psr_cells(m, To, rho.copy(), Yo, dt.copy())
    Th, Yh = T.copy(), Y.copy()
    ns = np.zeros(len(T), np.int32)
    host_chem.host_psr_fast(C.byref(m), len(T), _P(Th), _P(rho), _P(Yh), _P(dt), _P(ns))
    st, msg, ok = W.reactor_error_bounds(Th, Yh, To, Yo, W.FIELD_LIMITS)
    print(msg, "ignited (dT > 100 K): %d of %d" % (int((To - T > 100).sum()), len(T)))
    assert ok, msg
    assert not W.reactor_error_bounds(Th, Yh, To, Yo)[2]   # the batch bounds are too tight here


from workloads import SRI_PARAMS as _SRI_PARAMS, variant_mechanism as _variant_mechanism  # noqa: E402


def test_reader_sri_and_species_collider(tmp_path):
    """SRI / a b c d e / gives fall-off form 2 with its five parameters (three
    given: d = 1, e = 0); (+H2O) makes H2O the collider (kfal = index + 1)
    and no third-body sum."""
    m = _variant_mechanism(tmp_path)
    assert m.fall[3] == 2 and list(m.sri[3]) == list(_SRI_PARAMS) and m.kfal[3] == 0 and m.thb[3] == 1
    assert m.fall[11] == 4 and m.kfal[11] == 6 and m.thb[11] == 0     # H2O is species 5
    text = (tmp_path / "h2_sri_collider.inp").read_text().replace(
        "SRI / %s /" % "  ".join(repr(x) for x in _SRI_PARAMS), "SRI / 0.45 797.0 979.0 /")
    (tmp_path / "three.inp").write_text(text)
    from phd_gb300.mech import read_mechanism
    m3 = read_mechanism(str(tmp_path / "three.inp"), "h2air9")
    assert list(m3.sri[3]) == [0.45, 797.0, 979.0, 1.0, 0.0]
    assert all(m.kfal[i] == 0 for i in range(m.ii) if i != 11)


def _only(m, keep):
    """The mechanism with every reaction but `keep` switched off (A = 0, no
    fall-off)."""
    import copy
    m2 = copy.deepcopy(m)
    for i in range(m2.ii):
        if i != keep:
            m2.par[i][0] = 0.0
            m2.rpar[i][0] = 0.0
            m2.fall[i] = 0
    return m2


def _with_radicals(Y):
    """Batched-reactor compositions with H, O, OH and H2O2 added (1e-3 each,
    the rest scaled down), so that every reaction has reactants."""
    Y = Y * (1.0 - 4e-3)
    for k in (0, 2, 4, 7):
        Y[:, k] += 1e-3
    return np.ascontiguousarray(Y)


def test_sri_and_collider_rates_against_a_restatement(tmp_path):
    """The oracle's production rates of each of the two reactions alone
    against a numpy restatement of CKRATX (vode.f:1185-1236): the SRI factor
    (a exp(-b/T) + exp(-T/c))^X d T^e with X = 1 / (1 + log10(Pr)^2) and Pr
    from the efficiency-weighted third body; the Troe factor with Pr from
    the H2O concentration alone."""
    m = _variant_mechanism(tmp_path)
    T, rho, Y, dt = ics.batched_reactors(256, seed=41)
    Y = _with_radicals(Y)
    W = np.array([m.wt[k] for k in range(m.kk)])
    ih, io2, ih2o, ih2o2 = 0, 3, 5, 7
    for i in (3, 11):
        mi = _only(m, i)
        for q in range(len(T)):
            wdot = oracle.ck_wdot(mi, rho[q], T[q], Y[q])
            C = rho[q] * Y[q] / W
            Tq = T[q]
            A, b, ER = m.par[i][0], m.par[i][1], m.par[i][2]
            kf = A * np.exp(b * np.log(Tq) - ER / Tq)
            kl = m.low[i][0] * np.exp(m.low[i][1] * np.log(Tq) - m.low[i][2] / Tq)
            if i == 3:
                ctb = C.sum() + sum((m.eff[i][k] - 1.0) * C[k] for k in range(m.kk))
                pr = kl * ctb / kf
                a, bb, c, d, e = _SRI_PARAMS
                x = 1.0 / (1.0 + np.log10(max(pr, 1e-300)) ** 2)
                fc = (a * np.exp(-bb / Tq) + np.exp(-Tq / c)) ** x * d * Tq ** e
                rop = kf * fc * pr / (1.0 + pr) * C[ih] * C[io2]
                ref = {ih: -rop, io2: -rop, 6: rop}
            else:
                pr = kl * C[ih2o] / kf
                ta, t3, t1, t2 = (m.troe[i][k] for k in range(4))
                fcent = (1 - ta) * np.exp(-Tq / t3) + ta * np.exp(-Tq / t1) + np.exp(-t2 / Tq)
                lfc = np.log10(fcent)
                cpr = np.log10(pr) - (0.4 + 0.67 * lfc)
                nn = 0.75 - 1.27 * lfc
                fc = 10.0 ** (lfc / (1.0 + (cpr / (nn - 0.14 * cpr)) ** 2))
                rop = kf * fc * pr / (1.0 + pr) * C[ih2o2]
                ref = {ih2o2: -rop, 4: 2.0 * rop}
            for k in range(m.kk):
                assert abs(wdot[k] - ref.get(k, 0.0)) <= 1e-13 * abs(rop), (i, q, k, wdot[k], ref.get(k, 0.0))


@pytest.mark.parametrize("variant", ["sri_collider", "equilibrium", "landau_teller"])
def test_variant_mechanisms_device_forms_on_the_host(host_chem, tmp_path, variant):
    """With a variant mechanism (the SRI form and a single-species collider,
    or reverse rates from the equilibrium constant), the device integrator
    in the reference's operation order reproduces the oracle bit for bit on
    the host, and the reciprocal form agrees with it to 1e-12 of each
    component's largest rate."""
    import ctypes as C
    import workloads as W
    m = W.VARIANTS[variant](tmp_path)
    T, rho, Y, dt = ics.batched_reactors(512, seed=43)
    To, Yo = T.copy(), Y.copy()
    oracle.psr_cells(m, To, rho.copy(), Yo, dt.copy())
    Th, Yh = T.copy(), Y.copy()
    ns = np.zeros(len(T), np.int32)
    host_chem.host_psr(C.byref(m), len(T), _P(Th), _P(rho), _P(Yh), _P(dt), _P(ns))
    assert np.array_equal(Th, To) and np.array_equal(Yh, Yo)
    assert not np.array_equal(To, T)
    z = np.ascontiguousarray(np.concatenate([T[:, None], Y], axis=1))
    zr, zf = np.zeros_like(z), np.zeros_like(z)
    host_chem.host_fun_pair(C.byref(m), len(T), _P(rho), _P(z), _P(zr), _P(zf))
    scale = np.abs(zr).max(axis=0)
    err = (np.abs(zf - zr) / np.where(scale == 0, 1.0, scale)).max(axis=0)
    assert np.all(err < 1e-12), err


@pytest.mark.parametrize("variant", ["sri_collider", "equilibrium", "landau_teller"])
def test_generated_rhs_for_variant_mechanisms(tmp_path, variant):
    """mechgen writes a variant's right-hand side; compiled into the host
    harness in place of the shipped header (IZEM_CHEM_GEN_HEADER), it is the
    reciprocal table form bit for bit, and it recognises its own mechanism."""
    import ctypes as C
    import shutil
    import subprocess
    import workloads as W
    from phd_gb300 import mechgen
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    m = W.VARIANTS[variant](tmp_path)
    hdr = tmp_path / "chem_gen_variant.cuh"
    hdr.write_text(mechgen.generate(m, source="the %s test mechanism" % variant))
    here = os.path.dirname(os.path.abspath(__file__))
    so = str(tmp_path / "libchemgen.so")
    subprocess.check_call([nvcc, "-std=c++17", "-O2", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                           "-shared", "-gencode", "arch=compute_103a,code=sm_103a",
                           '-DIZEM_CHEM_GEN_HEADER="%s"' % str(hdr), "-o", so,
                           os.path.join(here, "harness", "chem_host_harness.cu")])
    lib = C.CDLL(so)
    T, rho, Y, dt = ics.batched_reactors(1024, seed=47)
    z = np.ascontiguousarray(np.concatenate([T[:, None], Y], axis=1))
    zt, zg = np.zeros_like(z), np.zeros_like(z)
    ok = C.c_int()
    lib.host_fun_gen_pair(C.byref(m), len(T), _P(rho), _P(z), _P(zt), _P(zg), C.byref(ok))
    assert ok.value == 1
    assert np.array_equal(zt, zg), np.abs(zt - zg).max(axis=0)
    if variant == "sri_collider":
        m.sri[3][4] = 0.2   # another SRI exponent: not the generated mechanism
    elif variant == "landau_teller":
        m.lt[1][1] = 11.0   # another Landau-Teller C: not the generated mechanism
    else:
        m.rev[0] = 0        # reaction 0 irreversible: not the generated mechanism
    lib.host_fun_gen_pair(C.byref(m), 4, _P(rho), _P(z), _P(np.zeros_like(z)), _P(np.zeros_like(z)), C.byref(ok))
    assert ok.value == 0


@pytest.mark.parametrize("line", ["   FORD / H2 0.5 /\n", "   RLT / 1.0 2.0 /\n"])
def test_reader_rejects_rate_forms_it_does_not_build(tmp_path, line):
    """Reaction-order data, and reverse Landau-Teller parameters on a
    reaction without explicit reverse parameters, are refused, not
    dropped."""
    from phd_gb300.mech import read_mechanism
    from phd_gb300.thd import DATA_DIR
    with open(os.path.join(DATA_DIR, "h2_sandiego12.inp")) as f:
        text = f.read()
    text = text.replace("HO2+H=>OH+OH                 7.08E13   0.00   0.294\n",
                        "HO2+H=>OH+OH                 7.08E13   0.00   0.294\n" + line)
    path = tmp_path / "bad.inp"
    path.write_text(text)
    with pytest.raises(ValueError):
        read_mechanism(str(path), "h2air9")


def test_landau_teller_rates_against_a_restatement(tmp_path):
    """H2+O<=>OH+H alone with Landau-Teller factors on both rates, from the
    oracle, against a numpy restatement of CKRATT: k_f = A T^b exp(-E/RT)
    exp(B/T^(1/3) + C/T^(2/3)), k_r = the REV rate times the RLT factor."""
    import workloads as W
    m = W.landau_teller_variant_mechanism(tmp_path)
    assert list(m.lt[1]) == list(W.LT_PARAMS) and list(m.rlt[1]) == list(W.RLT_PARAMS)
    mi = _only(m, 1)
    T, rho, Y, dt = ics.batched_reactors(128, seed=53)
    Y = _with_radicals(Y)
    Wt = np.array([m.wt[k] for k in range(m.kk)])
    for q in range(len(T)):
        wdot = oracle.ck_wdot(mi, rho[q], T[q], Y[q])
        C = rho[q] * Y[q] / Wt
        Tq = T[q]

        def lt(bc):
            return np.exp(bc[0] / Tq ** (1.0 / 3.0) + bc[1] / Tq ** (2.0 / 3.0))

        kf = m.par[1][0] * np.exp(m.par[1][1] * np.log(Tq) - m.par[1][2] / Tq) * lt(W.LT_PARAMS)
        kr = m.rpar[1][0] * np.exp(m.rpar[1][1] * np.log(Tq) - m.rpar[1][2] / Tq) * lt(W.RLT_PARAMS)
        rop = kf * C[1] * C[2] - kr * C[4] * C[0]       # H2 + O -> OH + H
        ref = {1: -rop, 2: -rop, 4: rop, 0: rop}
        scale = max(kf * C[1] * C[2], kr * C[4] * C[0])
        for k in range(m.kk):
            assert abs(wdot[k] - ref.get(k, 0.0)) <= 1e-13 * scale, (q, k, wdot[k], ref.get(k, 0.0))

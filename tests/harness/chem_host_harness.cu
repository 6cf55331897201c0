// Host build of the GPU stiff-chemistry integrator (phd_gb300/csrc/chem.cu,
// compiled with IZEM_CHEM_HOST_TEST so that its __device__ integrator
// functions are also host functions).  Used by tests/test_chem_cpu.py to
// show that the device algorithm reproduces the oracle bit for bit when both
// run without fused multiply-adds on the same CPU.
#define IZEM_CHEM_HOST_TEST 1
#include "../../phd_gb300/csrc/chem.cu"

// The host copies of what chem_upload_mech puts in constant memory.
static void set_mech(const izem_mech* m) {
  c_mech_host = *m;
  c_fast_host = chem_fast_constants(*m);
  c_need_eqk_host = 0;
  for (int i = 0; i < m->ii; ++i) c_need_eqk_host |= (m->rev[i] == 1);
}

extern "C" void host_psr(const izem_mech* m, int n, double* T, const double* rho, double* Y, const double* dt,
                         int* nst_out) {
  set_mech(m);
  for (int q = 0; q < n; ++q) {
    double z[10];
    z[0] = T[q];
    for (int k = 0; k < 9; ++k) z[1 + k] = Y[q * 9 + k];
    int nst = 0;
    reaction_v<10>(rho[q], z, dt[q], &nst);
    nst_out[q] = nst;
    T[q] = z[0];
    for (int k = 0; k < 9; ++k) Y[q * 9 + k] = z[1 + k];
  }
}

// The device right-hand side with reciprocals (ck_fun_fast) next to the
// reference-order one (ck_fun), both on the host.
extern "C" void host_fun_pair(const izem_mech* m, int n, const double* rho, const double* z, double* zp_ref,
                              double* zp_fast) {
  set_mech(m);
  for (int q = 0; q < n; ++q) {
    ck_fun<9>(rho[q], z + 10 * q, zp_ref + 10 * q);
    ck_fun_fast<9>(rho[q], z + 10 * q, zp_fast + 10 * q);
  }
}

// The integrator as the GPU kernels run it -- the right-hand side with
// reciprocals (ck_fun_fast) -- on the host, without fused multiply-adds and
// with the host's libm: what the reciprocal form alone changes against the
// oracle, apart from CUDA's exp/log and FMA contraction.
extern "C" void host_psr_fast(const izem_mech* m, int n, double* T, const double* rho, double* Y, const double* dt,
                              int* nst_out) {
  set_mech(m);
  for (int q = 0; q < n; ++q) {
    Rc<10> r;
    double z[10];
    z[0] = T[q];
    for (int k = 0; k < 9; ++k) z[1 + k] = Y[q * 9 + k];
    rc_start<10>(r, rho[q], z, dt[q]);
    while (rc_advance<10>(r)) ck_fun_fast<9>(r.rho, r.y, r.fo);
    nst_out[q] = r.nsteps;
    T[q] = r.y[0];
    for (int k = 0; k < 9; ++k) Y[q * 9 + k] = r.y[1 + k];
  }
}

// The right-hand side generated for the shipped mechanism (chem_gen.cuh)
// next to the generic device form (ck_fun_fast), both on the host.
extern "C" void host_fun_gen_pair(const izem_mech* m, int n, const double* rho, const double* z, double* zp_tab,
                                  double* zp_gen, int* matches) {
  set_mech(m);
  *matches = chem_gen::matches(*m) ? 1 : 0;
  for (int q = 0; q < n; ++q) {
    ck_fun_fast<9>(rho[q], z + 10 * q, zp_tab + 10 * q);
    chem_gen::FunT t;
    chem_gen::tpart(z[10 * q], t);
    chem_gen::cpart(rho[q], z + 10 * q, t, zp_gen + 10 * q);
  }
}

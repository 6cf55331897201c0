// CPU oracle for the IZEM right-hand-side hot path -- TEST INFRASTRUCTURE ONLY.
//
// This file restates, in C++17 and loop by loop, the Fortran routines of the
// reference solver (saras13015/Phd, devel-izem/src) that the GPU library
// replaces.  It is the oracle for the CUDA path: only tests, the smoke check
// and the CPU-baseline leg of the benchmark may load it; the product never
// links or calls it.  The reference cannot be compiled here (no Fortran
// compiler, MPI or HDF5), so this restatement is the oracle.  Each function
// cites the reference lines it follows; floating-point expressions keep the
// reference's operation order so that results agree to rounding.  Build with
// -ffp-contract=off so that no multiply-add is fused on either machine.
//
// Parity pinning: the flow restatement reproduces the reference's own FP64
// restart files of its 2-D WENO7 Sod run (testcases/sod) to about 5e-8 of
// the field maxima after 647-777 steps (tests/test_sod_pin.py); that case
// runs the ng = 4, ndim = 2 branches below and emulates the two effects of
// the reference's two MPI blocks on the shock sensor.  The chemistry
// restatement is cross-checked against an independent DVODE (scipy's BDF
// integrator) on the same reactor equations.
//
// Layout: one block of nx*ny*nz interior points with ng ghost layers,
// Fortran column-major, variable index slowest, exactly the reference's
// v(sx-ng:ex+ng, sy-ng:ey+ng, sz-ng:ez+ng, 1:nv) with sx = sy = sz = 1.

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <vector>
#include <memory>
#include <string>

#include "../include/izem_gpu.h"

namespace {

constexpr int NIV = 5;

// ---------------------------------------------------------------- block ----
struct Block {
  int nx, ny, nz, ng, nrv, nv;
  int gx, gy, gz;
  size_t ncell, nint;
  bool bnd[6];   // face is a physical boundary (neigh == MPI_PROC_NULL)
  int bc[6];
  size_t id(int i, int j, int k) const {
    return (size_t)(i - 1 + ng) + (size_t)gx * ((size_t)(j - 1 + ng) + (size_t)gy * (size_t)(k - 1 + ng));
  }
  size_t fid(int i, int j, int k) const {
    return (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1));
  }
  int n(int d) const { return d == 0 ? nx : (d == 1 ? ny : nz); }
};

struct EgInit;   // EGLIB initialisation data (eglib_oracle.inc)

struct Ctx {
  izem_cfg cfg;
  izem_thd thd;
  izem_adi adi;
  std::shared_ptr<EgInit> eg;   // set by or_set_eglib for cfg.eglib = 1
  Block b;
  std::vector<double> dxi[3];   // indexed (i-1+ng), length n+2ng
  int newton_warn = 0;
  int newton_it_max = 0;   // most iterations of any prim_inv_var call (test readout)
  int sensor_xblocks = 1;   // x-blocks of the reference's MPI run whose edges the sensor does not cross
  int newton_xblocks = 1;   // x-blocks whose Newton loops stop on their own test
  int sensor_type = IZEM_SENSOR_ADAMS_SHARIFF;   // SHOCK_SENSOR_TYPE
  double ducros_treduc = 0.2;                    // DUCROS_TREDUC
  // dvodesimp (module_reaction.f90:173-251): pure fuel Y1f and oxidiser Y0o,
  // H2 and N2 species indices (0-based)
  // LES with the Smagorinsky closure under EGLIB (or_set_les): MU_SGS_FACTOR,
  // SC_SGS, PR_SGS, PERCENT_WEIGHT_SGS
  bool les = false;
  double les_factor = 0.0, les_sc_sgs = 1.0, les_pr_sgs = 1.0, les_pw = 0.0;
  // mu_SGS of the last viscflux_LES_xyz call (fitted transport), read by the
  // Fourier time step; zero until then and under EGLIB, whose LES flux
  // routine keeps its own copy
  std::vector<double> mu_sgs;
  // coordinates of the interior points (code units) and the domain length
  // in x (Lx, module_tools.f90:319,489) for the jet boundaries
  std::vector<double> crd[3];
  double lx = 0.0;
  // parameters of the jet faces: the constants of bc_inflowjet
  // (module_BCs.f90:1680-1700) and bc_nscbc_out (:2390) unless overridden
  izem_jet jet{0.0010, 0.0001, 1000.0, 300.0, 101325.0 * 15.0, 101325.0, 0.0, 20.0, 1.0, 94232.25, 0.0, 0, 0, 0ULL};
  bool dvodesimp = false;
  double y1f[IZEM_NSMAX] = {}, y0o[IZEM_NSMAX] = {};
  int index_h2 = 0, index_n2 = 0;
  std::string err;
};

// domain_select (module_parallel.f90:1936-2020), restricted to the ids used
// on the hot path: 0 interior, -1/1 x-ghost slabs, -2/2 y, -3/3 z.
void domain_select(const Block& b, int id, int& i0, int& i1, int& j0, int& j1, int& k0, int& k1) {
  i0 = 1; i1 = b.nx; j0 = 1; j1 = b.ny; k0 = 1; k1 = b.nz;
  switch (id) {
    case -3: k0 = 1 - b.ng; k1 = 0; break;
    case -2: j0 = 1 - b.ng; j1 = 0; break;
    case -1: i0 = 1 - b.ng; i1 = 0; break;
    case 0: break;
    case 1: i0 = b.nx + 1; i1 = b.nx + b.ng; break;
    case 2: j0 = b.ny + 1; j1 = b.ny + b.ng; break;
    case 3: k0 = b.nz + 1; k1 = b.nz + b.ng; break;
    case -10: i1 = 1; break;          // Dirichlet planes (module_parallel.f90:1944-2000)
    case 10: i0 = b.nx; break;
    case -20: j1 = 1; break;
    case 20: j0 = b.ny; break;
    case -30: k1 = 1; break;
    case 30: k0 = b.nz; break;
    default: break;
  }
}

// ------------------------------------------------------------ thermo -------
// cp_scalar (module_thermodynamics.f90:767-862)
double cp_scalar(const izem_thd& t, double temp, const double* Y) {
  double cp = 0.0;
  for (int is = 0; is < t.nspc; ++is) {
    double t1 = temp * t.tinf, t2 = t1 * t1, t3 = t2 * t1, t4 = t3 * t1;
    const double* lo = t.heatcap[is][0];
    const double* hi = t.heatcap[is][1];
    double fac = Y[is] * t.gam2 * t.Wc_i[is];
    if (t1 < t.tpolymin[is]) {
      t1 = t.tpolymin[is]; t2 = t1 * t1; t3 = t2 * t1; t4 = t3 * t1;
      double cp0 = lo[0] + lo[1] * t1 + lo[2] * t2 + lo[3] * t3 + lo[4] * t4;
      double dcp0 = lo[1] + lo[2] * t1 * 2.0 + lo[3] * t2 * 3.0 + lo[4] * t3 * 4.0;
      cp = cp + fac * (dcp0 * (temp * t.tinf - t.tpolymin[is]) + cp0);
    } else if (t1 < t.tpolylim[is]) {
      cp = cp + fac * (lo[0] + lo[1] * t1 + lo[2] * t2 + lo[3] * t3 + lo[4] * t4);
    } else if (t1 < t.tpolymax[is]) {
      cp = cp + fac * (hi[0] + hi[1] * t1 + hi[2] * t2 + hi[3] * t3 + hi[4] * t4);
    } else {
      t1 = t.tpolymax[is]; t2 = t1 * t1; t3 = t2 * t1; t4 = t3 * t1;
      double cp0 = hi[0] + hi[1] * t1 + hi[2] * t2 + hi[3] * t3 + hi[4] * t4;
      double dcp0 = hi[1] + hi[2] * t1 * 2.0 + hi[3] * t2 * 3.0 + hi[4] * t3 * 4.0;
      cp = cp + fac * (dcp0 * (temp * t.tinf - t.tpolymax[is]) + cp0);
    }
  }
  return cp;
}

inline double h_poly(const double* a, double t1, double t2, double t3, double t4, double t5, double onethird) {
  return a[0] * t1 + a[1] * t2 * 0.50 + a[2] * t3 * onethird + a[3] * t4 * 0.25 + a[4] * t5 * 0.20 + a[5];
}
inline double cp_poly(const double* a, double t1, double t2, double t3, double t4) {
  return a[0] + a[1] * t1 + a[2] * t2 + a[3] * t3 + a[4] * t4;
}
inline double dcp_poly(const double* a, double t1, double t2, double t3) {
  return a[1] + a[2] * t1 * 2.0 + a[3] * t2 * 3.0 + a[4] * t3 * 4.0;
}

// ha_scalar (module_thermodynamics.f90:873-978)
void ha_scalar(const izem_thd& t, double temp, double* ha) {
  const double tinf_i = 1.0 / t.tinf, onethird = 1.0 / 3.0;
  for (int is = 0; is < t.nspc; ++is) {
    double t1 = temp * t.tinf, t2 = t1 * t1, t3 = t2 * t1, t4 = t3 * t1, t5 = t4 * t1;
    const double* lo = t.heatcap[is][0];
    const double* hi = t.heatcap[is][1];
    double h;
    if (t1 < t.tpolymin[is]) {
      t1 = t.tpolymin[is]; t2 = t1 * t1; t3 = t2 * t1; t4 = t3 * t1; t5 = t4 * t1;
      double ha0 = h_poly(lo, t1, t2, t3, t4, t5, onethird);
      double dha0 = cp_poly(lo, t1, t2, t3, t4);
      h = t.Wc_i[is] * tinf_i * (dha0 * (temp * t.tinf - t.tpolymin[is]) + ha0);
    } else if (t1 < t.tpolylim[is]) {
      h = t.Wc_i[is] * tinf_i * h_poly(lo, t1, t2, t3, t4, t5, onethird);
    } else if (t1 < t.tpolymax[is]) {
      h = t.Wc_i[is] * tinf_i * h_poly(hi, t1, t2, t3, t4, t5, onethird);
    } else {
      t1 = t.tpolymax[is]; t2 = t1 * t1; t3 = t2 * t1; t4 = t3 * t1; t5 = t4 * t1;
      double ha0 = h_poly(hi, t1, t2, t3, t4, t5, onethird);
      double dha0 = cp_poly(hi, t1, t2, t3, t4);
      h = t.Wc_i[is] * tinf_i * (dha0 * (temp * t.tinf - t.tpolymax[is]) + ha0);
    }
    ha[is] = 0.0 + h;
  }
}

// Wmix_i (module_thermodynamics.f90:700-728) on one sub-domain
void wmix_i(const Ctx& c, int dom, const double* v, double* W_i) {
  const Block& b = c.b;
  int i0, i1, j0, j1, k0, k1;
  domain_select(b, dom, i0, i1, j0, j1, k0, k1);
  // per point the species are summed in the reference's order
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = k0; k <= k1; ++k)
    for (int j = j0; j <= j1; ++j)
      for (int i = i0; i <= i1; ++i) {
        size_t p = b.id(i, j, k);
        double w = 0.0;
        for (int l = 0; l < b.nrv; ++l) w = w + (v[(NIV + l) * b.ncell + p] / v[p]) * c.thd.Wc_i[l];
        W_i[p] = w;
      }
}

// newton (module_thermodynamics.f90:271-508) for one cell; returns DF and
// writes cp and ha at the input temperature.
double newton_cell(const izem_thd& t, const Block& b, const double* v, size_t p, double T, double* cp_out, double* ha_out) {
  const double tinf_i = 1.0 / t.tinf, onethird = 1.0 / 3.0, gam2_i = 1.0 / t.gam2;
  const size_t nc = b.ncell;
  double rho_i = 1.0 / v[p];
  double v2 = v[nc + p], v3 = v[2 * nc + p], v4 = v[3 * nc + p];
  double F = -v[4 * nc + p] * rho_i + 0.5 * (v2 * v2 + v3 * v3 + v4 * v4) * (rho_i * rho_i);
  double Ya[IZEM_NSMAX];
  for (int is = 0; is < b.nrv; ++is) Ya[is] = v[(NIV + is) * nc + p] * rho_i;
  double cp = 0.0;
  for (int is = 0; is < b.nrv; ++is) {
    double t1 = T * t.tinf, t2 = t1 * t1, t3 = t2 * t1, t4 = t3 * t1, t5 = t4 * t1;
    double wrk1 = -T;
    const double* lo = t.heatcap[is][0];
    const double* hi = t.heatcap[is][1];
    double h;
    double fac = Ya[is] * t.gam2 * t.Wc_i[is];
    if (t1 < t.tpolymin[is]) {
      t1 = t.tpolymin[is]; t2 = t1 * t1; t3 = t2 * t1; t4 = t3 * t1; t5 = t4 * t1;
      double ha0 = h_poly(lo, t1, t2, t3, t4, t5, onethird);
      double dha0 = cp_poly(lo, t1, t2, t3, t4);
      h = 0.0 + t.Wc_i[is] * tinf_i * (dha0 * (T * t.tinf - t.tpolymin[is]) + ha0);
      double cp0 = dha0;
      double dcp0 = dcp_poly(lo, t1, t2, t3);
      cp = cp + fac * (dcp0 * (T * t.tinf - t.tpolymin[is]) + cp0);
    } else if (t1 < t.tpolylim[is]) {
      h = 0.0 + t.Wc_i[is] * tinf_i * h_poly(lo, t1, t2, t3, t4, t5, onethird);
      cp = cp + fac * cp_poly(lo, t1, t2, t3, t4);
    } else if (t1 < t.tpolymax[is]) {
      h = 0.0 + t.Wc_i[is] * tinf_i * h_poly(hi, t1, t2, t3, t4, t5, onethird);
      cp = cp + fac * cp_poly(hi, t1, t2, t3, t4);
    } else {
      t1 = t.tpolymax[is]; t2 = t1 * t1; t3 = t2 * t1; t4 = t3 * t1; t5 = t4 * t1;
      double ha0 = h_poly(hi, t1, t2, t3, t4, t5, onethird);
      double dha0 = cp_poly(hi, t1, t2, t3, t4);
      h = 0.0 + t.Wc_i[is] * tinf_i * (dha0 * (T * t.tinf - t.tpolymax[is]) + ha0);
      double cp0 = dha0;
      double dcp0 = dcp_poly(hi, t1, t2, t3);
      cp = cp + fac * (dcp0 * (T * t.tinf - t.tpolymax[is]) + cp0);
    }
    ha_out[is] = h;
    F = F + Ya[is] * (h + wrk1 * t.Wc_i[is]);
  }
  double wrk = 0.0;
  for (int is = 0; is < b.nrv; ++is) wrk = wrk + Ya[is] * t.Wc_i[is];
  *cp_out = cp;
  return F / (wrk - cp * gam2_i);
}

// prim_inv_var (module_thermodynamics.f90:79-186) / prim_inv_var_err_mach
// (:201-260) on one sub-domain: a global Newton loop whose stopping test is
// the maximum temperature correction over the whole sub-domain.
int prim_inv_var_region(Ctx& c, bool err_mach, int i0, int i1, int j0, int j1, int k0, int k1, double* v, double* T,
                        double* cp, double* ha) {
  const Block& b = c.b;
  const int itmax = err_mach ? 100 : 200;
  const double eps = err_mach ? 1.0e-10 : 1.0e-5;
  int it = 0;
  double error = 0.0;
  bool negT = false;
  while (true) {
    it = it + 1;
    if (it > itmax) break;
    double maxdf = 0.0;
    bool anynan = false;
    // every point's update is its own; the maximum is the same in any order
#pragma omp parallel for collapse(2) schedule(static) reduction(max : maxdf) reduction(|| : anynan, negT)
    for (int k = k0; k <= k1; ++k)
      for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i) {
          size_t p = b.id(i, j, k);
          double hak[IZEM_NSMAX];
          double cpp;
          double DF = newton_cell(c.thd, b, v, p, T[p], &cpp, hak);
          cp[p] = cpp;
          for (int is = 0; is < b.nrv; ++is) ha[is * b.ncell + p] = hak[is];
          T[p] = T[p] + DF;
          DF = DF * DF;
          if (!err_mach && T[p] < 0.0) negT = true;
          if (std::isnan(DF)) anynan = true;
          else if (DF > maxdf) maxdf = DF;
        }
    if (negT) {
      c.err = "negative temperature in prim_inv_var";
      return IZEM_ERR_NEG_TEMPERATURE;
    }
    error = anynan ? std::nan("") : std::sqrt(maxdf);
    if (error < eps) break;
  }
  if (it > itmax) c.newton_warn++;
  c.newton_it_max = std::max(c.newton_it_max, std::min(it, itmax));
  if (!err_mach && error != error) {
    c.err = "Newton error is a NaN";
    return IZEM_ERR_NAN;
  }
  return IZEM_OK;
}

int prim_inv_var(Ctx& c, int dom, bool err_mach, double* v, double* W_i, double* T, double* cp, double* ha) {
  const Block& b = c.b;
  int i0, i1, j0, j1, k0, k1;
  domain_select(b, dom, i0, i1, j0, j1, k0, k1);
  wmix_i(c, dom, v, W_i);
  // the reference's ranks each run the loop, and its stopping test, on
  // their own points (test-only emulation of an x-decomposition: the
  // interior and the ghost slabs that span x split into x-blocks)
  const int nxb = std::max(c.newton_xblocks, 1);
  if (nxb > 1 && i0 >= 1 && i1 <= b.nx) {
    const int bx = b.nx / nxb;
    for (int q = 0; q < nxb; ++q) {
      const int lo = std::max(i0, 1 + q * bx), hi = std::min(i1, (q + 1) * bx);
      if (lo > hi) continue;
      int rc = prim_inv_var_region(c, err_mach, lo, hi, j0, j1, k0, k1, v, T, cp, ha);
      if (rc) return rc;
    }
    return IZEM_OK;
  }
  return prim_inv_var_region(c, err_mach, i0, i1, j0, j1, k0, k1, v, T, cp, ha);
}

// force_sumY (module_thermodynamics.f90:1709-1860), npv = nvv = 0 branch
void force_sumY(const Ctx& c, int dom, double* v) {
  const Block& b = c.b;
  int i0, i1, j0, j1, k0, k1;
  domain_select(b, dom, i0, i1, j0, j1, k0, k1);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = k0; k <= k1; ++k)
    for (int j = j0; j <= j1; ++j)
      for (int i = i0; i <= i1; ++i) {
        size_t p = b.id(i, j, k);
        double rho = v[p], rho_i = 1.0 / rho, sum = 0.0, Ya;
        for (int l = 0; l < b.nrv - 1; ++l) {
          Ya = v[(NIV + l) * b.ncell + p] * rho_i;
          Ya = std::min(std::max(Ya, 0.0), 1.0);
          v[(NIV + l) * b.ncell + p] = rho * Ya;
          sum = sum + Ya;
        }
        Ya = 1.0 - sum;
        Ya = std::min(std::max(Ya, 0.0), 1.0);
        v[(NIV + b.nrv - 1) * b.ncell + p] = rho * Ya;
      }
}

// ---------------------------------------------------------- halos / BC -----
// comm_cons (module_parallel.f90:1715-1786) for a single periodic block:
// face-only ghost slabs are filled from the opposite interior side.
void comm_periodic(const Block& b, int nvar, double* a, size_t stride) {
#pragma omp parallel for schedule(static)
  for (int l = 0; l < nvar; ++l) {
    double* q = a + l * stride;
    if (b.bc[0] == IZEM_BC_PERIODIC)
      for (int k = 1; k <= b.nz; ++k)
        for (int j = 1; j <= b.ny; ++j)
          for (int g = 1; g <= b.ng; ++g) {
            q[b.id(1 - g, j, k)] = q[b.id(b.nx + 1 - g, j, k)];
            q[b.id(b.nx + g, j, k)] = q[b.id(g, j, k)];
          }
    if (b.bc[2] == IZEM_BC_PERIODIC)
      for (int k = 1; k <= b.nz; ++k)
        for (int g = 1; g <= b.ng; ++g)
          for (int i = 1; i <= b.nx; ++i) {
            q[b.id(i, 1 - g, k)] = q[b.id(i, b.ny + 1 - g, k)];
            q[b.id(i, b.ny + g, k)] = q[b.id(i, g, k)];
          }
    if (b.bc[4] == IZEM_BC_PERIODIC)
      for (int g = 1; g <= b.ng; ++g)
        for (int j = 1; j <= b.ny; ++j)
          for (int i = 1; i <= b.nx; ++i) {
            q[b.id(i, j, 1 - g)] = q[b.id(i, j, b.nz + 1 - g)];
            q[b.id(i, j, b.nz + g)] = q[b.id(i, j, g)];
          }
  }
}

// bc_extrapolation (module_BCs.f90:327-410)
void bc_extrapolation(const Block& b, int face, double* v) {
  for (int l = 0; l < b.nv; ++l) {
    double* q = v + l * b.ncell;
    if (face == 0 || face == 1) {
      for (int k = 1; k <= b.nz; ++k)
        for (int j = 1; j <= b.ny; ++j)
          for (int g = 1; g <= b.ng; ++g) {
            if (face == 0) q[b.id(1 - g, j, k)] = q[b.id(1, j, k)];
            else q[b.id(b.nx + g, j, k)] = q[b.id(b.nx, j, k)];
          }
    } else if (face == 2 || face == 3) {
      for (int k = 1; k <= b.nz; ++k)
        for (int g = 1; g <= b.ng; ++g)
          for (int i = 1; i <= b.nx; ++i) {
            if (face == 2) q[b.id(i, 1 - g, k)] = q[b.id(i, 1, k)];
            else q[b.id(i, b.ny + g, k)] = q[b.id(i, b.ny, k)];
          }
    } else {
      for (int g = 1; g <= b.ng; ++g)
        for (int j = 1; j <= b.ny; ++j)
          for (int i = 1; i <= b.nx; ++i) {
            if (face == 4) q[b.id(i, j, 1 - g)] = q[b.id(i, j, 1)];
            else q[b.id(i, j, b.nz + g)] = q[b.id(i, j, b.nz)];
          }
    }
  }
}

// bc_noreflection (module_BCs.f90:426-512): the ghost points of a
// non-reflecting face take the boundary point's conserved variables times
// 10 (the reference's "garbage" factor); the same loops as bc_extrapolation.
void bc_noreflection(const Block& b, int face, double* v) {
  const double garbage = 10.0;
  for (int l = 0; l < b.nv; ++l) {
    double* q = v + l * b.ncell;
    if (face == 0 || face == 1) {
      for (int k = 1; k <= b.nz; ++k)
        for (int j = 1; j <= b.ny; ++j)
          for (int g = 1; g <= b.ng; ++g) {
            if (face == 0) q[b.id(1 - g, j, k)] = q[b.id(1, j, k)] * garbage;
            else q[b.id(b.nx + g, j, k)] = q[b.id(b.nx, j, k)] * garbage;
          }
    } else if (face == 2 || face == 3) {
      for (int k = 1; k <= b.nz; ++k)
        for (int g = 1; g <= b.ng; ++g)
          for (int i = 1; i <= b.nx; ++i) {
            if (face == 2) q[b.id(i, 1 - g, k)] = q[b.id(i, 1, k)] * garbage;
            else q[b.id(i, b.ny + g, k)] = q[b.id(i, b.ny, k)] * garbage;
          }
    } else {
      for (int g = 1; g <= b.ng; ++g)
        for (int j = 1; j <= b.ny; ++j)
          for (int i = 1; i <= b.nx; ++i) {
            if (face == 4) q[b.id(i, j, 1 - g)] = q[b.id(i, j, 1)] * garbage;
            else q[b.id(i, j, b.nz + g)] = q[b.id(i, j, b.nz)] * garbage;
          }
    }
  }
}

const int kFaceDomain[6] = {-1, 1, -2, 2, -3, 3};
const int kDirichletDomain[6] = {-10, 10, -20, 20, -30, 30};

bool is_dirichlet(int bc) { return bc == IZEM_BC_INFLOWJET || bc == IZEM_BC_NSCBC_OUT; }

// Wmix_i_scalar (module_thermodynamics.f90:739-756)
double wmix_i_scalar(const izem_thd& t, int nrv, const double* Ya) {
  double w = 0.0;
  for (int l = 0; l < nrv; ++l) w = w + Ya[l] * t.Wc_i[l];
  return w;
}

// bc_inflowjet (module_BCs.f90:1646-1791), W face: the underexpanded jet of
// a 1 mm nozzle (nozzle pressure ratio 15, 1000 K, Mach 1.01 at the exit)
// into 300 K air at 20 m/s, tanh profiles in the radius sqrt(y^2 + z^2),
// the nozzle state ramped in with (t / 0.1 ms)^3.  Written at the ghost
// points and the first interior plane.  The reference computes the exit
// sound speed from a mass-fraction array of which only the entries below
// are set; the others are taken as 0.  Species sets of 2, 3 or 9 species.
// Seeded fluctuation of a jet inflow point: uniform in [-1, 1) from a hash
// (splitmix64 finaliser, Steele, Lea and Flood 2014) of the seed, the face
// point, the velocity component and the time interval n (stage time in 1 ns
// units, rounded down).
double jet_noise(unsigned long long seed, int j, int k, int comp, long long n) {
  unsigned long long x = seed ^ ((unsigned long long)(unsigned)j << 40) ^ ((unsigned long long)(unsigned)k << 20) ^
                         ((unsigned long long)comp * 0x9E3779B97F4A7C15ULL) ^ ((unsigned long long)n * 0xD1B54A32D192ED03ULL);
  for (int r = 0; r < 2; ++r) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    x = x ^ (x >> 31);
  }
  return (double)(x >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

// bc_inflowjet with the context's jet parameters (the reference's constants
// by default): round or planar profile, a given or sonic jet velocity, the
// ramp, and the seeded fluctuations when turb > 0.
void bc_inflowjet(const Ctx& c, double time, double* v) {
  const Block& b = c.b;
  const izem_adi& a = c.adi;
  const izem_thd& t = c.thd;
  const izem_jet& jp = c.jet;
  const int nrv = b.nrv;
  const size_t nc = b.ncell;
  const double hbuse = jp.width / a.l_ref, tmaxy = jp.ramp / a.time_ref;
  const double u_2 = jp.u_co / a.u_ref;
  double T_1 = jp.T_jet / a.t_ref;
  const double T_2 = jp.T_co / a.t_ref;
  double P_1 = jp.p_jet / a.p_ref;
  const double P_2 = jp.p_co / a.p_ref;
  double Ya_1 = jp.y_fuel;
  const double Ya_2 = 0.0;
  const double delt = 1.0 / (0.04 * hbuse), y0 = hbuse / 2.0;
  if (tmaxy > 0.0 && time <= tmaxy) {
    P_1 = (P_2 - (P_2 - P_1) * (time / tmaxy) * (time / tmaxy) * (time / tmaxy));
    Ya_1 = (Ya_2 - (Ya_2 - Ya_1) * (time / tmaxy) * (time / tmaxy) * (time / tmaxy));
    T_1 = (T_2 - (T_2 - T_1) * (time / tmaxy) * (time / tmaxy) * (time / tmaxy));
  }
  double Ya[IZEM_NSMAX] = {};
  if (nrv == 2) { Ya[0] = 0.233; Ya[1] = 0.767; }
  else if (nrv == 3) { Ya[0] = Ya_1; Ya[1] = 0.0; Ya[2] = 1.0 - Ya_1; }
  else { Ya[1] = Ya_1; Ya[3] = 0.0; Ya[8] = 1.0 - Ya_1; }
  double Ws_i = wmix_i_scalar(t, nrv, Ya);
  const double cps = cp_scalar(t, T_1, Ya);
  double gamma = t.gam2 * Ws_i / cps;
  gamma = 1.0 / (1.0 - gamma);
  const double cs = std::sqrt(gamma * Ws_i * T_1);
  const double u1p = jp.u_jet / a.u_ref;
  const double u_1 = u1p > 0.0 ? u1p : 1.01 * cs;
  for (int k = 1; k <= b.nz; ++k)
    for (int j = 1; j <= b.ny; ++j)
      for (int i = 1 - b.ng; i <= 1; ++i) {
        const double y = c.crd[1][j - 1], z = c.crd[2][k - 1];
        const double rrr = jp.planar ? std::fabs(y) : std::sqrt(y * y + z * z);
        const double th = std::tanh((rrr - y0) * delt);
        double ux = 0.5 * ((u_1 + u_2) - (u_1 - u_2) * th);
        double vy = 0.0, wz = 0.0;
        if (jp.turb > 0.0) {
          const double am = jp.turb * u_1 * (0.5 * (1.0 - th));
          const long long n = (long long)std::floor(time * (a.time_ref / 1.0e-9));
          ux = ux + am * jet_noise(jp.seed, j, k, 0, n);
          vy = am * jet_noise(jp.seed, j, k, 1, n);
          wz = am * jet_noise(jp.seed, j, k, 2, n);
        }
        const double T = 0.5 * ((T_1 + T_2) - (T_1 - T_2) * th);
        const double P = 0.5 * ((P_1 + P_2) - (P_1 - P_2) * th);
        for (int l = 0; l < nrv; ++l) Ya[l] = 0.0;
        if (nrv == 2) {
          Ya[0] = 0.233;
          Ya[1] = 1.0 - Ya[0];
        } else if (nrv == 3) {
          Ya[0] = 0.5 * ((Ya_1 + 0.0) - (Ya_1 - 0.0) * th);
          Ya[1] = 0.5 * ((0.0 + 0.233) - (0.0 - 0.233) * th);
          Ya[2] = 0.5 * ((1.0 - Ya_1 + 0.767) - (1.0 - Ya_1 - 0.767) * th);
        } else {
          Ya[1] = 0.5 * ((Ya_1 + 0.0) - (Ya_1 - 0.0) * th);
          Ya[3] = 0.5 * ((0.0 + 0.233) - (0.0 - 0.233) * th);
          Ya[8] = 0.5 * ((1.0 - Ya_1 + 0.767) - (1.0 - Ya_1 - 0.767) * th);
        }
        Ws_i = wmix_i_scalar(t, nrv, Ya);
        const double rho = P / (T * Ws_i);
        double has[IZEM_NSMAX];
        ha_scalar(t, T, has);
        double hm = 0.0;
        for (int l = 0; l < nrv; ++l) hm = hm + has[l] * Ya[l];
        const size_t p = b.id(i, j, k);
        v[p] = rho;
        v[nc + p] = rho * ux;
        v[2 * nc + p] = rho * vy;
        v[3 * nc + p] = rho * wz;
        v[4 * nc + p] = rho * hm - P + 0.5 * rho * (ux * ux + vy * vy + wz * wz);
        for (int l = 0; l < nrv; ++l) v[(NIV + l) * nc + p] = rho * Ya[l];
      }
}

// bc_nscbc_out (module_BCs.f90:2331-2516), E face: characteristic outflow
// with 4th-order one-sided derivatives at the last interior point, the
// incoming wave relaxed toward 94232.25 Pa (sigma 0.28, the domain length
// Lx); the same updated state, advanced by dt, at the last interior plane
// and the ghost points.
void bc_nscbc_out(const Ctx& c, double dtime, const double* T, const double* W_i, const double* cp, double* v) {
  const Block& b = c.b;
  const izem_adi& a = c.adi;
  const izem_thd& t = c.thd;
  const int nrv = b.nrv;
  const size_t nc = b.ncell;
  const double Pinf = c.jet.p_far / a.p_ref, sigma1 = 0.28, Lx = c.lx;
  static const double a4or[5] = {-3.0 / 12.0, 16.0 / 12.0, -36.0 / 12.0, 48.0 / 12.0, -25.0 / 12.0};   // m = -4..0
  const int ex = b.nx;
  const double dxe = c.dxi[0][ex - 1 + b.ng];
  for (int k = 1; k <= b.nz; ++k)
    for (int j = 1; j <= b.ny; ++j) {
      double Machm = 0.0;
      size_t p = b.id(ex, j, k);
      double rho = v[p], rho_i = 1.0 / rho;
      double ux = v[nc + p] * rho_i, vy = v[2 * nc + p] * rho_i, wz = v[3 * nc + p] * rho_i;
      double Pres = v[p] * T[p] * W_i[p];
      double gam = t.gam2 * W_i[p] / cp[p];
      gam = 1.0 / (1.0 - gam);
      double cs = std::sqrt(gam * Pres * rho_i);
      const double Mach = std::sqrt(ux * ux + vy * vy + wz * wz) / cs;
      Machm = std::max(Machm, Mach);
      double drho = 0.0, dux = 0.0, dvy = 0.0, dwz = 0.0, dPres = 0.0;
      double Ya[IZEM_NSMAX], dYa[IZEM_NSMAX] = {};
      for (int m = -4; m <= 0; ++m) {
        const size_t q = b.id(ex + m, j, k);
        rho = v[q];
        rho_i = 1.0 / rho;
        ux = v[nc + q] * rho_i;
        vy = v[2 * nc + q] * rho_i;
        wz = v[3 * nc + q] * rho_i;
        Pres = v[q] * T[q] * W_i[q];
        for (int l = 0; l < nrv; ++l) Ya[l] = v[(NIV + l) * nc + q] * rho_i;
        const double w = a4or[m + 4];
        drho = drho + w * rho;
        dux = dux + w * ux;
        dvy = dvy + w * vy;
        dwz = dwz + w * wz;
        dPres = dPres + w * Pres;
        for (int l = 0; l < nrv; ++l) dYa[l] = dYa[l] + w * Ya[l];
      }
      drho = -drho * dxe;
      dux = -dux * dxe;
      dvy = -dvy * dxe;
      dwz = -dwz * dxe;
      dPres = -dPres * dxe;
      for (int l = 0; l < nrv; ++l) dYa[l] = -dYa[l] * dxe;
      double L1 = 0.0, L2 = 0.0, L3 = 0.0, L4 = 0.0, L5 = 0.0, L5_Ya[IZEM_NSMAX] = {};
      gam = t.gam2 * W_i[p] / cp[p];
      gam = 1.0 / (1.0 - gam);
      cs = std::sqrt(gam * Pres * rho_i);
      if (ux - cs < 0.0) L1 = sigma1 * (1.0 - Machm * Machm) * cs / Lx * (Pres - Pinf);
      else L1 = (ux - cs) * (dPres - rho * cs * dux);
      if (ux + cs > 0.0) L5 = (ux + cs) * (dPres + rho * cs * dux);
      else L5 = (ux + cs) * (2.0 * dPres - L1 / (ux - cs));
      if (ux > 0.0) {
        L2 = ux * (cs * cs * drho - dPres);
        L3 = ux * dvy;
        L4 = ux * dwz;
        for (int l = 0; l < nrv; ++l) L5_Ya[l] = ux * dYa[l];
      } else {
        L2 = ux * cs * cs * drho - 0.5 * ux * (L5 / (ux + cs) + L1 / (ux - cs));
      }
      const double d2 = 0.5 * (L5 + L1);
      const double d1 = (L2 + d2) / (cs * cs);
      const double d3 = 0.5 * (L5 - L1) / (cs * rho);
      const double d4 = L3, d5 = L4;
      double has[IZEM_NSMAX];
      ha_scalar(t, T[p], has);
      double hm = 0.0;
      for (int l = 0; l < nrv; ++l) hm = hm + has[l] * Ya[l];
      const double kin = ux * ux + vy * vy + wz * wz;
      for (int i = ex; i <= ex + b.ng; ++i) {
        const size_t o = b.id(i, j, k);
        v[o] = rho - d1 * dtime;
        v[nc + o] = (rho * ux) - (ux * d1 + rho * d3) * dtime;
        v[2 * nc + o] = (rho * vy) - (vy * d1 + rho * d4) * dtime;
        v[3 * nc + o] = (rho * wz) - (wz * d1 + rho * d5) * dtime;
        v[4 * nc + o] = (rho * hm - Pres + 0.5 * rho * kin) -
                        (0.5 * kin * d1 + rho * (ux * d3 + vy * d4 + wz * d5) + d2 / (gam - 1.0)) * dtime;
        for (int l = 0; l < nrv; ++l) v[(NIV + l) * nc + o] = (rho * Ya[l]) - (Ya[l] * d1 + rho * L5_Ya[l]) * dtime;
      }
    }
}

// comm_cons + upd_boundaries + upd_prim_var_ghost (module_BCs.f90:41-296):
// the closure of the ghost points after the interior changed.  time and dt
// are what upd_boundaries is given (the jet faces read them).
int update_boundaries(Ctx& c, double* v, double* T, double* W_i, double* cp, double* ha, double time, double dt) {
  const Block& b = c.b;
  int rc = IZEM_OK;
  comm_periodic(b, b.nv, v, b.ncell);
  for (int f = 0; f < 6; ++f) {
    if (!b.bnd[f]) continue;
    if (b.bc[f] == IZEM_BC_EXTRAPOLATION) bc_extrapolation(b, f, v);
    else if (b.bc[f] == IZEM_BC_NOREFLECTION) bc_noreflection(b, f, v);
    else if (b.bc[f] == IZEM_BC_INFLOWJET) bc_inflowjet(c, time, v);
    else if (b.bc[f] == IZEM_BC_NSCBC_OUT) bc_nscbc_out(c, dt, T, W_i, cp, v);
    if (is_dirichlet(b.bc[f])) {   // upd_prim_var_dirichlet
      if (c.cfg.forcesum) force_sumY(c, kDirichletDomain[f], v);
      if ((rc = prim_inv_var(c, kDirichletDomain[f], false, v, W_i, T, cp, ha))) return rc;
    }
  }
  for (int f = 0; f < 6; ++f) {
    if (c.cfg.forcesum) force_sumY(c, kFaceDomain[f], v);
    rc = prim_inv_var(c, kFaceDomain[f], false, v, W_i, T, cp, ha);
    if (rc) return rc;
  }
  return IZEM_OK;
}

// upd_prim_var_domain, then the ghost closure (module_solver.f90:839-845)
// time: the stage time given to upd_boundaries; dt: the step.
int update_primitives(Ctx& c, double* v, double* T, double* W_i, double* cp, double* ha, double time = 0.0,
                      double dt = 0.0) {
  if (c.cfg.forcesum) force_sumY(c, 0, v);
  int rc = prim_inv_var(c, 0, false, v, W_i, T, cp, ha);
  if (rc) return rc;
  return update_boundaries(c, v, T, W_i, cp, ha, time, dt);
}

// closure of the initial conditions (module_ICs.f90:2874-2879)
int finalize_ic(Ctx& c, double* v, double* T, double* W_i, double* cp, double* ha) {
  const Block& b = c.b;
  comm_periodic(b, b.nv, v, b.ncell);
  int rc = prim_inv_var(c, 0, true, v, W_i, T, cp, ha);
  if (rc) return rc;
  for (int f = 0; f < 6; ++f) bc_extrapolation(b, f, v);   // upd_extrapolation: every face
  for (int f = 0; f < 6; ++f) {
    rc = prim_inv_var(c, kFaceDomain[f], true, v, W_i, T, cp, ha);
    if (rc) return rc;
  }
  return IZEM_OK;
}

// ------------------------------------------------------------ derivatives --
// module_deriv.f90 coefficient tables (:25-66)
const double alpha6[7] = {-1.0 / 60.0, 9.0 / 60.0, -45.0 / 60.0, 0.0, 45.0 / 60.0, -9.0 / 60.0, 1.0 / 60.0};
const double alpha8[9] = {3.0 / 840.0,    -32.0 / 840.0, 168.0 / 840.0, -672.0 / 840.0, 0.0,
                          672.0 / 840.0,  -168.0 / 840.0, 32.0 / 840.0, -3.0 / 840.0};
const double alph4[5] = {1.0 / 12.0, -8.0 / 12.0, 0.0, 8.0 / 12.0, -1.0 / 12.0};
const double alph4ol[5] = {-25.0 / 12.0, 48.0 / 12.0, -36.0 / 12.0, 16.0 / 12.0, -3.0 / 12.0};   // l = 0..4
const double alph4ul[5] = {-3.0 / 12.0, -10.0 / 12.0, 18.0 / 12.0, -6.0 / 12.0, 1.0 / 12.0};    // l = -1..3
const double alph4ur[5] = {1.0 / 12.0, -6.0 / 12.0, 18.0 / 12.0, -10.0 / 12.0, -3.0 / 12.0};    // l = -3..1
const double alph4or[5] = {-3.0 / 12.0, 16.0 / 12.0, -36.0 / 12.0, 48.0 / 12.0, -25.0 / 12.0}; // l = -4..0

// dx/dy/dz, d?_fixed1, d?_fixed2 (module_deriv.f90:212-2354): the three
// families share one arithmetic; `out_interior` selects the interior-sized
// output of d?_fixed2.  Only interior points are written.  Interior and
// inter-block points use the 6th-order (ng = 3) or 8th-order (ng = 4)
// central stencil; next to a physical boundary the rows are 4th order and,
// with ng = 4, the fourth row is 6th order.  In a 2-D run (ndim = 2) there
// is no z derivative: the reference's 2-D routines (viscflux_xy) have no z
// term, and a zero z derivative reproduces them.
void deriv(const Ctx& c, int d, const double* in, double* out, bool out_interior) {
  const Block& b = c.b;
  const int n = b.n(d), ng = b.ng;
  const double* di = c.dxi[d].data();
  const bool lo_b = b.bnd[2 * d], hi_b = b.bnd[2 * d + 1];
  const bool none = d == 2 && c.cfg.ndim == 2;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k <= b.nz; ++k)
    for (int j = 1; j <= b.ny; ++j)
      for (int i = 1; i <= b.nx; ++i) {
        int s = d == 0 ? i : (d == 1 ? j : k);
        auto at = [&](int off) {
          int ii = i, jj = j, kk = k;
          if (d == 0) ii += off; else if (d == 1) jj += off; else kk += off;
          return in[b.id(ii, jj, kk)];
        };
        double dd = 0.0, res;
        double dis = di[s - 1 + ng];
        if (none) {
          res = 0.0;
        } else if (lo_b && s == 1) {
          for (int l = 0; l <= 4; ++l) dd = dd + alph4ol[l] * at(l);
          res = dd * dis;
        } else if (lo_b && s == 2) {
          for (int l = -1; l <= 3; ++l) dd = dd + alph4ul[l + 1] * at(l);
          res = dd * dis;
        } else if (lo_b && s == 3) {
          for (int l = -2; l <= 2; ++l) dd = dd + alph4[l + 2] * at(l);
          res = dd * dis;
        } else if (ng == 4 && ((lo_b && s == 4) || (hi_b && s == n - 3))) {
          for (int l = -3; l <= 3; ++l) dd = dd + alpha6[l + 3] * at(l);
          res = dd * dis;
        } else if (hi_b && s == n - 2) {
          for (int l = -2; l <= 2; ++l) dd = dd + alph4[l + 2] * at(l);
          res = dd * dis;
        } else if (hi_b && s == n - 1) {
          for (int l = -3; l <= 1; ++l) dd = dd + alph4ur[l + 3] * at(l);
          res = -dd * dis;
        } else if (hi_b && s == n) {
          for (int l = -4; l <= 0; ++l) dd = dd + alph4or[l + 4] * at(l);
          res = -dd * dis;
        } else if (ng == 4) {
          for (int l = -4; l <= 4; ++l) dd = dd + alpha8[l + 4] * at(l);
          res = dd * dis;
        } else {
          for (int l = -3; l <= 3; ++l) dd = dd + alpha6[l + 3] * at(l);
          res = dd * dis;
        }
        if (out_interior) out[b.fid(i, j, k)] = res;
        else out[b.id(i, j, k)] = res;
      }
}

// compute_duixj + shock_sensor_ducros (module_tools.f90:2521-2719): the
// velocity gradients by dx_fixed1 / dy_fixed1 / dz_fixed1 of u = rho u * (1 /
// rho), then the sticky flag where (div u)^2 / ((div u)^2 + |curl u|^2 +
// eps30) > DUCROS_TREDUC.  The velocities are formed on every point with a
// density (the reference forms them on the interior and the face slabs,
// which are all that the derivatives read).
void shock_sensor_ducros(const Ctx& c, const double* v, uint8_t* sensor) {
  const Block& b = c.b;
  const int nd = c.cfg.ndim;
  const size_t nc = b.ncell, ni = b.nint;
  std::vector<double> u(3 * nc, 0.0), du(9 * ni, 0.0);
  for (size_t p = 0; p < nc; ++p) {
    if (v[p] == 0.0) continue;
    const double rho_i = 1.0 / v[p];
    for (int a = 0; a < 3; ++a) u[a * nc + p] = v[(1 + a) * nc + p] * rho_i;
  }
  // duixj (.., a nd + d + 1) = d u_a / d x_d: (1) du/dx (2) du/dy [(3) du/dz] ...
  for (int a = 0; a < nd; ++a)
    for (int d = 0; d < nd; ++d) deriv(c, d, u.data() + a * nc, du.data() + (a * nd + d) * ni, true);
  const double eps30 = 1.0e-30;
  for (int k = 1; k <= b.nz; ++k)
    for (int j = 1; j <= b.ny; ++j)
      for (int i = 1; i <= b.nx; ++i) {
        const size_t f = b.fid(i, j, k);
        auto D = [&](int q) { return du[(q - 1) * ni + f]; };
        double div, vort, wrk;
        if (nd == 3) {
          div = D(1) + D(5) + D(9);
          div = div * div;
          wrk = D(8) - D(6);
          vort = wrk * wrk;
          wrk = D(3) - D(7);
          wrk = wrk * wrk;
          vort = vort + wrk;
          wrk = D(4) - D(2);
          wrk = wrk * wrk;
          vort = vort + wrk;
        } else {
          div = D(1) + D(4);
          div = div * div;
          wrk = D(3) - D(2);
          vort = wrk * wrk;
        }
        const double ducloc = div / (div + vort + eps30);
        if (ducloc > c.ducros_treduc) sensor[b.id(i, j, k)] = 1;
      }
}

// ------------------------------------------------------------------ WENO ---
struct Weno {
  int ng;
  double cweno[5][4];  // cweno(-1:ng-1, 0:ng-1) stored at [r+1][j]
  double dweno[4], dtweno[4];
  double z1, z2, za, zb, zc, zd, ze, zf, zg, zh, zi, zl, zm, zn, zo, zp, zq, zr, zs, zt, zu;
};

// wenopar (module_weno.f90:60-225): ng = 4 (7th order) and ng = 3 (5th order)
Weno wenopar(int ng) {
  Weno w{};
  w.ng = ng;
  if (ng == 4) {
    const double c[5][4] = {{25.0 / 12.0, -23.0 / 12.0, 13.0 / 12.0, -1.0 / 4.0},
                            {1.0 / 4.0, 13.0 / 12.0, -5.0 / 12.0, 1.0 / 12.0},
                            {-1.0 / 12.0, 7.0 / 12.0, 7.0 / 12.0, -1.0 / 12.0},
                            {1.0 / 12.0, -5.0 / 12.0, 13.0 / 12.0, 1.0 / 4.0},
                            {-1.0 / 4.0, 13.0 / 12.0, -23.0 / 12.0, 25.0 / 12.0}};
    for (int r = 0; r < 5; ++r)
      for (int j = 0; j < 4; ++j) w.cweno[r][j] = c[r][j];
    w.dweno[0] = 4.0 / 35.0; w.dweno[1] = 18.0 / 35.0; w.dweno[2] = 12.0 / 35.0; w.dweno[3] = 1.0 / 35.0;
    for (int r = 0; r < 4; ++r) w.dtweno[r] = w.dweno[3 - r];
    w.za = 547.0; w.zb = -1854.0; w.zc = 4642.0; w.zd = -3882.0; w.ze = -17246.0; w.zf = 2107.0;
    w.zg = 7043.0; w.zh = -9402.0; w.zi = 11003.0; w.zl = 7042.0; w.zm = 3443.0; w.zn = -5966.0;
    w.zo = -2522.0; w.zp = 1602.0; w.zq = 2843.0; w.zr = 267.0; w.zs = 1922.0; w.zt = -494.0; w.zu = -1642.0;
    return w;
  }
  w.cweno[0][0] = 11.0 / 6.0; w.cweno[0][1] = -7.0 / 6.0; w.cweno[0][2] = 1.0 / 3.0;
  w.cweno[1][0] = 1.0 / 3.0;  w.cweno[1][1] = 5.0 / 6.0;  w.cweno[1][2] = -1.0 / 6.0;
  w.cweno[2][0] = -1.0 / 6.0; w.cweno[2][1] = 5.0 / 6.0;  w.cweno[2][2] = 1.0 / 3.0;
  w.cweno[3][0] = 1.0 / 3.0;  w.cweno[3][1] = -7.0 / 6.0; w.cweno[3][2] = 11.0 / 6.0;
  w.dweno[0] = 3.0 / 10.0; w.dweno[1] = 3.0 / 5.0; w.dweno[2] = 1.0 / 10.0;
  w.dtweno[0] = w.dweno[2]; w.dtweno[1] = w.dweno[1]; w.dtweno[2] = w.dweno[0];
  w.z1 = 13.0 / 12.0; w.z2 = 1.0 / 4.0; w.za = -2.0; w.zb = -4.0; w.zc = 3.0; w.zd = -1.0;
  return w;
}

// wenorec_nw (module_weno.f90:236-275).  vp/vm are 1-based arrays of length
// 2ng.  For ng = 3, `fix` selects the textbook upwind-biased stencil
// instead of the reference's mirrored one; the ng = 4 stencil is the
// textbook 7th-order one in the reference already.
void wenorec_nw(int ng, const double* vp, const double* vm, double& vminus, double& vplus, bool fix) {
  if (ng == 4) {
    const double denom = 1.0 / 420.0;
    vminus = (-3.0 * vp[1] + 25.0 * vp[2] - 101.0 * vp[3] + 319.0 * vp[4] + 214.0 * vp[5] - 38.0 * vp[6] +
              4.0 * vp[7]) * denom;
    vplus = (-3.0 * vm[8] + 25.0 * vm[7] - 101.0 * vm[6] + 319.0 * vm[5] + 214.0 * vm[4] - 38.0 * vm[3] +
             4.0 * vm[2]) * denom;
    return;
  }
  const double denom = 1.0 / 60.0;
  if (!fix) {
    vminus = (-3.0 * vp[1] + 27.0 * vp[2] + 47.0 * vp[3] - 13.0 * vp[4] + 2.0 * vp[5]) * denom;
    vplus = (-3.0 * vm[6] + 27.0 * vm[5] + 47.0 * vm[4] - 13.0 * vm[3] + 2.0 * vm[2]) * denom;
  } else {
    vminus = (2.0 * vp[1] - 13.0 * vp[2] + 47.0 * vp[3] + 27.0 * vp[4] - 3.0 * vp[5]) * denom;
    vplus = (2.0 * vm[6] - 13.0 * vm[5] + 47.0 * vm[4] + 27.0 * vm[3] - 3.0 * vm[2]) * denom;
  }
}

// wenorec (module_weno.f90:286-527): nonlinear reconstruction of the '-'
// state from vp (stencil centre i = ng) and of the '+' state from vm
// (centre i = ng + 1), 1-based arrays of length 2ng.
void wenorec(const Weno& w, const double* vp, const double* vm, double& vminus, double& vplus) {
  const double eps_weno = 1.0e-10;
  const int ng = w.ng;
  double vpr[4], vmr[4], beta[4], alfa[4], omega[4], sum;
  auto betas = [&](const double* q, int ii) {
    if (ng == 4) {
      beta[0] = q[ii] * (w.zf * q[ii] + w.zh * q[ii + 1] + w.zl * q[ii + 2] + w.zb * q[ii + 3]) +
                q[ii + 1] * (w.zi * q[ii + 1] + w.ze * q[ii + 2] + w.zc * q[ii + 3]) +
                q[ii + 2] * (w.zg * q[ii + 2] + w.zd * q[ii + 3]) + q[ii + 3] * (w.za * q[ii + 3]);
      beta[1] = q[ii - 1] * (w.za * q[ii - 1] + w.zo * q[ii] + w.zs * q[ii + 1] + w.zt * q[ii + 2]) +
                q[ii] * (w.zm * q[ii] + w.zn * q[ii + 1] + w.zp * q[ii + 2]) +
                q[ii + 1] * (w.zq * q[ii + 1] + w.zu * q[ii + 2]) + q[ii + 2] * (w.zr * q[ii + 2]);
      beta[2] = q[ii - 2] * (w.zr * q[ii - 2] + w.zu * q[ii - 1] + w.zp * q[ii] + w.zt * q[ii + 1]) +
                q[ii - 1] * (w.zq * q[ii - 1] + w.zn * q[ii] + w.zs * q[ii + 1]) +
                q[ii] * (w.zm * q[ii] + w.zo * q[ii + 1]) + q[ii + 1] * (w.za * q[ii + 1]);
      beta[3] = q[ii - 3] * (w.za * q[ii - 3] + w.zd * q[ii - 2] + w.zc * q[ii - 1] + w.zb * q[ii]) +
                q[ii - 2] * (w.zg * q[ii - 2] + w.ze * q[ii - 1] + w.zl * q[ii]) +
                q[ii - 1] * (w.zi * q[ii - 1] + w.zh * q[ii]) + q[ii] * (w.zf * q[ii]);
      return;
    }
    double a = q[ii] + w.za * q[ii + 1] + q[ii + 2];
    double bq = w.zc * q[ii] + w.zb * q[ii + 1] + q[ii + 2];
    beta[0] = w.z1 * a * a + w.z2 * bq * bq;
    a = q[ii - 1] + w.za * q[ii] + q[ii + 1];
    bq = q[ii - 1] + w.zd * q[ii + 1];
    beta[1] = w.z1 * a * a + w.z2 * bq * bq;
    a = q[ii - 2] + w.za * q[ii - 1] + q[ii];
    bq = q[ii - 2] + w.zb * q[ii - 1] + w.zc * q[ii];
    beta[2] = w.z1 * a * a + w.z2 * bq * bq;
  };
  int i = ng;
  for (int r = 0; r < ng; ++r) {
    vpr[r] = 0.0;
    for (int j = 0; j < ng; ++j) vpr[r] = vpr[r] + w.cweno[r + 1][j] * vp[i - r + j];
  }
  betas(vp, i);
  sum = 0.0;
  for (int r = 0; r < ng; ++r) {
    alfa[r] = w.dweno[r] / ((eps_weno + beta[r]) * (eps_weno + beta[r]));
    sum = sum + alfa[r];
  }
  sum = 1.0 / sum;
  for (int r = 0; r < ng; ++r) omega[r] = alfa[r] * sum;
  vminus = 0.0;
  for (int r = 0; r < ng; ++r) vminus = vminus + omega[r] * vpr[r];

  i = ng + 1;
  for (int r = 0; r < ng; ++r) {
    vmr[r] = 0.0;
    for (int j = 0; j < ng; ++j) vmr[r] = vmr[r] + w.cweno[r][j] * vm[i - r + j];
  }
  betas(vm, i);
  sum = 0.0;
  for (int r = 0; r < ng; ++r) {
    alfa[r] = w.dtweno[r] / ((eps_weno + beta[r]) * (eps_weno + beta[r]));
    sum = sum + alfa[r];
  }
  sum = 1.0 / sum;
  for (int r = 0; r < ng; ++r) omega[r] = alfa[r] * sum;
  vplus = 0.0;
  for (int r = 0; r < ng; ++r) vplus = vplus + omega[r] * vmr[r];
}

// The left and right characteristic vectors of the flux Jacobian along
// axis d at one state: euler_LLF_x/_y/_z build them at the Roe state
// (module_weno.f90:775-951), bc_noreflectionweno at a boundary point's own
// state (:2224-2418, and the same blocks for the other faces).
struct CharState {
  double uc[3];
  const double* Yc;
  const double* psi_c;
  double ht_c, q, cs_c, cs_c_i, b1, b2, xi;
};

void char_vectors(int d, int nv, int nrv, const CharState& cs, double el[][IZEM_NSMAX + 5],
                  double er[][IZEM_NSMAX + 5]) {
  const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
  const double* uc = cs.uc;
  const double* Yc = cs.Yc;
  const double* psi_c = cs.psi_c;
  const double ht_c = cs.ht_c, q = cs.q, cs_c = cs.cs_c, cs_c_i = cs.cs_c_i, b1 = cs.b1, b2 = cs.b2, xi = cs.xi;
  const double un = uc[d];
  double wrk;
  // left eigenvectors (module_weno.f90:775-874)
  for (int a = 0; a < nv; ++a)
    for (int e = 0; e < nv; ++e) el[a][e] = 0.0;
  el[0][0] = 0.5 * (b1 + un * cs_c_i);
  el[2][0] = 0.5 * (b1 - un * cs_c_i);
  for (int a = 0; a < 3; ++a) {
    if (a == d) {
      el[0][1 + a] = -0.5 * (b2 * un + cs_c_i);
      el[2][1 + a] = -0.5 * (b2 * un - cs_c_i);
    } else {
      el[0][1 + a] = -0.5 * (b2 * uc[a]);
      el[2][1 + a] = -0.5 * (b2 * uc[a]);
    }
    el[1][1 + a] = b2 * uc[a];
  }
  el[0][4] = 0.5 * b2; el[2][4] = 0.5 * b2;
  el[1][0] = 1.0 - b1; el[1][4] = -b2;
  el[3][0] = -uc[t1]; el[3][1 + t1] = 1.0;
  el[4][0] = -uc[t2]; el[4][1 + t2] = 1.0;
  wrk = 0.5 * b2;
  for (int l = NIV; l < nv; ++l) el[0][l] = wrk * psi_c[l - NIV];
  for (int l = NIV; l < nv; ++l) el[1][l] = -el[0][l] - el[0][l];
  for (int l = NIV; l < nv; ++l) el[2][l] = el[0][l];
  el[5][0] = (1 + xi) * q;
  for (int a = 0; a < 3; ++a) el[5][1 + a] = -(1 + xi) * uc[a];
  el[5][4] = (1 + xi);
  for (int l = NIV; l < nv; ++l) el[5][l] = xi * psi_c[l - NIV];
  for (int l = 6; l < nv; ++l) {
    double Y = Yc[l - 6];
    el[l][0] = -b1 * Y;
    for (int a = 0; a < 3; ++a) el[l][1 + a] = b2 * uc[a] * Y;
    el[l][4] = -b2 * Y;
  }
  for (int s1 = 1; s1 <= nrv - 1; ++s1)
    for (int s2 = 1; s2 <= nrv; ++s2) el[s1 + 5][s2 + 4] = -b2 * Yc[s1 - 1] * psi_c[s2 - 1];
  for (int l = 1; l <= nrv - 1; ++l) el[l + 5][l + 4] = el[l + 5][l + 4] + 1.0;
  // right eigenvectors (module_weno.f90:881-951)
  for (int a = 0; a < nv; ++a)
    for (int e = 0; e < nv; ++e) er[a][e] = 0.0;
  er[0][0] = 1.0; er[0][1] = 1.0; er[0][2] = 1.0;
  er[1 + d][0] = un - cs_c; er[1 + d][1] = un; er[1 + d][2] = un + cs_c;
  er[1 + t1][0] = uc[t1]; er[1 + t1][1] = uc[t1]; er[1 + t1][2] = uc[t1]; er[1 + t1][3] = 1.0;
  er[1 + t2][0] = uc[t2]; er[1 + t2][1] = uc[t2]; er[1 + t2][2] = uc[t2]; er[1 + t2][4] = 1.0;
  er[4][0] = ht_c - un * cs_c; er[4][1] = q; er[4][2] = ht_c + un * cs_c; er[4][3] = uc[t1]; er[4][4] = uc[t2];
  for (int l = NIV; l < nv; ++l) { er[l][0] = Yc[l - NIV]; er[l][2] = Yc[l - NIV]; }
  for (int l = NIV + 1; l <= nv; ++l) er[l - 2][l - 1] = 1.0;
  er[nv - 1][5] = -1.0 / psi_c[nrv - 1];
  wrk = -1.0 / psi_c[nrv - 1];
  for (int l = 1; l <= nrv - 1; ++l) er[nv - 1][l + 5] = wrk * psi_c[l - 1];
}

// euler_LLF_x/_y/_z (module_weno.f90:537-1044, 1055-1590, 1595-2125).
// The three routines differ only in the sweep axis d and in which velocity
// components are normal / tangential; they are restated once over d.
int euler_flux(Ctx& c, int d, const double* v, const double* T, const double* W_i, const double* cp,
               const double* ha, const uint8_t* sensor, double* fl) {
  const Block& b = c.b;
  const izem_thd& t = c.thd;
  const int ng = b.ng, nv = b.nv, nrv = b.nrv, st_m1 = 2 * ng;
  const size_t nc = b.ncell;
  const Weno w = wenopar(ng);
  const int n = b.n(d);
  const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;  // tangential components
  const double* di = c.dxi[d].data();
  const bool fixlin = c.cfg.weno5_linear_fix != 0;
  int m1 = d == 0 ? b.ny : b.nx, m2 = d == 2 ? b.ny : b.nz;
  bool negp = false;
  // MPI block of a point along the sweep (x only; ghosts belong to the edge blocks)
  const int nxb = d == 0 ? std::max(c.sensor_xblocks, 1) : 1, bxs = n / nxb;
  auto xblk = [&](int s) { return (std::min(std::max(s, 1), n) - 1) / bxs; };
#pragma omp parallel for collapse(2) schedule(dynamic)
  for (int q2 = 1; q2 <= m2; ++q2)
    for (int q1 = 1; q1 <= m1; ++q1) {
      auto cell = [&](int s) {
        if (d == 0) return b.id(s, q1, q2);
        if (d == 1) return b.id(q1, s, q2);
        return b.id(q1, q2, s);
      };
      const int len = n + 2 * ng;
      std::vector<double> rho_i(len), uu[3], P(len), gam(len), cs(len), ht(len), et(len), Ya(len * nrv);
      for (int a = 0; a < 3; ++a) uu[a].assign(len, 0.0);
      std::vector<double> fhat((n + 1) * nv), fhatR((n + 1) * nv);
      auto ix = [&](int s) { return s - 1 + ng; };
      for (int s = 1 - ng; s <= n + ng; ++s) {
        size_t p = cell(s);
        rho_i[ix(s)] = 1.0 / v[p];
        uu[d][ix(s)] = v[(1 + d) * nc + p] * rho_i[ix(s)];
        P[ix(s)] = v[p] * T[p] * W_i[p];
        if (P[ix(s)] <= 0.0) {
#pragma omp atomic write
          negp = true;
        }
        gam[ix(s)] = t.gam2 * W_i[p] / cp[p];
        gam[ix(s)] = 1.0 / (1.0 - gam[ix(s)]);
        cs[ix(s)] = std::sqrt(gam[ix(s)] * P[ix(s)] * rho_i[ix(s)]);
      }
      for (int s = 0; s <= n + 1; ++s) {
        size_t p = cell(s);
        uu[t1][ix(s)] = v[(1 + t1) * nc + p] * rho_i[ix(s)];
        uu[t2][ix(s)] = v[(1 + t2) * nc + p] * rho_i[ix(s)];
        for (int l = 0; l < nrv; ++l) Ya[ix(s) * nrv + l] = v[(NIV + l) * nc + p] * rho_i[ix(s)];
        double h = 0.0;
        for (int l = 0; l < nrv; ++l) h = h + ha[l * nc + p] * Ya[ix(s) * nrv + l];
        double ux = uu[0][ix(s)], vy = uu[1][ix(s)], wz = uu[2][ix(s)];
        ht[ix(s)] = h + 0.5 * (ux * ux + vy * vy + wz * wz);
        et[ix(s)] = v[4 * nc + p] * rho_i[ix(s)];
      }
      double f_s[9][2 * IZEM_NSMAX + 6], L_s[9][2 * IZEM_NSMAX + 6];
      double el[IZEM_NSMAX + 5][IZEM_NSMAX + 5], er[IZEM_NSMAX + 5][IZEM_NSMAX + 5];
      double gplus[9], gminus[9], ghat[IZEM_NSMAX + 5];
      for (int il = 0; il <= n; ++il) {
        int ir = il + 1;
        for (int st = 1; st <= st_m1; ++st) {
          int is = il + st - ng;
          size_t p = cell(is);
          double un = uu[d][ix(is)];
          f_s[st][0] = v[(1 + d) * nc + p];
          for (int a = 0; a < 3; ++a) f_s[st][1 + a] = v[(1 + a) * nc + p] * un;
          f_s[st][1 + d] = v[(1 + d) * nc + p] * un + P[ix(is)];
          f_s[st][4] = un * (v[4 * nc + p] + P[ix(is)]);
          for (int l = NIV; l < nv; ++l) f_s[st][l] = v[l * nc + p] * un;
          L_s[st][0] = std::fabs(un - cs[ix(is)]);
          L_s[st][1] = std::fabs(un);
          L_s[st][2] = std::fabs(un + cs[ix(is)]);
          for (int l = 3; l < nv; ++l) L_s[st][l] = L_s[st][1];
        }
        // Roe's average (module_weno.f90:726-761)
        size_t pl = cell(il), pr = cell(ir);
        double r = std::sqrt(v[pr] * rho_i[ix(il)]);
        double r1 = 1.0 / (r + 1.0);
        double uc[3];
        for (int a = 0; a < 3; ++a) uc[a] = (r * uu[a][ix(ir)] + uu[a][ix(il)]) * r1;
        double Yc[IZEM_NSMAX];
        for (int l = 0; l < nrv; ++l) Yc[l] = (r * (Ya[ix(ir) * nrv + l]) + Ya[ix(il) * nrv + l]) * r1;
        double ht_c = (r * ht[ix(ir)] + ht[ix(il)]) * r1;
        double et_c = (r * et[ix(ir)] + et[ix(il)]) * r1;
        (void)pl;
        double W_i_c = 0.0;
        for (int l = 0; l < nrv; ++l) W_i_c = W_i_c + Yc[l] * t.Wc_i[l];
        double T_c = (ht_c - et_c) / W_i_c;
        double cp_c = cp_scalar(t, T_c, Yc);
        double gam_c = t.gam2 * W_i_c / cp_c;
        gam_c = 1.0 / (1.0 - gam_c);
        double cs_c = std::sqrt(gam_c * T_c * W_i_c);
        double ha_c[IZEM_NSMAX], psi_c[IZEM_NSMAX];
        ha_scalar(t, T_c, ha_c);
        double wrk = (gam_c / (gam_c - 1.0)) * T_c;
        for (int l = 0; l < nrv; ++l) {
          psi_c[l] = -(r * ha_c[l] + ha_c[l]) * r1;
          psi_c[l] = psi_c[l] + wrk * t.Wc_i[l];
        }
        double cs_c_i = 1.0 / cs_c, cs_c_2 = cs_c * cs_c;
        double q = 0.5 * (uc[0] * uc[0] + uc[1] * uc[1] + uc[2] * uc[2]);
        double b2 = (gam_c - 1.0) / cs_c_2;
        double b1 = b2 * q;
        double xi = b1 - b2 * ht_c;
        double un = uc[d];
        CharState chs;
        for (int a = 0; a < 3; ++a) chs.uc[a] = uc[a];
        chs.Yc = Yc; chs.psi_c = psi_c;
        chs.ht_c = ht_c; chs.q = q; chs.cs_c = cs_c; chs.cs_c_i = cs_c_i; chs.b1 = b1; chs.b2 = b2; chs.xi = xi;
        char_vectors(d, nv, nrv, chs, el, er);
        // characteristic LLF-WENO (module_weno.f90:953-989).  The sensor
        // is evaluated on each MPI block's interior and never exchanged, so
        // a block sees its neighbours' points as unflagged: a face is
        // evaluated with the flags of the block that uses it, and a face on
        // a block edge twice (left block's view into fhat, right block's
        // view into fhatR).
        const int vL = xblk(il), vR = xblk(ir);
        bool shkL = false, shkR = false;
        for (int s = il - ng + 1; s <= il + ng; ++s) {
          if (!sensor[cell(s)]) continue;
          if (xblk(s) == vL) shkL = true;
          if (xblk(s) == vR) shkR = true;
        }
        for (int view = 0; view < (vL == vR ? 1 : 2); ++view) {
        const bool shk = (view ? shkR : shkL) && c.cfg.weno_avg;
        double* fout = view ? fhatR.data() : fhat.data();
        for (int m = 0; m < nv; ++m) {
          double eigenmax = -1.0;
          for (int st = 1; st <= st_m1; ++st) eigenmax = std::max(L_s[st][m], eigenmax);
          for (int st = 1; st <= st_m1; ++st) {
            double wc = 0.0, gc = 0.0;
            int is = il + st - ng;
            size_t p = cell(is);
            for (int mm = 0; mm < nv; ++mm) {
              wc = wc + el[m][mm] * v[mm * nc + p];
              gc = gc + el[m][mm] * f_s[st][mm];
            }
            gplus[st] = 0.5 * (gc + eigenmax * wc);
            gminus[st] = gc - gplus[st];
          }
          double gl, gr;
          if (shk) wenorec(w, gplus, gminus, gl, gr);
          else wenorec_nw(ng, gplus, gminus, gl, gr, fixlin);
          ghat[m] = gl + gr;
        }
        for (int m = 0; m < nv; ++m) {
          double fh = 0.0;
          for (int mm = 0; mm < nv; ++mm) fh = fh + er[m][mm] * ghat[mm];
          fout[il * nv + m] = fh;
        }
        }
      }
      for (int m = 0; m < nv; ++m)
        for (int s = 1; s <= n; ++s) {
          const double* fleft = xblk(s - 1) == xblk(s) ? fhat.data() : fhatR.data();
          double df = (fhat[s * nv + m] - fleft[(s - 1) * nv + m]) * di[s - 1 + ng];
          int i, j, k;
          if (d == 0) { i = s; j = q1; k = q2; }
          else if (d == 1) { i = q1; j = s; k = q2; }
          else { i = q1; j = q2; k = s; }
          size_t f = (size_t)m * b.nint + b.fid(i, j, k);
          // fl_W / fl_E (and S, N, B, F): 0 at the boundary points of a
          // non-reflecting face (module_weno.f90:620-623, 1002, 1018)
          double flag = 1.0;
          if ((s == 1 && b.bc[2 * d] == IZEM_BC_NOREFLECTION) || (s == n && b.bc[2 * d + 1] == IZEM_BC_NOREFLECTION))
            flag = 0.0;
          if (d == 0) fl[f] = df * flag;
          else fl[f] = fl[f] + df * flag;
        }
    }
  if (negp) {
    c.err = "negative pressure in euler_LLF";
    return IZEM_ERR_NEG_PRESSURE;
  }
  return IZEM_OK;
}

// shock_sensor_modified_adams_shariff (module_tools.f90:2733-2814)
void shock_sensor(const Ctx& c, const double* v, const double* T, const double* W_i, uint8_t* sensor) {
  const Block& b = c.b;
  const double mrw = c.cfg.max_rel_weight;
  std::vector<double> rho_i(b.ncell, 0.0), P(b.ncell, 0.0);
  for (int k = 1; k <= b.nz; ++k)
    for (int j = 1; j <= b.ny; ++j)
      for (int i = 1; i <= b.nx; ++i) {
        size_t p = b.id(i, j, k);
        rho_i[p] = 1.0 / v[p];
        P[p] = v[p] * T[p] * W_i[p];
      }
  auto test = [&](size_t p, size_t q) {
    double drho = std::fabs(v[q] - v[p]) * std::min(rho_i[p], rho_i[q]);
    double dpres = std::fabs(P[q] - P[p]) / std::min(P[p], P[q]);
    if (drho > mrw && dpres > mrw) sensor[p] = 1;
  };
  // On each MPI block the x loop runs to ex - 1 with min(i+1, ex): a
  // block's last point is never compared with the next block's first one.
  const int bx = b.nx / std::max(c.sensor_xblocks, 1);
  for (int k = 1; k <= b.nz; ++k)
    for (int j = 1; j <= b.ny; ++j)
      for (int i = 1; i <= b.nx - 1; ++i)
        if (i % bx != 0) test(b.id(i, j, k), b.id(std::min(i + 1, b.nx), j, k));
  for (int k = 1; k <= b.nz; ++k)
    for (int i = 1; i <= b.nx; ++i)
      for (int j = 1; j <= b.ny - 1; ++j) test(b.id(i, j, k), b.id(i, std::min(j + 1, b.ny), k));
  for (int i = 1; i <= b.nx; ++i)
    for (int j = 1; j <= b.ny; ++j)
      for (int k = 1; k <= b.nz - 1; ++k) test(b.id(i, j, k), b.id(i, j, std::min(k + 1, b.nz)));
}

// prim_vis_vars (module_thermodynamics.f90:989-1230) for one point
void prim_vis_point(const Ctx& c, double rho, double T, double W_i, const double* Xa, double* dm, double* mu, double* ct) {
  const izem_thd& t = c.thd;
  const int ns = c.b.nrv;
  const double epsm12 = 1.0e-12;
  const double Kl = 0.5 * 1.0e-5 / t.laminf;
  const double Ku = 1.0e-1 / t.muinf;
  double lt[4];
  lt[0] = 1.0;
  lt[1] = std::log(T * t.tinf);
  lt[2] = lt[1] * lt[1];
  lt[3] = lt[2] * lt[1];
  double P = rho * T * W_i;
  for (int m = 0; m < ns; ++m) {
    double wrk1 = 0.0, dsum = 0.0;
    for (int l = 0; l < ns; ++l) {
      if (m != l) {
        double dkj = 0.0;
        for (int n = 0; n < 4; ++n) dkj = dkj + t.cofd[m][l][n] * lt[n];
        wrk1 = wrk1 + (Xa[l] + epsm12) * t.Wc[l] * W_i;
        dsum = dsum + (Xa[l] + epsm12) * (1.0 / std::exp(dkj));
      }
    }
    double Kd = 1.0e-4 * t.p0 / (t.pinf * t.dinf[m]);
    dm[m] = wrk1 * Kd / (dsum * P);
  }
  double ctsum = 0.0, w1 = 0.0, wrk2[IZEM_NSMAX];
  for (int l = 0; l < ns; ++l) {
    double a = 0.0;
    for (int m = 0; m < 4; ++m) a = a + t.coflam[l][m] * lt[m];
    double c1 = std::exp(a);
    double c2 = Xa[l];
    ctsum = ctsum + c2 / c1;
    w1 = w1 + c2 * c1;
  }
  *ct = Kl * (1.0 / ctsum + w1);
  for (int l = 0; l < ns; ++l) {
    double a = 0.0;
    for (int m = 0; m < 4; ++m) a = a + t.cofeta[l][m] * lt[m];
    wrk2[l] = std::exp(a);
  }
  double mus = 0.0;
  for (int m = 0; m < ns; ++m) {
    double c4 = 0.0;
    for (int l = 0; l < ns; ++l) {
      double c1 = std::pow(t.W[l] / t.W[m], 0.25);
      double c2 = 1.0 / std::sqrt((1.0 + t.W[m] / t.W[l]) * 8.0);
      double c3 = 1.0 + c1 * std::sqrt(wrk2[m] / wrk2[l]);
      c2 = c3 * c3 * c2;
      c4 = c4 + c2 * Xa[l];
    }
    mus = mus + Ku * (wrk2[m] * Xa[m] / c4);
  }
  *mu = mus;
}

// viscflux_xyz (module_viscflux.f90:1660-2189)
int visc_flux_fit(Ctx& c, const double* v, const double* T, const double* W_i, const double* cp, const double* ha,
                  double* fl) {
  (void)cp;
  const Block& b = c.b;
  const izem_thd& t = c.thd;
  const izem_adi& a = c.adi;
  const int nrv = b.nrv;
  const size_t nc = b.ncell;
  const int nfluid = 12, nderiv = nfluid + 3 * nrv;
  const double twothirds = 2.0 / 3.0;
  const double rvd0 = a.sqgmr / a.sc, rlam0 = a.sqgmr * a.ggmopr;
  std::vector<double> ux(nc, 0.0), vy(nc, 0.0), wz(nc, 0.0), Xa(nc * nrv, 0.0);
  std::vector<double> fd(nc * nderiv, std::nan(""));
  for (int dom = -3; dom <= 3; ++dom) {
    int i0, i1, j0, j1, k0, k1;
    domain_select(b, dom, i0, i1, j0, j1, k0, k1);
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = k0; k <= k1; ++k)
      for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i) {
          size_t p = b.id(i, j, k);
          for (int l = 0; l < nrv; ++l) Xa[l * nc + p] = v[(NIV + l) * nc + p] / (v[p] * W_i[p] * t.Wc[l]);
          double rho_i = 1.0 / v[p];
          ux[p] = v[nc + p] * rho_i;
          vy[p] = v[2 * nc + p] * rho_i;
          wz[p] = v[3 * nc + p] * rho_i;
        }
  }
  const double* src[4] = {ux.data(), vy.data(), wz.data(), T};
  for (int s = 0; s < 4; ++s)
    for (int d = 0; d < 3; ++d) deriv(c, d, src[s], fd.data() + (size_t)(3 * s + d) * nc, false);
  for (int l = 0; l < nrv; ++l)
    for (int d = 0; d < 3; ++d) deriv(c, d, Xa.data() + (size_t)l * nc, fd.data() + (size_t)(nfluid + 3 * l + d) * nc, false);
  comm_periodic(b, nderiv, fd.data(), nc);   // comm_deriv
  // LES (viscflux_LES_xyz, module_viscflux.f90:2200-2977): the W_i
  // gradients (fd nSGS+1..3) and, on the interior, the criterion of
  // shock_det_ducros_slv (module_tools.f90:2099-2181; 1 elsewhere), both
  // communicated with the other derivatives
  const bool les = c.les;
  std::vector<double> gw, crit;
  if (les) {
    gw.assign(3 * nc, std::nan(""));
    crit.assign(nc, 1.0);
    for (int d = 0; d < 3; ++d) deriv(c, d, W_i, gw.data() + (size_t)d * nc, false);
    const double eps30 = 1.0e-30;
    for (int k = 1; k <= b.nz; ++k)
      for (int j = 1; j <= b.ny; ++j)
        for (int i = 1; i <= b.nx; ++i) {
          const size_t p = b.id(i, j, k);
          auto D = [&](int q) { return fd[(size_t)(q - 1) * nc + p]; };
          double div = D(1) + D(5) + D(9);
          div = div * div;
          double wrk = D(8) - D(6);
          double vort = wrk * wrk;
          wrk = D(3) - D(7);
          wrk = wrk * wrk;
          vort = vort + wrk;
          wrk = D(4) - D(2);
          wrk = wrk * wrk;
          vort = vort + wrk;
          const double r = div / (div + vort + eps30);
          crit[p] = r > c.les_pw ? 0.0 : 1.0;
        }
    comm_periodic(b, 3, gw.data(), nc);
    comm_periodic(b, 1, crit.data(), nc);
    if (c.mu_sgs.size() != nc) c.mu_sgs.assign(nc, 0.0);
  }
  double cs2 = c.les_factor;
  cs2 = cs2 * cs2 / a.sqgmr;
  const double sc_sgs_i = 1.0 / c.les_sc_sgs, pr_sgs_i = 1.0 / c.les_pr_sgs;
  const double third = 1.0 / 3.0;

  std::vector<double> sxx(nc, 0.0), sxy(nc, 0.0), sxz(nc, 0.0), syy(nc, 0.0), syz(nc, 0.0), szz(nc, 0.0);
  std::vector<double> qx(nc, 0.0), qy(nc, 0.0), qz(nc, 0.0);
  std::vector<double> txx, txy, txz, tyy, tyz, tzz;   // LES: the stresses of the momentum divergence
  if (les) {
    txx.assign(nc, 0.0); txy.assign(nc, 0.0); txz.assign(nc, 0.0);
    tyy.assign(nc, 0.0); tyz.assign(nc, 0.0); tzz.assign(nc, 0.0);
  }
  for (int dom = -3; dom <= 3; ++dom) {
    int i0, i1, j0, j1, k0, k1;
    domain_select(b, dom, i0, i1, j0, j1, k0, k1);
    // a non-periodic face has no ghost stresses in use; skip its slab
    if (dom != 0) {
      int f = dom < 0 ? 2 * (-dom - 1) : 2 * (dom - 1) + 1;
      if (b.bnd[f]) continue;
    }
#pragma omp parallel for collapse(2) schedule(dynamic)
    for (int k = k0; k <= k1; ++k)
      for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i) {
          size_t p = b.id(i, j, k);
          double X[IZEM_NSMAX], dm[IZEM_NSMAX], mu, ct;
          for (int l = 0; l < nrv; ++l) X[l] = Xa[l * nc + p];
          prim_vis_point(c, v[p], T[p], W_i[p], X, dm, &mu, &ct);
          auto F = [&](int idx) -> double& { return fd[(size_t)(idx - 1) * nc + p]; };
          double rho_i = 1.0 / v[p];
          double uxs = v[nc + p] * rho_i, vys = v[2 * nc + p] * rho_i, wzs = v[3 * nc + p] * rho_i;
          // mu_SGS_smagorinsky (module_SGS_models.f90:176-304, 3-D branch)
          // with filter_width's delta; kept for the Fourier time step
          double mu_sgs = 0.0;
          if (les) {
            const double dxv = c.dxi[0][i - 1 + b.ng], dyv = c.dxi[1][j - 1 + b.ng], dzv = c.dxi[2][k - 1 + b.ng];
            const double delta = 1.0 / std::pow(dxv * dyv * dzv, third);
            const double d2 = delta * delta;
            const double s11 = F(1), s12 = 0.5 * (F(2) + F(4)), s13 = 0.5 * (F(3) + F(7));
            const double s22 = F(5), s23 = 0.5 * (F(6) + F(8)), s33 = F(9);
            double sb = s11 * s11 + s12 * s12 + s13 * s13 + s12 * s12 + s22 * s22 + s23 * s23 + s13 * s13 +
                        s23 * s23 + s33 * s33;
            sb = std::sqrt(sb + sb);
            mu_sgs = v[p] * cs2 * d2 * sb * crit[p];
            c.mu_sgs[p] = mu_sgs;
          }
          double rmu = -a.sqgmr * mu;
          double rvd = rvd0 * v[p];
          sxx[p] = twothirds * rmu * (F(1) + F(1) - (F(5) + F(9)));
          sxy[p] = rmu * (F(4) + F(2));
          sxz[p] = rmu * (F(7) + F(3));
          syy[p] = twothirds * rmu * (F(5) + F(5) - (F(1) + F(9)));
          syz[p] = rmu * (F(8) + F(6));
          szz[p] = twothirds * rmu * (F(9) + F(9) - (F(1) + F(5)));
          if (les) {   // the SGS-scaled stresses of the momentum divergence
            const double rmu_sgs = -a.sqgmr * mu_sgs / rmu;
            const double fs = 1.0 + rmu_sgs;
            txx[p] = sxx[p] * fs; txy[p] = sxy[p] * fs; txz[p] = sxz[p] * fs;
            tyy[p] = syy[p] * fs; tyz[p] = syz[p] * fs; tzz[p] = szz[p] * fs;
          }
          double vdcx = 0.0, vdcy = 0.0, vdcz = 0.0;
          for (int l = 1; l <= nrv; ++l) {
            double wrk = dm[l - 1] * t.Wc[l - 1] * W_i[p];
            vdcx = vdcx + wrk * F(nfluid + 3 * l - 2);
            vdcy = vdcy + wrk * F(nfluid + 3 * l - 1);
            vdcz = vdcz + wrk * F(nfluid + 3 * l);
          }
          double vdhx = 0.0, vdhy = 0.0, vdhz = 0.0;
          if (!les) {
            for (int l = 1; l <= nrv; ++l) {
              double Ya = v[(NIV + l - 1) * nc + p] * rho_i;
              double vdtx = vdcx * Ya, vdty = vdcy * Ya, vdtz = vdcz * Ya;
              double wrk = -dm[l - 1] * t.Wc[l - 1] * W_i[p];
              vdtx = vdtx + wrk * F(nfluid + 3 * l - 2);
              vdty = vdty + wrk * F(nfluid + 3 * l - 1);
              vdtz = vdtz + wrk * F(nfluid + 3 * l);
              F(nfluid + 3 * l - 2) = rvd * vdtx;
              F(nfluid + 3 * l - 1) = rvd * vdty;
              F(nfluid + 3 * l) = rvd * vdtz;
              double h = ha[(l - 1) * nc + p];
              vdhx = vdhx + h * F(nfluid + 3 * l - 2);
              vdhy = vdhy + h * F(nfluid + 3 * l - 1);
              vdhz = vdhz + h * F(nfluid + 3 * l);
            }
          } else {
            // the species fluxes of viscflux_LES_xyz: the enthalpy flux from
            // the molecular part, then the SGS diffusion and the SGS
            // W_i-gradient terms
            const double dm_sgs = a.sc * mu_sgs * rho_i * sc_sgs_i;
            for (int l = 1; l <= nrv; ++l) {
              const double Ya = v[(NIV + l - 1) * nc + p] * rho_i;
              double vdtx = vdcx * Ya, vdty = vdcy * Ya, vdtz = vdcz * Ya;
              const double dxadx = F(nfluid + 3 * l - 2), dxady = F(nfluid + 3 * l - 1), dxadz = F(nfluid + 3 * l);
              const double dmrw = -dm[l - 1] * t.Wc[l - 1] * W_i[p];
              const double h = ha[(l - 1) * nc + p];
              vdhx = vdhx + h * rvd * (vdtx + dmrw * dxadx);
              vdhy = vdhy + h * rvd * (vdty + dmrw * dxady);
              vdhz = vdhz + h * rvd * (vdtz + dmrw * dxadz);
              double wrk = dmrw - dm_sgs * t.Wc[l - 1] * W_i[p];
              vdtx = vdtx + wrk * dxadx;
              vdty = vdty + wrk * dxady;
              vdtz = vdtz + wrk * dxadz;
              wrk = -dm_sgs * t.Wc[l - 1] * X[l - 1];
              vdtx = vdtx + wrk * gw[p];
              vdty = vdty + wrk * gw[nc + p];
              vdtz = vdtz + wrk * gw[2 * nc + p];
              F(nfluid + 3 * l - 2) = rvd * vdtx;
              F(nfluid + 3 * l - 1) = rvd * vdty;
              F(nfluid + 3 * l) = rvd * vdtz;
            }
          }
          const double ct_sgs = les ? a.pr * mu_sgs * cp[p] * pr_sgs_i : 0.0;
          double rlam = les ? -rlam0 * (ct + ct_sgs) : -rlam0 * ct;
          qx[p] = uxs * sxx[p] + vys * sxy[p] + wzs * sxz[p] + rlam * F(10) + vdhx;
          qy[p] = uxs * sxy[p] + vys * syy[p] + wzs * syz[p] + rlam * F(11) + vdhy;
          qz[p] = uxs * sxz[p] + vys * syz[p] + wzs * szz[p] + rlam * F(12) + vdhz;
        }
  }
  const size_t ni = b.nint;
  std::vector<double> wx(ni), wy(ni), wzv(ni);
  auto accum = [&](int var, const double* ax, const double* ay, const double* az) {
    deriv(c, 0, ax, wx.data(), true);
    deriv(c, 1, ay, wy.data(), true);
    deriv(c, 2, az, wzv.data(), true);
#pragma omp parallel for schedule(static)
    for (size_t p = 0; p < ni; ++p) fl[var * ni + p] = fl[var * ni + p] + (wx[p] + wy[p] + wzv[p]);
  };
  if (les) {
    accum(1, txx.data(), txy.data(), txz.data());
    accum(2, txy.data(), tyy.data(), tyz.data());
    accum(3, txz.data(), tyz.data(), tzz.data());
  } else {
    accum(1, sxx.data(), sxy.data(), sxz.data());
    accum(2, sxy.data(), syy.data(), syz.data());
    accum(3, sxz.data(), syz.data(), szz.data());
  }
  accum(4, qx.data(), qy.data(), qz.data());
  for (int l = 0; l < nrv; ++l)
    accum(NIV + l, fd.data() + (size_t)(nfluid + 3 * l) * nc, fd.data() + (size_t)(nfluid + 3 * l + 1) * nc,
          fd.data() + (size_t)(nfluid + 3 * l + 2) * nc);
  return IZEM_OK;
}

#include "eglib_oracle.inc"

// viscflux_xyz or, with EGLIB, viscflux_eg_xyz (the choice in rk3, module_solver.f90:777-820)
int visc_flux(Ctx& c, const double* v, const double* T, const double* W_i, const double* cp, const double* ha,
              double* fl) {
  if (c.cfg.eglib) {
    if (!c.eg) { c.err = "EGLIB transport requested but no linking data set"; return IZEM_ERR_STATE; }
    return visc_flux_eg(c, *c.eg, v, T, W_i, cp, ha, fl);
  }
  return visc_flux_fit(c, v, T, W_i, cp, ha, fl);
}

// bc_noreflectionweno (module_weno.f90:2129-4498), one face: at every
// boundary point, the characteristic vectors at the point's own state, the
// eigenvalues of the waves leaving the domain (min(., 0) on the low faces,
// max(., 0) on the high ones), the one-sided derivative of the conserved
// variables over 2ng-1 points with wenopar's cnr weights (:199-217), and
// fl += R diag(L_s) L dw * dx_i.  The six face blocks of the reference
// differ only in the axis, the side and the sign; they are restated once.
void bc_noreflectionweno(Ctx& c, int face, const double* v, const double* T, const double* W_i, const double* cp,
                         const double* ha, double* fl) {
  const Block& b = c.b;
  const izem_thd& t = c.thd;
  const int ng = b.ng, nv = b.nv, nrv = b.nrv, d = face / 2, hi = face & 1;
  const size_t nc = b.ncell;
  // cnr: for ng = 4 the 7-point one-sided first derivative; for ng = 3 the
  // reference keeps its first five weights (their sum is -31/30, not 0)
  const double cnr[7] = {-49.0 / 20.0, 6.0, -15.0 / 2.0, 20.0 / 3.0, -15.0 / 4.0, 6.0 / 5.0, -1.0 / 6.0};
  const int st_m2 = ng + ng - 1;
  const int sc = hi ? b.n(d) : 1;
  const double* di = c.dxi[d].data();
  const int m1 = d == 0 ? b.ny : b.nx, m2 = d == 2 ? b.ny : b.nz;
  for (int q2 = 1; q2 <= m2; ++q2)
    for (int q1 = 1; q1 <= m1; ++q1) {
      auto cell = [&](int s) {
        if (d == 0) return b.id(s, q1, q2);
        if (d == 1) return b.id(q1, s, q2);
        return b.id(q1, q2, s);
      };
      const size_t p = cell(sc);
      const double rho_i = 1.0 / v[p];
      double uc[3];
      uc[0] = v[nc + p] * rho_i;
      const double P = v[p] * T[p] * W_i[p];
      double gam_c = t.gam2 * W_i[p] / cp[p];
      gam_c = 1.0 / (1.0 - gam_c);
      const double cs_c = std::sqrt(gam_c * P * rho_i);
      uc[1] = v[2 * nc + p] * rho_i;
      uc[2] = v[3 * nc + p] * rho_i;
      double Y_c[IZEM_NSMAX], psi_c[IZEM_NSMAX];
      for (int l = 0; l < nrv; ++l) Y_c[l] = v[(NIV + l) * nc + p] * rho_i;
      double ht_c = 0.0;
      double wrk = (gam_c / (gam_c - 1.0)) * T[p];
      for (int l = 0; l < nrv; ++l) {
        ht_c = ht_c + ha[l * nc + p] * Y_c[l];
        psi_c[l] = -ha[l * nc + p];
        psi_c[l] = psi_c[l] + wrk * t.Wc_i[l];
      }
      const double cs_c_i = 1.0 / cs_c, cs_c_2 = cs_c * cs_c;
      const double q = 0.5 * (uc[0] * uc[0] + uc[1] * uc[1] + uc[2] * uc[2]);
      ht_c = ht_c + q;
      const double b2 = (gam_c - 1.0) / cs_c_2;
      const double b1 = b2 * q;
      const double xi = b1 - b2 * ht_c;
      double el[IZEM_NSMAX + 5][IZEM_NSMAX + 5], er[IZEM_NSMAX + 5][IZEM_NSMAX + 5];
      CharState chs;
      for (int a = 0; a < 3; ++a) chs.uc[a] = uc[a];
      chs.Yc = Y_c; chs.psi_c = psi_c;
      chs.ht_c = ht_c; chs.q = q; chs.cs_c = cs_c; chs.cs_c_i = cs_c_i; chs.b1 = b1; chs.b2 = b2; chs.xi = xi;
      char_vectors(d, nv, nrv, chs, el, er);
      const double un = uc[d];
      auto side = [&](double x) { return hi ? std::max(x, 0.0) : std::min(x, 0.0); };
      double L_s[IZEM_NSMAX + 5], dw[IZEM_NSMAX + 5], dwc[IZEM_NSMAX + 5];
      L_s[0] = side(un - cs_c);
      L_s[1] = side(un);
      L_s[2] = side(un + cs_c);
      L_s[3] = side(un);
      L_s[4] = side(un);
      for (int m = NIV; m < nv; ++m) L_s[m] = side(un);
      for (int m = 0; m < nv; ++m) {
        dw[m] = 0.0;
        for (int st = 1; st <= st_m2; ++st) {
          if (hi) dw[m] = dw[m] - cnr[st - 1] * v[m * nc + cell(sc - st + 1)];
          else dw[m] = dw[m] + cnr[st - 1] * v[m * nc + cell(sc + st - 1)];
        }
      }
      for (int m = 0; m < nv; ++m) {
        dwc[m] = 0.0;
        for (int mm = 0; mm < nv; ++mm) dwc[m] = dwc[m] + el[m][mm] * dw[mm];
      }
      int i, j, k;
      if (d == 0) { i = sc; j = q1; k = q2; }
      else if (d == 1) { i = q1; j = sc; k = q2; }
      else { i = q1; j = q2; k = sc; }
      for (int m = 0; m < nv; ++m) {
        double df = 0.0;
        for (int mm = 0; mm < nv; ++mm) df = df + er[m][mm] * L_s[mm] * dwc[mm];
        size_t f = (size_t)m * b.nint + b.fid(i, j, k);
        fl[f] = fl[f] + df * di[sc - 1 + ng];
      }
    }
}

// NR_boundaries (module_BCs.f90:185-212): every non-reflecting face, W to F
void nr_boundaries(Ctx& c, const double* v, const double* T, const double* W_i, const double* cp, const double* ha,
                   double* fl) {
  for (int f = 0; f < 2 * c.cfg.ndim; ++f)
    if (c.b.bc[f] == IZEM_BC_NOREFLECTION) bc_noreflectionweno(c, f, v, T, W_i, cp, ha, fl);
}

// rk3 (module_solver.f90:694-856)
int rk3(Ctx& c, double dt, double time0, double* v, double* T, double* W_i, double* cp, double* ha,
        uint8_t* sensor) {
  const Block& b = c.b;
  if ((is_dirichlet(b.bc[0]) || is_dirichlet(b.bc[1])) && c.crd[0].empty()) {
    c.err = "jet boundaries need the coordinates (or_set_coords)";
    return IZEM_ERR_STATE;
  }
  const double tk3[3] = {0.0, 0.5, 1.0};   // stage times (module_solver.f90:727,756)
  const double bk3[3] = {0.00, 0.75, 1.00 / 3.00};
  const double ck3[3] = {1.00, 0.25, 2.00 / 3.00};
  const size_t ni = b.nint, nc = b.ncell;
  std::vector<double> v0(ni * b.nv), f(ni * b.nv, 0.0);
#pragma omp parallel for collapse(2) schedule(static)
  for (int l = 0; l < b.nv; ++l)
    for (int k = 1; k <= b.nz; ++k)
      for (int j = 1; j <= b.ny; ++j)
        for (int i = 1; i <= b.nx; ++i) v0[l * ni + b.fid(i, j, k)] = v[l * nc + b.id(i, j, k)];
  for (int ik = 0; ik < 3; ++ik) {
    // module_solver.f90:758-766
    if (c.sensor_type == IZEM_SENSOR_DUCROS) shock_sensor_ducros(c, v, sensor);
    else shock_sensor(c, v, T, W_i, sensor);
    int rc;
    for (int d = 0; d < c.cfg.ndim; ++d)   // euler_LLF_z only when ndim == 3 (module_solver.f90:769-774)
      if ((rc = euler_flux(c, d, v, T, W_i, cp, ha, sensor, f.data()))) return rc;
    if (c.cfg.vis)
      if ((rc = visc_flux(c, v, T, W_i, cp, ha, f.data()))) return rc;
    nr_boundaries(c, v, T, W_i, cp, ha, f.data());   // module_solver.f90:824
#pragma omp parallel for collapse(2) schedule(static)
    for (int l = 0; l < b.nv; ++l)
      for (int k = 1; k <= b.nz; ++k)
        for (int j = 1; j <= b.ny; ++j)
          for (int i = 1; i <= b.nx; ++i) {
            size_t p = l * nc + b.id(i, j, k), q = l * ni + b.fid(i, j, k);
            v[p] = v0[q] * bk3[ik] + ck3[ik] * (v[p] - dt * f[q]);
          }
    if ((rc = update_primitives(c, v, T, W_i, cp, ha, time0 + dt * tk3[ik], dt))) return rc;
  }
  return IZEM_OK;
}

// timestep (module_solver.f90:202-408): convective and chemical criteria
void timestep(const Ctx& c, double DTmax, const double* v, const double* T, const double* W_i, const double* cp,
              double* dt4, double* dtmin) {
  const Block& b = c.b;
  const izem_thd& t = c.thd;
  double dtc = 1.0;
  for (int q = 0; q < 4; ++q) dt4[q] = 1.0;
  for (int k = 1; k <= b.nz; ++k)
    for (int j = 1; j <= b.ny; ++j)
      for (int i = 1; i <= b.nx; ++i) {
        size_t p = b.id(i, j, k), nc = b.ncell;
        double rho_i = 1.0 / v[p];
        double ux = v[nc + p] * rho_i, vy = v[2 * nc + p] * rho_i, wz = v[3 * nc + p] * rho_i;
        double gamma = t.gam2 * W_i[p] / cp[p];
        gamma = 1.0 / (1.0 - gamma);
        double P = v[p] * T[p] * W_i[p];
        double csound = std::sqrt(gamma * P * rho_i);
        double ax = (std::fabs(ux) + csound) * c.dxi[0][i - 1 + b.ng];
        double ay = (std::fabs(vy) + csound) * c.dxi[1][j - 1 + b.ng];
        double az = (std::fabs(wz) + csound) * c.dxi[2][k - 1 + b.ng];
        dtc = std::max(std::max(std::max(dtc, ax), ay), az);
      }
  dt4[0] = c.cfg.cfl / dtc;
  if (c.cfg.vis && c.cfg.vis_dt) {
    // Fourier criteria (module_solver.f90:294-367) from the simple transport
    // fits (prim_vis_vars_wo_mu, module_thermodynamics.f90:1243-1420) even
    // under EGLIB, with the filter width of filter_width (module_tools.f90:
    // 2328-2378), and mu_SGS of the last fitted-transport LES flux (zero
    // without it, when its terms add exactly 0): ldmax is picked on the
    // molecular D_k, then the subgrid diffusivity is added to that species'.
    const int nrv = b.nrv;
    const size_t nc = b.ncell, np = (size_t)b.nx * b.ny * b.nz;
    std::vector<double> dm(nrv * np), d2(np), rct(np), dsgs(np);
    const double third = 1.0 / 3.0;
    for (int k = 1; k <= b.nz; ++k)
      for (int j = 1; j <= b.ny; ++j)
        for (int i = 1; i <= b.nx; ++i) {
          const size_t p = b.id(i, j, k), q = (size_t)(i - 1) + (size_t)b.nx * ((j - 1) + (size_t)b.ny * (k - 1));
          double X[IZEM_NSMAX], d[IZEM_NSMAX], mu, ct;
          for (int l = 0; l < nrv; ++l) X[l] = v[(NIV + l) * nc + p] / (v[p] * W_i[p] * t.Wc[l]);
          prim_vis_point(c, v[p], T[p], W_i[p], X, d, &mu, &ct);
          // the subgrid diffusivity and conductivity of the last LES flux
          const double msgs = c.mu_sgs.empty() ? 0.0 : c.mu_sgs[p];
          for (int l = 0; l < nrv; ++l) dm[l * np + q] = d[l];
          dsgs[q] = c.adi.sc * msgs / (v[p] * c.les_sc_sgs);
          const double dx = c.dxi[0][i - 1 + b.ng], dy = c.dxi[1][j - 1 + b.ng], dz = c.dxi[2][k - 1 + b.ng];
          const double delta = c.cfg.ndim == 2 ? 1.0 / std::sqrt(dx * dy) : 1.0 / std::pow(dx * dy * dz, third);
          d2[q] = delta * delta;
          rct[q] = d2[q] * v[p] / (ct / cp[p] + c.adi.pr * msgs * (1.0 / c.les_pr_sgs));
        }
    // the species of the largest diffusivity: first in (l, k, j, i) order
    int ldmax = 0;
    double diffmax = dm[0];
    for (int l = 0; l < nrv; ++l)
      for (size_t q = 0; q < np; ++q)
        if (diffmax < dm[l * np + q]) { ldmax = l; diffmax = dm[l * np + q]; }
    double m2 = d2[0] / (dm[ldmax * np] + dsgs[0]), m3 = rct[0];
    for (size_t q = 0; q < np; ++q) {
      m2 = std::min(m2, d2[q] / (dm[ldmax * np + q] + dsgs[q]));
      m3 = std::min(m3, rct[q]);
    }
    const double rvd0_i = c.adi.sc / c.adi.sqgmr, rlamcp0_i = c.adi.pr / c.adi.sqgmr;
    dt4[1] = rvd0_i * c.cfg.fo * m2;
    dt4[2] = rlamcp0_i * c.cfg.fo * m3;
  }
  if (c.cfg.reaction) {
    dt4[3] = *dtmin * c.cfg.cpr / DTmax;
    dt4[3] = std::min(dt4[3], 1.0);
    dt4[3] = std::max(dt4[3], dt4[0] * c.cfg.cflmin / c.cfg.cfl);
  }
  *dtmin = std::min(std::min(dt4[0], dt4[1]), std::min(dt4[2], dt4[3]));
}

#include "chem_oracle.inc"

// reaction_dvode (module_reaction.f90:102-321) followed by the rest of
// reaction_selec (:83-86): upd_prim_var_woT on the interior, comm_cons,
// upd_boundaries, upd_prim_var_ghost.  With dvodesimp a cell is integrated
// only if psr_simp_chemkin's increments (CKWYR rates x molar mass x dt /
// rho, psr_simp_chemkin.f:31-42; the reference passes it four of its five
// arguments, so its stated semantics are restated) move some species by more
// than 1e-12 and its H2 and N2 both differ from the pure fuel and from the
// pure oxidiser by more than 1e-6 (:185-215); that branch also clips the
// closing species (:233-240).
int update_boundaries(Ctx& c, double* v, double* T, double* W_i, double* cp, double* ha, double time, double dt);

// reaction_selec (module_reaction.f90:47-100): the reactors of the window,
// then upd_prim_var_woT, comm_cons, upd_boundaries (given time and the half
// step dt) and upd_prim_var_ghost.
int chem_step(Ctx& c, const izem_mech& mech, double dt, double time, double* v, double* T, double* W_i, double* cp,
              double* ha, double* DTmax_out, int* max_steps) {
  const Block& b = c.b;
  const izem_adi& a = c.adi;
  const double dt_phys = dt * a.time_ref;
  const double tref_i = 1.0 / a.t_ref;
  const double rho_cgs = a.rho_ref * 1.0e-3;
  const int ng = b.ng, nrv = b.nrv;
  const int ix = std::max(ng + 1, 1), fx = std::min(b.nx, b.nx - ng - 1);
  const int iy = std::max(ng + 1, 1), fy = std::min(b.ny, b.ny - ng - 1);
  const int iz = std::max(ng + 1, 1), fz = std::min(b.ny, b.nz - ng - 1);   // reference: min(ey, ...)
  double DTmax = 0.0;
  int fail = 0, mxs = 0;
#pragma omp parallel for collapse(2) schedule(dynamic) reduction(max : DTmax, mxs) reduction(+ : fail)
  for (int k = iz; k <= fz; ++k)
    for (int j = iy; j <= fy; ++j)
      for (int i = ix; i <= fx; ++i) {
        const size_t p = b.id(i, j, k);
        const double rho_i = 1.0 / v[p];
        double z[IZEM_NSMAX + 1];
        for (int l = 0; l < nrv; ++l) z[1 + l] = v[(NIV + l) * b.ncell + p] * rho_i;
        const double rho0 = v[p];
        const double rho_phys = rho0 * rho_cgs;
        const double T0_phys = T[p] * a.t_ref;
        z[0] = T0_phys;
        if (c.dvodesimp) {
          double wdot[IZEM_NSMAX];
          ck_wyr(mech, rho_phys, T0_phys, z + 1, wdot);
          const double myc = dt_phys / rho_phys;
          bool call_w = false;
          for (int l = 0; l < nrv; ++l)
            if (std::fabs(wdot[l] * mech.wt[l] * myc) > 1.0e-12) call_w = true;
          const double yh = z[1 + c.index_h2], yn = z[1 + c.index_n2];
          const bool call_f = std::fabs(yh - c.y1f[c.index_h2]) > 1.0e-6 && std::fabs(yn - c.y1f[c.index_n2]) > 1.0e-6;
          const bool call_o = std::fabs(yh - c.y0o[c.index_h2]) > 1.0e-6 && std::fabs(yn - c.y0o[c.index_n2]) > 1.0e-6;
          if (!(call_w && call_f && call_o)) continue;
        }
        int nst = 0;
        const int istate = reaction_v(mech, rho_phys, z, dt_phys, &nst);
        if (istate <= -2) fail += 1;
        mxs = std::max(mxs, nst);
        const double T_phys = z[0];
        T[p] = T_phys * tref_i;
        DTmax = std::max(DTmax, std::fabs(T_phys - T0_phys));
        double sumY = 0.0;
        for (int l = 0; l < nrv - 1; ++l) {
          double Ya = std::min(std::max(z[1 + l], 0.0), 1.0);
          v[(NIV + l) * b.ncell + p] = rho0 * Ya;
          sumY = sumY + Ya;
        }
        const double ylast = c.dvodesimp ? std::min(std::max(1.0 - sumY, 0.0), 1.0) : 1.0 - sumY;
        v[(NIV + nrv - 1) * b.ncell + p] = rho0 * ylast;
      }
  *DTmax_out = DTmax;
  if (max_steps) *max_steps = mxs;
  // upd_prim_var_woT on the interior (module_thermodynamics.f90:522-689)
  wmix_i(c, 0, v, W_i);
  for (int k = 1; k <= b.nz; ++k)
    for (int j = 1; j <= b.ny; ++j)
      for (int i = 1; i <= b.nx; ++i) {
        size_t p = b.id(i, j, k);
        double hak[IZEM_NSMAX], cpp;
        (void)newton_cell(c.thd, b, v, p, T[p], &cpp, hak);
        cp[p] = cpp;
        for (int is = 0; is < nrv; ++is) ha[is * b.ncell + p] = hak[is];
      }
  int rc = update_boundaries(c, v, T, W_i, cp, ha, time, dt);
  if (rc) return rc;
  if (fail) {
    c.err = "DVODE failed (ISTATE <= -2) on some cells";
    return IZEM_ERR_CHEM;
  }
  return IZEM_OK;
}

}  // namespace

// ============================================================== C API =====
extern "C" {

void* or_create(const izem_cfg* cfg, const izem_thd* thd, const izem_adi* adi, const double* dx_i,
                const double* dy_i, const double* dz_i) {
  if (!cfg || !thd || !adi || (cfg->ng != 3 && cfg->ng != 4) || (cfg->ndim != 2 && cfg->ndim != 3) ||
      (cfg->ndim == 2 && cfg->nz != 1) || cfg->nrv < 2 || cfg->nrv > IZEM_NSMAX)
    return nullptr;
  for (int f = 0; f < 6; ++f) {
    const int bc = cfg->bc[f];
    if (bc < IZEM_BC_PERIODIC || bc > IZEM_BC_NOREFLECTION) return nullptr;
    if ((bc == IZEM_BC_INFLOWJET && f != 0) || (bc == IZEM_BC_NSCBC_OUT && f != 1)) return nullptr;
  }
  if (cfg->bc[0] == IZEM_BC_INFLOWJET && cfg->nrv != 2 && cfg->nrv != 3 && cfg->nrv != 9) return nullptr;
  Ctx* c = new Ctx();
  c->cfg = *cfg;
  c->thd = *thd;
  c->adi = *adi;
  Block& b = c->b;
  b.nx = cfg->nx; b.ny = cfg->ny; b.nz = cfg->nz; b.ng = cfg->ng; b.nrv = cfg->nrv; b.nv = NIV + cfg->nrv;
  b.gx = b.nx + 2 * b.ng; b.gy = b.ny + 2 * b.ng; b.gz = b.nz + 2 * b.ng;
  b.ncell = (size_t)b.gx * b.gy * b.gz;
  b.nint = (size_t)b.nx * b.ny * b.nz;
  for (int f = 0; f < 6; ++f) {
    b.bc[f] = cfg->bc[f];
    b.bnd[f] = cfg->bc[f] != IZEM_BC_PERIODIC;
  }
  const double* di[3] = {dx_i, dy_i, dz_i};
  for (int d = 0; d < 3; ++d) c->dxi[d].assign(di[d], di[d] + b.n(d) + 2 * b.ng);
  return c;
}

void or_destroy(void* h) { delete static_cast<Ctx*>(h); }

// Coordinates of the interior points (code units) and Lx, for the jet boundaries.
int or_set_coords(void* h, const double* x, const double* y, const double* z, double lx) {
  Ctx* c = static_cast<Ctx*>(h);
  if (!x || !y || !z) return IZEM_ERR_ARG;
  const double* src[3] = {x, y, z};
  for (int d = 0; d < 3; ++d) c->crd[d].assign(src[d], src[d] + c->b.n(d));
  c->lx = lx;
  return IZEM_OK;
}

int or_set_les(void* h, int enable, double mu_sgs_factor, double sc_sgs, double pr_sgs, double percent_weight_sgs) {
  Ctx* c = static_cast<Ctx*>(h);
  if (!enable) {
    c->les = false;
    c->mu_sgs.clear();
    return IZEM_OK;
  }
  if (!c->cfg.vis || c->cfg.ndim != 3 || !(mu_sgs_factor >= 0.0) || !(sc_sgs > 0.0) || !(pr_sgs > 0.0) ||
      !(percent_weight_sgs >= 0.0))
    return IZEM_ERR_ARG;
  c->les_factor = mu_sgs_factor;
  c->les_sc_sgs = sc_sgs;
  c->les_pr_sgs = pr_sgs;
  c->les_pw = percent_weight_sgs;
  c->les = true;
  return IZEM_OK;
}

int or_set_chem_skip(void* h, int enable, const double* y1f, const double* y0o, int index_h2, int index_n2) {
  Ctx* c = static_cast<Ctx*>(h);
  const int nrv = c->b.nrv;
  if (!enable) {
    c->dvodesimp = false;
    return IZEM_OK;
  }
  if (!y1f || !y0o || index_h2 < 0 || index_h2 >= nrv || index_n2 < 0 || index_n2 >= nrv || index_h2 == index_n2)
    return IZEM_ERR_ARG;
  for (int l = 0; l < nrv; ++l) { c->y1f[l] = y1f[l]; c->y0o[l] = y0o[l]; }
  c->index_h2 = index_h2;
  c->index_n2 = index_n2;
  c->dvodesimp = true;
  return IZEM_OK;
}

// The reference's run decomposed x into nblk equal MPI blocks: the shock
// sensor of each block stops at its own last point (module_tools.f90:2761-2770).
int or_set_sensor_xblocks(void* h, int nblk) {
  Ctx* c = static_cast<Ctx*>(h);
  if (nblk < 1 || c->b.nx % nblk) return IZEM_ERR_ARG;
  c->sensor_xblocks = nblk;
  return IZEM_OK;
}

int or_set_newton_xblocks(void* h, int nblk) {
  Ctx* c = static_cast<Ctx*>(h);
  if (nblk < 1 || c->b.nx % nblk) return IZEM_ERR_ARG;
  c->newton_xblocks = nblk;
  return IZEM_OK;
}

int or_set_jet(void* h, const izem_jet* p) {
  if (!h || !p) return IZEM_ERR_ARG;
  static_cast<Ctx*>(h)->jet = *p;
  return IZEM_OK;
}

int or_last_error(void* h, char* buf, int n) {
  Ctx* c = static_cast<Ctx*>(h);
  if (buf && n > 0) { std::snprintf(buf, n, "%s", c->err.c_str()); }
  return c->newton_warn;
}

int or_newton_it_max(void* h) { return static_cast<Ctx*>(h)->newton_it_max; }

void or_cp_scalar(void* h, double T, const double* Y, double* cp) { *cp = cp_scalar(static_cast<Ctx*>(h)->thd, T, Y); }
void or_ha_scalar(void* h, double T, double* ha) { ha_scalar(static_cast<Ctx*>(h)->thd, T, ha); }

int or_shock_sensor(void* h, const double* v, const double* T, const double* W_i, uint8_t* sensor) {
  Ctx& c = *static_cast<Ctx*>(h);
  if (c.sensor_type == IZEM_SENSOR_DUCROS) shock_sensor_ducros(c, v, sensor);
  else shock_sensor(c, v, T, W_i, sensor);
  return 0;
}

int or_set_shock_sensor(void* h, int type, double ducros_treduc) {
  Ctx& c = *static_cast<Ctx*>(h);
  if ((type != IZEM_SENSOR_ADAMS_SHARIFF && type != IZEM_SENSOR_DUCROS) || c.cfg.ndim < 2 ||
      !(ducros_treduc >= 0.0 && ducros_treduc <= 1.0))
    return IZEM_ERR_ARG;
  c.sensor_type = type;
  c.ducros_treduc = ducros_treduc;
  return IZEM_OK;
}
int or_euler_flux(void* h, int dir, const double* v, const double* T, const double* W_i, const double* cp,
                  const double* ha, const uint8_t* sensor, double* fl) {
  return euler_flux(*static_cast<Ctx*>(h), dir, v, T, W_i, cp, ha, sensor, fl);
}
int or_nr_flux(void* h, const double* v, const double* T, const double* W_i, const double* cp, const double* ha,
               double* fl) {
  nr_boundaries(*static_cast<Ctx*>(h), v, T, W_i, cp, ha, fl);
  return IZEM_OK;
}

int or_visc_flux(void* h, const double* v, const double* T, const double* W_i, const double* cp,
                 const double* ha, double* fl) {
  return visc_flux(*static_cast<Ctx*>(h), v, T, W_i, cp, ha, fl);
}
int or_set_eglib(void* h, const izem_eglib* L) {
  if (!h || !L || L->ns != static_cast<Ctx*>(h)->b.nrv) return IZEM_ERR_ARG;
  auto e = std::make_shared<EgInit>();
  eg_init(*L, *e);
  static_cast<Ctx*>(h)->eg = e;
  return IZEM_OK;
}
// One point of EGLIB precision 1 (no context): T [K], X, Y, cp [erg/g/K],
// mean molar mass [g/mol] -> eta, lambda, chi (ns), rho*D (ns x ns, [l][m]).
void or_eg_point(const izem_eglib* L, double T, const double* X, const double* Y, const double* cp, double ww,
                 double* eta, double* tc, double* chit, double* D) {
  EgInit E;
  eg_init(*L, E);
  double Dm[EGN][EGN];
  eg_point(E, T, X, Y, cp, ww, eta, tc, chit, Dm);
  for (int l = 0; l < L->ns; ++l)
    for (int m = 0; m < L->ns; ++m) D[l * L->ns + m] = Dm[l][m];
}
int or_prim_inv_var(void* h, int dom, int err_mach, double* v, double* W_i, double* T, double* cp, double* ha) {
  return prim_inv_var(*static_cast<Ctx*>(h), dom, err_mach != 0, v, W_i, T, cp, ha);
}
int or_force_sumY(void* h, int dom, double* v) {
  force_sumY(*static_cast<Ctx*>(h), dom, v);
  return 0;
}
int or_update_primitives(void* h, double* v, double* T, double* W_i, double* cp, double* ha) {
  return update_primitives(*static_cast<Ctx*>(h), v, T, W_i, cp, ha);
}
int or_finalize_ic(void* h, double* v, double* T, double* W_i, double* cp, double* ha) {
  return finalize_ic(*static_cast<Ctx*>(h), v, T, W_i, cp, ha);
}
int or_rk3(void* h, double dt, double time0, double* v, double* T, double* W_i, double* cp, double* ha,
           uint8_t* sensor) {
  return rk3(*static_cast<Ctx*>(h), dt, time0, v, T, W_i, cp, ha, sensor);
}
int or_timestep(void* h, double DTmax, const double* v, const double* T, const double* W_i, const double* cp,
                double* dt4, double* dtmin) {
  timestep(*static_cast<Ctx*>(h), DTmax, v, T, W_i, cp, dt4, dtmin);
  return 0;
}

int or_chem_step(void* h, const izem_mech* mech, double dt, double time, double* v, double* T, double* W_i,
                 double* cp, double* ha, double* DTmax, int* max_steps) {
  Ctx* c = static_cast<Ctx*>(h);
  if ((is_dirichlet(c->b.bc[0]) || is_dirichlet(c->b.bc[1])) && c->crd[0].empty()) {
    c->err = "jet boundaries need the coordinates (or_set_coords)";
    return IZEM_ERR_STATE;
  }
  return chem_step(*c, *mech, dt, time, v, T, W_i, cp, ha, DTmax, max_steps);
}

// Independent constant-volume reactors (PSR_CHEMKIN per cell): T [K],
// rho [g/cm^3], Y (n x kk, row per cell), dt [s] per cell.
void or_psr_cells(const izem_mech* mech, int n, double* T, const double* rho, double* Y, const double* dt, int* istate,
                  int* nsteps) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int q = 0; q < n; ++q) {
    double z[IZEM_NSMAX + 1];
    z[0] = T[q];
    for (int k = 0; k < mech->kk; ++k) z[1 + k] = Y[(size_t)q * mech->kk + k];
    int nst = 0;
    istate[q] = reaction_v(*mech, rho[q], z, dt[q], &nst);
    nsteps[q] = nst;
    T[q] = z[0];
    for (int k = 0; k < mech->kk; ++k) Y[(size_t)q * mech->kk + k] = z[1 + k];
  }
}

// Reactor right-hand side FUN (for cross-checks against other integrators).
void or_ck_fun(const izem_mech* mech, double rho, const double* z, double* zp) { ck_fun(*mech, rho, z, zp); }
void or_ck_wdot(const izem_mech* mech, double rho, double T, const double* Y, double* wdot) {
  ck_wyr(*mech, rho, T, Y, wdot);
}

// dscalar + inversion (module_deriv.f90:80-205, module_tools.f90:374-426):
// central 6th order (ng = 3) or 8th order with 6th-order fourth rows (ng = 4)
void or_metrics_dscalar(int n, int ng, const double* coord, double* d_i) {
  std::vector<double> dv(n, 1.0);
  auto v = [&](int m) { return coord[m - 1]; };
  for (int m = 1 + ng; m <= n - ng; ++m) {
    double dd = 0.0;
    if (ng == 4)
      for (int l = -4; l <= 4; ++l) dd = dd + alpha8[l + 4] * v(m + l);
    else
      for (int l = -3; l <= 3; ++l) dd = dd + alpha6[l + 3] * v(m + l);
    dv[m - 1] = dd * 1.0;
  }
  if (ng == 4)
    for (int m : {4, n - 3}) {
      double dd = 0.0;
      for (int l = -3; l <= 3; ++l) dd = dd + alpha6[l + 3] * v(m + l);
      dv[m - 1] = dd * 1.0;
    }
  { int m = 1; double dd = 0.0; for (int l = 0; l <= 4; ++l) dd = dd + alph4ol[l] * v(m + l); dv[m - 1] = dd * 1.0; }
  { int m = 2; double dd = 0.0; for (int l = -1; l <= 3; ++l) dd = dd + alph4ul[l + 1] * v(m + l); dv[m - 1] = dd * 1.0; }
  { int m = 3; double dd = 0.0; for (int l = -2; l <= 2; ++l) dd = dd + alph4[l + 2] * v(m + l); dv[m - 1] = dd * 1.0; }
  { int m = n - 2; double dd = 0.0; for (int l = -2; l <= 2; ++l) dd = dd + alph4[l + 2] * v(m + l); dv[m - 1] = dd * 1.0; }
  { int m = n - 1; double dd = 0.0; for (int l = -3; l <= 1; ++l) dd = dd + alph4ur[l + 3] * v(m + l); dv[m - 1] = -dd * 1.0; }
  { int m = n; double dd = 0.0; for (int l = -4; l <= 0; ++l) dd = dd + alph4or[l + 4] * v(m + l); dv[m - 1] = -dd * 1.0; }
  for (int m = 0; m < n; ++m) d_i[m] = 1.0 / dv[m];
}

}  // extern "C"

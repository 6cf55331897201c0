// State update kernels: SSP-RK3 stage update (module_solver.f90:828-837),
// force_sumY (module_thermodynamics.f90:1709-1760), Wmix_i (:700-728), the
// Newton temperature iteration with the reference's per-sub-domain global
// stopping test (prim_inv_var :79-186, newton :271-508), halo wrap /
// extrapolation (comm_cons, bc_extrapolation module_BCs.f90:327-410) and the
// convective time-step reduction (timestep, module_solver.f90:249-277).
#pragma once
#include "common.cuh"
#include "thermo.cuh"
#include "kernels_euler.cuh"

template <int NRV>
__device__ __forceinline__ void force_sumY_cell(double* v, long long nc, long long p) {
  const double rho = v[p];
  const double rho_i = 1.0 / rho;
  double sum = 0.0, Ya;
#pragma unroll
  for (int l = 0; l < NRV - 1; ++l) {
    Ya = v[(IZEM_NIV + l) * nc + p] * rho_i;
    Ya = fmin(fmax(Ya, 0.0), 1.0);
    v[(IZEM_NIV + l) * nc + p] = rho * Ya;
    sum = sum + Ya;
  }
  Ya = 1.0 - sum;
  Ya = fmin(fmax(Ya, 0.0), 1.0);
  v[(IZEM_NIV + NRV - 1) * nc + p] = rho * Ya;
}

template <int NRV>
__device__ __forceinline__ double wmix_cell(const double* v, long long nc, long long p) {
  double w = 0.0;
  const double rho = v[p];
#pragma unroll
  for (int l = 0; l < NRV; ++l) w = w + (v[(IZEM_NIV + l) * nc + p] / rho) * c_thd.Wc_i[l];
  return w;
}

// RK stage: v = v0*bk + ck*(v - dt*f) on the interior, then force_sumY and
// W_i.  Stage 0 first stores v0 = v.
template <int NRV>
__global__ void k_rk_update(Geo g, int stage, int forcesum, const double* __restrict__ dt_dev,
                            double* __restrict__ v, double* __restrict__ v0, const double* __restrict__ fl,
                            double* __restrict__ W_i) {
  constexpr int NV = IZEM_NIV + NRV;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= g.nint) return;
  const double bk3[3] = {0.00, 0.75, 1.00 / 3.00};
  const double ck3[3] = {1.00, 0.25, 2.00 / 3.00};
  const double bk = bk3[stage], ck = ck3[stage];
  const double dt = *dt_dev;
  int i = (int)(idx % g.n[0]) + 1;
  long long r = idx / g.n[0];
  int j = (int)(r % g.n[1]) + 1;
  int k = (int)(r / g.n[1]) + 1;
  const long long nc = g.ncell, ni = g.nint;
  const long long p = gid(g, i, j, k);
#pragma unroll
  for (int l = 0; l < NV; ++l) {
    double vv = v[l * nc + p];
    double v0v;
    if (stage == 0) { v0v = vv; v0[l * ni + idx] = vv; }
    else v0v = v0[l * ni + idx];
    v[l * nc + p] = v0v * bk + ck * (vv - dt * fl[l * ni + idx]);
  }
  if (forcesum) force_sumY_cell<NRV>(v, nc, p);
  W_i[p] = wmix_cell<NRV>(v, nc, p);
}

// W_i on the interior (Wmix_i(0)) for initial conditions.
template <int NRV>
__global__ void k_wmix_interior(Geo g, const double* __restrict__ v, double* __restrict__ W_i) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= g.nint) return;
  int i = (int)(idx % g.n[0]) + 1;
  long long r = idx / g.n[0];
  int j = (int)(r % g.n[1]) + 1;
  int k = (int)(r / g.n[1]) + 1;
  const long long p = gid(g, i, j, k);
  W_i[p] = wmix_cell<NRV>(v, g.ncell, p);
}

// upd_prim_var_domain on the interior without an RK update: force_sumY, W_i.
template <int NRV>
__global__ void k_prep_interior(Geo g, int forcesum, double* __restrict__ v, double* __restrict__ W_i) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= g.nint) return;
  int i = (int)(idx % g.n[0]) + 1;
  long long r = idx / g.n[0];
  int j = (int)(r % g.n[1]) + 1;
  int k = (int)(r / g.n[1]) + 1;
  const long long p = gid(g, i, j, k);
  if (forcesum) force_sumY_cell<NRV>(v, g.ncell, p);
  W_i[p] = wmix_cell<NRV>(v, g.ncell, p);
}

// upd_prim_var_woT on the interior (module_thermodynamics.f90:522-689):
// W_i, cp and h_k at the current temperature, no Newton solve.
template <int NRV>
__global__ void k_prim_woT(Geo g, const double* __restrict__ v, const double* __restrict__ T, double* __restrict__ W_i,
                           double* __restrict__ cp, double* __restrict__ ha) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= g.nint) return;
  int i = (int)(idx % g.n[0]) + 1;
  long long r = idx / g.n[0];
  int j = (int)(r % g.n[1]) + 1;
  int k = (int)(r / g.n[1]) + 1;
  const long long nc = g.ncell;
  const long long p = gid(g, i, j, k);
  W_i[p] = wmix_cell<NRV>(v, nc, p);
  const double rho_i = 1.0 / v[p];
  const double Tp = T[p];
  double cpm = 0.0;
#pragma unroll
  for (int l = 0; l < NRV; ++l) {
    double cpk;
    const double h = th_species(l, Tp, &cpk);
    ha[l * nc + p] = h;
    const double Ya = v[(IZEM_NIV + l) * nc + p] * rho_i;
    cpm = cpm + Ya * c_thd.gam2 * c_thd.Wc_i[l] * cpk;
  }
  cp[p] = cpm;
}

// Ghost slabs: fill v from the periodic partner or by zero-gradient
// extrapolation, then force_sumY and W_i on the ghost point.
// mode 0: periodic faces wrap, boundary faces extrapolate (comm_cons +
// upd_boundaries); mode 1: every face extrapolates (upd_extrapolation).
template <int NRV>
__global__ void k_halo(Geo g, int mode, int forcesum, double* __restrict__ v, double* __restrict__ W_i) {
  constexpr int NV = IZEM_NIV + NRV;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long ntot = slab_count(g) - g.nint;
  if (idx >= ntot) return;
  int i, j, k, dom;
  if (!slab_point(g, idx + g.nint, i, j, k, dom)) return;
  const int f = dom - 1, d = f >> 1;
  int c[3] = {i, j, k};
  if (mode == 0 && g.bc[f] == IZEM_BC_PERIODIC) c[d] = (f & 1) ? c[d] - g.n[d] : c[d] + g.n[d];
  else c[d] = (f & 1) ? g.n[d] : 1;
  const long long nc = g.ncell;
  const long long p = gid(g, i, j, k), q = gid(g, c[0], c[1], c[2]);
#pragma unroll
  for (int l = 0; l < NV; ++l) v[l * nc + p] = v[l * nc + q];
  if (forcesum) force_sumY_cell<NRV>(v, nc, p);
  W_i[p] = wmix_cell<NRV>(v, nc, p);
}

// One Newton iteration (newton + the T update of prim_inv_var) on the
// interior (ghost = 0) or on all six ghost slabs (ghost = 1); each
// sub-domain stops on its own maximum correction.
template <int NRV>
__global__ void k_newton_iter(Geo g, int ghost, const double* __restrict__ v, double* __restrict__ T,
                              double* __restrict__ cp, double* __restrict__ ha, DevStatus* st, int check_negT) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  int i, j, k, dom;
  if (ghost) {
    const long long ntot = slab_count(g) - g.nint;
    if (idx >= ntot) return;
    if (!slab_point(g, idx + g.nint, i, j, k, dom)) return;
  } else {
    if (idx >= g.nint) return;
    i = (int)(idx % g.n[0]) + 1;
    long long r = idx / g.n[0];
    j = (int)(r % g.n[1]) + 1;
    k = (int)(r / g.n[1]) + 1;
    dom = 0;
  }
  if (st->done[dom]) return;
  const long long nc = g.ncell;
  const long long p = gid(g, i, j, k);
  const double rho_i = 1.0 / v[p];
  const double v2 = v[nc + p], v3 = v[2 * nc + p], v4 = v[3 * nc + p];
  double F = -v[4 * nc + p] * rho_i + 0.5 * (v2 * v2 + v3 * v3 + v4 * v4) * (rho_i * rho_i);
  const double Tp = T[p];
  double Ya[NRV];
#pragma unroll
  for (int l = 0; l < NRV; ++l) Ya[l] = v[(IZEM_NIV + l) * nc + p] * rho_i;
  double cpm = 0.0;
#pragma unroll
  for (int l = 0; l < NRV; ++l) {
    double cpk;
    const double h = th_species(l, Tp, &cpk);
    ha[l * nc + p] = h;
    cpm = cpm + Ya[l] * c_thd.gam2 * c_thd.Wc_i[l] * cpk;
    F = F + Ya[l] * (h + (-Tp) * c_thd.Wc_i[l]);
  }
  double wrk = 0.0;
#pragma unroll
  for (int l = 0; l < NRV; ++l) wrk = wrk + Ya[l] * c_thd.Wc_i[l];
  cp[p] = cpm;
  const double DF = F / (wrk - cpm * c_thd.gam2_i);
  const double Tn = Tp + DF;
  T[p] = Tn;
  if (check_negT && Tn < 0.0) atomicExch(&st->neg_temperature, 1);
  const double df2 = DF * DF;
  if (df2 != df2) atomicExch(&st->newton_nan, 1);
  else atomic_max_nonneg(&st->maxdf_bits[dom], df2);
}

// Stopping test of prim_inv_var for sub-domains [d0, d1].
__global__ void k_newton_check(DevStatus* st, int d0, int d1, double eps, int itmax) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int d = d0; d <= d1; ++d) {
    if (st->done[d]) continue;
    st->it[d] += 1;
    const double err = sqrt(__longlong_as_double((long long)st->maxdf_bits[d]));
    st->maxdf_bits[d] = 0ULL;
    if (err < eps) st->done[d] = 1;
    else if (st->it[d] >= itmax) { st->done[d] = 1; st->newton_unconverged += 1; }
  }
}

__global__ void k_newton_reset(DevStatus* st, int d0, int d1) {
  int d = d0 + threadIdx.x;
  if (d <= d1) { st->done[d] = 0; st->it[d] = 0; st->maxdf_bits[d] = 0ULL; }
}

// After the captured iterations: any sub-domain still running is reported.
__global__ void k_newton_final(DevStatus* st, int d0, int d1) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int d = d0; d <= d1; ++d)
    if (!st->done[d]) st->newton_unconverged += 1;
}

// Convective time-step criterion: max over the interior of (|u_d|+c) dx_i.
template <int NRV>
__global__ void k_dtc(Geo g, Metrics mt, const double* __restrict__ v, const double* __restrict__ T,
                      const double* __restrict__ W_i, const double* __restrict__ cp, DevStatus* st) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double m = 0.0;
  if (idx < g.nint) {
    int c[3];
    c[0] = (int)(idx % g.n[0]) + 1;
    long long r = idx / g.n[0];
    c[1] = (int)(r % g.n[1]) + 1;
    c[2] = (int)(r / g.n[1]) + 1;
    const long long nc = g.ncell;
    const long long p = gid(g, c[0], c[1], c[2]);
    const double rho_i = 1.0 / v[p];
    const double ux = v[nc + p] * rho_i, vy = v[2 * nc + p] * rho_i, wz = v[3 * nc + p] * rho_i;
    double gamma = c_thd.gam2 * W_i[p] / cp[p];
    gamma = 1.0 / (1.0 - gamma);
    const double P = v[p] * T[p] * W_i[p];
    const double cs = sqrt(gamma * P * rho_i);
    const double ax = (fabs(ux) + cs) * mt.dxi[0][c[0] - 1 + g.ng];
    const double ay = (fabs(vy) + cs) * mt.dxi[1][c[1] - 1 + g.ng];
    const double az = (fabs(wz) + cs) * mt.dxi[2][c[2] - 1 + g.ng];
    m = fmax(fmax(ax, ay), az);
  }
  // warp reduction then one atomic per warp
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&st->dtc_bits, m);
}

__device__ inline void atomic_min_pos(unsigned long long* addr, double v) {
  atomicMin(addr, (unsigned long long)__double_as_longlong(v));
}

// Fourier time-step criteria (module_solver.f90:294-367) at the interior
// points: the mixture-averaged D_k and lambda of prim_vis_vars_wo_mu
// (module_thermodynamics.f90:1243-1420, the simple fits even under EGLIB)
// with X_k of molefrac (:1669-1698), and delta^2 of filter_width
// (module_tools.f90:2328-2378).  Per species the max of D_k and the min of
// delta^2 / D_k, and the min of delta^2 rho / (lambda / cp), reduced into the
// status word; the host picks the species of the largest D_k.  The LES terms
// of the reference (mu_SGS = 0 without LES) add exactly zero and are left out.
template <int NRV>
__global__ void k_dtv(Geo g, Metrics mt, const double* __restrict__ v, const double* __restrict__ T,
                      const double* __restrict__ W_i, const double* __restrict__ cp, DevStatus* st) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const double big = __longlong_as_double(0x7ff0000000000000LL);   // +inf: identity of min
  double dmx[NRV], dmn[NRV], rct = big;
#pragma unroll
  for (int l = 0; l < NRV; ++l) { dmx[l] = 0.0; dmn[l] = big; }
  if (idx < g.nint) {
    int c[3];
    c[0] = (int)(idx % g.n[0]) + 1;
    long long r = idx / g.n[0];
    c[1] = (int)(r % g.n[1]) + 1;
    c[2] = (int)(r / g.n[1]) + 1;
    const long long nc = g.ncell;
    const long long p = gid(g, c[0], c[1], c[2]);
    const double rho = v[p], Tp = T[p], Wi = W_i[p];
    double X[NRV];
#pragma unroll
    for (int l = 0; l < NRV; ++l) X[l] = v[(IZEM_NIV + l) * nc + p] / (rho * Wi * c_thd.Wc[l]);
    const double lt1 = log(Tp * c_thd.tinf);
    const double lt2 = lt1 * lt1, lt3 = lt2 * lt1;
    const double P = rho * Tp * Wi;
    const double epsm12 = 1.0e-12;
    double dm[NRV], wk1[NRV], xe[NRV], aw[NRV];
#pragma unroll
    for (int l = 0; l < NRV; ++l) {
      xe[l] = X[l] + epsm12;
      aw[l] = xe[l] * c_thd.Wc[l] * Wi;
      dm[l] = 0.0;
      wk1[l] = 0.0;
    }
    // D_kl symmetric: one exponential per pair, sums over l in ascending order
#pragma unroll
    for (int m = 0; m < NRV; ++m)
#pragma unroll
      for (int l = m + 1; l < NRV; ++l) {
        const double* cf = c_thd.cofd[m][l];
        const double e = 1.0 / exp(0.0 + cf[0] * 1.0 + cf[1] * lt1 + cf[2] * lt2 + cf[3] * lt3);
        dm[m] = dm[m] + xe[l] * e;
        dm[l] = dm[l] + xe[m] * e;
        wk1[m] = wk1[m] + aw[l];
        wk1[l] = wk1[l] + aw[m];
      }
    double ct = 0.0, w1 = 0.0;
#pragma unroll
    for (int l = 0; l < NRV; ++l) {
      const double* cl = c_thd.coflam[l];
      const double c1 = exp(0.0 + cl[0] * 1.0 + cl[1] * lt1 + cl[2] * lt2 + cl[3] * lt3);
      ct = ct + X[l] / c1;
      w1 = w1 + X[l] * c1;
    }
    ct = c_thd.Kl * (1.0 / ct + w1);
    const double dx = mt.dxi[0][c[0] - 1 + g.ng], dy = mt.dxi[1][c[1] - 1 + g.ng], dz = mt.dxi[2][c[2] - 1 + g.ng];
    const double delta = g.ndim == 2 ? 1.0 / sqrt(dx * dy) : 1.0 / pow(dx * dy * dz, 1.0 / 3.0);
    const double d2 = delta * delta;
#pragma unroll
    for (int l = 0; l < NRV; ++l) {
      dmx[l] = wk1[l] * c_thd.Kd[l] / (dm[l] * P);
      dmn[l] = d2 / dmx[l];
    }
    rct = d2 * rho / (ct / cp[p]);
  }
#pragma unroll
  for (int l = 0; l < NRV; ++l)
    for (int o = 16; o > 0; o >>= 1) {
      dmx[l] = fmax(dmx[l], __shfl_down_sync(0xffffffffu, dmx[l], o));
      dmn[l] = fmin(dmn[l], __shfl_down_sync(0xffffffffu, dmn[l], o));
    }
  for (int o = 16; o > 0; o >>= 1) rct = fmin(rct, __shfl_down_sync(0xffffffffu, rct, o));
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int l = 0; l < NRV; ++l) {
      atomic_max_nonneg(&st->fo_dmax_bits[l], dmx[l]);
      atomic_min_pos(&st->fo_dmin_bits[l], dmn[l]);
    }
    atomic_min_pos(&st->fo_ctmin_bits, rct);
  }
}

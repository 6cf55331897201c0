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

// Ghost slabs: fill v from the periodic partner, by zero-gradient
// extrapolation, or (non-reflecting faces) with the boundary state times 10,
// then force_sumY and W_i on the ghost point.
// mode 0: periodic faces wrap, boundary faces extrapolate (comm_cons +
// upd_boundaries); mode 1: every face extrapolates (upd_extrapolation).
// mask: the faces (bit f) this launch treats; mode 2: no copy, only the
// force_sumY and W_i of ghost points that a Dirichlet face kernel wrote.
template <int NRV>
__global__ void k_halo(Geo g, int mode, int forcesum, double* __restrict__ v, double* __restrict__ W_i,
                       int mask = 0x3f) {
  constexpr int NV = IZEM_NIV + NRV;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long ntot = slab_count(g) - g.nint;
  if (idx >= ntot) return;
  int i, j, k, dom;
  if (!slab_point(g, idx + g.nint, i, j, k, dom)) return;
  const int f = dom - 1, d = f >> 1;
  if (!((mask >> f) & 1)) return;
  int c[3] = {i, j, k};
  if (mode == 0 && g.bc[f] == IZEM_BC_PERIODIC) c[d] = (f & 1) ? c[d] - g.n[d] : c[d] + g.n[d];
  else c[d] = (f & 1) ? g.n[d] : 1;
  const long long nc = g.ncell;
  const long long p = gid(g, i, j, k), q = gid(g, c[0], c[1], c[2]);
  if (mode == 0 && g.bc[f] == IZEM_BC_NOREFLECTION) {
    // bc_noreflection (module_BCs.f90:426-512): the boundary state times 10
#pragma unroll
    for (int l = 0; l < NV; ++l) v[l * nc + p] = v[l * nc + q] * 10.0;
  } else if (mode != 2) {
#pragma unroll
    for (int l = 0; l < NV; ++l) v[l * nc + p] = v[l * nc + q];
  }
  if (forcesum) force_sumY_cell<NRV>(v, nc, p);
  W_i[p] = wmix_cell<NRV>(v, nc, p);
}

// One Newton iteration (newton + the T update of prim_inv_var) on the
// interior (ghost = 0) or on all six ghost slabs (ghost = 1); each
// sub-domain stops on its own maximum correction.
template <int NRV>
__global__ void k_newton_iter(Geo g, int ghost, const double* __restrict__ v, double* __restrict__ T,
                              double* __restrict__ cp, double* __restrict__ ha, DevStatus* st, int check_negT,
                              int bx) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  int i, j, k, dom;
  if (ghost == 2) {
    // the Dirichlet planes i = 1 (sub-domain 7) and i = nx (8) of jet faces
    const long long np = (long long)g.n[1] * g.n[2];
    if (idx >= 2 * np) return;
    const int face = (int)(idx / np);
    if (g.bc[face] != IZEM_BC_INFLOWJET && g.bc[face] != IZEM_BC_NSCBC_OUT) return;
    const long long r = idx - face * np;
    i = face ? g.n[0] : 1;
    j = (int)(r % g.n[1]) + 1;
    k = (int)(r / g.n[1]) + 1;
    dom = 7 + face;
  } else if (ghost) {
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
  // the interior and the y / z ghost slabs span x: with an emulated
  // x-decomposition (bx < nx) each x-block of them stops on its own test
  if (bx < g.n[0] && (dom == 0 || (dom >= 3 && dom <= 6))) dom += 10 * ((i - 1) / bx);
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
  const bool nan = df2 != df2;
  if (nan) atomicExch(&st->newton_nan, 1);
  // the sub-domain's largest correction, combined over the warp's lanes of
  // the same sub-domain (a NaN counts as 0 here; the flag records it)
  atomic_max_nonneg_warp(&st->maxdf_bits[dom], nan ? 0.0 : df2);
}

// Stopping test of prim_inv_var (module_thermodynamics.f90:110-115,161-162)
// for sub-domains [d0, d1]: a sub-domain stops when its largest correction
// is below eps, or after itmax iterations with a convergence warning, as the
// reference's `it > itmax` exit.  Inside a captured graph (use_cond) the
// launch also sets the condition of the enclosing WHILE node: the loop runs
// while any sub-domain is still iterating.  Every iteration moves each live
// sub-domain one step closer to itmax, so the loop ends after at most itmax
// passes.
__global__ void k_newton_check(DevStatus* st, int d0, int d1, int nxb, double eps, int itmax,
                               cudaGraphConditionalHandle cond, int use_cond) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned live = 0;
  for (int b = 0; b < nxb; ++b)
    for (int d = d0 + 10 * b; d <= d1 + 10 * b; ++d) {
      if (st->done[d]) continue;
      st->it[d] += 1;
      const double err = sqrt(__longlong_as_double((long long)st->maxdf_bits[d]));
      st->maxdf_bits[d] = 0ULL;
      if (err < eps) st->done[d] = 1;
      else if (st->it[d] >= itmax) { st->done[d] = 1; st->newton_unconverged += 1; }
      if (st->done[d]) st->newton_it_max = max(st->newton_it_max, st->it[d]);
      else live = 1;
    }
  if (use_cond) cudaGraphSetConditional(cond, live);
}

// Slots of sub-domains [d0, d1] of every x-block start iterating; the slots
// of x-blocks b > 0 of a sub-domain that does not span x receive no points
// and stop on their first test.
__global__ void k_newton_reset(DevStatus* st, int d0, int d1, int nxb) {
  const int b = threadIdx.x / 16, d = d0 + threadIdx.x % 16;
  if (b < nxb && d <= d1) {
    const int q = d + 10 * b;
    st->done[q] = 0;
    st->it[q] = 0;
    st->maxdf_bits[q] = 0ULL;
  }
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
                      const double* __restrict__ W_i, const double* __restrict__ cp, DevStatus* st,
                      const double* __restrict__ mu_sgs = nullptr, double sc = 0.0, double sc_sgs = 1.0,
                      double pr = 0.0, double pr_sgs_i = 1.0) {
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
    // mu_SGS of the last fitted-transport LES flux (null: zero); the species
    // of the largest molecular D_k is picked on the host from dmx
    const double msgs = mu_sgs ? mu_sgs[p] : 0.0;
    const double dsgs = sc * msgs / (rho * sc_sgs);
#pragma unroll
    for (int l = 0; l < NRV; ++l) {
      dmx[l] = wk1[l] * c_thd.Kd[l] / (dm[l] * P);
      dmn[l] = d2 / (dmx[l] + dsgs);
    }
    rct = d2 * rho / (ct / cp[p] + pr * msgs * pr_sgs_i);
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

// Jet boundaries (module_BCs.f90).  The step start time and the step are
// read from device memory (tdt[0] = dt, tdt[1] = time0), so that the
// captured RK3 graph sees each step's values; tk is the stage fraction of
// timek = time0 + dt tk3(ik) (module_solver.f90:756).
struct JetArgs {
  const double* y;      // interior coordinates (code units), ny
  const double* z;      // nz
  const double* tdt;    // device: dt, time0
  double tk;
  double lx;            // domain length in x (code units)
  double hbuse, tmaxy, u2, T1, T2, P1, P2, pinf;   // the routines' constants in code units
  double u1;            // jet velocity (code units); 0: 1.01 x the jet's sound speed
  double ya1;           // fuel mass fraction of the jet
  double turb;          // relative amplitude of the seeded fluctuations
  double tq_i;          // 1 / the time quantum of the fluctuations (code units)
  unsigned long long seed;
  int planar;           // tanh profile in |y| instead of sqrt(y^2 + z^2)
  const double* dxi0;   // x metrics, ghosted index
};

// bc_inflowjet (module_BCs.f90:1646-1791), W face: one thread per (j, k)
// writes the ghost points and the first interior plane.  The exit sound
// speed uses a mass-fraction array whose unset entries are taken as 0.
template <int NRV>
__global__ void k_bc_inflowjet(Geo g, JetArgs ja, double* __restrict__ v) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)g.n[1] * g.n[2]) return;
  const int j = (int)(idx % g.n[1]) + 1, k = (int)(idx / g.n[1]) + 1;
  const double time = ja.tdt[1] + ja.tdt[0] * ja.tk;
  double T_1 = ja.T1, P_1 = ja.P1, Ya_1 = ja.ya1;
  const double T_2 = ja.T2, P_2 = ja.P2, Ya_2 = 0.0, u_2 = ja.u2;
  if (ja.tmaxy > 0.0 && time <= ja.tmaxy) {
    P_1 = (P_2 - (P_2 - P_1) * (time / ja.tmaxy) * (time / ja.tmaxy) * (time / ja.tmaxy));
    Ya_1 = (Ya_2 - (Ya_2 - Ya_1) * (time / ja.tmaxy) * (time / ja.tmaxy) * (time / ja.tmaxy));
    T_1 = (T_2 - (T_2 - T_1) * (time / ja.tmaxy) * (time / ja.tmaxy) * (time / ja.tmaxy));
  }
  double Ya[NRV];
#pragma unroll
  for (int l = 0; l < NRV; ++l) Ya[l] = 0.0;
  if constexpr (NRV == 2) { Ya[0] = 0.233; Ya[1] = 0.767; }
  else if constexpr (NRV == 3) { Ya[0] = Ya_1; Ya[1] = 0.0; Ya[2] = 1.0 - Ya_1; }
  else if constexpr (NRV == 9) { Ya[1] = Ya_1; Ya[3] = 0.0; Ya[8] = 1.0 - Ya_1; }
  double Ws_i = 0.0;
#pragma unroll
  for (int l = 0; l < NRV; ++l) Ws_i = Ws_i + Ya[l] * c_thd.Wc_i[l];
  const double cps = th_cp_mix<NRV>(T_1, Ya);
  double gamma = c_thd.gam2 * Ws_i / cps;
  gamma = 1.0 / (1.0 - gamma);
  const double cs = sqrt(gamma * Ws_i * T_1);
  const double u_1 = ja.u1 > 0.0 ? ja.u1 : 1.01 * cs;
  const double delt = 1.0 / (0.04 * ja.hbuse), y0 = ja.hbuse / 2.0;
  const double yy = ja.y[j - 1], zz = ja.z[k - 1];
  const double rrr = ja.planar ? fabs(yy) : sqrt(yy * yy + zz * zz);
  const double th = tanh((rrr - y0) * delt);
  double ux = 0.5 * ((u_1 + u_2) - (u_1 - u_2) * th);
  const double T = 0.5 * ((T_1 + T_2) - (T_1 - T_2) * th);
  const double P = 0.5 * ((P_1 + P_2) - (P_1 - P_2) * th);
  double vy = 0.0, wz = 0.0;
  if (ja.turb > 0.0) {
    const double a = ja.turb * u_1 * (0.5 * (1.0 - th));
    const long long n = (long long)floor(time * ja.tq_i);
    ux = ux + a * jet_noise(ja.seed, j, k, 0, n);
    vy = a * jet_noise(ja.seed, j, k, 1, n);
    wz = a * jet_noise(ja.seed, j, k, 2, n);
  }
#pragma unroll
  for (int l = 0; l < NRV; ++l) Ya[l] = 0.0;
  if constexpr (NRV == 2) {
    Ya[0] = 0.233;
    Ya[1] = 1.0 - Ya[0];
  } else if constexpr (NRV == 3) {
    Ya[0] = 0.5 * ((Ya_1 + 0.0) - (Ya_1 - 0.0) * th);
    Ya[1] = 0.5 * ((0.0 + 0.233) - (0.0 - 0.233) * th);
    Ya[2] = 0.5 * ((1.0 - Ya_1 + 0.767) - (1.0 - Ya_1 - 0.767) * th);
  } else if constexpr (NRV == 9) {
    Ya[1] = 0.5 * ((Ya_1 + 0.0) - (Ya_1 - 0.0) * th);
    Ya[3] = 0.5 * ((0.0 + 0.233) - (0.0 - 0.233) * th);
    Ya[8] = 0.5 * ((1.0 - Ya_1 + 0.767) - (1.0 - Ya_1 - 0.767) * th);
  }
  Ws_i = 0.0;
#pragma unroll
  for (int l = 0; l < NRV; ++l) Ws_i = Ws_i + Ya[l] * c_thd.Wc_i[l];
  const double rho = P / (T * Ws_i);
  double hm = 0.0;
#pragma unroll
  for (int l = 0; l < NRV; ++l) {
    double cpk;
    hm = hm + th_species(l, T, &cpk) * Ya[l];
  }
  const long long nc = g.ncell;
  for (int i = 1 - g.ng; i <= 1; ++i) {
    const long long p = gid(g, i, j, k);
    v[p] = rho;
    v[nc + p] = rho * ux;
    v[2 * nc + p] = rho * vy;
    v[3 * nc + p] = rho * wz;
    v[4 * nc + p] = rho * hm - P + 0.5 * rho * (ux * ux + vy * vy + wz * wz);
#pragma unroll
    for (int l = 0; l < NRV; ++l) v[(IZEM_NIV + l) * nc + p] = rho * Ya[l];
  }
}

// bc_nscbc_out (module_BCs.f90:2331-2516), E face: one thread per (j, k);
// 4th-order one-sided derivatives at the last interior point, the incoming
// wave relaxed toward the far-field pressure, the state advanced by dt
// written at the last interior plane and the ghost points.
template <int NRV>
__global__ void k_bc_nscbc_out(Geo g, JetArgs ja, const double* __restrict__ T, const double* __restrict__ W_i,
                               const double* __restrict__ cp, double* __restrict__ v) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)g.n[1] * g.n[2]) return;
  const int j = (int)(idx % g.n[1]) + 1, k = (int)(idx / g.n[1]) + 1;
  const double a4or[5] = {-3.0 / 12.0, 16.0 / 12.0, -36.0 / 12.0, 48.0 / 12.0, -25.0 / 12.0};   // m = -4..0
  const double dtime = ja.tdt[0], sigma1 = 0.28, Pinf = ja.pinf, Lx = ja.lx;
  const int ex = g.n[0];
  const double dxe = ja.dxi0[ex - 1 + g.ng];
  const long long nc = g.ncell;
  const long long p = gid(g, ex, j, k);
  double Machm = 0.0;
  double rho = v[p], rho_i = 1.0 / rho;
  double ux = v[nc + p] * rho_i, vy = v[2 * nc + p] * rho_i, wz = v[3 * nc + p] * rho_i;
  double Pres = v[p] * T[p] * W_i[p];
  double gam = c_thd.gam2 * W_i[p] / cp[p];
  gam = 1.0 / (1.0 - gam);
  double cs = sqrt(gam * Pres * rho_i);
  const double Mach = sqrt(ux * ux + vy * vy + wz * wz) / cs;
  Machm = fmax(Machm, Mach);
  double drho = 0.0, dux = 0.0, dvy = 0.0, dwz = 0.0, dPres = 0.0;
  double Ya[NRV], dYa[NRV];
#pragma unroll
  for (int l = 0; l < NRV; ++l) dYa[l] = 0.0;
#pragma unroll
  for (int m = -4; m <= 0; ++m) {
    const long long q = gid(g, ex + m, j, k);
    rho = v[q];
    rho_i = 1.0 / rho;
    ux = v[nc + q] * rho_i;
    vy = v[2 * nc + q] * rho_i;
    wz = v[3 * nc + q] * rho_i;
    Pres = v[q] * T[q] * W_i[q];
#pragma unroll
    for (int l = 0; l < NRV; ++l) Ya[l] = v[(IZEM_NIV + l) * nc + q] * rho_i;
    const double w = a4or[m + 4];
    drho = drho + w * rho;
    dux = dux + w * ux;
    dvy = dvy + w * vy;
    dwz = dwz + w * wz;
    dPres = dPres + w * Pres;
#pragma unroll
    for (int l = 0; l < NRV; ++l) dYa[l] = dYa[l] + w * Ya[l];
  }
  drho = -drho * dxe;
  dux = -dux * dxe;
  dvy = -dvy * dxe;
  dwz = -dwz * dxe;
  dPres = -dPres * dxe;
#pragma unroll
  for (int l = 0; l < NRV; ++l) dYa[l] = -dYa[l] * dxe;
  double L1 = 0.0, L2 = 0.0, L3 = 0.0, L4 = 0.0, L5 = 0.0, L5_Ya[NRV];
#pragma unroll
  for (int l = 0; l < NRV; ++l) L5_Ya[l] = 0.0;
  gam = c_thd.gam2 * W_i[p] / cp[p];
  gam = 1.0 / (1.0 - gam);
  cs = sqrt(gam * Pres * rho_i);
  if (ux - cs < 0.0) L1 = sigma1 * (1.0 - Machm * Machm) * cs / Lx * (Pres - Pinf);
  else L1 = (ux - cs) * (dPres - rho * cs * dux);
  if (ux + cs > 0.0) L5 = (ux + cs) * (dPres + rho * cs * dux);
  else L5 = (ux + cs) * (2.0 * dPres - L1 / (ux - cs));
  if (ux > 0.0) {
    L2 = ux * (cs * cs * drho - dPres);
    L3 = ux * dvy;
    L4 = ux * dwz;
#pragma unroll
    for (int l = 0; l < NRV; ++l) L5_Ya[l] = ux * dYa[l];
  } else {
    L2 = ux * cs * cs * drho - 0.5 * ux * (L5 / (ux + cs) + L1 / (ux - cs));
  }
  const double d2 = 0.5 * (L5 + L1);
  const double d1 = (L2 + d2) / (cs * cs);
  const double d3 = 0.5 * (L5 - L1) / (cs * rho);
  const double d4 = L3, d5 = L4;
  double hm = 0.0;
#pragma unroll
  for (int l = 0; l < NRV; ++l) {
    double cpk;
    hm = hm + th_species(l, T[p], &cpk) * Ya[l];
  }
  const double kin = ux * ux + vy * vy + wz * wz;
  for (int i = ex; i <= ex + g.ng; ++i) {
    const long long o = gid(g, i, j, k);
    v[o] = rho - d1 * dtime;
    v[nc + o] = (rho * ux) - (ux * d1 + rho * d3) * dtime;
    v[2 * nc + o] = (rho * vy) - (vy * d1 + rho * d4) * dtime;
    v[3 * nc + o] = (rho * wz) - (wz * d1 + rho * d5) * dtime;
    v[4 * nc + o] = (rho * hm - Pres + 0.5 * rho * kin) -
                    (0.5 * kin * d1 + rho * (ux * d3 + vy * d4 + wz * d5) + d2 / (gam - 1.0)) * dtime;
#pragma unroll
    for (int l = 0; l < NRV; ++l)
      v[(IZEM_NIV + l) * nc + o] = (rho * Ya[l]) - (Ya[l] * d1 + rho * L5_Ya[l]) * dtime;
  }
}

// upd_prim_var_dirichlet's force_sumY and W_i on the Dirichlet planes i = 1
// and i = nx of jet faces (before their Newton solve).
template <int NRV>
__global__ void k_dirichlet_prep(Geo g, int forcesum, double* __restrict__ v, double* __restrict__ W_i) {
  const long long np = (long long)g.n[1] * g.n[2];
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= 2 * np) return;
  const int face = (int)(idx / np);
  if (g.bc[face] != IZEM_BC_INFLOWJET && g.bc[face] != IZEM_BC_NSCBC_OUT) return;
  const long long r = idx - face * np;
  const long long p = gid(g, face ? g.n[0] : 1, (int)(r % g.n[1]) + 1, (int)(r / g.n[1]) + 1);
  if (forcesum) force_sumY_cell<NRV>(v, g.ncell, p);
  W_i[p] = wmix_cell<NRV>(v, g.ncell, p);
}

// Viscous and species-diffusion fluxes with fitted mixture transport:
// viscflux_xyz (module_viscflux.f90:1660-2189), prim_vis_vars
// (module_thermodynamics.f90:989-1230), the central / one-sided first
// derivatives of module_deriv.f90 (dx, d?_fixed1, d?_fixed2 share one
// arithmetic) and comm_deriv (module_parallel.f90:1788) as a periodic wrap.
#pragma once
#include "common.cuh"
#include "kernels_euler.cuh"

// module_deriv.f90:25-66 and dx (:212-478): 4th-order rows next to a
// physical boundary; then, with ng = 4, one 6th-order row and the 8th-order
// central stencil, with ng = 3 the 6th-order central stencil.
__device__ __forceinline__ double deriv_at(const double* __restrict__ a, long long p, long long stride, int s, int n,
                                           int lo_b, int hi_b, double di, int ng) {
  if (lo_b && s <= 3) {
    if (s == 1) {
      double dd = (-25.0 / 12.0) * a[p] + (48.0 / 12.0) * a[p + stride] + (-36.0 / 12.0) * a[p + 2 * stride] +
                  (16.0 / 12.0) * a[p + 3 * stride] + (-3.0 / 12.0) * a[p + 4 * stride];
      return dd * di;
    } else if (s == 2) {
      double dd = (-3.0 / 12.0) * a[p - stride] + (-10.0 / 12.0) * a[p] + (18.0 / 12.0) * a[p + stride] +
                  (-6.0 / 12.0) * a[p + 2 * stride] + (1.0 / 12.0) * a[p + 3 * stride];
      return dd * di;
    } else {
      double dd = (1.0 / 12.0) * a[p - 2 * stride] + (-8.0 / 12.0) * a[p - stride] + (8.0 / 12.0) * a[p + stride] +
                  (-1.0 / 12.0) * a[p + 2 * stride];
      return dd * di;
    }
  }
  if (hi_b && s >= n - 2) {
    if (s == n - 2) {
      double dd = (1.0 / 12.0) * a[p - 2 * stride] + (-8.0 / 12.0) * a[p - stride] + (8.0 / 12.0) * a[p + stride] +
                  (-1.0 / 12.0) * a[p + 2 * stride];
      return dd * di;
    } else if (s == n - 1) {
      double dd = (1.0 / 12.0) * a[p - 3 * stride] + (-6.0 / 12.0) * a[p - 2 * stride] + (18.0 / 12.0) * a[p - stride] +
                  (-10.0 / 12.0) * a[p] + (-3.0 / 12.0) * a[p + stride];
      return -dd * di;
    } else {
      double dd = (-3.0 / 12.0) * a[p - 4 * stride] + (16.0 / 12.0) * a[p - 3 * stride] + (-36.0 / 12.0) * a[p - 2 * stride] +
                  (48.0 / 12.0) * a[p - stride] + (-25.0 / 12.0) * a[p];
      return -dd * di;
    }
  }
  if (ng == 4 && !((lo_b && s == 4) || (hi_b && s == n - 3))) {
    double dd = (3.0 / 840.0) * a[p - 4 * stride] + (-32.0 / 840.0) * a[p - 3 * stride] +
                (168.0 / 840.0) * a[p - 2 * stride] + (-672.0 / 840.0) * a[p - stride] + (672.0 / 840.0) * a[p + stride] +
                (-168.0 / 840.0) * a[p + 2 * stride] + (32.0 / 840.0) * a[p + 3 * stride] + (-3.0 / 840.0) * a[p + 4 * stride];
    return dd * di;
  }
  double dd = (-1.0 / 60.0) * a[p - 3 * stride] + (9.0 / 60.0) * a[p - 2 * stride] + (-45.0 / 60.0) * a[p - stride] +
              (45.0 / 60.0) * a[p + stride] + (-9.0 / 60.0) * a[p + 2 * stride] + (1.0 / 60.0) * a[p + 3 * stride];
  return dd * di;
}

struct Metrics {
  const double* dxi[3];   // indexed (s - 1 + ng)
};

// Smagorinsky closure of viscflux_eg_LES_xyz (module_eg_lib.f90:2687-3352)
// and viscflux_LES_xyz (module_viscflux.f90:2200-2977) with
// mu_SGS_smagorinsky (module_SGS_models.f90:176-304); the isotropic SGS
// tensor is off (TAU_ISO_SGS_SWITCH = F), so its terms add exactly zero.
struct SgsArgs {
  const double* les;     // 4 ghosted components: dW_i/dx, dW_i/dy, dW_i/dz, shock-detector criterion
  const double* cp;      // ghosted cp (code units)
  const double* dxi[3];  // inverse spacings, ghosted index
  double cs2;            // MU_SGS_FACTOR^2 / sqgmr
  double sc;             // Sc of the reference scales
  double sc_sgs_i, pr_sgs_i;   // 1 / SC_SGS, 1 / PR_SGS
  double pr;             // Pr of the reference scales (fitted transport)
  double* mu_sgs;        // fitted transport: mu_SGS of every evaluated point, for the time step
};

// d?_fixed1 (module_deriv.f90:926-1171 and the y, z copies) at one interior
// point in IEEE round-to-nearest operations without contraction, in the
// reference's loop order (dd = dd + alpha(l) v(i+l), zero weights included,
// then dd dx_i): the same bits as a host evaluation of those loops.
__device__ __forceinline__ double deriv_rn(const double* __restrict__ a, long long p, long long stride, int s, int n,
                                          int lo_b, int hi_b, double di, int ng) {
  const double a4ol[5] = {-25.0 / 12.0, 48.0 / 12.0, -36.0 / 12.0, 16.0 / 12.0, -3.0 / 12.0};
  const double a4ul[5] = {-3.0 / 12.0, -10.0 / 12.0, 18.0 / 12.0, -6.0 / 12.0, 1.0 / 12.0};
  const double a4[5] = {1.0 / 12.0, -8.0 / 12.0, 0.0, 8.0 / 12.0, -1.0 / 12.0};
  const double a4ur[5] = {1.0 / 12.0, -6.0 / 12.0, 18.0 / 12.0, -10.0 / 12.0, -3.0 / 12.0};
  const double a4or[5] = {-3.0 / 12.0, 16.0 / 12.0, -36.0 / 12.0, 48.0 / 12.0, -25.0 / 12.0};
  const double a6[7] = {-1.0 / 60.0, 9.0 / 60.0, -45.0 / 60.0, 0.0, 45.0 / 60.0, -9.0 / 60.0, 1.0 / 60.0};
  const double a8[9] = {3.0 / 840.0,   -32.0 / 840.0, 168.0 / 840.0, -672.0 / 840.0, 0.0,
                        672.0 / 840.0, -168.0 / 840.0, 32.0 / 840.0, -3.0 / 840.0};
  const double* w;
  int l0, l1;
  bool neg = false;
  if (lo_b && s == 1) { w = a4ol; l0 = 0; l1 = 4; }
  else if (lo_b && s == 2) { w = a4ul; l0 = -1; l1 = 3; }
  else if (lo_b && s == 3) { w = a4; l0 = -2; l1 = 2; }
  else if (ng == 4 && ((lo_b && s == 4) || (hi_b && s == n - 3))) { w = a6; l0 = -3; l1 = 3; }
  else if (hi_b && s == n - 2) { w = a4; l0 = -2; l1 = 2; }
  else if (hi_b && s == n - 1) { w = a4ur; l0 = -3; l1 = 1; neg = true; }
  else if (hi_b && s == n) { w = a4or; l0 = -4; l1 = 0; neg = true; }
  else if (ng == 4) { w = a8; l0 = -4; l1 = 4; }
  else { w = a6; l0 = -3; l1 = 3; }
  double dd = 0.0;
  for (int l = l0; l <= l1; ++l) dd = __dadd_rn(dd, __dmul_rn(w[l - l0], a[p + l * stride]));
  return neg ? __dmul_rn(-dd, di) : __dmul_rn(dd, di);
}

// compute_duixj + shock_sensor_ducros (module_tools.f90:2521-2719): at every
// interior point the velocity gradient tensor (dx_fixed1 of u = rho u / rho),
// then the flag is set (never cleared) where
// (div u)^2 / ((div u)^2 + |curl u|^2 + 1e-30) > ducros_treduc.  The
// criterion's operations are uncontracted, in the reference's order.
__global__ void k_sensor_ducros(Geo g, Metrics mt, const double* __restrict__ prim, double treduc,
                                uint8_t* __restrict__ sensor) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= g.nint) return;
  int c[3];
  c[0] = (int)(idx % g.n[0]) + 1;
  long long r = idx / g.n[0];
  c[1] = (int)(r % g.n[1]) + 1;
  c[2] = (int)(r / g.n[1]) + 1;
  const long long nc = g.ncell;
  const long long p = gid(g, c[0], c[1], c[2]);
  const long long strides[3] = {1LL, (long long)g.g[0], (long long)g.g[0] * g.g[1]};
  const int nd = g.ndim;
  double du[9];   // du_a / dx_d at a * nd + d, a = u, v (, w)
  for (int a = 0; a < nd; ++a)
    for (int d = 0; d < nd; ++d)
      du[a * nd + d] = deriv_rn(prim + (PR_U + a) * nc, p, strides[d], c[d], g.n[d], g.bnd[2 * d], g.bnd[2 * d + 1],
                                mt.dxi[d][c[d] - 1 + g.ng], g.ng);
  double div, vort, wrk;
  if (nd == 3) {
    div = __dadd_rn(__dadd_rn(du[0], du[4]), du[8]);
    div = __dmul_rn(div, div);
    wrk = __dsub_rn(du[7], du[5]);
    vort = __dmul_rn(wrk, wrk);
    wrk = __dsub_rn(du[2], du[6]);
    wrk = __dmul_rn(wrk, wrk);
    vort = __dadd_rn(vort, wrk);
    wrk = __dsub_rn(du[3], du[1]);
    wrk = __dmul_rn(wrk, wrk);
    vort = __dadd_rn(vort, wrk);
  } else {
    div = __dadd_rn(du[0], du[3]);
    div = __dmul_rn(div, div);
    wrk = __dsub_rn(du[2], du[1]);
    vort = __dmul_rn(wrk, wrk);
  }
  const double ducloc = __ddiv_rn(div, __dadd_rn(__dadd_rn(div, vort), 1.0e-30));
  if (ducloc > treduc) sensor[p] = 1;
}

// First derivatives of u, v, w, T (fd 1..12) and of the mole fractions
// (fd 13.. : 3 per species) at interior points (module_viscflux.f90:1764-1804).
template <int NRV>
__global__ void k_grad(Geo g, Metrics mt, const double* __restrict__ prim, const double* __restrict__ T,
                       const double* __restrict__ Xa, double* __restrict__ fd) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= g.nint) return;
  int c[3];
  c[0] = (int)(idx % g.n[0]) + 1;
  long long r = idx / g.n[0];
  c[1] = (int)(r % g.n[1]) + 1;
  c[2] = (int)(r / g.n[1]) + 1;
  const long long nc = g.ncell;
  const long long p = gid(g, c[0], c[1], c[2]);
  const long long strides[3] = {1LL, (long long)g.g[0], (long long)g.g[0] * g.g[1]};
  const double* src[4] = {prim + PR_U * nc, prim + PR_V * nc, prim + PR_W * nc, T};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double di = mt.dxi[d][c[d] - 1 + g.ng];
    const int lo = g.bnd[2 * d], hi = g.bnd[2 * d + 1];
    const bool none = d == 2 && g.ndim == 2;   // a 2-D run has no z derivative
#pragma unroll
    for (int s = 0; s < 4; ++s)
      fd[(3 * s + d) * nc + p] = none ? 0.0 : deriv_at(src[s], p, strides[d], c[d], g.n[d], lo, hi, di, g.ng);
#pragma unroll
    for (int l = 0; l < NRV; ++l)
      fd[(12 + 3 * l + d) * nc + p] = none ? 0.0 : deriv_at(Xa + l * nc, p, strides[d], c[d], g.n[d], lo, hi, di, g.ng);
  }
}

// Periodic wrap of the face-ghost slabs of an ncomp-component ghosted array.
__global__ void k_wrap_periodic(Geo g, int ncomp, double* __restrict__ a) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long ntot = slab_count(g) - g.nint;
  if (idx >= ntot) return;
  int i, j, k, dom;
  if (!slab_point(g, idx + g.nint, i, j, k, dom)) return;
  const int f = dom - 1, d = f >> 1;
  if (g.bc[f] != IZEM_BC_PERIODIC) return;
  int c[3] = {i, j, k};
  c[d] = (f & 1) ? c[d] - g.n[d] : c[d] + g.n[d];
  const long long p = gid(g, i, j, k), q = gid(g, c[0], c[1], c[2]);
  for (int m = 0; m < ncomp; ++m) a[(long long)m * g.ncell + p] = a[(long long)m * g.ncell + q];
}

// Transport properties, stresses, diffusion velocities with correction
// velocity, and heat flux at interior points and at the ghost slabs of
// periodic faces (domain_id = -3..3).  Writes tau (6), q (3) and overwrites
// the species gradients of fd with rho Y_k V_k (module_viscflux.f90:1943-2062).
template <int NRV, bool LES = false>
__global__ void k_visc_point(Geo g, const double* __restrict__ v, const double* __restrict__ T,
                             const double* __restrict__ W_i, const double* __restrict__ ha,
                             const double* __restrict__ Xa, double* __restrict__ fd,
                             double* __restrict__ tau, double* __restrict__ qv, SgsArgs sa = SgsArgs{}) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  int i, j, k, dom;
  if (!slab_point(g, idx, i, j, k, dom)) return;
  if (dom > 0 && g.bnd[dom - 1]) return;
  const long long nc = g.ncell;
  const long long p = gid(g, i, j, k);
  const double rho = v[p], Tp = T[p], Wi = W_i[p];
  double X[NRV];
#pragma unroll
  for (int l = 0; l < NRV; ++l) X[l] = Xa[l * nc + p];
  // ---- prim_vis_vars for one point
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
#pragma unroll
  for (int m = 0; m < NRV; ++m)
#pragma unroll
    for (int l = m + 1; l < NRV; ++l) {
      const double* cf = c_thd.cofd[m][l];
      const double dkj = 0.0 + cf[0] * 1.0 + cf[1] * lt1 + cf[2] * lt2 + cf[3] * lt3;
      const double e = 1.0 / exp(dkj);
      dm[m] = dm[m] + xe[l] * e;   // order over l preserved for every m
      dm[l] = dm[l] + xe[m] * e;
      wk1[m] = wk1[m] + aw[l];
      wk1[l] = wk1[l] + aw[m];
    }
#pragma unroll
  for (int m = 0; m < NRV; ++m) dm[m] = wk1[m] * c_thd.Kd[m] / (dm[m] * P);
  double ct = 0.0, w1 = 0.0, eta[NRV], seta[NRV], reta[NRV];
#pragma unroll
  for (int l = 0; l < NRV; ++l) {
    const double* cl = c_thd.coflam[l];
    const double c1 = exp(0.0 + cl[0] * 1.0 + cl[1] * lt1 + cl[2] * lt2 + cl[3] * lt3);
    ct = ct + X[l] / c1;
    w1 = w1 + X[l] * c1;
    const double* ce = c_thd.cofeta[l];
    eta[l] = exp(0.0 + ce[0] * 1.0 + ce[1] * lt1 + ce[2] * lt2 + ce[3] * lt3);
    seta[l] = sqrt(eta[l]);
    reta[l] = 1.0 / seta[l];
  }
  ct = c_thd.Kl * (1.0 / ct + w1);
  double mu = 0.0;
#pragma unroll
  for (int m = 0; m < NRV; ++m) {
    double c4 = 0.0;
#pragma unroll
    for (int l = 0; l < NRV; ++l) {
      const double c3 = 1.0 + c_thd.wilke_c1[m][l] * (seta[m] * reta[l]);
      c4 = c4 + c3 * c3 * c_thd.wilke_c2[m][l] * X[l];
    }
    mu = mu + c_thd.Ku * (eta[m] * X[m] / c4);
  }
  // ---- stresses, diffusion and heat fluxes
  auto F = [&](int q1) -> double { return fd[(long long)(q1 - 1) * nc + p]; };
  const double rho_i = 1.0 / rho;
  const double uxs = v[nc + p] * rho_i, vys = v[2 * nc + p] * rho_i, wzs = v[3 * nc + p] * rho_i;
  // LES (viscflux_LES_xyz): mu_SGS_smagorinsky with filter_width's delta,
  // kept for the Fourier time step
  double mu_sgs = 0.0;
  if constexpr (LES) {
    const double dxv = sa.dxi[0][i - 1 + g.ng], dyv = sa.dxi[1][j - 1 + g.ng], dzv = sa.dxi[2][k - 1 + g.ng];
    const double delta = 1.0 / pow(dxv * dyv * dzv, 1.0 / 3.0);
    const double s11 = F(1), s12 = 0.5 * (F(2) + F(4)), s13 = 0.5 * (F(3) + F(7));
    const double s22 = F(5), s23 = 0.5 * (F(6) + F(8)), s33 = F(9);
    double sb = s11 * s11 + s12 * s12 + s13 * s13 + s12 * s12 + s22 * s22 + s23 * s23 + s13 * s13 + s23 * s23 +
                s33 * s33;
    sb = sqrt(sb + sb);
    mu_sgs = rho * sa.cs2 * (delta * delta) * sb * sa.les[3 * nc + p];
    sa.mu_sgs[p] = mu_sgs;
  }
  const double rmu = -c_thd.sqgmr * mu;
  const double rvd = c_thd.rvd0 * rho;
  const double twothirds = 2.0 / 3.0;
  const double sxx = twothirds * rmu * (F(1) + F(1) - (F(5) + F(9)));
  const double sxy = rmu * (F(4) + F(2));
  const double sxz = rmu * (F(7) + F(3));
  const double syy = twothirds * rmu * (F(5) + F(5) - (F(1) + F(9)));
  const double syz = rmu * (F(8) + F(6));
  const double szz = twothirds * rmu * (F(9) + F(9) - (F(1) + F(5)));
  double vdcx = 0.0, vdcy = 0.0, vdcz = 0.0;
#pragma unroll
  for (int l = 0; l < NRV; ++l) {
    const double wrk = dm[l] * c_thd.Wc[l] * Wi;
    vdcx = vdcx + wrk * F(13 + 3 * l);
    vdcy = vdcy + wrk * F(14 + 3 * l);
    vdcz = vdcz + wrk * F(15 + 3 * l);
  }
  double vdhx = 0.0, vdhy = 0.0, vdhz = 0.0;
  if constexpr (!LES) {
#pragma unroll
    for (int l = 0; l < NRV; ++l) {
      const double Ya = v[(IZEM_NIV + l) * nc + p] * rho_i;
      const double wrk = -dm[l] * c_thd.Wc[l] * Wi;
      const double vtx = vdcx * Ya + wrk * F(13 + 3 * l);
      const double vty = vdcy * Ya + wrk * F(14 + 3 * l);
      const double vtz = vdcz * Ya + wrk * F(15 + 3 * l);
      const double jx = rvd * vtx, jy = rvd * vty, jz = rvd * vtz;
      fd[(long long)(12 + 3 * l) * nc + p] = jx;
      fd[(long long)(13 + 3 * l) * nc + p] = jy;
      fd[(long long)(14 + 3 * l) * nc + p] = jz;
      const double h = ha[l * nc + p];
      vdhx = vdhx + h * jx;
      vdhy = vdhy + h * jy;
      vdhz = vdhz + h * jz;
    }
  } else {
    // the species fluxes of viscflux_LES_xyz: the enthalpy flux from the
    // molecular part, then the SGS diffusion and W_i-gradient terms
    const double dm_sgs = sa.sc * mu_sgs * rho_i * sa.sc_sgs_i;
    const double gwx = sa.les[p], gwy = sa.les[nc + p], gwz = sa.les[2 * nc + p];
#pragma unroll
    for (int l = 0; l < NRV; ++l) {
      const double Ya = v[(IZEM_NIV + l) * nc + p] * rho_i;
      const double dxa = F(13 + 3 * l), dya = F(14 + 3 * l), dza = F(15 + 3 * l);
      const double dmrw = -dm[l] * c_thd.Wc[l] * Wi;
      double vtx = vdcx * Ya, vty = vdcy * Ya, vtz = vdcz * Ya;
      const double hr = ha[l * nc + p] * rvd;
      vdhx = vdhx + hr * (vtx + dmrw * dxa);
      vdhy = vdhy + hr * (vty + dmrw * dya);
      vdhz = vdhz + hr * (vtz + dmrw * dza);
      double wrk = dmrw - dm_sgs * c_thd.Wc[l] * Wi;
      vtx = vtx + wrk * dxa;
      vty = vty + wrk * dya;
      vtz = vtz + wrk * dza;
      wrk = -dm_sgs * c_thd.Wc[l] * X[l];
      vtx = vtx + wrk * gwx;
      vty = vty + wrk * gwy;
      vtz = vtz + wrk * gwz;
      fd[(long long)(12 + 3 * l) * nc + p] = rvd * vtx;
      fd[(long long)(13 + 3 * l) * nc + p] = rvd * vty;
      fd[(long long)(14 + 3 * l) * nc + p] = rvd * vtz;
    }
  }
  double rlam;
  if constexpr (LES) {
    rlam = -c_thd.rlam0 * (ct + sa.pr * mu_sgs * sa.cp[p] * sa.pr_sgs_i);
    // the momentum divergence takes the SGS-scaled stresses, the heat flux
    // below the molecular ones
    const double fs = 1.0 + -c_thd.sqgmr * mu_sgs / rmu;
    tau[0 * nc + p] = sxx * fs; tau[1 * nc + p] = sxy * fs; tau[2 * nc + p] = sxz * fs;
    tau[3 * nc + p] = syy * fs; tau[4 * nc + p] = syz * fs; tau[5 * nc + p] = szz * fs;
  } else {
    rlam = -c_thd.rlam0 * ct;
    tau[0 * nc + p] = sxx; tau[1 * nc + p] = sxy; tau[2 * nc + p] = sxz;
    tau[3 * nc + p] = syy; tau[4 * nc + p] = syz; tau[5 * nc + p] = szz;
  }
  qv[0 * nc + p] = uxs * sxx + vys * sxy + wzs * sxz + rlam * F(10) + vdhx;
  qv[1 * nc + p] = uxs * sxy + vys * syy + wzs * syz + rlam * F(11) + vdhy;
  qv[2 * nc + p] = uxs * sxz + vys * syz + wzs * szz + rlam * F(12) + vdhz;
}

// Divergence of the viscous fluxes added to f (module_viscflux.f90:2098-2183).
template <int NRV>
__global__ void k_visc_div(Geo g, Metrics mt, const double* __restrict__ tau, const double* __restrict__ qv,
                           const double* __restrict__ fd, double* __restrict__ fl) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= g.nint) return;
  int c[3];
  c[0] = (int)(idx % g.n[0]) + 1;
  long long r = idx / g.n[0];
  c[1] = (int)(r % g.n[1]) + 1;
  c[2] = (int)(r / g.n[1]) + 1;
  const long long nc = g.ncell;
  const long long p = gid(g, c[0], c[1], c[2]);
  const long long st[3] = {1LL, (long long)g.g[0], (long long)g.g[0] * g.g[1]};
  double di[3];
  int lo[3], hi[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    di[d] = mt.dxi[d][c[d] - 1 + g.ng];
    lo[d] = g.bnd[2 * d];
    hi[d] = g.bnd[2 * d + 1];
  }
  auto div3 = [&](const double* ax, const double* ay, const double* az) {
    const double wx = deriv_at(ax, p, st[0], c[0], g.n[0], lo[0], hi[0], di[0], g.ng);
    const double wy = deriv_at(ay, p, st[1], c[1], g.n[1], lo[1], hi[1], di[1], g.ng);
    const double wz = g.ndim == 2 ? 0.0 : deriv_at(az, p, st[2], c[2], g.n[2], lo[2], hi[2], di[2], g.ng);
    return wx + wy + wz;
  };
  const long long ni = g.nint;
  fl[1 * ni + idx] = fl[1 * ni + idx] + div3(tau + 0 * nc, tau + 1 * nc, tau + 2 * nc);
  fl[2 * ni + idx] = fl[2 * ni + idx] + div3(tau + 1 * nc, tau + 3 * nc, tau + 4 * nc);
  fl[3 * ni + idx] = fl[3 * ni + idx] + div3(tau + 2 * nc, tau + 4 * nc, tau + 5 * nc);
  fl[4 * ni + idx] = fl[4 * ni + idx] + div3(qv + 0 * nc, qv + 1 * nc, qv + 2 * nc);
#pragma unroll
  for (int l = 0; l < NRV; ++l)
    fl[(IZEM_NIV + l) * ni + idx] = fl[(IZEM_NIV + l) * ni + idx] +
        div3(fd + (12 + 3 * l) * nc, fd + (13 + 3 * l) * nc, fd + (14 + 3 * l) * nc);
}

// Convective part of the RHS: primitive pre-pass (K1), characteristic
// LLF-WENO face fluxes (K2), flux difference, Adams-Shariff sensor (K3).
//
// Reference: module_weno.f90 euler_LLF_x/_y/_z (:537-2125), wenorec_nw
// (:236-275), wenorec (:286-527); module_tools.f90 sensor (:2733-2814).
#pragma once
#include "common.cuh"
#include "thermo.cuh"

enum { PR_RHOI = 0, PR_U = 1, PR_V = 2, PR_W = 3, PR_P = 4, PR_CS = 5, PR_HT = 6, PR_ET = 7, PR_N = 8 };

// Maps a linear index over the interior + face-ghost slabs (the points the
// reference's pencil pre-passes touch) to (i,j,k).  Returns false past the end.
__device__ __forceinline__ bool slab_point(const Geo& g, long long idx, int& i, int& j, int& k, int& dom) {
  const long long nin = g.nint;
  if (idx < nin) {
    i = (int)(idx % g.n[0]) + 1;
    long long r = idx / g.n[0];
    j = (int)(r % g.n[1]) + 1;
    k = (int)(r / g.n[1]) + 1;
    dom = 0;
    return true;
  }
  idx -= nin;
  // face f: ng layers x the two interior extents of the other axes
  for (int f = 0; f < 6; ++f) {
    int d = f >> 1;
    int a1 = d == 0 ? 1 : 0, a2 = d == 2 ? 1 : 2;
    long long sz = (long long)g.ng * g.n[a1] * g.n[a2];
    if (idx < sz) {
      int c1 = (int)(idx % g.n[a1]) + 1;
      long long r = idx / g.n[a1];
      int c2 = (int)(r % g.n[a2]) + 1;
      int layer = (int)(r / g.n[a2]) + 1;     // 1..ng
      int s = (f & 1) ? g.n[d] + layer : 1 - layer;
      int c[3];
      c[d] = s; c[a1] = c1; c[a2] = c2;
      i = c[0]; j = c[1]; k = c[2];
      dom = 1 + f;
      return true;
    }
    idx -= sz;
  }
  return false;
}

__host__ __device__ inline long long slab_count(const Geo& g) {
  long long s = g.nint;
  for (int d = 0; d < 3; ++d) {
    int a1 = d == 0 ? 1 : 0, a2 = d == 2 ? 1 : 2;
    s += 2LL * g.ng * g.n[a1] * g.n[a2];
  }
  return s;
}

// K1: per-point primitives used by the sweeps (module_weno.f90:634-667 and
// the y/z copies): 1/rho, u, v, w, P = rho T W_i, c = sqrt(gam P / rho),
// h_t = sum h_k Y_k + |u|^2/2, e_t = rho e_t / rho.  Also the mole fractions
// of molefrac (module_thermodynamics.f90:1669-1697) for the viscous flux.
template <int NRV>
__global__ void k_prim(Geo g, const double* __restrict__ v, const double* __restrict__ T,
                       const double* __restrict__ W_i, const double* __restrict__ cp,
                       const double* __restrict__ ha, double* __restrict__ prim,
                       double* __restrict__ Xa, DevStatus* st) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  int i, j, k, dom;
  if (!slab_point(g, idx, i, j, k, dom)) return;
  const long long nc = g.ncell;
  long long p = gid(g, i, j, k);
  double rho = v[p];
  double rho_i = 1.0 / rho;
  double ux = v[nc + p] * rho_i, vy = v[2 * nc + p] * rho_i, wz = v[3 * nc + p] * rho_i;
  double Wi = W_i[p];
  double P = rho * T[p] * Wi;
  if (P <= 0.0) atomicExch(&st->neg_pressure, 1);
  double gam = c_thd.gam2 * Wi / cp[p];
  gam = 1.0 / (1.0 - gam);
  double cs = sqrt(gam * P * rho_i);
  double ht = 0.0;
#pragma unroll
  for (int l = 0; l < NRV; ++l) {
    double rY = v[(IZEM_NIV + l) * nc + p];
    ht = ht + ha[l * nc + p] * (rY * rho_i);
    if (Xa) Xa[l * nc + p] = rY / (rho * Wi * c_thd.Wc[l]);
  }
  ht = ht + 0.5 * (ux * ux + vy * vy + wz * wz);
  prim[PR_RHOI * nc + p] = rho_i;
  prim[PR_U * nc + p] = ux;
  prim[PR_V * nc + p] = vy;
  prim[PR_W * nc + p] = wz;
  prim[PR_P * nc + p] = P;
  prim[PR_CS * nc + p] = cs;
  prim[PR_HT * nc + p] = ht;
  prim[PR_ET * nc + p] = v[4 * nc + p] * rho_i;
}

// Nonlinear WENO5 reconstruction (wenorec, ng = 3) of one characteristic
// field; gp/gm hold the 2ng = 6 stencil values (index 0 = point il-2).
__device__ __forceinline__ double weno5_nl(const double* vp, const double* vm) {
  const double eps = 1.0e-10;
  const double z1 = 13.0 / 12.0, z2 = 1.0 / 4.0;
  // '-' state at i+1/2, centre vp[2]
  double a, b, b0, b1, b2;
  double q0 = (1.0 / 3.0) * vp[2] + (5.0 / 6.0) * vp[3] + (-1.0 / 6.0) * vp[4];
  double q1 = (-1.0 / 6.0) * vp[1] + (5.0 / 6.0) * vp[2] + (1.0 / 3.0) * vp[3];
  double q2 = (1.0 / 3.0) * vp[0] + (-7.0 / 6.0) * vp[1] + (11.0 / 6.0) * vp[2];
  a = vp[2] + -2.0 * vp[3] + vp[4]; b = 3.0 * vp[2] + -4.0 * vp[3] + vp[4];
  b0 = z1 * a * a + z2 * b * b;
  a = vp[1] + -2.0 * vp[2] + vp[3]; b = vp[1] + -1.0 * vp[3];
  b1 = z1 * a * a + z2 * b * b;
  a = vp[0] + -2.0 * vp[1] + vp[2]; b = vp[0] + -4.0 * vp[1] + 3.0 * vp[2];
  b2 = z1 * a * a + z2 * b * b;
  double al0 = (3.0 / 10.0) / ((eps + b0) * (eps + b0));
  double al1 = (3.0 / 5.0) / ((eps + b1) * (eps + b1));
  double al2 = (1.0 / 10.0) / ((eps + b2) * (eps + b2));
  double s = 1.0 / (al0 + al1 + al2);
  double vminus = al0 * s * q0 + al1 * s * q1 + al2 * s * q2;
  // '+' state at i+1/2, centre vm[3]
  q0 = (11.0 / 6.0) * vm[3] + (-7.0 / 6.0) * vm[4] + (1.0 / 3.0) * vm[5];
  q1 = (1.0 / 3.0) * vm[2] + (5.0 / 6.0) * vm[3] + (-1.0 / 6.0) * vm[4];
  q2 = (-1.0 / 6.0) * vm[1] + (5.0 / 6.0) * vm[2] + (1.0 / 3.0) * vm[3];
  a = vm[3] + -2.0 * vm[4] + vm[5]; b = 3.0 * vm[3] + -4.0 * vm[4] + vm[5];
  b0 = z1 * a * a + z2 * b * b;
  a = vm[2] + -2.0 * vm[3] + vm[4]; b = vm[2] + -1.0 * vm[4];
  b1 = z1 * a * a + z2 * b * b;
  a = vm[1] + -2.0 * vm[2] + vm[3]; b = vm[1] + -4.0 * vm[2] + 3.0 * vm[3];
  b2 = z1 * a * a + z2 * b * b;
  al0 = (1.0 / 10.0) / ((eps + b0) * (eps + b0));
  al1 = (3.0 / 5.0) / ((eps + b1) * (eps + b1));
  al2 = (3.0 / 10.0) / ((eps + b2) * (eps + b2));
  s = 1.0 / (al0 + al1 + al2);
  double vplus = al0 * s * q0 + al1 * s * q1 + al2 * s * q2;
  return vminus + vplus;
}

// Nonlinear WENO7 reconstruction (wenorec, ng = 4, module_weno.f90:286-527):
// vp/vm hold the 2ng = 8 stencil values (index 0 = point il-3).
__device__ __forceinline__ double weno7_nl(const double* vp, const double* vm) {
  const double eps = 1.0e-10;
  const double za = 547.0, zb = -1854.0, zc = 4642.0, zd = -3882.0, ze = -17246.0, zf = 2107.0, zg = 7043.0,
               zh = -9402.0, zi = 11003.0, zl = 7042.0, zm = 3443.0, zn = -5966.0, zo = -2522.0, zp = 1602.0,
               zq = 2843.0, zr = 267.0, zs = 1922.0, zt = -494.0, zu = -1642.0;
  // cweno(r, j), r = -1..3
  const double cw[5][4] = {{25.0 / 12.0, -23.0 / 12.0, 13.0 / 12.0, -1.0 / 4.0},
                           {1.0 / 4.0, 13.0 / 12.0, -5.0 / 12.0, 1.0 / 12.0},
                           {-1.0 / 12.0, 7.0 / 12.0, 7.0 / 12.0, -1.0 / 12.0},
                           {1.0 / 12.0, -5.0 / 12.0, 13.0 / 12.0, 1.0 / 4.0},
                           {-1.0 / 4.0, 13.0 / 12.0, -23.0 / 12.0, 25.0 / 12.0}};
  const double dw[4] = {4.0 / 35.0, 18.0 / 35.0, 12.0 / 35.0, 1.0 / 35.0};
  auto betas = [&](const double* q, int i, double* be) {   // q 0-based, centre i
    be[0] = q[i] * (zf * q[i] + zh * q[i + 1] + zl * q[i + 2] + zb * q[i + 3]) +
            q[i + 1] * (zi * q[i + 1] + ze * q[i + 2] + zc * q[i + 3]) + q[i + 2] * (zg * q[i + 2] + zd * q[i + 3]) +
            q[i + 3] * (za * q[i + 3]);
    be[1] = q[i - 1] * (za * q[i - 1] + zo * q[i] + zs * q[i + 1] + zt * q[i + 2]) +
            q[i] * (zm * q[i] + zn * q[i + 1] + zp * q[i + 2]) + q[i + 1] * (zq * q[i + 1] + zu * q[i + 2]) +
            q[i + 2] * (zr * q[i + 2]);
    be[2] = q[i - 2] * (zr * q[i - 2] + zu * q[i - 1] + zp * q[i] + zt * q[i + 1]) +
            q[i - 1] * (zq * q[i - 1] + zn * q[i] + zs * q[i + 1]) + q[i] * (zm * q[i] + zo * q[i + 1]) +
            q[i + 1] * (za * q[i + 1]);
    be[3] = q[i - 3] * (za * q[i - 3] + zd * q[i - 2] + zc * q[i - 1] + zb * q[i]) +
            q[i - 2] * (zg * q[i - 2] + ze * q[i - 1] + zl * q[i]) + q[i - 1] * (zi * q[i - 1] + zh * q[i]) +
            q[i] * (zf * q[i]);
  };
  double be[4], al[4], s, vminus = 0.0, vplus = 0.0;
  // '-' state at i+1/2: centre vp[3], cweno(r, j) on vp[3 - r + j]
  betas(vp, 3, be);
  s = 0.0;
#pragma unroll
  for (int r = 0; r < 4; ++r) { al[r] = dw[r] / ((eps + be[r]) * (eps + be[r])); s = s + al[r]; }
  s = 1.0 / s;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    double q = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j) q = q + cw[r + 1][j] * vp[3 - r + j];
    vminus = vminus + (al[r] * s) * q;
  }
  // '+' state at i+1/2: centre vm[4], cweno(r-1, j) on vm[4 - r + j], weights reversed
  betas(vm, 4, be);
  s = 0.0;
#pragma unroll
  for (int r = 0; r < 4; ++r) { al[r] = dw[3 - r] / ((eps + be[r]) * (eps + be[r])); s = s + al[r]; }
  s = 1.0 / s;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    double q = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j) q = q + cw[r][j] * vm[4 - r + j];
    vplus = vplus + (al[r] * s) * q;
  }
  return vminus + vplus;
}

template <int NG>
__device__ __forceinline__ double weno_nl(const double* vp, const double* vm) {
  if constexpr (NG == 4) return weno7_nl(vp, vm);
  else return weno5_nl(vp, vm);
}

// K2: one thread per cell face along axis D.  Characteristic projections use
// the structure of the left eigenvectors (module_weno.f90:775-874): the three
// acoustic/entropy rows are dense over (rho, m, rho e_t) plus a rank-one
// species term psi.w; the shear rows have two entries; the species rows are
// Y_s (a.w) + w_s.  The result equals the reference's dense nv x nv product
// up to rounding.  Linear (sensor-off) faces accumulate the WENO5 stencil
// while streaming over the 2NG stencil points; sensed faces keep the 2NG
// values.  NG = 3 is WENO5, NG = 4 WENO7 (module_weno.f90, ng branches).
//
// Sensor blocks (x sweep only): with bx < n[0] the x direction is read as
// n[0] / bx blocks of bx points, as in a run decomposed into MPI blocks whose
// shock sensor is never exchanged (module_weno.f90:973 reads the block's own
// flags; its ghosts stay unflagged).  A face then sees only the flags of the
// block that uses it.  With edge = 0 the kernel writes every face as seen by
// its left cell's block; with edge = 1 it runs over the faces on block edges
// only (nfaces = (n[0]/bx - 1) n[1] n[2]) and writes them as seen by the
// right block into fhat.
template <int NRV, int D, int NG>
__global__ void __launch_bounds__(256) k_euler_face(Geo g, int weno_avg, int linfix,
                                                    const double* __restrict__ v,
                                                    const double* __restrict__ prim,
                                                    const uint8_t* __restrict__ sensor,
                                                    double* __restrict__ fhat, long long nfaces, int bx, int edge) {
  constexpr int NV = IZEM_NIV + NRV;
  constexpr int T1 = D == 0 ? 1 : 0;
  constexpr int T2 = D == 2 ? 1 : 2;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= nfaces) return;
  int c[3];
  if (D == 0 && edge) {
    const int ne = g.n[0] / bx - 1;
    long long r = idx;
    c[0] = ((int)(r % ne) + 1) * bx;   // face between the last cell of a block and the next
    r /= ne;
    c[1] = (int)(r % g.n[1]) + 1;
    c[2] = (int)(r / g.n[1]) + 1;
  } else {
    long long r = idx;
    int e0 = D == 0 ? g.n[0] + 1 : g.n[0];
    int e1 = D == 1 ? g.n[1] + 1 : g.n[1];
    c[0] = (int)(r % e0); r /= e0;
    c[1] = (int)(r % e1); r /= e1;
    c[2] = (int)r;
    // faces run 0..n along D (face s between cells s and s+1); cells 1..n across
    if (D != 0) c[0] += 1;
    if (D != 1) c[1] += 1;
    if (D != 2) c[2] += 1;
  }
  const long long nc = g.ncell;
  const long long stride = D == 0 ? 1LL : (D == 1 ? (long long)g.g[0] : (long long)g.g[0] * g.g[1]);
  const long long pl = gid(g, c[0], c[1], c[2]);   // cell il
  const long long pr = pl + stride;                  // cell il+1
  const long long p0 = pl - (NG - 1) * stride;       // stencil point il-ng+1

  // ---- Roe average compatible with the EOS (module_weno.f90:726-761)
  const double rho_i_l = prim[PR_RHOI * nc + pl], rho_i_r = prim[PR_RHOI * nc + pr];
  const double r = sqrt(v[pr] * rho_i_l);
  const double r1 = 1.0 / (r + 1.0);
  double uc[3];
  uc[0] = (r * prim[PR_U * nc + pr] + prim[PR_U * nc + pl]) * r1;
  uc[1] = (r * prim[PR_V * nc + pr] + prim[PR_V * nc + pl]) * r1;
  uc[2] = (r * prim[PR_W * nc + pr] + prim[PR_W * nc + pl]) * r1;
  double Yc[NRV];
  double W_i_c = 0.0;
#pragma unroll
  for (int l = 0; l < NRV; ++l) {
    Yc[l] = (r * (v[(IZEM_NIV + l) * nc + pr] * rho_i_r) + v[(IZEM_NIV + l) * nc + pl] * rho_i_l) * r1;
    W_i_c = W_i_c + Yc[l] * c_thd.Wc_i[l];
  }
  const double ht_c = (r * prim[PR_HT * nc + pr] + prim[PR_HT * nc + pl]) * r1;
  const double et_c = (r * prim[PR_ET * nc + pr] + prim[PR_ET * nc + pl]) * r1;
  const double T_c = (ht_c - et_c) / W_i_c;
  double psi[NRV];
  const double cp_c = th_cp_ha<NRV>(T_c, Yc, psi);   // psi <- h_k(T_c)
  double gam_c = c_thd.gam2 * W_i_c / cp_c;
  gam_c = 1.0 / (1.0 - gam_c);
  const double cs_c = sqrt(gam_c * T_c * W_i_c);
  {
    const double wrk = (gam_c / (gam_c - 1.0)) * T_c;
#pragma unroll
    for (int l = 0; l < NRV; ++l) psi[l] = -(r * psi[l] + psi[l]) * r1 + wrk * c_thd.Wc_i[l];
  }
  const double cs_c_i = 1.0 / cs_c;
  const double q = 0.5 * (uc[0] * uc[0] + uc[1] * uc[1] + uc[2] * uc[2]);
  const double b2 = (gam_c - 1.0) / (cs_c * cs_c);
  const double b1 = b2 * q;
  const double xi = b1 - b2 * ht_c;
  const double un = uc[D];
  // left-eigenvector coefficients
  const double A0 = 0.5 * (b1 + un * cs_c_i), An = -0.5 * (b2 * un + cs_c_i);
  const double C0 = 0.5 * (b1 - un * cs_c_i), Cn = -0.5 * (b2 * un - cs_c_i);
  const double At1 = -0.5 * (b2 * uc[T1]), At2 = -0.5 * (b2 * uc[T2]);
  const double hb2 = 0.5 * b2;
  const double B1 = b2 * uc[0], B2 = b2 * uc[1], B3 = b2 * uc[2];
  const double opx = 1.0 + xi;
  const double E0 = opx * q, E1 = -opx * uc[0], E2 = -opx * uc[1], E3 = -opx * uc[2];

  // ---- stencil eigenvalue maxima (LLF) and shock flag
  double lm0 = -1.0, lm1 = -1.0, lm2 = -1.0;
  bool shk = false;
  // the block whose flags count (x sweep with sensor blocks only)
  const bool blocks = D == 0 && bx < g.n[0];
  auto xblock = [&](int s) { return (min(max(s, 1), g.n[0]) - 1) / bx; };
  const int view = blocks ? xblock(edge ? c[0] + 1 : c[0]) : 0;
#pragma unroll
  for (int st = 0; st < 2 * NG; ++st) {
    const long long ps = p0 + st * stride;
    const double u_s = prim[(PR_U + D) * nc + ps], c_s = prim[PR_CS * nc + ps];
    lm0 = fmax(fabs(u_s - c_s), lm0);
    lm1 = fmax(fabs(u_s), lm1);
    lm2 = fmax(fabs(u_s + c_s), lm2);
    const bool counts = !blocks || xblock(c[0] - NG + 1 + st) == view;
    shk = shk || (counts && sensor[ps] != 0);
  }
  shk = shk && (weno_avg != 0);

  double gh[NV];
  if (!shk) {
    // linear reconstruction (wenorec_nw).  The LLF speed of each field is
    // the same at every stencil point and the projection L is linear, so
    //   sum_st c_st (L f_st +/- lam L w_st) / 2 = (L F +/- lam L W) / 2
    // with F = sum_st c_st f_st and W = sum_st c_st w_st: the raw stencil
    // sums are accumulated while streaming over the points and projected
    // once each (the reference projects every point, module_weno.f90:953-989;
    // the two agree to rounding).
    // WENO5: the reference's (mirrored) coefficients on points 0..4 ('-') and
    // 1..5 ('+'), or the textbook ones (linfix); WENO7: the 7th-order
    // stencil on points 0..6 and 1..7
    const double cmr[8] = {-3.0, 27.0, 47.0, -13.0, 2.0, 0.0, 0.0, 0.0};
    const double cpr[8] = {0.0, 2.0, -13.0, 47.0, 27.0, -3.0, 0.0, 0.0};
    const double cmf[8] = {2.0, -13.0, 47.0, 27.0, -3.0, 0.0, 0.0, 0.0};
    const double cpf[8] = {0.0, -3.0, 27.0, 47.0, -13.0, 2.0, 0.0, 0.0};
    const double cm7[8] = {-3.0, 25.0, -101.0, 319.0, 214.0, -38.0, 4.0, 0.0};
    const double cp7[8] = {0.0, 4.0, -38.0, 214.0, 319.0, -101.0, 25.0, -3.0};
    double Wm[NV], Fm[NV], Wp[NV], Fp[NV];
#pragma unroll
    for (int m = 0; m < NV; ++m) { Wm[m] = 0.0; Fm[m] = 0.0; Wp[m] = 0.0; Fp[m] = 0.0; }
#pragma unroll
    for (int st = 0; st < 2 * NG; ++st) {
      const long long ps = p0 + st * stride;
      double w[NV], f[NV];
#pragma unroll
      for (int m = 0; m < NV; ++m) w[m] = v[m * nc + ps];
      const double u_s = prim[(PR_U + D) * nc + ps], P_s = prim[PR_P * nc + ps];
      f[0] = w[1 + D];
      f[1] = w[1] * u_s; f[2] = w[2] * u_s; f[3] = w[3] * u_s;
      f[1 + D] = w[1 + D] * u_s + P_s;
      f[4] = u_s * (w[4] + P_s);
#pragma unroll
      for (int l = IZEM_NIV; l < NV; ++l) f[l] = w[l] * u_s;
      const double ccm = NG == 4 ? cm7[st] : (linfix ? cmf[st] : cmr[st]);
      const double ccp = NG == 4 ? cp7[st] : (linfix ? cpf[st] : cpr[st]);
#pragma unroll
      for (int m = 0; m < NV; ++m) {
        Wm[m] = Wm[m] + ccm * w[m];
        Fm[m] = Fm[m] + ccm * f[m];
        Wp[m] = Wp[m] + ccp * w[m];
        Fp[m] = Fp[m] + ccp * f[m];
      }
    }
    // the structured left-eigenvector product of the nonlinear branch, on one vector
    auto project = [&](const double* w, double* pw) {
      double sw = 0.0;
#pragma unroll
      for (int l = 0; l < NRV; ++l) sw = sw + psi[l] * w[IZEM_NIV + l];
      const double Gw = -b1 * w[0] + B1 * w[1] + B2 * w[2] + B3 * w[3] - b2 * w[4] - b2 * sw;
      pw[0] = A0 * w[0] + An * w[1 + D] + At1 * w[1 + T1] + At2 * w[1 + T2] + hb2 * w[4] + hb2 * sw;
      pw[1] = w[0] + Gw;
      pw[2] = C0 * w[0] + Cn * w[1 + D] + At1 * w[1 + T1] + At2 * w[1 + T2] + hb2 * w[4] + hb2 * sw;
      pw[3] = -uc[T1] * w[0] + w[1 + T1];
      pw[4] = -uc[T2] * w[0] + w[1 + T2];
      pw[5] = E0 * w[0] + E1 * w[1] + E2 * w[2] + E3 * w[3] + opx * w[4] + xi * sw;
#pragma unroll
      for (int s = 0; s < NRV - 1; ++s) pw[6 + s] = Yc[s] * Gw + w[IZEM_NIV + s];
    };
    double pWm[NV], pFm[NV], pWp[NV], pFp[NV];
    project(Wm, pWm);
    project(Fm, pFm);
    project(Wp, pWp);
    project(Fp, pFp);
    constexpr double den = NG == 4 ? 1.0 / 420.0 : 1.0 / 60.0;
#pragma unroll
    for (int m = 0; m < NV; ++m) {
      const double lam = m == 0 ? lm0 : (m == 2 ? lm2 : lm1);
      const double am = 0.5 * (pFm[m] + lam * pWm[m]);   // sum c gplus
      const double ap = 0.5 * (pFp[m] - lam * pWp[m]);   // sum c gminus
      gh[m] = am * den + ap * den;
    }
  } else {
    // nonlinear reconstruction (wenorec): keep the 2NG stencil values of every field
    double gpl[NV][2 * NG], gmi[NV][2 * NG];
#pragma unroll 1
    for (int st = 0; st < 2 * NG; ++st) {
      const long long ps = p0 + st * stride;
      double w[NV], f[NV];
#pragma unroll
      for (int m = 0; m < NV; ++m) w[m] = v[m * nc + ps];
      const double u_s = prim[(PR_U + D) * nc + ps], P_s = prim[PR_P * nc + ps];
      f[0] = w[1 + D];
      f[1] = w[1] * u_s; f[2] = w[2] * u_s; f[3] = w[3] * u_s;
      f[1 + D] = w[1 + D] * u_s + P_s;
      f[4] = u_s * (w[4] + P_s);
#pragma unroll
      for (int l = IZEM_NIV; l < NV; ++l) f[l] = w[l] * u_s;
      double sw = 0.0, sf = 0.0;
#pragma unroll
      for (int l = 0; l < NRV; ++l) { sw = sw + psi[l] * w[IZEM_NIV + l]; sf = sf + psi[l] * f[IZEM_NIV + l]; }
      const double Gw = -b1 * w[0] + B1 * w[1] + B2 * w[2] + B3 * w[3] - b2 * w[4] - b2 * sw;
      const double Gf = -b1 * f[0] + B1 * f[1] + B2 * f[2] + B3 * f[3] - b2 * f[4] - b2 * sf;
      double pw[NV], pf[NV];
      pw[0] = A0 * w[0] + An * w[1 + D] + At1 * w[1 + T1] + At2 * w[1 + T2] + hb2 * w[4] + hb2 * sw;
      pf[0] = A0 * f[0] + An * f[1 + D] + At1 * f[1 + T1] + At2 * f[1 + T2] + hb2 * f[4] + hb2 * sf;
      pw[1] = w[0] + Gw;
      pf[1] = f[0] + Gf;
      pw[2] = C0 * w[0] + Cn * w[1 + D] + At1 * w[1 + T1] + At2 * w[1 + T2] + hb2 * w[4] + hb2 * sw;
      pf[2] = C0 * f[0] + Cn * f[1 + D] + At1 * f[1 + T1] + At2 * f[1 + T2] + hb2 * f[4] + hb2 * sf;
      pw[3] = -uc[T1] * w[0] + w[1 + T1];
      pf[3] = -uc[T1] * f[0] + f[1 + T1];
      pw[4] = -uc[T2] * w[0] + w[1 + T2];
      pf[4] = -uc[T2] * f[0] + f[1 + T2];
      pw[5] = E0 * w[0] + E1 * w[1] + E2 * w[2] + E3 * w[3] + opx * w[4] + xi * sw;
      pf[5] = E0 * f[0] + E1 * f[1] + E2 * f[2] + E3 * f[3] + opx * f[4] + xi * sf;
#pragma unroll
      for (int s = 0; s < NRV - 1; ++s) {
        pw[6 + s] = Yc[s] * Gw + w[IZEM_NIV + s];
        pf[6 + s] = Yc[s] * Gf + f[IZEM_NIV + s];
      }
#pragma unroll
      for (int m = 0; m < NV; ++m) {
        const double lam = m == 0 ? lm0 : (m == 2 ? lm2 : lm1);
        const double gp = 0.5 * (pf[m] + lam * pw[m]);
        gpl[m][st] = gp;
        gmi[m][st] = pf[m] - gp;
      }
    }
#pragma unroll 1
    for (int m = 0; m < NV; ++m) gh[m] = weno_nl<NG>(gpl[m], gmi[m]);
  }

  // ---- fhat = R ghat (module_weno.f90:881-989)
  double fh[NV];
  fh[0] = gh[0] + gh[1] + gh[2];
  fh[1 + D] = (un - cs_c) * gh[0] + un * gh[1] + (un + cs_c) * gh[2];
  fh[1 + T1] = uc[T1] * gh[0] + uc[T1] * gh[1] + uc[T1] * gh[2] + gh[3];
  fh[1 + T2] = uc[T2] * gh[0] + uc[T2] * gh[1] + uc[T2] * gh[2] + gh[4];
  fh[4] = (ht_c - un * cs_c) * gh[0] + q * gh[1] + (ht_c + un * cs_c) * gh[2] + uc[T1] * gh[3] + uc[T2] * gh[4] + gh[5];
#pragma unroll
  for (int s = 0; s < NRV - 1; ++s) fh[IZEM_NIV + s] = Yc[s] * gh[0] + Yc[s] * gh[2] + gh[6 + s];
  {
    const double wrk = -1.0 / psi[NRV - 1];
    double acc = Yc[NRV - 1] * gh[0] + Yc[NRV - 1] * gh[2] + wrk * gh[5];
#pragma unroll
    for (int s = 0; s < NRV - 1; ++s) acc = acc + (wrk * psi[s]) * gh[6 + s];
    fh[NV - 1] = acc;
  }
#pragma unroll
  for (int m = 0; m < NV; ++m) fhat[m * nfaces + idx] = fh[m];
}

// fl(i) = (fhat(i) - fhat(i-1)) * dx_i(i); the x sweep overwrites, y and z
// accumulate (module_weno.f90:995-1020, 1534-1558).
// With sensor blocks (bx < n[0], x sweep) the first cell of every block but
// the first takes its left face from fhat_edge, the block-edge faces as seen
// by that block (k_euler_face with edge = 1).
template <int D>
__global__ void k_flux_diff(Geo g, int nv, const double* __restrict__ fhat, long long nfaces,
                            const double* __restrict__ dxi, double* __restrict__ fl, int accumulate, int bx,
                            const double* __restrict__ fhat_edge, long long nedge) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= g.nint) return;
  int i = (int)(idx % g.n[0]) + 1;
  long long r = idx / g.n[0];
  int j = (int)(r % g.n[1]) + 1;
  int k = (int)(r / g.n[1]) + 1;
  // face index of the right face (s) in the face grid of axis D
  long long fr, fl_;
  int s;
  if (D == 0) { s = i; fr = (long long)i + (long long)(g.n[0] + 1) * ((j - 1) + (long long)g.n[1] * (k - 1)); fl_ = fr - 1; }
  else if (D == 1) { s = j; fr = (long long)(i - 1) + (long long)g.n[0] * (j + (long long)(g.n[1] + 1) * (k - 1)); fl_ = fr - g.n[0]; }
  else { s = k; fr = (long long)(i - 1) + (long long)g.n[0] * ((j - 1) + (long long)g.n[1] * k); fl_ = fr - (long long)g.n[0] * g.n[1]; }
  const double di = dxi[s - 1 + g.ng];
  const double* fleft = fhat;
  long long nleft = nfaces;
  if (D == 0 && bx < g.n[0] && i > 1 && (i - 1) % bx == 0) {
    const int ne = g.n[0] / bx - 1;
    fleft = fhat_edge;
    nleft = nedge;
    fl_ = (long long)((i - 1) / bx - 1) + (long long)ne * ((j - 1) + (long long)g.n[1] * (k - 1));
  }
  // fl_W / fl_E (and S, N, B, F): the boundary points of a non-reflecting
  // face take 0 times their flux difference (module_weno.f90:620-623, 1002,
  // 1018); bc_noreflectionweno supplies their normal term
  const double flag = ((s == 1 && g.bc[2 * D] == IZEM_BC_NOREFLECTION) ||
                       (s == g.n[D] && g.bc[2 * D + 1] == IZEM_BC_NOREFLECTION))
                          ? 0.0
                          : 1.0;
  for (int m = 0; m < nv; ++m) {
    double df = (fhat[m * nfaces + fr] - fleft[m * nleft + fl_]) * di;
    long long o = (long long)m * g.nint + idx;
    fl[o] = accumulate ? fl[o] + df * flag : df * flag;
  }
}

// bc_noreflectionweno (module_weno.f90:2129-4498), one face per launch, one
// thread per boundary point.  At the point's own state: the characteristic
// vectors of the flux Jacobian along the face normal D (the structure of
// k_euler_face's projections), the eigenvalues of the waves leaving the
// domain (min(., 0) on the low face, max(., 0) on the high one), and the
// one-sided derivative of the conserved variables over 2NG-1 points with
// wenopar's cnr weights (:199-217; for NG = 3 the reference keeps the first
// five of the 7-point set).  fl += R diag(L_s) L dw * dx_i.
template <int NRV, int D, int NG>
__global__ void k_bc_nr(Geo g, int hi, const double* __restrict__ v, const double* __restrict__ T,
                        const double* __restrict__ W_i, const double* __restrict__ cp,
                        const double* __restrict__ ha, const double* __restrict__ dxi, double* __restrict__ fl) {
  constexpr int NV = IZEM_NIV + NRV;
  constexpr int T1 = D == 0 ? 1 : 0;
  constexpr int T2 = D == 2 ? 1 : 2;
  const int m1 = D == 0 ? g.n[1] : g.n[0], m2 = D == 2 ? g.n[1] : g.n[2];
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)m1 * m2) return;
  const int q1 = (int)(idx % m1) + 1, q2 = (int)(idx / m1) + 1;
  const int sc = hi ? g.n[D] : 1;
  int c[3];
  c[D] = sc;
  c[D == 0 ? 1 : 0] = q1;
  c[D == 2 ? 1 : 2] = q2;
  const long long nc = g.ncell;
  const long long stride = D == 0 ? 1LL : (D == 1 ? (long long)g.g[0] : (long long)g.g[0] * g.g[1]);
  const long long p = gid(g, c[0], c[1], c[2]);
  const double rho_i = 1.0 / v[p];
  double uc[3];
  uc[0] = v[nc + p] * rho_i;
  uc[1] = v[2 * nc + p] * rho_i;
  uc[2] = v[3 * nc + p] * rho_i;
  const double P = v[p] * T[p] * W_i[p];
  double gam_c = c_thd.gam2 * W_i[p] / cp[p];
  gam_c = 1.0 / (1.0 - gam_c);
  const double cs_c = sqrt(gam_c * P * rho_i);
  double Yc[NRV], psi[NRV];
  double ht_c = 0.0;
  {
    const double wrk = (gam_c / (gam_c - 1.0)) * T[p];
#pragma unroll
    for (int l = 0; l < NRV; ++l) {
      Yc[l] = v[(IZEM_NIV + l) * nc + p] * rho_i;
      const double h = ha[l * nc + p];
      ht_c = ht_c + h * Yc[l];
      psi[l] = -h + wrk * c_thd.Wc_i[l];
    }
  }
  const double cs_c_i = 1.0 / cs_c;
  const double q = 0.5 * (uc[0] * uc[0] + uc[1] * uc[1] + uc[2] * uc[2]);
  ht_c = ht_c + q;
  const double b2 = (gam_c - 1.0) / (cs_c * cs_c);
  const double b1 = b2 * q;
  const double xi = b1 - b2 * ht_c;
  const double un = uc[D];
  // one-sided derivative (times the spacing) into the domain
  const double cnr[7] = {-49.0 / 20.0, 6.0, -15.0 / 2.0, 20.0 / 3.0, -15.0 / 4.0, 6.0 / 5.0, -1.0 / 6.0};
  const double sgn = hi ? -1.0 : 1.0;
  double w[NV];
#pragma unroll
  for (int m = 0; m < NV; ++m) w[m] = 0.0;
#pragma unroll
  for (int st = 0; st < 2 * NG - 1; ++st) {
    const long long ps = hi ? p - st * stride : p + st * stride;
    const double cw = sgn * cnr[st];
#pragma unroll
    for (int m = 0; m < NV; ++m) w[m] = w[m] + cw * v[m * nc + ps];
  }
  // L w (module_weno.f90:2224-2332 and the other faces' copies)
  double sw = 0.0;
#pragma unroll
  for (int l = 0; l < NRV; ++l) sw = sw + psi[l] * w[IZEM_NIV + l];
  const double hb2 = 0.5 * b2;
  const double Gw = -b1 * w[0] + b2 * uc[0] * w[1] + b2 * uc[1] * w[2] + b2 * uc[2] * w[3] - b2 * w[4] - b2 * sw;
  double pw[NV];
  pw[0] = 0.5 * (b1 + un * cs_c_i) * w[0] - 0.5 * (b2 * un + cs_c_i) * w[1 + D] - 0.5 * (b2 * uc[T1]) * w[1 + T1] -
          0.5 * (b2 * uc[T2]) * w[1 + T2] + hb2 * w[4] + hb2 * sw;
  pw[1] = w[0] + Gw;
  pw[2] = 0.5 * (b1 - un * cs_c_i) * w[0] - 0.5 * (b2 * un - cs_c_i) * w[1 + D] - 0.5 * (b2 * uc[T1]) * w[1 + T1] -
          0.5 * (b2 * uc[T2]) * w[1 + T2] + hb2 * w[4] + hb2 * sw;
  pw[3] = -uc[T1] * w[0] + w[1 + T1];
  pw[4] = -uc[T2] * w[0] + w[1 + T2];
  {
    const double opx = 1.0 + xi;
    pw[5] = opx * q * w[0] - opx * uc[0] * w[1] - opx * uc[1] * w[2] - opx * uc[2] * w[3] + opx * w[4] + xi * sw;
  }
#pragma unroll
  for (int s = 0; s < NRV - 1; ++s) pw[6 + s] = Yc[s] * Gw + w[IZEM_NIV + s];
  // the waves leaving the domain
  auto side = [&](double x) { return hi ? fmax(x, 0.0) : fmin(x, 0.0); };
  double gh[NV];
  gh[0] = side(un - cs_c) * pw[0];
  gh[2] = side(un + cs_c) * pw[2];
#pragma unroll
  for (int m = 0; m < NV; ++m)
    if (m != 0 && m != 2) gh[m] = side(un) * pw[m];
  // R gh (module_weno.f90:2334-2418)
  double fh[NV];
  fh[0] = gh[0] + gh[1] + gh[2];
  fh[1 + D] = (un - cs_c) * gh[0] + un * gh[1] + (un + cs_c) * gh[2];
  fh[1 + T1] = uc[T1] * gh[0] + uc[T1] * gh[1] + uc[T1] * gh[2] + gh[3];
  fh[1 + T2] = uc[T2] * gh[0] + uc[T2] * gh[1] + uc[T2] * gh[2] + gh[4];
  fh[4] = (ht_c - un * cs_c) * gh[0] + q * gh[1] + (ht_c + un * cs_c) * gh[2] + uc[T1] * gh[3] + uc[T2] * gh[4] + gh[5];
#pragma unroll
  for (int s = 0; s < NRV - 1; ++s) fh[IZEM_NIV + s] = Yc[s] * gh[0] + Yc[s] * gh[2] + gh[6 + s];
  {
    const double wrk = -1.0 / psi[NRV - 1];
    double acc = Yc[NRV - 1] * gh[0] + Yc[NRV - 1] * gh[2] + wrk * gh[5];
#pragma unroll
    for (int s = 0; s < NRV - 1; ++s) acc = acc + (wrk * psi[s]) * gh[6 + s];
    fh[NV - 1] = acc;
  }
  const double di = dxi[sc - 1 + g.ng];
  const long long o = fidx(g, c[0], c[1], c[2]);
#pragma unroll
  for (int m = 0; m < NV; ++m) fl[(long long)m * g.nint + o] += fh[m] * di;
}

// K3: Adams-Shariff sensor, sticky (only ever sets).  Interior neighbour tests
// along +x, +y, +z (module_tools.f90:2756-2812).
// With x blocks of bx points (bx < n[0]) a block's last point is not
// compared with the next block's first (each MPI block loops to its own ex).
__global__ void k_sensor(Geo g, double mrw, const double* __restrict__ v, const double* __restrict__ T,
                         const double* __restrict__ W_i, uint8_t* __restrict__ sensor, int bx) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= g.nint) return;
  int c[3];
  c[0] = (int)(idx % g.n[0]) + 1;
  long long r = idx / g.n[0];
  c[1] = (int)(r % g.n[1]) + 1;
  c[2] = (int)(r / g.n[1]) + 1;
  const long long p = gid(g, c[0], c[1], c[2]);
  const double rho = v[p];
  const double rho_i = 1.0 / rho;
  const double P = rho * T[p] * W_i[p];
  bool set = false;
  const long long strides[3] = {1LL, (long long)g.g[0], (long long)g.g[0] * g.g[1]};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (c[d] <= g.n[d] - 1 && !(d == 0 && c[0] % bx == 0)) {
      const long long q = p + strides[d];
      const double rq = v[q];
      const double rho_iq = 1.0 / rq;
      const double Pq = rq * T[q] * W_i[q];
      const double drho = fabs(rq - rho) * fmin(rho_i, rho_iq);
      const double dpres = fabs(Pq - P) / fmin(P, Pq);
      if (drho > mrw && dpres > mrw) set = true;
    }
  }
  if (set) sensor[p] = 1;
}

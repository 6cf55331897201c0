// EGLIB precision-1 mixture transport and the viscous flux that uses it:
// viscflux_eg_xyz with egvars (module_eg_lib.f90:106-310, 2140-2676).
//
// Per point, the kernel evaluates the EGlib 3.4 routines that egvars calls
// with eglib_precision = 1 (A. Ern and V. Giovangigli, devel-izem/src/eglib/
// EGSlib.f): EGSPAR/LSPAR with IFLAG = 7 (pure viscosities, reciprocal binary
// diffusion coefficients, collision-integral ratios A*, B*, C*, internal heat
// capacities and Parker's rotational relaxation), EGSE2 (shear viscosity, one
// conjugate-gradient step on the matrix H with the 1000 K A*), EGSLCT2
// (conductivity and rescaled thermal diffusion ratios, a direct
// factorisation of Lambda_[e]) and EGSDR1 (rho times the flux diffusion
// matrix, two stationary steps on L_[00] and the mass-conservation
// projection), in the reference's operation order.  EGSL2 and EGSK2, also
// called there, only produce values that the reference discards (the
// conductivity is recomputed by EGSLCT2 and the volume viscosity is set to
// zero, module_eg_lib.f90:288).
//
// The species gradients keep the fitted-transport layout of fd
// (12 + 3 l + d) so that k_visc_div is shared; the pressure gradients of
// the EGLIB flux (fd 13-15 in the reference) sit after them (12 + 3 NRV + d).
#pragma once
#include <cmath>
#include "common.cuh"
#include "kernels_visc.cuh"

struct DevEg {
  int ns;
  int lin[IZEM_NSMAX];
  double wt[IZEM_NSMAX], eps[IZEM_NSMAX], dip[IZEM_NSMAX], zrot[IZEM_NSMAX];
  double cofe[IZEM_NSMAX][4];
  double cofd[IZEM_NSMAX][IZEM_NSMAX][4];
  double ctaij[IZEM_NSMAX][IZEM_NSMAX];              // A*_ij at 1000 K
  double fita[IZEM_NSMAX][IZEM_NSMAX][7];            // A*, B*, C* in powers of ln T
  double fitb[IZEM_NSMAX][IZEM_NSMAX][7];
  double fitc[IZEM_NSMAX][IZEM_NSMAX][7];
  // egvars scalings (module_eg_lib.f90:140-145)
  double cp_cgs, eta_adim, lbda_adim, rd_adim;
  // species and pair constants of the device evaluation (molar masses,
  // Parker's reference factor, EGLIB's fixed coefficients folded together)
  double wtru[IZEM_NSMAX];        // W_k / RU
  double cx[IZEM_NSMAX];          // CROT / (AAAA max(1, ZROT) pi): cxi = cx * BBBB
  double bdiag[IZEM_NSMAX];       // 5 PATMOS W / (6 RU): D_int,kk = bdiag / (T A*_kk eta_k)
  double lfac[IZEM_NSMAX];        // 5 PATMOS W / (3 RU): FAC of Lambda_[e] = lfac / (T eta_k)
  double wsinv[IZEM_NSMAX][IZEM_NSMAX];                    // 1 / (W_i + W_j)
  double hoff[IZEM_NSMAX][IZEM_NSMAX];                     // A*(1000) - 5/3
  double hdi[IZEM_NSMAX][IZEM_NSMAX], hdj[IZEM_NSMAX][IZEM_NSMAX];   // A* W_j/W_i + 5/3, A* W_i/W_j + 5/3
  double p1[IZEM_NSMAX][IZEM_NSMAX];                       // wwi wwj
  double tti[IZEM_NSMAX][IZEM_NSMAX], ttj[IZEM_NSMAX][IZEM_NSMAX];   // 4/3 wioj, 4/3 wjoi
  double c1j[IZEM_NSMAX][IZEM_NSMAX], c2j[IZEM_NSMAX][IZEM_NSMAX], c3j[IZEM_NSMAX][IZEM_NSMAX];
  double c1i[IZEM_NSMAX][IZEM_NSMAX], c2i[IZEM_NSMAX][IZEM_NSMAX], c3i[IZEM_NSMAX][IZEM_NSMAX];
  double c4[IZEM_NSMAX][IZEM_NSMAX];
};

static __constant__ DevEg c_eg;

// Host: EGINI's set-up (EGini.f:58-301) from the linking data -- pair well
// depths with the polar correction (LEVEPS), A* at 1000 K, and the A*, B*,
// C* fits re-expanded in ln T for every pair (EGABC).  The fit constants are
// EGLIB's published collision-integral ratio fits.
inline void eg_prepare(const izem_eglib& L, const izem_thd& t, const izem_adi& a, DevEg& E) {
  static const double fa0[7] = {.1106910525e+01, -.7065517161e-02, -.1671975393e-01, .1188708609e-01,
                                .7569367323e-03, -.1313998345e-02, .1720853282e-03};
  static const double fb0[7] = {.1199673577e+01, -.1140928763e+00, -.2147636665e-02, .2512965407e-01,
                                -.3030372973e-02, -.1445009039e-02, .2492954809e-03};
  static const double fc0[7] = {.8386993788e+00, .4748325276e-01, .3250097527e-01, -.1625859588e-01,
                                -.2260153363e-02, .1844922811e-02, -.2115417788e-03};
  const int n = L.ns;
  E = DevEg{};
  E.ns = n;
  for (int k = 0; k < n; ++k) {
    E.lin[k] = L.lin[k];
    E.wt[k] = L.wt[k];
    E.eps[k] = L.eps[k];
    E.dip[k] = L.dip[k];
    E.zrot[k] = L.zrot[k];
    for (int q = 0; q < 4; ++q) E.cofe[k][q] = L.cofe[k][q];
    for (int l = 0; l < n; ++l)
      for (int q = 0; q < 4; ++q) E.cofd[k][l][q] = L.cofd[k][l][q];
  }
  double lneps[IZEM_NSMAX][IZEM_NSMAX];
  const double fac = 1.0e-12, dipmin = 1.0e-20, boltz = 1.38056e-16;
  auto cube = [](double s) { return s * s * s; };
  for (int j = 0; j < n; ++j)
    for (int k = 0; k <= j; ++k) {
      double e = std::sqrt(L.eps[j] * L.eps[k]);
      int polar = -1, nonpolar = -1;
      if (L.dip[j] < dipmin && L.dip[k] > dipmin) { polar = k; nonpolar = j; }
      else if (L.dip[j] > dipmin && L.dip[k] < dipmin) { polar = j; nonpolar = k; }
      if (polar >= 0) {
        const double xi = 1.0 + 0.25 * (L.pol[nonpolar] / cube(L.sig[nonpolar])) * (fac / boltz) *
                                    (L.dip[polar] * L.dip[polar] / (L.eps[polar] * cube(L.sig[polar]))) *
                                    std::sqrt(L.eps[polar] / L.eps[nonpolar]);
        e = e * (xi * xi);
      }
      lneps[k][j] = lneps[j][k] = std::log(e);
    }
  const double l1000 = std::log(1.0e3);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      const double t1 = l1000 - lneps[i][j];
      const double t2 = t1 * t1, t3 = t1 * t2, t4 = t1 * t3, t5 = t1 * t4, t6 = t1 * t5;
      E.ctaij[i][j] = fa0[0] + fa0[1] * t1 + fa0[2] * t2 + fa0[3] * t3 + fa0[4] * t4 + fa0[5] * t5 + fa0[6] * t6;
    }
  for (int j = 0; j < n; ++j)
    for (int i = j; i < n; ++i)
      for (int m = 0; m < 7; ++m) {
        double sa = 0.0, sb = 0.0, sc = 0.0;
        for (int k = m; k <= 6; ++k) {
          double prod = 1.0;
          for (int l = 1; l <= k - m; ++l) prod = prod * (-lneps[i][j]) * double(m + l) / double(l);
          sa = sa + fa0[k] * prod;
          sb = sb + fb0[k] * prod;
          sc = sc + fc0[k] * prod;
        }
        E.fita[i][j][m] = E.fita[j][i][m] = sa;
        E.fitb[i][j][m] = E.fitb[j][i][m] = sb;
        E.fitc[i][j][m] = E.fitc[j][i][m] = sc;
      }
  const double ru = 8.314e7, patmos = 1.01325e6, pi = 3.1415926535;
  for (int k = 0; k < n; ++k) {
    const double crot = L.lin[k] == 1 ? 1.0 : (L.lin[k] == 2 ? 1.5 : 0.0);
    const double dr = L.eps[k] / 298.0, sqdr = std::sqrt(dr);
    const double aaaa = 1.0 + 2.7842 * sqdr + 4.4674 * dr + 5.5683 * (sqdr * dr);
    E.wtru[k] = L.wt[k] / ru;
    E.cx[k] = crot / (aaaa * std::max(1.0, L.zrot[k]) * pi);
    E.bdiag[k] = 5.0 * patmos * L.wt[k] / (6.0 * ru);
    E.lfac[k] = 5.0 * patmos * L.wt[k] / (3.0 * ru);
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      const double wi = L.wt[i], wj = L.wt[j];
      const double wwi = wi / (wi + wj), wwj = wj / (wi + wj);
      const double wioj = 3.0 * wi / wj - 2.0, wjoi = 3.0 * wj / wi - 2.0;
      const double A = E.ctaij[i][j];
      E.wsinv[i][j] = 1.0 / (wi + wj);
      E.hoff[i][j] = A - 5.0 / 3.0;
      E.hdi[i][j] = A * wj / wi + 5.0 / 3.0;
      E.hdj[i][j] = A * wi / wj + 5.0 / 3.0;
      const double p1 = wwi * wwj;
      E.p1[i][j] = p1;
      E.tti[i][j] = 4.0 / 3.0 * wioj;
      E.ttj[i][j] = 4.0 / 3.0 * wjoi;
      E.c1j[i][j] = 7.5 * wwi * wwi;
      E.c2j[i][j] = wwj * wwj;
      E.c3j[i][j] = 4.0 / 15.0 * p1 * wioj * wioj;
      E.c1i[i][j] = 7.5 * wwj * wwj;
      E.c2i[i][j] = wwi * wwi;
      E.c3i[i][j] = 4.0 / 15.0 * p1 * wjoi * wjoi;
      E.c4[i][j] = 20.0 / 3.0 * p1;
    }
  E.cp_cgs = 1.0e4 * a.cp_ref;
  E.eta_adim = 1.0e-1 / t.muinf;
  E.lbda_adim = 1.0e-5 / t.laminf;
  E.rd_adim = 1.0e-1 / (a.rho_ref * t.dinf[0]);
}

// packed symmetric index of EGLIB (0-based, i <= j)
template <int N>
__device__ __forceinline__ int egs(int i, int j) { return N * i - (i * (i + 1)) / 2 + j; }

template <int N>
__device__ __forceinline__ double eg_poly6(const double* f, double d1, double d2, double d3, double d4, double d5,
                                           double d6) {
  return f[0] + f[1] * d1 + f[2] * d2 + f[3] * d3 + f[4] * d4 + f[5] * d5 + f[6] * d6;
}

// One point: T [K], mole fractions, species cp [erg/g/K] -> eta [g/cm/s],
// lambda [erg/cm/s/K], chi (N), rho * D [g/cm/s] as D[l*N+m].  The same
// EGLIB formulas as the routines named above, with the factors that depend
// only on the species (molar masses, EGLIB's fixed coefficients, Parker's
// reference value) folded on the host, reciprocals instead of divisions,
// 1/eta from exp(-ln eta), and the packed factorisation with its scaling
// applied in place: the same quantities up to rounding.
template <int N>
__device__ void eg_point_dev(double T, const double* X, const double* cpms, double& eta_mix, double& tc,
                             double* chit, double* D) {
  constexpr int NP = N * (N + 1) / 2;
  const double patmos = 1.01325e6, ru = 8.314e7;
  const double Tinv = 1.0 / T;
  // ---- LSPAR (IFLAG = 7): pure viscosities, reciprocal binary diffusion
  // coefficients, internal heat capacities, Parker's rotational relaxation,
  // internal self-diffusion on the diagonal of BIN
  const double d1 = log(T);
  const double d2 = d1 * d1, d3 = d2 * d1, d4 = d3 * d1, d5 = d4 * d1, d6 = d5 * d1;
  double eta_i[N], bin[NP], cint[N], cxi[N];
#pragma unroll
  for (int k = 0; k < N; ++k) {
    const double* ce = c_eg.cofe[k];
    eta_i[k] = exp(-(ce[0] + ce[1] * d1 + ce[2] * d2 + ce[3] * d3));   // 1 / eta_k
  }
#pragma unroll
  for (int k = 0; k < N; ++k)
#pragma unroll
    for (int l = k + 1; l < N; ++l) {
      const double* cf = c_eg.cofd[k][l];
      bin[egs<N>(k, l)] = exp(-(cf[0] + cf[1] * d1 + cf[2] * d2 + cf[3] * d3));
    }
  const double pfac = 1.0 + 2.985e3 / (T * sqrt(T));   // polar correction of D_int
#pragma unroll
  for (int k = 0; k < N; ++k) {
    cint[k] = c_eg.lin[k] ? cpms[k] * c_eg.wtru[k] - 2.5 : 0.0;
    const double dd = c_eg.eps[k] * Tinv, sqdd = sqrt(dd);
    cxi[k] = c_eg.cx[k] * (1.0 + 2.7842 * sqdd + 4.4674 * dd + 5.5683 * (sqdd * dd));
    const double aii = eg_poly6<N>(c_eg.fita[k][k], d1, d2, d3, d4, d5, d6);
    double b = c_eg.bdiag[k] * Tinv * eta_i[k] / aii;
    if (c_eg.dip[k] != 0.0) b = b * pfac;
    bin[egs<N>(k, k)] = b;
  }
  // ---- EGSPAR: regularised mole and mass fractions
  double sum = 0.0;
#pragma unroll
  for (int i = 0; i < N; ++i) sum = sum + X[i];
  const double xm = sum * (1.0 / double(N)), sss = 1.0e-16;
  double xtr[N], ytr[N], aux[N];
  double wwtr = 0.0;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    xtr[i] = X[i] + sss * (xm - X[i]);
    wwtr = wwtr + xtr[i] * c_eg.wt[i];
  }
  const double wwtr_i = 1.0 / wwtr;
  double ysum = 0.0;
#pragma unroll
  for (int i = 0; i < N; ++i) { ytr[i] = xtr[i] * c_eg.wt[i] * wwtr_i; ysum = ysum + ytr[i]; }
#pragma unroll
  for (int i = 0; i < N; ++i) aux[i] = ysum - ytr[i];
  double g[NP], an[N];
  // ---- EGSE2: matrix H with the 1000 K A*, one conjugate-gradient step
  {
    const double fac = (6.0 * ru / (5.0 * patmos)) * T;
#pragma unroll
    for (int i = 0; i < N; ++i) g[egs<N>(i, i)] = xtr[i] * xtr[i] * eta_i[i];
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
      for (int j = i + 1; j < N; ++j) {
        const double a = xtr[i] * xtr[j] * fac * bin[egs<N>(i, j)] * c_eg.wsinv[i][j];
        g[egs<N>(i, j)] = a * c_eg.hoff[i][j];
        g[egs<N>(i, i)] = g[egs<N>(i, i)] + a * c_eg.hdi[i][j];
        g[egs<N>(j, j)] = g[egs<N>(j, j)] + a * c_eg.hdj[i][j];
      }
    double zn[N], tmp[N], aaa = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      zn[i] = xtr[i] / g[egs<N>(i, i)];
      aaa = aaa + zn[i] * xtr[i];
      tmp[i] = g[egs<N>(i, i)] * zn[i];
    }
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
      for (int j = i + 1; j < N; ++j) {
        tmp[i] = tmp[i] + g[egs<N>(i, j)] * zn[j];
        tmp[j] = tmp[j] + g[egs<N>(i, j)] * zn[i];
      }
    double bbb = 0.0, dot = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i) { bbb = bbb + zn[i] * tmp[i]; dot = dot + zn[i] * xtr[i]; }
    eta_mix = aaa / bbb * dot;
  }
  // ---- EGSLCT2: matrix Lambda_[e], factorisation, solve
  {
    double beta[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      beta[i] = (2.5 + cint[i]) * xtr[i];
      const double xx = xtr[i] * xtr[i];
      g[egs<N>(i, i)] = c_eg.lfac[i] * Tinv * eta_i[i] * xx * (1.0 + (8.0 / 15.0) * cxi[i]) + xx * cint[i] * bin[egs<N>(i, i)];
    }
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
      for (int j = i + 1; j < N; ++j) {
        const double A = eg_poly6<N>(c_eg.fita[i][j], d1, d2, d3, d4, d5, d6);
        const double B = eg_poly6<N>(c_eg.fitb[i][j], d1, d2, d3, d4, d5, d6);
        const double a = xtr[i] * xtr[j] * bin[egs<N>(i, j)];
        const double b3 = 6.25 - 3.0 * B;
        const double bbb = c_eg.p1[i][j] * (13.75 - 3.0 * B - 4.0 * A + A * (c_eg.tti[i][j] * cxi[i] + c_eg.ttj[i][j] * cxi[j]));
        const double a4 = 4.0 * A * c_eg.p1[i][j];
        const double bbj = c_eg.c1j[i][j] + b3 * c_eg.c2j[i][j] + a4 + A * (c_eg.c3j[i][j] * cxi[i] + c_eg.c4[i][j] * cxi[j]);
        const double bbi = c_eg.c1i[i][j] + b3 * c_eg.c2i[i][j] + a4 + A * (c_eg.c3i[i][j] * cxi[j] + c_eg.c4[i][j] * cxi[i]);
        g[egs<N>(i, j)] = -bbb * a;
        g[egs<N>(i, i)] = g[egs<N>(i, i)] + a * (bbj + cint[i]);
        g[egs<N>(j, j)] = g[egs<N>(j, j)] + a * (bbi + cint[j]);
      }
    // EGSDEC (packed LDL^T) and EGSSOL
#pragma unroll 1
    for (int k = 0; k < N; ++k) {
      double w[N];
      for (int j = 0; j < k; ++j) w[j] = g[egs<N>(j, j)] * g[egs<N>(j, k)];
      const int kk = egs<N>(k, k);
      double gkk = g[kk];
      for (int j = 0; j < k; ++j) gkk = gkk - w[j] * g[egs<N>(j, k)];
      g[kk] = gkk;
      const double rk = 1.0 / gkk;
      for (int i = k + 1; i < N; ++i) {
        double gki = g[egs<N>(k, i)];
        for (int j = 0; j < k; ++j) gki = gki - g[egs<N>(j, i)] * w[j];
        g[egs<N>(k, i)] = gki * rk;
      }
    }
#pragma unroll
    for (int i = 0; i < N; ++i) an[i] = beta[i];
#pragma unroll
    for (int j = 0; j < N - 1; ++j)
#pragma unroll
      for (int k = j + 1; k < N; ++k) an[k] = an[k] - g[egs<N>(j, k)] * an[j];
#pragma unroll
    for (int j = 0; j < N; ++j) an[j] = an[j] / g[egs<N>(j, j)];
#pragma unroll
    for (int j = N - 1; j >= 1; --j)
#pragma unroll
      for (int k = 0; k < j; ++k) an[k] = an[k] - g[egs<N>(k, j)] * an[j];
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i) s = s + an[i] * beta[i];
    tc = s * patmos * Tinv;
#pragma unroll
    for (int i = 0; i < N; ++i) chit[i] = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
      for (int j = i + 1; j < N; ++j) {
        const double C = eg_poly6<N>(c_eg.fitc[i][j], d1, d2, d3, d4, d5, d6);
        const double term = 0.5 * bin[egs<N>(i, j)] * (6.0 * C - 5.0) *
                            (c_eg.wt[i] * an[j] - c_eg.wt[j] * an[i]) * c_eg.wsinv[i][j];
        chit[i] = chit[i] + xtr[j] * term;
        chit[j] = chit[j] - xtr[i] * term;
      }
  }
  // ---- EGSDR1: matrix L_[00], two stationary steps, mass-conservation projection
  {
    double gd[N], dmi[N], tmp[N];
#pragma unroll
    for (int i = 0; i < N; ++i) gd[i] = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
      for (int j = i + 1; j < N; ++j) {
        const double a = xtr[i] * xtr[j] * bin[egs<N>(i, j)];
        g[egs<N>(i, j)] = a;   // holds -L_ij
        gd[i] = gd[i] + a;
        gd[j] = gd[j] + a;
      }
#pragma unroll
    for (int i = 0; i < N; ++i) dmi[i] = aux[i] / gd[i];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      D[i * N + i] = ytr[i] * (dmi[i] * (1.0 + ytr[i]));
#pragma unroll
      for (int j = i + 1; j < N; ++j) {
        const double dij = dmi[i] * dmi[j] * g[egs<N>(i, j)];
        D[i * N + j] = ytr[i] * dij;
        D[j * N + i] = ytr[j] * dij;
      }
    }
    const double rsumy = 1.0 / sum;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      double t = 0.0;
#pragma unroll
      for (int j = 0; j < N; ++j) t = t + D[i * N + j] * ytr[j];
      const double a = t * rsumy;
#pragma unroll
      for (int j = 0; j < N; ++j) D[i * N + j] = D[i * N + j] - a;
    }
#pragma unroll
    for (int i = 0; i < N; ++i) tmp[i] = 0.0;
#pragma unroll
    for (int j = 0; j < N; ++j)
#pragma unroll
      for (int i = 0; i < N; ++i) tmp[i] = tmp[i] + D[j * N + i];
    const double aa = (patmos / ru) * wwtr * Tinv;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const double yr = ytr[i] * rsumy;
#pragma unroll
      for (int j = 0; j < N; ++j) D[i * N + j] = aa * (D[i * N + j] - yr * tmp[j]);
    }
  }
}

// Species cp of egvars (module_eg_lib.f90:170-240): NASA-7 with the linear
// extrapolation outside [Tpolymin, Tpolymax], in erg/g/K.
template <int N>
__device__ __forceinline__ void eg_species_cp(double T, double* cpk) {
#pragma unroll
  for (int is = 0; is < N; ++is) {
    double t1 = T * c_thd.tinf, t2 = t1 * t1, t3 = t2 * t1, t4 = t3 * t1;
    const double* lo = c_thd.hc[is][0];
    const double* hi = c_thd.hc[is][1];
    double cpv;
    if (t1 < c_thd.tpolymin[is]) {
      t1 = c_thd.tpolymin[is]; t2 = t1 * t1; t3 = t2 * t1; t4 = t3 * t1;
      const double cp0 = lo[0] + lo[1] * t1 + lo[2] * t2 + lo[3] * t3 + lo[4] * t4;
      const double dcp0 = lo[1] + lo[2] * t1 * 2.0 + lo[3] * t2 * 3.0 + lo[4] * t3 * 4.0;
      cpv = c_thd.gam2 * c_thd.Wc_i[is] * (dcp0 * (T * c_thd.tinf - c_thd.tpolymin[is]) + cp0);
    } else if (t1 < c_thd.tpolylim[is]) {
      cpv = c_thd.gam2 * c_thd.Wc_i[is] * (lo[0] + lo[1] * t1 + lo[2] * t2 + lo[3] * t3 + lo[4] * t4);
    } else if (t1 < c_thd.tpolymax[is]) {
      cpv = c_thd.gam2 * c_thd.Wc_i[is] * (hi[0] + hi[1] * t1 + hi[2] * t2 + hi[3] * t3 + hi[4] * t4);
    } else {
      t1 = c_thd.tpolymax[is]; t2 = t1 * t1; t3 = t2 * t1; t4 = t3 * t1;
      const double cp0 = hi[0] + hi[1] * t1 + hi[2] * t2 + hi[3] * t3 + hi[4] * t4;
      const double dcp0 = hi[1] + hi[2] * t1 * 2.0 + hi[3] * t2 * 3.0 + hi[4] * t3 * 4.0;
      cpv = c_thd.gam2 * c_thd.Wc_i[is] * (dcp0 * (T * c_thd.tinf - c_thd.tpolymax[is]) + cp0);
    }
    cpk[is] = cpv * c_eg.cp_cgs;
  }
}

// Pressure gradients of the EGLIB flux (fd slots 12 + 3 NRV + d) from the
// primitive pressure P = rho T W_i.
template <int NRV>
__global__ void k_grad_p(Geo g, Metrics mt, const double* __restrict__ prim, double* __restrict__ fd) {
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
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double di = mt.dxi[d][c[d] - 1 + g.ng];
    fd[(12 + 3 * NRV + d) * nc + p] =
        deriv_at(prim + PR_P * nc, p, strides[d], c[d], g.n[d], g.bnd[2 * d], g.bnd[2 * d + 1], di, g.ng);
  }
}

// The W_i gradients of viscflux_eg_LES_xyz (dx_fixed1 etc., module_eg_lib.f90:
// 2866-2871) and the criterion of shock_det_slv (module_tools.f90:1945-2085)
// at the interior points: 0 where, on the 2 ng-point stencil of the point's
// x or y face, the relative density jump and the relative pressure jump of
// some neighbour pair both exceed PERCENT_WEIGHT_SGS, else 1.  The
// reference's z pass writes with the y pass's final j_l and the final k, a
// ghost corner that no later step reads, so only the x and y passes shape
// the criterion.  3-D only.
// With ducros != 0 (LES with the fitted transport, viscflux_LES_xyz) the
// criterion is shock_det_ducros_slv's (module_tools.f90:2099-2181): 0 where
// (div u)^2 / ((div u)^2 + |curl u|^2 + 1e-30) > PERCENT_WEIGHT_SGS, else 1,
// from velocity gradients by uncontracted dx_fixed1 stencils (deriv_rn), so
// that the 0/1 decision is the host evaluation's.
__global__ void k_les_prep(Geo g, Metrics mt, const double* __restrict__ v, const double* __restrict__ T,
                           const double* __restrict__ W_i, double pw, double* __restrict__ les,
                           const double* __restrict__ prim = nullptr, int ducros = 0) {
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
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double di = mt.dxi[d][c[d] - 1 + g.ng];
    les[d * nc + p] = deriv_at(W_i, p, strides[d], c[d], g.n[d], g.bnd[2 * d], g.bnd[2 * d + 1], di, g.ng);
  }
  double crit = 1.0;
  if (ducros) {
    double du[9];
    for (int a = 0; a < 3; ++a)
      for (int d = 0; d < 3; ++d)
        du[a * 3 + d] = deriv_rn(prim + (PR_U + a) * nc, p, strides[d], c[d], g.n[d], g.bnd[2 * d], g.bnd[2 * d + 1],
                                 mt.dxi[d][c[d] - 1 + g.ng], g.ng);
    double div = __dadd_rn(__dadd_rn(du[0], du[4]), du[8]);
    div = __dmul_rn(div, div);
    double wrk = __dsub_rn(du[7], du[5]);
    double vort = __dmul_rn(wrk, wrk);
    wrk = __dsub_rn(du[2], du[6]);
    vort = __dadd_rn(vort, __dmul_rn(wrk, wrk));
    wrk = __dsub_rn(du[3], du[1]);
    vort = __dadd_rn(vort, __dmul_rn(wrk, wrk));
    const double ratio = __ddiv_rn(div, __dadd_rn(__dadd_rn(div, vort), 1.0e-30));
    les[3 * nc + p] = ratio > pw ? 0.0 : 1.0;
    return;
  }
  for (int d = 0; d < 2; ++d)
    for (int st = 1; st <= 2 * g.ng; ++st) {
      const int s = c[d] + st - g.ng;           // i_s, from c - ng + 1 to c + ng
      const int sp = min(s + 1, g.n[d]);        // min(i_s + 1, ex)
      const long long pa = p + (long long)(s - c[d]) * strides[d];
      const long long pb = p + (long long)(sp - c[d]) * strides[d];
      const double drho = fabs(v[pb] - v[pa]) / fmin(v[pb], v[pa]);
      const double pp = v[pb] * T[pb] * W_i[pb];
      const double pm = v[pa] * T[pa] * W_i[pa];
      const double dpres = fabs(pp - pm) / fmin(pp, pm);
      if (drho > pw && dpres > pw) crit = 0.0;
    }
  les[3 * nc + p] = crit;
}

// egvars + the stresses, rho Y_k V_k and heat flux of viscflux_eg_xyz at
// interior points and the ghost slabs of periodic faces.  Writes tau (6),
// q (3) and overwrites the species gradients of fd with rho Y_k V_k.  With
// LES the terms of viscflux_eg_LES_xyz (module_eg_lib.f90:3017-3239): the
// divergence gets the stresses scaled by 1 + mu_SGS / mu, the species
// fluxes the SGS diffusion and W_i-gradient terms, the heat flux the SGS
// conductivity mu_SGS cp / Pr_SGS; the work term keeps the molecular
// stresses.  The reference reuses its temperature-gradient scalar wrk1 for
// the SGS factor of each species, so the x thermal-diffusion term of species
// l >= 2 uses the SGS factor of species l - 1; that is reproduced.
template <int NRV, bool LES = false>
__global__ void __launch_bounds__(256) k_visc_point_eg(Geo g, const double* __restrict__ v,
                                                       const double* __restrict__ T, const double* __restrict__ W_i,
                                                       const double* __restrict__ ha, const double* __restrict__ Xa,
                                                       const double* __restrict__ prim, double* __restrict__ fd,
                                                       double* __restrict__ tau, double* __restrict__ qv,
                                                       SgsArgs sa = SgsArgs{}) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  int i, j, k, dom;
  if (!slab_point(g, idx, i, j, k, dom)) return;
  if (dom > 0 && g.bnd[dom - 1]) return;
  const long long nc = g.ncell;
  const long long p = gid(g, i, j, k);
  const double rho = v[p], Tp = T[p], Wi = W_i[p];
  const double rho_i = 1.0 / rho;
  // ---- egvars
  double Xe[NRV], cpk[NRV];
  {
    const double wrk = rho_i * (1.0 / Wi);
#pragma unroll
    for (int l = 0; l < NRV; ++l) Xe[l] = v[(IZEM_NIV + l) * nc + p] * wrk * c_thd.Wc_i[l];
    eg_species_cp<NRV>(Tp, cpk);
  }
  double eta_eg, ct_eg, tdr[NRV], rd[NRV * NRV];
  eg_point_dev<NRV>(Tp * c_thd.tinf, Xe, cpk, eta_eg, ct_eg, tdr, rd);
  const double mu = eta_eg * c_eg.eta_adim;
  const double ct = ct_eg * c_eg.lbda_adim;
  // ---- fluxes
  auto F = [&](int q1) -> double { return fd[(long long)(q1 - 1) * nc + p]; };
  const double rmu = -c_thd.sqgmr * mu;
  const double rmk = -c_thd.sqgmr * 0.0;
  const double bulk = rmk * (F(1) + F(5) + F(9));
  const double twothirds = 2.0 / 3.0;
  const double sxx = bulk + twothirds * rmu * (F(1) + F(1) - (F(5) + F(9)));
  const double sxy = rmu * (F(4) + F(2));
  const double sxz = rmu * (F(7) + F(3));
  const double syy = bulk + twothirds * rmu * (F(5) + F(5) - (F(1) + F(9)));
  const double syz = rmu * (F(8) + F(6));
  const double szz = bulk + twothirds * rmu * (F(9) + F(9) - (F(1) + F(5)));
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
  }
  const double Ps = 1.0 / prim[PR_P * nc + p];
  const double Ts = 1.0 / Tp;
  const double w1 = F(10) * Ts, w2 = F(11) * Ts, w3 = F(12) * Ts;
  const double w4 = fd[(12 + 3 * NRV) * nc + p] * Ps;
  const double w5 = fd[(13 + 3 * NRV) * nc + p] * Ps;
  const double w6 = fd[(14 + 3 * NRV) * nc + p] * Ps;
  double dx[NRV], dy[NRV], dz[NRV], xt[NRV], xa[NRV];
#pragma unroll
  for (int l = 0; l < NRV; ++l) {
    const double X = Xa[l * nc + p];
    xa[l] = X;
    const double xy = X - v[(IZEM_NIV + l) * nc + p] * rho_i;
    dx[l] = F(13 + 3 * l) + xy * w4;
    dy[l] = F(14 + 3 * l) + xy * w5;
    dz[l] = F(15 + 3 * l) + xy * w6;
    xt[l] = X * tdr[l];
  }
  const double rvd0 = c_thd.rvd0;
  const double uxs = v[nc + p] * rho_i, vys = v[2 * nc + p] * rho_i, wzs = v[3 * nc + p] * rho_i;
  double sx = 0.0, sy = 0.0, sz = 0.0;
  const double dm_sgs = mu_sgs * rho_i * sa.sc_sgs_i;
  double w1c = w1;   // the reference's wrk1
#pragma unroll
  for (int l = 0; l < NRV; ++l) {
    double jx = 0.0, jy = 0.0, jz = 0.0;
#pragma unroll
    for (int m = 0; m < NRV; ++m) {
      const double r = rd[l * NRV + m] * c_eg.rd_adim;
      jx = jx + r * (dx[m] + xt[m] * (LES ? w1c : w1));
      jy = jy + r * (dy[m] + xt[m] * w2);
      jz = jz + r * (dz[m] + xt[m] * w3);
    }
    if constexpr (LES) {
      const double wk = rho * dm_sgs * sa.sc * c_thd.Wc[l];
      const double fw = 1.0 + wk * Wi;
      const double wx = wk * xa[l];
      jx = -rvd0 * (jx * fw + wx * sa.les[p]);
      jy = -rvd0 * (jy * fw + wx * sa.les[nc + p]);
      jz = -rvd0 * (jz * fw + wx * sa.les[2 * nc + p]);
      w1c = wk;
    } else {
      jx = -rvd0 * jx;
      jy = -rvd0 * jy;
      jz = -rvd0 * jz;
    }
    fd[(long long)(12 + 3 * l) * nc + p] = jx;
    fd[(long long)(13 + 3 * l) * nc + p] = jy;
    fd[(long long)(14 + 3 * l) * nc + p] = jz;
    const double h = ha[l * nc + p] + Tp * c_thd.Wc_i[l] * tdr[l];
    sx = sx + jx * h;
    sy = sy + jy * h;
    sz = sz + jz * h;
  }
  double wl;
  if constexpr (LES) {
    const double ct_sgs = mu_sgs * sa.cp[p] * sa.pr_sgs_i;
    wl = -c_thd.rlam0 * (ct + ct_sgs);
    const double fs = 1.0 + -c_thd.sqgmr * mu_sgs / rmu;
    tau[0 * nc + p] = bulk + (sxx - bulk) * fs; tau[1 * nc + p] = sxy * fs; tau[2 * nc + p] = sxz * fs;
    tau[3 * nc + p] = bulk + (syy - bulk) * fs; tau[4 * nc + p] = syz * fs; tau[5 * nc + p] = bulk + (szz - bulk) * fs;
  } else {
    wl = -c_thd.rlam0 * ct;
    tau[0 * nc + p] = sxx; tau[1 * nc + p] = sxy; tau[2 * nc + p] = sxz;
    tau[3 * nc + p] = syy; tau[4 * nc + p] = syz; tau[5 * nc + p] = szz;
  }
  qv[0 * nc + p] = sx + wl * F(10) + uxs * sxx + vys * sxy + wzs * sxz;
  qv[1 * nc + p] = sy + wl * F(11) + uxs * sxy + vys * syy + wzs * syz;
  qv[2 * nc + p] = sz + wl * F(12) + uxs * sxz + vys * syz + wzs * szz;
}

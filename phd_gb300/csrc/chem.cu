// Batched stiff chemistry on the GPU: one constant-volume reactor per cell,
// integrated by a device restatement of DVODE (BDF, internally generated
// full Jacobian, MF = 22) inside the reference's REACTION_V retry loop.
//
// Reference: module_reaction.f90:102-321 (reaction_dvode), chemkin/
// reaction_v.f:1-114 (REACTION_V, FUN; ITOL=1, RTOL=1e-6, ATOL=1e-10),
// chemkin/vode.f (CKWYR :1797, CKRATT :935, CKRATX :1130, CKCVBS :64, CKHMS
// :228, DVODE :4286-7790).
//
// Execution model: a persistent kernel whose threads each take the next
// cell from a global counter (atomicAdd) when their current cell finishes,
// so cells with few BDF steps do not wait for cells with many.  Every loop
// is bounded (MXSTEP = 500 steps per DVODE call, 20 calls, at most 10
// corrector failures and 7 error-test failures per step): the kernel
// cannot spin.  Per-thread DVODE arrays (Nordsieck history, iteration
// matrix and its saved Jacobian) live in local memory.
#include <cstdio>
#include <cstring>
#include <cmath>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include "../../include/izem_gpu.h"
#include "chem.h"

namespace {

__constant__ izem_mech c_mech_dev;
__constant__ int c_need_eqk_dev;   // some reaction uses the equilibrium reverse rate
#ifdef IZEM_CHEM_HOST_TEST
izem_mech c_mech_host;
int c_need_eqk_host = 0;
#define HD __host__ __device__
#ifdef __CUDA_ARCH__
#define c_mech c_mech_dev
#define c_need_eqk c_need_eqk_dev
#else
#define c_mech c_mech_host
#define c_need_eqk c_need_eqk_host
#endif
#else
#define HD __device__
#define c_mech c_mech_dev
#define c_need_eqk c_need_eqk_dev
#endif

constexpr int MXSP = 6;

HD __forceinline__ double powi(double x, int m) {
  unsigned n = m < 0 ? -m : m;
  double y = (n % 2) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2) y = y * x;
  }
  return m < 0 ? 1.0 / y : y;
}

template <int KK>
struct Thermo {
  // cv (mean, mass) and h_k at T (CKCVBS, CKHMS)
  HD static void cv_h(double T, const double* Y, double* cvb, double* h) {
    const double T2 = T * T, T3 = T * T2, T4 = T2 * T2;
    const double rut = T * c_mech.ru;
    double cv = 0.0;
#pragma unroll
    for (int k = 0; k < KK; ++k) {
      const double* a = c_mech.a[k][T > c_mech.tmid[k] ? 1 : 0];
      const double cps = 1.0 * a[0] + T * a[1] + T2 * a[2] + T3 * a[3] + T4 * a[4];
      const double cvk = c_mech.ru * cps / c_mech.wt[k] - c_mech.ru / c_mech.wt[k];
      cv = cv + Y[k] * cvk;
      const double hs = 1.0 * a[0] + (T / 2) * a[1] + (T2 / 3) * a[2] + (T3 / 4) * a[3] + (T4 / 5) * a[4];
      h[k] = rut * (hs + a[5] / T) / c_mech.wt[k];
    }
    *cvb = cv;
  }
};

// CKWYR: molar production rates (mol cm^-3 s^-1)
template <int KK>
HD void ck_wyr(double rho, double T, const double* Y, double* wdot) {
  const int ii = c_mech.ii;
  const double alogt = log(T);
  double C[KK], rop[IZEM_MAXREAC];
  double ctot = 0.0;
#pragma unroll
  for (int k = 0; k < KK; ++k) {
    C[k] = rho * Y[k] / c_mech.wt[k];
    ctot = ctot + C[k];
    wdot[k] = 0.0;
  }
  double smh[KK];
  if (c_need_eqk) {
    const double T2 = T * T, T3 = T * T2, T4 = T2 * T2;
#pragma unroll
    for (int k = 0; k < KK; ++k) {
      const double* a = c_mech.a[k][T > c_mech.tmid[k] ? 1 : 0];
      const double s = (alogt - 1.0) * a[0] + (T / 2) * a[1] + (T2 / 6) * a[2] + (T3 / 12) * a[3] + (T4 / 20) * a[4];
      smh[k] = s + a[6] - a[5] / T;
    }
  }
  for (int i = 0; i < ii; ++i) {
    double rkft = c_mech.par[i][0] * exp(c_mech.par[i][1] * alogt - c_mech.par[i][2] / T);
    double rkrt = 0.0;
    const int rv = c_mech.rev[i];
    if (rv == 1) {
      double sumsmh = 0.0;
      int nus = 0;
      for (int n = 0; n < MXSP; ++n) {
        const int kk = c_mech.nuk[i][n];
        if (kk >= 0) sumsmh = sumsmh + double(c_mech.nu[i][n]) * smh[kk];
        nus += c_mech.nu[i][n];
      }
      double eqk = sumsmh != 0.0 ? exp(fmin(sumsmh, 690.77552789821368)) : 1.0;
      eqk = eqk * powi(c_mech.patm / (c_mech.ru * T), nus);
      rkrt = rkft / fmax(eqk, 1.0e-300);
    } else if (rv == 2) {
      rkrt = c_mech.rpar[i][0] * exp(c_mech.rpar[i][1] * alogt - c_mech.rpar[i][2] / T);
    }
    double ctb = 1.0;
    if (c_mech.thb[i]) {
      ctb = ctot;
      for (int k = 0; k < KK; ++k)
        if (c_mech.eff[i][k] != 1.0) ctb = ctb + (c_mech.eff[i][k] - 1.0) * C[k];
    }
    const int fo = c_mech.fall[i];
    if (fo) {
      const double rklow = c_mech.low[i][0] * exp(c_mech.low[i][1] * alogt - c_mech.low[i][2] / T);
      const double pr = rklow * ctb / rkft;
      ctb = 1.0;
      double pcor = pr / (1.0 + pr);
      if (fo > 1) {
        const double prlog = log10(fmax(pr, 1.0e-300));
        const double ta = c_mech.troe[i][0];
        double fcent = (1.0 - ta) * exp(-T / c_mech.troe[i][1]) + ta * exp(-T / c_mech.troe[i][2]);
        if (fo == 4) fcent = fcent + exp(-c_mech.troe[i][3] / T);
        const double fclog = log10(fmax(fcent, 1.0e-300));
        const double xn = 0.75 - 1.27 * fclog;
        const double cprlog = prlog - (0.4 + 0.67 * fclog);
        const double q = cprlog / (xn - 0.14 * cprlog);
        const double flog = fclog / (1.0 + q * q);
        pcor = pow(10.0, flog) * pcor;
      }
      rkft = rkft * pcor;
      rkrt = rkrt * pcor;
    }
    rkft = rkft * ctb;
    rkrt = rkrt * ctb;
    double rkf = 0.0, rkr = 0.0;
    if (c_mech.nu[i][0] != 0) {
      rkf = rkft * powi(C[c_mech.nuk[i][0]], -c_mech.nu[i][0]);
      rkr = rkrt * powi(C[c_mech.nuk[i][3]], c_mech.nu[i][3]);
      if (c_mech.nuk[i][1] >= 0) {
        rkf = rkf * powi(C[c_mech.nuk[i][1]], -c_mech.nu[i][1]);
        if (c_mech.nuk[i][2] >= 0) rkf = rkf * powi(C[c_mech.nuk[i][2]], -c_mech.nu[i][2]);
      }
      if (c_mech.nuk[i][4] >= 0) {
        rkr = rkr * powi(C[c_mech.nuk[i][4]], c_mech.nu[i][4]);
        if (c_mech.nuk[i][5] >= 0) rkr = rkr * powi(C[c_mech.nuk[i][5]], c_mech.nu[i][5]);
      }
    }
    rop[i] = rkf - rkr;
  }
  // CKWYR accumulation order: stoichiometric slot outer, reaction inner
  for (int n = 0; n < MXSP; ++n)
    for (int i = 0; i < ii; ++i) {
      const int k = c_mech.nuk[i][n];
      if (k >= 0) wdot[k] = wdot[k] + rop[i] * double(c_mech.nu[i][n]);
    }
}

// FUN: z = [T, Y], dz/dt for the constant-volume reactor
template <int KK>
HD void ck_fun(double rho, const double* z, double* zp) {
  double wdot[KK], h[KK], cvb;
  Thermo<KK>::cv_h(z[0], z + 1, &cvb, h);
  ck_wyr<KK>(rho, z[0], z + 1, wdot);
  const double rho_i = 1.0 / rho;
  double sum = 0.0;
#pragma unroll
  for (int k = 0; k < KK; ++k) {
    zp[k + 1] = wdot[k] * c_mech.wt[k] * rho_i;
    sum = sum + h[k] * wdot[k] * c_mech.wt[k] + (-c_mech.ru * z[0]) * wdot[k];
  }
  zp[0] = -sum / (rho * cvb);
}

// ------------------------------------------------------------- DVODE -------
template <int N>
struct Dv {
  double rho;
  double acnrm, conp, crate, drc, el[7], eta, etamax, h, hnew, hscal, prl1, rc, rl1, tau[7], tq[5], tn, hu;
  int icf, ipup, jcur, jstart, kflag, l, lmax, newh, newq, nq, nqnyh, nqwait, nslj, nslp, nst;
  double etaq, etaqm1;
  double yh[6 * N];
  double ewt[N], savf[N], acor[N];
  double wm[N * N], wmjs[N * N];
  int ipvt[N];
};

constexpr double kUround = 2.220446049250313e-16;   // D1MACH(4) for IEEE double
constexpr double kRtol = 1.0e-6, kAtol = 1.0e-10;

template <int N>
HD __forceinline__ double dvnorm(const double* v, const double* w) {
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < N; ++i) { const double x = v[i] * w[i]; s = s + x * x; }
  return sqrt(s / double(N));
}

template <int N>
HD int dgefa(double* a, int* ipvt) {
  int info = 0;
  for (int k = 0; k < N - 1; ++k) {
    int l = k;
    double dmax = fabs(a[k + k * N]);
    for (int i = k + 1; i < N; ++i) {
      const double v = fabs(a[i + k * N]);
      if (v > dmax) { dmax = v; l = i; }
    }
    ipvt[k] = l;
    if (a[l + k * N] == 0.0) { info = k + 1; continue; }
    if (l != k) { const double t = a[l + k * N]; a[l + k * N] = a[k + k * N]; a[k + k * N] = t; }
    const double t = -1.0 / a[k + k * N];
    for (int i = k + 1; i < N; ++i) a[i + k * N] = t * a[i + k * N];
    for (int j = k + 1; j < N; ++j) {
      double tj = a[l + j * N];
      if (l != k) { a[l + j * N] = a[k + j * N]; a[k + j * N] = tj; }
      if (tj != 0.0)
        for (int i = k + 1; i < N; ++i) a[i + j * N] = a[i + j * N] + tj * a[i + k * N];
    }
  }
  ipvt[N - 1] = N - 1;
  if (a[(N - 1) + (N - 1) * N] == 0.0) info = N;
  return info;
}

template <int N>
HD void dgesl(const double* a, const int* ipvt, double* b) {
  for (int k = 0; k < N - 1; ++k) {
    const int l = ipvt[k];
    const double t = b[l];
    if (l != k) { b[l] = b[k]; b[k] = t; }
    if (t != 0.0)
      for (int i = k + 1; i < N; ++i) b[i] = b[i] + t * a[i + k * N];
  }
  for (int k = N - 1; k >= 0; --k) {
    b[k] = b[k] / a[k + k * N];
    const double t = -b[k];
    if (t != 0.0)
      for (int i = 0; i < k; ++i) b[i] = b[i] + t * a[i + k * N];
  }
}

template <int N>
HD void dvset(Dv<N>& d) {
  const int nq = d.nq, L = d.l;
  double* el = d.el;
  for (int i = 2; i < L; ++i) el[i] = 0.0;
  el[0] = 1.0;
  el[1] = 1.0;
  double alph0 = -1.0, ahatn0 = -1.0, hsum = d.h, rxi = 1.0, rxis = 1.0;
  if (nq != 1) {
    for (int j = 1; j <= nq - 2; ++j) {
      hsum = hsum + d.tau[j - 1];
      rxi = d.h / hsum;
      alph0 = alph0 - 1.0 / double(j + 1);
      for (int iback = 1; iback <= j + 1; ++iback) {
        const int i = (j + 3) - iback;
        el[i - 1] = el[i - 1] + el[i - 2] * rxi;
      }
    }
    alph0 = alph0 - 1.0 / double(nq);
    rxis = -el[1] - alph0;
    hsum = hsum + d.tau[nq - 2];
    rxi = d.h / hsum;
    ahatn0 = -el[1] - rxi;
    for (int iback = 1; iback <= nq; ++iback) {
      const int i = (nq + 2) - iback;
      el[i - 1] = el[i - 1] + el[i - 2] * rxis;
    }
  }
  const double t1 = 1.0 - ahatn0 + alph0;
  const double t2 = 1.0 + double(nq) * t1;
  d.tq[1] = fabs(alph0 * t2 / t1);
  d.tq[4] = fabs(t2 / (el[L - 1] * rxi / rxis));
  if (d.nqwait == 1) {
    const double cnqm1 = rxis / el[L - 1];
    const double t3 = alph0 + 1.0 / double(nq);
    const double t4 = ahatn0 + rxi;
    double elp = t3 / (1.0 - t4 + t3);
    d.tq[0] = fabs(elp / cnqm1);
    hsum = hsum + d.tau[nq - 1];
    rxi = d.h / hsum;
    const double t5 = alph0 - 1.0 / double(nq + 1);
    const double t6 = ahatn0 - rxi;
    elp = t2 / (1.0 - t6 + t5);
    d.tq[2] = fabs(elp * rxi * (double(L) + 1.0) * t5);
  }
  d.tq[3] = 0.1 * d.tq[1];
}

template <int N>
HD void dvjust(Dv<N>& d, int iord) {
  const int nq = d.nq;
  if (nq == 2 && iord != 1) return;
  double* el = d.el;
  for (int j = 0; j < d.lmax; ++j) el[j] = 0.0;
  el[2] = 1.0;
  if (iord != 1) {
    double hsum = 0.0;
    for (int j = 1; j <= nq - 2; ++j) {
      hsum = hsum + d.tau[j - 1];
      const double xi = hsum / d.hscal;
      for (int iback = 1; iback <= j + 1; ++iback) {
        const int i = (j + 4) - iback;
        el[i - 1] = el[i - 1] * xi + el[i - 2];
      }
    }
    for (int j = 3; j <= nq; ++j)
      for (int i = 0; i < N; ++i) d.yh[i + (j - 1) * N] = d.yh[i + (j - 1) * N] - d.yh[i + (d.l - 1) * N] * el[j - 1];
    return;
  }
  double alph0 = -1.0, alph1 = 1.0, prod = 1.0, xiold = 1.0, hsum = d.hscal;
  for (int j = 1; j <= nq - 1; ++j) {
    hsum = hsum + d.tau[j];
    const double xi = hsum / d.hscal;
    prod = prod * xi;
    alph0 = alph0 - 1.0 / double(j + 1);
    alph1 = alph1 + 1.0 / xi;
    for (int iback = 1; iback <= j + 1; ++iback) {
      const int i = (j + 4) - iback;
      el[i - 1] = el[i - 1] * xiold + el[i - 2];
    }
    xiold = xi;
  }
  const double t1 = (-alph0 - alph1) / prod;
  const int lp1 = d.l + 1;
  for (int i = 0; i < N; ++i) d.yh[i + (lp1 - 1) * N] = t1 * d.yh[i + (d.lmax - 1) * N];
  for (int j = 3; j <= nq + 1; ++j) {
    const double a = el[j - 1];
    if (a != 0.0)
      for (int i = 0; i < N; ++i) d.yh[i + (j - 1) * N] = d.yh[i + (j - 1) * N] + a * d.yh[i + (lp1 - 1) * N];
  }
}

template <int N>
HD int dvjac(Dv<N>& d, double* y, double* ftem) {
  int jok = 1;
  if (d.nst == 0 || d.nst > d.nslj + 50) jok = -1;
  if (d.icf == 1 && d.drc < 0.2) jok = -1;
  if (d.icf == 2) jok = -1;
  if (jok == -1) {
    d.nslj = d.nst;
    d.jcur = 1;
    double fac = dvnorm<N>(d.savf, d.ewt);
    double r0 = 1000.0 * fabs(d.h) * kUround * double(N) * fac;
    if (r0 == 0.0) r0 = 1.0;
    const double srur = 1.4901161193847656e-08;   // sqrt(UROUND)
    for (int j = 0; j < N; ++j) {
      const double yj = y[j];
      const double r = fmax(srur * fabs(yj), r0 / d.ewt[j]);
      y[j] = y[j] + r;
      fac = 1.0 / r;
      ck_fun<N - 1>(d.rho, y, ftem);
      for (int i = 0; i < N; ++i) d.wmjs[i + j * N] = (ftem[i] - d.savf[i]) * fac;
      y[j] = yj;
    }
  } else {
    d.jcur = 0;
  }
  const double con = -(d.h * d.rl1);
  for (int q = 0; q < N * N; ++q) d.wm[q] = con * d.wmjs[q];
  for (int i = 0; i < N; ++i) d.wm[i + i * N] = d.wm[i + i * N] + 1.0;
  return dgefa<N>(d.wm, d.ipvt) != 0 ? 1 : 0;
}

template <int N>
HD int dvnlsd(Dv<N>& d, double* y, double* ftem, int nflag) {
  if (d.jstart == 0) d.nslp = 0;
  if (nflag == 0) d.icf = 0;
  if (nflag == -2) d.ipup = 2;
  if (d.jstart == 0) d.ipup = 2;
  d.drc = fabs(d.rc - 1.0);
  if (d.drc > 0.3 || d.nst >= d.nslp + 20) d.ipup = 2;
  for (int pass = 0; pass < 2; ++pass) {
    int m = 0;
    double delp = 0.0;
    for (int i = 0; i < N; ++i) y[i] = d.yh[i];
    ck_fun<N - 1>(d.rho, y, d.savf);
    if (d.ipup > 0) {
      const int ierpj = dvjac<N>(d, y, ftem);
      d.ipup = 0;
      d.rc = 1.0;
      d.drc = 0.0;
      d.crate = 1.0;
      d.nslp = d.nst;
      if (ierpj != 0) { d.icf = 2; d.ipup = 2; return -1; }
    }
    for (int i = 0; i < N; ++i) d.acor[i] = 0.0;
    for (int it = 0; it < 3; ++it) {
      for (int i = 0; i < N; ++i) y[i] = (d.rl1 * d.h) * d.savf[i] - (d.rl1 * d.yh[i + N] + d.acor[i]);
      dgesl<N>(d.wm, d.ipvt, y);
      if (d.rc != 1.0) {
        const double cscale = 2.0 / (1.0 + d.rc);
        for (int i = 0; i < N; ++i) y[i] = cscale * y[i];
      }
      const double del = dvnorm<N>(y, d.ewt);
      for (int i = 0; i < N; ++i) d.acor[i] = d.acor[i] + y[i];
      for (int i = 0; i < N; ++i) y[i] = d.yh[i] + d.acor[i];
      if (m != 0) d.crate = fmax(0.3 * d.crate, del / delp);
      const double dcon = del * fmin(1.0, d.crate) / d.tq[3];
      if (dcon <= 1.0) {
        d.jcur = 0;
        d.icf = 0;
        d.acnrm = (m == 0) ? del : dvnorm<N>(d.acor, d.ewt);
        return 0;
      }
      m = m + 1;
      if (m == 3 || (m >= 2 && del > 2.0 * delp)) break;
      delp = del;
      ck_fun<N - 1>(d.rho, y, d.savf);
    }
    if (d.jcur == 1) break;
    d.icf = 1;
    d.ipup = 2;
  }
  d.icf = 2;
  d.ipup = 2;
  return -1;
}

// one DVSTEP; returns KFLAG (0, -1 error test, -2 convergence)
template <int N>
HD int dvstep(Dv<N>& d, double* y, double* ftem) {
  d.kflag = 0;
  const double told = d.tn;
  int ncf = 0, nflag = 0;
  d.jcur = 0;
  bool rescale;
  if (d.jstart > 0) {
    rescale = false;
    if (d.newh != 0) {
      if (d.newq < d.nq) { dvjust<N>(d, -1); d.nq = d.newq; d.l = d.nq + 1; d.nqwait = d.l; }
      else if (d.newq > d.nq) { dvjust<N>(d, 1); d.nq = d.newq; d.l = d.nq + 1; d.nqwait = d.l; }
      rescale = true;
    }
  } else {
    d.lmax = 6;
    d.nq = 1;
    d.l = 2;
    d.nqnyh = N;
    d.tau[0] = d.h;
    d.prl1 = 1.0;
    d.rc = 0.0;
    d.etamax = 1.0e4;
    d.nqwait = 2;
    d.hscal = d.h;
    rescale = false;
  }
  for (int guard = 0; guard < 64; ++guard) {
    if (rescale) {
      double r = 1.0;
      for (int j = 2; j <= d.l; ++j) {
        r = r * d.eta;
        for (int i = 0; i < N; ++i) d.yh[i + (j - 1) * N] = r * d.yh[i + (j - 1) * N];
      }
      d.h = d.hscal * d.eta;
      d.hscal = d.h;
      d.rc = d.rc * d.eta;
      d.nqnyh = d.nq * N;
    }
    rescale = true;
    d.tn = d.tn + d.h;
    for (int jb = 1; jb <= d.nq; ++jb)
      for (int i = d.nqnyh - jb * N; i < d.nqnyh; ++i) d.yh[i] = d.yh[i] + d.yh[i + N];
    dvset<N>(d);
    d.rl1 = 1.0 / d.el[1];
    d.rc = d.rc * (d.rl1 / d.prl1);
    d.prl1 = d.rl1;
    nflag = dvnlsd<N>(d, y, ftem, nflag);
    if (nflag != 0) {
      ncf = ncf + 1;
      d.etamax = 1.0;
      d.tn = told;
      for (int jb = 1; jb <= d.nq; ++jb)
        for (int i = d.nqnyh - jb * N; i < d.nqnyh; ++i) d.yh[i] = d.yh[i] - d.yh[i + N];
      if (ncf == 10) { d.kflag = -2; d.jstart = 1; return d.kflag; }
      d.eta = 0.25;
      nflag = -1;
      continue;
    }
    const double dsm = d.acnrm / d.tq[1];
    if (dsm <= 1.0) {
      d.kflag = 0;
      d.nst = d.nst + 1;
      d.hu = d.h;
      for (int iback = 1; iback <= d.nq; ++iback) {
        const int i = d.l - iback;
        d.tau[i] = d.tau[i - 1];
      }
      d.tau[0] = d.h;
      for (int j = 1; j <= d.l; ++j) {
        const double a = d.el[j - 1];
        if (a != 0.0)
          for (int i = 0; i < N; ++i) d.yh[i + (j - 1) * N] = d.yh[i + (j - 1) * N] + a * d.acor[i];
      }
      d.nqwait = d.nqwait - 1;
      if (!(d.l == d.lmax || d.nqwait != 1)) {
        for (int i = 0; i < N; ++i) d.yh[i + (d.lmax - 1) * N] = d.acor[i];
        d.conp = d.tq[4];
      }
      if (d.etamax != 1.0) {
        const double flotl = double(d.l);
        d.etaq = 1.0 / (pow(6.0 * dsm, 1.0 / flotl) + 1.0e-6);
        if (d.nqwait != 0) {
          d.eta = d.etaq;
          d.newq = d.nq;
        } else {
          d.nqwait = 2;
          d.etaqm1 = 0.0;
          if (d.nq != 1) {
            double col[N];
            for (int i = 0; i < N; ++i) col[i] = d.yh[i + (d.l - 1) * N];
            const double ddn = dvnorm<N>(col, d.ewt) / d.tq[0];
            d.etaqm1 = 1.0 / (pow(6.0 * ddn, 1.0 / (flotl - 1.0)) + 1.0e-6);
          }
          double etaqp1 = 0.0;
          if (d.l != d.lmax) {
            const double cnquot = (d.tq[4] / d.conp) * powi(d.h / d.tau[1], d.l);
            for (int i = 0; i < N; ++i) d.savf[i] = d.acor[i] - cnquot * d.yh[i + (d.lmax - 1) * N];
            const double dup = dvnorm<N>(d.savf, d.ewt) / d.tq[2];
            etaqp1 = 1.0 / (pow(10.0 * dup, 1.0 / (flotl + 1.0)) + 1.0e-6);
          }
          if (d.etaq >= etaqp1) {
            if (d.etaq < d.etaqm1) { d.eta = d.etaqm1; d.newq = d.nq - 1; }
            else { d.eta = d.etaq; d.newq = d.nq; }
          } else if (etaqp1 > d.etaqm1) {
            d.eta = etaqp1;
            d.newq = d.nq + 1;
            for (int i = 0; i < N; ++i) d.yh[i + (d.lmax - 1) * N] = d.acor[i];
          } else { d.eta = d.etaqm1; d.newq = d.nq - 1; }
        }
        if (d.eta < 1.5 || d.etamax == 1.0) { d.newq = d.nq; d.newh = 0; d.eta = 1.0; d.hnew = d.h; }
        else { d.eta = fmin(d.eta, d.etamax); d.newh = 1; d.hnew = d.h * d.eta; }
      } else {
        if (d.nqwait < 2) d.nqwait = 2;
        d.newq = d.nq; d.newh = 0; d.eta = 1.0; d.hnew = d.h;
      }
      d.etamax = 10.0;   // ETAMX2 = ETAMX3 = 10
      const double r = 1.0 / d.tq[1];
      for (int i = 0; i < N; ++i) d.acor[i] = r * d.acor[i];
      d.jstart = 1;
      return 0;
    }
    // error test failed
    d.kflag = d.kflag - 1;
    nflag = -2;
    d.tn = told;
    for (int jb = 1; jb <= d.nq; ++jb)
      for (int i = d.nqnyh - jb * N; i < d.nqnyh; ++i) d.yh[i] = d.yh[i] - d.yh[i + N];
    d.etamax = 1.0;
    if (d.kflag > -3) {
      d.eta = 1.0 / (pow(6.0 * dsm, 1.0 / double(d.l)) + 1.0e-6);
      d.eta = fmax(d.eta, 0.1);
      if (d.kflag <= -2 && d.eta > 0.2) d.eta = 0.2;
      continue;
    }
    if (d.kflag == -7) { d.kflag = -1; d.jstart = 1; return d.kflag; }
    if (d.nq != 1) {
      d.eta = 0.1;
      dvjust<N>(d, -1);
      d.l = d.nq;
      d.nq = d.nq - 1;
      d.nqwait = d.l;
      continue;
    }
    d.eta = 0.1;
    d.h = d.h * d.eta;
    d.hscal = d.h;
    d.tau[0] = d.h;
    ck_fun<N - 1>(d.rho, y, d.savf);
    for (int i = 0; i < N; ++i) d.yh[i + N] = d.h * d.savf[i];
    d.nqwait = 10;
    rescale = false;
  }
  d.kflag = -2;
  d.jstart = 1;
  return d.kflag;
}

// DVODE (ISTATE = 1 fresh start, ITASK = 1): returns ISTATE
template <int N>
HD int dvode(Dv<N>& d, double* y, double* t, double tout, int* nst_total) {
  double ftem[N];
  if (tout == *t) return 1;
  d.tn = *t;
  d.jstart = 0;
  d.nslj = 0;
  d.nst = 0;
  d.hu = 0.0;
  d.icf = 0;
  d.ipup = 0;
  d.jcur = 0;
  d.newh = 0;
  d.newq = 1;
  d.conp = 0.0;
  d.crate = 0.0;
  d.drc = 0.0;
  d.acnrm = 0.0;
  d.nslp = 0;
  ck_fun<N - 1>(d.rho, y, d.yh + N);
  for (int i = 0; i < N; ++i) d.yh[i] = y[i];
  d.nq = 1;
  d.h = 1.0;
  for (int i = 0; i < N; ++i) d.ewt[i] = 1.0 / (kRtol * fabs(d.yh[i]) + kAtol);
  // DVHIN
  double h0;
  {
    const double tdist = fabs(tout - *t);
    const double tround = kUround * fmax(fabs(*t), fabs(tout));
    if (tdist < 2.0 * tround) return -3;
    const double hlb = 100.0 * tround;
    double hub = 0.1 * tdist;
    for (int i = 0; i < N; ++i) {
      const double delyi = 0.1 * fabs(d.yh[i]) + kAtol;
      const double afi = fabs(d.yh[i + N]);
      if (afi * hub > delyi) hub = delyi / afi;
    }
    double hg = sqrt(hlb * hub), hnew = hg;
    if (hub < hlb) {
      h0 = hg;
    } else {
      int iter = 0;
      while (true) {
        for (int i = 0; i < N; ++i) y[i] = d.yh[i] + hg * d.yh[i + N];
        ck_fun<N - 1>(d.rho, y, ftem);
        for (int i = 0; i < N; ++i) ftem[i] = (ftem[i] - d.yh[i + N]) / hg;
        const double yddnrm = dvnorm<N>(ftem, d.ewt);
        hnew = (yddnrm * hub * hub > 2.0) ? sqrt(2.0 / yddnrm) : sqrt(hg * hub);
        iter = iter + 1;
        if (iter >= 4) break;
        const double hrat = hnew / hg;
        if (hrat > 0.5 && hrat < 2.0) break;
        if (iter >= 2 && hnew > 2.0 * hg) { hnew = hg; break; }
        hg = hnew;
      }
      h0 = hnew * 0.5;
      if (h0 < hlb) h0 = hlb;
      if (h0 > hub) h0 = hub;
    }
    h0 = copysign(h0, tout - *t);
  }
  d.h = h0;
  for (int i = 0; i < N; ++i) d.yh[i + N] = h0 * d.yh[i + N];
  bool first = true;
  for (int guard = 0; guard < 600; ++guard) {
    if (!first) {
      if (d.nst >= 500) {
        for (int i = 0; i < N; ++i) y[i] = d.yh[i];
        *t = d.tn;
        *nst_total += d.nst;
        return -1;
      }
      for (int i = 0; i < N; ++i) d.ewt[i] = 1.0 / (kRtol * fabs(d.yh[i]) + kAtol);
    }
    first = false;
    if (kUround * dvnorm<N>(d.yh, d.ewt) > 1.0) {
      for (int i = 0; i < N; ++i) y[i] = d.yh[i];
      *t = d.tn;
      *nst_total += d.nst;
      return -2;
    }
    const int kflag = dvstep<N>(d, y, ftem);
    if (kflag != 0) {
      for (int i = 0; i < N; ++i) y[i] = d.yh[i];
      *t = d.tn;
      *nst_total += d.nst;
      return kflag == -1 ? -4 : -5;
    }
    if ((d.tn - tout) * d.h < 0.0) continue;
    // DVINDY (K = 0)
    const double s = (tout - d.tn) / d.h;
    for (int i = 0; i < N; ++i) y[i] = d.yh[i + (d.l - 1) * N];
    for (int jb = 1; jb <= d.nq; ++jb) {
      const int j = d.nq - jb;
      for (int i = 0; i < N; ++i) y[i] = d.yh[i + j * N] + s * y[i];
    }
    *t = tout;
    *nst_total += d.nst;
    return 2;
  }
  *nst_total += d.nst;
  return -1;
}

// REACTION_V: up to 20 fresh DVODE starts
template <int N>
HD int reaction_v(double rho, double* z, double tf, int* nsteps) {
  Dv<N> d;
  d.rho = rho;
  double ti = 0.0;
  int istate = 1;
  *nsteps = 0;
  for (int ib = 0; ib < 20 && istate != 2; ++ib) istate = dvode<N>(d, z, &ti, tf, nsteps);
  return istate;
}

// ---------------------------------------------------------------- kernels ---
template <int KK>
__global__ void __launch_bounds__(128) k_psr_field(ChemField f, unsigned* counter, ChemStats* stats) {
  constexpr int N = KK + 1;
  const long long ncell = (long long)f.wx * f.wy * f.wz;
  while (true) {
    const long long q = atomicAdd(counter, 1u);
    if (q >= ncell) break;
    const int i = f.ix + (int)(q % f.wx);
    const long long r = q / f.wx;
    const int j = f.iy + (int)(r % f.wy);
    const int k = f.iz + (int)(r / f.wy);
    const long long p = (long long)(i - 1 + f.ng) + (long long)f.gx * ((long long)(j - 1 + f.ng) + (long long)f.gy * (long long)(k - 1 + f.ng));
    const long long nc = f.ncell;
    const double rho0 = f.v[p];
    const double rho_i = 1.0 / rho0;
    double z[N];
#pragma unroll
    for (int l = 0; l < KK; ++l) z[1 + l] = f.v[(5 + l) * nc + p] * rho_i;
    const double T0 = f.T[p] * f.t_ref;
    z[0] = T0;
    int nst = 0;
    const int istate = reaction_v<N>(rho0 * f.rho_cgs, z, f.dt_phys, &nst);
    if (istate <= -2) atomicAdd(&stats->failed, 1);
    atomicMax(&stats->max_steps, nst);
    atomicAdd(&stats->total_steps, (unsigned long long)nst);
    f.T[p] = z[0] * f.tref_i;
    const double dT = fabs(z[0] - T0);
    atomicMax(&stats->dtmax_bits, (unsigned long long)__double_as_longlong(dT));
    double sumY = 0.0;
#pragma unroll
    for (int l = 0; l < KK - 1; ++l) {
      const double Ya = fmin(fmax(z[1 + l], 0.0), 1.0);
      f.v[(5 + l) * nc + p] = rho0 * Ya;
      sumY = sumY + Ya;
    }
    f.v[(5 + KK - 1) * nc + p] = rho0 * (1.0 - sumY);
    if (f.dT_out) f.dT_out[q] = z[0] - T0;
  }
}

template <int KK>
__global__ void __launch_bounds__(128) k_psr_batch(int n, double* T, const double* rho, double* Y, const double* dt,
                                                   int* istate, int* nsteps, unsigned* counter, ChemStats* stats) {
  constexpr int N = KK + 1;
  while (true) {
    const unsigned q = atomicAdd(counter, 1u);
    if (q >= (unsigned)n) break;
    double z[N];
    z[0] = T[q];
#pragma unroll
    for (int l = 0; l < KK; ++l) z[1 + l] = Y[(size_t)q * KK + l];
    int nst = 0;
    const int is = reaction_v<N>(rho[q], z, dt[q], &nst);
    if (is <= -2) atomicAdd(&stats->failed, 1);
    atomicMax(&stats->max_steps, nst);
    atomicAdd(&stats->total_steps, (unsigned long long)nst);
    T[q] = z[0];
#pragma unroll
    for (int l = 0; l < KK; ++l) Y[(size_t)q * KK + l] = z[1 + l];
    if (istate) istate[q] = is;
    if (nsteps) nsteps[q] = nst;
  }
}

// ------------------------------------------------ surrogate support --------
// Inputs of the learned surrogate: T [K], ln p [atm], ln(Y_k + 1e-10),
// ln dt [s], normalised by the training means / standard deviations.
template <int KK>
__global__ void k_featurize(int n, const double* T, const double* rho, const double* Y, const double* dt,
                            const float* norm, __nv_bfloat16* x, int ldx) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  double f[KK + 3];
  const double Tq = T[q];
  double wmi = 0.0;
#pragma unroll
  for (int k = 0; k < KK; ++k) wmi += fmax(Y[(size_t)q * KK + k], 0.0) / c_mech.wt[k];
  const double p_atm = rho[q] * c_mech.ru * Tq * wmi / c_mech.patm;
  f[0] = Tq;
  f[1] = log(p_atm);
#pragma unroll
  for (int k = 0; k < KK; ++k) f[2 + k] = log(fmax(Y[(size_t)q * KK + k], 0.0) + 1.0e-10);
  f[KK + 2] = log(dt[q]);
#pragma unroll
  for (int c = 0; c < KK + 3; ++c) x[(size_t)q * ldx + c] = __float2bfloat16((float)((f[c] - norm[c]) / norm[KK + 3 + c]));
  for (int c = KK + 3; c < ldx; ++c) x[(size_t)q * ldx + c] = __float2bfloat16(0.f);
}

struct GateArgs {
  double tmin, tmax, dtmin, dtmax;   // training envelope
  double tol_el;                     // relative element residual
  double tol_T_abs, tol_T_rel;       // energy-consistency of dT [K]
  double tol_ens_abs, tol_ens_rel;   // agreement of two independently trained networks on dT [K]
};

// Decode the surrogate output, gate it, and write accepted cells in place.
// Gate: (1) state inside the training envelope; (2) element conservation of
// the predicted dY (H, O, N, from the species composition); (3) the
// predicted dT agrees with the temperature that conserves internal energy
// (constant-volume reactor) for the predicted composition.  Accepted cells
// take the energy-consistent temperature.  Rejected cells are appended to
// `list` for the BDF integrator.
template <int KK>
__global__ void k_decode_gate(int n, const float* out, const float* out2, int ldo, const float* norm, const float* norm2,
                              double* T, const double* rho, double* Y, const double* dt, GateArgs ga, const int* kncf,
                              int nele, int* list, unsigned* count, double* dT_pred, ChemStats* stats) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int NI = KK + 3, NO = KK + 1;
  const float* mo = norm + 2 * NI;
  const float* so = norm + 2 * NI + NO;
  double dY[KK], Yn[KK];
  const double T0 = T[q];
  bool ok = T0 >= ga.tmin && T0 <= ga.tmax && dt[q] >= ga.dtmin && dt[q] <= ga.dtmax;
#pragma unroll
  for (int k = 0; k < KK; ++k) dY[k] = (double)out[(size_t)q * ldo + k] * so[k] + mo[k];
  const double dTp = (double)out[(size_t)q * ldo + KK] * so[KK] + mo[KK];
  if (dT_pred) dT_pred[q] = dTp;
  if (out2) {
    const double dT2 = (double)out2[(size_t)q * ldo + KK] * norm2[2 * NI + NO + KK] + norm2[2 * NI + KK];
    if (fabs(dT2 - dTp) > ga.tol_ens_abs + ga.tol_ens_rel * fabs(dTp)) ok = false;
  }
  // element residuals
  for (int e = 0; e < nele && ok; ++e) {
    double r = 0.0, sc = 0.0;
    for (int k = 0; k < KK; ++k) {
      const double nk = (double)kncf[k * nele + e] / c_mech.wt[k];
      r += nk * dY[k];
      sc += nk * fmax(Y[(size_t)q * KK + k], 0.0);
    }
    if (sc > 0.0 && fabs(r) > ga.tol_el * sc) ok = false;
  }
  double sum = 0.0;
#pragma unroll
  for (int k = 0; k < KK; ++k) { Yn[k] = fmax(Y[(size_t)q * KK + k] + dY[k], 0.0); sum += Yn[k]; }
#pragma unroll
  for (int k = 0; k < KK; ++k) Yn[k] = Yn[k] / sum;
  // internal energy balance: sum Y0 u(T0) = sum Yn u(T1), Newton on T1
  double e0 = 0.0;
  {
    double h[KK], cvb;
    Thermo<KK>::cv_h(T0, Y + (size_t)q * KK, &cvb, h);
#pragma unroll
    for (int k = 0; k < KK; ++k) e0 += Y[(size_t)q * KK + k] * (h[k] - c_mech.ru * T0 / c_mech.wt[k]);
  }
  double T1 = T0 + dTp;
  if (!(T1 > 200.0 && T1 < 6000.0)) ok = false;
  for (int it = 0; it < 4 && ok; ++it) {
    double h[KK], cvb, e1 = 0.0;
    Thermo<KK>::cv_h(T1, Yn, &cvb, h);
#pragma unroll
    for (int k = 0; k < KK; ++k) e1 += Yn[k] * (h[k] - c_mech.ru * T1 / c_mech.wt[k]);
    T1 = T1 - (e1 - e0) / cvb;
  }
  const double dTe = T1 - T0;
  if (ok && fabs(dTp - dTe) > ga.tol_T_abs + ga.tol_T_rel * fabs(dTe)) ok = false;
  if (ok) {
    T[q] = T1;
#pragma unroll
    for (int k = 0; k < KK; ++k) Y[(size_t)q * KK + k] = Yn[k];
  } else {
    const unsigned slot = atomicAdd(count, 1u);
    list[slot] = q;
  }
}

template <int KK>
__global__ void __launch_bounds__(128) k_psr_list(const int* list, const unsigned* count, double* T, const double* rho,
                                                  double* Y, const double* dt, unsigned* counter, ChemStats* stats) {
  constexpr int N = KK + 1;
  const unsigned n = *count;
  while (true) {
    const unsigned w = atomicAdd(counter, 1u);
    if (w >= n) break;
    const int q = list[w];
    double z[N];
    z[0] = T[q];
#pragma unroll
    for (int l = 0; l < KK; ++l) z[1 + l] = Y[(size_t)q * KK + l];
    int nst = 0;
    const int is = reaction_v<N>(rho[q], z, dt[q], &nst);
    if (is <= -2) atomicAdd(&stats->failed, 1);
    atomicMax(&stats->max_steps, nst);
    atomicAdd(&stats->total_steps, (unsigned long long)nst);
    T[q] = z[0];
#pragma unroll
    for (int l = 0; l < KK; ++l) Y[(size_t)q * KK + l] = z[1 + l];
  }
}

int chem_grid(int* blocks) {
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_psr_batch<9>, 128, 0) != cudaSuccess) return -1;
  *blocks = sms * (per > 0 ? per : 1);
  return 0;
}

}  // namespace

// ---------------------------------------------------------- host side -------
cudaError_t chem_upload_mech(const izem_mech* m) {
  cudaError_t e = cudaMemcpyToSymbol(c_mech_dev, m, sizeof(izem_mech));
  if (e != cudaSuccess) return e;
  int need = 0;
  for (int i = 0; i < m->ii; ++i) need |= (m->rev[i] == 1);
  return cudaMemcpyToSymbol(c_need_eqk_dev, &need, sizeof(int));
}

cudaError_t chem_launch_field(const ChemField& f, unsigned* d_counter, ChemStats* d_stats, cudaStream_t s, int kk) {
  int blocks = 0;
  if (chem_grid(&blocks)) return cudaErrorUnknown;
  cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  if (kk != 9) return cudaErrorInvalidValue;
  k_psr_field<9><<<blocks, 128, 0, s>>>(f, d_counter, d_stats);
  return cudaGetLastError();
}

cudaError_t chem_launch_batch(int n, double* T, const double* rho, double* Y, const double* dt, int* istate, int* nsteps,
                              unsigned* d_counter, ChemStats* d_stats, cudaStream_t s, int kk) {
  int blocks = 0;
  if (chem_grid(&blocks)) return cudaErrorUnknown;
  cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  if (kk != 9) return cudaErrorInvalidValue;
  k_psr_batch<9><<<blocks, 128, 0, s>>>(n, T, rho, Y, dt, istate, nsteps, d_counter, d_stats);
  return cudaGetLastError();
}

cudaError_t chem_launch_featurize(int n, const double* T, const double* rho, const double* Y, const double* dt,
                                  const float* d_norm, void* x_bf16, int ldx, cudaStream_t s) {
  k_featurize<9><<<(n + 127) / 128, 128, 0, s>>>(n, T, rho, Y, dt, d_norm, (__nv_bfloat16*)x_bf16, ldx);
  return cudaGetLastError();
}

cudaError_t chem_launch_decode_gate(int n, const float* out, const float* out2, int ldo, const float* d_norm,
                                    const float* d_norm2, double* T, const double* rho, double* Y, const double* dt,
                                    const double* gate9, const int* d_kncf, int nele, int* list, unsigned* count,
                                    double* dT_pred, ChemStats* stats, cudaStream_t s) {
  GateArgs ga{gate9[0], gate9[1], gate9[2], gate9[3], gate9[4], gate9[5], gate9[6], gate9[7], gate9[8]};
  k_decode_gate<9><<<(n + 127) / 128, 128, 0, s>>>(n, out, out2, ldo, d_norm, d_norm2, T, rho, Y, dt, ga, d_kncf, nele,
                                                   list, count, dT_pred, stats);
  return cudaGetLastError();
}

cudaError_t chem_launch_list(const int* list, const unsigned* count, double* T, const double* rho, double* Y,
                             const double* dt, unsigned* d_counter, ChemStats* d_stats, cudaStream_t s) {
  int blocks = 0;
  if (chem_grid(&blocks)) return cudaErrorUnknown;
  cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  k_psr_list<9><<<blocks, 128, 0, s>>>(list, count, T, rho, Y, dt, d_counter, d_stats);
  return cudaGetLastError();
}

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
// so cells with few BDF steps do not wait for cells with many.  The method
// is written as a resumable state machine (rc_advance) that stops at every
// right-hand-side evaluation, so the threads of a warp -- each on its own
// cell, at its own point of the method -- evaluate FUN together instead of
// one divergent branch at a time.  Every loop is bounded (MXSTEP = 500
// steps per DVODE call, 20 calls, at most 10 corrector failures and 7
// error-test failures per step): the kernel cannot spin.  Per-thread DVODE
// arrays (Nordsieck history, iteration matrix and its saved Jacobian) live
// in local memory.
#include <cstdio>
#include <cstring>
#include <cmath>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include "../../include/izem_gpu.h"
#include "chem.h"
#include "atomics.cuh"

// This source builds two translation units, compiled in parallel:
// IZEM_CHEM_UNIT 0 (chem.cu) holds the host side and the kernels that walk
// the uploaded mechanism's tables; 1 (chem_generated.cu) the kernels with
// the right-hand side generated for the shipped mechanism.
#ifndef IZEM_CHEM_UNIT
#define IZEM_CHEM_UNIT 0
#endif

// The persistent kernels of one register-budget variant and right-hand-side form.
struct ChemKernelSet {
  void (*field)(ChemField, unsigned*, ChemStats*);
  void (*batch)(int, double*, const double*, double*, const double*, int*, int*, unsigned*, ChemStats*);
  void (*list)(const int*, const unsigned*, double*, const double*, double*, const double*, unsigned*, ChemStats*);
};

namespace {

__constant__ izem_mech c_mech_dev;
__constant__ int c_need_eqk_dev;   // some reaction uses the equilibrium reverse rate

// Mechanism constants of the device right-hand side (ck_fun_fast).
struct ChemFast {
  double wt_inv[IZEM_NSMAX];          // 1 / W_k
  double ru_wt[IZEM_NSMAX];           // RU / W_k
  double troe_inv[IZEM_MAXREAC][2];   // 1 / T***, 1 / T*
  double sri_cinv[IZEM_MAXREAC];      // 1 / c of the SRI form
};
__constant__ ChemFast c_fast_dev;
#ifdef IZEM_CHEM_HOST_TEST
ChemFast c_fast_host;
#ifdef __CUDA_ARCH__
#define c_fast c_fast_dev
#else
#define c_fast c_fast_host
#endif
#else
#define c_fast c_fast_dev
#endif
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
// exponents of the Landau-Teller factor exp(B / T^(1/3) + C / T^(2/3))
// (CKRATT's PM_V_1 and PM_V_2, vode.f:975-976)
constexpr double kLtP1 = 1.0 / 3.0;
constexpr double kLtP2 = 2.0 * kLtP1;

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
    if (c_mech.lt[i][0] != 0.0 || c_mech.lt[i][1] != 0.0)   // Landau-Teller
      rkft = rkft * exp(c_mech.lt[i][0] / pow(T, kLtP1) + c_mech.lt[i][1] / pow(T, kLtP2));
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
    if (c_mech.rlt[i][0] != 0.0 || c_mech.rlt[i][1] != 0.0)   // reverse Landau-Teller
      rkrt = rkrt * exp(c_mech.rlt[i][0] / pow(T, kLtP1) + c_mech.rlt[i][1] / pow(T, kLtP2));
    double ctb = 1.0;
    if (c_mech.thb[i]) {
      ctb = ctot;
      for (int k = 0; k < KK; ++k)
        if (c_mech.eff[i][k] != 1.0) ctb = ctb + (c_mech.eff[i][k] - 1.0) * C[k];
    }
    const int fo = c_mech.fall[i];
    if (fo) {
      const double rklow = c_mech.low[i][0] * exp(c_mech.low[i][1] * alogt - c_mech.low[i][2] / T);
      const int kf = c_mech.kfal[i];   // collider: (+M), or species kf - 1 alone
      const double pr = rklow * (kf ? C[kf - 1] : ctb) / rkft;
      if (!kf) ctb = 1.0;
      double pcor = pr / (1.0 + pr);
      if (fo == 2) {
        const double prlog = log10(fmax(pr, 1.0e-300));
        const double xp = 1.0 / (1.0 + prlog * prlog);
        const double* sr = c_mech.sri[i];
        pcor = pow(sr[0] * exp(-sr[1] / T) + exp(-T / sr[2]), xp) * sr[3] * pow(T, sr[4]) * pcor;
      } else if (fo > 1) {
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


inline ChemFast chem_fast_constants(const izem_mech& m) {
  ChemFast f{};
  for (int k = 0; k < m.kk && k < IZEM_NSMAX; ++k) {
    f.wt_inv[k] = 1.0 / m.wt[k];
    f.ru_wt[k] = m.ru / m.wt[k];
  }
  for (int i = 0; i < m.ii && i < IZEM_MAXREAC; ++i) {
    f.troe_inv[i][0] = m.troe[i][1] != 0.0 ? 1.0 / m.troe[i][1] : 0.0;
    f.troe_inv[i][1] = m.troe[i][2] != 0.0 ? 1.0 / m.troe[i][2] : 0.0;
    f.sri_cinv[i] = m.fall[i] == 2 && m.sri[i][2] != 0.0 ? 1.0 / m.sri[i][2] : 0.0;
  }
  return f;
}

// The temperature-only terms of ck_fun_fast: species c_v and h, the forward
// and reverse rate constants, and the fall-off low-pressure rates and
// log10 F_cent.  The finite-difference Jacobian perturbs one variable per
// column, so its nine species columns share the temperature of the call
// before them and can reuse these terms (rc_drive).
template <int KK>
struct FunT {
  double T;                                    // temperature the entries belong to
  double rut;                                  // RU * T
  double cvk[KK], h[KK];
  double kf[IZEM_MAXREAC], kr[IZEM_MAXREAC];   // before third-body and fall-off factors
  double klow[IZEM_MAXREAC], fclog[IZEM_MAXREAC];
};

template <int KK>
HD void fun_tpart(double T, FunT<KK>& t) {
  const double Tinv = 1.0 / T;
  const double alogt = log(T);
  const double T2 = T * T, T3 = T * T2, T4 = T2 * T2;
  t.T = T;
  t.rut = T * c_mech.ru;
  double smh[KK];
#pragma unroll
  for (int k = 0; k < KK; ++k) {
    const double* a = c_mech.a[k][T > c_mech.tmid[k] ? 1 : 0];
    const double cps = a[0] + T * a[1] + T2 * a[2] + T3 * a[3] + T4 * a[4];
    t.cvk[k] = c_fast.ru_wt[k] * (cps - 1.0);
    const double hs = a[0] + (0.5 * T) * a[1] + (T2 * (1.0 / 3.0)) * a[2] + (0.25 * T3) * a[3] + (0.2 * T4) * a[4];
    t.h[k] = t.rut * (hs + a[5] * Tinv) * c_fast.wt_inv[k];
    if (c_need_eqk) {
      const double sv = (alogt - 1.0) * a[0] + (0.5 * T) * a[1] + (T2 * (1.0 / 6.0)) * a[2] +
                        (T3 * (1.0 / 12.0)) * a[3] + (T4 * 0.05) * a[4];
      smh[k] = sv + a[6] - a[5] * Tinv;
    }
  }
  const int ii = c_mech.ii;
  for (int i = 0; i < ii; ++i) {
    double rkft = c_mech.par[i][0] * exp(c_mech.par[i][1] * alogt - c_mech.par[i][2] * Tinv);
    if (c_mech.lt[i][0] != 0.0 || c_mech.lt[i][1] != 0.0)   // Landau-Teller
      rkft = rkft * exp(c_mech.lt[i][0] / pow(T, kLtP1) + c_mech.lt[i][1] / pow(T, kLtP2));
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
      eqk = eqk * powi(c_mech.patm * Tinv / c_mech.ru, nus);
      rkrt = rkft / fmax(eqk, 1.0e-300);
    } else if (rv == 2) {
      rkrt = c_mech.rpar[i][0] * exp(c_mech.rpar[i][1] * alogt - c_mech.rpar[i][2] * Tinv);
    }
    if (c_mech.rlt[i][0] != 0.0 || c_mech.rlt[i][1] != 0.0)   // reverse Landau-Teller
      rkrt = rkrt * exp(c_mech.rlt[i][0] / pow(T, kLtP1) + c_mech.rlt[i][1] / pow(T, kLtP2));
    t.kf[i] = rkft;
    t.kr[i] = rkrt;
    const int fo = c_mech.fall[i];
    if (fo) {
      t.klow[i] = c_mech.low[i][0] * exp(c_mech.low[i][1] * alogt - c_mech.low[i][2] * Tinv);
      if (fo == 2) {   // SRI: ln(a exp(-b/T) + exp(-T/c)) in the fclog slot
        const double* sr = c_mech.sri[i];
        t.fclog[i] = log(sr[0] * exp(-sr[1] * Tinv) + exp(-T * c_fast.sri_cinv[i]));
      } else if (fo > 1) {
        constexpr double kInvLn10 = 0.4342944819032518277;
        const double ta = c_mech.troe[i][0];
        double fcent = (1.0 - ta) * exp(-T * c_fast.troe_inv[i][0]) + ta * exp(-T * c_fast.troe_inv[i][1]);
        if (fo == 4) fcent = fcent + exp(-c_mech.troe[i][3] * Tinv);
        t.fclog[i] = log(fmax(fcent, 1.0e-300)) * kInvLn10;
      }
    }
  }
}

// The composition-dependent rest of ck_fun_fast, from the temperature terms t.
template <int KK>
HD void fun_cpart(double rho, const double* z, const FunT<KK>& t, double* zp) {
  constexpr double kLn10 = 2.302585092994045684, kInvLn10 = 0.4342944819032518277;
  const double* Y = z + 1;
  double cv = 0.0, C[KK], wdot[KK];
  double ctot = 0.0;
#pragma unroll
  for (int k = 0; k < KK; ++k) {
    cv = cv + Y[k] * t.cvk[k];
    C[k] = rho * Y[k] * c_fast.wt_inv[k];
    ctot = ctot + C[k];
    wdot[k] = 0.0;
  }
  double rop[IZEM_MAXREAC];
  const int ii = c_mech.ii;
  for (int i = 0; i < ii; ++i) {
    double rkft = t.kf[i], rkrt = t.kr[i];
    double ctb = 1.0;
    if (c_mech.thb[i]) {
      ctb = ctot;
      for (int k = 0; k < KK; ++k)
        if (c_mech.eff[i][k] != 1.0) ctb = ctb + (c_mech.eff[i][k] - 1.0) * C[k];
    }
    const int fo = c_mech.fall[i];
    if (fo) {
      const int kf = c_mech.kfal[i];   // collider: (+M), or species kf - 1 alone
      const double pr = t.klow[i] * (kf ? C[kf - 1] : ctb) / rkft;
      if (!kf) ctb = 1.0;
      double pcor = pr / (1.0 + pr);
      if (fo == 2) {
        const double prlog = log(fmax(pr, 1.0e-300)) * kInvLn10;
        const double xp = 1.0 / (1.0 + prlog * prlog);
        pcor = exp(xp * t.fclog[i]) * c_mech.sri[i][3] * pow(t.T, c_mech.sri[i][4]) * pcor;
      } else if (fo > 1) {
        const double prlog = log(fmax(pr, 1.0e-300)) * kInvLn10;
        const double fclog = t.fclog[i];
        const double xn = 0.75 - 1.27 * fclog;
        const double cprlog = prlog - (0.4 + 0.67 * fclog);
        const double q = cprlog / (xn - 0.14 * cprlog);
        const double flog = fclog / (1.0 + q * q);
        pcor = exp(flog * kLn10) * pcor;
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
  for (int n = 0; n < MXSP; ++n)
    for (int i = 0; i < ii; ++i) {
      const int k = c_mech.nuk[i][n];
      if (k >= 0) wdot[k] = wdot[k] + rop[i] * double(c_mech.nu[i][n]);
    }
  const double rho_i = 1.0 / rho;
  double sum = 0.0;
#pragma unroll
  for (int k = 0; k < KK; ++k) {
    zp[k + 1] = wdot[k] * c_mech.wt[k] * rho_i;
    sum = sum + t.h[k] * wdot[k] * c_mech.wt[k] + (-t.rut) * wdot[k];
  }
  zp[0] = -sum / (rho * cv);
}

// The constant-volume reactor right-hand side of ck_fun with the divisions
// by T, by the molar masses and by the Troe and SRI temperatures replaced by
// multiplications with reciprocals, and 10^x / log10 by exp / log: the same
// CHEMKIN expressions (CKCVBS, CKHMS, CKRATT, CKRATX, CKWYR) with different
// rounding (a few ulp per term) and about a sixth of the FP64 instructions
// of the divisions.  The BDF kernels call it in two parts (fun_tpart,
// fun_cpart); ck_fun above keeps the reference's operation order for the
// host build that is compared with the oracle bit for bit.
template <int KK>
HD void ck_fun_fast(double rho, const double* z, double* zp) {
  FunT<KK> t;
  fun_tpart<KK>(z[0], t);
  fun_cpart<KK>(rho, z, t, zp);
}

// The generated right-hand side: the shipped mechanism's, or another one
// that mechgen wrote (-DIZEM_CHEM_GEN_HEADER="\"path\"" at build time).
#ifdef IZEM_CHEM_GEN_HEADER
#include IZEM_CHEM_GEN_HEADER
#else
#include "chem_gen.cuh"
#endif

// Right-hand-side policies of the BDF driver: the generic form, which walks
// the uploaded mechanism's tables, and the generated form of the mechanism
// the library was built with (chem_gen.cuh, phd_gb300/mechgen.py), which
// performs the same operations in the same order with the tables as
// literals.  chem_upload_mech picks the generated form when the uploaded
// mechanism is that one.
template <int KK>
struct RhsTables {
  using Terms = FunT<KK>;
  static HD __forceinline__ void tpart(double T, Terms& t) { fun_tpart<KK>(T, t); }
  static HD __forceinline__ void cpart(double rho, const double* z, const Terms& t, double* zp) {
    fun_cpart<KK>(rho, z, t, zp);
  }
};
struct RhsGenerated {
  using Terms = chem_gen::FunT;
  static HD __forceinline__ void tpart(double T, Terms& t) { chem_gen::tpart(T, t); }
  static HD __forceinline__ void cpart(double rho, const double* z, const Terms& t, double* zp) {
    chem_gen::cpart(rho, z, t, zp);
  }
};

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

// LINPACK DGEFA/DGESL (vode.f:7033/7630).  The outer loops stay rolled: the
// integrator's control code runs divergently across a warp, and unrolled it
// is large enough to miss in the instruction cache.
template <int N>
HD int dgefa(double* a, int* ipvt) {
  int info = 0;
#pragma unroll 1
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
#pragma unroll 1
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
#pragma unroll 1
  for (int k = 0; k < N - 1; ++k) {
    const int l = ipvt[k];
    const double t = b[l];
    if (l != k) { b[l] = b[k]; b[k] = t; }
    if (t != 0.0)
      for (int i = k + 1; i < N; ++i) b[i] = b[i] + t * a[i + k * N];
  }
#pragma unroll 1
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

// ------------------------------------------ DVODE as a resumable machine ----
// The integrator below is DVODE's BDF path (DVODE -> DVHIN, DVSTEP -> DVNLSD
// -> DVJAC, vode.f:4286-7790) inside REACTION_V's restart loop, written in
// reverse-communication form: rc_advance() runs the control logic of one
// cell until it needs the right-hand side FUN at the current y, stores its
// position in `pc` and returns true; the caller evaluates FUN(y) into fo and
// calls rc_advance() again.  Every right-hand-side evaluation of the method
// is one of six such requests:
//   F0    the initial derivative (DVODE, before DVHIN)
//   HIN   a trial derivative of the initial-step iteration (DVHIN)
//   PRED  f at the predicted state (DVNLSD, each pass)
//   JAC   one column of the finite-difference Jacobian (DVJAC)
//   CORR  f after a corrector update (DVNLSD)
//   ERRF  f after repeated error-test failures at order 1 (DVSTEP)
// A warp's threads, each on its own cell and at its own point of the method,
// so all evaluate FUN together in one converged call per round, and only the
// (cheaper) control logic diverges.  The arithmetic and its order are those
// of a straight-line restatement of DVODE; results are identical to it.
enum : int {
  ST_DVODE = 0, ST_F0, ST_HIN_ITER, ST_HIN_F, ST_MAIN, ST_STEP_BEGIN, ST_STEP_LOOP, ST_NLS_PASS, ST_NLS_PRED_F,
  ST_JAC_COL, ST_JAC_COL_F, ST_NLS_ITER, ST_NLS_CORR_F, ST_ERRF_F, ST_DONE
};

template <int N>
struct Rc : Dv<N> {
  double y[N], fo[N];                       // FUN argument / result
  double tcur, tout;                        // REACTION_V's time and target
  double hg, hub, hlb, hnew;                // DVHIN
  double told;                              // DVSTEP
  double delp;                              // DVNLSD
  double yj, rfac, r0;                      // DVJAC
  int pc, ib, istate, nsteps;               // REACTION_V
  int first, mguard, iter;                  // DVODE main loop, DVHIN
  int ncf, nflag, rescale, sguard;          // DVSTEP
  int pass, m, it, jcol;                    // DVNLSD, DVJAC
};

template <int N>
HD void rc_start(Rc<N>& r, double rho, const double* z, double tf) {
  r.rho = rho;
  for (int i = 0; i < N; ++i) r.y[i] = z[i];
  r.tcur = 0.0;
  r.tout = tf;
  r.istate = 1;
  r.ib = 0;
  r.nsteps = 0;
  r.pc = ST_DVODE;
}

// REACTION_V: after each DVODE return, restart while ISTATE != 2, at most 20 calls.
template <int N>
HD __forceinline__ void rc_after_dvode(Rc<N>& r, int istate) {
  r.istate = istate;
  r.ib = r.ib + 1;
  r.pc = (r.ib < 20 && istate != 2) ? ST_DVODE : ST_DONE;
}

// DVODE after DVHIN: scale the first Nordsieck column and enter the step loop.
template <int N>
HD __forceinline__ void rc_hin_finish(Rc<N>& r, double h0) {
  h0 = copysign(h0, r.tout - r.tcur);
  r.h = h0;
  for (int i = 0; i < N; ++i) r.yh[i + N] = h0 * r.yh[i + N];
  r.first = 1;
  r.mguard = 0;
  r.pc = ST_MAIN;
}

// DVODE after a DVSTEP return with flag kflag.
template <int N>
HD void rc_step_return(Rc<N>& r, int kflag) {
  if (kflag != 0) {
    for (int i = 0; i < N; ++i) r.y[i] = r.yh[i];
    r.tcur = r.tn;
    r.nsteps += r.nst;
    rc_after_dvode(r, kflag == -1 ? -4 : -5);
    return;
  }
  if ((r.tn - r.tout) * r.h < 0.0) {
    r.mguard = r.mguard + 1;
    r.pc = ST_MAIN;
    return;
  }
  // DVINDY (K = 0)
  const double s = (r.tout - r.tn) / r.h;
  for (int i = 0; i < N; ++i) r.y[i] = r.yh[i + (r.l - 1) * N];
  for (int jb = 1; jb <= r.nq; ++jb) {
    const int j = r.nq - jb;
    for (int i = 0; i < N; ++i) r.y[i] = r.yh[i + j * N] + s * r.y[i];
  }
  r.tcur = r.tout;
  r.nsteps += r.nst;
  rc_after_dvode(r, 2);
}

// DVNLSD's exit: sets the flag and continues DVSTEP.  Returns true when
// DVSTEP needs FUN (the order-1 restart after repeated error-test failures).
template <int N>
HD bool rc_nls_return(Rc<N>& r, int ret) {
  r.nflag = ret;
  if (r.nflag != 0) {
    r.ncf = r.ncf + 1;
    r.etamax = 1.0;
    r.tn = r.told;
    for (int jb = 1; jb <= r.nq; ++jb)
      for (int i = r.nqnyh - jb * N; i < r.nqnyh; ++i) r.yh[i] = r.yh[i] - r.yh[i + N];
    if (r.ncf == 10) { r.kflag = -2; r.jstart = 1; rc_step_return(r, r.kflag); return false; }
    r.eta = 0.25;
    r.nflag = -1;
    r.sguard = r.sguard + 1;
    r.pc = ST_STEP_LOOP;
    return false;
  }
  const double dsm = r.acnrm / r.tq[1];
  if (dsm <= 1.0) {
    r.kflag = 0;
    r.nst = r.nst + 1;
    r.hu = r.h;
    for (int iback = 1; iback <= r.nq; ++iback) {
      const int i = r.l - iback;
      r.tau[i] = r.tau[i - 1];
    }
    r.tau[0] = r.h;
    for (int j = 1; j <= r.l; ++j) {
      const double a = r.el[j - 1];
      if (a != 0.0)
        for (int i = 0; i < N; ++i) r.yh[i + (j - 1) * N] = r.yh[i + (j - 1) * N] + a * r.acor[i];
    }
    r.nqwait = r.nqwait - 1;
    if (!(r.l == r.lmax || r.nqwait != 1)) {
      for (int i = 0; i < N; ++i) r.yh[i + (r.lmax - 1) * N] = r.acor[i];
      r.conp = r.tq[4];
    }
    if (r.etamax != 1.0) {
      const double flotl = double(r.l);
      r.etaq = 1.0 / (pow(6.0 * dsm, 1.0 / flotl) + 1.0e-6);
      if (r.nqwait != 0) {
        r.eta = r.etaq;
        r.newq = r.nq;
      } else {
        r.nqwait = 2;
        r.etaqm1 = 0.0;
        if (r.nq != 1) {
          double col[N];
          for (int i = 0; i < N; ++i) col[i] = r.yh[i + (r.l - 1) * N];
          const double ddn = dvnorm<N>(col, r.ewt) / r.tq[0];
          r.etaqm1 = 1.0 / (pow(6.0 * ddn, 1.0 / (flotl - 1.0)) + 1.0e-6);
        }
        double etaqp1 = 0.0;
        if (r.l != r.lmax) {
          const double cnquot = (r.tq[4] / r.conp) * powi(r.h / r.tau[1], r.l);
          for (int i = 0; i < N; ++i) r.savf[i] = r.acor[i] - cnquot * r.yh[i + (r.lmax - 1) * N];
          const double dup = dvnorm<N>(r.savf, r.ewt) / r.tq[2];
          etaqp1 = 1.0 / (pow(10.0 * dup, 1.0 / (flotl + 1.0)) + 1.0e-6);
        }
        if (r.etaq >= etaqp1) {
          if (r.etaq < r.etaqm1) { r.eta = r.etaqm1; r.newq = r.nq - 1; }
          else { r.eta = r.etaq; r.newq = r.nq; }
        } else if (etaqp1 > r.etaqm1) {
          r.eta = etaqp1;
          r.newq = r.nq + 1;
          for (int i = 0; i < N; ++i) r.yh[i + (r.lmax - 1) * N] = r.acor[i];
        } else { r.eta = r.etaqm1; r.newq = r.nq - 1; }
      }
      if (r.eta < 1.5 || r.etamax == 1.0) { r.newq = r.nq; r.newh = 0; r.eta = 1.0; r.hnew = r.h; }
      else { r.eta = fmin(r.eta, r.etamax); r.newh = 1; r.hnew = r.h * r.eta; }
    } else {
      if (r.nqwait < 2) r.nqwait = 2;
      r.newq = r.nq; r.newh = 0; r.eta = 1.0; r.hnew = r.h;
    }
    r.etamax = 10.0;   // ETAMX2 = ETAMX3 = 10
    const double rr = 1.0 / r.tq[1];
    for (int i = 0; i < N; ++i) r.acor[i] = rr * r.acor[i];
    r.jstart = 1;
    rc_step_return(r, 0);
    return false;
  }
  // error test failed
  r.kflag = r.kflag - 1;
  r.nflag = -2;
  r.tn = r.told;
  for (int jb = 1; jb <= r.nq; ++jb)
    for (int i = r.nqnyh - jb * N; i < r.nqnyh; ++i) r.yh[i] = r.yh[i] - r.yh[i + N];
  r.etamax = 1.0;
  if (r.kflag > -3) {
    r.eta = 1.0 / (pow(6.0 * dsm, 1.0 / double(r.l)) + 1.0e-6);
    r.eta = fmax(r.eta, 0.1);
    if (r.kflag <= -2 && r.eta > 0.2) r.eta = 0.2;
    r.sguard = r.sguard + 1;
    r.pc = ST_STEP_LOOP;
    return false;
  }
  if (r.kflag == -7) { r.kflag = -1; r.jstart = 1; rc_step_return(r, r.kflag); return false; }
  if (r.nq != 1) {
    r.eta = 0.1;
    dvjust<N>(r, -1);
    r.l = r.nq;
    r.nq = r.nq - 1;
    r.nqwait = r.l;
    r.sguard = r.sguard + 1;
    r.pc = ST_STEP_LOOP;
    return false;
  }
  r.eta = 0.1;
  r.h = r.h * r.eta;
  r.hscal = r.h;
  r.tau[0] = r.h;
  r.pc = ST_ERRF_F;
  return true;
}

// Second half of DVJAC (iteration matrix and LU) and its return into DVNLSD.
// Returns true when the Newton iteration starts (ST_NLS_ITER), false when
// DVNLSD returned (state already advanced).
template <int N>
HD void rc_jac_lu(Rc<N>& r) {
  const double con = -(r.h * r.rl1);
#pragma unroll 1
  for (int q = 0; q < N * N; ++q) r.wm[q] = con * r.wmjs[q];
  for (int i = 0; i < N; ++i) r.wm[i + i * N] = r.wm[i + i * N] + 1.0;
  const int ierpj = dgefa<N>(r.wm, r.ipvt) != 0 ? 1 : 0;
  r.ipup = 0;
  r.rc = 1.0;
  r.drc = 0.0;
  r.crate = 1.0;
  r.nslp = r.nst;
  if (ierpj != 0) {
    r.icf = 2;
    r.ipup = 2;
    if (rc_nls_return(r, -1)) return;   // pc already ST_ERRF_F
    return;
  }
  for (int i = 0; i < N; ++i) r.acor[i] = 0.0;
  r.it = 0;
  r.pc = ST_NLS_ITER;
}

// Runs the method until FUN(y) is needed (returns true; the result goes to
// fo) or the cell is finished (returns false; pc == ST_DONE, y holds the
// final state, istate and nsteps are REACTION_V's).
template <int N>
HD bool rc_advance(Rc<N>& r) {
  for (int guard = 0; guard < 512; ++guard) {
    switch (r.pc) {
      case ST_DVODE: {   // DVODE entry (ISTATE = 1, ITASK = 1)
        if (r.tout == r.tcur) { rc_after_dvode(r, 1); break; }
        r.tn = r.tcur;
        r.jstart = 0; r.nslj = 0; r.nst = 0; r.hu = 0.0; r.icf = 0; r.ipup = 0; r.jcur = 0; r.newh = 0;
        r.newq = 1; r.conp = 0.0; r.crate = 0.0; r.drc = 0.0; r.acnrm = 0.0; r.nslp = 0;
        r.pc = ST_F0;
        return true;
      }
      case ST_F0: {
        for (int i = 0; i < N; ++i) r.yh[i + N] = r.fo[i];
        for (int i = 0; i < N; ++i) r.yh[i] = r.y[i];
        r.nq = 1;
        r.h = 1.0;
        for (int i = 0; i < N; ++i) r.ewt[i] = 1.0 / (kRtol * fabs(r.yh[i]) + kAtol);
        // DVHIN
        const double tdist = fabs(r.tout - r.tcur);
        const double tround = kUround * fmax(fabs(r.tcur), fabs(r.tout));
        if (tdist < 2.0 * tround) { rc_after_dvode(r, -3); break; }
        r.hlb = 100.0 * tround;
        r.hub = 0.1 * tdist;
        for (int i = 0; i < N; ++i) {
          const double delyi = 0.1 * fabs(r.yh[i]) + kAtol;
          const double afi = fabs(r.yh[i + N]);
          if (afi * r.hub > delyi) r.hub = delyi / afi;
        }
        r.hg = sqrt(r.hlb * r.hub);
        r.hnew = r.hg;
        if (r.hub < r.hlb) { rc_hin_finish(r, r.hg); break; }
        r.iter = 0;
        r.pc = ST_HIN_ITER;
        break;
      }
      case ST_HIN_ITER: {
        for (int i = 0; i < N; ++i) r.y[i] = r.yh[i] + r.hg * r.yh[i + N];
        r.pc = ST_HIN_F;
        return true;
      }
      case ST_HIN_F: {
        double ft[N];
        for (int i = 0; i < N; ++i) ft[i] = (r.fo[i] - r.yh[i + N]) / r.hg;
        const double yddnrm = dvnorm<N>(ft, r.ewt);
        r.hnew = (yddnrm * r.hub * r.hub > 2.0) ? sqrt(2.0 / yddnrm) : sqrt(r.hg * r.hub);
        r.iter = r.iter + 1;
        bool done = r.iter >= 4;
        if (!done) {
          const double hrat = r.hnew / r.hg;
          if (hrat > 0.5 && hrat < 2.0) done = true;
          else if (r.iter >= 2 && r.hnew > 2.0 * r.hg) { r.hnew = r.hg; done = true; }
        }
        if (!done) { r.hg = r.hnew; r.pc = ST_HIN_ITER; break; }
        double h0 = r.hnew * 0.5;
        if (h0 < r.hlb) h0 = r.hlb;
        if (h0 > r.hub) h0 = r.hub;
        rc_hin_finish(r, h0);
        break;
      }
      case ST_MAIN: {   // one pass of DVODE's step loop (at most 600)
        if (r.mguard >= 600) { r.nsteps += r.nst; rc_after_dvode(r, -1); break; }
        if (!r.first) {
          if (r.nst >= 500) {
            for (int i = 0; i < N; ++i) r.y[i] = r.yh[i];
            r.tcur = r.tn;
            r.nsteps += r.nst;
            rc_after_dvode(r, -1);
            break;
          }
          for (int i = 0; i < N; ++i) r.ewt[i] = 1.0 / (kRtol * fabs(r.yh[i]) + kAtol);
        }
        r.first = 0;
        if (kUround * dvnorm<N>(r.yh, r.ewt) > 1.0) {
          for (int i = 0; i < N; ++i) r.y[i] = r.yh[i];
          r.tcur = r.tn;
          r.nsteps += r.nst;
          rc_after_dvode(r, -2);
          break;
        }
        r.pc = ST_STEP_BEGIN;
        break;
      }
      case ST_STEP_BEGIN: {   // DVSTEP entry
        r.kflag = 0;
        r.told = r.tn;
        r.ncf = 0;
        r.nflag = 0;
        r.jcur = 0;
        if (r.jstart > 0) {
          r.rescale = 0;
          if (r.newh != 0) {
            if (r.newq < r.nq) { dvjust<N>(r, -1); r.nq = r.newq; r.l = r.nq + 1; r.nqwait = r.l; }
            else if (r.newq > r.nq) { dvjust<N>(r, 1); r.nq = r.newq; r.l = r.nq + 1; r.nqwait = r.l; }
            r.rescale = 1;
          }
        } else {
          r.lmax = 6;
          r.nq = 1;
          r.l = 2;
          r.nqnyh = N;
          r.tau[0] = r.h;
          r.prl1 = 1.0;
          r.rc = 0.0;
          r.etamax = 1.0e4;
          r.nqwait = 2;
          r.hscal = r.h;
          r.rescale = 0;
        }
        r.sguard = 0;
        r.pc = ST_STEP_LOOP;
        break;
      }
      case ST_STEP_LOOP: {   // one attempt of DVSTEP (at most 64)
        if (r.sguard >= 64) { r.kflag = -2; r.jstart = 1; rc_step_return(r, r.kflag); break; }
        if (r.rescale) {
          double rr = 1.0;
          for (int j = 2; j <= r.l; ++j) {
            rr = rr * r.eta;
            for (int i = 0; i < N; ++i) r.yh[i + (j - 1) * N] = rr * r.yh[i + (j - 1) * N];
          }
          r.h = r.hscal * r.eta;
          r.hscal = r.h;
          r.rc = r.rc * r.eta;
          r.nqnyh = r.nq * N;
        }
        r.rescale = 1;
        r.tn = r.tn + r.h;
        for (int jb = 1; jb <= r.nq; ++jb)
          for (int i = r.nqnyh - jb * N; i < r.nqnyh; ++i) r.yh[i] = r.yh[i] + r.yh[i + N];
        dvset<N>(r);
        r.rl1 = 1.0 / r.el[1];
        r.rc = r.rc * (r.rl1 / r.prl1);
        r.prl1 = r.rl1;
        // DVNLSD entry
        if (r.jstart == 0) r.nslp = 0;
        if (r.nflag == 0) r.icf = 0;
        if (r.nflag == -2) r.ipup = 2;
        if (r.jstart == 0) r.ipup = 2;
        r.drc = fabs(r.rc - 1.0);
        if (r.drc > 0.3 || r.nst >= r.nslp + 20) r.ipup = 2;
        r.pass = 0;
        r.pc = ST_NLS_PASS;
        break;
      }
      case ST_NLS_PASS: {
        if (r.pass >= 2) {
          r.icf = 2;
          r.ipup = 2;
          if (rc_nls_return(r, -1)) return true;
          break;
        }
        r.m = 0;
        r.delp = 0.0;
        for (int i = 0; i < N; ++i) r.y[i] = r.yh[i];
        r.pc = ST_NLS_PRED_F;
        return true;
      }
      case ST_NLS_PRED_F: {
        for (int i = 0; i < N; ++i) r.savf[i] = r.fo[i];
        if (r.ipup > 0) {   // DVJAC
          int jok = 1;
          if (r.nst == 0 || r.nst > r.nslj + 50) jok = -1;
          if (r.icf == 1 && r.drc < 0.2) jok = -1;
          if (r.icf == 2) jok = -1;
          if (jok == -1) {
            r.nslj = r.nst;
            r.jcur = 1;
            const double fac = dvnorm<N>(r.savf, r.ewt);
            r.r0 = 1000.0 * fabs(r.h) * kUround * double(N) * fac;
            if (r.r0 == 0.0) r.r0 = 1.0;
            r.jcol = 0;
            r.pc = ST_JAC_COL;
            break;
          }
          r.jcur = 0;
          rc_jac_lu(r);
          if (r.pc == ST_ERRF_F) return true;
          break;
        }
        for (int i = 0; i < N; ++i) r.acor[i] = 0.0;
        r.it = 0;
        r.pc = ST_NLS_ITER;
        break;
      }
      case ST_JAC_COL: {
        if (r.jcol >= N) {
          rc_jac_lu(r);
          if (r.pc == ST_ERRF_F) return true;
          break;
        }
        const double srur = 1.4901161193847656e-08;   // sqrt(UROUND)
        // columns are independent: the species columns (1..N-1) come first,
        // at the temperature of the FUN call before the Jacobian, and the
        // temperature column last (rc_drive reuses the temperature terms)
        const int j = (r.jcol + 1) % N;
        r.yj = r.y[j];
        const double rj = fmax(srur * fabs(r.yj), r.r0 / r.ewt[j]);
        r.y[j] = r.y[j] + rj;
        r.rfac = 1.0 / rj;
        r.pc = ST_JAC_COL_F;
        return true;
      }
      case ST_JAC_COL_F: {
        const int j = (r.jcol + 1) % N;
        for (int i = 0; i < N; ++i) r.wmjs[i + j * N] = (r.fo[i] - r.savf[i]) * r.rfac;
        r.y[j] = r.yj;
        r.jcol = r.jcol + 1;
        r.pc = ST_JAC_COL;
        break;
      }
      case ST_NLS_ITER: {   // corrector iteration (at most 3)
        bool fail = r.it >= 3;
        if (!fail) {
          for (int i = 0; i < N; ++i) r.y[i] = (r.rl1 * r.h) * r.savf[i] - (r.rl1 * r.yh[i + N] + r.acor[i]);
          dgesl<N>(r.wm, r.ipvt, r.y);
          if (r.rc != 1.0) {
            const double cscale = 2.0 / (1.0 + r.rc);
            for (int i = 0; i < N; ++i) r.y[i] = cscale * r.y[i];
          }
          const double del = dvnorm<N>(r.y, r.ewt);
          for (int i = 0; i < N; ++i) r.acor[i] = r.acor[i] + r.y[i];
          for (int i = 0; i < N; ++i) r.y[i] = r.yh[i] + r.acor[i];
          if (r.m != 0) r.crate = fmax(0.3 * r.crate, del / r.delp);
          const double dcon = del * fmin(1.0, r.crate) / r.tq[3];
          if (dcon <= 1.0) {
            r.jcur = 0;
            r.icf = 0;
            r.acnrm = (r.m == 0) ? del : dvnorm<N>(r.acor, r.ewt);
            if (rc_nls_return(r, 0)) return true;
            break;
          }
          r.m = r.m + 1;
          if (r.m == 3 || (r.m >= 2 && del > 2.0 * r.delp)) {
            fail = true;
          } else {
            r.delp = del;
            r.pc = ST_NLS_CORR_F;
            return true;
          }
        }
        // corrector failed on this pass
        if (r.jcur == 1) {
          r.icf = 2;
          r.ipup = 2;
          if (rc_nls_return(r, -1)) return true;
          break;
        }
        r.icf = 1;
        r.ipup = 2;
        r.pass = r.pass + 1;
        r.pc = ST_NLS_PASS;
        break;
      }
      case ST_NLS_CORR_F: {
        for (int i = 0; i < N; ++i) r.savf[i] = r.fo[i];
        r.it = r.it + 1;
        r.pc = ST_NLS_ITER;
        break;
      }
      case ST_ERRF_F: {
        for (int i = 0; i < N; ++i) r.savf[i] = r.fo[i];
        for (int i = 0; i < N; ++i) r.yh[i + N] = r.h * r.savf[i];
        r.nqwait = 10;
        r.rescale = 0;
        r.sguard = r.sguard + 1;
        r.pc = ST_STEP_LOOP;
        break;
      }
      default:
        return false;   // ST_DONE
    }
  }
  // no path of the method takes this many transitions without a FUN request
  r.istate = -99;
  r.pc = ST_DONE;
  return false;
}

// One cell from start to finish on the calling thread (host checks, and any
// caller that does not batch FUN evaluations across threads).
template <int N>
HD int reaction_v(double rho, double* z, double tf, int* nsteps) {
  Rc<N> r;
  rc_start<N>(r, rho, z, tf);
  while (rc_advance<N>(r)) ck_fun<N - 1>(r.rho, r.y, r.fo);
  for (int i = 0; i < N; ++i) z[i] = r.y[i];
  *nsteps = r.nsteps;
  return r.istate;
}

// ---------------------------------------------------------------- kernels ---
// Persistent driver shared by the chemistry kernels: each thread takes cells
// from *counter until all n are taken.  Per round, a thread either finishes
// its cell (store) or advances it to its next right-hand-side request; the
// requests of all threads are then evaluated in one converged FUN call.
// The loop ends: every cell's integration is bounded by DVODE's own limits
// (20 restarts, 600 steps, 64 attempts per step, 2 corrector passes), and
// kMaxFun caps the FUN rounds of one cell above that bound.
constexpr long long kMaxFun = 1LL << 25;

template <int KK, class Rhs, class Load, class Store>
__device__ __forceinline__ void rc_drive(unsigned n, unsigned* counter, Load load, Store store) {
  constexpr int N = KK + 1;
  Rc<N> r;
  typename Rhs::Terms ft;   // temperature terms of this thread's last right-hand side
  ft.T = -1.0;
  unsigned q = 0;
  bool active = false;
  long long nfun = 0;
  while (true) {
    if (!active) {
      q = atomicAdd(counter, 1u);
      if (q >= n) return;
      double rho, tf, z[N];
      load(q, rho, z, tf);
      rc_start<N>(r, rho, z, tf);
      active = true;
      nfun = 0;
    }
    bool need = rc_advance<N>(r);
    if (need && ++nfun > kMaxFun) { r.istate = -99; need = false; }
    if (need) {
      // The temperature terms are recomputed unless every evaluating lane
      // of the warp is at the temperature of its previous call (the
      // species columns of a Jacobian): a per-lane choice would only make
      // the warp wait for its slowest lane.  Reused terms are the bits the
      // recomputation would give.
      if (!__all_sync(__activemask(), r.y[0] == ft.T)) Rhs::tpart(r.y[0], ft);
      Rhs::cpart(r.rho, r.y, ft, r.fo);
    } else {
      store(q, r);
      active = false;
    }
  }
}

template <int KK>
__device__ __forceinline__ void chem_stats_add(ChemStats* stats, int istate, int nst) {
  if (istate <= -2) atomicAdd(&stats->failed, 1);
  atomicMax(&stats->max_steps, nst);
  atomicAdd(&stats->total_steps, (unsigned long long)nst);
}

// Ghosted linear index of window cell q (i fastest): the reaction_dvode
// loop order over the chemistry window (module_reaction.f90:155-171).
__device__ __forceinline__ long long window_point(const ChemField& f, unsigned q) {
  const int i = f.ix + (int)(q % f.wx);
  const long long r = q / f.wx;
  const int j = f.iy + (int)(r % f.wy);
  const int k = f.iz + (int)(r / f.wy);
  return (long long)(i - 1 + f.ng) + (long long)f.gx * ((long long)(j - 1 + f.ng) + (long long)f.gy * (long long)(k - 1 + f.ng));
}

// Window -> independent reactors in physical units: T [K], rho [g/cm^3],
// Y (n x KK, row-major), dt [s] (the inputs reaction_dvode hands PSR_CHEMKIN).
template <int KK>
__global__ void k_chem_gather(ChemField f, double* T, double* rho, double* Y, double* dt) {
  const long long n = (long long)f.wx * f.wy * f.wz;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const long long p = window_point(f, (unsigned)q);
  const long long nc = f.ncell;
  const double rho0 = f.v[p];
  const double rho_i = 1.0 / rho0;
#pragma unroll
  for (int l = 0; l < KK; ++l) Y[q * KK + l] = f.v[(5 + l) * nc + p] * rho_i;
  T[q] = f.T[p] * f.t_ref;
  rho[q] = rho0 * f.rho_cgs;
  dt[q] = f.dt_phys;
}

// Reactors -> window, with reaction_dvode's post-processing (module_reaction.f90:
// 275-290): Y clipped to [0,1], the last species closes the sum, T back to code
// units; max |dT| into the statistics.
template <int KK>
__global__ void k_chem_scatter(ChemField f, const double* T, const double* Y, ChemStats* stats) {
  const long long n = (long long)f.wx * f.wy * f.wz;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const long long p = window_point(f, (unsigned)q);
  const long long nc = f.ncell;
  const double rho0 = f.v[p];
  const double T0 = f.T[p] * f.t_ref;
  f.T[p] = T[q] * f.tref_i;
  const double dT = fabs(T[q] - T0);
  atomic_max_nonneg_warp(&stats->dtmax_bits, dT);
  double sumY = 0.0;
#pragma unroll
  for (int l = 0; l < KK - 1; ++l) {
    const double Ya = fmin(fmax(Y[q * KK + l], 0.0), 1.0);
    f.v[(5 + l) * nc + p] = rho0 * Ya;
    sumY = sumY + Ya;
  }
  f.v[(5 + KK - 1) * nc + p] = rho0 * (1.0 - sumY);
  if (f.dT_out) f.dT_out[q] = T[q] - T0;
}

// The dvodesimp selection of reaction_dvode (module_reaction.f90:173-215):
// a gathered reactor goes to the integrator only if some species would move
// by more than 1e-12 in dt at its initial production rates (psr_simp_chemkin:
// CKWYR rates x molar mass x dt / rho, psr_simp_chemkin.f:31-42) and it is
// neither the pure fuel nor the pure oxidiser (H2 and N2 both off by more
// than 1e-6).  The selected reactors are appended to list.
template <int KK>
__global__ void k_chem_select(int n, const double* T, const double* rho, const double* Y, const double* dt,
                              ChemSkip sk, int* list, unsigned* count) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  double y[KK], w[KK];
#pragma unroll
  for (int l = 0; l < KK; ++l) y[l] = Y[(long long)q * KK + l];
  ck_wyr<KK>(rho[q], T[q], y, w);
  const double myc = dt[q] / rho[q];
  bool call_w = false;
#pragma unroll
  for (int l = 0; l < KK; ++l)
    if (fabs(w[l] * c_mech.wt[l] * myc) > 1.0e-12) call_w = true;
  const double yh = y[sk.ih2], yn = y[sk.in2];
  const bool call_f = fabs(yh - sk.yf_h2) > 1.0e-6 && fabs(yn - sk.yf_n2) > 1.0e-6;
  const bool call_o = fabs(yh - sk.yo_h2) > 1.0e-6 && fabs(yn - sk.yo_n2) > 1.0e-6;
  if (call_w && call_f && call_o) list[atomicAdd(count, 1u)] = q;
}

// Selected reactors -> window with the dvodesimp branch's post-processing
// (module_reaction.f90:219-245): as k_chem_scatter, except that the closing
// species is clipped to [0, 1] as well.  Cells not in the list keep their
// state and do not enter max |dT|.
template <int KK>
__global__ void k_chem_scatter_list(ChemField f, const int* list, const unsigned* count, const double* T,
                                    const double* Y, ChemStats* stats) {
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= *count) return;
  const int q = list[t];
  const long long p = window_point(f, (unsigned)q);
  const long long nc = f.ncell;
  const double rho0 = f.v[p];
  const double T0 = f.T[p] * f.t_ref;
  f.T[p] = T[q] * f.tref_i;
  const double dT = fabs(T[q] - T0);
  atomic_max_nonneg_warp(&stats->dtmax_bits, dT);
  double sumY = 0.0;
#pragma unroll
  for (int l = 0; l < KK - 1; ++l) {
    const double Ya = fmin(fmax(Y[(long long)q * KK + l], 0.0), 1.0);
    f.v[(5 + l) * nc + p] = rho0 * Ya;
    sumY = sumY + Ya;
  }
  const double Yl = fmin(fmax(1.0 - sumY, 0.0), 1.0);
  f.v[(5 + KK - 1) * nc + p] = rho0 * Yl;
}

// The persistent chemistry kernels come in variants that differ only in
// the register budget the compiler is held to (128 threads per block, at
// least MINB blocks resident per SM): fewer registers give more resident
// warps to hide the FP64 and local-memory latency of the BDF state machine,
// more registers fewer spills.  The source is the same in every variant;
// the compiler may fuse a multiply and an add into an FMA differently under
// another register limit, so the variants agree within the integrator's
// tolerance rather than to the bit.
constexpr int kChemThreads = 128;

template <int KK, int MINB, class Rhs>
__global__ void __launch_bounds__(kChemThreads, MINB) k_psr_field(ChemField f, unsigned* counter, ChemStats* stats) {
  constexpr int N = KK + 1;
  const long long ncell = (long long)f.wx * f.wy * f.wz;
  const long long nc = f.ncell;
  auto point = [&](unsigned q) { return window_point(f, q); };
  auto load = [&](unsigned q, double& rho, double* z, double& tf) {
    const long long p = point(q);
    const double rho0 = f.v[p];
    const double rho_i = 1.0 / rho0;
#pragma unroll
    for (int l = 0; l < KK; ++l) z[1 + l] = f.v[(5 + l) * nc + p] * rho_i;
    z[0] = f.T[p] * f.t_ref;
    rho = rho0 * f.rho_cgs;
    tf = f.dt_phys;
  };
  auto store = [&](unsigned q, const Rc<N>& r) {
    const long long p = point(q);
    const double rho0 = f.v[p];
    const double T0 = f.T[p] * f.t_ref;
    chem_stats_add<KK>(stats, r.istate, r.nsteps);
    f.T[p] = r.y[0] * f.tref_i;
    const double dT = fabs(r.y[0] - T0);
    atomicMax(&stats->dtmax_bits, (unsigned long long)__double_as_longlong(dT));
    double sumY = 0.0;
#pragma unroll
    for (int l = 0; l < KK - 1; ++l) {
      const double Ya = fmin(fmax(r.y[1 + l], 0.0), 1.0);
      f.v[(5 + l) * nc + p] = rho0 * Ya;
      sumY = sumY + Ya;
    }
    f.v[(5 + KK - 1) * nc + p] = rho0 * (1.0 - sumY);
    if (f.dT_out) f.dT_out[q] = r.y[0] - T0;
  };
  rc_drive<KK, Rhs>((unsigned)ncell, counter, load, store);
}

template <int KK, int MINB, class Rhs>
__global__ void __launch_bounds__(kChemThreads, MINB) k_psr_batch(int n, double* T, const double* rho, double* Y,
                                                                  const double* dt, int* istate, int* nsteps,
                                                                  unsigned* counter, ChemStats* stats) {
  constexpr int N = KK + 1;
  auto load = [&](unsigned q, double& rh, double* z, double& tf) {
    z[0] = T[q];
#pragma unroll
    for (int l = 0; l < KK; ++l) z[1 + l] = Y[(size_t)q * KK + l];
    rh = rho[q];
    tf = dt[q];
  };
  auto store = [&](unsigned q, const Rc<N>& r) {
    chem_stats_add<KK>(stats, r.istate, r.nsteps);
    T[q] = r.y[0];
#pragma unroll
    for (int l = 0; l < KK; ++l) Y[(size_t)q * KK + l] = r.y[1 + l];
    if (istate) istate[q] = r.istate;
    if (nsteps) nsteps[q] = r.nsteps;
  };
  rc_drive<KK, Rhs>((unsigned)n, counter, load, store);
}

// ------------------------------------------------ surrogate support --------
// Inputs of the learned surrogate: T [K], ln p [atm], ln(Y_k + 1e-10),
// ln dt [s], normalised by the training means / standard deviations.
// The features are formed in FP64 as on the host that trains the networks,
// so a device row rounds to the same BF16 values as the host's (the
// reciprocal multiplications below move an FP64 value by an ulp at most,
// which changes its BF16 rounding only when it lies within that ulp of a
// BF16 rounding boundary); one pass writes the inputs of both networks of
// an ensemble (x2 may be null); rows are 16 BF16 values, written as two
// 16-byte stores.  Launched with at least 32 threads per block.
template <int KK>
__global__ void k_featurize(int n, const double* T, const double* rho, const double* Y, const double* dt,
                            const float* norm, __nv_bfloat16* x, const float* norm2, __nv_bfloat16* x2) {
  static_assert(KK + 3 <= 16, "one 16-wide input row");
  // 1 / std of each input of both networks, once per block
  __shared__ double s_inv[2][16];
  if (threadIdx.x < 32) {
    const int net = threadIdx.x >> 4, c = threadIdx.x & 15;
    const float* nm = net ? norm2 : norm;
    s_inv[net][c] = (nm && c < KK + 3) ? 1.0 / (double)nm[KK + 3 + c] : 0.0;
  }
  __syncthreads();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  double f[16];
  const double Tq = T[q];
  double wmi = 0.0;
#pragma unroll
  for (int k = 0; k < KK; ++k) wmi += fmax(Y[(size_t)q * KK + k], 0.0) * c_fast.wt_inv[k];
  const double p_atm = rho[q] * c_mech.ru * Tq * wmi / c_mech.patm;
  f[0] = Tq;
  f[1] = log(p_atm);
#pragma unroll
  for (int k = 0; k < KK; ++k) f[2 + k] = log(fmax(Y[(size_t)q * KK + k], 0.0) + 1.0e-10);
  f[KK + 2] = log(dt[q]);
  for (int net = 0; net < 2; ++net) {
    const float* nm = net ? norm2 : norm;
    __nv_bfloat16* out = net ? x2 : x;
    if (!out) break;
    uint32_t pk[8];
#pragma unroll
    for (int c = 0; c < 16; c += 2) {
      const float a = c < KK + 3 ? (float)((f[c] - nm[c]) * s_inv[net][c]) : 0.f;
      const float b = c + 1 < KK + 3 ? (float)((f[c + 1] - nm[c + 1]) * s_inv[net][c + 1]) : 0.f;
      __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
      pk[c / 2] = *reinterpret_cast<uint32_t*>(&h);
    }
    uint4* dst = reinterpret_cast<uint4*>(out + (size_t)q * 16);
    dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
  }
}

struct GateArgs {
  double tmin, tmax, dtmin, dtmax;   // training envelope
  double tol_el;                     // relative element residual
  double tol_T_abs, tol_T_rel;       // energy-consistency of dT [K]
  double tol_ens_abs, tol_ens_rel;   // agreement of two independently trained networks on dT [K]
  double dT_cap;                     // largest predicted |dT| accepted [K]
  int residual;                      // the networks predict the increment minus dt f(y0)
};

// Mean cv and species h at T (CKCVBS, CKHMS) with the reciprocal constants
// of ck_fun_fast (the species loop of fun_tpart), and the mixture's specific
// internal energy sum_k Y_k (h_k - RU T / W_k).  For the surrogate's decode:
// a few ulp from Thermo's reference-order values, a third of its FP64 work.
template <int KK>
__device__ __forceinline__ double thermo_fast_e(double T, const double* Y, double* cvb) {
  const double Tinv = 1.0 / T;
  const double T2 = T * T, T3 = T * T2, T4 = T2 * T2;
  const double rut = T * c_mech.ru;
  double cv = 0.0, e = 0.0;
#pragma unroll
  for (int k = 0; k < KK; ++k) {
    const double* a = c_mech.a[k][T > c_mech.tmid[k] ? 1 : 0];
    const double cps = a[0] + T * a[1] + T2 * a[2] + T3 * a[3] + T4 * a[4];
    cv = cv + Y[k] * (c_fast.ru_wt[k] * (cps - 1.0));
    const double hs = a[0] + (0.5 * T) * a[1] + (T2 * (1.0 / 3.0)) * a[2] + (0.25 * T3) * a[3] + (0.2 * T4) * a[4];
    const double h = rut * (hs + a[5] * Tinv) * c_fast.wt_inv[k];
    e = e + Y[k] * (h - c_fast.ru_wt[k] * T);
  }
  *cvb = cv;
  return e;
}

// Decode the surrogate output, gate it, and write accepted cells in place.
// Gate: (1) state inside the training envelope, and a predicted |dT| not
// above the cap (igniting cells, where the network's error is largest, go
// to the integrator); (2) element conservation of
// the predicted dY (H, O, N, from the species composition); (3) the
// predicted dT agrees with the temperature that conserves internal energy
// (constant-volume reactor) for the predicted composition.  Accepted cells
// take the energy-consistent temperature.  Rejected cells are appended to
// `list` as base + q (their index in the whole batch) for the BDF integrator.
template <int KK, class Rhs>
__global__ void k_decode_gate(int n, const float* out, const float* out2, int ldo, const float* norm, const float* norm2,
                              double* T, const double* rho, double* Y, const double* dt, GateArgs ga, const int* kncf,
                              int nele, int* list, int base, unsigned* count, double* dT_pred, ChemStats* stats) {
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
  double dTp = (double)out[(size_t)q * ldo + KK] * so[KK] + mo[KK];
  if (out2) {
    // two independently trained networks: predict with their mean, and
    // reject the cell where their temperature increments disagree
    const float* mo2 = norm2 + 2 * NI;
    const float* so2 = norm2 + 2 * NI + NO;
#pragma unroll
    for (int k = 0; k < KK; ++k) dY[k] = 0.5 * (dY[k] + ((double)out2[(size_t)q * ldo + k] * so2[k] + mo2[k]));
    const double dT2 = (double)out2[(size_t)q * ldo + KK] * so2[KK] + mo2[KK];
    if (fabs(dT2 - dTp) > ga.tol_ens_abs + ga.tol_ens_rel * fabs(dTp)) ok = false;
    dTp = 0.5 * (dTp + dT2);
  }
  if (ga.residual) {
    // networks trained on the increment minus the explicit one: add
    // dt f(y0), the reactor right-hand side at the start state
    double z0[KK + 1], f0[KK + 1];
    z0[0] = T0;
#pragma unroll
    for (int k = 0; k < KK; ++k) z0[1 + k] = Y[(size_t)q * KK + k];
    typename Rhs::Terms t0;
    Rhs::tpart(T0, t0);
    Rhs::cpart(rho[q], z0, t0, f0);
#pragma unroll
    for (int k = 0; k < KK; ++k) dY[k] = dY[k] + dt[q] * f0[1 + k];
    dTp = dTp + dt[q] * f0[0];
  }
  if (!(fabs(dTp) <= ga.dT_cap)) ok = false;
  if (dT_pred) dT_pred[q] = dTp;
  // element residuals
  for (int e = 0; e < nele && ok; ++e) {
    double r = 0.0, sc = 0.0;
    for (int k = 0; k < KK; ++k) {
      const double nk = (double)kncf[k * nele + e] * c_fast.wt_inv[k];
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
  double cvb;
  double Y0[KK];
#pragma unroll
  for (int k = 0; k < KK; ++k) Y0[k] = Y[(size_t)q * KK + k];
  const double e0 = thermo_fast_e<KK>(T0, Y0, &cvb);
  double T1 = T0 + dTp;
  if (!(T1 > 200.0 && T1 < 6000.0)) ok = false;
  for (int it = 0; it < 4 && ok; ++it) {
    const double e1 = thermo_fast_e<KK>(T1, Yn, &cvb);
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
    list[slot] = base + q;
  }
}

// The reactor right-hand side dz/dt, z = [T, Y_1..Y_K] (FUN of REACTION_V,
// the right-hand side the BDF kernels call: generated for the mechanism or
// walking its tables), at n states; zdot is n x (KK + 1).
template <int KK, class Rhs>
__global__ void k_reactor_rhs(int n, const double* __restrict__ T, const double* __restrict__ rho,
                              const double* __restrict__ Y, double* __restrict__ zdot) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  double z[KK + 1], f[KK + 1];
  z[0] = T[q];
#pragma unroll
  for (int k = 0; k < KK; ++k) z[1 + k] = Y[(size_t)q * KK + k];
  typename Rhs::Terms t;
  Rhs::tpart(z[0], t);
  Rhs::cpart(rho[q], z, t, f);
#pragma unroll
  for (int c = 0; c <= KK; ++c) zdot[(size_t)q * (KK + 1) + c] = f[c];
}

template <int KK, int MINB, class Rhs>
__global__ void __launch_bounds__(kChemThreads, MINB) k_psr_list(const int* list, const unsigned* count, double* T,
                                                                 const double* rho, double* Y, const double* dt,
                                                                 unsigned* counter, ChemStats* stats) {
  constexpr int N = KK + 1;
  auto load = [&](unsigned w, double& rh, double* z, double& tf) {
    const int q = list[w];
    z[0] = T[q];
#pragma unroll
    for (int l = 0; l < KK; ++l) z[1 + l] = Y[(size_t)q * KK + l];
    rh = rho[q];
    tf = dt[q];
  };
  auto store = [&](unsigned w, const Rc<N>& r) {
    const int q = list[w];
    chem_stats_add<KK>(stats, r.istate, r.nsteps);
    T[q] = r.y[0];
#pragma unroll
    for (int l = 0; l < KK; ++l) Y[(size_t)q * KK + l] = r.y[1 + l];
  };
  rc_drive<KK, Rhs>(*count, counter, load, store);
}

// The three persistent kernels of one register-budget variant with one
// right-hand-side form.
template <int MINB, class Rhs>
constexpr ChemKernelSet chem_set_of() {
  return ChemKernelSet{k_psr_field<9, MINB, Rhs>, k_psr_batch<9, MINB, Rhs>, k_psr_list<9, MINB, Rhs>};
}

}  // namespace

#ifndef IZEM_CHEM_HOST_TEST
#if IZEM_CHEM_UNIT == 1
// This unit (chem_generated.cu): the kernels with the generated right-hand side.
extern const ChemKernelSet kChemGenSets[IZEM_CHEM_VARIANTS] = {
    chem_set_of<8, RhsGenerated>(), chem_set_of<7, RhsGenerated>(), chem_set_of<6, RhsGenerated>(),
    chem_set_of<5, RhsGenerated>(), chem_set_of<4, RhsGenerated>()};
#else
extern const ChemKernelSet kChemGenSets[IZEM_CHEM_VARIANTS];

namespace {

constexpr int kChemMinBlocks[IZEM_CHEM_VARIANTS] = {8, 7, 6, 5, 4};
const ChemKernelSet kChemTabSets[IZEM_CHEM_VARIANTS] = {
    chem_set_of<8, RhsTables<9>>(), chem_set_of<7, RhsTables<9>>(), chem_set_of<6, RhsTables<9>>(),
    chem_set_of<5, RhsTables<9>>(), chem_set_of<4, RhsTables<9>>()};

// Variant of the persistent chemistry kernels in use: 7 blocks of 128
// threads per SM until an autotuning pass (izem_gpu_autotune) times the
// variants on the caller's reactors and keeps the fastest (the same for every
// context of the process).
int g_chem_variant = 1;
// 1 when the uploaded mechanism is the one chem_gen.cuh was generated from
int g_chem_gen = 0;
bool g_chem_gen_allowed = true;

const ChemKernelSet& chem_kernels(int v) { return g_chem_gen ? kChemGenSets[v] : kChemTabSets[v]; }

int chem_grid(int* blocks) {
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, chem_kernels(g_chem_variant).batch, kChemThreads, 0) !=
      cudaSuccess)
    return -1;
  *blocks = sms * (per > 0 ? per : 1);
  return 0;
}

}  // namespace

// ---------------------------------------------------------- host side -------
int chem_set_variant(int v) {
  if (v < 0 || v >= IZEM_CHEM_VARIANTS) return -1;
  g_chem_variant = v;
  return 0;
}
int chem_variant() { return g_chem_variant; }
int chem_generated_rhs() { return g_chem_gen; }
void chem_allow_generated(bool allow) { g_chem_gen_allowed = allow; }
int chem_variant_min_blocks(int v) { return (v >= 0 && v < IZEM_CHEM_VARIANTS) ? kChemMinBlocks[v] : 0; }
int chem_variant_registers(int v) {
  cudaFuncAttributes a{};
  if (v < 0 || v >= IZEM_CHEM_VARIANTS || cudaFuncGetAttributes(&a, chem_kernels(v).batch) != cudaSuccess) return 0;
  return a.numRegs;
}

bool chem_mech_valid(const izem_mech* m) {
  if (!m || m->kk != 9 || m->ii < 0 || m->ii > IZEM_MAXREAC) return false;
  for (int i = 0; i < m->ii; ++i) {
    for (int n = 0; n < MXSP; ++n)
      if (m->nuk[i][n] < -1 || m->nuk[i][n] >= m->kk) return false;
    if (m->rev[i] < 0 || m->rev[i] > 2 || m->fall[i] < 0 || m->fall[i] > 4) return false;
    if (m->fall[i] && (m->kfal[i] < 0 || m->kfal[i] > m->kk)) return false;
    if (m->fall[i] >= 3 && (m->troe[i][1] == 0.0 || m->troe[i][2] == 0.0)) return false;
    if (m->fall[i] == 2 && m->sri[i][2] == 0.0) return false;
    if ((m->rlt[i][0] != 0.0 || m->rlt[i][1] != 0.0) && m->rev[i] != 2) return false;   // RLT needs REV
  }
  return true;
}

cudaError_t chem_upload_mech(const izem_mech* m) {
  cudaError_t e = cudaMemcpyToSymbol(c_mech_dev, m, sizeof(izem_mech));
  if (e != cudaSuccess) return e;
  ChemFast f = chem_fast_constants(*m);
  if ((e = cudaMemcpyToSymbol(c_fast_dev, &f, sizeof(ChemFast))) != cudaSuccess) return e;
  int need = 0;
  for (int i = 0; i < m->ii; ++i) need |= (m->rev[i] == 1);
  g_chem_gen = (g_chem_gen_allowed && chem_gen::matches(*m)) ? 1 : 0;
  return cudaMemcpyToSymbol(c_need_eqk_dev, &need, sizeof(int));
}

cudaError_t chem_launch_field(const ChemField& f, unsigned* d_counter, ChemStats* d_stats, cudaStream_t s, int kk) {
  int blocks = 0;
  if (chem_grid(&blocks)) return cudaErrorUnknown;
  cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  if (kk != 9) return cudaErrorInvalidValue;
  chem_kernels(g_chem_variant).field<<<blocks, kChemThreads, 0, s>>>(f, d_counter, d_stats);
  return cudaGetLastError();
}

cudaError_t chem_launch_batch(int n, double* T, const double* rho, double* Y, const double* dt, int* istate, int* nsteps,
                              unsigned* d_counter, ChemStats* d_stats, cudaStream_t s, int kk) {
  int blocks = 0;
  if (chem_grid(&blocks)) return cudaErrorUnknown;
  cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  if (kk != 9) return cudaErrorInvalidValue;
  chem_kernels(g_chem_variant).batch<<<blocks, kChemThreads, 0, s>>>(n, T, rho, Y, dt, istate, nsteps, d_counter,
                                                                      d_stats);
  return cudaGetLastError();
}

cudaError_t chem_launch_gather(const ChemField& f, double* T, double* rho, double* Y, double* dt, cudaStream_t s) {
  const long long n = (long long)f.wx * f.wy * f.wz;
  k_chem_gather<9><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(f, T, rho, Y, dt);
  return cudaGetLastError();
}

cudaError_t chem_launch_select(int n, const double* T, const double* rho, const double* Y, const double* dt,
                               const ChemSkip& sk, int* list, unsigned* count, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_chem_select<9><<<(n + 127) / 128, 128, 0, s>>>(n, T, rho, Y, dt, sk, list, count);
  return cudaGetLastError();
}

cudaError_t chem_launch_scatter_list(const ChemField& f, int n, const int* list, const unsigned* count,
                                     const double* T, const double* Y, ChemStats* d_stats, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_chem_scatter_list<9><<<(n + 255) / 256, 256, 0, s>>>(f, list, count, T, Y, d_stats);
  return cudaGetLastError();
}

cudaError_t chem_launch_scatter(const ChemField& f, const double* T, const double* Y, ChemStats* d_stats, cudaStream_t s) {
  const long long n = (long long)f.wx * f.wy * f.wz;
  k_chem_scatter<9><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(f, T, Y, d_stats);
  return cudaGetLastError();
}

cudaError_t chem_launch_featurize(int n, const double* T, const double* rho, const double* Y, const double* dt,
                                  const float* d_norm, void* x_bf16, const float* d_norm2, void* x2_bf16,
                                  cudaStream_t s) {
  k_featurize<9><<<(n + 127) / 128, 128, 0, s>>>(n, T, rho, Y, dt, d_norm, (__nv_bfloat16*)x_bf16, d_norm2,
                                                 (__nv_bfloat16*)x2_bf16);
  return cudaGetLastError();
}

cudaError_t chem_launch_decode_gate(int n, const float* out, const float* out2, int ldo, const float* d_norm,
                                    const float* d_norm2, double* T, const double* rho, double* Y, const double* dt,
                                    const double* gate10, const int* d_kncf, int nele, int* list, int base,
                                    unsigned* count, double* dT_pred, ChemStats* stats, int residual,
                                    cudaStream_t s) {
  GateArgs ga{gate10[0], gate10[1], gate10[2], gate10[3], gate10[4],
              gate10[5], gate10[6], gate10[7], gate10[8], gate10[9], residual};
  auto kern = g_chem_gen ? k_decode_gate<9, RhsGenerated> : k_decode_gate<9, RhsTables<9>>;
  kern<<<(n + 127) / 128, 128, 0, s>>>(n, out, out2, ldo, d_norm, d_norm2, T, rho, Y, dt, ga, d_kncf, nele,
                                                   list, base, count, dT_pred, stats);
  return cudaGetLastError();
}

cudaError_t chem_launch_rhs(int n, const double* T, const double* rho, const double* Y, double* zdot, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  auto kern = g_chem_gen ? k_reactor_rhs<9, RhsGenerated> : k_reactor_rhs<9, RhsTables<9>>;
  kern<<<(n + 127) / 128, 128, 0, s>>>(n, T, rho, Y, zdot);
  return cudaGetLastError();
}

cudaError_t chem_launch_list(const int* list, const unsigned* count, double* T, const double* rho, double* Y,
                             const double* dt, unsigned* d_counter, ChemStats* d_stats, cudaStream_t s) {
  int blocks = 0;
  if (chem_grid(&blocks)) return cudaErrorUnknown;
  cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  chem_kernels(g_chem_variant).list<<<blocks, kChemThreads, 0, s>>>(list, count, T, rho, Y, dt, d_counter, d_stats);
  return cudaGetLastError();
}
#endif  // IZEM_CHEM_UNIT
#endif  // IZEM_CHEM_HOST_TEST

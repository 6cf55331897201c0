// Device NASA-7 thermodynamics: the scalar routines of
// module_thermodynamics.f90 (cp_scalar :767-862, ha_scalar :873-978, newton
// :271-508), with the reference's linear extrapolation outside
// [Tpolymin, Tpolymax] and its operation order.
#pragma once
#include "common.cuh"

__device__ __forceinline__ double th_hpoly(const double* a, double t1, double t2, double t3, double t4, double t5) {
  return a[0] * t1 + a[1] * t2 * 0.50 + a[2] * t3 * c_thd.onethird + a[3] * t4 * 0.25 + a[4] * t5 * 0.20 + a[5];
}
__device__ __forceinline__ double th_cppoly(const double* a, double t1, double t2, double t3, double t4) {
  return a[0] + a[1] * t1 + a[2] * t2 + a[3] * t3 + a[4] * t4;
}
__device__ __forceinline__ double th_dcppoly(const double* a, double t1, double t2, double t3) {
  return a[1] + a[2] * t1 * 2.0 + a[3] * t2 * 3.0 + a[4] * t3 * 4.0;
}

// Per-species h (code units) and cp/R-weighted contribution at temperature T
// (code units).  Returns h; writes the cp polynomial value (cp_k/R including
// the linear extrapolation) to *cpk.
__device__ __forceinline__ double th_species(int is, double T, double* cpk) {
  double t1 = T * c_thd.tinf, t2, t3, t4, t5;
  const double tmin = c_thd.tpolymin[is], tmax = c_thd.tpolymax[is];
  const double fac = c_thd.Wc_i[is] * c_thd.tinf_i;
  if (t1 < tmin) {
    const double* a = c_thd.hc[is][0];
    t1 = tmin; t2 = t1 * t1; t3 = t2 * t1; t4 = t3 * t1; t5 = t4 * t1;
    double ha0 = th_hpoly(a, t1, t2, t3, t4, t5);
    double dha0 = th_cppoly(a, t1, t2, t3, t4);
    double dcp0 = th_dcppoly(a, t1, t2, t3);
    double dT = T * c_thd.tinf - tmin;
    *cpk = dcp0 * dT + dha0;
    return fac * (dha0 * dT + ha0);
  }
  t2 = t1 * t1; t3 = t2 * t1; t4 = t3 * t1; t5 = t4 * t1;
  if (t1 < c_thd.tpolylim[is]) {
    const double* a = c_thd.hc[is][0];
    *cpk = th_cppoly(a, t1, t2, t3, t4);
    return fac * th_hpoly(a, t1, t2, t3, t4, t5);
  }
  if (t1 < tmax) {
    const double* a = c_thd.hc[is][1];
    *cpk = th_cppoly(a, t1, t2, t3, t4);
    return fac * th_hpoly(a, t1, t2, t3, t4, t5);
  }
  {
    const double* a = c_thd.hc[is][1];
    t1 = tmax; t2 = t1 * t1; t3 = t2 * t1; t4 = t3 * t1; t5 = t4 * t1;
    double ha0 = th_hpoly(a, t1, t2, t3, t4, t5);
    double dha0 = th_cppoly(a, t1, t2, t3, t4);
    double dcp0 = th_dcppoly(a, t1, t2, t3);
    double dT = T * c_thd.tinf - tmax;
    *cpk = dcp0 * dT + dha0;
    return fac * (dha0 * dT + ha0);
  }
}

// cp_scalar: cp = sum_k Y_k gam2 Wc_i,k cp_k/R
template <int NRV>
__device__ __forceinline__ double th_cp_mix(double T, const double* Y) {
  double cp = 0.0;
#pragma unroll
  for (int is = 0; is < NRV; ++is) {
    double cpk;
    (void)th_species(is, T, &cpk);
    cp = cp + Y[is] * c_thd.gam2 * c_thd.Wc_i[is] * cpk;
  }
  return cp;
}

// cp_scalar and ha_scalar evaluated together at the same temperature
template <int NRV>
__device__ __forceinline__ double th_cp_ha(double T, const double* Y, double* ha) {
  double cp = 0.0;
#pragma unroll
  for (int is = 0; is < NRV; ++is) {
    double cpk;
    ha[is] = th_species(is, T, &cpk);
    cp = cp + Y[is] * c_thd.gam2 * c_thd.Wc_i[is] * cpk;
  }
  return cp;
}

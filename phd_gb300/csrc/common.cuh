// Shared device definitions for the IZEM RHS kernels (sm_103a).
#pragma once
#include <cstdint>
#include "atomics.cuh"
#include <cuda_runtime.h>
#include "../../include/izem_gpu.h"

#define IZEM_NIV 5
#define IZEM_NVMAX (IZEM_NIV + IZEM_NSMAX)

// Block geometry: one block of nx*ny*nz interior points with ng ghost layers
// in the reference's Fortran column-major layout (sx = sy = sz = 1).
struct Geo {
  int n[3];
  int ng;
  int g[3];        // ghosted extents n+2ng
  long long ncell; // ghosted points
  long long nint;  // interior points
  int bnd[6];      // face is a physical (non-periodic) boundary
  int bc[6];
  int ndim;        // 3, or 2 (nz = 1: no z sweep, no z derivatives)
};

__host__ __device__ inline long long gid(const Geo& g, int i, int j, int k) {
  return (long long)(i - 1 + g.ng) + (long long)g.g[0] * ((long long)(j - 1 + g.ng) + (long long)g.g[1] * (long long)(k - 1 + g.ng));
}
__host__ __device__ inline long long fidx(const Geo& g, int i, int j, int k) {
  return (long long)(i - 1) + (long long)g.n[0] * ((long long)(j - 1) + (long long)g.n[1] * (long long)(k - 1));
}

// Species data in code units, broadcast from constant memory.  Pairwise
// constants of the Wilke viscosity rule are precomputed on the host with the
// same IEEE operations the reference evaluates per point.
struct DevThd {
  int nspc;
  double gam2, gam2_i, tinf, tinf_i, onethird;
  double Wc[IZEM_NSMAX], Wc_i[IZEM_NSMAX];
  double tpolymin[IZEM_NSMAX], tpolymax[IZEM_NSMAX], tpolylim[IZEM_NSMAX];
  double hc[IZEM_NSMAX][2][7];
  double cofd[IZEM_NSMAX][IZEM_NSMAX][IZEM_NPOLY];
  double coflam[IZEM_NSMAX][IZEM_NPOLY];
  double cofeta[IZEM_NSMAX][IZEM_NPOLY];
  double wilke_c1[IZEM_NSMAX][IZEM_NSMAX];   // (W_l/W_m)^0.25      [m][l]
  double wilke_c2[IZEM_NSMAX][IZEM_NSMAX];   // 1/sqrt((1+W_m/W_l)*8) [m][l]
  double Kd[IZEM_NSMAX];
  double Kl, Ku;
  // viscous-flux constants (module_viscflux.f90:1717-1719)
  double sqgmr, rvd0, rlam0;
};

// One copy per translation unit (whole-program compilation); each unit that
// uses it uploads the same host structure.
static __constant__ DevThd c_thd;

// Device status word shared by all kernels of a context.
// Newton stopping slots: sub-domain d (0 interior, 1-6 ghost faces, 7-8 the
// Dirichlet planes of the W and E faces) of x-block b is slot d + 10 b; one
// x-block unless the reference's x-decomposition is emulated.
constexpr int kNewtonXBlocksMax = 8;
constexpr int kNewtonSlots = 10 * kNewtonXBlocksMax;

struct DevStatus {
  // per slot max dT^2 (bit pattern of a non-negative double), iterations, stop flag
  unsigned long long maxdf_bits[kNewtonSlots];
  int it[kNewtonSlots];
  int done[kNewtonSlots];
  int neg_pressure;
  int neg_temperature;
  int newton_nan;
  int newton_unconverged;
  int newton_it_max;                 // most iterations any sub-domain used since the host last read it
  unsigned long long dtc_bits;       // timestep: max (|u|+c)/dx (bit pattern)
  // timestep, Fourier criteria (bit patterns of positive doubles): per
  // species max of D_k and min of delta^2 / D_k, and min of delta^2 rho cp / lambda
  unsigned long long fo_dmax_bits[IZEM_NSMAX];
  unsigned long long fo_dmin_bits[IZEM_NSMAX];
  unsigned long long fo_ctmin_bits;
  int timeout;
  int chem_fail;
};


// Seeded fluctuation of the jet inflow: uniform in [-1, 1) from a hash
// (splitmix64 finaliser, Steele, Lea and Flood 2014) of the seed, the face
// point (j, k), the velocity component and the time interval n (the stage
// time in units of a fixed quantum, rounded down: runs whose times differ
// in the last bits draw the same values).
__host__ __device__ inline double jet_noise(unsigned long long seed, int j, int k, int comp, long long n) {
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

// Host interface of the batched chemistry kernels (chem.cu).
#pragma once
#include <cuda_runtime.h>
#include "../../include/izem_gpu.h"

// One chemistry half-step over the reference's interior window of a field.
struct ChemField {
  double* v;        // ghosted conserved variables (device)
  double* T;        // ghosted temperature, code units (device)
  double* dT_out;   // optional: per-window-cell temperature increment [K]
  long long ncell;
  int gx, gy, ng;
  int ix, iy, iz;   // first cell of the window (1-based interior index)
  int wx, wy, wz;   // window extents
  double t_ref, tref_i, rho_cgs, dt_phys;
};

struct ChemStats {
  int failed;                      // cells whose final ISTATE <= -2
  int max_steps;                   // largest BDF step count of a cell
  unsigned long long total_steps;  // summed BDF steps
  unsigned long long dtmax_bits;   // max |dT| [K] as a double bit pattern
};

cudaError_t chem_upload_mech(const izem_mech* m);
// true when the kernels can evaluate m: 9 species, at most IZEM_MAXREAC
// reactions, species indices in range, known reverse and fall-off kinds, a
// collider in range, and nonzero Troe and SRI temperatures where the rate
// divides by them (the two device forms would otherwise disagree: one
// divides by zero, the other multiplies by a zero reciprocal)
bool chem_mech_valid(const izem_mech* m);
// Register-budget variants of the persistent chemistry kernels (128 threads
// per block; variant v keeps at least 8 - v blocks resident per SM), chosen
// by the autotuner.  chem_set_variant returns -1 for an unknown variant.
#define IZEM_CHEM_VARIANTS 5
int chem_set_variant(int v);
int chem_variant();
// 1 when the kernels use the right-hand side generated for the uploaded
// mechanism (chem_gen.cuh), 0 when they walk its tables
int chem_generated_rhs();
// false: walk the tables even for the shipped mechanism (from the next upload)
void chem_allow_generated(bool allow);
int chem_variant_min_blocks(int v);
int chem_variant_registers(int v);
cudaError_t chem_launch_field(const ChemField& f, unsigned* d_counter, ChemStats* d_stats, cudaStream_t s, int kk);
cudaError_t chem_launch_batch(int n, double* T, const double* rho, double* Y, const double* dt, int* istate,
                              int* nsteps, unsigned* d_counter, ChemStats* d_stats, cudaStream_t s, int kk);

// chemistry window <-> independent reactors (physical units)
cudaError_t chem_launch_gather(const ChemField& f, double* T, double* rho, double* Y, double* dt, cudaStream_t s);
cudaError_t chem_launch_scatter(const ChemField& f, const double* T, const double* Y, ChemStats* d_stats, cudaStream_t s);
// dvodesimp (module_reaction.f90:173-251): the pure-stream compositions of
// H2 and N2 and their species indices (0-based)
struct ChemSkip {
  double yf_h2, yf_n2, yo_h2, yo_n2;
  int ih2, in2;
};
// gathered reactors that the skip test sends to the integrator -> list, count
cudaError_t chem_launch_select(int n, const double* T, const double* rho, const double* Y, const double* dt,
                               const ChemSkip& sk, int* list, unsigned* count, cudaStream_t s);
// listed reactors -> window (the skip branch's clipping); n bounds *count
cudaError_t chem_launch_scatter_list(const ChemField& f, int n, const int* list, const unsigned* count,
                                     const double* T, const double* Y, ChemStats* d_stats, cudaStream_t s);

// learned-surrogate support (chem.cu)
// inputs of one network, or of both networks of an ensemble (d_norm2 and
// x2_bf16 null for one); rows of 16 BF16 values, 16-byte aligned
cudaError_t chem_launch_featurize(int n, const double* T, const double* rho, const double* Y, const double* dt,
                                  const float* d_norm, void* x_bf16, const float* d_norm2, void* x2_bf16,
                                  cudaStream_t s);
cudaError_t chem_launch_decode_gate(int n, const float* out, const float* out2, int ldo, const float* d_norm,
                                    const float* d_norm2, double* T, const double* rho, double* Y, const double* dt,
                                    const double* gate10, const int* d_kncf, int nele, int* list, int base,
                                    unsigned* count, double* dT_pred, ChemStats* stats, int residual,
                                    cudaStream_t s);
// the reactor right-hand side dz/dt (z = [T, Y]) at n states: zdot n x 10
cudaError_t chem_launch_rhs(int n, const double* T, const double* rho, const double* Y, double* zdot, cudaStream_t s);
cudaError_t chem_launch_list(const int* list, const unsigned* count, double* T, const double* rho, double* Y,
                             const double* dt, unsigned* d_counter, ChemStats* d_stats, cudaStream_t s);

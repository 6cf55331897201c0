// Host-side context of the IZEM GPU library (one per block / per process).
#pragma once
#include <string>
#include <vector>
#include <utility>
#include <cuda_runtime.h>
#include "common.cuh"

struct izem_ctx {
  izem_cfg cfg;
  izem_thd thd;
  izem_adi adi;
  DevThd devthd;
  Geo g;
  int nv = 0;
  cudaStream_t stream = nullptr;
  // device state (reference layout) and scratch
  double *v = nullptr, *T = nullptr, *W_i = nullptr, *cp = nullptr, *ha = nullptr;
  double *v0 = nullptr, *f = nullptr, *prim = nullptr, *Xa = nullptr, *fhat = nullptr;
  double *fd = nullptr, *tau = nullptr, *qv = nullptr, *d_dt = nullptr;
  double* dxi[3] = {nullptr, nullptr, nullptr};
  uint8_t* sensor = nullptr;
  DevStatus* d_status = nullptr;
  DevStatus* h_status = nullptr;
  double* h_dt = nullptr;
  std::vector<double*> allocs;
  bool grid_set = false;
  // CUDA graphs captured once and replayed: one RK3 step, the primitives
  // update, the initial-condition closure and the tail of a chemistry half
  // step.  Their Newton solves are conditional WHILE nodes.
  enum { GR_RK3, GR_PRIM, GR_IC, GR_CHEM_AFTER, GR_N };
  cudaGraph_t graph[GR_N] = {};
  cudaGraphExec_t graph_exec[GR_N] = {};
  bool capturing = false;
  cudaStream_t side = nullptr;            // captures the bodies of conditional nodes
  int* h_done = nullptr;                  // pinned: stop flags read by direct-launch Newton loops
  int newton_it_max = 0;                  // most Newton iterations of any sub-domain since the last izem_gpu_newton_stats reset
  // timing
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  bool kt_enabled = false;
  std::vector<std::string> kt_names;
  std::vector<int> kt_launches;
  std::vector<double> kt_ms;
  std::vector<std::vector<std::pair<cudaEvent_t, cudaEvent_t>>> kt_pending;
  bool have_eg = false;   // EGLIB linking data uploaded (izem_gpu_set_eglib)
  // threads per block chosen by izem_gpu_autotune (face fluxes, viscous point kernel)
  int tb_euler = 128, tb_visc = 128;
  // sensor x-blocks (izem_gpu_set_sensor_xblocks): block size in x (nx for
  // one block) and the block-edge faces as seen by the right block
  int sensor_bx = 0;
  int newton_bx = 0;   // x-block size of the Newton stopping test (nx: one block)
  int nsm = 0;         // SMs of the context's device (the host-transfer kernel's grid)
  int sensor_type = 0;          // IZEM_SENSOR_ADAMS_SHARIFF or IZEM_SENSOR_DUCROS
  double ducros_treduc = 0.2;   // DUCROS_TREDUC
  double* fhat_edge = nullptr;
  long long nedge = 0;
  // chemistry
  bool have_mech = false;
  izem_mech mech;
  unsigned* d_counter = nullptr;
  void* d_chem_stats = nullptr;   // ChemStats
  void* h_chem_stats = nullptr;
  // learned surrogate for chemistry mode IZEM_CHEM_MLP
  izem_mlp* sur_m = nullptr;
  izem_mlp* sur_m2 = nullptr;
  double sur_gate[10] = {};
  std::vector<int> sur_kncf;
  int sur_nele = 0;
  long long sur_cap = 0;                  // reactor buffers for the window
  double *b_T = nullptr, *b_rho = nullptr, *b_Y = nullptr, *b_dt = nullptr;
  int sur_stats[3] = {};                  // fallback cells, max BDF steps, failed
  float sur_ms[2] = {};                   // total, network
  long long sur_cells = 0;
  // dvodesimp skip test for chemistry mode IZEM_CHEM_BDF (izem_gpu_set_chem_skip)
  bool skip_on = false;
  double skip_y[4] = {};                  // fuel H2, fuel N2, oxidiser H2, oxidiser N2
  int skip_ih2 = 0, skip_in2 = 0;
  int* b_list = nullptr;                  // selected reactors (sur_cap entries)
  unsigned* d_list_count = nullptr;
  long long list_cap = 0;
  // jet faces (izem_gpu_set_coords): interior y, z coordinates and the
  // constants of bc_inflowjet / bc_nscbc_out
  bool have_coords = false;
  double *d_y = nullptr, *d_z = nullptr;
  JetArgs jet{};
  izem_jet jet_par{};                     // the jet faces' parameters (izem_gpu_set_jet)
  // LES closure (izem_gpu_set_les)
  bool les_on = false;
  double les_cs2 = 0.0, les_sc_sgs_i = 0.0, les_pr_sgs_i = 0.0, les_pw = 0.0;
  double* les = nullptr;                  // 4 ghosted components (W_i gradient, criterion)
  double les_sc_sgs = 1.0;                // SC_SGS
  double* mu_sgs = nullptr;               // fitted-transport LES: mu_SGS for the Fourier time step (ghosted)
  int newton_warn = 0;
  std::string err;
};

int ctx_alloc(izem_ctx* c);
int ctx_fail(izem_ctx* c, int code, const char* what, cudaError_t e);

// C-ABI context of the GB300 IZEM RHS library: device-resident state, kernel
// sequencing of one SSP-RK3 step, CUDA-graph capture, timing and status.
//
// Reference sequencing: rk3 (module_solver.f90:694-856) calls the shock
// sensor, euler_LLF_x/y/z, viscflux_xyz, the stage update, then
// upd_prim_var_domain, comm_cons, upd_boundaries and upd_prim_var_ghost.
#include <cstdio>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>
#include <algorithm>
#include <cuda_runtime.h>

#include "common.cuh"
#include "thermo.cuh"
#include "kernels_euler.cuh"
#include "kernels_visc.cuh"
#include "kernels_eglib.cuh"
#include "kernels_state.cuh"
#include "izem_ctx.h"
#include "chem.h"



namespace {

constexpr int kThreads = 128;
constexpr int kNewtonChunk = 4;    // direct-launch Newton: iterations between two host reads of the stop flags

unsigned grid_for(long long n, int threads = kThreads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

// ------------------------------------------------------------ helpers -------
int ctx_fail(izem_ctx* c, int code, const char* what, cudaError_t e) {
  char buf[512];
  if (e != cudaSuccess) std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  else std::snprintf(buf, sizeof(buf), "%s", what);
  c->err = buf;
  return code;
}

#define CK(call)                                                        \
  do {                                                                  \
    cudaError_t e_ = (call);                                            \
    if (e_ != cudaSuccess) return ctx_fail(c, IZEM_ERR_CUDA, #call, e_); \
  } while (0)

int kt_id(izem_ctx* c, const char* name) {
  for (size_t q = 0; q < c->kt_names.size(); ++q)
    if (c->kt_names[q] == name) return (int)q;
  c->kt_names.push_back(name);
  c->kt_launches.push_back(0);
  c->kt_ms.push_back(0.0);
  c->kt_pending.push_back({});
  return (int)c->kt_names.size() - 1;
}

// Launch wrapper: with kernel timing on, bracket the launch by events on the
// context stream and keep the pair for later accumulation.
template <typename F>
int launch(izem_ctx* c, const char* name, F&& fn) {
  if (c->kt_enabled && !c->capturing) {
    int id = kt_id(c, name);
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaEventRecord(a, c->stream));
    fn();
    CK(cudaGetLastError());
    CK(cudaEventRecord(b, c->stream));
    c->kt_pending[id].push_back({a, b});
    return IZEM_OK;
  }
  fn();
  CK(cudaGetLastError());
  return IZEM_OK;
}

int kt_collect(izem_ctx* c) {
  for (size_t q = 0; q < c->kt_names.size(); ++q) {
    for (auto& pr : c->kt_pending[q]) {
      CK(cudaEventSynchronize(pr.second));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, pr.first, pr.second));
      c->kt_ms[q] += ms;
      c->kt_launches[q] += 1;
      cudaEventDestroy(pr.first);
      cudaEventDestroy(pr.second);
    }
    c->kt_pending[q].clear();
  }
  return IZEM_OK;
}

int read_status(izem_ctx* c) {
  CK(cudaMemcpyAsync(c->h_status, c->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  DevStatus& s = *c->h_status;
  int rc = IZEM_OK;
  if (s.neg_pressure) rc = ctx_fail(c, IZEM_ERR_NEG_PRESSURE, "negative pressure in the convective flux pre-pass", cudaSuccess);
  else if (s.neg_temperature) rc = ctx_fail(c, IZEM_ERR_NEG_TEMPERATURE, "negative temperature in the Newton solve", cudaSuccess);
  else if (s.newton_nan) rc = ctx_fail(c, IZEM_ERR_NAN, "Newton temperature correction is NaN", cudaSuccess);
  else if (s.timeout) rc = ctx_fail(c, IZEM_ERR_TIMEOUT, "bounded device wait gave up", cudaSuccess);
  else if (s.chem_fail) rc = ctx_fail(c, IZEM_ERR_CHEM, "stiff chemistry integration failed on some cells", cudaSuccess);
  c->newton_warn += s.newton_unconverged;
  c->newton_it_max = std::max(c->newton_it_max, s.newton_it_max);
  if (s.newton_it_max) CK(cudaMemsetAsync(&c->d_status->newton_it_max, 0, sizeof(int), c->stream));
  if (rc != IZEM_OK || s.newton_unconverged) {
    // clear sticky flags so that the context stays usable
    CK(cudaMemsetAsync(c->d_status, 0, sizeof(DevStatus), c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  return rc;
}

// Runs the work that `enqueue` launches.  With kernel timing off it is
// captured once into graph slot `slot` and the graph is replayed on later
// calls; with kernel timing on the launches go out directly, each bracketed
// by events.  Both forms launch the same kernels with the same arguments.
template <class F>
int run_graph(izem_ctx* c, int slot, F enqueue) {
  if (c->kt_enabled) return enqueue();
  if (!c->graph_exec[slot]) {
    c->capturing = true;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue();
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    c->capturing = false;
    if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
    if (e != cudaSuccess) return ctx_fail(c, IZEM_ERR_CUDA, "cudaStreamEndCapture", e);
    c->graph[slot] = graph;
    e = cudaGraphInstantiate(&c->graph_exec[slot], graph, 0);
    if (e != cudaSuccess) {
      c->graph_exec[slot] = nullptr;
      cudaGraphDestroy(graph);
      c->graph[slot] = nullptr;
      return ctx_fail(c, IZEM_ERR_CUDA, "cudaGraphInstantiate", e);
    }
  }
  CK(cudaGraphLaunch(c->graph_exec[slot], c->stream));
  return IZEM_OK;
}

// The jet faces' constants in code units, as bc_inflowjet and bc_nscbc_out
// divide them, from the context's parameters.
void jet_args(izem_ctx* c) {
  const izem_adi& a = c->adi;
  const izem_jet& p = c->jet_par;
  JetArgs& j = c->jet;
  j.hbuse = p.width / a.l_ref;
  j.tmaxy = p.ramp / a.time_ref;
  j.u2 = p.u_co / a.u_ref;
  j.T1 = p.T_jet / a.t_ref;
  j.T2 = p.T_co / a.t_ref;
  j.P1 = p.p_jet / a.p_ref;
  j.P2 = p.p_co / a.p_ref;
  j.pinf = p.p_far / a.p_ref;
  j.u1 = p.u_jet / a.u_ref;
  j.ya1 = p.y_fuel;
  j.turb = p.turb;
  j.tq_i = a.time_ref / 1.0e-9;   // fluctuations drawn anew every 1 ns
  j.seed = p.seed;
  j.planar = p.planar;
}

// Drops every captured graph; the next call of each entry point captures
// again (after a change of launch shapes, kernel variants or options).
void drop_graphs(izem_ctx* c) {
  for (int q = 0; q < izem_ctx::GR_N; ++q) {
    if (c->graph_exec[q]) cudaGraphExecDestroy(c->graph_exec[q]);
    if (c->graph[q]) cudaGraphDestroy(c->graph[q]);
    c->graph_exec[q] = nullptr;
    c->graph[q] = nullptr;
  }
}

// ------------------------------------------------------- stage building -----
// prim_inv_var's Newton loop (module_thermodynamics.f90:79-186) on one kind
// of sub-domain; every sub-domain stops on its own test, after at most itmax
// iterations.  ghost: 0 the interior (sub-domain 0), 1 the ghost slabs (1-6),
// 2 the Dirichlet planes of jet faces (7-8).
//
// Captured into a graph, the loop is a conditional WHILE node whose body is
// one iteration and the stopping test; the test launch clears the condition
// when every sub-domain has stopped, so the graph runs exactly the
// iterations the reference runs.  Launched directly (kernel timing), the
// host runs the iterations in chunks and reads the stop flags between them;
// iterations after a sub-domain has stopped leave it untouched, so both
// forms give the same bits.
template <int NRV>
int enq_newton(izem_ctx* c, int ghost, double eps, int itmax, int check_negT) {
  const Geo& g = c->g;
  const int d0 = ghost == 2 ? 7 : (ghost ? 1 : 0), d1 = ghost == 2 ? 8 : (ghost ? 6 : 0);
  const long long n = ghost == 2 ? 2LL * g.n[1] * g.n[2] : (ghost ? slab_count(g) - g.nint : g.nint);
  const char* iname = ghost == 2 ? "newton_iter_plane" : (ghost ? "newton_iter_ghost" : "newton_iter");
  int rc;
  const int nxb = g.n[0] / c->newton_bx, bx = c->newton_bx;
  if ((rc = launch(c, "newton_reset", [&] { k_newton_reset<<<1, 16 * kNewtonXBlocksMax, 0, c->stream>>>(c->d_status, d0, d1, nxb); })))
    return rc;
  auto iterate = [&](cudaGraphConditionalHandle cond, int use_cond) -> int {
    int r = launch(c, iname, [&] {
      k_newton_iter<NRV><<<grid_for(n), kThreads, 0, c->stream>>>(g, ghost, c->v, c->T, c->cp, c->ha, c->d_status, check_negT,
                                                                  bx);
    });
    if (r) return r;
    return launch(c, "newton_check", [&] {
      k_newton_check<<<1, 32, 0, c->stream>>>(c->d_status, d0, d1, nxb, eps, itmax, cond, use_cond);
    });
  };
  if (c->capturing) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t graph = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    CK(cudaStreamGetCaptureInfo(c->stream, &cs, nullptr, &graph, &deps, nullptr, &ndeps));
    cudaGraphConditionalHandle cond;
    // the condition is 1 at every launch of the graph: the loop body runs at
    // least once, as the reference's first iteration always does
    CK(cudaGraphConditionalHandleCreate(&cond, graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &np));
    CK(cudaStreamUpdateCaptureDependencies(c->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaStream_t main = c->stream;
    cudaError_t e = cudaStreamBeginCaptureToGraph(c->side, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return ctx_fail(c, IZEM_ERR_CUDA, "cudaStreamBeginCaptureToGraph", e);
    c->stream = c->side;   // the body's launches go to the side stream
    rc = iterate(cond, 1);
    c->stream = main;
    cudaGraph_t body = nullptr;
    e = cudaStreamEndCapture(c->side, &body);
    if (rc) return rc;
    if (e != cudaSuccess) return ctx_fail(c, IZEM_ERR_CUDA, "cudaStreamEndCapture (Newton loop body)", e);
    return IZEM_OK;
  }
  for (int it = 0; it < itmax; it += kNewtonChunk) {
    for (int q = 0; q < kNewtonChunk && it + q < itmax; ++q)
      if ((rc = iterate(0, 0))) return rc;
    CK(cudaMemcpyAsync(c->h_done, c->d_status->done, kNewtonSlots * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    bool all = true;
    for (int b = 0; b < nxb; ++b)
      for (int d = d0; d <= d1; ++d) all = all && c->h_done[d + 10 * b] != 0;
    if (all) break;
  }
  return IZEM_OK;
}

template <int NRV>
int enq_prim(izem_ctx* c) {
  const Geo& g = c->g;
  long long n = slab_count(g);
  return launch(c, "prim", [&] {
    k_prim<NRV><<<grid_for(n), kThreads, 0, c->stream>>>(g, c->v, c->T, c->W_i, c->cp, c->ha, c->prim,
                                                          c->cfg.vis ? c->Xa : nullptr, c->d_status);
  });
}

template <int NRV>
int enq_euler(izem_ctx* c, int d) {
  const Geo& g = c->g;
  constexpr int NV = IZEM_NIV + NRV;
  long long nf = (long long)(g.n[0] + (d == 0)) * (g.n[1] + (d == 1)) * (g.n[2] + (d == 2));
  int rc;
  const char* names[3] = {"euler_face_x", "euler_face_y", "euler_face_z"};
#define IZEM_FACE(DD, NGV)                                                                                         \
  k_euler_face<NRV, DD, NGV><<<grid_for(nf, c->tb_euler), c->tb_euler, 0, c->stream>>>(                                \
      g, c->cfg.weno_avg, c->cfg.weno5_linear_fix, c->v, c->prim, c->sensor, c->fhat, nf, c->sensor_bx, 0)
  rc = launch(c, names[d], [&] {
    if (g.ng == 4) {   // WENO7
      if (d == 0) IZEM_FACE(0, 4);
      if (d == 1) IZEM_FACE(1, 4);
      if (d == 2) IZEM_FACE(2, 4);
    } else {
      if (d == 0) IZEM_FACE(0, 3);
      if (d == 1) IZEM_FACE(1, 3);
      if (d == 2) IZEM_FACE(2, 3);
    }
  });
#undef IZEM_FACE
  if (rc) return rc;
  if (d == 0 && c->sensor_bx < g.n[0]) {   // block-edge faces as seen by the right block
    rc = launch(c, "euler_face_edge", [&] {
#define IZEM_EDGE(NGV)                                                                                            \
  k_euler_face<NRV, 0, NGV><<<grid_for(c->nedge, c->tb_euler), c->tb_euler, 0, c->stream>>>(                      \
      g, c->cfg.weno_avg, c->cfg.weno5_linear_fix, c->v, c->prim, c->sensor, c->fhat_edge, c->nedge, c->sensor_bx, 1)
      if (g.ng == 4) IZEM_EDGE(4);
      else IZEM_EDGE(3);
#undef IZEM_EDGE
    });
  }
  if (rc) return rc;
  return launch(c, "flux_diff", [&] {
    const int bx = c->sensor_bx;
    if (d == 0) k_flux_diff<0><<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, NV, c->fhat, nf, c->dxi[0], c->f, 0, bx, c->fhat_edge, c->nedge);
    if (d == 1) k_flux_diff<1><<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, NV, c->fhat, nf, c->dxi[1], c->f, 1, bx, c->fhat_edge, c->nedge);
    if (d == 2) k_flux_diff<2><<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, NV, c->fhat, nf, c->dxi[2], c->f, 1, bx, c->fhat_edge, c->nedge);
  });
}

template <int NRV>
int enq_visc(izem_ctx* c) {
  const Geo& g = c->g;
  Metrics mt;
  for (int d = 0; d < 3; ++d) mt.dxi[d] = c->dxi[d];
  const bool eg = c->cfg.eglib != 0;
  const int nderiv = (eg ? 15 : 12) + 3 * NRV;
  int rc;
  if ((rc = launch(c, "visc_grad", [&] { k_grad<NRV><<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, mt, c->prim, c->T, c->Xa, c->fd); })))
    return rc;
  if (eg && (rc = launch(c, "visc_grad_p", [&] { k_grad_p<NRV><<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, mt, c->prim, c->fd); })))
    return rc;
  const bool les = c->les_on;
  if (les && (rc = launch(c, "les_prep", [&] {
                // the criterion of shock_det_slv under EGLIB, of shock_det_ducros_slv with the fitted transport
                k_les_prep<<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, mt, c->v, c->T, c->W_i, c->les_pw, c->les,
                                                                         c->prim, eg ? 0 : 1);
              })))
    return rc;
  long long ns = slab_count(g) - g.nint;
  if ((rc = launch(c, "visc_wrap", [&] { k_wrap_periodic<<<grid_for(ns), kThreads, 0, c->stream>>>(g, nderiv, c->fd); })))
    return rc;
  if (les && (rc = launch(c, "les_wrap", [&] { k_wrap_periodic<<<grid_for(ns), kThreads, 0, c->stream>>>(g, 4, c->les); })))
    return rc;
  SgsArgs sa{};
  if (les) {
    sa.les = c->les;
    sa.cp = c->cp;
    for (int d = 0; d < 3; ++d) sa.dxi[d] = c->dxi[d];
    sa.cs2 = c->les_cs2;
    sa.sc = c->adi.sc;
    sa.sc_sgs_i = c->les_sc_sgs_i;
    sa.pr_sgs_i = c->les_pr_sgs_i;
    sa.pr = c->adi.pr;
    sa.mu_sgs = c->mu_sgs;
  }
  if (les && eg) {
    const long long ns_all = slab_count(g);
    if ((rc = launch(c, "visc_point_eg", [&] {
           k_visc_point_eg<NRV, true><<<grid_for(ns_all, c->tb_visc), c->tb_visc, 0, c->stream>>>(
               g, c->v, c->T, c->W_i, c->ha, c->Xa, c->prim, c->fd, c->tau, c->qv, sa);
         })))
      return rc;
  } else if (les) {
    if ((rc = launch(c, "visc_point", [&] {
           k_visc_point<NRV, true><<<grid_for(slab_count(g), c->tb_visc), c->tb_visc, 0, c->stream>>>(
               g, c->v, c->T, c->W_i, c->ha, c->Xa, c->fd, c->tau, c->qv, sa);
         })))
      return rc;
  } else if (eg) {
    const long long ns_all = slab_count(g);
    if ((rc = launch(c, "visc_point_eg", [&] {
           k_visc_point_eg<NRV><<<grid_for(ns_all, c->tb_visc), c->tb_visc, 0, c->stream>>>(g, c->v, c->T, c->W_i, c->ha, c->Xa,
                                                                                         c->prim, c->fd, c->tau, c->qv);
         })))
      return rc;
  } else if ((rc = launch(c, "visc_point", [&] {
         k_visc_point<NRV><<<grid_for(slab_count(g), c->tb_visc), c->tb_visc, 0, c->stream>>>(g, c->v, c->T, c->W_i, c->ha, c->Xa, c->fd, c->tau, c->qv);
       })))
    return rc;
  return launch(c, "visc_div", [&] { k_visc_div<NRV><<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, mt, c->tau, c->qv, c->fd, c->f); });
}

// NR_boundaries (module_BCs.f90:185-212): bc_noreflectionweno on every
// non-reflecting face, W to F, after the viscous fluxes (module_solver.f90:824)
template <int NRV>
int enq_nr(izem_ctx* c) {
  const Geo& g = c->g;
  int rc = IZEM_OK;
  for (int f = 0; f < 2 * g.ndim && !rc; ++f) {
    if (g.bc[f] != IZEM_BC_NOREFLECTION) continue;
    const int d = f >> 1, hi = f & 1;
    const long long np = (long long)(d == 0 ? g.n[1] : g.n[0]) * (d == 2 ? g.n[1] : g.n[2]);
    rc = launch(c, "bc_nr", [&] {
#define IZEM_NR(DD, NGV)                                                                                           \
  k_bc_nr<NRV, DD, NGV><<<grid_for(np), kThreads, 0, c->stream>>>(g, hi, c->v, c->T, c->W_i, c->cp, c->ha, c->dxi[DD], c->f)
      if (g.ng == 4) {
        if (d == 0) IZEM_NR(0, 4);
        if (d == 1) IZEM_NR(1, 4);
        if (d == 2) IZEM_NR(2, 4);
      } else {
        if (d == 0) IZEM_NR(0, 3);
        if (d == 1) IZEM_NR(1, 3);
        if (d == 2) IZEM_NR(2, 3);
      }
#undef IZEM_NR
    });
  }
  return rc;
}

static bool jet_face(int bc) { return bc == IZEM_BC_INFLOWJET || bc == IZEM_BC_NSCBC_OUT; }

// comm_cons, upd_boundaries, upd_prim_var_ghost (module_BCs.f90:41-296):
// the ghost closure after the interior changed.  The jet faces read the
// step and time from device memory: tdt[0] = dt, tdt[1] = time0, and the
// time they are given is time0 + tk dt.
template <int NRV>
int enq_boundaries(izem_ctx* c, const double* tdt, double tk) {
  const Geo& g = c->g;
  int rc;
  long long ns = slab_count(g) - g.nint;
  const bool jet = jet_face(g.bc[0]) || jet_face(g.bc[1]);
  if (!jet) {
    if ((rc = launch(c, "halo", [&] { k_halo<NRV><<<grid_for(ns), kThreads, 0, c->stream>>>(g, 0, c->cfg.forcesum, c->v, c->W_i); })))
      return rc;
    return enq_newton<NRV>(c, 1, 1.0e-5, 200, 1);
  }
  // faces in the reference's order: periodic copies first (comm_cons), then
  // W and E (the jet faces, closed on their boundary planes), then the
  // extrapolated faces
  int per = 0, ext = 0, dir = 0;
  for (int f = 0; f < 6; ++f) {
    if (g.bc[f] == IZEM_BC_PERIODIC) per |= 1 << f;
    else if (g.bc[f] == IZEM_BC_EXTRAPOLATION || g.bc[f] == IZEM_BC_NOREFLECTION) ext |= 1 << f;
    else dir |= 1 << f;
  }
  JetArgs ja = c->jet;
  ja.tdt = tdt;
  ja.tk = tk;
  const long long np = (long long)g.n[1] * g.n[2];
  if (per && (rc = launch(c, "halo", [&] { k_halo<NRV><<<grid_for(ns), kThreads, 0, c->stream>>>(g, 0, c->cfg.forcesum, c->v, c->W_i, per); })))
    return rc;
  if (g.bc[0] == IZEM_BC_INFLOWJET &&
      (rc = launch(c, "bc_inflowjet", [&] { k_bc_inflowjet<NRV><<<grid_for(np), kThreads, 0, c->stream>>>(g, ja, c->v); })))
    return rc;
  if (g.bc[1] == IZEM_BC_NSCBC_OUT && (rc = launch(c, "bc_nscbc_out", [&] {
                                         k_bc_nscbc_out<NRV><<<grid_for(np), kThreads, 0, c->stream>>>(g, ja, c->T, c->W_i, c->cp, c->v);
                                       })))
    return rc;
  if ((rc = launch(c, "dirichlet_prep", [&] {
         k_dirichlet_prep<NRV><<<grid_for(2 * np), kThreads, 0, c->stream>>>(g, c->cfg.forcesum, c->v, c->W_i);
       })))
    return rc;
  if ((rc = enq_newton<NRV>(c, 2, 1.0e-5, 200, 1))) return rc;
  if (ext && (rc = launch(c, "halo", [&] { k_halo<NRV><<<grid_for(ns), kThreads, 0, c->stream>>>(g, 0, c->cfg.forcesum, c->v, c->W_i, ext); })))
    return rc;
  if ((rc = launch(c, "halo", [&] { k_halo<NRV><<<grid_for(ns), kThreads, 0, c->stream>>>(g, 2, c->cfg.forcesum, c->v, c->W_i, dir); })))
    return rc;
  return enq_newton<NRV>(c, 1, 1.0e-5, 200, 1);
}

// upd_prim_var_domain's Newton, then the ghost closure (module_solver.f90:
// 840-847).  stage: the RK stage whose time goes to the jet faces (timek =
// time0 + dt tk3(stage)), -1 for time 0 and dt 0.
template <int NRV>
int enq_update_primitives_after(izem_ctx* c, int stage = -1) {
  int rc;
  if ((rc = enq_newton<NRV>(c, 0, 1.0e-5, 200, 1))) return rc;
  const double tk3[3] = {0.0, 0.5, 1.0};
  return enq_boundaries<NRV>(c, stage >= 0 ? c->d_dt : c->d_dt + 2, stage >= 0 ? tk3[stage] : 0.0);
}

// The stage's shock sensor (module_solver.f90:758-766): Adams-Shariff on the
// conserved state, or Ducros on the velocity gradients of the primitives
// (which it then leaves computed).
template <int NRV>
int enq_sensor_prim(izem_ctx* c) {
  const Geo& g = c->g;
  int rc;
  if (c->sensor_type == IZEM_SENSOR_DUCROS) {
    if ((rc = enq_prim<NRV>(c))) return rc;
    Metrics mt;
    for (int d = 0; d < 3; ++d) mt.dxi[d] = c->dxi[d];
    return launch(c, "sensor", [&] {
      k_sensor_ducros<<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, mt, c->prim, c->ducros_treduc, c->sensor);
    });
  }
  if ((rc = launch(c, "sensor", [&] { k_sensor<<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, c->cfg.max_rel_weight, c->v, c->T, c->W_i, c->sensor, c->sensor_bx); })))
    return rc;
  return enq_prim<NRV>(c);
}

template <int NRV>
int enq_stage(izem_ctx* c, int stage) {
  const Geo& g = c->g;
  int rc;
  if ((rc = enq_sensor_prim<NRV>(c))) return rc;
  for (int d = 0; d < c->cfg.ndim; ++d)   // euler_LLF_z only in 3-D (module_solver.f90:769-774)
    if ((rc = enq_euler<NRV>(c, d))) return rc;
  if (c->cfg.vis)
    if ((rc = enq_visc<NRV>(c))) return rc;
  if ((rc = enq_nr<NRV>(c))) return rc;
  if ((rc = launch(c, "rk_update", [&] {
         k_rk_update<NRV><<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, stage, c->cfg.forcesum, c->d_dt, c->v, c->v0, c->f, c->W_i);
       })))
    return rc;
  return enq_update_primitives_after<NRV>(c, stage);
}

// ------------------------------------------------------ NRV dispatch --------
#define IZEM_DISPATCH(c, FN, ...)                          \
  ((c)->cfg.nrv == 2 ? FN<2>(__VA_ARGS__)                  \
   : (c)->cfg.nrv == 9 ? FN<9>(__VA_ARGS__)                \
   : ctx_fail((c), IZEM_ERR_ARG, "nrv not compiled", cudaSuccess))

template <int NRV>
int do_rk3_enqueue(izem_ctx* c) {
  for (int s = 0; s < 3; ++s) {
    int rc = enq_stage<NRV>(c, s);
    if (rc) return rc;
  }
  return IZEM_OK;
}

template <int NRV>
int do_finalize_ic(izem_ctx* c) {
  const Geo& g = c->g;
  int rc;
  if ((rc = launch(c, "wmix", [&] { k_wmix_interior<NRV><<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, c->v, c->W_i); })))
    return rc;
  if ((rc = enq_newton<NRV>(c, 0, 1.0e-10, 100, 0))) return rc;
  long long ns = slab_count(g) - g.nint;
  if ((rc = launch(c, "halo", [&] { k_halo<NRV><<<grid_for(ns), kThreads, 0, c->stream>>>(g, 1, 0, c->v, c->W_i); }))) return rc;
  return enq_newton<NRV>(c, 1, 1.0e-10, 100, 0);
}

template <int NRV>
int do_update_primitives(izem_ctx* c) {
  const Geo& g = c->g;
  int rc;
  // upd_prim_var_domain on the current interior state (force_sumY + W_i)
  if ((rc = launch(c, "prep_interior", [&] {
         k_prep_interior<NRV><<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, c->cfg.forcesum, c->v, c->W_i);
       })))
    return rc;
  return enq_update_primitives_after<NRV>(c);
}

// reaction_selec tail (module_reaction.f90:83-86): upd_prim_var_woT, then
// the ghost closure given the half step and the time (d_dt[4], d_dt[5]).
template <int NRV>
int do_chem_after(izem_ctx* c) {
  const Geo& g = c->g;
  int rc;
  if ((rc = launch(c, "prim_woT", [&] {
         k_prim_woT<NRV><<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, c->v, c->T, c->W_i, c->cp, c->ha);
       })))
    return rc;
  return enq_boundaries<NRV>(c, c->d_dt + 4, 0.0);
}

template <int NRV>
int do_timestep(izem_ctx* c) {
  const Geo& g = c->g;
  Metrics mt;
  for (int d = 0; d < 3; ++d) mt.dxi[d] = c->dxi[d];
  int rc = launch(c, "timestep", [&] {
    k_dtc<NRV><<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, mt, c->v, c->T, c->W_i, c->cp, c->d_status);
  });
  if (rc || !(c->cfg.vis && c->cfg.vis_dt)) return rc;
  return launch(c, "timestep_fourier", [&] {
    // with the fitted-transport LES, mu_SGS of the last flux evaluation
    const bool msgs = c->les_on && !c->cfg.eglib && c->mu_sgs;
    k_dtv<NRV><<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, mt, c->v, c->T, c->W_i, c->cp, c->d_status,
                                                            msgs ? c->mu_sgs : nullptr, c->adi.sc, c->les_sc_sgs,
                                                            c->adi.pr, c->les_pr_sgs_i);
  });
}

// the sensor alone (the Ducros sensor needs the primitives' velocities)
template <int NRV>
int do_sensor(izem_ctx* c) {
  if (c->sensor_type == IZEM_SENSOR_DUCROS) return enq_sensor_prim<NRV>(c);
  const Geo& g = c->g;
  return launch(c, "sensor", [&] { k_sensor<<<grid_for(g.nint), kThreads, 0, c->stream>>>(g, c->cfg.max_rel_weight, c->v, c->T, c->W_i, c->sensor, c->sensor_bx); });
}

template <int NRV>
int do_euler(izem_ctx* c, int d) {
  int rc = enq_prim<NRV>(c);
  if (rc) return rc;
  return enq_euler<NRV>(c, d);
}

template <int NRV>
int do_visc(izem_ctx* c) {
  int rc = enq_prim<NRV>(c);
  if (rc) return rc;
  return enq_visc<NRV>(c);
}

template <int NRV>
int do_nr(izem_ctx* c) {
  return enq_nr<NRV>(c);
}


// ---------------------------------------------------------- autotuning -------
// Times each candidate launch configuration on the context's current state
// with CUDA events and keeps the fastest.  Block size changes only how the
// points are grouped, never a point's arithmetic, so every candidate gives
// identical results.
constexpr int kTuneCand[3] = {64, 128, 256};

template <class F>
float tune_time(izem_ctx* c, int reps, F body) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  body();   // untimed first pass
  cudaEventRecord(a, c->stream);
  for (int r = 0; r < reps; ++r) body();
  cudaEventRecord(b, c->stream);
  float ms = -1.f;
  if (cudaEventSynchronize(b) == cudaSuccess) cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms < 0.f ? 1e30f : ms / reps;
}

void tune_report(std::string& rep, const char* name, const float* ms, int chosen) {
  char buf[256];
  std::snprintf(buf, sizeof(buf), "%s\"%s\": {\"64\": %.4f, \"128\": %.4f, \"256\": %.4f, \"chosen\": %d}",
                rep.size() > 1 ? ", " : "", name, ms[0], ms[1], ms[2], chosen);
  rep += buf;
}

template <int NRV>
int tune_flow(izem_ctx* c, std::string* rep) {
  int rc = enq_prim<NRV>(c);
  if (rc) return rc;
  float ms[3] = {1e30f, 1e30f, 1e30f};   // untimed candidates never win
  int best = 1;
  for (int q = 0; q < 3; ++q) {
    c->tb_euler = kTuneCand[q];
    ms[q] = tune_time(c, 2, [&] { for (int d = 0; d < c->cfg.ndim; ++d) (void)enq_euler<NRV>(c, d); });
    if (ms[q] < ms[best]) best = q;
  }
  c->tb_euler = kTuneCand[best];
  tune_report(*rep, "euler_face", ms, c->tb_euler);
  if (c->cfg.vis) {
    best = 1;
    for (float& x : ms) x = 1e30f;
    for (int q = 0; q < 3; ++q) {
      c->tb_visc = kTuneCand[q];
      ms[q] = tune_time(c, 2, [&] { (void)enq_visc<NRV>(c); });
      if (ms[q] < ms[best]) best = q;
    }
    c->tb_visc = kTuneCand[best];
    tune_report(*rep, c->cfg.eglib ? "visc_point_eg" : "visc_point", ms, c->tb_visc);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? IZEM_OK : ctx_fail(c, IZEM_ERR_CUDA, "autotune", e);
}

// ================================================================ C ABI =====
extern "C" {

int izem_gpu_init(const izem_cfg* cfg, const izem_thd* thd, const izem_adi* adi, izem_ctx** out) {
  if (!cfg || !thd || !adi || !out) return IZEM_ERR_ARG;
  *out = nullptr;
  // WENO5 (ng = 3) or WENO7 (ng = 4) in 2-D or 3-D; 2-D runs have nz = 1;
  // EGLIB transport in 3-D only
  const bool ng_ok = cfg->ng == 3 || cfg->ng == 4;
  const bool dim_ok = cfg->ndim == 3 || (cfg->ndim == 2 && cfg->nz == 1 && !cfg->eglib);
  if (!ng_ok || !dim_ok || !(cfg->nrv == 2 || cfg->nrv == 9) || thd->nspc != cfg->nrv) return IZEM_ERR_ARG;
  const int nmin = 2 * cfg->ng + 1;
  if (cfg->nx < nmin || cfg->ny < nmin || (cfg->ndim == 3 && cfg->nz < nmin)) return IZEM_ERR_ARG;
  for (int f = 0; f < 6; ++f) {
    const int bc = cfg->bc[f];
    if (bc < IZEM_BC_PERIODIC || bc > IZEM_BC_NOREFLECTION) return IZEM_ERR_ARG;
    // bc_inflowjet declares the W face only, bc_nscbc_out the E face only
    if ((bc == IZEM_BC_INFLOWJET && f != IZEM_FACE_W) || (bc == IZEM_BC_NSCBC_OUT && f != IZEM_FACE_E))
      return IZEM_ERR_ARG;
  }
  for (int d = 0; d < 3; ++d)
    if ((cfg->bc[2 * d] == IZEM_BC_PERIODIC) != (cfg->bc[2 * d + 1] == IZEM_BC_PERIODIC)) return IZEM_ERR_ARG;
  izem_ctx* c = new izem_ctx();
  c->cfg = *cfg;
  c->thd = *thd;
  c->adi = *adi;
  Geo& g = c->g;
  g.n[0] = cfg->nx; g.n[1] = cfg->ny; g.n[2] = cfg->nz; g.ng = cfg->ng; g.ndim = cfg->ndim;
  c->sensor_bx = cfg->nx;   // one block
  c->newton_bx = cfg->nx;
  for (int d = 0; d < 3; ++d) g.g[d] = g.n[d] + 2 * g.ng;
  g.ncell = (long long)g.g[0] * g.g[1] * g.g[2];
  g.nint = (long long)g.n[0] * g.n[1] * g.n[2];
  for (int f = 0; f < 6; ++f) { g.bc[f] = cfg->bc[f]; g.bnd[f] = cfg->bc[f] != IZEM_BC_PERIODIC; }
  c->nv = IZEM_NIV + cfg->nrv;

  // constant species data in code units (thd_init) plus derived constants
  DevThd h;
  std::memset(&h, 0, sizeof(h));
  h.nspc = thd->nspc;
  h.gam2 = thd->gam2;
  h.gam2_i = 1.0 / thd->gam2;
  h.tinf = thd->tinf;
  h.tinf_i = 1.0 / thd->tinf;
  h.onethird = 1.0 / 3.0;
  for (int k = 0; k < thd->nspc; ++k) {
    h.Wc[k] = thd->Wc[k];
    h.Wc_i[k] = thd->Wc_i[k];
    h.tpolymin[k] = thd->tpolymin[k];
    h.tpolymax[k] = thd->tpolymax[k];
    h.tpolylim[k] = thd->tpolylim[k];
    std::memcpy(h.hc[k], thd->heatcap[k], sizeof(h.hc[k]));
    for (int l = 0; l < thd->nspc; ++l) {
      std::memcpy(h.cofd[k][l], thd->cofd[k][l], sizeof(h.cofd[k][l]));
      h.wilke_c1[k][l] = std::pow(thd->W[l] / thd->W[k], 0.25);
      h.wilke_c2[k][l] = 1.0 / std::sqrt((1.0 + thd->W[k] / thd->W[l]) * 8.0);
    }
    std::memcpy(h.coflam[k], thd->coflam[k], sizeof(h.coflam[k]));
    std::memcpy(h.cofeta[k], thd->cofeta[k], sizeof(h.cofeta[k]));
    h.Kd[k] = 1.0e-4 * thd->p0 / (thd->pinf * thd->dinf[k]);
  }
  h.Kl = 0.5 * 1.0e-5 / thd->laminf;
  h.Ku = 1.0e-1 / thd->muinf;
  h.sqgmr = adi->sqgmr;
  h.rvd0 = adi->sqgmr / adi->sc;
  h.rlam0 = adi->sqgmr * adi->ggmopr;
  c->devthd = h;

  int rc = ctx_alloc(c);
  if (rc) {
    std::fprintf(stderr, "izem_gpu_init: %s\n", c->err.c_str());
    izem_gpu_destroy(c);
    return rc;
  }
  *out = c;
  return IZEM_OK;
}

}  // extern "C"

int ctx_alloc(izem_ctx* c) {
  const Geo& g = c->g;
  const int nv = c->nv, nrv = c->cfg.nrv;
  CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
  {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, dev));
  }
  CK(cudaMallocHost(&c->h_done, kNewtonSlots * sizeof(int)));
  CK(cudaMemcpyToSymbol(c_thd, &c->devthd, sizeof(DevThd)));
  auto alloc = [&](double** p, size_t n) -> cudaError_t {
    cudaError_t e = cudaMalloc(p, n * sizeof(double));
    if (e == cudaSuccess) c->allocs.push_back(*p);
    return e;
  };
  const size_t nc = (size_t)g.ncell, ni = (size_t)g.nint;
  size_t maxf = 0;
  for (int d = 0; d < 3; ++d) {
    size_t nf = (size_t)(g.n[0] + (d == 0)) * (g.n[1] + (d == 1)) * (g.n[2] + (d == 2));
    if (nf > maxf) maxf = nf;
  }
  cudaError_t e = cudaSuccess;
  if ((e = alloc(&c->v, nv * nc)) || (e = alloc(&c->T, nc)) || (e = alloc(&c->W_i, nc)) || (e = alloc(&c->cp, nc)) ||
      (e = alloc(&c->ha, nrv * nc)) || (e = alloc(&c->v0, nv * ni)) || (e = alloc(&c->f, nv * ni)) ||
      (e = alloc(&c->prim, PR_N * nc)) || (e = alloc(&c->Xa, nrv * nc)) || (e = alloc(&c->fhat, nv * maxf)) ||
      (e = alloc(&c->fd, (15 + 3 * nrv) * nc)) || (e = alloc(&c->tau, 6 * nc)) || (e = alloc(&c->qv, 3 * nc)) ||
      (e = alloc(&c->d_dt, 6)))
    return ctx_fail(c, e == cudaErrorMemoryAllocation ? IZEM_ERR_NOMEM : IZEM_ERR_CUDA, "device allocation", e);
  for (int d = 0; d < 3; ++d)
    if ((e = alloc(&c->dxi[d], g.g[d]))) return ctx_fail(c, IZEM_ERR_CUDA, "device allocation", e);
  CK(cudaMalloc(&c->sensor, nc));
  CK(cudaMemset(c->sensor, 0, nc));
  CK(cudaMalloc(&c->d_status, sizeof(DevStatus)));
  CK(cudaMemset(c->d_status, 0, sizeof(DevStatus)));
  CK(cudaMallocHost(&c->h_status, sizeof(DevStatus)));
  CK(cudaMallocHost(&c->h_dt, 4 * sizeof(double)));
  // dt, time0 of the RK3 step; zeros for calls outside rk3; the half step
  // and time of the last chemistry step
  CK(cudaMemset(c->d_dt, 0, 6 * sizeof(double)));
  // zero the arrays whose ghost corners are never written
  CK(cudaMemset(c->v, 0, nv * nc * sizeof(double)));
  CK(cudaMemset(c->fd, 0, (15 + 3 * nrv) * nc * sizeof(double)));
  CK(cudaMemset(c->tau, 0, 6 * nc * sizeof(double)));
  CK(cudaMemset(c->qv, 0, 3 * nc * sizeof(double)));
  CK(cudaMemset(c->f, 0, nv * ni * sizeof(double)));
  CK(cudaEventCreate(&c->t0));
  CK(cudaEventCreate(&c->t1));
  return IZEM_OK;
}

extern "C" {

void izem_gpu_destroy(izem_ctx* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  drop_graphs(c);
  for (double* p : c->allocs) cudaFree(p);
  if (c->sensor) cudaFree(c->sensor);
  if (c->fhat_edge) cudaFree(c->fhat_edge);
  if (c->d_status) cudaFree(c->d_status);
  if (c->d_counter) cudaFree(c->d_counter);
  if (c->d_chem_stats) cudaFree(c->d_chem_stats);
  if (c->h_chem_stats) cudaFreeHost(c->h_chem_stats);
  cudaFree(c->b_T); cudaFree(c->b_rho); cudaFree(c->b_Y); cudaFree(c->b_dt);
  cudaFree(c->b_list); cudaFree(c->d_list_count); cudaFree(c->les); cudaFree(c->mu_sgs); cudaFree(c->d_y); cudaFree(c->d_z);
  if (c->h_status) cudaFreeHost(c->h_status);
  if (c->h_dt) cudaFreeHost(c->h_dt);
  for (auto& v : c->kt_pending)
    for (auto& pr : v) { cudaEventDestroy(pr.first); cudaEventDestroy(pr.second); }
  if (c->t0) cudaEventDestroy(c->t0);
  if (c->t1) cudaEventDestroy(c->t1);
  if (c->h_done) cudaFreeHost(c->h_done);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

void izem_jet_reference(izem_jet* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  // bc_inflowjet's constants (module_BCs.f90:1680-1700) and bc_nscbc_out's
  // far-field pressure (:2390)
  p->width = 0.0010;
  p->ramp = 0.0001;
  p->T_jet = 1000.0;
  p->T_co = 300.0;
  p->p_jet = 101325.0 * 15.0;
  p->p_co = 101325.0;
  p->u_jet = 0.0;
  p->u_co = 20.0;
  p->y_fuel = 1.0;
  p->p_far = 94232.25;
}

int izem_gpu_newton_stats(izem_ctx* c, int* max_iters, int* unconverged, int reset) {
  if (!c) return IZEM_ERR_ARG;
  if (max_iters) *max_iters = c->newton_it_max;
  if (unconverged) *unconverged = c->newton_warn;
  if (reset) {
    c->newton_it_max = 0;
    c->newton_warn = 0;
  }
  return IZEM_OK;
}

int izem_gpu_last_error(izem_ctx* c, char* buf, int n) {
  if (!c) return IZEM_ERR_ARG;
  if (buf && n > 0) std::snprintf(buf, n, "%s", c->err.c_str());
  return c->newton_warn;
}

int izem_gpu_set_grid(izem_ctx* c, const double* dx_i, const double* dy_i, const double* dz_i) {
  if (!c || !dx_i || !dy_i || !dz_i) return IZEM_ERR_ARG;
  const double* s[3] = {dx_i, dy_i, dz_i};
  for (int d = 0; d < 3; ++d) CK(cudaMemcpy(c->dxi[d], s[d], c->g.g[d] * sizeof(double), cudaMemcpyHostToDevice));
  c->grid_set = true;
  return IZEM_OK;
}

// ------------------------------------------------------- host transfers ---
// State copies between the device and the caller's host arrays.  Pinned or
// registered host memory (cudaHostAlloc, cudaHostRegister: mapped into the
// device's address space under unified addressing) is moved by the SMs with
// 16-byte loads and stores over NVLink-C2C, 4 blocks of 512 threads per SM in
// a grid-stride loop.  On GB300 that holds 190-210 GB/s each way also when
// the link has been idle, where the copy engines' first transfers after an
// idle second ran at 20-120 GB/s.  Pageable memory, addresses that are not
// 16-byte aligned, and the last bytes of a size that is not a multiple of 16
// go through cudaMemcpyAsync.
namespace {
__global__ void k_xfer16(const uint4* __restrict__ s, uint4* __restrict__ d, long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {
    const uint4 a = s[i], b = s[i + stride], e = s[i + 2 * stride], f = s[i + 3 * stride];
    d[i] = a;
    d[i + stride] = b;
    d[i + 2 * stride] = e;
    d[i + 3 * stride] = f;
  }
  for (; i < n; i += stride) d[i] = s[i];
}

// device address of a pinned / registered host pointer, or null (pageable)
const void* host_mapped(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}
}  // namespace

static int xfer(izem_ctx* c, void* dst, const void* src, size_t bytes, bool h2d) {
  if (!bytes) return IZEM_OK;
  const void* dev_host = host_mapped(h2d ? src : dst);
  const void* s = h2d ? dev_host : src;
  void* d = h2d ? dst : const_cast<void*>(dev_host);
  const size_t body = bytes & ~(size_t)15;
  if (!dev_host || ((uintptr_t)s & 15) || ((uintptr_t)d & 15) || !body) {
    CK(cudaMemcpyAsync(dst, src, bytes, h2d ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, c->stream));
    return IZEM_OK;
  }
  const long long n16 = (long long)(body / 16);
  const long long blocks = std::min<long long>(4LL * std::max(c->nsm, 1), (n16 + 511) / 512);
  int rc = launch(c, "host_xfer", [&] {
    k_xfer16<<<(unsigned)blocks, 512, 0, c->stream>>>((const uint4*)s, (uint4*)d, n16);
  });
  if (rc) return rc;
  if (bytes > body)
    CK(cudaMemcpyAsync((char*)dst + body, (const char*)src + body, bytes - body,
                       h2d ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, c->stream));
  return IZEM_OK;
}

int izem_gpu_upload_state(izem_ctx* c, const double* v, const double* T, const double* W_i, const double* cp,
                          const double* ha, const uint8_t* sensor) {
  if (!c) return IZEM_ERR_ARG;
  const size_t nc = (size_t)c->g.ncell;
  int rc;
  if (v && (rc = xfer(c, c->v, v, c->nv * nc * sizeof(double), true))) return rc;
  if (T && (rc = xfer(c, c->T, T, nc * sizeof(double), true))) return rc;
  if (W_i && (rc = xfer(c, c->W_i, W_i, nc * sizeof(double), true))) return rc;
  if (cp && (rc = xfer(c, c->cp, cp, nc * sizeof(double), true))) return rc;
  if (ha && (rc = xfer(c, c->ha, ha, c->cfg.nrv * nc * sizeof(double), true))) return rc;
  if (sensor && (rc = xfer(c, c->sensor, sensor, nc, true))) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return IZEM_OK;
}

int izem_gpu_download_state(izem_ctx* c, double* v, double* T, double* W_i, double* cp, double* ha, uint8_t* sensor) {
  if (!c) return IZEM_ERR_ARG;
  const size_t nc = (size_t)c->g.ncell;
  int rc;
  if (v && (rc = xfer(c, v, c->v, c->nv * nc * sizeof(double), false))) return rc;
  if (T && (rc = xfer(c, T, c->T, nc * sizeof(double), false))) return rc;
  if (W_i && (rc = xfer(c, W_i, c->W_i, nc * sizeof(double), false))) return rc;
  if (cp && (rc = xfer(c, cp, c->cp, nc * sizeof(double), false))) return rc;
  if (ha && (rc = xfer(c, ha, c->ha, c->cfg.nrv * nc * sizeof(double), false))) return rc;
  if (sensor && (rc = xfer(c, sensor, c->sensor, nc, false))) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return IZEM_OK;
}

int izem_gpu_download_flux(izem_ctx* c, double* fl) {
  if (!c || !fl) return IZEM_ERR_ARG;
  CK(cudaMemcpyAsync(fl, c->f, c->nv * (size_t)c->g.nint * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return IZEM_OK;
}

int izem_gpu_zero_flux(izem_ctx* c) {
  if (!c) return IZEM_ERR_ARG;
  CK(cudaMemsetAsync(c->f, 0, c->nv * (size_t)c->g.nint * sizeof(double), c->stream));
  return IZEM_OK;
}

int izem_gpu_shock_sensor(izem_ctx* c) {
  if (!c) return IZEM_ERR_ARG;
  int rc = IZEM_DISPATCH(c, do_sensor, c);
  if (rc) return rc;
  return read_status(c);
}

int izem_gpu_euler_flux(izem_ctx* c, int dir) {
  if (!c || dir < 0 || dir >= c->cfg.ndim) return IZEM_ERR_ARG;
  if (!c->grid_set) return ctx_fail(c, IZEM_ERR_STATE, "grid not set", cudaSuccess);
  int rc = IZEM_DISPATCH(c, do_euler, c, dir);
  if (rc) return rc;
  return read_status(c);
}

int izem_gpu_visc_flux(izem_ctx* c) {
  if (c && c->cfg.eglib && !c->have_eg)
    return ctx_fail(c, IZEM_ERR_STATE, "EGLIB transport requested (cfg.eglib) but izem_gpu_set_eglib not called", cudaSuccess);
  if (!c) return IZEM_ERR_ARG;
  if (!c->grid_set) return ctx_fail(c, IZEM_ERR_STATE, "grid not set", cudaSuccess);
  int rc = IZEM_DISPATCH(c, do_visc, c);
  if (rc) return rc;
  return read_status(c);
}

int izem_gpu_nr_flux(izem_ctx* c) {
  if (!c) return IZEM_ERR_ARG;
  if (!c->grid_set) return ctx_fail(c, IZEM_ERR_STATE, "grid not set", cudaSuccess);
  int rc = IZEM_DISPATCH(c, do_nr, c);
  if (rc) return rc;
  return read_status(c);
}

int izem_gpu_update_primitives(izem_ctx* c) {
  if (!c) return IZEM_ERR_ARG;
  if ((jet_face(c->cfg.bc[0]) || jet_face(c->cfg.bc[1])) && !c->have_coords)
    return ctx_fail(c, IZEM_ERR_STATE, "jet faces need izem_gpu_set_coords", cudaSuccess);
  int rc = run_graph(c, izem_ctx::GR_PRIM, [&] { return IZEM_DISPATCH(c, do_update_primitives, c); });
  if (rc) return rc;
  return read_status(c);
}

int izem_gpu_finalize_ic(izem_ctx* c) {
  if (!c) return IZEM_ERR_ARG;
  int rc = run_graph(c, izem_ctx::GR_IC, [&] { return IZEM_DISPATCH(c, do_finalize_ic, c); });
  if (rc) return rc;
  return read_status(c);
}

int izem_gpu_rk3(izem_ctx* c, double dt, double time0) {
  if (!c) return IZEM_ERR_ARG;
  if (!c->grid_set) return ctx_fail(c, IZEM_ERR_STATE, "grid not set", cudaSuccess);
  if ((jet_face(c->cfg.bc[0]) || jet_face(c->cfg.bc[1])) && !c->have_coords)
    return ctx_fail(c, IZEM_ERR_STATE, "jet faces need izem_gpu_set_coords", cudaSuccess);
  if (c->cfg.vis && c->cfg.eglib && !c->have_eg)
    return ctx_fail(c, IZEM_ERR_STATE, "EGLIB transport requested (cfg.eglib) but izem_gpu_set_eglib not called", cudaSuccess);
  c->h_dt[0] = dt;
  c->h_dt[1] = time0;
  CK(cudaMemcpyAsync(c->d_dt, c->h_dt, 2 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  int rc = run_graph(c, izem_ctx::GR_RK3, [&] { return IZEM_DISPATCH(c, do_rk3_enqueue, c); });
  if (rc) return rc;
  return read_status(c);
}

int izem_gpu_timestep(izem_ctx* c, double DTmax, double dt_4[4], double* dtmin) {
  if (!c || !dt_4 || !dtmin) return IZEM_ERR_ARG;
  CK(cudaMemsetAsync(&c->d_status->dtc_bits, 0, sizeof(unsigned long long), c->stream));
  const bool fourier = c->cfg.vis && c->cfg.vis_dt;
  if (fourier) {
    // max slots from 0; min slots from bytes 0x7f (1.4e306, above any criterion)
    CK(cudaMemsetAsync(c->d_status->fo_dmax_bits, 0, sizeof(c->d_status->fo_dmax_bits), c->stream));
    CK(cudaMemsetAsync(c->d_status->fo_dmin_bits, 0x7f, sizeof(c->d_status->fo_dmin_bits), c->stream));
    CK(cudaMemsetAsync(&c->d_status->fo_ctmin_bits, 0x7f, sizeof(unsigned long long), c->stream));
  }
  int rc = IZEM_DISPATCH(c, do_timestep, c);
  if (rc) return rc;
  rc = read_status(c);
  if (rc) return rc;
  double m;
  std::memcpy(&m, &c->h_status->dtc_bits, sizeof(double));
  double dtc = std::fmax(1.0, m);
  for (int q = 0; q < 4; ++q) dt_4[q] = 1.0;
  dt_4[0] = c->cfg.cfl / dtc;
  if (fourier) {
    // the species of the largest D_k: the first that reaches the maximum, as
    // the reference's scan in (l, k, j, i) order with a strict comparison
    const DevStatus& s = *c->h_status;
    auto dbl = [](unsigned long long b) { double x; std::memcpy(&x, &b, sizeof(double)); return x; };
    int ldmax = 0;
    double dmax = dbl(s.fo_dmax_bits[0]);
    for (int l = 1; l < c->cfg.nrv; ++l)
      if (dmax < dbl(s.fo_dmax_bits[l])) { ldmax = l; dmax = dbl(s.fo_dmax_bits[l]); }
    const double rvd0_i = c->adi.sc / c->adi.sqgmr, rlamcp0_i = c->adi.pr / c->adi.sqgmr;
    dt_4[1] = rvd0_i * c->cfg.fo * dbl(s.fo_dmin_bits[ldmax]);
    dt_4[2] = rlamcp0_i * c->cfg.fo * dbl(s.fo_ctmin_bits);
  }
  if (c->cfg.reaction) {
    dt_4[3] = *dtmin * c->cfg.cpr / DTmax;
    dt_4[3] = std::fmin(dt_4[3], 1.0);
    dt_4[3] = std::fmax(dt_4[3], dt_4[0] * c->cfg.cflmin / c->cfg.cfl);
  }
  *dtmin = std::fmin(std::fmin(dt_4[0], dt_4[1]), std::fmin(dt_4[2], dt_4[3]));
  return IZEM_OK;
}

int izem_gpu_set_eglib(izem_ctx* c, const izem_eglib* L) {
  if (!c || !L) return IZEM_ERR_ARG;
  if (L->ns != c->cfg.nrv)
    return ctx_fail(c, IZEM_ERR_ARG, "EGLIB linking data must have nrv species", cudaSuccess);
  DevEg e;
  eg_prepare(*L, c->thd, c->adi, e);
  CK(cudaMemcpyToSymbol(c_eg, &e, sizeof(DevEg)));
  c->have_eg = true;
  return IZEM_OK;
}

int izem_gpu_set_mechanism(izem_ctx* c, const izem_mech* mech) {
  if (!c || !mech) return IZEM_ERR_ARG;
  if (mech->kk != c->cfg.nrv || mech->kk != 9 || mech->ii > IZEM_MAXREAC)
    return ctx_fail(c, IZEM_ERR_ARG, "mechanism species count must match nrv (9-species set)", cudaSuccess);
  if (!chem_mech_valid(mech))
    return ctx_fail(c, IZEM_ERR_ARG, "mechanism tables out of range (species index, reverse or fall-off kind, "
                    "collider, or a zero Troe/SRI temperature)", cudaSuccess);
  c->mech = *mech;
  CK(chem_upload_mech(mech));
  if (!c->d_counter) {
    CK(cudaMalloc(&c->d_counter, sizeof(unsigned)));
    CK(cudaMalloc(&c->d_chem_stats, sizeof(ChemStats)));
    CK(cudaMallocHost(&c->h_chem_stats, sizeof(ChemStats)));
  }
  c->have_mech = true;
  return IZEM_OK;
}

int izem_gpu_set_surrogate(izem_ctx* c, izem_mlp* m, izem_mlp* m2, const double* gate10, const int* kncf, int nele) {
  if (!c || !m || !gate10 || !kncf || nele <= 0) return IZEM_ERR_ARG;
  c->sur_m = m;
  c->sur_m2 = m2;
  std::memcpy(c->sur_gate, gate10, sizeof(c->sur_gate));
  c->sur_kncf.assign(kncf, kncf + (size_t)c->cfg.nrv * nele);
  c->sur_nele = nele;
  return IZEM_OK;
}

int izem_gpu_chem_surrogate_stats(izem_ctx* c, long long* cells, int* fallback, float* ms_total, float* ms_network) {
  if (!c) return IZEM_ERR_ARG;
  if (cells) *cells = c->sur_cells;
  if (fallback) *fallback = c->sur_stats[0];
  if (ms_total) *ms_total = c->sur_ms[0];
  if (ms_network) *ms_network = c->sur_ms[1];
  return IZEM_OK;
}

// The rest of reaction_selec after the reactors (module_reaction.f90:83-86):
// upd_prim_var_woT, halo, boundaries, ghost primitives; then the statistics.
static int chem_finish(izem_ctx* c, int mode, int sur_rc, double* DTmax) {
  int rc = run_graph(c, izem_ctx::GR_CHEM_AFTER, [&] { return IZEM_DISPATCH(c, do_chem_after, c); });
  if (rc) return rc;
  CK(cudaMemcpyAsync(c->h_chem_stats, c->d_chem_stats, sizeof(ChemStats), cudaMemcpyDeviceToHost, c->stream));
  rc = read_status(c);
  if (rc) return rc;
  ChemStats& cs = *(ChemStats*)c->h_chem_stats;
  if (mode == IZEM_CHEM_MLP) { cs.failed = c->sur_stats[2]; cs.max_steps = c->sur_stats[1]; }
  std::memcpy(DTmax, &cs.dtmax_bits, sizeof(double));
  if (cs.failed || sur_rc == IZEM_ERR_CHEM)
    return ctx_fail(c, IZEM_ERR_CHEM, "stiff integration failed (ISTATE <= -2) on some cells", cudaSuccess);
  return IZEM_OK;
}

int izem_gpu_chem_step(izem_ctx* c, double dt, double time, int mode, double* DTmax) {
  if (!c || !DTmax) return IZEM_ERR_ARG;
  if ((jet_face(c->cfg.bc[0]) || jet_face(c->cfg.bc[1])) && !c->have_coords)
    return ctx_fail(c, IZEM_ERR_STATE, "jet faces need izem_gpu_set_coords", cudaSuccess);
  if (!c->have_mech) return ctx_fail(c, IZEM_ERR_STATE, "no mechanism set", cudaSuccess);
  if (mode != IZEM_CHEM_BDF && mode != IZEM_CHEM_MLP) return ctx_fail(c, IZEM_ERR_ARG, "unknown chemistry mode", cudaSuccess);
  if (mode == IZEM_CHEM_MLP && !c->sur_m) return ctx_fail(c, IZEM_ERR_STATE, "no surrogate set", cudaSuccess);
  const Geo& g = c->g;
  ChemField f;
  f.v = c->v;
  f.T = c->T;
  f.dT_out = nullptr;
  f.ncell = g.ncell;
  f.gx = g.g[0];
  f.gy = g.g[1];
  f.ng = g.ng;
  const int ng = g.ng;
  // reaction_dvode window (module_reaction.f90:155-159): fz uses ey
  f.ix = ng + 1; f.iy = ng + 1; f.iz = ng + 1;
  const int fx = std::min(g.n[0], g.n[0] - ng - 1), fy = std::min(g.n[1], g.n[1] - ng - 1);
  const int fz = std::min(g.n[1], g.n[2] - ng - 1);
  f.wx = fx - f.ix + 1; f.wy = fy - f.iy + 1; f.wz = fz - f.iz + 1;
  f.t_ref = c->adi.t_ref;
  f.tref_i = 1.0 / c->adi.t_ref;
  f.rho_cgs = c->adi.rho_ref * 1.0e-3;
  f.dt_phys = dt * c->adi.time_ref;
  // the half step and the time that the boundary closure of the tail reads
  c->h_dt[2] = dt;
  c->h_dt[3] = time;
  CK(cudaMemcpyAsync(c->d_dt + 4, c->h_dt + 2, 2 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemsetAsync(c->d_chem_stats, 0, sizeof(ChemStats), c->stream));
  int sur_rc = IZEM_OK;
  const bool skip = mode == IZEM_CHEM_BDF && c->skip_on;
  if (f.wx > 0 && f.wy > 0 && f.wz > 0 && mode == IZEM_CHEM_BDF && !skip) {
    int rc = launch(c, "chem_psr", [&] { (void)chem_launch_field(f, c->d_counter, (ChemStats*)c->d_chem_stats, c->stream, 9); });
    if (rc) return rc;
  } else if (f.wx > 0 && f.wy > 0 && f.wz > 0) {
    // window -> reactors, gated surrogate with BDF fallback (its own stream), reactors -> window
    const long long n = (long long)f.wx * f.wy * f.wz;
    if (n > INT32_MAX) return ctx_fail(c, IZEM_ERR_ARG, "chemistry window too large for the surrogate path", cudaSuccess);
    if (n > c->sur_cap) {
      cudaFree(c->b_T); cudaFree(c->b_rho); cudaFree(c->b_Y); cudaFree(c->b_dt);
      c->b_T = c->b_rho = c->b_Y = c->b_dt = nullptr;
      CK(cudaMalloc(&c->b_T, n * sizeof(double)));
      CK(cudaMalloc(&c->b_rho, n * sizeof(double)));
      CK(cudaMalloc(&c->b_Y, n * 9 * sizeof(double)));
      CK(cudaMalloc(&c->b_dt, n * sizeof(double)));
      c->sur_cap = n;
    }
    int rc = launch(c, "chem_gather", [&] { (void)chem_launch_gather(f, c->b_T, c->b_rho, c->b_Y, c->b_dt, c->stream); });
    if (rc) return rc;
    if (skip) {
      // dvodesimp: select, integrate the selected reactors, write them back
      if (n > c->list_cap) {
        cudaFree(c->b_list);
        c->b_list = nullptr;
        CK(cudaMalloc(&c->b_list, n * sizeof(int)));
        c->list_cap = n;
      }
      if (!c->d_list_count) CK(cudaMalloc(&c->d_list_count, sizeof(unsigned)));
      CK(cudaMemsetAsync(c->d_list_count, 0, sizeof(unsigned), c->stream));
      ChemSkip sk{c->skip_y[0], c->skip_y[1], c->skip_y[2], c->skip_y[3], c->skip_ih2, c->skip_in2};
      rc = launch(c, "chem_select", [&] {
        (void)chem_launch_select((int)n, c->b_T, c->b_rho, c->b_Y, c->b_dt, sk, c->b_list, c->d_list_count, c->stream);
      });
      if (rc) return rc;
      rc = launch(c, "chem_psr", [&] {
        (void)chem_launch_list(c->b_list, c->d_list_count, c->b_T, c->b_rho, c->b_Y, c->b_dt, c->d_counter,
                               (ChemStats*)c->d_chem_stats, c->stream);
      });
      if (rc) return rc;
      rc = launch(c, "chem_scatter", [&] {
        (void)chem_launch_scatter_list(f, (int)n, c->b_list, c->d_list_count, c->b_T, c->b_Y,
                                       (ChemStats*)c->d_chem_stats, c->stream);
      });
      if (rc) return rc;
      return chem_finish(c, mode, sur_rc, DTmax);
    }
    CK(cudaStreamSynchronize(c->stream));
    sur_rc = izem_gpu_psr_batch_mlp(c->sur_m, c->sur_m2, &c->mech, (int)n, c->b_T, c->b_rho, c->b_Y, c->b_dt, 1,
                                    c->sur_gate, c->sur_kncf.data(), c->sur_nele, nullptr, c->sur_stats, c->sur_ms);
    c->sur_cells = n;
    if (sur_rc != IZEM_OK && sur_rc != IZEM_ERR_CHEM)
      return ctx_fail(c, sur_rc, "surrogate chemistry step failed", cudaSuccess);
    rc = launch(c, "chem_scatter", [&] { (void)chem_launch_scatter(f, c->b_T, c->b_Y, (ChemStats*)c->d_chem_stats, c->stream); });
    if (rc) return rc;
  }
  return chem_finish(c, mode, sur_rc, DTmax);
}

int izem_gpu_set_chem_skip(izem_ctx* c, int enable, const double* Y_fuel, const double* Y_oxidizer, int index_h2,
                           int index_n2) {
  if (!c) return IZEM_ERR_ARG;
  if (!enable) {
    c->skip_on = false;
    return IZEM_OK;
  }
  const int nrv = c->cfg.nrv;
  if (!Y_fuel || !Y_oxidizer || index_h2 < 0 || index_h2 >= nrv || index_n2 < 0 || index_n2 >= nrv ||
      index_h2 == index_n2)
    return IZEM_ERR_ARG;
  c->skip_y[0] = Y_fuel[index_h2];
  c->skip_y[1] = Y_fuel[index_n2];
  c->skip_y[2] = Y_oxidizer[index_h2];
  c->skip_y[3] = Y_oxidizer[index_n2];
  c->skip_ih2 = index_h2;
  c->skip_in2 = index_n2;
  c->skip_on = true;
  return IZEM_OK;
}

int izem_gpu_chem_stats(izem_ctx* c, int* failed, int* max_steps, unsigned long long* total_steps) {
  if (!c || !c->h_chem_stats) return IZEM_ERR_ARG;
  const ChemStats& cs = *(const ChemStats*)c->h_chem_stats;
  if (failed) *failed = cs.failed;
  if (max_steps) *max_steps = cs.max_steps;
  if (total_steps) *total_steps = cs.total_steps;
  return IZEM_OK;
}

int izem_gpu_psr_batch(const izem_mech* mech, int n, double* T, const double* rho, double* Y, const double* dt,
                       int* istate, int* nsteps, int device_ptrs, float* kernel_ms) {
  if (!mech || n <= 0 || !T || !rho || !Y || !dt || !chem_mech_valid(mech)) return IZEM_ERR_ARG;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return IZEM_ERR_CUDA;
  unsigned* counter = nullptr;
  ChemStats* st = nullptr;
  double *dT = nullptr, *drho = nullptr, *dY = nullptr, *ddt = nullptr;
  int *dis = nullptr, *dns = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = IZEM_OK;
  const size_t kk = mech->kk;
  auto fail = [&](int code) { rc = code; };
  do {
    if (chem_upload_mech(mech) != cudaSuccess) { fail(IZEM_ERR_CUDA); break; }
    if (cudaMalloc(&counter, sizeof(unsigned)) != cudaSuccess || cudaMalloc(&st, sizeof(ChemStats)) != cudaSuccess) {
      fail(IZEM_ERR_NOMEM); break;
    }
    cudaMemsetAsync(st, 0, sizeof(ChemStats), s);
    if (device_ptrs) {
      dT = T; drho = const_cast<double*>(rho); dY = Y; ddt = const_cast<double*>(dt); dis = istate; dns = nsteps;
    } else {
      if (cudaMalloc(&dT, n * sizeof(double)) || cudaMalloc(&drho, n * sizeof(double)) ||
          cudaMalloc(&dY, n * kk * sizeof(double)) || cudaMalloc(&ddt, n * sizeof(double)) ||
          cudaMalloc(&dis, n * sizeof(int)) || cudaMalloc(&dns, n * sizeof(int))) { fail(IZEM_ERR_NOMEM); break; }
      cudaMemcpyAsync(dT, T, n * sizeof(double), cudaMemcpyHostToDevice, s);
      cudaMemcpyAsync(drho, rho, n * sizeof(double), cudaMemcpyHostToDevice, s);
      cudaMemcpyAsync(dY, Y, n * kk * sizeof(double), cudaMemcpyHostToDevice, s);
      cudaMemcpyAsync(ddt, dt, n * sizeof(double), cudaMemcpyHostToDevice, s);
    }
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    if (chem_launch_batch(n, dT, drho, dY, ddt, dis, dns, counter, st, s, 9) != cudaSuccess) { fail(IZEM_ERR_CUDA); break; }
    cudaEventRecord(e1, s);
    if (!device_ptrs) {
      cudaMemcpyAsync(T, dT, n * sizeof(double), cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(Y, dY, n * kk * sizeof(double), cudaMemcpyDeviceToHost, s);
      if (istate) cudaMemcpyAsync(istate, dis, n * sizeof(int), cudaMemcpyDeviceToHost, s);
      if (nsteps) cudaMemcpyAsync(nsteps, dns, n * sizeof(int), cudaMemcpyDeviceToHost, s);
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) { fail(IZEM_ERR_CUDA); break; }
    if (kernel_ms) cudaEventElapsedTime(kernel_ms, e0, e1);
  } while (0);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (!device_ptrs) { cudaFree(dT); cudaFree(drho); cudaFree(dY); cudaFree(ddt); cudaFree(dis); cudaFree(dns); }
  cudaFree(counter);
  cudaFree(st);
  cudaStreamDestroy(s);
  return rc;
}

int izem_gpu_autotune(izem_ctx* c, double chem_dt, char* report, int report_len) {
  if (!c) return IZEM_ERR_ARG;
  if (!c->grid_set) return ctx_fail(c, IZEM_ERR_STATE, "grid not set", cudaSuccess);
  if (c->cfg.vis && c->cfg.eglib && !c->have_eg)
    return ctx_fail(c, IZEM_ERR_STATE, "EGLIB transport requested (cfg.eglib) but izem_gpu_set_eglib not called", cudaSuccess);
  // the captured RK3 graph holds the old launch configurations
  drop_graphs(c);
  const bool kt = c->kt_enabled;
  c->kt_enabled = false;
  std::string rep = "{";
  int rc = IZEM_DISPATCH(c, tune_flow, c, &rep);
  if (rc == IZEM_OK && c->have_mech && chem_dt > 0.0) {
    // the persistent chemistry kernel on a copy of this context's reaction window
    const Geo& g = c->g;
    ChemField f{};
    f.v = c->v; f.T = c->T; f.ncell = g.ncell; f.gx = g.g[0]; f.gy = g.g[1]; f.ng = g.ng;
    const int ng = g.ng;
    f.ix = ng + 1; f.iy = ng + 1; f.iz = ng + 1;
    const int fx = std::min(g.n[0], g.n[0] - ng - 1), fy = std::min(g.n[1], g.n[1] - ng - 1);
    const int fz = std::min(g.n[1], g.n[2] - ng - 1);
    f.wx = fx - f.ix + 1; f.wy = fy - f.iy + 1; f.wz = fz - f.iz + 1;
    f.t_ref = c->adi.t_ref; f.tref_i = 1.0 / c->adi.t_ref;
    f.rho_cgs = c->adi.rho_ref * 1.0e-3; f.dt_phys = chem_dt * c->adi.time_ref;
    const long long n = (f.wx > 0 && f.wy > 0 && f.wz > 0) ? (long long)f.wx * f.wy * f.wz : 0;
    if (n > 0 && n <= INT32_MAX) {
      double *T = nullptr, *rho = nullptr, *Y = nullptr, *dt = nullptr, *T0 = nullptr, *Y0 = nullptr;
      cudaError_t e = cudaSuccess;
      if ((e = cudaMalloc(&T, n * 8)) || (e = cudaMalloc(&rho, n * 8)) || (e = cudaMalloc(&Y, n * 72)) ||
          (e = cudaMalloc(&dt, n * 8)) || (e = cudaMalloc(&T0, n * 8)) || (e = cudaMalloc(&Y0, n * 72))) {
        rc = ctx_fail(c, IZEM_ERR_NOMEM, "autotune buffers", e);
      } else {
        // the register-budget variants of the persistent kernel (128 threads,
        // 8 down to 4 resident blocks per SM)
        chem_launch_gather(f, T0, rho, Y0, dt, c->stream);
        float ms[IZEM_CHEM_VARIANTS];
        for (float& x : ms) x = 1e30f;   // untimed candidates never win
        int best = chem_variant();
        for (int q = 0; q < IZEM_CHEM_VARIANTS; ++q) {
          chem_set_variant(q);
          auto body = [&] {
            cudaMemcpyAsync(T, T0, n * 8, cudaMemcpyDeviceToDevice, c->stream);
            cudaMemcpyAsync(Y, Y0, n * 72, cudaMemcpyDeviceToDevice, c->stream);
            (void)chem_launch_batch((int)n, T, rho, Y, dt, nullptr, nullptr, c->d_counter,
                                    (ChemStats*)c->d_chem_stats, c->stream, 9);
          };
          ms[q] = tune_time(c, 1, body);
          if (ms[q] < ms[best]) best = q;
        }
        chem_set_variant(best);
        char buf[160];
        std::snprintf(buf, sizeof(buf), "%s\"chem_psr\": {", rep.size() > 1 ? ", " : "");
        rep += buf;
        for (int q = 0; q < IZEM_CHEM_VARIANTS; ++q) {
          std::snprintf(buf, sizeof(buf), "\"128x%d (%d regs)\": %.4f, ", chem_variant_min_blocks(q),
                        chem_variant_registers(q), ms[q]);
          rep += buf;
        }
        std::snprintf(buf, sizeof(buf), "\"chosen\": \"128x%d (%d regs)\"}", chem_variant_min_blocks(best),
                      chem_variant_registers(best));
        rep += buf;
      }
      cudaFree(T); cudaFree(rho); cudaFree(Y); cudaFree(dt); cudaFree(T0); cudaFree(Y0);
    }
  }
  rep += "}";
  c->kt_enabled = kt;
  if (report && report_len > 0) std::snprintf(report, report_len, "%s", rep.c_str());
  if (rc == IZEM_OK) CK(cudaStreamSynchronize(c->stream));
  return rc;
}

int izem_gpu_set_sensor_xblocks(izem_ctx* c, int nblk) {
  if (!c || nblk < 1 || nblk > kNewtonXBlocksMax || c->cfg.nx % nblk != 0 || c->cfg.nx / nblk < c->cfg.ng)
    return IZEM_ERR_ARG;
  drop_graphs(c);
  if (c->fhat_edge) { CK(cudaFree(c->fhat_edge)); c->fhat_edge = nullptr; }
  c->sensor_bx = c->cfg.nx / nblk;
  c->newton_bx = c->cfg.nx / nblk;
  c->nedge = (long long)(nblk - 1) * c->cfg.ny * c->cfg.nz;
  if (c->nedge > 0) CK(cudaMalloc(&c->fhat_edge, (size_t)c->nv * c->nedge * sizeof(double)));
  return IZEM_OK;
}

int izem_gpu_set_coords(izem_ctx* c, const double* x, const double* y, const double* z, double lx) {
  if (!c || !x || !y || !z) return IZEM_ERR_ARG;
  (void)x;
  drop_graphs(c);   // captured graphs hold the jet constants by value
  if (!c->d_y) {
    CK(cudaMalloc(&c->d_y, c->g.n[1] * sizeof(double)));
    CK(cudaMalloc(&c->d_z, c->g.n[2] * sizeof(double)));
  }
  CK(cudaMemcpy(c->d_y, y, c->g.n[1] * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_z, z, c->g.n[2] * sizeof(double), cudaMemcpyHostToDevice));
  JetArgs& j = c->jet;
  j.y = c->d_y;
  j.z = c->d_z;
  j.lx = lx;
  j.dxi0 = c->dxi[0];
  izem_jet_reference(&c->jet_par);
  jet_args(c);
  c->have_coords = true;
  return IZEM_OK;
}

int izem_gpu_set_jet(izem_ctx* c, const izem_jet* p) {
  if (!c || !p) return IZEM_ERR_ARG;
  if (!c->have_coords) return ctx_fail(c, IZEM_ERR_STATE, "izem_gpu_set_jet needs izem_gpu_set_coords first", cudaSuccess);
  if (!(p->width > 0.0) || !(p->ramp >= 0.0) || !(p->T_jet > 0.0) || !(p->T_co > 0.0) || !(p->p_jet > 0.0) ||
      !(p->p_co > 0.0) || !(p->u_jet >= 0.0) || !(p->y_fuel >= 0.0 && p->y_fuel <= 1.0) || !(p->p_far > 0.0) ||
      !(p->turb >= 0.0))
    return ctx_fail(c, IZEM_ERR_ARG, "jet parameters out of range", cudaSuccess);
  drop_graphs(c);   // captured graphs hold the jet constants by value
  c->jet_par = *p;
  jet_args(c);
  return IZEM_OK;
}

int izem_gpu_set_shock_sensor(izem_ctx* c, int type, double ducros_treduc) {
  if (!c) return IZEM_ERR_ARG;
  if (type != IZEM_SENSOR_ADAMS_SHARIFF && type != IZEM_SENSOR_DUCROS)
    return ctx_fail(c, IZEM_ERR_ARG, "unknown shock sensor type", cudaSuccess);
  if (type == IZEM_SENSOR_DUCROS && c->cfg.ndim < 2)
    return ctx_fail(c, IZEM_ERR_ARG, "the Ducros sensor needs a 2-D or 3-D block", cudaSuccess);
  if (!(ducros_treduc >= 0.0 && ducros_treduc <= 1.0))
    return ctx_fail(c, IZEM_ERR_ARG, "DUCROS_TREDUC outside [0, 1]", cudaSuccess);
  drop_graphs(c);   // the captured RK3 graph holds the other sensor kernel
  c->sensor_type = type;
  c->ducros_treduc = ducros_treduc;
  return IZEM_OK;
}

int izem_gpu_set_les(izem_ctx* c, int enable, double mu_sgs_factor, double sc_sgs, double pr_sgs,
                     double percent_weight_sgs) {
  if (!c) return IZEM_ERR_ARG;
  // the captured RK3 graph holds the other viscous kernel
  drop_graphs(c);
  if (!enable) {
    c->les_on = false;
    if (c->mu_sgs) CK(cudaMemset(c->mu_sgs, 0, (size_t)c->g.ncell * sizeof(double)));
    return IZEM_OK;
  }
  if (!c->cfg.vis || c->cfg.ndim != 3)
    return ctx_fail(c, IZEM_ERR_ARG, "LES closure needs VIS and a 3-D block", cudaSuccess);
  if (!(mu_sgs_factor >= 0.0) || !(sc_sgs > 0.0) || !(pr_sgs > 0.0) || !(percent_weight_sgs >= 0.0))
    return ctx_fail(c, IZEM_ERR_ARG, "LES parameters out of range", cudaSuccess);
  if (!c->les) {
    CK(cudaMalloc(&c->les, 4 * (size_t)c->g.ncell * sizeof(double)));
    CK(cudaMemset(c->les, 0, 4 * (size_t)c->g.ncell * sizeof(double)));
  }
  double cs2 = mu_sgs_factor;
  cs2 = cs2 * cs2 / c->adi.sqgmr;
  c->les_cs2 = cs2;
  c->les_sc_sgs_i = 1.0 / sc_sgs;
  c->les_sc_sgs = sc_sgs;
  c->les_pr_sgs_i = 1.0 / pr_sgs;
  if (!c->cfg.eglib && !c->mu_sgs) {   // viscflux_LES_xyz hands mu_SGS to the time step
    CK(cudaMalloc(&c->mu_sgs, (size_t)c->g.ncell * sizeof(double)));
    CK(cudaMemset(c->mu_sgs, 0, (size_t)c->g.ncell * sizeof(double)));
  }
  c->les_pw = percent_weight_sgs;
  c->les_on = true;
  return IZEM_OK;
}

int izem_gpu_set_chem_variant(int variant) { return chem_set_variant(variant) == 0 ? IZEM_OK : IZEM_ERR_ARG; }

// FP64 FMA throughput of the current device: 8 independent FMA chains per
// thread, 8 blocks of 256 threads per SM, timed with CUDA events; the
// denominator of the FP64 rooflines.
namespace {
__global__ void k_fp64_fma(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) x[q] = threadIdx.x * 1.0e-3 + q;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int q = 0; q < 8; ++q) x[q] = fma(x[q], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) s += x[q];
  if (s == -1.0) out[0] = s;   // never true; keeps the chains
}
}  // namespace

int izem_gpu_fp64_rate(double* gflops) {
  if (!gflops) return IZEM_ERR_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return IZEM_ERR_CUDA;
  double* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return IZEM_ERR_NOMEM;
  int rc = IZEM_OK;
  const int iters = 2048, threads = 256, blocks = 8 * sms;
  double best = 0.0;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = IZEM_ERR_CUDA;
  for (int r = 0; r < 4 && rc == IZEM_OK; ++r) {   // the first launch warms up
    cudaEventRecord(e0);
    k_fp64_fma<<<blocks, threads>>>(out, iters, 0.9999999, 1.0e-7);
    cudaEventRecord(e1);
    float ms = 0.f;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      rc = IZEM_ERR_CUDA;
      break;
    }
    const double flop = 2.0 * 8.0 * iters * (double)threads * blocks;
    if (r > 0 && ms > 0.f) best = std::max(best, flop / (ms * 1.0e-3) / 1.0e9);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  *gflops = best;
  return rc;
}

int izem_gpu_chem_generated(void) { return chem_generated_rhs(); }

int izem_gpu_allow_chem_generated(int allow) {
  chem_allow_generated(allow != 0);
  return IZEM_OK;
}

int izem_gpu_chem_autotune(const izem_mech* mech, int n, const double* T, const double* rho, const double* Y,
                           const double* dt, int device_ptrs, char* report, int report_len) {
  if (!mech || n <= 0 || !T || !rho || !Y || !dt || !chem_mech_valid(mech)) return IZEM_ERR_ARG;
  // the first 2^20 reactors are the sample: a smaller one is dominated by the
  // tail of its slowest cells and ranks the variants differently
  const int ns = n < (1 << 20) ? n : (1 << 20);
  const cudaMemcpyKind kind = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return IZEM_ERR_CUDA;
  double *T0 = nullptr, *Y0 = nullptr, *r = nullptr, *d = nullptr, *Tw = nullptr, *Yw = nullptr;
  unsigned* counter = nullptr;
  ChemStats* st = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  int rc = IZEM_OK;
  float ms[IZEM_CHEM_VARIANTS];
  for (float& x : ms) x = 1e30f;   // untimed candidates never win
  int best = chem_variant();
  do {
    if (chem_upload_mech(mech) != cudaSuccess) { rc = IZEM_ERR_CUDA; break; }
    if (cudaMalloc(&T0, ns * 8) || cudaMalloc(&Y0, (size_t)ns * 72) || cudaMalloc(&r, ns * 8) ||
        cudaMalloc(&d, ns * 8) || cudaMalloc(&Tw, ns * 8) || cudaMalloc(&Yw, (size_t)ns * 72) ||
        cudaMalloc(&counter, sizeof(unsigned)) || cudaMalloc(&st, sizeof(ChemStats))) { rc = IZEM_ERR_NOMEM; break; }
    cudaMemcpyAsync(T0, T, ns * 8, kind, s);
    cudaMemcpyAsync(Y0, Y, (size_t)ns * 72, kind, s);
    cudaMemcpyAsync(r, rho, ns * 8, kind, s);
    cudaMemcpyAsync(d, dt, ns * 8, kind, s);
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    for (int q = 0; q < IZEM_CHEM_VARIANTS && rc == IZEM_OK; ++q) {
      chem_set_variant(q);
      ms[q] = 1e30f;
      for (int rep = 0; rep < 2; ++rep) {   // untimed first pass, then the timed one
        cudaMemcpyAsync(Tw, T0, ns * 8, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(Yw, Y0, (size_t)ns * 72, cudaMemcpyDeviceToDevice, s);
        cudaEventRecord(a, s);
        if (chem_launch_batch(ns, Tw, r, Yw, d, nullptr, nullptr, counter, st, s, 9) != cudaSuccess) {
          rc = IZEM_ERR_CUDA;
          break;
        }
        cudaEventRecord(b, s);
        if (cudaEventSynchronize(b) != cudaSuccess) { rc = IZEM_ERR_CUDA; break; }
        if (rep == 1) cudaEventElapsedTime(&ms[q], a, b);
      }
      if (rc == IZEM_OK && ms[q] < ms[best]) best = q;
    }
  } while (0);
  chem_set_variant(best);
  if (rc == IZEM_OK && report && report_len > 0) {
    std::string rep = "{\"sample\": " + std::to_string(ns);
    char buf[96];
    for (int q = 0; q < IZEM_CHEM_VARIANTS; ++q) {
      std::snprintf(buf, sizeof(buf), ", \"128x%d (%d regs)\": %.4f", chem_variant_min_blocks(q),
                    chem_variant_registers(q), ms[q]);
      rep += buf;
    }
    std::snprintf(buf, sizeof(buf), ", \"chosen\": \"128x%d (%d regs)\"}", chem_variant_min_blocks(best),
                  chem_variant_registers(best));
    rep += buf;
    std::snprintf(report, report_len, "%s", rep.c_str());
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  cudaFree(T0); cudaFree(Y0); cudaFree(r); cudaFree(d); cudaFree(Tw); cudaFree(Yw); cudaFree(counter); cudaFree(st);
  cudaStreamDestroy(s);
  return rc;
}

int izem_gpu_timer_start(izem_ctx* c) {
  if (!c) return IZEM_ERR_ARG;
  CK(cudaEventRecord(c->t0, c->stream));
  return IZEM_OK;
}

int izem_gpu_timer_stop(izem_ctx* c, float* ms) {
  if (!c || !ms) return IZEM_ERR_ARG;
  CK(cudaEventRecord(c->t1, c->stream));
  CK(cudaEventSynchronize(c->t1));
  CK(cudaEventElapsedTime(ms, c->t0, c->t1));
  return IZEM_OK;
}

int izem_gpu_set_kernel_timing(izem_ctx* c, int enable) {
  if (!c) return IZEM_ERR_ARG;
  int rc = kt_collect(c);
  if (rc) return rc;
  c->kt_enabled = enable != 0;
  for (size_t q = 0; q < c->kt_names.size(); ++q) { c->kt_ms[q] = 0.0; c->kt_launches[q] = 0; }
  return IZEM_OK;
}

int izem_gpu_kernel_times(izem_ctx* c, int max_kernels, char* names, int name_len, int* launches, double* ms, int* n_kernels) {
  if (!c || !n_kernels) return IZEM_ERR_ARG;
  int rc = kt_collect(c);
  if (rc) return rc;
  int n = (int)c->kt_names.size();
  *n_kernels = n;
  for (int q = 0; q < n && q < max_kernels; ++q) {
    if (names) std::snprintf(names + (size_t)q * name_len, name_len, "%s", c->kt_names[q].c_str());
    if (launches) launches[q] = c->kt_launches[q];
    if (ms) ms[q] = c->kt_ms[q];
  }
  return IZEM_OK;
}

int izem_gpu_synchronize(izem_ctx* c) {
  if (!c) return IZEM_ERR_ARG;
  CK(cudaStreamSynchronize(c->stream));
  return read_status(c);
}

int izem_abi_sizes(size_t* a, size_t* b, size_t* d) {
  if (!a || !b || !d) return IZEM_ERR_ARG;
  *a = sizeof(izem_cfg);
  *b = sizeof(izem_thd);
  *d = sizeof(izem_adi);
  return IZEM_OK;
}

int izem_metrics_dscalar(int n, int ng, const double* coord, double* d_i) {
  if ((ng != 3 && ng != 4) || n < 2 * ng + 1 || !coord || !d_i) return IZEM_ERR_ARG;
  std::vector<double> dv(n, 1.0);
  const double a6[7] = {-1.0 / 60.0, 9.0 / 60.0, -45.0 / 60.0, 0.0, 45.0 / 60.0, -9.0 / 60.0, 1.0 / 60.0};
  const double a4[5] = {1.0 / 12.0, -8.0 / 12.0, 0.0, 8.0 / 12.0, -1.0 / 12.0};
  const double a4ol[5] = {-25.0 / 12.0, 48.0 / 12.0, -36.0 / 12.0, 16.0 / 12.0, -3.0 / 12.0};
  const double a4ul[5] = {-3.0 / 12.0, -10.0 / 12.0, 18.0 / 12.0, -6.0 / 12.0, 1.0 / 12.0};
  const double a4ur[5] = {1.0 / 12.0, -6.0 / 12.0, 18.0 / 12.0, -10.0 / 12.0, -3.0 / 12.0};
  const double a4or[5] = {-3.0 / 12.0, 16.0 / 12.0, -36.0 / 12.0, 48.0 / 12.0, -25.0 / 12.0};
  auto x = [&](int m) { return coord[m - 1]; };
  // central rows: 6th order (ng = 3), or 8th order with 6th-order fourth rows (ng = 4)
  const double a8[9] = {3.0 / 840.0, -32.0 / 840.0, 168.0 / 840.0, -672.0 / 840.0, 0.0,
                        672.0 / 840.0, -168.0 / 840.0, 32.0 / 840.0, -3.0 / 840.0};
  for (int m = 1 + ng; m <= n - ng; ++m) {
    double dd = 0.0;
    if (ng == 4)
      for (int l = -4; l <= 4; ++l) dd = dd + a8[l + 4] * x(m + l);
    else
      for (int l = -3; l <= 3; ++l) dd = dd + a6[l + 3] * x(m + l);
    dv[m - 1] = dd * 1.0;
  }
  if (ng == 4)
    for (int m : {4, n - 3}) {
      double dd = 0.0;
      for (int l = -3; l <= 3; ++l) dd = dd + a6[l + 3] * x(m + l);
      dv[m - 1] = dd * 1.0;
    }
  { double dd = 0.0; for (int l = 0; l <= 4; ++l) dd = dd + a4ol[l] * x(1 + l); dv[0] = dd * 1.0; }
  { double dd = 0.0; for (int l = -1; l <= 3; ++l) dd = dd + a4ul[l + 1] * x(2 + l); dv[1] = dd * 1.0; }
  { double dd = 0.0; for (int l = -2; l <= 2; ++l) dd = dd + a4[l + 2] * x(3 + l); dv[2] = dd * 1.0; }
  { double dd = 0.0; for (int l = -2; l <= 2; ++l) dd = dd + a4[l + 2] * x(n - 2 + l); dv[n - 3] = dd * 1.0; }
  { double dd = 0.0; for (int l = -3; l <= 1; ++l) dd = dd + a4ur[l + 3] * x(n - 1 + l); dv[n - 2] = -dd * 1.0; }
  { double dd = 0.0; for (int l = -4; l <= 0; ++l) dd = dd + a4or[l + 4] * x(n + l); dv[n - 1] = -dd * 1.0; }
  for (int m = 0; m < n; ++m) d_i[m] = 1.0 / dv[m];
  return IZEM_OK;
}

}  // extern "C"

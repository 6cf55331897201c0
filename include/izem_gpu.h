/*
 * izem_gpu.h -- C ABI of the GB300 (sm_103a) implementation of the IZEM
 * right-hand-side hot path: characteristic WENO convective fluxes, fitted or
 * EGLIB mixture transport viscous fluxes, stiff CHEMKIN chemistry integrated
 * per cell by a BDF method, and the SSP-RK3 conservative update.
 *
 * The Fortran host keeps its module interfaces (module_solver, module_weno,
 * module_viscflux, module_reaction) and forwards their bodies through
 * iso_c_binding to these entry points.  Every array argument is the base
 * address of a Fortran column-major array with the reference's own bounds
 * (sx-ng:ex+ng, sy-ng:ey+ng, sz-ng:ez+ng[, 1:nv]); i is fastest, the variable
 * index slowest.  Plain pointers and sizes only: no C++ or torch types.
 *
 * Every entry point returns 0 (IZEM_OK) on success or one of the IZEM_ERR_*
 * codes; izem_gpu_last_error() gives the message.  The reference maps these
 * conditions to abort_mpi (devel-izem/src/module_parallel.f90:200).
 */
#ifndef IZEM_GPU_H
#define IZEM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IZEM_NSMAX 10      /* maximum reactive species (9-species H2/air set) */
#define IZEM_NPOLY 4       /* transport fit order (tranfit.out: Npoly = 4)    */

/* Boundary kinds of the faces W,E,S,N,B,F (module_parameters: bc(1:6),
 * module_BCs.f90): periodic (comm_cons), bc_extrapolation
 * (:327-412), bc_inflowjet on the W face only (:1646-1791) and bc_nscbc_out
 * on the E face only (:2331-2516); the last two are Dirichlet faces closed by
 * upd_prim_var_dirichlet (:297-314) and need izem_gpu_set_coords.
 * IZEM_BC_NOREFLECTION (NOREFLECTION, any face): the ghost points hold the
 * boundary point's state times 10 (bc_noreflection, :426-512), the Euler
 * sweep across the face drops its flux difference at the boundary points
 * (module_weno.f90:620-623, 1002, 1018 and the y, z counterparts), and
 * every stage adds the one-sided characteristic term of bc_noreflectionweno
 * (module_weno.f90:2129-4498) after the viscous fluxes. */
enum {
  IZEM_BC_PERIODIC = 0,
  IZEM_BC_EXTRAPOLATION = 1,
  IZEM_BC_INFLOWJET = 2,
  IZEM_BC_NSCBC_OUT = 3,
  IZEM_BC_NOREFLECTION = 4
};
enum { IZEM_FACE_W = 0, IZEM_FACE_E, IZEM_FACE_S, IZEM_FACE_N, IZEM_FACE_B, IZEM_FACE_F };

/* Shock sensors (SHOCK_SENSOR_TYPE, module_solver.f90:758-766). */
enum { IZEM_SENSOR_ADAMS_SHARIFF = 0, IZEM_SENSOR_DUCROS = 1 };

/* Status codes. */
enum {
  IZEM_OK = 0,
  IZEM_ERR_ARG = 1,            /* bad argument / unsupported configuration          */
  IZEM_ERR_CUDA = 2,           /* CUDA runtime failure (message has the detail)    */
  IZEM_ERR_NEG_PRESSURE = 3,   /* euler_LLF_*: P <= 0 (module_weno.f90:1027-1036)  */
  IZEM_ERR_NEG_TEMPERATURE = 4,/* prim_inv_var: T < 0 (module_thermodynamics:125)  */
  IZEM_ERR_NAN = 5,            /* Newton error is NaN (module_thermodynamics:182)  */
  IZEM_ERR_CHEM = 6,           /* stiff integrator failed on at least one cell     */
  IZEM_ERR_TIMEOUT = 7,        /* a bounded device-side wait gave up               */
  IZEM_ERR_NOMEM = 8,          /* device allocation failed                         */
  IZEM_ERR_STATE = 9,          /* call made in the wrong order (e.g. no grid set)  */
  IZEM_ERR_TOO_LARGE = 10      /* request above a fixed capacity (no-alloc calls)  */
};

/* Hot-path switches and sizes: the subset of the reference's globals that the
 * RHS reads (module_parameters.f90:35-56, module_input.f90:266-400,622-770). */
typedef struct izem_cfg {
  int    nx, ny, nz;        /* interior points of this block: ex-sx+1, ...      */
  int    ng;                /* ghost depth = (order_weno+1)/2: 3 WENO5, 4 WENO7 */
  int    ndim;              /* 3, or 2 with nz = 1                              */
  int    nrv;               /* reactive species, 2..IZEM_NSMAX                  */
  int    bc[6];             /* IZEM_BC_* per face W,E,S,N,B,F                   */
  int    weno_avg;          /* [WENO] WEIGHTS: nonlinear weights where sensed   */
  double max_rel_weight;    /* [WENO] PERCENT_WEIGHT (Adams-Shariff threshold)  */
  int    vis;               /* [GENERAL] VIS                                    */
  int    eglib;             /* [GENERAL] EGLIB (EGLIB transport, precision 1)   */
  int    forcesum;          /* [GENERAL] FORCESUM                               */
  int    reaction;          /* [REACTING] REACTION                              */
  int    vis_dt;            /* [TIMESTEPPING] VIS_DT (Fourier criteria)         */
  double cfl, cflmin, cpr, fo;   /* [TIMESTEPPING] CFL CFLMIN CPR FO            */
  int    weno5_linear_fix;  /* 0: reference linear WENO5 stencil (mirrored);
                               1: textbook upwind-biased stencil                 */
} izem_cfg;

/* Species data in code units (thd_type, thd/type_thd.f90:10-92), filled from
 * therm.dat + tranfit.out by thd_init (thd/thd_tools_perfectgas.f90:12-229). */
typedef struct izem_thd {
  int    nspc;
  double gam2;              /* (gamma_inf-1)/gamma_inf                          */
  double tinf;              /* T_ref [K]                                        */
  double pinf, p0;          /* p_ref [Pa], 101325 Pa                            */
  double muinf, laminf;     /* mu_ref [kg/m/s], lambda_ref [W/m/K]              */
  double dinf[IZEM_NSMAX];  /* D_ref [m^2/s]                                    */
  double W[IZEM_NSMAX];     /* molar masses [kg/mol]                            */
  double Wc[IZEM_NSMAX];    /* W / W_ref                                        */
  double Wc_i[IZEM_NSMAX];  /* 1 / Wc                                           */
  double tpolymin[IZEM_NSMAX], tpolymax[IZEM_NSMAX], tpolylim[IZEM_NSMAX];
  double heatcap[IZEM_NSMAX][2][7];   /* [species][0 low / 1 high][a1..a7]      */
  double cofd[IZEM_NSMAX][IZEM_NSMAX][IZEM_NPOLY]; /* ln D_kl fit in ln T       */
  double coflam[IZEM_NSMAX][IZEM_NPOLY];           /* ln lambda_k fit           */
  double cofeta[IZEM_NSMAX][IZEM_NPOLY];           /* ln eta_k fit              */
} izem_thd;

/* Non-dimensional references (adi_type, module_adim.f90:31-90), computed by
 * constants (module_tools.f90:453-571). */
typedef struct izem_adi {
  double gamma_inf, re, pr, le, ma, sc;
  double sqgmr, ggmopr;
  double t_ref, l_ref, r_ref, w_ref, cp_ref, mu_ref, c_inf, u_ref, time_ref;
  double rho_ref, p_ref, lbda_ref, d_ref;
} izem_adi;

/* Gas-phase mechanism in CHEMKIN-II form (the linking data that ckinterp
 * writes to chem.bin and CKINIT reads, devel-izem/src/chemkin/vode.f:391):
 * species molar masses, NASA-7 thermo with CHEMKIN's mid-temperature switch,
 * and per reaction: stoichiometry (up to 3 reactants, 3 products), forward
 * Arrhenius (A, b, E/R), reverse kind, third-body efficiencies, fall-off
 * (LOW with the Lindemann, SRI or Troe broadening of CKRATX,
 * vode.f:1185-1236; the collider (+M) or one species (+K)), Landau-Teller
 * factors (CKRATT, vode.f:973-981, 1032-1041).  Units: mol, cm, s, K,
 * erg.  The last four members were added after the others; a zero-filled
 * tail means no SRI reaction, (+M) colliders and no Landau-Teller factor. */
#define IZEM_MAXREAC 32
typedef struct izem_mech {
  int    kk, ii;
  double ru, patm;                        /* erg/mol/K, dyn/cm^2              */
  double wt[IZEM_NSMAX];                  /* g/mol                           */
  double tmid[IZEM_NSMAX];                /* T > tmid: high-T coefficients    */
  double a[IZEM_NSMAX][2][7];             /* [k][0 low / 1 high][a1..a7]      */
  int    nuk[IZEM_MAXREAC][6];            /* species index, -1 = none;
                                             slots 0-2 reactants, 3-5 products */
  int    nu[IZEM_MAXREAC][6];             /* stoichiometric coefficients      */
  double par[IZEM_MAXREAC][3];            /* A, b, E/R                        */
  int    rev[IZEM_MAXREAC];               /* 0 irreversible, 1 equilibrium,
                                             2 explicit REV                   */
  double rpar[IZEM_MAXREAC][3];           /* REV A, b, E/R                    */
  int    thb[IZEM_MAXREAC];               /* 1: +M or (+M) third body         */
  double eff[IZEM_MAXREAC][IZEM_NSMAX];   /* third-body efficiencies          */
  int    fall[IZEM_MAXREAC];              /* 0 none, 1 Lindemann, 2 SRI,
                                             3/4 Troe with 3/4 parameters     */
  double low[IZEM_MAXREAC][3];            /* LOW A, b, E/R                    */
  double troe[IZEM_MAXREAC][4];           /* a, T***, T*, T**                 */
  double sri[IZEM_MAXREAC][5];            /* SRI a, b [K], c [K], d, e        */
  int    kfal[IZEM_MAXREAC];              /* fall-off collider: 0 (+M), k+1
                                             species k alone, (+K)            */
  double lt[IZEM_MAXREAC][2];             /* Landau-Teller B, C of the forward
                                             rate: k_f exp(B/T^1/3 + C/T^2/3);
                                             0, 0 for none                    */
  double rlt[IZEM_MAXREAC][2];            /* the same for an explicit (REV)
                                             reverse rate (RLT)               */
} izem_mech;

/* EGLIB linking data (the contents of the Linkeg file that EGINI reads,
 * devel-izem/src/eglib/EGini.f:265-276): per species molar mass, geometry
 * (0 atom, 1 linear, 2 nonlinear), Lennard-Jones eps/k [K] and diameter
 * [Angstrom], dipole [Debye], polarizability [Angstrom^3], rotational
 * relaxation number at 298 K, and the fits ln(eta [g/cm/s]) and
 * ln(D_kl [cm^2/s] at 1 atm) as cubics in ln T.  Used by the EGLIB
 * precision-1 viscous flux (cfg.eglib = 1). */
typedef struct izem_eglib {
  int    ns;
  int    lin[IZEM_NSMAX];
  double wt[IZEM_NSMAX], eps[IZEM_NSMAX], sig[IZEM_NSMAX];
  double dip[IZEM_NSMAX], pol[IZEM_NSMAX], zrot[IZEM_NSMAX];
  double cofe[IZEM_NSMAX][4];
  double cofd[IZEM_NSMAX][IZEM_NSMAX][4];
} izem_eglib;

typedef struct izem_ctx izem_ctx;

/* Create a context on the current CUDA device.  Allocates the device-resident
 * state (v, T, W_i, cp, ha, shock sensor) and the RK3 scratch (v0, f).
 * Supported: ng = 3 (WENO5) or ng = 4 (WENO7), two or nine species, in 3-D
 * or 2-D; ndim = 2 needs nz = 1 (no z sweep, no z derivatives); EGLIB
 * transport in 3-D.  Other configurations return IZEM_ERR_ARG.
 * Replaces the allocations at module_solver.f90:736-739 and the per-call
 * temporaries of module_weno.f90:588-607, module_viscflux.f90:1708-1714. */
int  izem_gpu_init(const izem_cfg* cfg, const izem_thd* thd, const izem_adi* adi,
                   izem_ctx** out);
void izem_gpu_destroy(izem_ctx* ctx);
int  izem_gpu_last_error(izem_ctx* ctx, char* buf, int n);

/* Newton temperature solves (prim_inv_var, module_thermodynamics.f90:79-186):
 * the most iterations any sub-domain needed, and the number of solves that
 * reached itmax without meeting the stopping test (the reference's
 * "WARNING: failure in temperatures convergence", :161), counted since the
 * context was created or since the last call with reset != 0.  Every solve
 * iterates until the reference's test holds or itmax (200; 100 for the
 * initial-condition closure) iterations have run. */
int  izem_gpu_newton_stats(izem_ctx* ctx, int* max_iters, int* unconverged, int reset);

/* Inverted metrics dx_i(sx-ng:ex+ng) etc. (module_tools.f90:223-452, already
 * multiplied by L_ref as in adimensionalize, module_tools.f90:185-187). */
int  izem_gpu_set_grid(izem_ctx* ctx, const double* dx_i, const double* dy_i,
                       const double* dz_i);

/* Host <-> device copies of the ghosted state.  shock_sensor is one byte per
 * ghosted point (Fortran logical converted by the shim).  Any pointer may be
 * NULL to skip that array. */
int  izem_gpu_upload_state(izem_ctx* ctx, const double* v, const double* T,
                           const double* W_i, const double* cp, const double* ha,
                           const uint8_t* shock_sensor);
int  izem_gpu_download_state(izem_ctx* ctx, double* v, double* T, double* W_i,
                             double* cp, double* ha, uint8_t* shock_sensor);
/* Copy the RK flux array f(sx:ex,sy:ey,sz:ez,1:nv) to the host. */
int  izem_gpu_download_flux(izem_ctx* ctx, double* fl);
/* Zero the device flux array (test helper for the accumulating y/z sweeps). */
int  izem_gpu_zero_flux(izem_ctx* ctx);

/* The stage's shock sensor on the device, setting the sticky mask (never
 * cleared): shock_sensor_modified_adams_shariff (module_tools.f90:2733-2814)
 * by default, or compute_duixj + shock_sensor_ducros (:2521-2719) after
 * izem_gpu_set_shock_sensor(ctx, IZEM_SENSOR_DUCROS, ...). */
int  izem_gpu_shock_sensor(izem_ctx* ctx);

/* SHOCK_SENSOR_TYPE and DUCROS_TREDUC (module_input.f90:347-348, defaults
 * ADAMSSHARIFF and 0.2): type IZEM_SENSOR_ADAMS_SHARIFF or
 * IZEM_SENSOR_DUCROS (2-D and 3-D blocks; the flag is set where
 * (div u)^2 / ((div u)^2 + |curl u|^2 + 1e-30) > ducros_treduc, the velocity
 * gradients by dx_fixed1 and its y, z copies).  Takes effect at the next
 * stage; the RK3 graph is captured again. */
int  izem_gpu_set_shock_sensor(izem_ctx* ctx, int type, double ducros_treduc);

/* euler_LLF_x/_y/_z (module_weno.f90:537,1055,1595): dir 0 overwrites f,
 * dir 1 and 2 accumulate into f. */
int  izem_gpu_euler_flux(izem_ctx* ctx, int dir);

/* viscflux_xyz (module_viscflux.f90:1660-2189), or with cfg.eglib = 1
 * viscflux_eg_xyz (module_eg_lib.f90:2140-2676, EGLIB precision 1):
 * accumulates into f. */
int  izem_gpu_visc_flux(izem_ctx* ctx);

/* NR_boundaries (module_BCs.f90:185-212): for each face of kind
 * IZEM_BC_NOREFLECTION in the order W,E,S,N,B,F, bc_noreflectionweno
 * (module_weno.f90:2129-4498) adds to f at the face's boundary points
 * R diag(lambda-) L (dv/dn), with L, R the characteristic vectors at the
 * point's own state, lambda- the eigenvalues leaving the domain (min(.,0) on
 * W, S, B; max(.,0) on E, N, F) and dv/dn the one-sided derivative over
 * 2ng-1 points (wenopar's cnr weights, :199-217).  No-op without such
 * faces. */
int  izem_gpu_nr_flux(izem_ctx* ctx);

/* EGLIB linking data for cfg.eglib = 1 (init_eglib + EGINI,
 * module_eg_lib.f90:44-96, eglib/EGini.f:58-301); call once after
 * izem_gpu_init and before any viscous flux. */
int  izem_gpu_set_eglib(izem_ctx* ctx, const izem_eglib* eglib);

/* upd_prim_var_domain + comm_cons + upd_boundaries + upd_prim_var_ghost
 * (module_BCs.f90:41-296): force_sumY, Newton temperature per sub-domain with
 * the reference's global stopping test, halo wrap / extrapolation. */
int  izem_gpu_update_primitives(izem_ctx* ctx);

/* Initial-condition closure of the reference's init routines (e.g.
 * module_ICs.f90:2874-2879): comm_cons, prim_inv_var_err_mach on the interior,
 * upd_extrapolation, prim_inv_var_err_mach on each ghost face. */
int  izem_gpu_finalize_ic(izem_ctx* ctx);

/* rk3 (module_solver.f90:694-856): three SSP-RK3 stages on the device
 * state, captured once into a CUDA graph and replayed. */
int  izem_gpu_rk3(izem_ctx* ctx, double dt, double time0);

/* timestep (module_solver.f90:202-408): dt_4 and dtmin (non-dimensional).
 * dtmin is in/out: its input value is the previous step's dtmin (used by the
 * chemical criterion), DTmax the previous chemistry's max |dT|.  With
 * cfg.vis and cfg.vis_dt, dt_4[1] and dt_4[2] are the Fourier criteria of
 * mass and thermal diffusion (:294-367) from the mixture-averaged fits, as
 * the reference uses them even under EGLIB; otherwise they stay 1. */
int  izem_gpu_timestep(izem_ctx* ctx, double DTmax, double dt_4[4], double* dtmin);

/* Mechanism for the chemistry steps (the chem.bin data; see izem_mech). */
int  izem_gpu_set_mechanism(izem_ctx* ctx, const izem_mech* mech);

/* reaction_selec with reaction_dvode (module_reaction.f90:47-321): one
 * Strang half step of length dt (code units) on every cell of the interior
 * window (ng+1 cells are skipped at every global face, as in the reference),
 * each integrated as a constant-volume reactor by the BDF method (DVODE
 * MF=22, RTOL 1e-6, ATOL 1e-10, <= 20 restarts) in a persistent
 * work-stealing kernel; then upd_prim_var_woT, comm_cons, upd_boundaries
 * (given `time` and dt, as reaction_selec passes them: the jet faces read
 * them) and the ghost Newton solve.  mode IZEM_CHEM_BDF: the BDF method on
 * every cell; IZEM_CHEM_MLP: the learned surrogate set by
 * izem_gpu_set_surrogate with its error gate, rejected cells by the BDF
 * method (no counterpart in the reference).  DTmax receives max |dT| [K].
 * Blocks with jet faces need izem_gpu_set_coords first. */
enum { IZEM_CHEM_BDF = 0, IZEM_CHEM_MLP = 1 };
int  izem_gpu_chem_step(izem_ctx* ctx, double dt, double time, int mode, double* DTmax);

/* [REACTING] DVODESIMP with Y1F, Y0O, INDEX_H2, INDEX_N2 (module_reaction.f90:
 * 173-251): with enable != 0, mode IZEM_CHEM_BDF integrates only the window
 * cells whose initial production rates move some mass fraction by more than
 * 1e-12 in dt (psr_simp_chemkin: CKWYR x molar mass x dt / rho) and whose H2
 * and N2 both differ by more than 1e-6 from the pure fuel Y_fuel and from the
 * pure oxidiser Y_oxidizer (arrays of nrv mass fractions); the other cells
 * keep their state and do not enter DTmax, and the integrated cells clip the
 * closing species to [0, 1] as that branch does.  index_h2 and index_n2 are
 * 0-based species indices (the deck's INDEX_* minus 1).  enable = 0 restores
 * the integration of every cell.  The reference calls psr_simp_chemkin with
 * four of its five arguments; this is the routine's stated semantics. */
int  izem_gpu_set_chem_skip(izem_ctx* ctx, int enable, const double* Y_fuel, const double* Y_oxidizer,
                            int index_h2, int index_n2);

/* Coordinates of the interior points in code units (x, y, z: nx, ny, nz
 * values; the reference's x/L_ref arrays) and the domain length in x, Lx
 * (module_tools.f90:319,489), for the jet faces IZEM_BC_INFLOWJET (radius
 * sqrt(y^2 + z^2)) and IZEM_BC_NSCBC_OUT (Lx).  Required before
 * izem_gpu_rk3 when a jet face is set; the time0 argument of izem_gpu_rk3
 * then gives the stage times timek = time0 + dt tk3 (module_solver.f90:756),
 * and the time argument of izem_gpu_chem_step the chemistry tail's time. */
int  izem_gpu_set_coords(izem_ctx* ctx, const double* x, const double* y, const double* z, double lx);

/* Parameters of the jet faces.  izem_jet_reference fills the constants that
 * bc_inflowjet (module_BCs.f90:1680-1700) and bc_nscbc_out (:2390) hard-code,
 * which izem_gpu_set_coords installs: a round sonic nozzle of 1 mm with
 * pure fuel at 1000 K and 15 atm into 300 K air at 1 atm and 20 m/s, ramped
 * in as (t / 0.1 ms)^3, and the outflow relaxed toward 94232.25 Pa.  Other
 * values run the same profile formulas with another nozzle (no counterpart
 * in the reference): a planar slot (tanh profile in |y|), a given jet
 * velocity, a fuel/N2 jet, no ramp, and seeded velocity fluctuations
 * u' = turb u_jet (1 - tanh) / 2 r with r uniform in [-1, 1), a hash of the
 * seed, the face point and the stage time's 1 ns interval, on all three
 * components. */
typedef struct izem_jet {
  double width;            /* [m] nozzle diameter, or slot width (planar)        */
  double ramp;             /* [s] ramp time of the nozzle state; 0: none         */
  double T_jet, T_co;      /* [K] nozzle and coflow temperatures                 */
  double p_jet, p_co;      /* [Pa] nozzle and coflow pressures                   */
  double u_jet;            /* [m/s] jet velocity; 0: 1.01 x its sound speed       */
  double u_co;             /* [m/s] coflow velocity                              */
  double y_fuel;           /* H2 mass fraction of the jet (the rest N2)          */
  double p_far;            /* [Pa] far-field pressure of the outflow             */
  double turb;             /* relative amplitude of the fluctuations; 0: none    */
  int    planar;           /* 0: round jet, 1: planar slot                       */
  int    reserved;
  unsigned long long seed; /* seed of the fluctuations                           */
} izem_jet;
void izem_jet_reference(izem_jet* p);
/* Installs p for the jet faces of ctx (after izem_gpu_set_coords). */
int  izem_gpu_set_jet(izem_ctx* ctx, const izem_jet* p);

/* [IFLES] LES = T with MU_SGS_MODEL = SMAGORINSKY: MU_SGS_FACTOR, SC_SGS,
 * PR_SGS and the shock-detector threshold PERCENT_WEIGHT_SGS, with
 * mu_SGS_smagorinsky (module_SGS_models.f90:176-304).
 * - Under EGLIB (cfg.eglib = 1): the viscous fluxes of viscflux_eg_LES_xyz
 *   (module_eg_lib.f90:2687-3352), the criterion of shock_det_slv
 *   (module_tools.f90:1945-2085).  The time step is unchanged: the
 *   reference's mu_SGS array seen by timestep stays 0 under EGLIB.
 * - With the fitted transport: viscflux_LES_xyz (module_viscflux.f90:
 *   2200-2977), the criterion of shock_det_ducros_slv (module_tools.f90:
 *   2099-2181); mu_SGS of every flux evaluation is kept and enters the
 *   Fourier criteria of izem_gpu_timestep (module_solver.f90:294-367).
 * TAU_ISO_SGS_SWITCH = F (the deck default): the isotropic SGS tensor is not
 * built.  Needs cfg.vis and ndim = 3; enable = 0 restores the laminar
 * fluxes (and zeroes the kept mu_SGS). */
int  izem_gpu_set_les(izem_ctx* ctx, int enable, double mu_sgs_factor, double sc_sgs, double pr_sgs,
                      double percent_weight_sgs);
/* Statistics of the last chemistry step: cells whose integration failed
 * (ISTATE <= -2), largest and summed BDF step counts. */
int  izem_gpu_chem_stats(izem_ctx* ctx, int* failed, int* max_steps, unsigned long long* total_steps);

/* Independent constant-volume reactors (PSR_CHEMKIN per cell, chemkin/
 * psr_chemkin.f): T [K] in/out, rho [g/cm^3], Y (n rows of kk) in/out,
 * dt [s] per cell.  istate/nsteps may be NULL.  With device_ptrs = 1 every
 * array is a device pointer (no copies); kernel_ms receives the kernel time. */
int  izem_gpu_psr_batch(const izem_mech* mech, int n, double* T, const double* rho, double* Y,
                        const double* dt, int* istate, int* nsteps, int device_ptrs, float* kernel_ms);

/* ---- learned chemistry surrogate (no counterpart in the reference) -------
 * A 12 -> 4 x 256 (GELU) -> 10 MLP, BF16 weights and activations with FP32
 * accumulation on the tensor cores, trained on the GPU (Adam) on samples
 * labelled by izem_gpu_psr_batch.  Inputs: T [K], ln p [atm], ln(Y+1e-10)
 * for the 9 species, ln dt [s]; outputs dY (9) and dT [K]; both normalised
 * by norm = {in_mean[12], in_std[12], out_mean[10], out_std[10]}.
 * Parameters W_l are [in][out] row-major FP32 with padded sizes
 * 16-256-256-256-256-16. */
typedef struct izem_mlp izem_mlp;
int  izem_mlp_create(izem_mlp** out);
void izem_mlp_destroy(izem_mlp* m);
int  izem_mlp_set_params(izem_mlp* m, const float* const* W, const float* const* b);
int  izem_mlp_get_params(izem_mlp* m, float* const* W, float* const* b);
int  izem_mlp_set_norm(izem_mlp* m, const float* norm);
int  izem_mlp_forward(izem_mlp* m, int M, const float* x, float* y);
int  izem_mlp_grads(izem_mlp* m, int M, const float* x, const float* t, double* loss,
                    float* const* gW, float* const* gb);
int  izem_mlp_train(izem_mlp* m, long long n, const float* x, const float* t, int device_ptrs,
                    int epochs, int batch, float lr, unsigned seed, double* losses);
/* Surrogate chemistry step on independent reactors with the per-cell error
 * gate (training envelope, a cap on the predicted |dT|, element conservation
 * of dY, internal-energy consistency of dT, agreement with a second
 * independently trained network m2 when m2 is not NULL, the prediction then
 * being the mean of the two); rejected cells are integrated by the BDF
 * method (no counterpart in the reference).
 * gate10 = {Tmin, Tmax, dtmin, dtmax, tol_el, tol_T_abs, tol_T_rel,
 * tol_ens_abs, tol_ens_rel, dT_cap}; kncf[kk][nele] element counts; stats3 =
 * {fallback cells, max BDF steps, failed cells}; ms2 = {total ms, MLP ms}. */
int  izem_gpu_psr_batch_mlp(izem_mlp* m, izem_mlp* m2, const izem_mech* mech, int n, double* T,
                            const double* rho, double* Y, const double* dt, int device_ptrs,
                            const double* gate10, const int* kncf, int nele, double* dT_pred,
                            int* stats3, float* ms2);
/* Target form of a network (no counterpart in the reference): residual = 1
 * when it was trained on the chemistry increment minus the explicit one,
 * dt f(y0) with f the reactor right-hand side at the start state; the gated
 * step then adds dt f(y0) back before its tests.  Both networks of an
 * ensemble must have the same form.  Default 0. */
int  izem_mlp_set_residual(izem_mlp* m, int residual);
/* The constant-volume reactor right-hand side dz/dt, z = [T, Y_1..Y_9]
 * (FUN of REACTION_V, chemkin/reaction_v.f), at n states: T [K], rho
 * [g/cm^3], Y (n x 9) -> zdot (n x 10).  Device arrays when device_ptrs,
 * host arrays otherwise. */
int  izem_gpu_reactor_rhs(const izem_mech* mech, int n, const double* T, const double* rho, const double* Y,
                          double* zdot, int device_ptrs);
/* The cells that the last izem_gpu_psr_batch_mlp call on m sent to the BDF
 * integrator (no counterpart in the reference): their indices in that
 * call's batch, in no particular order; up to cap of them are written to
 * out (host memory), and *count receives their number. */
int  izem_mlp_fallback_cells(izem_mlp* m, int* out, int cap, int* count);
/* No counterpart in the reference.  Inference for callers that cannot
 * allocate device memory while they run -- a solver whose own arena (or a
 * framework's caching allocator) already holds the GPU's memory, or one that
 * calls the surrogate inside its time-step loop, where cudaMalloc/cudaFree
 * would synchronise the whole device.  It runs the tensor-core inference
 * kernel of izem_mlp_forward on the same BF16 inputs, so the two give the
 * same outputs bit for bit.
 * d_x (M x 12) and d_y (M x 10) are FP32 device arrays, the work is queued
 * on `stream` (a cudaStream_t; NULL is the default stream) and the call
 * returns without waiting.  The device that was current when the handle
 * was created must be current for the call (its weights live there);
 * otherwise the call returns IZEM_ERR_ARG.  No memory is allocated or freed:
 * the kernel's BF16 inputs and FP32 outputs use one fixed device array of
 * 384 KiB per GPU, which
 * every GPU that loads the library holds until the process exits, so M is
 * at most IZEM_MLP_NOALLOC_MAX_ROWS (larger M returns IZEM_ERR_TOO_LARGE;
 * split the batch).  The first call on a device looks up that array's
 * address; make it before any stream capture.  All calls share the array:
 * calls that may overlap on the GPU (different streams, or several host
 * threads) race and must be serialised by the caller.  The handle's
 * parameters are allocated once by izem_mlp_create. */
#define IZEM_MLP_NOALLOC_MAX_ROWS 4096
int  izem_mlp_forward_noalloc(izem_mlp* m, int M, const float* d_x, float* d_y, void* stream);
/* Surrogate used by izem_gpu_chem_step(..., IZEM_CHEM_MLP, ...): networks m
 * (and optional partner m2, see izem_gpu_psr_batch_mlp), gate10 and the
 * element counts kncf[nrv][nele] (no counterpart in the reference).  The
 * handles stay owned by the caller.  izem_gpu_chem_surrogate_stats reports
 * the last such step: window cells, cells sent to the BDF method, total and
 * network-only milliseconds. */
int  izem_gpu_set_surrogate(izem_ctx* ctx, izem_mlp* m, izem_mlp* m2, const double* gate10,
                            const int* kncf, int nele);
int  izem_gpu_chem_surrogate_stats(izem_ctx* ctx, long long* cells, int* fallback, float* ms_total,
                                   float* ms_network);

/* Autotuning (no counterpart in the reference): times the candidate thread
 * blocks (64, 128, 256) of the face-flux and viscous point kernels on the
 * context's current state, and -- when a mechanism is set and chem_dt > 0
 * -- the register-budget variants of the persistent chemistry kernels
 * (128 threads, 8 to 4 resident blocks per SM) on a copy of the reaction
 * window for a half step chem_dt (code units); keeps the fastest of each.
 * The flow kernels' results do not depend on the choice; the chemistry
 * variants are separate compilations of the same source, whose results
 * agree within the integrator's tolerance (the compiler may fuse a multiply
 * and an add differently under another register limit).  report (may be
 * NULL, at least 2048
 * bytes otherwise) receives the timings as JSON.  Call after the state is
 * uploaded, before the timed steps. */
int  izem_gpu_autotune(izem_ctx* ctx, double chem_dt, char* report, int report_len);
/* Pins the register-budget variant of the persistent chemistry kernels
 * (0..4: 128 threads and 8 - v resident blocks per SM) for every context of
 * the process, as izem_gpu_autotune would choose it (no counterpart in the
 * reference); IZEM_ERR_ARG outside 0..4. */
int  izem_gpu_set_chem_variant(int variant);
/* 1 when the chemistry kernels evaluate the reactor right-hand side from
 * code generated for the mechanism last passed to izem_gpu_set_mechanism
 * (the shipped H2/air mechanism; the same operations in the same order as
 * the table-driven form, with the tables as literals), 0 when they walk the
 * mechanism's tables (any other mechanism).  No counterpart in the
 * reference. */
int  izem_gpu_chem_generated(void);
/* FP64 FMA throughput of the current device in GFLOP/s (8 independent FMA
 * chains per thread over 8 x 256 threads per SM, best of three timed
 * launches): the FP64 peak the rooflines are quoted against.  No
 * counterpart in the reference. */
int  izem_gpu_fp64_rate(double* gflops);
/* Checks the bounded waits of the tensor-core kernels (no counterpart in the
 * reference): a kernel polls an mbarrier that nothing arrives on `polls`
 * times (1 .. 2^20), as those kernels poll theirs, and *gave_up receives 1
 * when it stopped waiting (always, on a working device); the context stays
 * usable. */
int  izem_gpu_wait_selftest(int polls, int* gave_up);
/* allow = 0 makes the chemistry kernels walk the mechanism's tables even
 * for the shipped mechanism (to compare the two forms); allow = 1 (the
 * default) uses the generated form whenever it applies.  Takes effect at
 * the next izem_gpu_set_mechanism / izem_gpu_psr_batch. */
int  izem_gpu_allow_chem_generated(int allow);
/* Reproduce a run of the reference decomposed into nblk equal MPI blocks
 * along x (its NUMPROCX) on this single context: the reference never
 * exchanges the shock sensor, so each block tests only its own points
 * (module_tools.f90:2761-2770) and picks nonlinear weights from its own
 * flags (module_weno.f90:973), and the face on a block edge is computed
 * twice, once as each neighbouring block sees it.  Each rank also runs the
 * Newton loop of prim_inv_var (module_thermodynamics.f90:79-186) and its
 * stopping test on its own points: the interior and the y / z ghost slabs
 * stop per x-block.  nblk = 1 (the default) is one block.  No counterpart
 * as an entry point in the reference; IZEM_ERR_ARG unless nblk (at most 8)
 * divides nx into blocks of at least ng points. */
int  izem_gpu_set_sensor_xblocks(izem_ctx* ctx, int nblk);
/* The same choice for independent reactors (no counterpart in the
 * reference): times the five variants on the first min(n, 2^20) reactors of
 * a batch laid out as for izem_gpu_psr_batch (copies; the caller's arrays
 * are not changed) and keeps the fastest for the process.  report (may be
 * NULL) receives the timings as JSON. */
int  izem_gpu_chem_autotune(const izem_mech* mech, int n, const double* T, const double* rho, const double* Y,
                            const double* dt, int device_ptrs, char* report, int report_len);

/* Device timing of the calls above on the context's stream (CUDA events). */
int  izem_gpu_timer_start(izem_ctx* ctx);
int  izem_gpu_timer_stop(izem_ctx* ctx, float* ms);
/* Per-kernel timing: when enabled, every kernel launch is bracketed by CUDA
 * events on the context's stream; izem_gpu_kernel_times returns, for each
 * kernel id, the launch count and the summed device milliseconds. */
int  izem_gpu_set_kernel_timing(izem_ctx* ctx, int enable);
int  izem_gpu_kernel_times(izem_ctx* ctx, int max_kernels, char* names, int name_len,
                           int* launches, double* ms, int* n_kernels);
int  izem_gpu_synchronize(izem_ctx* ctx);

/* Helper used by the host to build dx_i: dscalar on the global coordinate
 * array (module_deriv.f90:80-205) followed by the inversion in metrics
 * (module_tools.f90:424-426).  coord has n entries; d_i receives n entries. */
int  izem_metrics_dscalar(int n, int ng, const double* coord, double* d_i);

/* sizeof of the three configuration structures, for binding generators and
 * layout checks (izem_cfg, izem_thd, izem_adi).  No device call. */
int  izem_abi_sizes(size_t* cfg, size_t* thd, size_t* adi);

#ifdef __cplusplus
}
#endif
#endif /* IZEM_GPU_H */

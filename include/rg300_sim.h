/*
 * rg300 standalone time stepping -- C ABI.
 *
 * Replaces EQS_UVS2D::Execute (EqsUVS2D.cpp:71-1096) for decks that the
 * reference reads from its region/control/time-step/material files, when the
 * caller has no reference MODEL to hand over: the library builds the wet
 * model, boundary elements, boundary conditions, equation numbering and CRS
 * pattern itself (MODEL::Initialize Model.cpp:121, BCONSET::InitBcon
 * BconSet.cpp:92, EQS::SetEqno SetEqno.cpp:52, EQS::SetIndexMat
 * IndexMat.cpp:91) and runs every Newton iteration on the GPU.
 *
 * Supported subset: six-node triangles, Manning friction (TYPE::friction
 * kMANN), constant eddy viscosity (kVtConstant), no dispersion, QINLET /
 * QTINLET discharge inlets, OUTLET water level, automatic slip walls,
 * dry/rewet method 2 (GRID::DryRewet DryRewet.cpp:696), relaxation method 0
 * or 2.
 */
#ifndef RG300_SIM_H
#define RG300_SIM_H

#include "rg300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rg_sim rg_sim;

typedef enum { RG_BC_QINLET = 1, RG_BC_QTINLET = 2, RG_BC_OUTLET = 3 } rg_bc_kind;

/* one $TM_LINE boundary condition (Timeint.cpp:2240-2345) */
typedef struct {
  int           kind;          /* rg_bc_kind */
  int           line;          /* control-line number (material id of the line elements) */
  int           npts;          /* 1 for QINLET/OUTLET, hydrograph length for QTINLET */
  const double* t;             /* QTINLET times [s] */
  const double* Q;             /* discharge [m^3/s] (inlets) */
  const double* S;             /* water level [m] (QINLET profile level, OUTLET level) */
} rg_line_bc;

/* $RELAX, $DRYREW, $CONVERGENCE, $SOLVER, $TM_WEIGHT, physical constants */
typedef struct {
  double g, vk;                /* PROJECT::g, PROJECT::vk */
  double dry_limit, rewet_limit;
  int    dryrew_method, dryrew_freq, countdown;
  int    relax_method;         /* 0 or 2 */
  double max_delta_uv, max_delta_s, max_us;
  double conv_uv, conv_s;      /* correction criterion (EqsUVS2D.cpp:436-438) */
  int    max_newton;           /* PROJECT::actualCycit */
  int    solver_maxiter;       /* $SOLVER maxIter */
  double solver_maxdiff;       /* $SOLVER maxDiff */
  double theta;                /* TIMEINT::thetaFlow */
} rg_deck_params;

typedef struct {
  int           np;            /* region nodes */
  const double* x;
  const double* y;
  const double* z;             /* bed elevation (NODE::zor) */
  int           ne;            /* region six-node triangles */
  const int*    elem_nodes;    /* 6 per triangle: corners ccw, then mid-sides 0-1, 1-2, 2-0 */
  const int*    elem_mat;      /* material index per triangle */
  int           nmat;
  const double* mat_n;         /* Manning n ($BOTTOM no MANN n) */
  const double* mat_vt;        /* eddy viscosity ($TURBULENCE no vt) */
  int           nseg;          /* control-line segments (corner, corner, mid-side) */
  const int*    seg_nodes;
  const int*    seg_line;
  int           nbc;
  const rg_line_bc* bc;
  rg_deck_params params;
} rg_deck;

typedef enum {
  RG_CRIT_CORRECTION = 0,      /* the reference's test: max |correction| <= convUV / convS */
  RG_CRIT_RESIDUAL   = 1       /* ||B_k||_2 / ||B_0||_2 <= residual_tol */
} rg_criterion;

typedef struct {
  int    steady;               /* $TM_STATIONARY */
  int    first_step;           /* first time step of the run (EQS_UVS2D::Predict) */
  int    criterion;            /* rg_criterion */
  double residual_tol;
  int    max_newton;           /* 0: params.max_newton */
  /* 0: every Newton iteration's BiCGStab runs to $SOLVER maxDiff (the
   * reference).  > 0: inexact Newton -- BiCGStab stops at the relative
   * residual max(maxDiff, linear_forcing); the Newton convergence test and
   * the converged solution are unchanged, the path to it takes fewer Krylov
   * iterations.  No counterpart in the reference. */
  double linear_forcing;
  /* 0: ILU(0) is factored in every Newton iteration (the reference).  n > 0:
   * the resident factors precondition up to n further Newton iterations (also
   * across time steps) while the numbering is unchanged; a solve with reused
   * factors that misses its tolerance (or breaks down) is repeated at once
   * with fresh factors.  No counterpart in the reference. */
  int    ilu_reuse;
  /* 0: the reference's Jacobian.  1: the Jacobian also carries the depth
   * derivative of the nodal Manning coefficient (rg_set_jacobian); the
   * residual, hence the converged solution, is unchanged.  No counterpart in
   * the reference. */
  int    friction_jacobian;
} rg_step_ctl;

typedef struct {
  int    newton_iterations;
  int    krylov_iterations;
  int    converged;
  int    neq;
  int    dryrew_events;
  int    dry_nodes;
  int    solver_status;
  int    n_hist;
  double residual_first;       /* ||B_0|| */
  double residual_ratio;       /* last ||B_k|| / ||B_0|| */
  double wall_ms;
  double residual_hist[64];
  int    warm_start;           /* 1: the step started from the state given to rg_sim_set_warm_start */
  double residual_warm;        /* ||B|| at that state (-1: none given) */
} rg_step_report;

/* device >= 0: GPU ordinal; RG_DEVICE_NONE: host model only (numbering and
 * boundary set-up can be inspected, rg_sim_step is refused) */
#define RG_DEVICE_NONE (-2)
rg_status rg_sim_create(const rg_deck* deck, int precision, int device, rg_sim** out);
rg_status rg_sim_destroy(rg_sim* sim);
const char* rg_sim_last_error(rg_sim* sim);
/* initial state ($ASC_INITFILE U V S); sets up the model as PROJECT::Compute
 * does before its time loop (Compute.cpp:170-180) */
rg_status rg_sim_set_state(rg_sim* sim, const double* U, const double* V, const double* S);
rg_status rg_sim_get_state(rg_sim* sim, double* U, double* V, double* S, double* z, int* nflag);
/* one time step [t, t+dt] (EQS_UVS2D::Execute + Compute.cpp:774-810) */
rg_status rg_sim_step(rg_sim* sim, double t, double dt, const rg_step_ctl* ctl, rg_step_report* rep);
/* Starting state of the next rg_sim_step's Newton iteration (e.g. the learned
 * prediction of include/rg300_mlp.h), used once: after the step's first
 * dry/rewet pass it replaces U, V, S on the wet nodes (mid-side S as corner
 * means, depth at least half the dry limit, velocity at slip-wall and inlet
 * nodes projected onto the free direction), and is kept only if its residual
 * ||B|| is below that of the last time level; the step's ||B_0|| stays the
 * last time level's, so the convergence target is unchanged.  NULL arrays
 * cancel a pending start.  No counterpart in the reference
 * (EQS_UVS2D::Predict, EqsUVS2D.cpp:1101, starts from the last time level). */
rg_status rg_sim_set_warm_start(rg_sim* sim, const double* U, const double* V, const double* S);
/* host wall time of the stages of rg_sim_step since the last reset, in ms
 * (indices rg_sim_stage; device work is included where the stage waits for
 * it).  ms[0..n-1] receive the sums; reset != 0 zeroes them afterwards. */
typedef enum {
  RG_STAGE_DRYREWET = 0,       /* dry/rewet passes on the host */
  RG_STAGE_FRICTION = 1,       /* nodal friction (GPU) */
  RG_STAGE_BCON = 2,           /* boundary conditions, location, normals, rotation (host) */
  RG_STAGE_NUMBERING = 3,      /* numbering and pattern after a model change (host) */
  RG_STAGE_UPLOAD = 4,         /* state, model and boundary uploads */
  RG_STAGE_DOWNLOAD = 5,       /* state downloads */
  RG_STAGE_ASSEMBLE = 6,       /* assembly and scaling (GPU) */
  RG_STAGE_FACTOR = 7,         /* ILU(0) factorisation (GPU) */
  RG_STAGE_KRYLOV = 8,         /* BiCGStab (GPU) */
  RG_STAGE_UPDATE = 9,         /* Newton update and time derivatives (GPU) */
  RG_STAGE_WARM = 10,          /* warm start: applying and testing the predicted start */
  RG_SIM_NSTAGE = 11
} rg_sim_stage;
rg_status rg_sim_stage_ms(rg_sim* sim, double* ms, int n, int reset);
/* MODEL::Continuity (Contin.cpp:43-170) of the simulation's current state on
 * the GPU in FP64: the discharge through every control line (section k+1 =
 * line number k+1, nsect = the largest line number).  With nsect_out only
 * (Qx = Qy = NULL) returns the section count. */
rg_status rg_sim_continuity(rg_sim* sim, int* nsect_out, double* Qx, double* Qy);
/* the host part of one Newton iteration's set-up with the given nodal
 * friction (InitBcon at time t_bc, SetLocation, SetNormal, SetRotation,
 * SetEqno when the model changed) -- no GPU work */
rg_status rg_sim_prepare_iteration(rg_sim* sim, double t_bc, const double* cf);
/* one dry/rewet pass on the host state (MODEL::DoDryRewet, DoDryRew.cpp:50) --
 * the first Newton iteration of a step starts with it */
rg_status rg_sim_dry_rewet(rg_sim* sim, int* dried, int* wetted);
/* the numbering, pattern and boundary data of the last Newton iteration */
rg_status rg_sim_get_numbering(rg_sim* sim, int* neq, int* eqno, int* width, int64_t* nnz);
rg_status rg_sim_get_pattern(rg_sim* sim, int* index);
rg_status rg_sim_get_boundary(rg_sim* sim, int* nflag, int* bckind, double* rot4, double* bcU, double* bcS);
/* the model element list of the last model build (MODEL::Initialize
 * Model.cpp:121-216): *ne elements, 6 node slots each (boundary lines use the
 * first three: corner, corner, mid-side), node count (6 or 3), ELEM::flag and
 * eddy viscosity; plus the open-boundary normal per node (NODE::niox/nioy).
 * NULL skips an output; call with only `ne` first to size the arrays. */
rg_status rg_sim_get_model(rg_sim* sim, int* ne, int* elem_nodes, int* elem_nnd, int* elem_flag, double* elem_vt,
                           double* niox, double* nioy);

/* the GPU context of a simulation (for rg_get_stats, rg_event_*, timings) */
rg_ctx* rg_sim_context(rg_sim* sim);

/* context-level helpers used by the time stepper (also usable by a caller that
 * drives rg_ctx itself) */
/* replace the model element list (MODEL::Initialize after dry/rewet) */
rg_status rg_set_elements(rg_ctx* ctx, int ne, const int* elem_nodes, const int* elem_nnd,
                          const int* elem_flag, const double* elem_vt);
/* previous time level NODE::vo (U, V, S and their time derivatives) */
rg_status rg_set_old(rg_ctx* ctx, const double* U, const double* V, const double* S,
                     const double* dUdt, const double* dVdt, const double* dSdt);
rg_status rg_get_dt(rg_ctx* ctx, double* dUdt, double* dVdt, double* dSdt);
/* EQS_UVS2D::Timegrad (EqsUVS2D.cpp:1183-1230) on the device state */
rg_status rg_timegrad(rg_ctx* ctx, double dt, double theta);
/* U = V = 0 at the listed nodes (kNoMoment, Transform.cpp:441-449) */
rg_status rg_zero_velocity(rg_ctx* ctx, int n, const int* nodes);

#ifdef __cplusplus
}
#endif

#endif

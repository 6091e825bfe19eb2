/*
 * rg300 -- GB300-native Newton step of Rismo2D's depth-averaged shallow-water
 * equations (Taylor-Hood P2 velocity / P1 water level), C ABI.
 *
 * The library replaces the hot path of EQS_UVS2D::Execute (EqsUVS2D.cpp:71):
 * element assembly (EQS_UVS2D::Coefs, CoefsUVS2D.cpp:49) into the CRS matrix
 * (CRSMAT::AssembleEqs_im, Assemble.cpp:195), L2 scaling (CRSMAT::ScaleL2Norm,
 * CRSMat.cpp:319), ILU(0) (PRECO_ILU0::Factor/Solve, Preco_ilu0.cpp:64/497),
 * right-preconditioned BiCGStab (BICGSTAB::Iterate, Bicgstab.cpp:66) and the
 * Newton correction (EqsUVS2D.cpp:455-759), all on one GPU.
 *
 * Conventions
 *  - plain pointers and sizes; every array argument is HOST memory unless the
 *    name ends in _dev; nothing here takes or returns framework types;
 *  - node arrays are indexed by the reference's region node index
 *    (NODE::Getno()); element arrays follow the model element list built by
 *    MODEL::Initialize (Model.cpp:121-216): each wet region triangle followed by
 *    the boundary line elements of its boundary mid-side nodes;
 *  - flag words are the reference's bit values (NODE::flag, ELEM::flag,
 *    BCON::kind; Node.h, Elem.h, Bcon.h);
 *  - every function returns an rg_status; no exception or exit() crosses the
 *    ABI.  A context is not thread-safe: use one host thread per context.
 */
#ifndef RG300_H
#define RG300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  RG_OK               = 0,
  RG_NOT_CONVERGED    = 1,   /* solver did not reach maxDiff: kErr_some_errors (Project.h:236-241) */
  RG_ERR_ARG          = 10,  /* invalid argument or call order */
  RG_ERR_CUDA         = 11,  /* CUDA runtime error (message in rg_last_error) */
  RG_ERR_ZERO_PIVOT   = 12,  /* ILU(0) pivot not repairable (Preco_ilu0.cpp:134-138) */
  RG_ERR_DEVICE_WAIT  = 13,  /* a bounded device-side wait ran out (dependency never satisfied) */
  RG_ERR_NONFINITE    = 14   /* NaN/Inf in a residual or dot product */
} rg_status;

typedef enum {
  RG_PREC_FP64  = 0,   /* plain FP64: Jacobian, matrix, ILU(0), Krylov vectors in double */
  RG_PREC_REF32 = 1,   /* the reference's storage: float matrix and ILU (REALPR, Defs.h:92),
                          double vectors and element arithmetic */
  RG_PREC_MIXED = 2    /* FP32 Jacobian, matrix, ILU(0) and Krylov inside FP64 iterative
                          refinement; FP64 residual B */
} rg_precision;

typedef struct rg_ctx rg_ctx;

/* Mesh and constants.  Replaces the data the reference reads through
 * MODEL::elem / NODE / TYPE / PROJECT (Model.h:113-120, Node.h, Type.h:172,
 * Project.h:435-445). */
typedef struct {
  int           np;            /* region nodes */
  const double* x;             /* np */
  const double* y;             /* np */
  int           ne;            /* model elements (region triangles + boundary lines) */
  const int*    elem_nodes;    /* 6 per element; lines use (corner, corner, mid-side) */
  const int*    elem_nnd;      /* 6 = P2 triangle, 3 = boundary line */
  const int*    elem_flag;     /* ELEM::flag (kBound 16, kInlet 1, kOutlet 2, kOpenBnd 4, kDry 128) */
  const double* elem_vt;       /* constant eddy viscosity of the element's material (TYPE::vt) */
  double        g;             /* PROJECT::g */
  double        hmin;          /* PROJECT::hmin = dryLimit / 2 (Project.cpp:1125) */
  double        vk;            /* PROJECT::vk kinematic viscosity */
} rg_mesh;

/* Create a context on CUDA device `device` (the caller's current device when
 * negative).  Replaces EQS_UVS2D construction plus the SHAPE tables
 * (Shape.cpp:89-205). */
rg_status rg_create(const rg_mesh* mesh, int precision, int device, rg_ctx** out);
rg_status rg_destroy(rg_ctx* ctx);
const char* rg_last_error(rg_ctx* ctx);
const char* rg_version(void);

/* Equation numbers and CRS pattern in the reference's layout
 * (EQS::SetEqno SetEqno.cpp:52-225, EQS::SetIndexMat IndexMat.cpp:91-342,
 * CRSMAT CRSMat.h:71-97): width[neq]; index holds the rows back to back, the
 * diagonal first in each row; eqno holds U, V, S equation numbers per node
 * (-1 = no equation).  Builds the element colouring, the element->CRS slot map
 * and the ILU(0) dependency schedule.  Call again whenever the reference
 * renumbers (model change after dry/rewet). */
rg_status rg_set_pattern(rg_ctx* ctx, int neq, const int* width, const int* index, const int* eqno);

/* Boundary data of the current Newton iteration (MODEL::SetRotation
 * Transform.cpp:269, BCONSET::InitBcon BconSet.cpp:92): NODE::flag, BCON::kind,
 * rotation matrix rows (rot[4*n+0..3] = Getrot(0,0),(0,1),(1,0),(1,1)),
 * open-boundary normal (niox, nioy), BCVAL::U (specific inflow) and BCVAL::S. */
rg_status rg_set_boundary(rg_ctx* ctx, const int* nflag, const int* bckind, const double* rot,
                          const double* niox, const double* nioy, const double* bcU, const double* bcS);

/* Node state (NODE::v, NODE::z, NODE::cf, NODE::cfw); NULL leaves a field unchanged. */
rg_status rg_set_state(rg_ctx* ctx, const double* U, const double* V, const double* S,
                       const double* dUdt, const double* dVdt, const double* dSdt,
                       const double* z, const double* cf, const double* cfw);
rg_status rg_get_state(rg_ctx* ctx, double* U, double* V, double* S, double* z);

/* 1/(theta dt) factors of the current iteration (EQS_UVS2D::relaxThdt_UV/_H,
 * EqsUVS2D.cpp:105-148). */
rg_status rg_set_relax(rg_ctx* ctx, double relaxThdt_UV, double relaxThdt_H);

/* Jacobian option, no counterpart in the reference.  friction_depth = 1 adds
 * to the U-H and V-H blocks the derivative of the bottom friction cf*|U|*U
 * (cf*|U|*V) with respect to the corner depths through the nodal Manning
 * coefficient: cf_k = C_k / max(h_k, hmin)^0.333333 (MODEL::DoFriction,
 * DoFriction.cpp:87-206) gives dcf_k/dh_k = -0.333333 cf_k / h_k above hmin.
 * The reference's Jacobian (CoefsUVS2D.cpp:749-1059) holds cf fixed, so its
 * Newton iteration converges only linearly where friction dominates (shallow
 * water).  The residual is unchanged: the converged solution is the same,
 * only the Newton path changes.  0 (default) restores the reference's
 * Jacobian. */
rg_status rg_set_jacobian(rg_ctx* ctx, int friction_depth);

/* Polling limit of the bounded device waits of the dependency-driven ILU(0)
 * factorisation and triangular solves (0 restores the built-in 2^20 polls).
 * A wait that runs out makes the call return RG_ERR_DEVICE_WAIT with the
 * kernel, row and awaited row in rg_last_error; the context stays usable.  A
 * short limit makes waits give up early (used to test that path).  No
 * counterpart in the reference. */
rg_status rg_set_wait_limit(rg_ctx* ctx, long long polls);

/* Mixed precision only: equations of nodes with depth S - z below `depth`
 * (near-dry nodes) are eliminated in FP64 in the ILU(0) factorisation -- their
 * multipliers and pivots computed in double from the FP32 pivot rows, then
 * stored in FP32 like every factor entry.  Default for a mixed-precision
 * context: 10 hmin (five times the dry limit when hmin is half of it); 0 turns
 * it off.  The zero-pivot repair path (rare) factors in FP32.  No counterpart
 * in the reference, whose factorisation rounds every entry to its float
 * matrix type (Preco_ilu0.cpp:160-185). */
rg_status rg_set_fp64_pivots(rg_ctx* ctx, double depth);

/* Assemble the Newton system on the GPU (CRSMAT::Init + AssembleEqs_im,
 * CRSMat.cpp:206, Assemble.cpp:195).  Optional outputs (NULL to skip):
 * B (neq doubles) and the matrix values in the reference's packed layout, as
 * float (A32) or double (A64). */
rg_status rg_assemble(rg_ctx* ctx, double* B_out, float* A32_out, double* A64_out);

/* Load an already assembled system (the reference's own CRSMAT values, packed
 * layout, and B) instead of assembling; exactly one of A32/A64 non-NULL. */
rg_status rg_load_system(rg_ctx* ctx, const float* A32, const double* A64, const double* B);

/* CRSMAT::ScaleL2Norm (CRSMat.cpp:319-346) of the resident system; returns
 * ||B||_2 in *scale (the Newton residual norm). */
rg_status rg_scale(rg_ctx* ctx, double* scale);

/* PRECO_ILU0::Factor (Preco_ilu0.cpp:64-189) of the resident matrix.
 * Optional output of the factors in the packed layout.  The factors stay
 * resident until the next factorisation or pattern: rg_ilu0_apply and
 * rg_bicgstab after a new rg_assemble / rg_load_system without a new
 * rg_ilu0_factor precondition with the factors of the earlier matrix. */
rg_status rg_ilu0_factor(rg_ctx* ctx, float* LU32_out, double* LU64_out);

/* PRECO_ILU0::Solve (Preco_ilu0.cpp:497-980) of a host vector. */
rg_status rg_ilu0_apply(rg_ctx* ctx, const double* B, double* X);

/* PRECO_ILU0::Solve in FP32, for mixed-precision contexts: the preconditioner
 * of the mixed path's inner BiCGStab (FP32 factors and vectors, summation
 * order free), on host float vectors.  RG_ERR_ARG for other precisions. */
rg_status rg_ilu0_apply_f32(rg_ctx* ctx, const float* B, float* X);

/* ILU(0) preconditioner applied to a DEVICE vector without allocating:
 * x_dev = M^-1 b_dev with the resident factors.  It has no counterpart in the
 * reference.  It is meant for callers that must not allocate during a solve: a
 * caller that plans all device memory up front, or one whose loop cannot take
 * the implicit synchronisation of cudaMalloc/cudaFree.
 *  - The intermediate vector of the two triangular solves is a fixed
 *    file-scope device array of RG_NOALLOC_MAX_EQ doubles (2 MiB); a system
 *    with more equations is rejected with RG_ERR_ARG (use rg_ilu0_apply).
 *    Nothing in that array has to start at zero.
 *  - The first call on a device looks up the array's address
 *    (cudaGetSymbolAddress); make that first call before any stream capture
 *    begins on the device.
 *  - All contexts of a process share the one array per device: calls that
 *    overlap in time on the same device (two host threads, or two contexts)
 *    race on it and must be serialised by the caller.
 *  - b_dev and x_dev hold neq doubles each and must not overlap (an overlap
 *    is rejected with RG_ERR_ARG); the call runs on the context's stream and
 *    returns when the result is in x_dev, so b_dev must be complete when the
 *    call is made. */
#define RG_NOALLOC_MAX_EQ (1 << 18)
rg_status rg_ilu0_apply_dev_noalloc(rg_ctx* ctx, const double* b_dev, double* x_dev);

/* CRSMAT::MulVec (CRSMat.cpp:466-496) of a host vector with the resident matrix. */
rg_status rg_spmv(rg_ctx* ctx, const double* x, double* r);

/* BICGSTAB::Iterate (Bicgstab.cpp:66-375) on the resident scaled system with
 * the resident ILU(0) factors, X = 0 start.  X_out (optional) receives the
 * correction.  Returns RG_OK when converged, RG_NOT_CONVERGED otherwise (the
 * best iterate is kept, as the reference does). */
rg_status rg_bicgstab(rg_ctx* ctx, int maxIter, double maxDiff, double* X_out,
                      int* iters, double* accuracy);

/* EQS::Solve (Solve.cpp:53-374) for solver type 5 with ILU(0): assemble,
 * scale, factor, BiCGStab.  This is the drop-in point the reference's
 * EQS_UVS2D::Execute calls (EqsUVS2D.cpp:365).  X_out (optional, neq) gets
 * the correction, scale_out the residual norm ||B||, iters_out the Krylov
 * iteration count. */
rg_status rg_solve(rg_ctx* ctx, int maxIter, double maxDiff, double* X_out,
                   double* scale_out, int* iters_out);

/* Newton correction of one iteration on the resident correction X
 * (EqsUVS2D.cpp:412-759 with EQS::Update Update.cpp:42-187): relaxation method
 * 0 or 2, rotation back to x/y, |U| cap, S update with the dry clamp of
 * dry/rewet methods 0/2/3, mid-side S and z as corner means.  model_nodes
 * lists the wet nodes (MODEL::node); region_nodes/ne_region give all region
 * triangles (mid-side interpolation).  stats[0..5] receive max|dU|, max|dV|,
 * max|dS|, relaxUs, relaxS, theNorm. */
typedef struct {
  int           relax_method;      /* PROJECT::relaxMethod: 0 or 2 */
  double        max_delta_uv;      /* PROJECT::maxDeltaUV */
  double        max_delta_s;       /* PROJECT::maxDeltaS */
  double        max_us;            /* PROJECT::maxUs */
  double        dry_limit;         /* DRYREW::dryLimit */
  int           dryrew_method;     /* DRYREW::method */
} rg_update_opts;

rg_status rg_set_update_lists(rg_ctx* ctx, int np_model, const int* model_nodes,
                              int ne_region, const int* region_nodes, const double* zor);
rg_status rg_newton_update(rg_ctx* ctx, const rg_update_opts* opts, double* stats);

/* Nodal Manning friction (MODEL::DoFriction DoFriction.cpp:57-216,
 * TYPE::friction kMANN Friction.cpp:238-240) over all region triangles with
 * per-element Manning n and area factor (GRID::AreaFactors ArFact.cpp:41). */
rg_status rg_set_friction(rg_ctx* ctx, const double* elem_n, const double* elem_areafact);
rg_status rg_friction(rg_ctx* ctx, double* cf_out);

/* MODEL::Continuity (Contin.cpp:43-170): the discharge through each control
 * section from the resident state, in FP64 on the device.  seg_nodes holds 3
 * nodes per line element (corner, corner, mid-side: the control file's
 * order), seg_section the 1-based section (line) number of each element;
 * Qx[k], Qy[k] receive the x and y parts of section k+1 (the reference prints
 * their sum, and each section's share of section 1).  Sums within a section
 * run in a fixed order. */
rg_status rg_continuity(rg_ctx* ctx, int nseg, const int* seg_nodes, const int* seg_section, int nsect,
                        double* Qx, double* Qy);

/* Device-time of the last call's kernels, by stage (ms), for measurement:
 * [0] assembly, [1] scale, [2] factor, [3] BiCGStab total, [4] SpMV (one),
 * [5] ILU apply (one), [6] update, [7] friction; [8] / [9] host time of the
 * last / of all rg_set_pattern calls (schedules and layouts are built there). */
rg_status rg_get_timings(rg_ctx* ctx, double* ms, int n);

/* Structure of the resident system: [0] neq, [1] nnz, [2] dependency depth of
 * the L solve, [3] of the U solve, [4] element colours, [5] L entries,
 * [6] / [7] wavefront chunks of the L / U solve, [8] / [9] their entries whose
 * source lies outside the shared-memory ring, [10] factorisations redone by
 * the zero-pivot repair path, [11] factorisations, [12] / [13] bytes copied
 * host->device / device->host by this context's calls so far, [14] kernels
 * launched so far. */
rg_status rg_get_stats(rg_ctx* ctx, int64_t* out, int n);

/* Per-kernel device time, for measurement.  While enabled, every launch of the
 * triangular solves (class 0), SpMV (1), ILU(0) factorisation (2) and element
 * assembly (3) is bracketed by CUDA events on the context's stream; the
 * elapsed times are summed when a call synchronises.  rg_profile_read gives
 * out[2k] = launches and out[2k+1] = total milliseconds of class k.  No
 * counterpart in the reference, which times with the host clock only. */
rg_status rg_profile(rg_ctx* ctx, int enable, int reset);
rg_status rg_profile_read(rg_ctx* ctx, double* out, int n);

/* CUDA events on the context's stream (8 slots), for timing a caller's
 * sequence of calls on the device clock. */
rg_status rg_event_record(rg_ctx* ctx, int slot);
rg_status rg_event_elapsed(rg_ctx* ctx, int a, int b, double* ms);

#ifdef __cplusplus
}
#endif

#endif

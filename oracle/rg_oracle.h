/*
 * CPU restatement of the reference's shallow-water Newton step (parity oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this code; only tests/, the smoke check and bench.py's CPU-baseline leg
 * do, and only as the checker.  Each function restates one reference routine
 * (cited file:line) in plain serial C with the reference's arithmetic order, so
 * its results can be compared with the compiled reference (golden fixtures) and
 * with the CUDA path.
 *
 * Matrix storage follows the reference's CRSMAT (CRSMat.h:71-97): row i owns
 * width[i] = ptr[i+1]-ptr[i] entries, diagonal first, the remaining columns in
 * first-seen order; values are REALPR = float as shipped (Defs.h:92) in the
 * "_f32" functions and double in the "_f64" ones.
 */
#ifndef RG_ORACLE_H
#define RG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Node / element / boundary data of one Newton iteration (the inputs of
 * CRSMAT::AssembleEqs_im, Assemble.cpp:195, and EQS_UVS2D::Coefs,
 * CoefsUVS2D.cpp:49).  All node arrays are indexed by the region node index. */
typedef struct {
  int           np;
  const double *x, *y, *z;
  const double *U, *V, *S, *dUdt, *dVdt, *dSdt;
  const double *cf, *cfw, *uu, *uv, *vv;
  const int    *nflag;            /* NODE::flag (kRotat = 32) */
  const int    *bckind;           /* BCON::kind */
  const double *rot;              /* 4 per node: rot[0][0], [0][1], [1][0], [1][1] */
  const double *niox, *nioy;      /* open-boundary normal */
  const double *bcU, *bcS;        /* BCVAL::U (specific inflow q), BCVAL::S */
  const int    *eqno;             /* 3 per node: U, V, S equation numbers, -1 = none */
  int           ne;               /* model element list (region + boundary lines) */
  const int    *enodes;           /* 6 per element (3 used by line elements) */
  const int    *ennd;             /* 6 (triangle) or 3 (boundary line) */
  const int    *eflag;            /* ELEM::flag */
  const double *evt;              /* constant eddy viscosity of the element's type */
  double        g, hmin, vk;
  double        relaxThdt_UV, relaxThdt_H;
} orc_model;

/* element coefficients: estifm is 24x24 row-major, force 24 (maxEleq = 24) */
int  orc_coefs(const orc_model* m, int e, double* estifm, double* force);

/* assembly into the reference CRS layout; B overwritten; A zeroed first */
void orc_assemble_f32(const orc_model* m, int neq, const int64_t* ptr, const int* index,
                      float* A, double* B);
void orc_assemble_f64(const orc_model* m, int neq, const int64_t* ptr, const int* index,
                      double* A, double* B);

double orc_scale_l2_f32(int neq, const int64_t* ptr, float* A, double* B);
double orc_scale_l2_f64(int neq, const int64_t* ptr, double* A, double* B);

void orc_spmv_f32(int neq, const int64_t* ptr, const int* index, const float* A,
                  const double* x, double* r);
void orc_spmv_f64(int neq, const int64_t* ptr, const int* index, const double* A,
                  const double* x, double* r);

/* ILU(0) in place on a copy of A (ILU has A's layout); returns 0, or
 * 1 + the equation whose pivot could not be repaired */
int  orc_ilu0_factor_f32(int neq, const int64_t* ptr, const int* index, const float* A, float* ILU);
int  orc_ilu0_factor_f64(int neq, const int64_t* ptr, const int* index, const double* A, double* ILU);
void orc_ilu0_solve_f32(int neq, const int64_t* ptr, const int* index, const float* ILU,
                        const double* B, double* X);
void orc_ilu0_solve_f64(int neq, const int64_t* ptr, const int* index, const double* ILU,
                        const double* B, double* X);

/* right-preconditioned BiCGStab; returns 1 when converged (Bicgstab.cpp:366) */
int  orc_bicgstab_f32(int neq, const int64_t* ptr, const int* index, const float* A, const float* ILU,
                      const double* b, double* x, int maxIter, double maxDiff,
                      int* iters, double* accuracy);
int  orc_bicgstab_f64(int neq, const int64_t* ptr, const int* index, const double* A, const double* ILU,
                      const double* b, double* x, int maxIter, double maxDiff,
                      int* iters, double* accuracy);

/* Newton correction of one iteration (EqsUVS2D.cpp:455-759): relaxation
 * method 0 or 2, rotation back to x/y, |U| cap, S update with the dry clamp of
 * dry/rewet methods 0, 2 and 3, mid-side S and z.  State arrays are updated in
 * place.  stats[0..8] = max|dU|, max|dV|, max|dS| (Update.cpp:42-187 maxAbs),
 * relaxUs, relaxS, theNorm, #nodes whose |U| was capped, #nodes clamped. */
typedef struct {
  int     np_model;  const int* model_nodes;    /* wet node list (model->node) */
  int     ne_region; const int* region_nodes;   /* 6 per region element */
  const int* region_flag;                       /* ELEM::flag of region elements */
  double  maxDeltaUV, maxDeltaS, maxUs, dryLimit;
  int     relaxMethod, dryRewMethod;
} orc_update_cfg;

void orc_newton_update(const orc_update_cfg* c, const int* eqno, const int* nflag, const double* rot,
                       const double* X, double* U, double* V, double* S, double* z,
                       const double* zor, double hmin, double* stats);

/* nodal Manning friction (MODEL::DoFriction, DoFriction.cpp:57-216 with
 * TYPE::friction kMANN, Friction.cpp:238-240) over all region elements */
void orc_friction(int np, int ne_region, const int* region_nodes, const int* region_nnd,
                  const double* elem_n, const double* elem_areafact, const double* U,
                  const double* V, const double* S, const double* z, double hmin, double g,
                  double* cf);

/* CRS pattern of the equations of six-node triangles in the layout of
 * EQS::SetIndexMat (IndexMat.cpp:91-342): diagonal first, then the equations of
 * every node of every element that holds the row's node, first seen first
 * (elements in list order, nodes in element order, U V S per node).  eqno: 3
 * per node (-1: none).  ptr (neq + 1) is always filled; idx only when non-NULL.
 * Returns the entry count. */
int64_t orc_pattern(int np, int ne, const int* enodes, const int* eqno, int neq, int64_t* ptr, int* idx);

/* discharge through the control sections (MODEL::Continuity, Contin.cpp:43-170):
 * control line elements in file order, 3 Gauss points each; section of element t
 * is seg_section[t] (1-based); Qx, Qy: nsect sums */
void orc_continuity(int nseg, const int* seg_nodes, const int* seg_section, int nsect, const double* x,
                    const double* y, const double* U, const double* V, const double* S, const double* z,
                    double* Qx, double* Qy);

#ifdef __cplusplus
}
#endif

#endif

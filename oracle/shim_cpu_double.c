/*
 * CPU stand-in for the part of librg300 that the drop-in shim
 * (rismo2d_gb300/shim/rg300_eqs_solve.cpp) calls: rg_create, rg_destroy,
 * rg_last_error, rg_set_elements, rg_set_pattern, rg_set_state,
 * rg_set_boundary, rg_set_relax and rg_solve.
 *
 * TEST INFRASTRUCTURE ONLY.  It is linked into oracle/_ref/rismo2d_rg300_cpu
 * (oracle/Makefile target `shim_cpu`) so that the shim's marshalling of the
 * reference's MODEL, NODE, BCON and CRSMAT data runs end to end on a machine
 * without a GPU: the reference runs its own Newton loop, and every EQS::Solve
 * goes through the shim into these functions, which solve with the oracle's
 * restatement (rg_oracle.c) in the reference's storage (float matrix, double
 * vectors) -- assembly (Assemble.cpp:195), ScaleL2Norm (CRSMat.cpp:319),
 * ILU(0) (Preco_ilu0.cpp:64) and BiCGStab (Bicgstab.cpp:66).  The shipped
 * library never links it.
 */
#include "../include/rg300.h"
#include "../include/rg300_sim.h"
#include "rg_oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct rg_ctx {
  int np, ne, neq;
  double *x, *y, *evt;
  int *en, *ennd, *eflag;
  double g, hmin, vk, rUV, rH;
  int64_t* ptr;
  int *index, *eqno;
  double *U, *V, *S, *dU, *dV, *dS, *z, *cf, *cfw, *zero;
  int *nflag, *bckind;
  double *rot, *niox, *nioy, *bcU, *bcS;
  char err[256];
};

/* solves taken through the binding, reported at exit so a test can see the reroute happen */
static long g_solves = 0;
static void report_solves(void) { printf("rg300 CPU stand-in: %ld solves\n", g_solves); }

static void* dup(const void* src, size_t bytes) {
  void* p = malloc(bytes ? bytes : 1);
  if (p && src && bytes) memcpy(p, src, bytes);
  return p;
}

static void copy_into(double* dst, const double* src, int n) {
  if (src) memcpy(dst, src, (size_t)n * sizeof(double));
}

static rg_status fail(rg_ctx* c, rg_status st, const char* msg) {
  if (c) snprintf(c->err, sizeof(c->err), "%s", msg);
  return st;
}

rg_status rg_create(const rg_mesh* m, int precision, int device, rg_ctx** out) {
  (void)device;
  if (!m || !out || m->np <= 0) return RG_ERR_ARG;
  if (precision != RG_PREC_REF32) return RG_ERR_ARG;   /* the reference's storage only */
  rg_ctx* c = (rg_ctx*)calloc(1, sizeof(rg_ctx));
  if (!c) return RG_ERR_ARG;
  static int registered = 0;
  if (!registered) registered = atexit(report_solves) == 0;
  const int np = m->np;
  c->np = np;
  c->x = (double*)dup(m->x, np * sizeof(double));
  c->y = (double*)dup(m->y, np * sizeof(double));
  c->g = m->g;
  c->hmin = m->hmin;
  c->vk = m->vk;
  double** fields[] = {&c->U, &c->V, &c->S, &c->dU, &c->dV, &c->dS, &c->z, &c->cf, &c->cfw, &c->zero,
                       &c->niox, &c->nioy, &c->bcU, &c->bcS};
  for (size_t k = 0; k < sizeof(fields) / sizeof(fields[0]); k++) *fields[k] = (double*)calloc(np, sizeof(double));
  c->rot = (double*)calloc(4 * (size_t)np, sizeof(double));
  c->nflag = (int*)calloc(np, sizeof(int));
  c->bckind = (int*)calloc(np, sizeof(int));
  *out = c;
  return rg_set_elements(c, m->ne, m->elem_nodes, m->elem_nnd, m->elem_flag, m->elem_vt);
}

rg_status rg_destroy(rg_ctx* c) {
  if (!c) return RG_OK;
  void* ps[] = {c->x, c->y, c->evt, c->en, c->ennd, c->eflag, c->ptr, c->index, c->eqno, c->U, c->V, c->S,
                c->dU, c->dV, c->dS, c->z, c->cf, c->cfw, c->zero, c->nflag, c->bckind, c->rot, c->niox, c->nioy,
                c->bcU, c->bcS};
  for (size_t k = 0; k < sizeof(ps) / sizeof(ps[0]); k++) free(ps[k]);
  free(c);
  return RG_OK;
}

const char* rg_last_error(rg_ctx* c) { return c ? c->err : "no context"; }

rg_status rg_set_elements(rg_ctx* c, int ne, const int* en, const int* nnd, const int* flag, const double* vt) {
  if (!c || ne < 0 || (ne > 0 && (!en || !nnd || !flag || !vt))) return RG_ERR_ARG;
  free(c->en);
  free(c->ennd);
  free(c->eflag);
  free(c->evt);
  c->ne = ne;
  c->en = (int*)dup(en, 6 * (size_t)ne * sizeof(int));
  c->ennd = (int*)dup(nnd, (size_t)ne * sizeof(int));
  c->eflag = (int*)dup(flag, (size_t)ne * sizeof(int));
  c->evt = (double*)dup(vt, (size_t)ne * sizeof(double));
  return RG_OK;
}

rg_status rg_set_pattern(rg_ctx* c, int neq, const int* width, const int* index, const int* eqno) {
  if (!c || neq < 0 || (neq > 0 && (!width || !index)) || !eqno) return RG_ERR_ARG;
  free(c->ptr);
  free(c->index);
  free(c->eqno);
  c->neq = neq;
  c->ptr = (int64_t*)malloc(((size_t)neq + 1) * sizeof(int64_t));
  c->ptr[0] = 0;
  for (int i = 0; i < neq; i++) c->ptr[i + 1] = c->ptr[i] + width[i];
  c->index = (int*)dup(index, (size_t)c->ptr[neq] * sizeof(int));
  c->eqno = (int*)dup(eqno, 3 * (size_t)c->np * sizeof(int));
  return RG_OK;
}

rg_status rg_set_state(rg_ctx* c, const double* U, const double* V, const double* S, const double* dUdt,
                       const double* dVdt, const double* dSdt, const double* z, const double* cf,
                       const double* cfw) {
  if (!c) return RG_ERR_ARG;
  copy_into(c->U, U, c->np);
  copy_into(c->V, V, c->np);
  copy_into(c->S, S, c->np);
  copy_into(c->dU, dUdt, c->np);
  copy_into(c->dV, dVdt, c->np);
  copy_into(c->dS, dSdt, c->np);
  copy_into(c->z, z, c->np);
  copy_into(c->cf, cf, c->np);
  copy_into(c->cfw, cfw, c->np);
  return RG_OK;
}

rg_status rg_set_boundary(rg_ctx* c, const int* nflag, const int* bckind, const double* rot, const double* niox,
                          const double* nioy, const double* bcU, const double* bcS) {
  if (!c || !nflag || !bckind || !rot || !niox || !nioy || !bcU || !bcS) return RG_ERR_ARG;
  memcpy(c->nflag, nflag, (size_t)c->np * sizeof(int));
  memcpy(c->bckind, bckind, (size_t)c->np * sizeof(int));
  memcpy(c->rot, rot, 4 * (size_t)c->np * sizeof(double));
  copy_into(c->niox, niox, c->np);
  copy_into(c->nioy, nioy, c->np);
  copy_into(c->bcU, bcU, c->np);
  copy_into(c->bcS, bcS, c->np);
  return RG_OK;
}

rg_status rg_set_relax(rg_ctx* c, double relaxThdt_UV, double relaxThdt_H) {
  if (!c) return RG_ERR_ARG;
  c->rUV = relaxThdt_UV;
  c->rH = relaxThdt_H;
  return RG_OK;
}

rg_status rg_solve(rg_ctx* c, int maxIter, double maxDiff, double* X_out, double* scale_out, int* iters_out) {
  if (!c || !c->ptr) return fail(c, RG_ERR_ARG, "rg_solve: call rg_set_pattern first");
  g_solves++;
  const int neq = c->neq;
  const int64_t nnz = c->ptr[neq];
  orc_model m;
  memset(&m, 0, sizeof(m));
  m.np = c->np;
  m.x = c->x;
  m.y = c->y;
  m.z = c->z;
  m.U = c->U;
  m.V = c->V;
  m.S = c->S;
  m.dUdt = c->dU;
  m.dVdt = c->dV;
  m.dSdt = c->dS;
  m.cf = c->cf;
  m.cfw = c->cfw;
  m.uu = m.uv = m.vv = c->zero;   /* no dispersion terms: the library's integrand has none either */
  m.nflag = c->nflag;
  m.bckind = c->bckind;
  m.rot = c->rot;
  m.niox = c->niox;
  m.nioy = c->nioy;
  m.bcU = c->bcU;
  m.bcS = c->bcS;
  m.eqno = c->eqno;
  m.ne = c->ne;
  m.enodes = c->en;
  m.ennd = c->ennd;
  m.eflag = c->eflag;
  m.evt = c->evt;
  m.g = c->g;
  m.hmin = c->hmin;
  m.vk = c->vk;
  m.relaxThdt_UV = c->rUV;
  m.relaxThdt_H = c->rH;
  float* A = (float*)calloc((size_t)nnz + 1, sizeof(float));
  float* ILU = (float*)calloc((size_t)nnz + 1, sizeof(float));
  double* B = (double*)calloc((size_t)neq + 1, sizeof(double));
  double* X = (double*)calloc((size_t)neq + 1, sizeof(double));
  orc_assemble_f32(&m, neq, c->ptr, c->index, A, B);
  const double scale = orc_scale_l2_f32(neq, c->ptr, A, B);
  rg_status st = RG_OK;
  if (orc_ilu0_factor_f32(neq, c->ptr, c->index, A, ILU) != 0) {
    st = fail(c, RG_ERR_ZERO_PIVOT, "rg_solve: zero pivot");
  } else {
    int its = 0;
    double acc = 0.0;
    const int conv = orc_bicgstab_f32(neq, c->ptr, c->index, A, ILU, B, X, maxIter, maxDiff, &its, &acc);
    if (X_out) memcpy(X_out, X, (size_t)neq * sizeof(double));
    if (scale_out) *scale_out = scale;
    if (iters_out) *iters_out = its;
    st = conv ? RG_OK : RG_NOT_CONVERGED;
  }
  free(A);
  free(ILU);
  free(B);
  free(X);
  return st;
}

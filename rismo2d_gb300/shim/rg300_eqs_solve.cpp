// Drop-in of the GPU Newton solve into the reference solver, with no edit of
// its sources: EQS::Solve (Solve.cpp:53-374) is rerouted to librg300 when the
// equation system is EQS_UVS2D and the selected solver is BiCGStab (type 5,
// Solver.h:67) with ILU(0) (Precon.h / Solver.h:73).  Every other call goes to
// the reference's own EQS::Solve.
//
// Link (oracle/Makefile target `shim` does exactly this):
//   g++ ... reference objects ... rg300_eqs_solve.o
//       -Wl,--wrap=_ZN3EQS5SolveEP5MODELiPdS2_P7PROJECTP6SOLVERPP6PRECONi
//       -L<repo>/rismo2d_gb300 -lrg300 -lcudart
//
// The reference keeps its boundary conditions, friction, dry/rewet, numbering
// and Newton update on the host; per Newton iteration this shim hands the GPU
// the node state, the boundary data and (after a renumbering) the CRS pattern
// the reference built, and gets the correction X back.  The reference's
// classes keep their members protected, so the shim is compiled with them
// opened up, as a friend declaration would.

#define protected public
#define private public
#include "Defs.h"
#include "Report.h"
#include "Node.h"
#include "Elem.h"
#include "Model.h"
#include "Grid.h"
#include "Project.h"
#include "Type.h"
#include "CRSMat.h"
#include "Eqs.h"
#include "EqsUVS2D.h"
#include "Solver.h"
#include "Precon.h"
#undef protected
#undef private

#include "rg300.h"
#include "rg300_sim.h"

#include <cstdlib>
#include <vector>

namespace {

struct GpuSolve {
  rg_ctx* ctx = nullptr;
  int np = 0;
  MODEL* model = nullptr;        // model whose element list the context holds
  int model_ne = -1;
};
GpuSolve g;

// model element list in MODEL::elem order (Model.cpp:121-216)
void model_elements(MODEL* model, std::vector<int>& nodes, std::vector<int>& nnd, std::vector<int>& flag,
                    std::vector<double>& vt) {
  const int ne = model->ne;
  nodes.assign(6 * (size_t)ne, -1);
  nnd.resize(ne);
  flag.resize(ne);
  vt.resize(ne);
  for (int e = 0; e < ne; e++) {
    ELEM* el = model->elem[e];
    nnd[e] = el->Getnnd();
    flag[e] = el->flag;
    vt[e] = TYPE::Getid(el->type)->vt;
    for (int i = 0; i < el->Getnnd() && i < 6; i++) nodes[6 * e + i] = el->nd[i]->Getno();
  }
}

bool fail(rg_status st, const char* where) {
  if (st == RG_OK || st == RG_NOT_CONVERGED) return false;
  REPORT::rpt.Error(kUnexpectedFault, "%s: %s (status %d)", where, g.ctx ? rg_last_error(g.ctx) : "", (int)st);
  return true;
}

}  // namespace

extern "C" {

int __real__ZN3EQS5SolveEP5MODELiPdS2_P7PROJECTP6SOLVERPP6PRECONi(EQS*, MODEL*, int, double*, double*, PROJECT*,
                                                                 SOLVER*, PRECON**, int);

int __wrap__ZN3EQS5SolveEP5MODELiPdS2_P7PROJECTP6SOLVERPP6PRECONi(EQS* eqs, MODEL* model, int neq, double* B,
                                                                 double* X, PROJECT* project, SOLVER* slv,
                                                                 PRECON** pre, int assemble) {
  SOLVER* s = slv ? slv : project->actualSolver;
  EQS_UVS2D* uvs = dynamic_cast<EQS_UVS2D*>(eqs);
  if (!uvs || !s || !X || !assemble || s->solverType != kBicgstab || s->preconType != kPreco_ilu0)
    return __real__ZN3EQS5SolveEP5MODELiPdS2_P7PROJECTP6SOLVERPP6PRECONi(eqs, model, neq, B, X, project, slv, pre,
                                                                        assemble);
  GRID* rg = model->region;
  const int np = rg->Getnp();
  std::vector<int> nodes, nnd, flag;
  std::vector<double> vt;

  // context: mesh coordinates and the current model element list
  if (!g.ctx || g.np != np) {
    if (g.ctx) rg_destroy(g.ctx);
    std::vector<double> x(np), y(np);
    for (int n = 0; n < np; n++) {
      x[rg->Getnode(n)->Getno()] = rg->Getnode(n)->x;
      y[rg->Getnode(n)->Getno()] = rg->Getnode(n)->y;
    }
    model_elements(model, nodes, nnd, flag, vt);
    rg_mesh m = {np, x.data(), y.data(), model->ne, nodes.data(), nnd.data(), flag.data(), vt.data(),
                 project->g, project->hmin, project->vk};
    // RG300_PRECISION: 0 FP64, 1 the reference's float matrix / double vectors (default), 2 mixed
    const char* pe = getenv("RG300_PRECISION");
    const int prec = pe ? atoi(pe) : RG_PREC_REF32;
    if (fail(rg_create(&m, prec, -1, &g.ctx), "rg_create")) return kErr_interrupt;
    g.np = np;
    g.model = model;
    g.model_ne = model->ne;
    eqs->initStructure = true;
  }

  // numbering and pattern: the reference's own (EQS::SetIndexMat, Solve.cpp:164-176)
  if (eqs->initStructure) {
    eqs->KillCrsm();
    eqs->SetIndexMat(model, s->mceq);
    eqs->crsm->Alloc_A();
    eqs->initStructure = false;
    model_elements(model, nodes, nnd, flag, vt);
    if (fail(rg_set_elements(g.ctx, model->ne, nodes.data(), nnd.data(), flag.data(), vt.data()),
             "rg_set_elements"))
      return kErr_interrupt;
    CRSMAT* c = eqs->crsm;
    std::vector<int> width(c->m_width, c->m_width + c->m_neq), index, eqno(3 * (size_t)np, -1);
    for (int i = 0; i < c->m_neq; i++)
      for (int k = 0; k < c->m_width[i]; k++) index.push_back(c->m_index[i][k]);
    for (int n = 0; n < np; n++)
      for (int j = 0; j < 3; j++) eqno[3 * n + j] = eqs->nodeEqno[j][n];
    if (fail(rg_set_pattern(g.ctx, c->m_neq, width.data(), index.data(), eqno.data()), "rg_set_pattern"))
      return kErr_interrupt;
  }

  // node state and boundary data of this iteration, indexed by NODE::Getno()
  std::vector<double> U(np), V(np), S(np), dU(np), dV(np), dS(np), z(np), cf(np), cfw(np);
  std::vector<double> rot(4 * (size_t)np), niox(np), nioy(np), bcU(np), bcS(np);
  std::vector<int> nflag(np), bckind(np);
  for (int k = 0; k < np; k++) {
    NODE* nd = rg->Getnode(k);
    const int n = nd->Getno();
    U[n] = nd->v.U;
    V[n] = nd->v.V;
    S[n] = nd->v.S;
    dU[n] = nd->v.dUdt;
    dV[n] = nd->v.dVdt;
    dS[n] = nd->v.dSdt;
    z[n] = nd->z;
    cf[n] = nd->cf;
    cfw[n] = nd->cfw;
    nflag[n] = nd->flag;
    bckind[n] = nd->bc.kind;
    rot[4 * n + 0] = nd->bc.Getrot(0, 0);
    rot[4 * n + 1] = nd->bc.Getrot(0, 1);
    rot[4 * n + 2] = nd->bc.Getrot(1, 0);
    rot[4 * n + 3] = nd->bc.Getrot(1, 1);
    niox[n] = nd->bc.niox;
    nioy[n] = nd->bc.nioy;
    bcU[n] = nd->bc.val ? nd->bc.val->U : 0.0;
    bcS[n] = nd->bc.val ? nd->bc.val->S : 0.0;
  }
  if (fail(rg_set_state(g.ctx, U.data(), V.data(), S.data(), dU.data(), dV.data(), dS.data(), z.data(), cf.data(),
                        cfw.data()),
           "rg_set_state") ||
      fail(rg_set_boundary(g.ctx, nflag.data(), bckind.data(), rot.data(), niox.data(), nioy.data(), bcU.data(),
                           bcS.data()),
           "rg_set_boundary") ||
      fail(rg_set_relax(g.ctx, uvs->relaxThdt_UV, uvs->relaxThdt_H), "rg_set_relax"))
    return kErr_interrupt;

  // assemble, ScaleL2Norm, ILU(0), BiCGStab on the GPU
  double scale = 0.0;
  int its = 0;
  rg_status st = rg_solve(g.ctx, s->maxIter, s->maxDiff, X, &scale, &its);
  if (fail(st, "rg_solve")) return kErr_interrupt;
  s->iterCountCG = its;
  eqs->iterCountCG += its;
  if (st == RG_NOT_CONVERGED) {
    // the reference's handling of a solver that did not converge (Solve.cpp:329-357), proceed == 0
    REPORT::rpt.Warning(kSolverFault, "Solver %d has not converged - iteration continued", s->solverType);
    return kErr_some_errors;
  }
  return 0;
}

}  // extern "C"

// Host-side model of a shallow-water time step: the per-iteration bookkeeping
// of EQS_UVS2D::Execute (EqsUVS2D.cpp:71-1096) around the GPU hot path.
//
// Restated reference routines (host, changes only with the wet/dry state or
// the boundary data):
//   GRID::Connection        Connect.cpp:43-126     node -> wet element counts
//   MODEL::Boundary         Bound.cpp:50-164       boundary line elements
//   MODEL::Initialize       Model.cpp:121-216      wet node / element lists
//   MODEL::SetLocation      Locate.cpp:47-193      inlet/outlet/convex flags
//   MODEL::SetNormal        Transform.cpp:52-265   boundary normals
//   MODEL::SetRotation      Transform.cpp:269-498  slip / normal-flow rotation
//   BCONSET::InitBcon       BconSet.cpp:92-487     node boundary conditions
//   BCONLINE::Inlet/Outlet  BconLine.cpp:249-985   QINLET, QTINLET, OUTLET
//   EQS::SetEqno            SetEqno.cpp:52-543     numbering + frontal order
//   EQS::SetIndexMat        IndexMat.cpp:91-342    CRS pattern
//   GRID::DryRewet          DryRewet.cpp:696-990   dry/rewet method 2
//   GRID::AreaFactors       ArFact.cpp:41-97       inclined-element factor
//   EQS_UVS2D::Predict      EqsUVS2D.cpp:1101-1178
//   GRID::SetSlipFlow       SlipFlow.cpp:42-80
// The hot path (friction, assembly, scaling, ILU(0), BiCGStab, correction,
// time derivatives) runs on the GPU through the rg_* entry points.

#include "rg_internal.cuh"
#include "../../include/rg300_sim.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace {

// NODE::flag (Node.h)
enum : unsigned {
  N_INLET = 1, N_OUTLET = 2, N_OPENBND = 4, N_GRIDBND = 8, N_BOUND = 16, N_ROTAT = 32, N_DRY = 64,
  N_DRYPREV = 128, N_MARSH = 256, N_MARSHPREV = 512, N_CORN = 1024, N_MIDS = 2048, N_NOMOMENT = 4096
};
// ELEM::flag (Elem.h)
enum : unsigned {
  E_INLET = 1, E_OUTLET = 2, E_OPENBND = 4, E_BOUND = 16, E_REGION = 32, E_DRY = 128, E_DRYPREV = 256,
  E_MARSH = 512, E_MARSHPREV = 1024
};
// BCON::kind (Bcon.h)
enum : unsigned {
  B_INLET = 1, B_OUTLET = 2, B_OPENBND = 4, B_QINLET = 8, B_QTINLET = 16, B_SLIP = 128, B_SETUV = 512,
  B_SETS = 1024, B_FIXU = 32768, B_FIXV = 65536, B_AUTOSLIP = 4194304
};
enum { ROT_NONE = 0, ROT_TANGENT = 1, ROT_NORMAL = 2 };

struct BElem {       // boundary line element (corner, corner, mid-side)
  int nd[3];
  unsigned flag;
  int region;        // owning region triangle
};

struct LineBc {
  int line = 0;
  unsigned kind = 0;
  std::vector<double> t, Q, S;   // QINLET: one row; QTINLET: hydrograph
};

double interp_hydro(const LineBc& b, double t, double* Sspec) {
  // BCONLINE::FindInterval on time (BconLine.cpp:167-227), linear in between
  double Q = b.Q[0];
  *Sspec = b.S[0];
  const int n = (int)b.t.size();
  for (int i = 0; i < n - 1; i++) {
    double dx = b.t[i + 1] - b.t[i];
    double lx = t - b.t[i];
    if (std::fabs(dx) > 1.0e-20)
      lx /= dx;
    else
      lx = dx = 0.0;
    bool hit;
    double L;
    if (std::fabs(dx) < 1.0e-20 && std::fabs(lx) < 1.0e-20) {
      hit = true;   // ly == 0 for a time series
      L = 0.0;
    } else {
      hit = (lx > -0.001 && lx < 1.001);
      L = lx;
    }
    if (hit) {
      Q = b.Q[i] + L * (b.Q[i + 1] - b.Q[i]);
      *Sspec = b.S[i] + L * (b.S[i + 1] - b.S[i]);
      return Q;
    }
  }
  return Q;
}

// A fixed set of host threads for the data-parallel passes of the host model
// (dry/rewet, connectivity counts).  run(n, fn) calls fn(begin, end, t) on
// contiguous slices of [0, n), slice t on thread t, and returns when all are
// done; every pass it runs either writes per-item results or combines into
// shared words with commutative atomic operations, so results do not depend
// on the thread count.
class HostPool {
 public:
  explicit HostPool(int nthreads) : nt_(std::max(1, nthreads)) {
    for (int t = 1; t < nt_; t++) workers_.emplace_back([this, t] { worker(t); });
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lk(m_);
      stop_ = true;
    }
    cv_.notify_all();
    for (std::thread& w : workers_) w.join();
  }
  template <class F>
  void run(long long n, F&& fn) {
    if (nt_ == 1 || n < 8192) {
      fn(0ll, n, 0);
      return;
    }
    {
      std::lock_guard<std::mutex> lk(m_);
      task_ = [&fn, n, this](int t) { fn(n * t / nt_, n * (t + 1) / nt_, t); };
      pending_ = nt_ - 1;
      gen_++;
    }
    cv_.notify_all();
    task_(0);
    std::unique_lock<std::mutex> lk(m_);
    done_.wait(lk, [this] { return pending_ == 0; });
  }
  int threads() const { return nt_; }

 private:
  void worker(int t) {
    long long seen = 0;
    for (;;) {
      std::function<void(int)> task;
      {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_;
        task = task_;
      }
      task(t);
      std::lock_guard<std::mutex> lk(m_);
      if (--pending_ == 0) done_.notify_one();
    }
  }
  int nt_;
  std::vector<std::thread> workers_;
  std::mutex m_;
  std::condition_variable cv_, done_;
  std::function<void(int)> task_;
  long long gen_ = 0;
  int pending_ = 0;
  bool stop_ = false;
};

int host_threads() {
  const char* e = getenv("RG_HOST_THREADS");
  if (e && atoi(e) > 0) return std::min(atoi(e), 64);
  const unsigned h = std::thread::hardware_concurrency();
  return (int)std::min(16u, std::max(1u, h));
}

inline void atomic_or(unsigned* p, unsigned v) { __atomic_fetch_or(p, v, __ATOMIC_RELAXED); }
inline void atomic_and(unsigned* p, unsigned v) { __atomic_fetch_and(p, v, __ATOMIC_RELAXED); }

}  // namespace

struct rg_sim {
  rg_ctx* ctx = nullptr;
  int prec = RG_PREC_FP64;
  std::string err;

  // region
  int np = 0, ne = 0;
  std::vector<double> x, y, zor, z;
  std::vector<int> en;           // 6 per region triangle
  std::vector<double> en_n, en_vt, en_af;
  std::vector<unsigned> eflag, nflag;
  std::vector<int> noel, countdown;
  // control lines
  std::vector<int> seg_nodes, seg_line;
  std::vector<LineBc> bcl;
  // per-node boundary data
  std::vector<unsigned> bckind;
  std::vector<int> rot, has_val;
  std::vector<double> bnx, bny, niox, nioy, bcU, bcS;
  // state (host mirror)
  std::vector<double> U, V, S, dUdt, dVdt, dSdt, oU, oV, oS, odUdt, odVdt, odSdt, cf;
  // boundary elements, model lists
  std::vector<BElem> bel;
  std::vector<int> boundList;    // mid-side node -> boundary element
  std::vector<int> mnodes;       // wet nodes
  std::vector<int> melems;       // >= 0 region triangle, < 0: -(1+boundary element)
  int model_init = 0, eqs_init = -1;
  bool firstDryRew = true;
  // numbering and pattern
  int neq = 0;
  std::vector<int> eqno;         // 3 per node
  std::vector<int> width, index;
  // parameters
  rg_deck_params p{};
  double hmin = 0.0;
  bool have_state = false;
  // last step report detail
  std::vector<double> resid_hist;
  // warm start of the next step (rg_sim_set_warm_start)
  bool warm_pending = false;
  std::vector<double> wU, wV, wS;
  // ILU(0) reuse (rg_step_ctl::ilu_reuse): numbering generation and age of the resident factors
  int factor_eqs = -1, factor_age = 0;
  // boundary set-up cache: within one time step and one wet model the node
  // kinds, normals and rotations repeat; only the inlet values (friction,
  // dryness) change from one Newton iteration to the next
  bool bc_valid = false;
  std::vector<int> line_nodes;   // nodes of the control lines, ascending
  std::vector<int> zero_uv;      // kNoMoment nodes of the last full set-up
  std::vector<unsigned> ib_kind; // init_bcon work arrays (line nodes only are touched)
  std::vector<char> ib_has, ib_mark;
  std::vector<double> ib_vU, ib_vS;
  // page-locked host state (cudaHostRegister), unregistered on destroy
  std::vector<void*> pinned;
  // host threads of the dry/rewet and connectivity passes; dry/rewet work arrays
  std::unique_ptr<HostPool> pool;
  std::vector<int> mid_owner;    // mid-side node -> first triangle that has it
  std::vector<char> dw_nmark, dw_emark;
  std::vector<std::vector<int>> dw_marsh;   // per slice: non-dry triangles with a marsh corner
  std::vector<unsigned> dw_nflag0, dw_eflag0; // flags before the last dry/rewet pass
  // host wall time per stage of rg_sim_step (rg_sim_stage_ms)
  double stage_ms[RG_SIM_NSTAGE] = {};
  int stage_cur = -1;
  std::chrono::steady_clock::time_point stage_t0;
};

// close the running stage of rg_sim_step and start stage `next` (-1: none)
static void stage_switch(rg_sim* s, int next) {
  const auto now = std::chrono::steady_clock::now();
  if (s->stage_cur >= 0)
    s->stage_ms[s->stage_cur] += std::chrono::duration<double, std::milli>(now - s->stage_t0).count();
  s->stage_cur = next;
  s->stage_t0 = now;
}

static rg_status sfail(rg_sim* s, rg_status st, const std::string& m) {
  s->err = m;
  return st;
}

// ---- MODEL::Initialize and helpers ----------------------------------------

static void connection(rg_sim* s, unsigned dry) {
  int* noel = s->noel.data();
  s->pool->run(s->np, [&](long long b, long long e, int) { std::fill(noel + b, noel + e, 0); });
  s->pool->run(s->ne, [&](long long b, long long e, int) {
    for (long long k = b; k < e; k++) {
      if (dry && (s->eflag[k] & dry)) continue;
      for (int i = 0; i < 6; i++) __atomic_fetch_add(&noel[s->en[6 * k + i]], 1, __ATOMIC_RELAXED);
    }
  });
}

static void boundary(rg_sim* s) {
  for (int n = 0; n < s->np; n++) {
    s->nflag[n] &= ~N_BOUND;
    if (s->bckind[n] & B_AUTOSLIP) s->bckind[n] &= ~(B_AUTOSLIP | B_FIXU | B_FIXV);
  }
  for (int n = 0; n < s->np; n++)
    if (s->noel[n] == 1 && (s->nflag[n] & N_MIDS)) s->nflag[n] |= N_BOUND;
  s->bel.clear();
  std::fill(s->boundList.begin(), s->boundList.end(), -1);
  for (int e = 0; e < s->ne; e++) {
    if (s->eflag[e] & E_DRY) continue;
    const int* nd = &s->en[6 * e];
    for (int i = 3; i < 6; i++) {
      if (!(s->nflag[nd[i]] & N_BOUND)) continue;
      int left = i - 3, rght = (left + 1) % 3;
      BElem b;
      b.nd[0] = nd[left];
      b.nd[1] = nd[rght];
      b.nd[2] = nd[i];
      b.flag = E_BOUND;
      b.region = e;
      s->boundList[nd[i]] = (int)s->bel.size();
      s->nflag[nd[left]] |= N_BOUND;
      s->nflag[nd[rght]] |= N_BOUND;
      s->bel.push_back(b);
    }
  }
}

static void set_location(rg_sim* s) {
  for (BElem& b : s->bel) {
    bool inlet = true, outlet = true, open = true;
    for (int i = 0; i < 2; i++) {
      unsigned k = s->bckind[b.nd[i]];
      if (!(k & B_INLET)) inlet = false;
      if (!(k & B_OUTLET)) outlet = false;
      if (!(k & B_OPENBND)) open = false;
    }
    if (inlet) b.flag |= E_INLET;
    if (outlet) b.flag |= E_OUTLET;
    if (open) b.flag |= E_OPENBND;
    for (int i = 0; i < 3; i++) {
      if (inlet) s->nflag[b.nd[i]] |= N_INLET;
      if (outlet) s->nflag[b.nd[i]] |= N_OUTLET;
      if (open) s->nflag[b.nd[i]] |= N_OPENBND;
    }
  }
  for (int n = 0; n < s->np; n++) s->nflag[n] &= ~N_NOMOMENT;
  for (BElem& b : s->bel)
    for (int i = 0; i < 2; i++) {
      int k = b.nd[i];
      if (s->noel[k] == 1 && !(s->nflag[k] & (N_INLET | N_OUTLET | N_OPENBND))) s->nflag[k] |= N_NOMOMENT;
    }
}

static void initialize(rg_sim* s) {
  s->model_init++;
  connection(s, E_DRY);
  boundary(s);
  s->mnodes.clear();
  for (int n = 0; n < s->np; n++)
    if (!(s->nflag[n] & N_DRY)) s->mnodes.push_back(n);
  s->melems.clear();
  for (int e = 0; e < s->ne; e++) {
    if (s->eflag[e] & E_DRY) continue;
    s->melems.push_back(e);
    for (int i = 3; i < 6; i++) {
      int k = s->en[6 * e + i];
      if (s->nflag[k] & N_BOUND) s->melems.push_back(-1 - s->boundList[k]);
    }
  }
  set_location(s);
}

// ---- MODEL::SetNormal / SetRotation ----------------------------------------

static void set_normal(rg_sim* s) {
  std::fill(s->bnx.begin(), s->bnx.end(), 0.0);
  std::fill(s->bny.begin(), s->bny.end(), 0.0);
  std::fill(s->niox.begin(), s->niox.end(), 0.0);
  std::fill(s->nioy.begin(), s->nioy.end(), 0.0);
  // derivatives of the quadratic line shape at its nodes (xi = -1, 1, 0)
  const double xi[3] = {-1.0, 1.0, 0.0};
  for (const BElem& b : s->bel) {
    for (int i = 0; i < 3; i++) {
      double d[3] = {xi[i] - 0.5, xi[i] + 0.5, -2.0 * xi[i]};
      double nx = 0.0, ny = 0.0;
      for (int j = 0; j < 3; j++) {
        nx += 2.0 * (d[j] * s->y[b.nd[j]]);
        ny -= 2.0 * (d[j] * s->x[b.nd[j]]);
      }
      int k = b.nd[i];
      if (b.flag & (E_INLET | E_OUTLET | E_OPENBND)) {
        s->niox[k] += nx;
        s->nioy[k] += ny;
      } else {
        s->bnx[k] += nx;
        s->bny[k] += ny;
      }
    }
  }
  for (int n = 0; n < s->np; n++) {
    if (s->nflag[n] & N_DRY) continue;
    if (!(s->nflag[n] & N_BOUND)) continue;
    double len = std::sqrt(s->bnx[n] * s->bnx[n] + s->bny[n] * s->bny[n]);
    if (std::fabs(len) < 1.0e-12) {
      s->bnx[n] = s->bny[n] = 0.0;
    } else {
      s->bnx[n] /= len;
      s->bny[n] /= len;
    }
    len = std::sqrt(s->niox[n] * s->niox[n] + s->nioy[n] * s->nioy[n]);
    if (std::fabs(len) < 1.0e-12) {
      s->niox[n] = s->nioy[n] = 0.0;
    } else {
      s->niox[n] /= len;
      s->nioy[n] /= len;
    }
  }
}

static void set_rotation(rg_sim* s, std::vector<int>* zero_uv) {
  for (int n = 0; n < s->np; n++) {
    s->nflag[n] &= ~N_ROTAT;
    s->rot[n] = ROT_NONE;
    unsigned& k = s->bckind[n];
    if (k & B_INLET) k &= ~(B_FIXU | B_FIXV);
    if (k & B_AUTOSLIP) k &= ~(B_AUTOSLIP | B_FIXU | B_FIXV);
    bool bound = (s->nflag[n] & N_BOUND) != 0;
    if (bound && !(k & (B_INLET | B_OUTLET | B_OPENBND | B_SLIP | B_SETUV))) {
      s->rot[n] = ROT_TANGENT;
      k |= B_AUTOSLIP | B_FIXV;
    }
  }
  for (const BElem& b : s->bel) {
    if (b.flag & (E_OUTLET | E_OPENBND)) continue;
    for (int i = 0; i < 2; i++) {
      int n = b.nd[i];
      unsigned& k = s->bckind[n];
      if ((k & (B_OUTLET | B_OPENBND)) && !(k & (B_SLIP | B_SETUV))) {
        s->rot[n] = ROT_NORMAL;
        k |= B_AUTOSLIP | B_FIXV;
      }
    }
  }
  for (int n = 0; n < s->np; n++) {
    if (s->bckind[n] & B_AUTOSLIP) {
      double len = std::sqrt(s->bnx[n] * s->bnx[n] + s->bny[n] * s->bny[n]);
      if (len < 1.0e-12) s->nflag[n] |= N_NOMOMENT;
    }
  }
  for (int n = 0; n < s->np; n++) {
    unsigned& k = s->bckind[n];
    if (k & B_INLET) {
      s->nflag[n] |= N_ROTAT;
      k |= B_FIXV;
      s->rot[n] = ROT_NORMAL;
    }
    if ((s->nflag[n] & N_NOMOMENT) && !(k & (B_SETUV | B_OUTLET | B_OPENBND))) {
      k |= B_AUTOSLIP | B_FIXU | B_FIXV;
      s->U[n] = s->V[n] = 0.0;
      if (zero_uv) zero_uv->push_back(n);
    } else if ((k & B_FIXV) && (k & B_AUTOSLIP)) {
      s->nflag[n] |= N_ROTAT;
      s->rot[n] = (k & (B_OUTLET | B_OPENBND)) ? ROT_NORMAL : ROT_TANGENT;
    }
  }
}

static void getrot(const rg_sim* s, int n, double r[4]) {
  // BCON::Getrot (Bcon.cpp:209-238)
  switch (s->rot[n]) {
    case ROT_TANGENT:
      r[0] = s->bny[n];
      r[1] = s->bnx[n];
      r[2] = -s->bnx[n];
      r[3] = s->bny[n];
      break;
    case ROT_NORMAL:
      r[0] = s->niox[n];
      r[1] = s->nioy[n];
      r[2] = s->nioy[n];
      r[3] = -s->niox[n];
      break;
    default:
      r[0] = r[1] = r[2] = r[3] = 0.0;
  }
}

// ---- BCONSET::InitBcon ------------------------------------------------------

// returns true when the inlet was dry and its water level was initialised
// values_only: the node kinds and BCVAL::S are those of the last full call
// (same time, same wet model); only BCVAL::U (and S of a dry inlet) are
// recomputed, for the control-line nodes -- the same values a full call gives
static bool init_bcon(rg_sim* s, double t, bool values_only = false) {
  bool s_changed = false;
  const int np = s->np;
  std::vector<unsigned>& kind = s->ib_kind;
  std::vector<char>& has = s->ib_has;
  std::vector<double>& vU = s->ib_vU;
  std::vector<double>& vS = s->ib_vS;
  std::vector<char>& mark = s->ib_mark;
  if ((int)kind.size() != np) {
    kind.assign(np, 0);
    has.assign(np, 0);
    vU.assign(np, 0.0);
    vS.assign(np, 0.0);
    mark.assign(np, 0);
  }
  // only control-line nodes are ever written
  for (int n : s->line_nodes) {
    kind[n] = 0;
    has[n] = 0;
    vU[n] = vS[n] = 0.0;
  }
  for (const LineBc& b : s->bcl) {
    for (int n : s->line_nodes) mark[n] = 0;
    unsigned k = b.kind;
    if (k & B_QTINLET) k |= B_QINLET;
    if (k & B_QINLET) k |= B_INLET;
    if (k & B_INLET) {
      // BCONLINE::Inlet, QINLET / QTINLET (BconLine.cpp:260-511)
      double Sspec = b.S[0];
      double Qspec = (k & B_QTINLET) ? interp_hydro(b, t, &Sspec) : b.Q[0];
      double Q = 0.0;
      bool any = false;
      const double gx = std::sqrt(0.6);
      const double gp[3] = {-gx, 0.0, gx}, gw[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
      for (size_t c = 0; c < s->seg_line.size(); c++) {
        if (s->seg_line[c] != b.line) continue;
        const int* nd = &s->seg_nodes[3 * c];
        double q[3];
        for (int i = 0; i < 3; i++) {
          int n = nd[i];
          if (s->S[n] - s->z[n] < 1.0e-9 || (s->nflag[n] & (N_DRY | N_MARSH))) {
            q[i] = 0.0;
          } else {
            double h = Sspec - s->z[n];
            q[i] = (h > 0.0) ? std::sqrt(h * h * h) : 0.0;
            if (s->cf[n] > 0.0) q[i] /= std::sqrt(s->cf[n]);
            any = true;
          }
          mark[n] = 1;
        }
        for (int g = 0; g < 3; g++) {
          double x = gp[g];
          double N[3] = {x * (x - 1.0) / 2.0, x * (x + 1.0) / 2.0, 1.0 - x * x};
          double dN[3] = {x - 0.5, x + 0.5, -2.0 * x};
          double dx = dN[0] * s->x[nd[0]] + dN[1] * s->x[nd[1]] + dN[2] * s->x[nd[2]];
          double dy = dN[0] * s->y[nd[0]] + dN[1] * s->y[nd[1]] + dN[2] * s->y[nd[2]];
          double qg = N[0] * q[0] + N[1] * q[1] + N[2] * q[2];
          Q += gw[g] * std::sqrt(dx * dx + dy * dy) * qg;
        }
      }
      double Qratio = (std::fabs(Q) > 0.0) ? (-Qspec / Q) : 0.0;
      if (!any) {
        // dry inlet: initialise S along the line, integrate on zor (BconLine.cpp:380-455)
        Q = 0.0;
        for (size_t c = 0; c < s->seg_line.size(); c++) {
          if (s->seg_line[c] != b.line) continue;
          const int* nd = &s->seg_nodes[3 * c];
          double q[3];
          for (int i = 0; i < 3; i++) {
            s->S[nd[i]] = Sspec;
            double h = Sspec - s->zor[nd[i]];
            q[i] = (h > 0.0) ? std::sqrt(h * h * h) : 0.0;
          }
          for (int g = 0; g < 3; g++) {
            double x = gp[g];
            double N[3] = {x * (x - 1.0) / 2.0, x * (x + 1.0) / 2.0, 1.0 - x * x};
            double dN[3] = {x - 0.5, x + 0.5, -2.0 * x};
            double dx = dN[0] * s->x[nd[0]] + dN[1] * s->x[nd[1]] + dN[2] * s->x[nd[2]];
            double dy = dN[0] * s->y[nd[0]] + dN[1] * s->y[nd[1]] + dN[2] * s->y[nd[2]];
            double qg = N[0] * q[0] + N[1] * q[1] + N[2] * q[2];
            Q += gw[g] * std::sqrt(dx * dx + dy * dy) * qg;
          }
        }
        Qratio = (std::fabs(Q) > 0.0) ? (-Qspec / Q) : 0.0;
        s_changed = true;
      }
      for (int n : s->line_nodes) {
        if (!mark[n]) continue;
        double qn = 0.0;
        if (!(s->nflag[n] & (N_DRY | N_MARSH))) {
          double h = Sspec - s->z[n];
          qn = (h > 0.0) ? std::sqrt(h * h * h) : 0.0;
          if (s->cf[n] > 0.0) qn /= std::sqrt(s->cf[n]);
        }
        if (!has[n]) {
          kind[n] = k;
          has[n] = 1;
          vU[n] = qn * Qratio;
          vS[n] = Sspec;
        } else if (!(kind[n] & (B_OUTLET | B_SLIP | B_SETUV))) {
          kind[n] |= k;
          vU[n] = qn * Qratio;
          vS[n] = Sspec;
        }
      }
    } else if (k & B_OUTLET) {
      // BCONLINE::Outlet, constant S along the line (BconLine.cpp:861-903)
      for (size_t c = 0; c < s->seg_line.size(); c++) {
        if (s->seg_line[c] != b.line) continue;
        const int* nd = &s->seg_nodes[3 * c];
        for (int i = 0; i < 3; i++) {
          int n = nd[i];
          if (mark[n]) continue;
          mark[n] = 1;
          if (!has[n]) {
            kind[n] = k;
            has[n] = 1;
            vS[n] = b.S[0];
          } else if (!(kind[n] & (B_INLET | B_QINLET | B_QTINLET))) {
            kind[n] |= k;
            vS[n] = b.S[0];
          }
        }
      }
    }
  }
  if (values_only) {
    for (int n : s->line_nodes) s->bcU[n] = has[n] ? vU[n] : 0.0;
    return s_changed;
  }
  for (int n = 0; n < np; n++) {
    unsigned k = kind[n];
    if (has[n] && (k & B_INLET)) k &= ~(B_OUTLET | B_SLIP | B_SETUV);
    s->bckind[n] = has[n] ? k : 0;
    s->has_val[n] = has[n];
    s->bcU[n] = has[n] ? vU[n] : 0.0;
    s->bcS[n] = has[n] ? vS[n] : 0.0;
  }
  return s_changed;
}

// ---- EQS::SetEqno / LastEquation / ResetEqOrder / SetIndexMat ----------------

static void elem_nodes(const rg_sim* s, int me, const int** nd, int* nnd) {
  if (me >= 0) {
    *nd = &s->en[6 * me];
    *nnd = 6;
  } else {
    *nd = s->bel[-1 - me].nd;
    *nnd = 3;
  }
}

static rg_status set_eqno(rg_sim* s) {
  const unsigned fix[3] = {B_FIXU, B_FIXV, B_SETS};
  std::vector<int>& eq = s->eqno;
  std::fill(eq.begin(), eq.end(), -1);
  int neq = 0;
  for (int n : s->mnodes) {
    if (s->nflag[n] & N_CORN) {
      for (int j = 0; j < 3; j++)
        if (!(s->bckind[n] & fix[j])) eq[3 * n + j] = neq++;
    } else {
      for (int j = 0; j < 2; j++)
        if (!(s->bckind[n] & fix[j])) eq[3 * n + j] = neq++;
    }
  }
  // last occurrence of every equation in element order (SetEqno.cpp:231-384)
  std::vector<int> counter(neq, 0);
  const size_t nme = s->melems.size();
  for (size_t e = 0; e < nme; e++) {
    const int* nd;
    int nnd;
    elem_nodes(s, s->melems[e], &nd, &nnd);
    for (int i = 0; i < nnd; i++)
      for (int j = 0; j < 3; j++) {
        int q = eq[3 * nd[i] + j];
        if (q >= 0) counter[q]++;
      }
  }
  std::vector<int> ord(neq, -1);
  int m = 0;
  for (size_t e = 0; e < nme; e++) {
    const int* nd;
    int nnd;
    elem_nodes(s, s->melems[e], &nd, &nnd);
    for (int i = 0; i < nnd; i++)
      for (int j = 0; j < 3; j++) {
        int q = eq[3 * nd[i] + j];
        if (q >= 0) {
          if (--counter[q] == 0) ord[q] = m++;
        }
      }
  }
  if (m != neq) return sfail(s, RG_ERR_ARG, "equation numbering: inconsistent last occurrences");
  for (size_t k = 0; k < eq.size(); k++)
    if (eq[k] >= 0) eq[k] = ord[eq[k]];
  s->neq = neq;
  // CRS pattern, diagonal first then first-seen columns (IndexMat.cpp:126-288).  The
  // columns of a row are the equations of every node of every model element that holds
  // the row's node, first seen first (elements in model order, nodes in element order,
  // U V S per node), so all rows of one node share one neighbour list; each node's
  // rows are built on the host threads from a node -> element list.
  const int np = s->np;
  std::vector<long long> nptr(np + 1, 0);
  for (size_t e = 0; e < nme; e++) {
    const int* nd;
    int nnd;
    elem_nodes(s, s->melems[e], &nd, &nnd);
    for (int i = 0; i < nnd; i++) nptr[nd[i] + 1]++;
  }
  for (int n = 0; n < np; n++) nptr[n + 1] += nptr[n];
  std::vector<int> nel(nptr[np]);
  {
    std::vector<long long> fill(nptr.begin(), nptr.end() - 1);
    for (size_t e = 0; e < nme; e++) {
      const int* nd;
      int nnd;
      elem_nodes(s, s->melems[e], &nd, &nnd);
      for (int i = 0; i < nnd; i++) nel[fill[nd[i]]++] = (int)e;
    }
  }
  constexpr int kMaxNb = 256;
  // neighbour nodes of n in first-seen order; false if there are more than kMaxNb
  auto neighbours = [&](int n, int* nb, int* cnt) -> bool {
    int c = 0;
    for (long long q = nptr[n]; q < nptr[n + 1]; q++) {
      const int* nd;
      int nnd;
      elem_nodes(s, s->melems[nel[q]], &nd, &nnd);
      for (int i = 0; i < nnd; i++) {
        const int m2 = nd[i];
        bool seen = false;
        for (int t = 0; t < c; t++)
          if (nb[t] == m2) {
            seen = true;
            break;
          }
        if (seen) continue;
        if (c == kMaxNb) return false;
        nb[c++] = m2;
      }
    }
    *cnt = c;
    return true;
  };
  s->width.assign(neq, 0);
  std::atomic<int> overflow{0};
  HostPool& pool = *s->pool;
  pool.run(np, [&](long long b, long long e, int) {
    int nb[kMaxNb], c = 0;
    for (long long n = b; n < e; n++) {
      if (nptr[n] == nptr[n + 1]) continue;
      if (!neighbours((int)n, nb, &c)) {
        overflow = 1;
        return;
      }
      int cols = 0;
      for (int t = 0; t < c; t++)
        for (int l = 0; l < 3; l++) cols += eq[3 * nb[t] + l] >= 0;
      for (int j = 0; j < 3; j++)
        if (eq[3 * n + j] >= 0) s->width[eq[3 * n + j]] = cols;
    }
  });
  if (overflow) return sfail(s, RG_ERR_ARG, "CRS pattern: a node has more than 256 neighbours");
  std::vector<long long> rp(neq + 1, 0);
  for (int i = 0; i < neq; i++) rp[i + 1] = rp[i] + s->width[i];
  s->index.assign((size_t)rp[neq], 0);
  pool.run(np, [&](long long b, long long e, int) {
    int nb[kMaxNb], c = 0;
    for (long long n = b; n < e; n++) {
      if (nptr[n] == nptr[n + 1] || !neighbours((int)n, nb, &c)) continue;
      for (int j = 0; j < 3; j++) {
        const int row = eq[3 * n + j];
        if (row < 0) continue;
        int* out = s->index.data() + rp[row];
        int o = 0;
        out[o++] = row;
        for (int t = 0; t < c; t++)
          for (int l = 0; l < 3; l++) {
            const int col = eq[3 * nb[t] + l];
            if (col >= 0 && col != row) out[o++] = col;
          }
      }
    }
  });
  return RG_OK;
}

// ---- GRID::DryRewet, method 2 -----------------------------------------------

static void dry_rewet(rg_sim* s, int* dried, int* wetted) {
  // GRID::DryRewet method 2 (DryRewet.cpp:696-990), the passes of the
  // reference in its order; node and element passes run on the host threads
  // (per-item writes, commutative flag updates), the marsh-corner water
  // levels -- which read levels set earlier in the same pass -- in element order
  const double dryLimit = s->p.dry_limit, rewetLimit = s->p.rewet_limit;
  const int countDown = s->p.countdown;
  const int np = s->np, ne = s->ne;
  std::vector<char>& nmark = s->dw_nmark;
  std::vector<char>& emark = s->dw_emark;
  nmark.resize(np);
  emark.resize(ne);
  unsigned* nflag = s->nflag.data();
  unsigned* eflag = s->eflag.data();
  const int* en = s->en.data();
  double* S = s->S.data();
  double* z = s->z.data();
  const double* zor = s->zor.data();
  HostPool& pool = *s->pool;
  pool.run(np, [&](long long b, long long e, int) {
    for (long long n = b; n < e; n++) {
      nmark[n] = (nflag[n] & N_DRY) != 0;
      nflag[n] &= ~N_MARSH;
      double H = S[n] - zor[n];
      if (H < dryLimit) {
        nflag[n] |= N_DRY;
        s->countdown[n] = countDown;
      } else {
        if (s->countdown[n] > 0)
          s->countdown[n]--;
        else
          nflag[n] &= ~N_DRY;
      }
      z[n] = zor[n];
    }
  });
  pool.run(ne, [&](long long b, long long ee, int) {
    for (long long e = b; e < ee; e++) {
      emark[e] = (eflag[e] & E_DRY) != 0;
      eflag[e] &= ~(E_DRY | E_MARSH);
      const int* nd = &en[6 * e];
      int ndry = 0;
      for (int i = 0; i < 3; i++)
        if (nflag[nd[i]] & N_DRY) ndry++;
      if (ndry == 3) {
        eflag[e] |= E_DRY;
      } else if (ndry) {
        eflag[e] |= E_MARSH;
        for (int i = 0; i < 3; i++)
          if (nflag[nd[i]] & N_DRY) atomic_or(&nflag[nd[i]], N_MARSH);
      }
    }
  });
  pool.run(np, [&](long long b, long long e, int) {
    for (long long n = b; n < e; n++) nflag[n] |= N_DRY;
  });
  // wet triangles clear kDry on their nodes; the ones with a marsh corner are listed in order
  const int nt = pool.threads();
  s->dw_marsh.resize(nt);
  for (auto& l : s->dw_marsh) l.clear();
  pool.run(ne, [&](long long b, long long ee, int t) {
    std::vector<int>& lst = s->dw_marsh[t];
    for (long long e = b; e < ee; e++) {
      if (eflag[e] & E_DRY) continue;
      const int* nd = &en[6 * e];
      for (int i = 0; i < 6; i++) atomic_and(&nflag[nd[i]], ~(unsigned)N_DRY);
      if ((nflag[nd[0]] | nflag[nd[1]] | nflag[nd[2]]) & N_MARSH) lst.push_back((int)e);
    }
  });
  for (const std::vector<int>& lst : s->dw_marsh)
    for (int e : lst) {
      const int* nd = &en[6 * e];
      for (int i = 0; i < 3; i++) {
        const int ni = nd[i];
        if (!(nflag[ni] & N_MARSH)) continue;
        if (nmark[ni] || s->firstDryRew) {
          int j = (i + 1) % 3, k = (i + 2) % 3;
          double Si;
          bool mj = (nflag[nd[j]] & N_MARSH) != 0, mk = (nflag[nd[k]] & N_MARSH) != 0;
          if (!mj && !mk)
            Si = (S[nd[j]] + S[nd[k]]) / 2.0;
          else if (!mj)
            Si = S[nd[j]];
          else if (!mk)
            Si = S[nd[k]];
          else
            Si = S[nd[(i + 2) % 3]];   // all corners marsh cannot happen for a marsh element
          S[ni] = Si;
          if (S[ni] > zor[ni] + rewetLimit) S[ni] = zor[ni] + rewetLimit;
          if (S[ni] < zor[ni] + dryLimit) z[ni] = S[ni] - dryLimit;
        } else {
          if (S[ni] < zor[ni] + dryLimit) z[ni] = S[ni] - dryLimit;
        }
      }
    }
  // mid-side levels from the corners: every triangle of a mid-side gives the same
  // value, the first one writes it; any marsh triangle may flag it
  pool.run(ne, [&](long long b, long long ee, int) {
    for (long long e = b; e < ee; e++) {
      const int* nd = &en[6 * e];
      for (int i = 3; i < 6; i++) {
        int l = nd[i - 3], r = nd[(i - 2) % 3];
        const double Sm = 0.5 * (S[l] + S[r]);
        const double zm = 0.5 * (z[l] + z[r]);
        if (s->mid_owner[nd[i]] == e) {
          S[nd[i]] = Sm;
          z[nd[i]] = zm;
        }
        if ((eflag[e] & E_MARSH) && zm + dryLimit / 10.0 < zor[nd[i]]) atomic_or(&nflag[nd[i]], N_MARSH);
      }
    }
  });
  pool.run(np, [&](long long b, long long e, int) {
    for (long long n = b; n < e; n++) {
      if (nflag[n] & N_DRY) {
        s->U[n] = s->V[n] = 0.0;
        S[n] = z[n] = zor[n];
        s->dUdt[n] = s->dVdt[n] = s->dSdt[n] = 0.0;
      }
    }
  });
  int d = 0, w = 0;
  for (int e = 0; e < ne; e++) {
    if ((eflag[e] & E_DRY) && !emark[e]) d++;
    if (!(eflag[e] & E_DRY) && emark[e]) w++;
  }
  *dried = d;
  *wetted = w;
}

// ---- device sync helpers ------------------------------------------------------

static rg_status push_state(rg_sim* s) {
  return rg_set_state(s->ctx, s->U.data(), s->V.data(), s->S.data(), s->dUdt.data(), s->dVdt.data(),
                      s->dSdt.data(), s->z.data(), nullptr, nullptr);
}

static rg_status pull_state(rg_sim* s) {
  rg_status st = rg_get_state(s->ctx, s->U.data(), s->V.data(), s->S.data(), s->z.data());
  if (st != RG_OK) return st;
  return rg_get_dt(s->ctx, s->dUdt.data(), s->dVdt.data(), s->dSdt.data());
}

static rg_status push_boundary(rg_sim* s) {
  std::vector<int> nf(s->np), bk(s->np);
  std::vector<double> r4(4 * (size_t)s->np);
  for (int n = 0; n < s->np; n++) {
    nf[n] = (int)s->nflag[n];
    bk[n] = (int)s->bckind[n];
    getrot(s, n, &r4[4 * (size_t)n]);
  }
  return rg_set_boundary(s->ctx, nf.data(), bk.data(), r4.data(), s->niox.data(), s->nioy.data(), s->bcU.data(),
                         s->bcS.data());
}

static rg_status push_model(rg_sim* s) {
  // element list in the order of MODEL::elem
  const size_t nme = s->melems.size();
  std::vector<int> enodes(6 * nme, -1), ennd(nme), eflag(nme);
  std::vector<double> evt(nme);
  for (size_t e = 0; e < nme; e++) {
    int me = s->melems[e];
    if (me >= 0) {
      for (int i = 0; i < 6; i++) enodes[6 * e + i] = s->en[6 * me + i];
      ennd[e] = 6;
      eflag[e] = (int)s->eflag[me];
      evt[e] = s->en_vt[me];
    } else {
      const BElem& b = s->bel[-1 - me];
      for (int i = 0; i < 3; i++) enodes[6 * e + i] = b.nd[i];
      ennd[e] = 3;
      eflag[e] = (int)b.flag;
      evt[e] = s->en_vt[b.region];
    }
  }
  rg_status st = rg_set_elements(s->ctx, (int)nme, enodes.data(), ennd.data(), eflag.data(), evt.data());
  if (st != RG_OK) return st;
  std::vector<int> eq(s->eqno.begin(), s->eqno.end());
  st = rg_set_pattern(s->ctx, s->neq, s->width.data(), s->index.data(), eq.data());
  if (st != RG_OK) return st;
  return rg_set_update_lists(s->ctx, (int)s->mnodes.size(), s->mnodes.data(), s->ne, s->en.data(), s->zor.data());
}

// MODEL::DoDryRewet (DoDryRew.cpp:50-239) with method 2 on the host state
static void slip_flow(rg_sim* s) {
  // GRID::SetSlipFlow (SlipFlow.cpp:42-80)
  double r[4];
  for (int n = 0; n < s->np; n++) {
    if (!(s->nflag[n] & N_ROTAT)) continue;
    getrot(s, n, r);
    double Ut = r[0] * s->U[n] + r[2] * s->V[n];
    s->U[n] = r[0] * Ut;
    s->V[n] = r[2] * Ut;
    Ut = r[0] * s->dUdt[n] + r[2] * s->dVdt[n];
    s->dUdt[n] = r[0] * Ut;
    s->dVdt[n] = r[2] * Ut;
  }
}

static void do_dry_rewet(rg_sim* s, int* del, int* wel) {
  // the boundary set-up stays valid when the pass leaves every node and element flag as it was
  s->dw_nflag0 = s->nflag;
  s->dw_eflag0 = s->eflag;
  connection(s, 0);
  *del = *wel = 0;
  if (s->p.dryrew_method == 2) dry_rewet(s, del, wel);
  if (*del + *wel) {
    initialize(s);
    set_normal(s);
    set_rotation(s, nullptr);
    slip_flow(s);
  } else {
    connection(s, E_DRY);
  }
  if (*del + *wel || s->nflag != s->dw_nflag0 || s->eflag != s->dw_eflag0) s->bc_valid = false;
  s->firstDryRew = false;
}

// =============================================================================

extern "C" {

rg_status rg_sim_create(const rg_deck* d, int precision, int device, rg_sim** out) {
  if (!d || !out || d->np <= 0 || d->ne <= 0 || !d->x || !d->y || !d->z || !d->elem_nodes || !d->elem_mat ||
      d->nmat <= 0 || !d->mat_n || !d->mat_vt)
    return RG_ERR_ARG;
  for (int e = 0; e < 6 * d->ne; e++)
    if (d->elem_nodes[e] < 0 || d->elem_nodes[e] >= d->np) return RG_ERR_ARG;
  for (int e = 0; e < d->ne; e++)
    if (d->elem_mat[e] < 0 || d->elem_mat[e] >= d->nmat) return RG_ERR_ARG;
  for (int k = 0; k < 3 * d->nseg; k++)
    if (d->seg_nodes[k] < 0 || d->seg_nodes[k] >= d->np) return RG_ERR_ARG;
  rg_sim* s = new rg_sim();
  *out = s;
  s->prec = precision;
  s->p = d->params;
  s->hmin = s->p.dry_limit / 2.0;   // PROJECT::hmin (Project.cpp:1125)
  s->np = d->np;
  s->ne = d->ne;
  s->x.assign(d->x, d->x + d->np);
  s->y.assign(d->y, d->y + d->np);
  s->zor.assign(d->z, d->z + d->np);
  // mid-side bed elevation is the mean of the corners (GRID::InputRegion, Grid.cpp:350-372)
  for (int e = 0; e < d->ne; e++) {
    const int* nd = d->elem_nodes + 6 * (size_t)e;
    for (int i = 3; i < 6; i++) s->zor[nd[i]] = 0.5 * (s->zor[nd[i - 3]] + s->zor[nd[(i - 2) % 3]]);
  }
  s->z = s->zor;
  s->en.assign(d->elem_nodes, d->elem_nodes + 6 * (size_t)d->ne);
  s->pool.reset(new HostPool(host_threads()));
  s->mid_owner.assign(d->np, -1);
  for (int e = 0; e < d->ne; e++)
    for (int i = 3; i < 6; i++)
      if (s->mid_owner[s->en[6 * e + i]] < 0) s->mid_owner[s->en[6 * e + i]] = e;
  s->en_n.resize(d->ne);
  s->en_vt.resize(d->ne);
  for (int e = 0; e < d->ne; e++) {
    s->en_n[e] = d->mat_n[d->elem_mat[e]];
    s->en_vt[e] = d->mat_vt[d->elem_mat[e]];
  }
  s->seg_nodes.assign(d->seg_nodes, d->seg_nodes + 3 * (size_t)d->nseg);
  s->seg_line.assign(d->seg_line, d->seg_line + d->nseg);
  s->line_nodes = s->seg_nodes;
  std::sort(s->line_nodes.begin(), s->line_nodes.end());
  s->line_nodes.erase(std::unique(s->line_nodes.begin(), s->line_nodes.end()), s->line_nodes.end());
  for (int b = 0; b < d->nbc; b++) {
    const rg_line_bc& lb = d->bc[b];
    LineBc l;
    l.line = lb.line;
    if (lb.kind == RG_BC_QINLET) {
      l.kind = B_QINLET;
      l.t = {0.0};
      l.Q = {lb.Q[0]};
      l.S = {lb.S[0]};
    } else if (lb.kind == RG_BC_QTINLET) {
      if (lb.npts < 1) return sfail(s, RG_ERR_ARG, "QTINLET needs points");
      l.kind = B_QTINLET;
      l.t.assign(lb.t, lb.t + lb.npts);
      l.Q.assign(lb.Q, lb.Q + lb.npts);
      l.S.assign(lb.S, lb.S + lb.npts);
    } else if (lb.kind == RG_BC_OUTLET) {
      l.kind = B_OUTLET;
      l.S = {lb.S[0]};
    } else {
      return sfail(s, RG_ERR_ARG, "unsupported boundary condition kind");
    }
    s->bcl.push_back(l);
  }
  const size_t np = d->np;
  s->eflag.assign(d->ne, E_REGION);
  s->nflag.assign(np, 0);
  for (int e = 0; e < d->ne; e++) {
    for (int i = 0; i < 3; i++) s->nflag[s->en[6 * e + i]] |= N_CORN;
    for (int i = 3; i < 6; i++) s->nflag[s->en[6 * e + i]] |= N_MIDS;
  }
  s->noel.assign(np, 0);
  s->countdown.assign(np, 0);
  s->boundList.assign(np, -1);
  s->bckind.assign(np, 0);
  s->rot.assign(np, 0);
  s->has_val.assign(np, 0);
  for (auto* v : {&s->bnx, &s->bny, &s->niox, &s->nioy, &s->bcU, &s->bcS, &s->U, &s->V, &s->S, &s->dUdt, &s->dVdt,
                  &s->dSdt, &s->oU, &s->oV, &s->oS, &s->odUdt, &s->odVdt, &s->odSdt, &s->cf})
    v->assign(np, 0.0);
  s->eqno.assign(3 * np, -1);
  // area factors of inclined elements (ArFact.cpp:41-97), from the initial bed
  s->en_af.resize(d->ne);
  for (int e = 0; e < d->ne; e++) {
    const int* nd = &s->en[6 * e];
    double xx[3], yy[3], zz[3];
    xx[0] = s->x[nd[0]];
    yy[0] = s->y[nd[0]];
    zz[0] = s->zor[nd[0]];
    for (int i = 1; i < 3; i++) {
      xx[i] = s->x[nd[i]] - xx[0];
      yy[i] = s->y[nd[i]] - yy[0];
      zz[i] = s->zor[nd[i]] - zz[0];
    }
    double t1 = yy[1] * zz[2] - yy[2] * zz[1];
    double t2 = zz[1] * xx[2] - zz[2] * xx[1];
    double t3 = xx[1] * yy[2] - xx[2] * yy[1];
    s->en_af[e] = std::sqrt(t1 * t1 + t2 * t2 + t3 * t3) / t3;
  }
  if (device == RG_DEVICE_NONE) return RG_OK;   // host model only (no GPU context)
  // the GPU context holds the mesh; elements are (re)loaded per model change
  rg_mesh m;
  std::vector<int> en1(6, 0), nnd1(1, 6), fl1(1, E_REGION);
  std::vector<double> vt1(1, 0.0);
  en1 = std::vector<int>(s->en.begin(), s->en.begin() + 6);
  m.np = d->np;
  m.x = s->x.data();
  m.y = s->y.data();
  m.ne = 1;
  m.elem_nodes = en1.data();
  m.elem_nnd = nnd1.data();
  m.elem_flag = fl1.data();
  m.elem_vt = vt1.data();
  m.g = s->p.g;
  m.hmin = s->hmin;
  m.vk = s->p.vk;
  rg_status st = rg_create(&m, precision, device, &s->ctx);
  if (st != RG_OK) return sfail(s, st, s->ctx ? rg_last_error(s->ctx) : "rg_create failed");
  st = rg_set_update_lists(s->ctx, 0, nullptr, s->ne, s->en.data(), s->zor.data());
  if (st != RG_OK) return sfail(s, st, rg_last_error(s->ctx));
  st = rg_set_friction(s->ctx, s->en_n.data(), s->en_af.data());
  if (st != RG_OK) return sfail(s, st, rg_last_error(s->ctx));
  // page-lock the node arrays the Newton loop moves between host and device (they keep their size)
  for (std::vector<double>* v : {&s->U, &s->V, &s->S, &s->dUdt, &s->dVdt, &s->dSdt, &s->z, &s->cf, &s->bcU})
    if (cudaHostRegister(v->data(), v->size() * sizeof(double), cudaHostRegisterDefault) == cudaSuccess)
      s->pinned.push_back(v->data());
    else
      (void)cudaGetLastError();   // stays pageable: slower copies, same results
  return RG_OK;
}

rg_ctx* rg_sim_context(rg_sim* s) { return s ? s->ctx : nullptr; }

rg_status rg_sim_destroy(rg_sim* s) {
  if (!s) return RG_OK;
  for (void* p : s->pinned) cudaHostUnregister(p);
  if (s->ctx) rg_destroy(s->ctx);
  delete s;
  return RG_OK;
}

const char* rg_sim_last_error(rg_sim* s) {
  if (!s) return "null simulation";
  if (!s->err.empty()) return s->err.c_str();
  return s->ctx ? rg_last_error(s->ctx) : "";
}

rg_status rg_sim_set_state(rg_sim* s, const double* U, const double* V, const double* S) {
  if (!s || !U || !V || !S) return RG_ERR_ARG;
  s->U.assign(U, U + s->np);
  s->V.assign(V, V + s->np);
  s->S.assign(S, S + s->np);
  std::fill(s->dUdt.begin(), s->dUdt.end(), 0.0);
  std::fill(s->dVdt.begin(), s->dVdt.end(), 0.0);
  std::fill(s->dSdt.begin(), s->dSdt.end(), 0.0);
  s->oU = s->U;
  s->oV = s->V;
  s->oS = s->S;
  s->odUdt = s->dUdt;
  s->odVdt = s->dVdt;
  s->odSdt = s->dSdt;
  // model set-up as at the start of PROJECT::Compute (Compute.cpp:170-180)
  std::fill(s->cf.begin(), s->cf.end(), 0.0);
  initialize(s);
  // boundary nodes of the whole grid keep kGridBnd for good (Model.cpp:301-307)
  for (int n = 0; n < s->np; n++)
    if (s->nflag[n] & N_BOUND) s->nflag[n] |= N_GRIDBND;
  init_bcon(s, 0.0);
  set_location(s);
  s->have_state = true;
  s->eqs_init = -1;
  s->factor_eqs = -1;
  return RG_OK;
}

rg_status rg_sim_get_state(rg_sim* s, double* U, double* V, double* S, double* z, int* nflag) {
  if (!s) return RG_ERR_ARG;
  if (U) std::copy(s->U.begin(), s->U.end(), U);
  if (V) std::copy(s->V.begin(), s->V.end(), V);
  if (S) std::copy(s->S.begin(), s->S.end(), S);
  if (z) std::copy(s->z.begin(), s->z.end(), z);
  if (nflag)
    for (int n = 0; n < s->np; n++) nflag[n] = (int)s->nflag[n];
  return RG_OK;
}

rg_status rg_sim_dry_rewet(rg_sim* s, int* dried, int* wetted) {
  if (!s || !s->have_state) return RG_ERR_ARG;
  int d = 0, w = 0;
  do_dry_rewet(s, &d, &w);
  if (dried) *dried = d;
  if (wetted) *wetted = w;
  return RG_OK;
}

rg_status rg_sim_prepare_iteration(rg_sim* s, double t_bc, const double* cf) {
  if (!s || !s->have_state) return RG_ERR_ARG;
  if (cf) s->cf.assign(cf, cf + s->np);
  s->bc_valid = false;
  init_bcon(s, t_bc);
  set_location(s);
  set_normal(s);
  set_rotation(s, nullptr);
  if (s->eqs_init != s->model_init) {
    s->eqs_init = s->model_init;
    return set_eqno(s);
  }
  return RG_OK;
}

rg_status rg_sim_get_numbering(rg_sim* s, int* neq, int* eqno, int* width, int64_t* nnz) {
  if (!s) return RG_ERR_ARG;
  if (neq) *neq = s->neq;
  if (eqno) std::copy(s->eqno.begin(), s->eqno.end(), eqno);
  if (width) std::copy(s->width.begin(), s->width.end(), width);
  if (nnz) *nnz = (int64_t)s->index.size();
  return RG_OK;
}

rg_status rg_sim_get_pattern(rg_sim* s, int* index) {
  if (!s || !index) return RG_ERR_ARG;
  std::copy(s->index.begin(), s->index.end(), index);
  return RG_OK;
}

rg_status rg_sim_get_boundary(rg_sim* s, int* nflag, int* bckind, double* rot4, double* bcU, double* bcS) {
  if (!s) return RG_ERR_ARG;
  for (int n = 0; n < s->np; n++) {
    if (nflag) nflag[n] = (int)s->nflag[n];
    if (bckind) bckind[n] = (int)s->bckind[n];
    if (rot4) getrot(s, n, rot4 + 4 * (size_t)n);
    if (bcU) bcU[n] = s->bcU[n];
    if (bcS) bcS[n] = s->bcS[n];
  }
  return RG_OK;
}

rg_status rg_sim_get_model(rg_sim* s, int* ne, int* elem_nodes, int* elem_nnd, int* elem_flag, double* elem_vt,
                           double* niox, double* nioy) {
  if (!s) return RG_ERR_ARG;
  const size_t nme = s->melems.size();
  if (ne) *ne = (int)nme;
  for (size_t e = 0; e < nme; e++) {
    const int me = s->melems[e];
    int nd[6] = {-1, -1, -1, -1, -1, -1}, nnd, fl;
    double vt;
    if (me >= 0) {
      for (int i = 0; i < 6; i++) nd[i] = s->en[6 * me + i];
      nnd = 6;
      fl = (int)s->eflag[me];
      vt = s->en_vt[me];
    } else {
      const BElem& b = s->bel[-1 - me];
      for (int i = 0; i < 3; i++) nd[i] = b.nd[i];
      nnd = 3;
      fl = (int)b.flag;
      vt = s->en_vt[b.region];
    }
    if (elem_nodes)
      for (int i = 0; i < 6; i++) elem_nodes[6 * e + i] = nd[i];
    if (elem_nnd) elem_nnd[e] = nnd;
    if (elem_flag) elem_flag[e] = fl;
    if (elem_vt) elem_vt[e] = vt;
  }
  for (int n = 0; n < s->np; n++) {
    if (niox) niox[n] = s->niox[n];
    if (nioy) nioy[n] = s->nioy[n];
  }
  return RG_OK;
}

rg_status rg_sim_stage_ms(rg_sim* s, double* ms, int n, int reset) {
  if (!s || n < 0 || (n > 0 && !ms)) return RG_ERR_ARG;
  for (int i = 0; i < n && i < RG_SIM_NSTAGE; i++) ms[i] = s->stage_ms[i];
  for (int i = RG_SIM_NSTAGE; i < n; i++) ms[i] = 0.0;
  if (reset)
    for (double& v : s->stage_ms) v = 0.0;
  return RG_OK;
}

rg_status rg_sim_continuity(rg_sim* s, int* nsect_out, double* Qx, double* Qy) {
  if (!s || !s->ctx) return RG_ERR_ARG;
  int nsect = 0;
  for (int l : s->seg_line) nsect = std::max(nsect, l);
  if (nsect_out) *nsect_out = nsect;
  if (!Qx && !Qy) return RG_OK;
  if (!Qx || !Qy || nsect == 0) return sfail(s, RG_ERR_ARG, "rg_sim_continuity: no control lines or no output");
  return rg_continuity(s->ctx, (int)s->seg_line.size(), s->seg_nodes.data(), s->seg_line.data(), nsect, Qx, Qy);
}

rg_status rg_sim_set_warm_start(rg_sim* s, const double* U, const double* V, const double* S) {
  if (!s || !s->have_state) return RG_ERR_ARG;
  if (!U || !V || !S) {
    s->warm_pending = false;
    return RG_OK;
  }
  s->wU.assign(U, U + s->np);
  s->wV.assign(V, V + s->np);
  s->wS.assign(S, S + s->np);
  s->warm_pending = true;
  return RG_OK;
}

rg_status rg_sim_step(rg_sim* s, double t, double dt, const rg_step_ctl* ctl, rg_step_report* rep) {
  if (!s || !ctl || !s->have_state || dt <= 0.0) return RG_ERR_ARG;
  if (!s->ctx) return sfail(s, RG_ERR_ARG, "rg_sim_step: created without a GPU context");
  auto t0 = std::chrono::steady_clock::now();
  s->bc_valid = false;   // new boundary time
  const bool steady = ctl->steady != 0;
  const double th = s->p.theta;
  double rUV, rH;
  if (steady) {
    rUV = rH = 0.0;   // relaxation method < 3, stationary (EqsUVS2D.cpp:117-126)
  } else {
    rUV = rH = 1.0 / dt / th;
  }
  rg_status st = rg_set_relax(s->ctx, rUV, rH);
  if (st != RG_OK) return st;
  st = rg_set_jacobian(s->ctx, ctl->friction_jacobian ? 1 : 0);
  if (st != RG_OK) return st;
  // Predict (EqsUVS2D.cpp:1101-1178)
  for (int n = 0; n < s->np; n++) s->dUdt[n] = s->dVdt[n] = s->dSdt[n] = 0.0;
  for (int n = 0; n < s->np; n++) {
    if (s->oS[n] < s->zor[n] + s->p.dry_limit) {
      if (ctl->first_step || (s->nflag[n] & N_DRYPREV)) {
        s->oU[n] = s->U[n];
        s->oV[n] = s->V[n];
        s->oS[n] = s->S[n];
      }
      s->odUdt[n] = s->odVdt[n] = s->odSdt[n] = 0.0;
    }
  }
  st = rg_set_old(s->ctx, s->oU.data(), s->oV.data(), s->oS.data(), s->odUdt.data(), s->odVdt.data(),
                  s->odSdt.data());
  if (st != RG_OK) return st;
  bool NRconv = true, DWconv = true;
  const int DWfreq = s->p.dryrew_freq;
  int nextDW = 0;
  int maxit = ctl->max_newton > 0 ? ctl->max_newton : s->p.max_newton;
  double first_norm = -1.0;
  double warm_res = -1.0;
  int warm_used = 0;
  int krylov_total = 0, newton = 0, dw_events = 0;
  bool converged = false;
  bool state_on_device = false;
  int status_solve = RG_OK;
  s->resid_hist.clear();
  rg_update_opts uo;
  uo.relax_method = s->p.relax_method;
  uo.max_delta_uv = s->p.max_delta_uv;
  uo.max_delta_s = s->p.max_delta_s;
  uo.max_us = s->p.max_us;
  uo.dry_limit = s->p.dry_limit;
  uo.dryrew_method = s->p.dryrew_method;
  double last_ratio = 1.0;
  const bool trace = getenv("RG_TRACE") != nullptr;
  const bool trace2 = trace && getenv("RG_TRACE")[0] == '2';
#define STAGE(name, idx)                                     \
  do {                                                       \
    stage_switch(s, idx);                                    \
    if (trace2) fprintf(stderr, "[rg]   stage %s\n", name); \
  } while (0)
  for (int it = 0; it < maxit; it++) {
    // dry / rewet every DWfreq iterations or when the corrections converged
    if (s->p.dryrew_method && DWfreq < s->p.max_newton) {
      if (nextDW >= 0 && (it == nextDW || NRconv)) {
        nextDW = it + DWfreq;
        if (state_on_device) {
          STAGE("pull_state", RG_STAGE_DOWNLOAD);
          st = pull_state(s);
          if (st != RG_OK) return st;
          state_on_device = false;
        }
        int del = 0, wel = 0;
        STAGE("dry_rewet", RG_STAGE_DRYREWET);
        do_dry_rewet(s, &del, &wel);
        if (trace2) fprintf(stderr, "[rg]   dried %d wetted %d\n", del, wel);
        dw_events++;
        // dry/rewet has converged when nothing got wet (EqsUVS2D.cpp:210-212)
        DWconv = (wel == 0);
        if (nextDW > maxit) {
          maxit = nextDW;
          nextDW = -1;
          DWconv = true;
        }
      }
    }
    NRconv = true;
    if (!state_on_device) {
      STAGE("push_state", RG_STAGE_UPLOAD);
      st = push_state(s);
      if (st != RG_OK) return st;
      state_on_device = true;
    }
    // friction (GPU), boundary data (host), assembly and scaling of the current state: ||B|| is the
    // Newton residual
    auto build_system = [&](double* scale) -> rg_status {
      rg_status st;
      // friction (GPU) and boundary data (host) of this iteration
      STAGE("friction", RG_STAGE_FRICTION);
      st = rg_friction(s->ctx, nullptr);
      if (st != RG_OK) return st;
      const int nline = (int)s->line_nodes.size();
      if (!s->bcl.empty()) {
        // the inlet distribution reads S, z and cf at the control-line nodes only: those
        // are gathered from the device (the host arrays elsewhere are refreshed by the
        // full transfers before the dry/rewet passes and at the end of the step)
        STAGE("inlet_state", RG_STAGE_DOWNLOAD);
        st = rg_gather_nodes(s->ctx, nline, s->line_nodes.data(), s->S.data(), s->z.data(), s->cf.data());
        if (st != RG_OK) return st;
      }
      STAGE("init_bcon", RG_STAGE_BCON);
      // the same time and wet model as the last set-up: kinds, normals and rotations repeat
      const bool refresh = s->bc_valid && s->eqs_init == s->model_init;
      if (init_bcon(s, t + dt, refresh)) {
        // a dry inlet set S along its line: back to the device at those nodes
        st = rg_scatter_nodes_S(s->ctx, nline, s->line_nodes.data(), s->S.data());
        if (st != RG_OK) return st;
      }
      if (refresh) {
        for (int n : s->zero_uv) s->U[n] = s->V[n] = 0.0;
      } else {
        set_location(s);
        set_normal(s);
        s->zero_uv.clear();
        set_rotation(s, &s->zero_uv);
      }
      if (!s->zero_uv.empty()) {
        st = rg_zero_velocity(s->ctx, (int)s->zero_uv.size(), s->zero_uv.data());
        if (st != RG_OK) return st;
      }
      if (s->eqs_init != s->model_init) {
        s->eqs_init = s->model_init;
        STAGE("set_eqno", RG_STAGE_NUMBERING);
        st = set_eqno(s);
        if (st != RG_OK) return st;
        STAGE("push_model", RG_STAGE_UPLOAD);
        st = push_model(s);
        if (st != RG_OK) return sfail(s, st, rg_last_error(s->ctx));
        st = rg_set_friction(s->ctx, s->en_n.data(), s->en_af.data());
        if (st != RG_OK) return st;
      }
      STAGE("push_boundary", RG_STAGE_UPLOAD);
      if (refresh) {
        st = rg_set_boundary(s->ctx, nullptr, nullptr, nullptr, nullptr, nullptr, s->bcU.data(), nullptr);
      } else {
        st = push_boundary(s);
        s->bc_valid = true;
      }
      if (st != RG_OK) return st;
      // assemble, scale: ||B_k|| is the Newton residual
      STAGE("assemble", RG_STAGE_ASSEMBLE);
      st = rg_assemble(s->ctx, nullptr, nullptr, nullptr);
      if (st != RG_OK) return st;
      return rg_scale(s->ctx, scale);
    };
    double scale = 0.0;
    st = build_system(&scale);
    if (st != RG_OK) return st;
    if (it == 0 && s->warm_pending) {
      STAGE("warm_start", RG_STAGE_WARM);
      // learned warm start: the predicted state replaces the last time level on the
      // wet nodes if its residual is the smaller one; ||B_0|| stays the plain start's
      s->warm_pending = false;
      const std::vector<double> pU = s->U, pV = s->V, pS = s->S;
      for (int n : s->mnodes) {
        s->U[n] = s->wU[n];
        s->V[n] = s->wV[n];
        s->S[n] = std::max(s->wS[n], s->z[n] + 0.5 * s->p.dry_limit);
      }
      // the fixed velocity component of slip-wall and inlet nodes is no Newton unknown:
      // project the prediction onto the free direction as GRID::SetSlipFlow does
      // (SlipFlow.cpp:42-80) for the last time level, so the fixed value stays the plain one
      for (int n : s->mnodes) {
        if (!(s->nflag[n] & N_ROTAT)) continue;
        double r[4];
        getrot(s, n, r);
        const double Ut = r[0] * s->U[n] + r[2] * s->V[n];
        s->U[n] = r[0] * Ut;
        s->V[n] = r[2] * Ut;
      }
      for (int e = 0; e < s->ne; e++) {   // mid-side S as the corner mean (k_upd_midside)
        if (s->eflag[e] & E_DRY) continue;
        const int* nd = &s->en[6 * e];
        for (int k = 0; k < 3; k++) s->S[nd[3 + k]] = 0.5 * (s->S[nd[k]] + s->S[nd[(k + 1) % 3]]);
      }
      st = push_state(s);
      if (st == RG_OK && !steady) st = rg_timegrad(s->ctx, dt, th);
      double wscale = 0.0;
      if (st == RG_OK) st = build_system(&wscale);
      if (st != RG_OK) return st;
      warm_res = wscale;
      if (wscale < scale) {
        warm_used = 1;
        first_norm = scale;
        scale = wscale;
      } else {
        s->U = pU;
        s->V = pV;
        s->S = pS;
        st = push_state(s);   // host time derivatives are still the predictor's zeros
        if (st == RG_OK) st = build_system(&scale);
        if (st != RG_OK) return st;
      }
    }
    if (first_norm < 0.0) first_norm = scale;
    s->resid_hist.push_back(scale);
    last_ratio = first_norm > 0.0 ? scale / first_norm : 0.0;
    if (ctl->criterion == RG_CRIT_RESIDUAL && it > 0 && last_ratio <= ctl->residual_tol && DWconv) {
      converged = true;
      break;
    }
    STAGE("factor", RG_STAGE_FACTOR);
    if (ctl->ilu_reuse <= 0 || s->factor_eqs != s->eqs_init || s->factor_age >= ctl->ilu_reuse) {
      st = rg_ilu0_factor(s->ctx, nullptr, nullptr);
      if (st != RG_OK) return st;
      s->factor_eqs = s->eqs_init;
      s->factor_age = 0;
    } else {
      s->factor_age++;   // the factors of an earlier Newton iteration precondition this one
    }
    STAGE("bicgstab", RG_STAGE_KRYLOV);
    int its = 0;
    // inexact Newton on request: the linear solve only as accurate as the forcing term
    const double lin_tol = std::max(s->p.solver_maxdiff, ctl->linear_forcing);
    st = rg_bicgstab(s->ctx, s->p.solver_maxiter, lin_tol, nullptr, &its, nullptr);
    krylov_total += its;
    if ((st == RG_NOT_CONVERGED || st == RG_ERR_NONFINITE) && s->factor_age > 0) {
      // the factors of an earlier iteration did not do: factor this matrix and solve again
      STAGE("factor", RG_STAGE_FACTOR);
      st = rg_ilu0_factor(s->ctx, nullptr, nullptr);
      if (st != RG_OK) return st;
      s->factor_eqs = s->eqs_init;
      s->factor_age = 0;
      STAGE("bicgstab", RG_STAGE_KRYLOV);
      st = rg_bicgstab(s->ctx, s->p.solver_maxiter, lin_tol, nullptr, &its, nullptr);
      krylov_total += its;
    }
    if (st != RG_OK && st != RG_NOT_CONVERGED) return st;
    if (st == RG_NOT_CONVERGED) {
      status_solve = RG_NOT_CONVERGED;
      s->factor_eqs = -1;   // fresh factors for the next iteration
    }
    double stats[6];
    STAGE("update", RG_STAGE_UPDATE);
    st = rg_newton_update(s->ctx, &uo, stats);
    if (st != RG_OK) return st;
    newton++;
    if (trace)
      fprintf(stderr, "[rg] t=%g it=%d neq=%d |B|=%.6e krylov=%d st=%d dU=%.3e dV=%.3e dS=%.3e dw=%d\n", t, it, s->neq,
              scale, its, (int)st, stats[0], stats[1], stats[2], dw_events);
    if (stats[0] > s->p.conv_uv || stats[1] > s->p.conv_uv || stats[2] > s->p.conv_s) NRconv = false;
    if (!steady) {
      STAGE("timegrad", RG_STAGE_UPDATE);
      st = rg_timegrad(s->ctx, dt, th);
      if (st != RG_OK) return st;
    }
    if (ctl->criterion == RG_CRIT_CORRECTION && NRconv && DWconv) {
      converged = true;
      break;
    }
  }
  STAGE("end_of_step", RG_STAGE_DOWNLOAD);
  if (state_on_device) {
    st = pull_state(s);
    if (st != RG_OK) return st;
  }
  stage_switch(s, -1);
  // GRID::SetSlipFlow at the end of the step (EqsUVS2D.cpp:1078)
  slip_flow(s);
  // end of the time step (Compute.cpp:774-810)
  for (int n = 0; n < s->np; n++) {
    if (s->nflag[n] & N_DRY)
      s->nflag[n] |= N_DRYPREV;
    else
      s->nflag[n] &= ~N_DRYPREV;
    if (s->nflag[n] & N_MARSH)
      s->nflag[n] |= N_MARSHPREV;
    else
      s->nflag[n] &= ~N_MARSHPREV;
    s->oU[n] = s->U[n];
    s->oV[n] = s->V[n];
    s->oS[n] = s->S[n];
    s->odUdt[n] = s->dUdt[n];
    s->odVdt[n] = s->dVdt[n];
    s->odSdt[n] = s->dSdt[n];
  }
  for (int e = 0; e < s->ne; e++) {
    if (s->eflag[e] & E_DRY)
      s->eflag[e] |= E_DRYPREV;
    else
      s->eflag[e] &= ~E_DRYPREV;
    if (s->eflag[e] & E_MARSH)
      s->eflag[e] |= E_MARSHPREV;
    else
      s->eflag[e] &= ~E_MARSHPREV;
  }
  auto t1 = std::chrono::steady_clock::now();
  if (rep) {
    rep->newton_iterations = newton;
    rep->krylov_iterations = krylov_total;
    rep->converged = converged ? 1 : 0;
    rep->residual_first = first_norm;
    rep->residual_ratio = last_ratio;
    rep->neq = s->neq;
    rep->dryrew_events = dw_events;
    rep->wall_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    int nh = (int)std::min<size_t>(s->resid_hist.size(), 64);
    rep->n_hist = nh;
    for (int i = 0; i < nh; i++) rep->residual_hist[i] = s->resid_hist[i];
    int nd = 0;
    for (int n = 0; n < s->np; n++)
      if (s->nflag[n] & N_DRY) nd++;
    rep->dry_nodes = nd;
    rep->solver_status = status_solve;
    rep->warm_start = warm_used;
    rep->residual_warm = warm_res;
  }
  return converged ? RG_OK : RG_NOT_CONVERGED;
}

}  // extern "C"

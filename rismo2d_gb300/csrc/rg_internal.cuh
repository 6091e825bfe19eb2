// Internal declarations of the rg300 library (not part of the C ABI).
#pragma once

#include "../../include/rg300.h"
#include "../../include/rg300_sim.h"

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

// widest CRS row the warp kernels handle (the reference's default mceq is 100,
// Project.cpp:1706-1752; P2 triangles give at most ~45)
#define RG_MAXW 128

// element-matrix size: 3 dof x 5 rows used by a P2 triangle (15), stored 16 wide
#define RG_EQ 15
#define RG_KSTRIDE 16

// reference flag bits (Node.h, Elem.h, Bcon.h)
#define RG_N_ROTAT    32
#define RG_E_INLET     1
#define RG_E_OUTLET    2
#define RG_E_OPENBND   4
#define RG_E_BOUND    16
#define RG_E_DRY     128
#define RG_B_INLET     1
#define RG_B_OUTLET    2
#define RG_B_OPENBND   4
#define RG_B_LOGLAW  256

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  cudaError_t alloc(size_t count) {
    if (count == n && p) return cudaSuccess;
    release();
    n = count;
    if (count == 0) return cudaSuccess;
    return cudaMalloc((void**)&p, count * sizeof(T));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  size_t bytes() const { return n * sizeof(T); }
};

// level-ordered chunk layout of one triangular factor (rg_trsv.cu).  A chunk
// image is meta[m] (int4: row, entry count, byte offset of its warp slice,
// pinned slot or -1) | b[m] | diag[m] (U solve) | warp slices.  A slice holds
// the entries of 32/G rows (G threads per row) column by column: column t has
// 32 source slots (int32) then 32 values, lane l = G*(row in slice) + g
// holding the row's entry j = G*t + g, so lane l reads its entry at
// slice + t*32*(4+sizeof(VT)) + 4*l (source) and + 128 + sizeof(VT)*l (value).
struct WaveChunk {
  long long img_off;   // byte offset of the chunk image (16-aligned)
  int img_bytes;       // multiple of 16
  int nrows;
  int pos0;            // level-order position of the chunk's first row
  int b_off;           // byte offsets inside the image: right-hand side, diagonal (U solve)
  int diag_off;
  int far_dep;         // split layouts: the last chunk holding a far source of this chunk (-1: none)
  int pad0, pad1, pad2, pad3;
};
constexpr int kWaveSlice = 32;      // rows per warp slice
// one CTA: 16 consumer warps, a producer warp and a publisher warp
constexpr int kWaveRows = 512;      // rows per chunk at most (one per consumer thread)
constexpr int kWaveThreads = kWaveRows + 64;
constexpr int kWaveMaxStages = 8;
// shared-memory ring of solved values and pinned slots for far sources, per value
// size: the FP64 ring holds half the slots so that both solves keep three stages
// in flight (the solve's rate is bounded by the copies in flight)
constexpr int kWaveRing = 16384, kWaveRing64 = 8192;
constexpr int kWavePin = 4096, kWavePin64 = 2048;
constexpr int kWaveStages32 = 3, kWaveStages64 = 3;
constexpr int wave_ring(int vtb) { return vtb == 8 ? kWaveRing64 : kWaveRing; }
constexpr int wave_pin(int vtb) { return vtb == 8 ? kWavePin64 : kWavePin; }
constexpr int wave_stages(int vtb) { return vtb == 8 ? kWaveStages64 : kWaveStages32; }
// dynamic shared memory available to the wavefront kernel
constexpr int kWaveSmem = 232448 - 2048;
struct WaveLayout {
  int n = 0, depth = 0;
  std::vector<WaveChunk> chunks;
  std::vector<unsigned char> img_host;
  long long img_bytes = 0;
  std::vector<int> order, bidx, ent_src, diag_src;
  std::vector<long long> ent_dst, diag_dst;
  // split layouts: the far entries of the row at level-order position p are
  // far_src[far_ptr[p], far_ptr[p + 1]) (source rows), their values packed into
  // the far value array from factor positions far_vsrc
  std::vector<long long> far_ptr;
  std::vector<int> far_src, far_vsrc;
  long long ring_misses = 0;
  int pinned = 0;
};
// ring: shared-memory ring slots; pin: fixed slots for sources read from
// farther back than the ring reaches (src encoding: [0, ring) ring slot,
// [ring, ring + pin) pinned slot, negative: -(row + 1) read from global
// memory).  split = true (FP32 solves, whose summation order is free): the
// entries whose source lies outside the ring and the pinned slots leave the
// chunk image for the far lists, summed into the right-hand side by helper
// blocks before the chunk is solved;
// bidx[p]: element index (in units of the vector type) of the right-hand side
// slot of level-order position p inside the image
WaveLayout build_wave_layout(int n, const std::vector<int>& ptr, const std::vector<int>& dep,
                             const std::vector<int>& src_pos, const std::vector<int>& diag_pos, bool lower,
                             int vt_bytes, int ring, int pin, int stage_cap, int rows_max, int lanes,
                             bool split = false);
// threads per row of the wavefront solves: one, i.e. the reference's summation
// order (bit-identical for double vectors); 2 or 4 split long rows
constexpr int kWaveLanes64 = 1, kWaveLanes32 = 1;

// per-solve scalars kept on the device (BiCGStab state, reductions)
struct KrylovScalars {
  double rho, alfa, omega, beta;
  double l2r0, diff, accuracy;
  double t1, t2;
  int it, done, conv, restarts;
};

struct WaveDev {
  DBuf<unsigned char> img;
  DBuf<WaveChunk> chunks;
  DBuf<int> order, bidx, ent_src, diag_src;
  // split layouts: far lists, their values, and the per-chunk flags and progress
  // word of the helper blocks
  DBuf<long long> far_ptr;
  DBuf<int> far_src, far_vsrc;
  DBuf<unsigned char> far_val;
  DBuf<int> chunk_ready;
  DBuf<unsigned long long> progress;
  bool split = false;
  long long nfar = 0;
  unsigned epoch = 0;
  DBuf<long long> ent_dst, diag_dst;
  long long nchunks = 0, nent = 0, ndiag = 0;
  int stage_bytes = 0, lanes = 1, depth = 0, max_chunk_bytes = 0;
  long long ring_misses = 0;
  // level schedule of the factorisation (L levels)
  std::vector<int> lev_ptr;
};

struct rg_ctx {
  int device = 0;
  int prec = RG_PREC_FP64;
  cudaStream_t st = nullptr;
  std::string err;
  int num_sms = 0;

  // mesh and constants
  int np = 0, ne = 0;
  double g = 9.81, hmin = 0.0, vk = 0.0, rUV = 0.0, rH = 0.0;
  int jac_friction = 0;       // rg_set_jacobian: depth derivative of the friction coefficient
  double fp64_pivot_depth = 0.0;   // rg_set_fp64_pivots: rows shallower than this factor in FP64 (mixed)
  DBuf<double> x, y, evt;
  DBuf<int> enodes, ennd, eflag;
  std::vector<int> h_enodes, h_ennd, h_eflag, h_region_nodes;

  // node state and boundary data
  DBuf<double> U, V, S, dUdt, dVdt, dSdt, z, cf, cfw;
  DBuf<double> oU, oV, oS, odUdt, odVdt, odSdt;   // previous time level (NODE::vo)
  DBuf<int> zero_nodes;
  DBuf<int> nflag, bckind;
  DBuf<double> rot, niox, nioy, bcU, bcS;
  bool have_boundary = false;

  // pattern (reference layout: diagonal first, first-seen column order)
  int neq = 0;
  int64_t nnz = 0;
  std::vector<int> h_rowptr, h_col;
  DBuf<int> eqno, rowptr, col;
  DBuf<int> slot;            // per element RG_EQ*RG_EQ CRS positions (-1 = none)
  DBuf<int> erow;            // per element RG_EQ equation numbers of its rows
  std::vector<int> color_ptr;
  DBuf<int> color_elem;      // elements grouped by colour (the assembly order)
  // two-phase assembly: element matrices by position in color_elem, then one
  // gather per CRS entry / equation over its contributions in that order
  DBuf<int> asm_reg, asm_bnd;        // positions of region triangles / boundary lines
  int n_asm_reg = 0, n_asm_bnd = 0;
  DBuf<long long> gat_ptr, grow_ptr; // per CRS entry (nnz + 1) / per equation (neq + 1)
  DBuf<int> gat_src;                 // position * RG_EQ*RG_EQ + r * RG_EQ + c
  DBuf<int> grow_src;                // position * RG_EQ + r
  DBuf<double> EK64, EF;             // element matrices (FP64 Jacobian), element residuals
  DBuf<double> geo;                  // per region triangle: Gauss-point weights and shape derivatives
  bool geo_valid = false;            // geo matches the current element lists
  DBuf<float> EK32;                  // element matrices (FP32 Jacobian)

  // values
  DBuf<double> A64, LU64;
  DBuf<float> A32, LU32;
  DBuf<double> B;
  bool have_system = false, have_factor = false;

  // ILU(0) factor schedule: per row, L positions sorted by column
  DBuf<int> lsort_ptr, lsort_pos;
  DBuf<int> fflag;           // row-done flags of the factorisation (epoch valued)
  int fepoch = 0;

  // triangular-solve operands split from the factors
  DBuf<int> Lptr, Lcol, Lsrc, Uptr, Ucol, Usrc;
  DBuf<double> Lv64, Uv64, Dv64;
  DBuf<float> Lv32, Uv32, Dv32;

  // Krylov vectors (double) and float copies for the mixed path
  DBuf<double> r0, ri, vi, pi, yi, zi, ti, tt, xm, X, tmp;
  DBuf<float> f_r0, f_ri, f_vi, f_pi, f_yi, f_zi, f_ti, f_x, f_xm, f_b, f_w;
  DBuf<double> partial;      // block partial sums of reductions
  DBuf<KrylovScalars> ks;
  KrylovScalars* ks_host = nullptr;   // pinned mirror
  DBuf<int> dev_err;         // device error word
  int* err_host = nullptr;

  // Newton update
  DBuf<int> model_nodes, region_nodes;
  DBuf<double> zor, upd;     // upd: reduction scratch
  int np_model = 0, ne_region = 0;
  DBuf<double> elem_n, elem_af;  // friction: Manning n, area factor per region triangle
  DBuf<int> fr_ptr, fr_el;       // node -> region triangles (element order)
  DBuf<double> fr_phmin;         // hmin^0.333333 as the friction kernel's pow gives it
  double fr_phmin_h = -1.0;      // the hmin it was computed for

  // continuity sections (rg_continuity): line elements sorted by section
  DBuf<int> sec_nodes, sec_ptr;
  DBuf<double> sec_q;
  int n_sec = 0;
  // node subsets read or written by the host model between full state transfers
  DBuf<int> sel_idx;
  DBuf<double> sel_val;
  std::vector<double> sel_host;

  // timings
  cudaEvent_t ev[16];
  double t_ms[10] = {0};   // device ms by stage; [8] / [9] host ms of the last / all rg_set_pattern calls

  int persist_blocks = 0;    // co-resident blocks for the persistent kernels
  WaveDev waveL, waveU;      // wavefront triangular solves
  DBuf<int> flev_ptr, flev_rows;   // level schedule of the factorisation
  DBuf<long long> fmap_off;          // per sorted L entry: offset into fmap
  DBuf<int> lsort_col;               // per sorted L entry: its column (the pivot row)
  DBuf<short> fmap;                  // fill map (position in the row, -1 = dropped)
  DBuf<unsigned char> fp64row;       // per equation: near-dry row, eliminated in FP64 (mixed)
  int use_wave = 1;
  int use_level_factor = 1;
  int n_repair_fallbacks = 0, n_factor_calls = 0;
  int depth_L = 0, depth_U = 0, n_colors = 0;
  int trace = 0;                // RG_TRACE level (diagnostics to stderr)   // dependency depth of the triangular solves
  cudaEvent_t user_ev[8];
  bool user_ev_ready = false;

  // host <-> device bytes moved by the ABI calls, kernel launches (cumulative)
  long long h2d_bytes = 0, d2h_bytes = 0;
  long long n_launches = 0;

  // per-kernel-class device time (rg_profile): event pairs around launches,
  // summed whenever the pool fills or a call synchronises
  static constexpr int kProfClasses = 4;
  static constexpr int kProfPairs = 2048;
  bool prof_on = false;
  std::vector<cudaEvent_t> prof_ev;        // 2 * kProfPairs
  std::vector<int> prof_cls;               // class of each recorded pair
  int prof_used = 0;
  long long prof_launches[kProfClasses] = {0};
  double prof_ms[kProfClasses] = {0};
};

// the context's stream as a launch argument, counting the launch
inline cudaStream_t rg_counted(rg_ctx* c) {
  c->n_launches++;
  return c->st;
}

// kernel classes of rg_profile
enum { RG_PROF_TRSV = 0, RG_PROF_SPMV = 1, RG_PROF_FACTOR = 2, RG_PROF_ASSEMBLE = 3 };
// open / close one timed launch of class `cls` (no-ops unless profiling)
cudaError_t prof_begin(rg_ctx* c, int cls);
cudaError_t prof_end(rg_ctx* c);
// wait for the recorded pairs and add them to the sums
cudaError_t prof_flush(rg_ctx* c);

// ---- launchers implemented in the .cu files -------------------------------
rg_status rg_fail(rg_ctx* c, rg_status s, const char* msg);
rg_status rg_cuda(rg_ctx* c, cudaError_t e, const char* where);
// read and clear the device error word; maps its bits to a status (rg_api.cu)
rg_status check_device_error(rg_ctx* c);
// S, z and the friction coefficient of the nodes idx[0..n) into S[idx[i]], z[idx[i]],
// cf[idx[i]] of full-size host arrays (any of them may be null); S[idx[i]] back to the device
rg_status rg_gather_nodes(rg_ctx* c, int n, const int* idx, double* S, double* z, double* cf);
rg_status rg_scatter_nodes_S(rg_ctx* c, int n, const int* idx, const double* S);

// Launch attributes and occupancy figures are properties of a device: a
// process may drive contexts on several GPUs, so they are cached per device.
constexpr int kMaxDevices = 64;
inline bool device_slot_ok(const rg_ctx* c) { return c->device >= 0 && c->device < kMaxDevices; }

// assembly (rg_assemble.cu)
cudaError_t launch_assemble(rg_ctx* c);
cudaError_t launch_friction(rg_ctx* c);

// linear algebra (rg_linalg.cu)
cudaError_t launch_scale(rg_ctx* c, double* scale_host);
cudaError_t launch_factor(rg_ctx* c);
cudaError_t launch_factor_level(rg_ctx* c);
cudaError_t launch_build_fmap(rg_ctx* c);
cudaError_t launch_near_dry_rows(rg_ctx* c);
cudaError_t launch_split(rg_ctx* c);
cudaError_t launch_spmv_d(rg_ctx* c, const double* x, double* r);
cudaError_t launch_ilu_apply_d(rg_ctx* c, const double* b, double* x);
cudaError_t launch_ilu_apply_w(rg_ctx* c, const double* b, double* w, double* x);
cudaError_t launch_ilu_apply_f(rg_ctx* c, const float* b, float* w, float* y);
rg_status   run_bicgstab(rg_ctx* c, int maxIter, double maxDiff, int* iters, double* acc);
cudaError_t launch_wave_solve(rg_ctx* c, bool dbl, const void* b, void* w, void* y, const KrylovScalars* ks);
cudaError_t launch_wave_pack(rg_ctx* c);
cudaError_t launch_update(rg_ctx* c, const rg_update_opts* o, double* stats);

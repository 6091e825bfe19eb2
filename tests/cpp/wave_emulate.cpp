// CPU emulation of the wavefront triangular solve (rg_trsv.cu) on the host
// layout built by build_wave_layout (rg_wave_layout.cpp).  Checks the layout
// invariants the TMA bulk copies rely on (16-byte alignment and sizes, stage
// capacities) and that the ring-slot assignment never reads an overwritten
// slot: every chunk is solved twice, once in row order and once in reverse,
// writing each result to the ring immediately, and both must match a plain
// sequential triangular solve exactly.  For split layouts it also runs the
// handshake of the helper blocks, the producer, the consumers and the progress
// publisher as a model under random interleavings and checks that every schedule
// completes (no deadlock).
#include "../../rismo2d_gb300/csrc/rg_internal.cuh"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

static int fails = 0;
#define CHECK(c, ...)                      \
  do {                                     \
    if (!(c)) {                            \
      fails++;                             \
      if (fails < 20) {                    \
        fprintf(stderr, "FAIL: " __VA_ARGS__); \
        fprintf(stderr, "\n");             \
      }                                    \
    }                                      \
  } while (0)

static long long g_far_entries = 0;   // far entries over all split runs
static long long g_protocol_runs = 0;  // interleavings of the split-solve handshake explored

// The handshake of a split solve (rg_trsv.cu) as a set of agents, run under random
// interleavings until every chunk is solved or no agent can move (a deadlock):
//   * producer: stages chunk p once the consumers have finished chunk p - nst (its
//     stage is free) and the chunk's flag is set (helpers flag every chunk);
//   * consumers: solve chunk c once it is staged;
//   * publisher: copies the consumers' count into the progress word, at any later time;
//   * helper h of H: takes chunks h, h + H, ... in order; a chunk without far entries
//     is flagged at once, a chunk with far entries once the progress word has passed
//     its far_dep (and, with l2_ahead > 0, once it is within l2_ahead chunks).
static bool protocol_completes(const std::vector<WaveChunk>& chunks, int nst, int H, int l2_ahead,
                               unsigned seed) {
  const int N = (int)chunks.size();
  std::mt19937 rng(seed);
  std::vector<char> flag(N, 0);
  std::vector<int> hnext(H);
  for (int h = 0; h < H; h++) hnext[h] = h;
  int staged = 0, solved = 0, progress = 0;
  while (solved < N) {
    std::vector<int> enabled;   // 0 producer, 1 consumers, 2 publisher, 3 + h helper h
    if (staged < N && (staged < nst || solved >= staged - nst + 1) && flag[staged]) enabled.push_back(0);
    if (solved < staged) enabled.push_back(1);
    if (progress < solved) enabled.push_back(2);
    for (int h = 0; h < H; h++) {
      const int k = hnext[h];
      if (k >= N) continue;
      long long dep = chunks[k].far_dep + 1;
      if (l2_ahead > 0) dep = std::max(dep, (long long)k - l2_ahead);
      if (progress >= dep) enabled.push_back(3 + h);
    }
    if (enabled.empty()) return false;
    const int a = enabled[rng() % enabled.size()];
    if (a == 0) {
      staged++;
    } else if (a == 1) {
      solved++;
    } else if (a == 2) {
      progress = solved;
    } else {
      const int h = a - 3;
      flag[hnext[h]] = 1;
      hnext[h] += H;
    }
  }
  return true;
}

template <class VT>
static void run(int n, int band, int seed, bool lower, int ring, int pin, int stage_cap, int lanes,
                bool split = false) {
  std::mt19937 rng(seed);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  // random triangular structure within a band
  std::vector<int> ptr(n + 1, 0), dep, srcpos;
  std::vector<double> val;
  for (int i = 0; i < n; i++) {
    int k = (int)(rng() % 9);
    for (int t = 0; t < k; t++) {
      int d = 1 + (int)(rng() % band);
      int j = lower ? i - d : i + d;
      if (j < 0 || j >= n) continue;
      bool dup = false;
      for (int q = ptr[i]; q < (int)dep.size(); q++) dup |= dep[q] == j;
      if (dup) continue;
      dep.push_back(j);
      srcpos.push_back((int)val.size());
      val.push_back(U(rng) * 0.3);
    }
    ptr[i + 1] = (int)dep.size();
  }
  std::vector<int> diag_pos(n);
  for (int i = 0; i < n; i++) {
    diag_pos[i] = (int)val.size();
    val.push_back(1.5 + U(rng) * 0.2);
  }
  const int vtb = sizeof(VT);
  const int rows_max = kWaveRows / lanes;
  const int rps = 32 / lanes;
  WaveLayout w = build_wave_layout(n, ptr, dep, srcpos, diag_pos, lower, vtb, ring, pin, stage_cap, rows_max, lanes,
                                   split);
  CHECK(!split || (long long)w.far_ptr.size() == (long long)n + 1, "far list per position");
  g_far_entries += (long long)w.far_src.size();
  if (split && ring - rows_max >= kWaveMaxStages * rows_max) {
    // the library's rings: the handshake completes for any helper count and schedule
    const int nst = vtb == 8 ? kWaveStages64 : kWaveStages32;
    for (int H : {1, 2, 7, 151})
      for (int l2 : {0, kWaveMaxStages, 64})
        for (unsigned sd = 0; sd < 3; sd++) {
          CHECK(protocol_completes(w.chunks, nst, H, l2, seed * 131u + sd), "split-solve handshake deadlocks: n=%d "
                "H=%d l2_ahead=%d", n, H, l2);
          g_protocol_runs++;
        }
  }
  // pack values as the device kernel does
  std::vector<unsigned char> img = w.img_host;
  for (size_t q = 0; q < w.ent_dst.size(); q++) {
    VT v = (VT)val[w.ent_src[q]];
    std::memcpy(&img[w.ent_dst[q]], &v, sizeof(VT));
  }
  for (size_t q = 0; q < w.diag_dst.size(); q++) {
    VT v = (VT)val[w.diag_src[q]];
    std::memcpy(&img[w.diag_dst[q]], &v, sizeof(VT));
  }
  std::vector<VT> b(n);
  for (auto& v : b) v = (VT)U(rng);
  // right-hand side into the images (k_gather_lev)
  for (int p = 0; p < n; p++) {
    CHECK((long long)w.bidx[p] * vtb + vtb <= (long long)img.size(), "rhs slot out of range");
    std::memcpy(&img[(size_t)w.bidx[p] * vtb], &b[w.order[p]], sizeof(VT));
  }
  // reference solve, the summation order of PRECO_ILU0::Solve
  std::vector<VT> xr(n);
  for (int t = 0; t < n; t++) {
    int i = lower ? t : n - 1 - t;
    VT acc = b[i];
    for (int q = ptr[i]; q < ptr[i + 1]; q++) {
      VT prod = (VT)val[srcpos[q]] * xr[dep[q]];
      acc = lower ? acc + prod : acc - prod;
    }
    xr[i] = lower ? acc : acc / (VT)val[diag_pos[i]];
  }
  const int sb = (split && ring + pin <= 65536) ? 2 : 4;   // 16-bit source slots in split layouts
  const long long stride = 32ll * (sb + vtb);
  for (int pass = 0; pass < 2; pass++) {
    std::vector<VT> ringv(ring + pin, (VT)NAN), x(n, (VT)NAN);
    std::vector<int> chunk_of(n, -1);
    std::vector<unsigned char> im = img;   // the helpers write the far sums into the images
    int written = 0, kchunk = -1;
    for (const WaveChunk& ch : w.chunks) {
      kchunk++;
      CHECK(ch.img_off % 16 == 0 && ch.img_bytes % 16 == 0, "image alignment");
      CHECK(ch.b_off % 16 == 0 && ch.diag_off % 16 == 0, "part alignment");
      CHECK(ch.img_bytes <= stage_cap || ch.nrows == 1, "stage capacity %d > %d", ch.img_bytes, stage_cap);
      CHECK(ch.nrows >= 1 && ch.nrows <= rows_max, "rows per chunk");
      CHECK(ch.pos0 == written, "chunk positions contiguous");
      unsigned char* st = &im[ch.img_off];
      if (split) {
        // a helper block: far sums of the chunk's rows into their right-hand sides, once
        // the chunks up to far_dep are solved; with the library's ring that is more than
        // kWaveMaxStages chunks back, so the producer never waits on itself
        bool any = false;
        for (int r = 0; r < ch.nrows; r++) {
          const int p = ch.pos0 + r;
          VT sum = 0;
          for (long long e = w.far_ptr[p]; e < w.far_ptr[p + 1]; e++) {
            const int j = w.far_src[e];
            CHECK(j >= 0 && j < n && !std::isnan((double)x[j]), "far source %d not solved before its chunk", j);
            CHECK(chunk_of[j] <= ch.far_dep, "far source %d after the chunk's far_dep", j);
            sum += (VT)val[w.far_vsrc[e]] * x[j];
            any = true;
          }
          VT br;
          std::memcpy(&br, st + ch.b_off + (size_t)vtb * r, sizeof(VT));
          br = lower ? br + sum : br - sum;
          std::memcpy(st + ch.b_off + (size_t)vtb * r, &br, sizeof(VT));
        }
        CHECK(any == (ch.far_dep >= 0), "far_dep marks the chunks with far entries");
        if (ring - rows_max >= kWaveMaxStages * rows_max)
          CHECK(ch.far_dep < 0 || ch.far_dep < kchunk - kWaveMaxStages, "far sources too recent for the helpers");
      } else {
        CHECK(ch.far_dep < 0, "no far lists without split");
      }
      for (int rr = 0; rr < ch.nrows; rr++) {
        int r = pass == 0 ? rr : ch.nrows - 1 - rr;
        int meta[4];
        std::memcpy(meta, st + 16 * r, 16);
        CHECK(meta[2] % 16 == 0 && meta[2] >= ch.diag_off, "slice offset");
        CHECK(meta[2] + (long long)((meta[1] + lanes - 1) / lanes) * stride <= ch.img_bytes,
              "slice inside the chunk image");
        VT b_r;
        std::memcpy(&b_r, st + ch.b_off + (size_t)vtb * r, sizeof(VT));
        // lane g of the row sums entries g, g + lanes, ...; one lane: from b in the factor's order
        VT part[4] = {0, 0, 0, 0};
        if (lanes == 1) part[0] = b_r;
        for (int e = 0; e < meta[1]; e++) {
          const int g = e % lanes, lane = (r % rps) * lanes + g;
          VT v;
          int src;
          if (sb == 2) {
            unsigned short s16;
            std::memcpy(&s16, st + meta[2] + (e / lanes) * stride + 2 * lane, 2);
            src = s16;
          } else {
            std::memcpy(&src, st + meta[2] + (e / lanes) * stride + 4 * lane, 4);
          }
          std::memcpy(&v, st + meta[2] + (e / lanes) * stride + 32 * sb + (size_t)vtb * lane, sizeof(VT));
          CHECK(src < ring + pin, "source slot out of range");
          CHECK(!split || src >= 0, "no global reads in split layouts");
          VT xv = src >= 0 ? ringv[src] : x[-src - 1];
          if (src < 0) CHECK(!std::isnan((double)xv), "global source not solved");
          VT prod = v * xv;
          part[g] = (lower || lanes > 1) ? part[g] + prod : part[g] - prod;
        }
        VT acc = part[0];
        if (lanes == 2) acc = part[0] + part[1];
        if (lanes == 4) acc = (part[0] + part[1]) + (part[2] + part[3]);
        if (lanes > 1) acc = lower ? b_r + acc : b_r - acc;
        VT xi;
        if (lower) {
          xi = acc;
        } else {
          VT d;
          std::memcpy(&d, st + ch.diag_off + (size_t)vtb * r, sizeof(VT));
          xi = acc / d;
        }
        ringv[(ch.pos0 + r) % ring] = xi;
        if (meta[3] >= 0) {
          CHECK(meta[3] >= ring && meta[3] < ring + pin, "pinned slot out of range");
          ringv[meta[3]] = xi;
        }
        x[meta[0]] = xi;
        chunk_of[meta[0]] = kchunk;
      }
      written += ch.nrows;
    }
    CHECK(written == n, "all rows solved");
    int bad = 0;
    double err = 0, scale = 1e-30;
    for (int i = 0; i < n; i++) {
      bad += !(x[i] == xr[i]);
      err = std::max(err, (double)std::fabs(x[i] - xr[i]));
      scale = std::max(scale, (double)std::fabs(xr[i]));
    }
    if (lanes == 1 && !split)   // same products in the same order: identical results
      CHECK(bad == 0, "n=%d band=%d lower=%d pass=%d: %d rows differ", n, band, (int)lower, pass, bad);
    else                        // split sums: a few ulps
      CHECK(err <= 1e-4 * scale, "n=%d band=%d lower=%d pass=%d lanes=%d err=%g", n, band, (int)lower, pass, lanes,
            err / scale);
  }
}

int main() {
  // the stage sizes of the library's shared-memory budget
  const int st32 = (int)(((kWaveSmem - (long long)(kWaveRing + kWavePin) * 4) / kWaveStages32) & ~255ll);
  const int st64 = (int)(((kWaveSmem - (long long)(kWaveRing64 + kWavePin64) * 8) / kWaveStages64) & ~255ll);
  for (int lower = 0; lower < 2; lower++) {
    for (int n : {1, 2, 7, 64, 1000, 20000}) {
      for (int band : {1, 3, 50, 600}) {
        run<double>(n, band, n + band, lower, kWaveRing64, kWavePin64, st64, kWaveLanes64);
        run<float>(n, band, n + band + 1, lower, kWaveRing, kWavePin, st32, kWaveLanes32);
        run<float>(n, band, n + band + 5, lower, kWaveRing, kWavePin, st32, 1);
        run<double>(n, band, n + band + 6, lower, kWaveRing64, kWavePin64, st64, 2);
        // tiny rings, pinned tables and stages force pinning, global reads and level splitting
        run<double>(n, band, n + band + 2, lower, 64, 16, 4096, 1);
        run<float>(n, band, n + band + 3, lower, 32, 0, 2048, 4);
        run<float>(n, band, n + band + 4, lower, 16, 4096, 2048, 4);
        // split layouts (far entries summed by helper blocks): the library's ring, and a
        // ring small enough for far entries on these bands
        run<float>(n, band, n + band + 7, lower, kWaveRing, kWavePin, st32, 1, true);
        run<double>(n, band, n + band + 11, lower, kWaveRing64, kWavePin64, st64, 1, true);
        run<float>(n, band, n + band + 8, lower, 2048, 8, st32, 1, true);
        run<float>(n, band * 8, n + band + 9, lower, 2048, 64, 8192, 1, true);
        run<double>(n, band * 8, n + band + 10, lower, 2048, 64, st64, 1, true);
      }
    }
  }
  CHECK(g_far_entries > 0, "the split runs exercise far entries");
  CHECK(g_protocol_runs > 0, "the handshake model ran");
  // the model is not vacuous: a chunk that waited on its own solution (far_dep >= k, which
  // the layout never produces) deadlocks under every schedule, and a far source just
  // before the chunk does not
  {
    std::vector<WaveChunk> bad(12);
    for (int k = 0; k < 12; k++) bad[k].far_dep = -1;
    bad[5].far_dep = 5;
    for (unsigned sd = 0; sd < 5; sd++)
      CHECK(!protocol_completes(bad, 3, 2, 0, sd), "the handshake model misses a self-dependent chunk");
    bad[5].far_dep = 4;
    for (unsigned sd = 0; sd < 5; sd++)
      CHECK(protocol_completes(bad, 3, 2, 0, sd), "the handshake model deadlocks on a far source just before");
  }
  if (fails) {
    fprintf(stderr, "%d failures\n", fails);
    return 1;
  }
  printf("wave layout emulation ok\n");
  return 0;
}

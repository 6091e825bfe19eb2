// CPU emulation of the wavefront triangular solve (rg_trsv.cu) on the host
// layout built by build_wave_layout (rg_wave_layout.cpp).  Checks the layout
// invariants the TMA bulk copies rely on (16-byte alignment and sizes, stage
// capacities) and that the ring-slot assignment never reads an overwritten
// slot: every chunk is solved twice, once in row order and once in reverse,
// writing each result to the ring immediately, and both must match a plain
// sequential triangular solve exactly.
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

template <class VT>
static void run(int n, int band, int seed, bool lower, int ring, int pin, int stage_cap, int bstage_cap) {
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
  WaveLayout w = build_wave_layout(n, ptr, dep, srcpos, diag_pos, lower, vtb, ring, pin, stage_cap, bstage_cap);
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
  std::vector<VT> blev(w.blev_len + 16, (VT)0);
  for (int p = 0; p < n; p++) blev[w.bidx[p]] = b[w.order[p]];
  // reference solve
  std::vector<VT> xr(n);
  for (int t = 0; t < n; t++) {
    int i = lower ? t : n - 1 - t;
    VT acc = 0;
    for (int q = ptr[i]; q < ptr[i + 1]; q++) acc += (VT)val[srcpos[q]] * xr[dep[q]];
    xr[i] = lower ? b[i] + acc : (b[i] - acc) / (VT)val[diag_pos[i]];
  }
  for (int pass = 0; pass < 2; pass++) {
    std::vector<VT> ringv(ring + pin, (VT)NAN), x(n, (VT)NAN);
    int written = 0;
    for (const WaveChunk& ch : w.chunks) {
      CHECK(ch.img_off % 16 == 0 && ch.img_bytes % 16 == 0, "image alignment");
      CHECK(ch.diag_off % 16 == 0 && ch.val_off % 16 == 0 && ch.src_off % 16 == 0, "part alignment");
      CHECK(ch.img_bytes <= stage_cap || ch.nrows == 1, "stage capacity %d > %d", ch.img_bytes, stage_cap);
      CHECK((ch.b_off * vtb) % 16 == 0 && ch.b_bytes % 16 == 0, "rhs alignment");
      CHECK(ch.b_bytes <= bstage_cap, "rhs stage capacity");
      CHECK(ch.pos0 == written, "chunk positions contiguous");
      const unsigned char* st = &img[ch.img_off];
      for (int rr = 0; rr < ch.nrows; rr++) {
        int r = pass == 0 ? rr : ch.nrows - 1 - rr;
        int meta[4];
        std::memcpy(meta, st + 16 * r, 16);
        VT acc = 0;
        for (int e = meta[1]; e < meta[1] + meta[2]; e++) {
          VT v;
          int src;
          std::memcpy(&v, st + ch.val_off + (size_t)vtb * e, sizeof(VT));
          std::memcpy(&src, st + ch.src_off + (size_t)4 * e, 4);
          CHECK(src < ring + pin, "source slot out of range");
          VT xv = src >= 0 ? ringv[src] : x[-src - 1];
          acc += v * xv;
        }
        VT bv = blev[ch.b_off + r];
        VT xi;
        if (lower) {
          xi = bv + acc;
        } else {
          VT d;
          std::memcpy(&d, st + ch.diag_off + (size_t)vtb * r, sizeof(VT));
          xi = (bv - acc) / d;
        }
        ringv[(ch.pos0 + r) % ring] = xi;
        if (meta[3] >= 0) {
          CHECK(meta[3] >= ring && meta[3] < ring + pin, "pinned slot out of range");
          ringv[meta[3]] = xi;
        }
        x[meta[0]] = xi;
      }
      written += ch.nrows;
    }
    CHECK(written == n, "all rows solved");
    double err = 0, scale = 1e-30;
    for (int i = 0; i < n; i++) {
      err = std::max(err, (double)std::fabs(x[i] - xr[i]));
      scale = std::max(scale, (double)std::fabs(xr[i]));
    }
    // same products, possibly different summation order: a few ulps
    CHECK(err <= (vtb == 8 ? 1e-12 : 1e-4) * scale, "n=%d band=%d lower=%d pass=%d err=%g", n, band, (int)lower,
          pass, err / scale);
  }
}

int main() {
  for (int lower = 0; lower < 2; lower++) {
    for (int n : {1, 2, 7, 64, 1000, 20000}) {
      for (int band : {1, 3, 50, 600}) {
        run<double>(n, band, n + band, lower, kWaveRing, kWavePin, kWaveStage64, kWaveBStage64);
        run<float>(n, band, n + band + 1, lower, kWaveRing, kWavePin, kWaveStage32, kWaveBStage32);
        // tiny rings, pinned tables and stages force pinning, global reads and level splitting
        run<double>(n, band, n + band + 2, lower, 64, 16, 1024, 64);
        run<float>(n, band, n + band + 3, lower, 32, 0, 512, 32);
        run<float>(n, band, n + band + 4, lower, 16, 4096, 512, 32);
      }
    }
  }
  if (fails) {
    fprintf(stderr, "%d failures\n", fails);
    return 1;
  }
  printf("wave layout emulation ok\n");
  return 0;
}

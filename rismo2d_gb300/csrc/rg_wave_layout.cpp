// Host-side layout of the wavefront triangular solves (rg_trsv.cu): level
// schedule of a triangular factor, split into stage-sized chunks, packed into
// one device image, with the shared-memory ring slot of every dependency.

#include "rg_internal.cuh"

#include <algorithm>
#include <cstring>


// Build the level-ordered chunk layout of one triangular factor.  `dep` lists,
// per row, the rows it reads (L: columns < row, U: columns > row); `src_pos`
// the factor positions of those entries; diag_pos the diagonal positions.
WaveLayout build_wave_layout(int n, const std::vector<int>& ptr, const std::vector<int>& dep,
                             const std::vector<int>& src_pos, const std::vector<int>& diag_pos, bool lower,
                             int vt_bytes, int ring, int stage_cap, int bstage_cap) {
  WaveLayout w;
  w.n = n;
  // levels
  std::vector<int> lev(n, 0);
  int nlev = 0;
  for (int t = 0; t < n; t++) {
    const int i = lower ? t : n - 1 - t;
    int l = 0;
    for (int q = ptr[i]; q < ptr[i + 1]; q++) l = std::max(l, lev[dep[q]] + 1);
    lev[i] = l;
    nlev = std::max(nlev, l + 1);
  }
  w.depth = nlev;
  std::vector<int> cnt(nlev + 1, 0);
  for (int i = 0; i < n; i++) cnt[lev[i] + 1]++;
  for (int l = 0; l < nlev; l++) cnt[l + 1] += cnt[l];
  std::vector<int> order(n), pos(n), fill(cnt.begin(), cnt.end() - 1);
  for (int t = 0; t < n; t++) {
    const int i = lower ? t : n - 1 - t;   // rows of a level in solve order
    const int p = fill[lev[i]]++;
    order[p] = i;
    pos[i] = p;
  }
  const int ent_bytes = (vt_bytes == 8) ? 16 : 8;
  auto a16 = [](long long v) { return (v + 15) & ~15ll; };
  // chunks: consecutive rows of a level, within the stage capacities
  std::vector<int> chunk_of(n);
  int p = 0;
  long long img_off = 0;
  int b_off = 0;
  const int b_align = 16 / vt_bytes;
  while (p < n) {
    const int l = lev[order[p]];
    const int lend = cnt[l + 1];
    WaveChunk ch{};
    ch.pos0 = p;
    int m = 0, ne = 0;
    while (p + m < lend) {
      const int i = order[p + m];
      const int k = ptr[i + 1] - ptr[i];
      long long bytes = a16(16ll * (m + 1)) + a16((long long)vt_bytes * (m + 1)) + (long long)ent_bytes * (ne + k);
      long long bb = a16((long long)vt_bytes * (m + 1));
      if (m > 0 && (a16(bytes) > stage_cap || bb > bstage_cap || m + 1 > 4096)) break;
      m++;
      ne += k;
    }
    ch.nrows = m;
    ch.diag_off = (int)a16(16ll * m);
    ch.ent_off = (int)(ch.diag_off + a16((long long)vt_bytes * m));
    ch.img_bytes = (int)a16(ch.ent_off + (long long)ent_bytes * ne);
    ch.img_off = img_off;
    ch.b_off = b_off;
    ch.b_bytes = (int)a16((long long)vt_bytes * m);
    img_off += ch.img_bytes;
    b_off += (int)(((m + b_align - 1) / b_align) * b_align);
    for (int r = 0; r < m; r++) chunk_of[p + r] = (int)w.chunks.size();
    w.chunks.push_back(ch);
    p += m;
  }
  w.img_bytes = img_off;
  w.blev_len = b_off + 16;
  w.order = order;
  w.bidx.resize(n);
  std::vector<unsigned char> img((size_t)img_off, 0);
  for (size_t c = 0; c < w.chunks.size(); c++) {
    const WaveChunk& ch = w.chunks[c];
    int e = 0;
    for (int r = 0; r < ch.nrows; r++) {
      const int pp = ch.pos0 + r;
      const int i = order[pp];
      w.bidx[pp] = ch.b_off + r;
      const int k = ptr[i + 1] - ptr[i];
      int4 mt = make_int4(i, e, k, 0);
      std::memcpy(&img[(size_t)ch.img_off + 16 * (size_t)r], &mt, 16);
      if (!lower) {
        w.diag_dst.push_back(ch.img_off + ch.diag_off + (long long)vt_bytes * r);
        w.diag_src.push_back(diag_pos[i]);
      }
      // end position of this chunk: everything up to it has been written
      const int chunk_end = ch.pos0 + ch.nrows;
      for (int q = ptr[i]; q < ptr[i + 1]; q++, e++) {
        const int j = dep[q];
        const int pj = pos[j];
        int src = (chunk_end - 1 - pj < ring) ? (pj % ring) : -(j + 1);
        const long long off = ch.img_off + ch.ent_off + (long long)ent_bytes * e;
        std::memcpy(&img[(size_t)off + vt_bytes], &src, 4);
        w.ent_dst.push_back(off);
        w.ent_src.push_back(src_pos[q]);
        if (src < 0) w.ring_misses++;
      }
    }
  }
  w.img_host.swap(img);
  return w;
}


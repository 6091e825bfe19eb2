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
                             int vt_bytes, int ring, int pin, int stage_cap, int bstage_cap) {
  WaveLayout w;
  w.n = n;
  // dependency levels, rows of a level in solve order
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
    const int i = lower ? t : n - 1 - t;
    const int p = fill[lev[i]]++;
    order[p] = i;
    pos[i] = p;
  }
  auto a16 = [](long long v) { return (v + 15) & ~15ll; };
  // chunk image: meta[m] (int4) | diag[m] (VT) | vals[ne] (VT) | srcs[ne] (int), each part 16-aligned
  auto img_size = [&](long long m, long long ne) {
    return a16(16 * m) + a16(vt_bytes * m) + a16(vt_bytes * ne) + a16(4 * ne);
  };
  std::vector<int> chunk_end(n);
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
      if (m > 0 && (img_size(m + 1, ne + k) > stage_cap || a16((long long)vt_bytes * (m + 1)) > bstage_cap ||
                    m + 1 > 4096))
        break;
      m++;
      ne += k;
    }
    ch.nrows = m;
    ch.nent = ne;
    ch.diag_off = (int)a16(16ll * m);
    ch.val_off = (int)(ch.diag_off + a16((long long)vt_bytes * m));
    ch.src_off = (int)(ch.val_off + a16((long long)vt_bytes * ne));
    ch.img_bytes = (int)img_size(m, ne);
    ch.img_off = img_off;
    ch.b_off = b_off;
    ch.b_bytes = (int)a16((long long)vt_bytes * m);
    img_off += ch.img_bytes;
    b_off += ((m + b_align - 1) / b_align) * b_align;
    for (int r = 0; r < m; r++) chunk_end[p + r] = p + m;
    w.chunks.push_back(ch);
    p += m;
  }
  // sources outside the ring: pin the most-read ones in a fixed shared-memory table
  std::vector<int> far_reads(n, 0);
  for (int i = 0; i < n; i++)
    for (int q = ptr[i]; q < ptr[i + 1]; q++) {
      const int j = dep[q];
      if (chunk_end[pos[i]] - 1 - pos[j] >= ring) far_reads[j]++;
    }
  std::vector<int> cand;
  for (int j = 0; j < n; j++)
    if (far_reads[j]) cand.push_back(j);
  std::stable_sort(cand.begin(), cand.end(), [&](int a, int b) { return far_reads[a] > far_reads[b]; });
  std::vector<int> pin_slot(n, -1);
  for (size_t k = 0; k < cand.size() && (int)k < pin; k++) pin_slot[cand[k]] = (int)k;
  w.pinned = (int)std::min<size_t>(cand.size(), (size_t)pin);
  w.img_bytes = img_off;
  w.blev_len = b_off + 16;
  w.order = order;
  w.bidx.resize(n);
  std::vector<unsigned char> img((size_t)img_off, 0);
  for (const WaveChunk& ch : w.chunks) {
    int e = 0;
    for (int r = 0; r < ch.nrows; r++) {
      const int pp = ch.pos0 + r;
      const int i = order[pp];
      w.bidx[pp] = ch.b_off + r;
      const int k = ptr[i + 1] - ptr[i];
      int mt[4] = {i, e, k, pin_slot[i] >= 0 ? ring + pin_slot[i] : -1};
      std::memcpy(&img[(size_t)ch.img_off + 16 * (size_t)r], mt, 16);
      if (!lower) {
        w.diag_dst.push_back(ch.img_off + ch.diag_off + (long long)vt_bytes * r);
        w.diag_src.push_back(diag_pos[i]);
      }
      const int cend = ch.pos0 + ch.nrows;
      for (int q = ptr[i]; q < ptr[i + 1]; q++, e++) {
        const int j = dep[q];
        const int pj = pos[j];
        int src;
        if (cend - 1 - pj < ring)
          src = pj % ring;
        else if (pin_slot[j] >= 0)
          src = ring + pin_slot[j];
        else
          src = -(j + 1);
        std::memcpy(&img[(size_t)(ch.img_off + ch.src_off) + 4 * (size_t)e], &src, 4);
        w.ent_dst.push_back(ch.img_off + ch.val_off + (long long)vt_bytes * e);
        w.ent_src.push_back(src_pos[q]);
        if (src < 0) w.ring_misses++;
      }
    }
  }
  w.img_host.swap(img);
  return w;
}

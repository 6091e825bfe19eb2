// Host-side layout of the wavefront triangular solves (rg_trsv.cu): level
// schedule of a triangular factor, split into stage-sized chunks, packed into
// one device image, with the shared-memory ring slot of every dependency.

#include "rg_internal.cuh"

#include <algorithm>
#include <cstring>
#include <numeric>

// Build the level-ordered chunk layout of one triangular factor.  `dep` lists,
// per row, the rows it reads (L: columns < row, U: columns > row) in the
// factor's row order; `src_pos` the factor positions of those entries;
// diag_pos the diagonal positions.
//
// Rows of one level do not depend on each other.  Inside a level they are
// ordered by entry count, longest first, so that the rows of a warp slice
// have similar lengths.  `lanes` threads share a row (a warp slice holds
// 32 / lanes rows): lane g of a row takes its entries g, g + lanes, ...; with
// one lane per row the entries are summed in the factor's order, which is the
// order of PRECO_ILU0::Solve (Preco_ilu0.cpp:517-530, 964-980).
//
// split = true: an entry whose source is neither in the ring nor pinned leaves
// the image for the far lists of its row (far_ptr/far_src/far_vsrc, by
// level-order position); each chunk records the last chunk holding one of its
// far sources (far_dep).  Otherwise such an entry reads its source from global
// memory (slot code -(row + 1)).
WaveLayout build_wave_layout(int n, const std::vector<int>& ptr, const std::vector<int>& dep,
                             const std::vector<int>& src_pos, const std::vector<int>& diag_pos, bool lower,
                             int vt_bytes, int ring, int pin, int stage_cap, int rows_max, int lanes, bool split) {
  WaveLayout w;
  w.n = n;
  const int rps = kWaveSlice / lanes;   // rows per warp slice
  // split layouts store 16-bit source slots: the ring and the pinned table must fit them
  split = split && ring + pin <= 65536;
  // all rows of a chunk write their ring slots at once: they must be distinct
  rows_max = std::min(rows_max, ring);
  // dependency levels
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
  // level order: by level, inside a level by entry count (descending), then solve order
  std::vector<int> order(n), pos(n), fill(cnt.begin(), cnt.end() - 1);
  for (int t = 0; t < n; t++) {
    const int i = lower ? t : n - 1 - t;
    order[fill[lev[i]]++] = i;
  }
  auto kof = [&](int i) { return ptr[i + 1] - ptr[i]; };
  for (int l = 0; l < nlev; l++)
    std::stable_sort(order.begin() + cnt[l], order.begin() + cnt[l + 1],
                     [&](int a, int b) { return kof(a) > kof(b); });
  for (int p = 0; p < n; p++) pos[order[p]] = p;

  auto a16 = [](long long v) { return (v + 15) & ~15ll; };
  // source slots: 16-bit in split layouts (every source is a ring or pinned slot, < 65536),
  // 32-bit otherwise (negative codes for sources read from global memory)
  const int sb = split ? 2 : 4;
  const long long stride = kWaveSlice * ((long long)sb + vt_bytes);   // bytes per entry column of a slice
  // chunk image: meta[m] (int4) | b[m] (VT) | diag[m] (VT, U only) | slices, each part 16-aligned
  auto head_bytes = [&](long long m) { return a16(16 * m) + a16(vt_bytes * m) + (lower ? 0 : a16(vt_bytes * m)); };
  // a source is read from the ring when it lies less than ring - rows_max positions
  // before the reading row (then it is less than ring positions before the end of the
  // reader's chunk, so its slot has not been reused)
  const int reach = ring - rows_max;
  auto in_ring = [&](int reader_pos, int j) { return reader_pos - pos[j] < reach; };
  // sources outside the ring: pin the most-read ones in a fixed shared-memory table
  std::vector<int> far_reads(n, 0);
  for (int i = 0; i < n; i++)
    for (int q = ptr[i]; q < ptr[i + 1]; q++) {
      const int j = dep[q];
      if (!in_ring(pos[i], j)) far_reads[j]++;
    }
  std::vector<int> cand;
  for (int j = 0; j < n; j++)
    if (far_reads[j]) cand.push_back(j);
  std::stable_sort(cand.begin(), cand.end(), [&](int a, int b) { return far_reads[a] > far_reads[b]; });
  std::vector<int> pin_slot(n, -1);
  for (size_t k = 0; k < cand.size() && (int)k < pin; k++) pin_slot[cand[k]] = (int)k;
  w.pinned = (int)std::min<size_t>(cand.size(), (size_t)pin);
  auto is_near = [&](int reader_pos, int j) { return in_ring(reader_pos, j) || pin_slot[j] >= 0; };
  // entries a row keeps in the image: all of them, or (split) its near ones
  std::vector<int> kimg(n);
  for (int i = 0; i < n; i++) {
    if (!split) {
      kimg[i] = kof(i);
      continue;
    }
    int k = 0;
    for (int q = ptr[i]; q < ptr[i + 1]; q++) k += is_near(pos[i], dep[q]);
    kimg[i] = k;
  }
  // a slice's width: the widest row of its (up to rps) rows, counted to the end of the level
  auto slice_width = [&](int p0, int lend) {
    int wmax = 0;
    for (int t = p0; t < std::min(p0 + rps, lend); t++) wmax = std::max(wmax, (kimg[order[t]] + lanes - 1) / lanes);
    return wmax;
  };
  std::vector<int> chunk_end(n), chunk_of(n);
  int p = 0;
  long long img_off = 0;
  while (p < n) {
    const int l = lev[order[p]];
    const int lend = cnt[l + 1];
    WaveChunk ch{};
    ch.pos0 = p;
    ch.far_dep = -1;
    int m = 0;
    long long ebytes = 0;
    while (p + m < lend && m < rows_max) {
      // a new slice starts every rps rows
      const long long add = (m % rps == 0) ? (long long)slice_width(p + m, lend) * stride : 0;
      if (m > 0 && head_bytes(m + 1) + ebytes + add > stage_cap) break;
      ebytes += add;
      m++;
    }
    ch.nrows = m;
    ch.b_off = (int)a16(16ll * m);
    ch.diag_off = (int)(ch.b_off + a16((long long)vt_bytes * m));
    ch.img_bytes = (int)(head_bytes(m) + ebytes);
    ch.img_off = img_off;
    img_off += ch.img_bytes;
    for (int r = 0; r < m; r++) {
      chunk_end[p + r] = p + m;
      chunk_of[p + r] = (int)w.chunks.size();
    }
    w.chunks.push_back(ch);
    p += m;
  }
  w.img_bytes = img_off;
  w.order = order;
  w.bidx.resize(n);
  std::vector<unsigned char> img((size_t)img_off, 0);
  if (split) w.far_ptr.assign(1, 0);
  for (WaveChunk& ch : w.chunks) {
    const int lend = cnt[lev[order[ch.pos0]] + 1];
    long long sbase = head_bytes(ch.nrows);   // byte offset of the current slice in the chunk
    int width = 0;
    for (int r = 0; r < ch.nrows; r++) {
      const int pp = ch.pos0 + r;
      const int i = order[pp];
      const int rs = r % rps;   // row inside its slice
      if (rs == 0) {
        if (r > 0) sbase += (long long)width * stride;
        width = slice_width(pp, lend);
      }
      w.bidx[pp] = (int)((ch.img_off + ch.b_off) / vt_bytes + r);
      int mt[4] = {i, kimg[i], (int)sbase, pin_slot[i] >= 0 ? ring + pin_slot[i] : -1};
      std::memcpy(&img[(size_t)ch.img_off + 16 * (size_t)r], mt, 16);
      if (!lower) {
        w.diag_dst.push_back(ch.img_off + ch.diag_off + (long long)vt_bytes * r);
        w.diag_src.push_back(diag_pos[i]);
      }
      int e = 0;   // entry index inside the image
      for (int q = ptr[i]; q < ptr[i + 1]; q++) {
        const int j = dep[q];
        const int pj = pos[j];
        int src;
        if (in_ring(pp, j)) {
          src = pj % ring;
        } else if (pin_slot[j] >= 0) {
          src = ring + pin_slot[j];
        } else {
          w.ring_misses++;
          if (split) {
            w.far_src.push_back(j);
            w.far_vsrc.push_back(src_pos[q]);
            ch.far_dep = std::max(ch.far_dep, chunk_of[pj]);
            continue;
          }
          src = -(j + 1);
        }
        const int lane = rs * lanes + e % lanes;
        const long long col = ch.img_off + sbase + (long long)(e / lanes) * stride;
        if (sb == 2) {
          const unsigned short s16 = (unsigned short)src;   // 0 <= src < ring + pin <= 65535 (checked by the caller)
          std::memcpy(&img[(size_t)(col + 2ll * lane)], &s16, 2);
        } else {
          std::memcpy(&img[(size_t)(col + 4ll * lane)], &src, 4);
        }
        w.ent_dst.push_back(col + (long long)sb * kWaveSlice + (long long)vt_bytes * lane);
        w.ent_src.push_back(src_pos[q]);
        e++;
      }
      if (split) w.far_ptr.push_back((long long)w.far_src.size());
    }
  }
  w.img_host.swap(img);
  return w;
}

// Host-side setup algorithms: DOF compaction, the reference's blocked
// symmetric pattern, the element->value map, element colouring and the
// device full-BSR structure.  Setup only; nothing here runs per step.
#include <algorithm>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <thread>

#include "od_internal.h"

namespace od {

// NodeIndexer::getGlobalIndex (core/nodeIndexer.cpp:12-25)
int global_index(const std::vector<int>& cd, int node, int axis) {
  int idx = 3 * node + axis;
  if (cd.empty()) return idx;
  int off = (int)(std::lower_bound(cd.begin(), cd.end(), idx) - cd.begin());
  if (off < (int)cd.size() && cd[off] == idx) return -1;
  return idx - off;
}

static void parallel_for(int n, int min_chunk, const std::function<void(int, int)>& fn) {
  unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  int nt = (int)std::min<long long>(hw, std::max(1, n / std::max(1, min_chunk)));
  if (nt <= 1) { fn(0, n); return; }
  std::vector<std::thread> th;
  int chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; t++) {
    int b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back(fn, b, e);
  }
  for (auto& x : th) x.join();
}

// Pattern of BlockedSymSparseMatrix built from getMatrixStructure
// (core/sparseMatrix.h:90-274, material/fullOrderNonlinear.h:46-71).  In
// compacted-DOF space every block starts at a multiple of 3, so a stored
// block of block column bc is identified by its block row br = r / 3; the
// diagonal block packs 6 values, the others 3 * min(3, n - 3 br); the
// n % 3 trailing columns are scalar columns.
void build_pattern(const std::vector<int>& gidx, int n_tets, int n, std::vector<int>& pcol,
                   std::vector<int>& rows, std::vector<int>& oris, int& nbc, int& nrem, int& nvals) {
  nbc = n / 3;
  nrem = n - 3 * nbc;
  const int tail = 3 * nbc;
  // block pairs (br, bc) as 64-bit keys, built per thread then merged
  unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  int nt = std::max(1, std::min<int>((int)hw, n_tets / 20000 + 1));
  std::vector<std::vector<uint64_t>> parts(nt);
  std::vector<std::vector<uint64_t>> tails(nt);
  int chunk = (n_tets + nt - 1) / nt;
  std::vector<std::thread> th;
  for (int t = 0; t < nt; t++) {
    th.emplace_back([&, t]() {
      int b = t * chunk, e = std::min(n_tets, b + chunk);
      auto& out = parts[t];
      auto& tl = tails[t];
      out.reserve((size_t)std::max(0, e - b) * 10);
      for (int el = b; el < e; el++) {
        const int* g = &gidx[12 * (size_t)el];
        int blk[12], nbk = 0;
        for (int k = 0; k < 12; k++) {
          if (g[k] < 0) continue;
          int bb = g[k] / 3;
          bool seen = false;
          for (int q = 0; q < nbk; q++) if (blk[q] == bb) { seen = true; break; }
          if (!seen) blk[nbk++] = bb;
        }
        for (int i = 0; i < nbk; i++)
          for (int j = 0; j < nbk; j++)
            if (blk[i] >= blk[j] && blk[j] < nbc) out.push_back(((uint64_t)blk[j] << 32) | (uint32_t)blk[i]);
        if (nrem > 0) {
          for (int x = 0; x < 12; x++) {
            if (g[x] < 0) continue;
            for (int y = 0; y < 12; y++) {
              if (g[y] < 0) continue;
              int r = std::max(g[x], g[y]), c = std::min(g[x], g[y]);
              if (c >= tail) tl.push_back(((uint64_t)c << 32) | (uint32_t)r);
            }
          }
        }
      }
      std::sort(out.begin(), out.end());
      out.erase(std::unique(out.begin(), out.end()), out.end());
      std::sort(tl.begin(), tl.end());
      tl.erase(std::unique(tl.begin(), tl.end()), tl.end());
    });
  }
  for (auto& x : th) x.join();
  std::vector<uint64_t> keys;
  {
    size_t tot = 0;
    for (auto& p : parts) tot += p.size();
    keys.reserve(tot);
    for (auto& p : parts) { keys.insert(keys.end(), p.begin(), p.end()); std::vector<uint64_t>().swap(p); }
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  }
  std::vector<uint64_t> tkeys;
  for (auto& p : tails) tkeys.insert(tkeys.end(), p.begin(), p.end());
  std::sort(tkeys.begin(), tkeys.end());
  tkeys.erase(std::unique(tkeys.begin(), tkeys.end()), tkeys.end());

  pcol.assign(nbc + nrem + 1, 0);
  oris.assign(nbc + nrem + 1, 0);
  rows.clear();
  rows.reserve(keys.size() + tkeys.size());
  long long nv = 0;
  size_t k = 0;
  for (int bc = 0; bc < nbc; bc++) {
    while (k < keys.size() && (int)(keys[k] >> 32) == bc) {
      int br = (int)(keys[k] & 0xffffffffu);
      int r0 = 3 * br;
      rows.push_back(r0);
      nv += (br == bc) ? 6 : 3 * std::min(3, n - r0);
      k++;
    }
    pcol[bc + 1] = (int)rows.size();
    oris[bc + 1] = (int)nv;
  }
  size_t q = 0;
  for (int c = 0; c < nrem; c++) {
    while (q < tkeys.size() && (int)(tkeys[q] >> 32) == tail + c) {
      rows.push_back((int)(tkeys[q] & 0xffffffffu));
      nv += 1;
      q++;
    }
    pcol[nbc + c + 1] = (int)rows.size();
    oris[nbc + c + 1] = (int)nv;
  }
  if (nv > 0x7fffffffLL) throw std::runtime_error("value count exceeds int32");
  nvals = (int)nv;
}

// value index of the lower entry (r >= c): BlockedSymSparseMatrix::getIndices
// (core/sparseMatrix.h:528-579)
static inline int value_index(int n, int nbc, const std::vector<int>& pcol, const std::vector<int>& rows,
                              const std::vector<int>& oris, int r, int c) {
  if (c / 3 < nbc) {
    int bc = c / 3, sc = c - 3 * bc, br = 3 * (r / 3);
    const int* b = rows.data() + pcol[bc];
    const int* e = rows.data() + pcol[bc + 1];
    const int* p = std::lower_bound(b, e, br);
    if (p == e || *p != br) return -1;
    int k = (int)(p - b), off = oris[bc];
    if (br == 3 * bc) {
      static const int di[3] = {0, 3, 5};
      return off + (r - br) - sc + di[sc];
    }
    bool hasDiag = rows[pcol[bc]] == 3 * bc;
    off += hasDiag ? 6 + 9 * (k - 1) : 9 * k;
    return off + sc * std::min(3, n - br) + (r - br);
  }
  int col = c - 3 * nbc + nbc;
  const int* b = rows.data() + pcol[col];
  const int* e = rows.data() + pcol[col + 1];
  const int* p = std::lower_bound(b, e, r);
  if (p == e || *p != r) return -1;
  return oris[col] + (int)(p - b);
}

// element -> value map (material/fullOrderNonlinear.h:73-110): packed local
// index (Element::getLocalMatrixIndex, core/element.h:109-118) -> value index
void build_emap(const std::vector<int>& gidx, int n_tets, int n, int nbc, const std::vector<int>& pcol,
                const std::vector<int>& rows, const std::vector<int>& oris, std::vector<int>& emap) {
  emap.assign((size_t)78 * n_tets, -1);
  parallel_for(n_tets, 4096, [&](int b, int e) {
    for (int el = b; el < e; el++) {
      const int* g = &gidx[12 * (size_t)el];
      int* m = &emap[78 * (size_t)el];
      int k = 0;
      for (int a = 0; a < 12; a++)
        for (int bb = a; bb < 12; bb++, k++) {
          if (g[a] < 0 || g[bb] < 0) continue;
          m[k] = value_index(n, nbc, pcol, rows, oris, std::max(g[a], g[bb]), std::min(g[a], g[bb]));
        }
    }
  });
}

// Greedy element colouring on shared nodes: two elements of one colour share
// no node, hence no compacted DOF, no matrix value and no force entry, so a
// colour can scatter without atomics.  Returns the colour count.
int color_elements(const std::vector<int>& nodes, int per_elem, int n_elem, int n_nodes,
                   std::vector<int>& perm, std::vector<int>& color_off) {
  const int W = 4;  // 4 x 64 = 256 colours
  std::vector<uint64_t> used((size_t)n_nodes * W, 0);
  std::vector<int> color(n_elem);
  int ncol = 0;
  for (int e = 0; e < n_elem; e++) {
    uint64_t m[W] = {0, 0, 0, 0};
    for (int k = 0; k < per_elem; k++) {
      const uint64_t* u = &used[(size_t)nodes[(size_t)per_elem * e + k] * W];
      for (int w = 0; w < W; w++) m[w] |= u[w];
    }
    int c = -1;
    for (int w = 0; w < W && c < 0; w++)
      if (~m[w]) c = 64 * w + __builtin_ctzll(~m[w]);
    if (c < 0) throw std::runtime_error("element colouring needs more than 256 colours");
    color[e] = c;
    ncol = std::max(ncol, c + 1);
    for (int k = 0; k < per_elem; k++) used[(size_t)nodes[(size_t)per_elem * e + k] * W + c / 64] |= (1ull << (c % 64));
  }
  color_off.assign(ncol + 1, 0);
  for (int e = 0; e < n_elem; e++) color_off[color[e] + 1]++;
  for (int c = 0; c < ncol; c++) color_off[c + 1] += color_off[c];
  perm.resize(n_elem);
  std::vector<int> pos(color_off.begin(), color_off.end() - 1);
  for (int e = 0; e < n_elem; e++) perm[pos[color[e]]++] = e;
  return ncol;
}

// Full BSR over padded 3-DOF blocks (both triangles) with, for every block,
// the location of its values in the reference lower layout.
void build_full_bsr(int n, int nbc, int nrem, const std::vector<int>& pcol, const std::vector<int>& rows,
                    const std::vector<int>& oris, HostBsr& out) {
  const int nb = nbc + (nrem > 0 ? 1 : 0);
  out.nb = nb;
  struct Ent { int col, off, kind; };
  std::vector<std::vector<Ent>> rowv(nb);
  std::vector<int> gen;
  // block columns
  for (int bc = 0; bc < nbc; bc++) {
    int off = oris[bc];
    for (int k = pcol[bc]; k < pcol[bc + 1]; k++) {
      int r0 = rows[k], br = r0 / 3;
      if (br == bc) {
        rowv[bc].push_back({bc, off, BK_DIAG});
        off += 6;
      } else {
        int w = std::min(3, n - r0);
        if (w == 3) {
          rowv[br].push_back({bc, off, BK_LOWER});
          rowv[bc].push_back({br, off, BK_UPPER});
        } else {
          int gi = (int)gen.size() / 9;
          for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) gen.push_back(r < w ? off + c * w + r : -1);
          rowv[br].push_back({bc, gi, BK_GENERAL});
          gi = (int)gen.size() / 9;
          for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) gen.push_back(c < w ? off + r * w + c : -1);
          rowv[bc].push_back({br, gi, BK_GENERAL});
        }
        off += 3 * w;
      }
    }
  }
  if (nrem > 0) {
    // scalar tail columns all fall into the last (padded) diagonal block
    int tbl[9];
    for (int i = 0; i < 9; i++) tbl[i] = -1;
    for (int r = nrem; r < 3; r++) tbl[r * 3 + r] = -2;  // padding DOFs: identity
    const int t0 = 3 * nbc;
    for (int c = 0; c < nrem; c++) {
      int col = nbc + c, off = oris[col];
      for (int q = pcol[col]; q < pcol[col + 1]; q++, off++) {
        int r = rows[q] - t0;
        tbl[r * 3 + c] = off;
        tbl[c * 3 + r] = off;
      }
    }
    int gi = (int)gen.size() / 9;
    for (int i = 0; i < 9; i++) gen.push_back(tbl[i]);
    rowv[nbc].push_back({nbc, gi, BK_GENERAL});
  }
  out.row_ptr.assign(nb + 1, 0);
  out.col.clear(); out.desc_off.clear(); out.desc_kind.clear();
  out.diag_pos.assign(nb, -1);
  for (int br = 0; br < nb; br++) {
    auto& v = rowv[br];
    std::sort(v.begin(), v.end(), [](const Ent& a, const Ent& b) { return a.col < b.col; });
    for (auto& e : v) {
      if (e.col == br) out.diag_pos[br] = (int)out.col.size();
      out.col.push_back(e.col);
      out.desc_off.push_back(e.off);
      out.desc_kind.push_back(e.kind);
    }
    out.row_ptr[br + 1] = (int)out.col.size();
  }
  out.gen.swap(gen);
}

// Level sets of a lower-triangular scalar CSR: forward level(i) = 1 + max
// level(j) over stored j < i; backward uses the transposed dependencies.
void build_ic_levels(const std::vector<int>& rp, const std::vector<int>& ci, int n,
                     std::vector<int>& rows_by_level, std::vector<int>& lvl_ptr, bool forward) {
  std::vector<int> lvl(n, 0);
  int maxl = 0;
  if (forward) {
    for (int i = 0; i < n; i++) {
      int l = 0;
      for (int q = rp[i]; q < rp[i + 1]; q++)
        if (ci[q] < i) l = std::max(l, lvl[ci[q]] + 1);
      lvl[i] = l;
      maxl = std::max(maxl, l);
    }
  } else {
    // row i of L^T depends on rows j > i with L_ji stored (row j, column i)
    std::vector<int> best(n, 0);
    for (int j = n - 1; j >= 0; j--) {
      lvl[j] = best[j];
      maxl = std::max(maxl, lvl[j]);
      for (int q = rp[j]; q < rp[j + 1]; q++) {
        int i = ci[q];
        if (i < j) best[i] = std::max(best[i], lvl[j] + 1);
      }
    }
  }
  lvl_ptr.assign(maxl + 2, 0);
  for (int i = 0; i < n; i++) lvl_ptr[lvl[i] + 1]++;
  for (int l = 0; l <= maxl; l++) lvl_ptr[l + 1] += lvl_ptr[l];
  rows_by_level.resize(n);
  std::vector<int> pos(lvl_ptr.begin(), lvl_ptr.end() - 1);
  for (int i = 0; i < n; i++) rows_by_level[pos[lvl[i]]++] = i;
}

// Slice structure of the FP32 inner-solve matrix (SELL-C-sigma with C =
// kSliceRows, sigma = kSliceWindow): block rows are ordered by block count,
// longest first, within each window (stable, so equal rows keep mesh order),
// cut into slices, and every slice is padded to its longest row rounded up
// to an even step count (so every slice starts on a 16-byte boundary of the
// value and column arrays, as bulk copies require).  Padding slots point at
// the slot's own slice row and take the value zero.
// lower = true keeps the blocks of the lower triangle only (block column <=
// block row, the reference's symmetric storage): src of a diagonal block is
// -(block + 2), its values go in halved (the SpMV applies every stored block
// and its transpose), padding -1.
void build_sliced(const std::vector<int>& row_ptr, const std::vector<int>& col, int nb, HostSliced& out,
                  bool lower) {
  const int S = kSliceRows;
  const int ns = (nb + S - 1) / S;
  out.ns = ns;
  out.lower = lower;
  std::vector<int> order(nb);
  for (int i = 0; i < nb; i++) order[i] = i;
  // a row's stored blocks: all, or those up to the diagonal (columns ascend)
  std::vector<int> rlen(nb);
  for (int r = 0; r < nb; r++) {
    int m = 0;
    for (int k = row_ptr[r]; k < row_ptr[r + 1]; k++)
      if (!lower || col[k] <= r) m++;
    rlen[r] = m;
  }
  auto len = [&](int r) { return rlen[r]; };
  for (int w0 = 0; w0 < nb; w0 += kSliceWindow) {
    const int w1 = std::min(nb, w0 + kSliceWindow);
    std::stable_sort(order.begin() + w0, order.begin() + w1, [&](int a, int b) { return len(a) > len(b); });
  }
  std::vector<int> inv(nb);
  out.perm.assign((size_t)ns * S, -1);
  for (int i = 0; i < nb; i++) {
    out.perm[i] = order[i];
    inv[order[i]] = i;
  }
  out.off.assign(ns + 1, 0);
  for (int sl = 0; sl < ns; sl++) {
    int m = 0;
    for (int t = 0; t < S; t++) {
      const int r = out.perm[(size_t)sl * S + t];
      if (r >= 0) m = std::max(m, len(r));
    }
    out.off[sl + 1] = out.off[sl] + m + (m & 1);
  }
  const size_t steps = (size_t)out.off[ns];
  out.col.assign(steps * S, 0);
  out.src.assign(steps * S, -1);
  for (int sl = 0; sl < ns; sl++) {
    for (int t = 0; t < S; t++) {
      const int rs = sl * S + t;
      const int r = out.perm[rs];
      const int k0 = out.off[sl], k1 = out.off[sl + 1];
      int m = 0;
      if (r >= 0) {
        m = len(r);
        int j = 0;
        for (int k = row_ptr[r]; k < row_ptr[r + 1]; k++) {
          if (lower && col[k] > r) continue;
          out.col[(size_t)(k0 + j) * S + t] = inv[col[k]];
          out.src[(size_t)(k0 + j) * S + t] = (lower && col[k] == r) ? -(k + 2) : k;
          j++;
        }
      }
      for (int k = k0 + m; k < k1; k++) out.col[(size_t)k * S + t] = rs;
    }
  }
}

}  // namespace od

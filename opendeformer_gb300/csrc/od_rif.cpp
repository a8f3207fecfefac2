// Incomplete LDL^T factor of the reference's InLDLTPreconditioner
// (solver/inLDLTPreconditioner.cpp:34-149): a robust incomplete
// factorisation run as a stabilised approximate-inverse (SAINV) sweep.
//
//   Z = I (columns z_j = e_j); for i = 0 .. n-1:
//     v   = A z_i,  d_i = z_i . v
//     p_j = v . z_j for every j > i that shares a row with v
//     L_ji = p_j / d_i             kept when |L_ji| >  ldlt_eps
//     z_j -= (p_j / d_i) z_i       entries kept when |.| > sainv_eps
//
// The sweep is strictly sequential in i and its fill is data-dependent, so
// it runs on the host; the device takes the per-iteration part (the two
// triangular sweeps of the apply).  Every accumulation below is made in the
// order the reference makes it (first-touch order of the sparse
// accumulators, newest-first walk of the per-row lists of Z entries), which
// makes the factor bit-identical to the reference's for the same matrix
// values.  Built with -ffp-contract=off so x86-64 and aarch64 agree.
#include <cmath>
#include <vector>

#include "od_internal.h"

namespace od {

// Scalar columns of the symmetric matrix held in the reference's lower
// block layout, both triangles, in the order of
// BlockedSymSparseMatrix::getFullIndices (core/sparseMatrix.h:454-523):
// column c lists (row, value index) pairs.
void rif_columns(int n, int nbc, const std::vector<int>& pcol, const std::vector<int>& rows, RifColumns& out) {
  out.n = n;
  out.ptr.assign(n + 1, 0);
  // pass 0 counts, pass 1 fills (same traversal both times)
  std::vector<int> fill;
  for (int pass = 0; pass < 2; pass++) {
    auto emit = [&](int col, int row, int idx) {
      if (pass == 0) {
        out.ptr[col + 1]++;
      } else {
        const int at = fill[col]++;
        out.row[at] = row;
        out.src[at] = idx;
      }
    };
    int idx = 0;
    for (int bc = 0; bc < nbc; bc++) {
      const int c0 = 3 * bc;
      int k = pcol[bc];
      const int e = pcol[bc + 1];
      if (k == e) continue;
      if (rows[k] == c0) {  // diagonal block: packed upper triangle of 6
        for (int a = 0; a < 3; a++) {
          emit(c0 + a, c0 + a, idx++);
          for (int b = a + 1; b < 3; b++) {
            emit(c0 + a, c0 + b, idx);
            emit(c0 + b, c0 + a, idx);
            idx++;
          }
        }
        k++;
      }
      for (; k < e; k++) {
        const int r0 = rows[k];
        const int width = k == e - 1 ? std::min(3, n - r0) : 3;
        for (int a = 0; a < 3; a++)
          for (int b = 0; b < width; b++) {
            emit(c0 + a, r0 + b, idx);
            emit(r0 + b, c0 + a, idx);
            idx++;
          }
      }
    }
    for (int c = 3 * nbc; c < n; c++) {  // scalar tail columns
      const int pc = nbc + (c - 3 * nbc);
      int k = pcol[pc];
      const int e = pcol[pc + 1];
      if (k == e) continue;
      if (rows[k] == c) { emit(c, c, idx++); k++; }
      for (; k < e; k++) {
        emit(c, rows[k], idx);
        emit(rows[k], c, idx);
        idx++;
      }
    }
    if (pass == 0) {
      for (int c = 0; c < n; c++) out.ptr[c + 1] += out.ptr[c];
      out.row.assign(out.ptr[n], 0);
      out.src.assign(out.ptr[n], 0);
      fill.assign(out.ptr.begin(), out.ptr.end() - 1);
    }
  }
}

namespace {

// sparse accumulator: entries in first-touch order, dense position index
struct Spa {
  std::vector<int> where;  // position + 1, 0 when absent
  std::vector<int> idx;
  std::vector<double> val;
  explicit Spa(int n) : where(n, 0) {}
  void add(int i, double x) {
    const int w = where[i];
    if (w) {
      val[w - 1] += x;
    } else {
      push(i, x);
    }
  }
  void push(int i, double x) {
    idx.push_back(i);
    val.push_back(x);
    where[i] = (int)idx.size();
  }
  double get(int i) const {
    const int w = where[i];
    return w ? val[w - 1] : 0.0;
  }
  void clear() {
    for (int i : idx) where[i] = 0;
    idx.clear();
    val.clear();
  }
};

// Entries of Z: each lives in its column's list (insertion order) and in
// its row's doubly linked list (newest first).  One 24-byte record per
// entry, so a row walk touches one cache line per entry.  Ids 0..n-1 are
// the row heads; freed ids are reused.
struct ZEntry {
  int next, prev, row, col;
  double val;
};

struct ZStore {
  std::vector<ZEntry> e;
  std::vector<int> free_ids;
  explicit ZStore(int n) {
    e.reserve((size_t)n * 8);
    for (int r = 0; r < n; r++) e.push_back({r, r, r, -1, 0.0});
  }
  int insert(int r, int c, double x) {
    int id;
    if (!free_ids.empty()) {
      id = free_ids.back();
      free_ids.pop_back();
    } else {
      id = (int)e.size();
      e.push_back({});
    }
    // right after the head: the row walk meets the newest entry first
    const int first = e[r].next;
    e[id] = {first, r, r, c, x};
    e[first].prev = id;
    e[r].next = id;
    return id;
  }
  void remove(int id) {
    const ZEntry& x = e[id];
    e[x.prev].next = x.next;
    e[x.next].prev = x.prev;
    free_ids.push_back(id);
  }
};

}  // namespace

void rif_factor(const RifColumns& A, const double* a, double sainv_eps, double ldlt_eps, RifFactor& F) {
  const int n = A.n;
  F.n = n;
  F.val.clear();
  F.row.clear();
  F.pcol.clear();
  F.dinv.assign(n, 0.0);
  if (n == 0) return;
  F.pcol.push_back(0);
  ZStore z(n);
  std::vector<std::vector<int>> colz(n);
  for (int i = 0; i < n; i++) colz[i].push_back(z.insert(i, i, 1.0));
  Spa v(n), low(n);
  std::vector<int> zi_idx;
  std::vector<double> zi_val;

  auto take_column = [&](int i) {
    zi_idx.clear();
    zi_val.clear();
    for (int id : colz[i]) {
      zi_idx.push_back(z.e[id].row);
      zi_val.push_back(z.e[id].val);
      z.remove(id);
    }
    std::vector<int>().swap(colz[i]);
  };
  // v = A z_i (SpMSV, core/numerMethod.h:283-299) and d_i = z_i . v
  auto times_a = [&]() -> double {
    for (size_t k = 0; k < zi_idx.size(); k++) {
      const int c = zi_idx[k];
      const double zc = zi_val[k];
      for (int q = A.ptr[c]; q < A.ptr[c + 1]; q++) v.add(A.row[q], a[A.src[q]] * zc);
    }
    double d = 0.0;
    for (size_t k = 0; k < zi_idx.size(); k++) d += zi_val[k] * v.get(zi_idx[k]);
    return d;
  };

  for (int i = 0; i < n - 1; i++) {
    take_column(i);
    const double inv = 1.0 / times_a();
    F.dinv[i] = inv;
    // p_j = v . z_j through the row lists of the rows v touches
    for (size_t k = 0; k < v.idx.size(); k++) {
      const double x = v.val[k];
      if (x == 0.0) continue;
      const int h = v.idx[k];
      for (int id = z.e[h].next; id != h; id = z.e[id].next) low.add(z.e[id].col, x * z.e[id].val);
    }
    for (size_t k = 0; k < low.idx.size(); k++) {
      const double l = low.val[k] * inv;
      if (std::fabs(l) > ldlt_eps) {
        F.val.push_back(l);
        F.row.push_back(low.idx[k]);
      }
    }
    F.pcol.push_back((int)F.val.size());
    v.clear();
    // z_j -= (p_j / d_i) z_i, then drop small entries of z_j
    for (size_t k = 0; k < low.idx.size(); k++) {
      double f = low.val[k];
      if (f == 0.0) continue;
      f *= inv;
      const int j = low.idx[k];
      for (int id : colz[j]) {
        v.push(z.e[id].row, z.e[id].val);
        z.remove(id);
      }
      colz[j].clear();
      for (size_t m = 0; m < zi_idx.size(); m++) v.add(zi_idx[m], -f * zi_val[m]);
      for (size_t m = 0; m < v.idx.size(); m++)
        if (std::fabs(v.val[m]) > sainv_eps) colz[j].push_back(z.insert(v.idx[m], j, v.val[m]));
      v.clear();
    }
    low.clear();
  }
  take_column(n - 1);
  F.dinv[n - 1] = 1.0 / times_a();
}

}  // namespace od

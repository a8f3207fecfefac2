// Threshold incomplete Cholesky of the reference's InCholeskyPreconditioner
// (solver/inCholeskyPreconditioner.cpp:18-130), made on the host as the
// reference makes it -- a left-looking sweep over the columns, each column
// needing every earlier column that reaches its row -- and then applied on
// the device by the triangular sweeps of od_ldlt.cu.
//
// Column i starts from A's stored lower column i (diagonal first, zero
// values left out, as BlockedSymSparseMatrix::getColumn gives it).  The
// earlier columns j with a stored entry in row i are found through per-row
// chains (chain[r] = the columns whose next unused entry is in row r, most
// recently linked first, with that entry's position); each subtracts L_ij
// times its entries below row i, then moves on to the chain of its next
// row.  With d the running diagonal (A_ii less the squares of the entries
// stored in row i), an off-diagonal v in row r is dropped when
// v^2 < |eps^2 d d_r| -- |v| relaxedScale then goes to both d and d_r -- and
// kept otherwise; L_ii = sqrt(d) (d <= 0 becomes eps^2 d^2), L_ri = v / L_ii,
// d_r -= L_ri^2.  The last column takes sqrt(d) alone.
//
// Every accumulation runs in the reference's order (the chain order decides
// the order of the updates), so the factor is bit-identical to the
// reference's for the same matrix values.  Built with -ffp-contract=off.
#include <algorithm>
#include <cmath>
#include <vector>

#include "od_internal.h"

namespace od {

// positions of the stored lower entries of every scalar column, in the
// order getColumn visits them (core/sparseMatrix.h:297-365)
void ric_columns(int n, int nbc, const std::vector<int>& pcol, const std::vector<int>& rows,
                 const std::vector<int>& oris, RicColumns& out) {
  out.n = n;
  out.ptr.assign(n + 1, 0);
  out.row.clear();
  out.src.clear();
  for (int c = 0; c < n; c++) {
    if (c / 3 < nbc) {
      const int bc = c / 3, off = c - 3 * bc;
      int at = oris[bc];
      int k = pcol[bc];
      const int e = pcol[bc + 1];
      if (k < e && rows[k] == 3 * bc) {   // packed diagonal block (0,0),(1,0),(2,0),(1,1),(2,1),(2,2)
        static const int first[3] = {0, 3, 5};
        for (int i = 0; i < 3 - off; i++) {
          out.row.push_back(c + i);
          out.src.push_back(at + first[off] + i);
        }
        at += 6;
        k++;
      }
      for (; k < e; k++) {
        const int r0 = rows[k];
        const int w = k == e - 1 ? std::min(3, n - r0) : 3;
        for (int i = 0; i < w; i++) {
          out.row.push_back(r0 + i);
          out.src.push_back(at + off * w + i);
        }
        at += 3 * w;
      }
    } else {
      const int col = nbc + (c - 3 * nbc);
      for (int q = pcol[col]; q < pcol[col + 1]; q++) {
        out.row.push_back(rows[q]);
        out.src.push_back(oris[col] + (q - pcol[col]));
      }
    }
    out.ptr[c + 1] = (int)out.row.size();
  }
}

namespace {

// column accumulator: entries in insertion order, dense position index
struct ColAcc {
  std::vector<int> where, idx;
  std::vector<double> val;
  explicit ColAcc(int n) : where(n, 0) {}
  void add(int i, double x) {
    const int w = where[i];
    if (w) {
      val[w - 1] += x;
    } else {
      idx.push_back(i);
      val.push_back(x);
      where[i] = (int)idx.size();
    }
  }
  void clear() {
    for (int i : idx) where[i] = 0;
    idx.clear();
    val.clear();
  }
};

}  // namespace

void ric_factor(const RicColumns& A, const double* a, double eps, double relax, RicFactor& F) {
  const int n = A.n;
  F.n = n;
  F.val.clear();
  F.row.clear();
  F.pcol.assign(1, 0);
  if (n == 0) return;
  // getDiagonal: the stored (c, c) value, 0 when absent
  std::vector<double> d(n, 0.0);
  for (int c = 0; c < n; c++)
    if (A.ptr[c] < A.ptr[c + 1] && A.row[A.ptr[c]] == c) d[c] = a[A.src[A.ptr[c]]];
  std::vector<int> chain_col(n, -1), chain_at(n, -1);
  const double eps2 = eps * eps;
  ColAcc w(n);
  std::vector<std::pair<int, double>> kept;

  auto load = [&](int c) {
    w.clear();
    for (int q = A.ptr[c]; q < A.ptr[c + 1]; q++) {
      const double x = a[A.src[q]];
      if (x != 0.0) w.add(A.row[q], x);
    }
  };
  auto finish = [&](int c) {
    double diag = d[c];
    kept.clear();
    for (size_t k = 1; k < w.idx.size(); k++) {   // everything after the first entry
      const int r = w.idx[k];
      const double v = w.val[k];
      if (v == 0.0) continue;
      if (v * v < std::fabs(eps2 * diag * d[r])) {
        const double comp = std::fabs(v) * relax;
        diag += comp;
        d[r] += comp;
      } else {
        kept.push_back({r, v});
      }
    }
    const int start = F.pcol[c];
    F.pcol.push_back(start + 1 + (int)kept.size());
    std::sort(kept.begin(), kept.end(),
              [](const std::pair<int, double>& x, const std::pair<int, double>& y) { return x.first < y.first; });
    if (!kept.empty()) {
      const int r = kept[0].first;
      chain_col[c] = chain_col[r];
      chain_at[c] = chain_at[r];
      chain_col[r] = c;
      chain_at[r] = start + 1;
    }
    if (diag <= 0.0) diag = eps2 * diag * diag;
    const double root = std::sqrt(diag);
    F.val.push_back(root);
    F.row.push_back(c);
    const double inv = 1.0 / root;
    for (const auto& e : kept) {
      const double l = e.second * inv;
      F.row.push_back(e.first);
      F.val.push_back(e.second * inv);
      d[e.first] -= l * l;
    }
  };

  load(0);
  finish(0);
  for (int i = 1; i < n - 1; i++) {
    load(i);
    int j = chain_col[i], at = chain_at[i];
    while (j >= 0) {
      const int next = at + 1, end = F.pcol[j + 1];
      const double upper = F.val[at];
      for (int k = next; k < end; k++) w.add(F.row[k], -upper * F.val[k]);
      const int nj = chain_col[j], nat = chain_at[j];
      if (next < end) {   // column j moves on to the chain of its next row
        const int r = F.row[next];
        chain_col[j] = chain_col[r];
        chain_at[j] = chain_at[r];
        chain_col[r] = j;
        chain_at[r] = next;
      }
      j = nj;
      at = nat;
    }
    finish(i);
  }
  F.val.push_back(std::sqrt(d[n - 1]));
  F.row.push_back(n - 1);
  F.pcol.push_back(F.pcol[n - 1] + 1);
}

}  // namespace od

// Node relabeling of the reference's MeshRelabeler (core/meshRelabler.cpp:
// 192-505): the Gibbs-Poole-Stockmeyer bandwidth and profile reduction, then
// the elements reordered by the sum of their new labels.  A host pass over
// the mesh, run before a scene is created: it shortens the column spans of
// the SpMV gathers (locality in L2) and the dependency chains of the
// triangular sweeps.
//
// Steps, as the reference takes them:
//  1. pseudo-diameter: from a node of minimum degree build its rooted level
//     structure (BFS levels); try every node of the deepest level, in
//     increasing degree: a deeper structure restarts the search from that
//     node, otherwise the narrowest one is the end;
//  2. width reduction: a node with the same level from both ends keeps it;
//     the others, grouped into connected components (the fixed nodes
//     removed), go as a whole to their start levels or end levels, whichever
//     crowds the component's fullest level less (ties: the narrower
//     structure); the first (smallest) component also decides the direction
//     of the final numbering;
//  3. numbering level by level from the lower-degree end: in each level the
//     first node is the lowest-degree neighbour of the earliest numbered node
//     of the previous level that has one, each numbered node pulls in its
//     unnumbered neighbours of the same level (highest degree first), and the
//     rest of the level follows in increasing degree.
// The reference breaks ties through hash-set and heap orders of its standard
// library; here every tie goes to the lower node index, so the labels are
// deterministic (and not the reference's).  The reference labels only the
// start node's connected component; here every component is labelled in
// turn (and nodes in no element go last).
#include <algorithm>
#include <climits>
#include <queue>
#include <vector>

#include "od_internal.h"

namespace od {
namespace {

struct Graph {
  int n = 0;
  std::vector<int> ptr, adj, deg;
};

// rooted level structure: lv[0] = {root}, lv[i] = nodes at distance i
struct Levels {
  std::vector<std::vector<int>> lv;
  int root() const { return lv[0][0]; }
  int depth() const { return (int)lv.size(); }
  int width() const {
    int w = 0;
    for (size_t i = 1; i < lv.size(); i++) w = std::max(w, (int)lv[i].size());
    return w;
  }
};

Levels levels_from(const Graph& g, int root, std::vector<int>& mark, int stamp) {
  Levels L;
  L.lv.push_back({root});
  mark[root] = stamp;
  for (;;) {
    std::vector<int> next;
    for (int v : L.lv.back())
      for (int q = g.ptr[v]; q < g.ptr[v + 1]; q++) {
        const int a = g.adj[q];
        if (mark[a] != stamp) {
          mark[a] = stamp;
          next.push_back(a);
        }
      }
    if (next.empty()) break;
    L.lv.push_back(std::move(next));
  }
  return L;
}

// labels the connected component of `seed` with labels next, next + 1, ...
void label_component(const Graph& g, int seed, std::vector<int>& label, int& next, std::vector<int>& mark,
                     int& stamp) {
  auto by_degree = [&](int a, int b) { return g.deg[a] != g.deg[b] ? g.deg[a] < g.deg[b] : a < b; };
  // 1. pseudo-diameter
  Levels S = levels_from(g, seed, mark, ++stamp), E;
  for (bool found = false; !found;) {
    found = true;
    int best = INT_MAX;
    std::vector<int> last = S.lv.back();
    std::stable_sort(last.begin(), last.end(), by_degree);
    for (int v : last) {
      Levels M = levels_from(g, v, mark, ++stamp);
      if (M.depth() > S.depth()) {
        S = std::move(M);
        found = false;
        break;
      }
      if (M.width() < best) {
        best = M.width();
        E = std::move(M);
      }
    }
  }
  const int ds = S.depth(), de = E.depth(), size = std::max(ds, de);
  const bool start_smaller = E.width() > S.width();
  // 2. width reduction: level from the start, level from the end
  std::vector<int> comp_nodes;   // component members (for the later passes)
  for (const auto& l : S.lv) comp_nodes.insert(comp_nodes.end(), l.begin(), l.end());
  std::vector<int> lstart(g.n, -1), lend(g.n, -1), newlev(g.n, -1);
  for (int i = 0; i < ds; i++)
    for (int v : S.lv[i]) lstart[v] = i;
  std::vector<int> remained;
  for (int i = 0; i < de; i++)
    for (int v : E.lv[i]) {
      lend[v] = de - 1 - i;
      if (lstart[v] == lend[v]) newlev[v] = lend[v];
      else remained.push_back(v);
    }
  // components of the remaining nodes (the fixed nodes taken out)
  std::vector<std::vector<int>> comps;
  ++stamp;
  for (int v : remained) {
    if (mark[v] == stamp) continue;
    comps.emplace_back();
    std::vector<int>& c = comps.back();
    std::queue<int> work;
    mark[v] = stamp;
    c.push_back(v);
    work.push(v);
    while (!work.empty()) {
      const int x = work.front();
      work.pop();
      for (int q = g.ptr[x]; q < g.ptr[x + 1]; q++) {
        const int a = g.adj[q];
        if (mark[a] != stamp && newlev[a] < 0) {
          mark[a] = stamp;
          c.push_back(a);
          work.push(a);
        }
      }
    }
  }
  std::stable_sort(comps.begin(), comps.end(),
                   [](const std::vector<int>& a, const std::vector<int>& b) { return a.size() < b.size(); });
  bool select_second = false;
  std::vector<int> cf(size), cs(size);
  for (size_t ci = 0; ci < comps.size(); ci++) {
    std::fill(cf.begin(), cf.end(), 0);
    std::fill(cs.begin(), cs.end(), 0);
    for (int v : comps[ci]) {
      cf[lstart[v]]++;
      cs[lend[v]]++;
    }
    const int mf = *std::max_element(cf.begin(), cf.end()), ms = *std::max_element(cs.begin(), cs.end());
    if (ci == 0 && (mf > ms || (mf == ms && !start_smaller))) select_second = true;
    const bool use_start = mf < ms || (mf == ms && start_smaller);
    for (int v : comps[ci]) newlev[v] = use_start ? lstart[v] : lend[v];
  }
  // level lists in increasing degree
  std::vector<std::vector<int>> L(size);
  for (int v : comp_nodes) L[newlev[v]].push_back(v);
  for (auto& l : L) std::stable_sort(l.begin(), l.end(), by_degree);
  // 3. numbering
  int root = S.root(), init = 0, pace = 1;
  bool interchange = false;
  if (g.deg[S.root()] > g.deg[E.root()]) {
    interchange = true;
    root = E.root();
    init = size - 1;
    pace = -1;
  }
  const int first_label = next;
  std::vector<char> pending(g.n, 0);
  for (int v : comp_nodes) pending[v] = 1;
  // the root is numbered first, in level init, wherever step 2 put it
  std::vector<int> head(size, 0);
  std::vector<int> work;      // nodes numbered in the current level, in order
  auto number = [&](int v, int lev) {
    std::vector<int> pull;    // unnumbered neighbours in the same level
    label[v] = next++;
    pending[v] = 0;
    work.push_back(v);
    for (int q = g.ptr[v]; q < g.ptr[v + 1]; q++) {
      const int a = g.adj[q];
      if (pending[a] && newlev[a] == lev) {
        pending[a] = 0;
        pull.push_back(a);
      }
    }
    std::stable_sort(pull.begin(), pull.end(),
                     [&](int a, int b) { return g.deg[a] != g.deg[b] ? g.deg[a] > g.deg[b] : a < b; });
    for (int a : pull) {
      label[a] = next++;
      work.push_back(a);
    }
  };
  auto rest_of_level = [&](int lev) {
    std::vector<int>& l = L[lev];
    for (int& h = head[lev]; h < (int)l.size(); h++)
      if (pending[l[h]]) number(l[h], lev);
  };
  newlev[root] = init;
  number(root, init);
  rest_of_level(init);
  for (int lev = init + pace; lev >= 0 && lev < size; lev += pace) {
    int pick = -1;
    for (size_t k = 0; k < work.size() && pick < 0; k++) {
      const int v = work[k];
      for (int q = g.ptr[v]; q < g.ptr[v + 1]; q++) {
        const int a = g.adj[q];
        if (pending[a] && newlev[a] == lev && (pick < 0 || g.deg[pick] > g.deg[a])) pick = a;
      }
    }
    work.clear();
    if (pick >= 0) number(pick, lev);
    rest_of_level(lev);
  }
  // every node of the component numbered; reverse the component's labels
  // unless the two direction choices agree
  if (interchange == select_second)
    for (int v : comp_nodes) label[v] = first_label + (next - 1 - label[v]);
}

}  // namespace

void relabel_nodes(int n_nodes, int n_elems, int per, const int* elems, std::vector<int>& label) {
  // the node graph: every pair of nodes of an element, neighbours ascending
  Graph g;
  g.n = n_nodes;
  std::vector<long long> pairs;
  pairs.reserve((size_t)n_elems * per * (per - 1));
  for (int e = 0; e < n_elems; e++)
    for (int a = 0; a < per; a++)
      for (int b = 0; b < per; b++)
        if (a != b) pairs.push_back((long long)elems[(size_t)e * per + a] * n_nodes + elems[(size_t)e * per + b]);
  std::sort(pairs.begin(), pairs.end());
  pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
  g.ptr.assign(n_nodes + 1, 0);
  g.adj.resize(pairs.size());
  for (size_t k = 0; k < pairs.size(); k++) {
    g.ptr[pairs[k] / n_nodes + 1]++;
    g.adj[k] = (int)(pairs[k] % n_nodes);
  }
  for (int v = 0; v < n_nodes; v++) g.ptr[v + 1] += g.ptr[v];
  g.deg.resize(n_nodes);
  for (int v = 0; v < n_nodes; v++) g.deg[v] = g.ptr[v + 1] - g.ptr[v];
  label.assign(n_nodes, -1);
  std::vector<int> mark(n_nodes, 0);
  int stamp = 0, next = 0;
  // components in turn, each from its lowest-index node of minimum degree
  for (;;) {
    int seed = -1;
    for (int v = 0; v < n_nodes; v++)
      if (label[v] < 0 && g.deg[v] > 0 && (seed < 0 || g.deg[v] < g.deg[seed])) seed = v;
    if (seed < 0) break;
    label_component(g, seed, label, next, mark, stamp);
  }
  for (int v = 0; v < n_nodes; v++)   // nodes in no element
    if (label[v] < 0) label[v] = next++;
}

}  // namespace od

using namespace od;

extern "C" od_status od_mesh_relabel(int n_nodes, int n_elems, int nodes_per_elem, int* elems, int* new_labels) {
  OD_CHECK_ARG(n_nodes >= 0 && n_elems >= 0 && nodes_per_elem >= 1 && nodes_per_elem <= 8,
               "od_mesh_relabel: bad sizes");
  OD_CHECK_ARG(new_labels && (n_elems == 0 || elems), "od_mesh_relabel: NULL argument");
  OD_CHECK_ARG((long long)n_nodes * n_nodes < (1LL << 62), "od_mesh_relabel: too many nodes");
  for (long long k = 0; k < (long long)n_elems * nodes_per_elem; k++)
    OD_CHECK_ARG(elems[k] >= 0 && elems[k] < n_nodes, "od_mesh_relabel: node id out of range");
  std::vector<int> label;
  relabel_nodes(n_nodes, n_elems, nodes_per_elem, elems, label);
  std::copy(label.begin(), label.end(), new_labels);
  // elements: new labels, ordered by the sum of their labels (stable)
  std::vector<long long> score(n_elems);
  std::vector<int> order(n_elems);
  for (int e = 0; e < n_elems; e++) {
    long long sc = 0;
    for (int a = 0; a < nodes_per_elem; a++) sc += label[elems[(size_t)e * nodes_per_elem + a]];
    score[e] = sc;
    order[e] = e;
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return score[a] < score[b]; });
  std::vector<int> out((size_t)n_elems * nodes_per_elem);
  for (int k = 0; k < n_elems; k++)
    for (int a = 0; a < nodes_per_elem; a++)
      out[(size_t)k * nodes_per_elem + a] = label[elems[(size_t)order[k] * nodes_per_elem + a]];
  std::copy(out.begin(), out.end(), elems);
  return OD_OK;
}

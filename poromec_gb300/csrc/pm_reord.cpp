// pm_reord.cpp -- node reordering of the 'mesh' macro: reverse Cuthill-McKee
// of the node graph (reord, Reord.f:1-44, with genrcm_v1 / fnroot_v1 /
// rcm_v1 / rootls_v1 / degree_v1, Reord.f:45-430).
//
// The reference orders the nodes before numbering the equations
// (Main.f:585-590, reordf = .true. by default, Main.f:255) with the
// reverse Cuthill-McKee algorithm of George and Liu (SPARSPAK, "Computer
// Solution of Large Sparse Positive Definite Systems", 1981): for each
// connected component, a pseudo-peripheral root found by the Gibbs-Poole-
// Stockmeyer level-structure search, then a breadth-first numbering in
// which the unnumbered neighbours of each node are taken in increasing
// degree (ties in adjacency order), reversed.  The node graph is graph_v1's
// (Graph.f:72-133): two nodes are adjacent when they share an element, and
// each adjacency list is sorted by node number.  The permutation decides
// the equation numbers and therefore the CSRD pattern, so it has to be the
// reference's exactly; every tie-break below follows those routines.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "../../include/poromec_gb300.h"

namespace pm {
namespace {

struct NodeGraph {
  std::vector<int64_t> ptr;  // adjacency of node v (0-based): adj[ptr[v] .. ptr[v+1])
  std::vector<int32_t> adj;  // sorted, unique, without v itself
};

int node_graph(int nnode, int numel, int nen, const int32_t* ix, NodeGraph& g) {
  std::vector<int64_t> cnt(nnode + 1, 0);
  for (int e = 0; e < numel; ++e)
    for (int a = 0; a < nen; ++a) {
      const int v = ix[(size_t)(nen + 1) * e + a];
      if (v < 0 || v > nnode) return PM_E_ARG;
      if (v > 0) cnt[v] += nen - 1;  // the bound of aponta_v1
    }
  for (int v = 0; v < nnode; ++v) cnt[v + 1] += cnt[v];
  std::vector<int32_t> raw(cnt[nnode]);
  std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
  for (int e = 0; e < numel; ++e) {
    const int32_t* c = ix + (size_t)(nen + 1) * e;
    for (int a = 0; a < nen; ++a) {
      if (c[a] == 0) continue;
      for (int b = 0; b < nen; ++b)
        if (c[b] != 0 && c[b] != c[a]) raw[fill[c[a] - 1]++] = c[b] - 1;
    }
  }
  g.ptr.assign(nnode + 1, 0);
  g.adj.clear();
  g.adj.reserve(raw.size() / 2);
  std::vector<int32_t> buf;
  for (int v = 0; v < nnode; ++v) {
    buf.assign(raw.begin() + cnt[v], raw.begin() + fill[v]);
    std::sort(buf.begin(), buf.end());
    buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
    g.adj.insert(g.adj.end(), buf.begin(), buf.end());
    g.ptr[v + 1] = (int64_t)g.adj.size();
  }
  return PM_OK;
}

// Breadth-first level structure from root over the nodes still unnumbered
// (live); levels are appended to ls, level k starting at lvl[k].  Returns
// the number of levels; ls holds the component.
int level_structure(const NodeGraph& g, int root, const std::vector<char>& live,
                    std::vector<char>& seen, std::vector<int32_t>& ls,
                    std::vector<int32_t>& lvl) {
  ls.clear();
  lvl.clear();
  ls.push_back(root);
  seen[root] = 1;
  size_t begin = 0;
  while (begin < ls.size()) {
    lvl.push_back((int32_t)begin);
    const size_t end = ls.size();
    for (size_t i = begin; i < end; ++i) {
      const int v = ls[i];
      for (int64_t k = g.ptr[v]; k < g.ptr[v + 1]; ++k) {
        const int w = g.adj[k];
        if (live[w] && !seen[w]) {
          seen[w] = 1;
          ls.push_back(w);
        }
      }
    }
    begin = end;
  }
  for (int v : ls) seen[v] = 0;
  lvl.push_back((int32_t)ls.size());
  return (int)lvl.size() - 1;
}

}  // namespace

int rcm_order(int nnode, int numel, int nen, const int32_t* ix, int32_t* num) {
  if (nnode < 1 || numel < 0 || nen < 1 || (!ix && numel > 0) || !num) return PM_E_ARG;
  NodeGraph g;
  if (int st = node_graph(nnode, numel, nen, ix, g)) return st;
  auto degree = [&](int v) { return (int)(g.ptr[v + 1] - g.ptr[v]); };
  std::vector<char> live(nnode, 1), seen(nnode, 0);
  std::vector<int32_t> ls, lvl, order;
  int placed = 0;
  for (int start = 0; start < nnode && placed < nnode; ++start) {
    if (!live[start]) continue;
    // pseudo-peripheral root (fnroot_v1): from the deepest level of the
    // current root's level structure take the first node of least degree,
    // keep it while its structure is deeper
    int root = start;
    int nlvl = level_structure(g, root, live, seen, ls, lvl);
    const int cc = (int)ls.size();
    while (nlvl > 1 && nlvl < cc) {
      int best = ls[lvl[nlvl - 1]], mindeg = cc;
      for (int j = lvl[nlvl - 1]; j < cc; ++j)
        if (degree(ls[j]) < mindeg) {
          best = ls[j];
          mindeg = degree(ls[j]);
        }
      root = best;
      const int deeper = level_structure(g, root, live, seen, ls, lvl);
      if (deeper <= nlvl) break;
      nlvl = deeper;
    }
    // Cuthill-McKee from the root (rcm_v1): each node's unnumbered
    // neighbours in adjacency order, stably sorted by degree
    order.clear();
    order.push_back(root);
    live[root] = 0;
    for (size_t i = 0; i < order.size(); ++i) {
      const int v = order[i];
      const size_t first = order.size();
      for (int64_t k = g.ptr[v]; k < g.ptr[v + 1]; ++k) {
        const int w = g.adj[k];
        if (live[w]) {
          live[w] = 0;
          order.push_back(w);
        }
      }
      for (size_t a = first + 1; a < order.size(); ++a) {  // stable insertion
        const int w = order[a];
        size_t b = a;
        while (b > first && degree(order[b - 1]) > degree(w)) {
          order[b] = order[b - 1];
          --b;
        }
        order[b] = w;
      }
    }
    // reversed into the permutation: num(i) is the node numbered i-th
    for (size_t i = 0; i < order.size(); ++i)
      num[placed + (int)i] = order[order.size() - 1 - i] + 1;
    placed += (int)order.size();
  }
  return PM_OK;
}

}  // namespace pm

extern "C" int pm_reord(int nnode, int numel, int nen, const int32_t* ix, int32_t* num) {
  return pm::rcm_order(nnode, numel, nen, ix, num);
}

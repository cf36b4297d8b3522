// jfem_graph.cu — reverse Cuthill–McKee node renumbering (host, C++).
//
// Restates symrcm of src/graph/graph_ordering.jl:21-98: breadth-first search
// from a given start node, each node's unvisited neighbours appended in order of
// increasing degree (a stable sort, so equal degrees keep the adjacency order),
// then the whole order reversed; bandwidth(G) = 2·max|v − w| + 1 over edges
// (:21-29).  The graph is the node graph of the mesh (nodes sharing an element),
// adjacency lists in ascending node number.  The reference's loop assumes a
// connected graph; here nodes unreachable from the start are appended by
// restarting the search from the lowest-numbered unvisited node, so every mesh
// gets a full permutation.  A preprocessing step for memory locality of the
// apply: sequential by nature (the order within a level depends on the parents'
// order), so it runs on the host.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/jfem.h"
#include "jfem_abi_guard.h"

namespace jfem {

static void node_graph(int64_t N, int64_t E, int nen, const int64_t* conn, int base, std::vector<int64_t>& ptr,
                       std::vector<int64_t>& adj) {
  std::vector<std::vector<int64_t>> nb((size_t)N);
  for (int64_t e = 0; e < E; ++e)
    for (int a = 0; a < nen; ++a)
      for (int b = 0; b < nen; ++b)
        if (a != b) nb[(size_t)(conn[e * nen + a] - base)].push_back(conn[e * nen + b] - base);
  ptr.assign((size_t)N + 1, 0);
  adj.clear();
  for (int64_t v = 0; v < N; ++v) {
    auto& l = nb[(size_t)v];
    std::sort(l.begin(), l.end());
    l.erase(std::unique(l.begin(), l.end()), l.end());
    adj.insert(adj.end(), l.begin(), l.end());
    ptr[(size_t)v + 1] = (int64_t)adj.size();
  }
}

static int64_t graph_bandwidth(int64_t N, const std::vector<int64_t>& ptr, const std::vector<int64_t>& adj,
                               const int64_t* newpos) {
  int64_t bw = -1;
  for (int64_t v = 0; v < N; ++v)
    for (int64_t k = ptr[(size_t)v]; k < ptr[(size_t)v + 1]; ++k) {
      const int64_t a = newpos ? newpos[v] : v, b = newpos ? newpos[adj[(size_t)k]] : adj[(size_t)k];
      bw = std::max(bw, a > b ? a - b : b - a);
    }
  return 2 * bw + 1;
}

}  // namespace jfem

extern "C" {

int jfem_rcm(int64_t n_nodes, int64_t n_elem, int nodes_per_elem, const int64_t* conn, int index_base,
             int64_t start, int64_t* perm, int64_t* bandwidth_before, int64_t* bandwidth_after) {
  ABI_TRY
  if (n_nodes <= 0 || n_elem < 0 || nodes_per_elem <= 0 || !conn || !perm) return JFEM_ERR_INVALID;
  for (int64_t k = 0; k < n_elem * nodes_per_elem; ++k)
    if (conn[k] - index_base < 0 || conn[k] - index_base >= n_nodes) return JFEM_ERR_INVALID;
  const int64_t s0 = start - index_base;
  if (s0 < 0 || s0 >= n_nodes) return JFEM_ERR_INVALID;
  std::vector<int64_t> ptr, adj;
  jfem::node_graph(n_nodes, n_elem, nodes_per_elem, conn, index_base, ptr, adj);
  std::vector<int64_t> order;
  order.reserve((size_t)n_nodes);
  std::vector<char> visited((size_t)n_nodes, 0);
  std::vector<int64_t> aux;
  auto degree = [&](int64_t v) { return ptr[(size_t)v + 1] - ptr[(size_t)v]; };
  int64_t next_unvisited = 0;
  int64_t s = s0;
  while ((int64_t)order.size() < n_nodes) {
    visited[(size_t)s] = 1;
    size_t head = order.size();
    order.push_back(s);
    for (; head < order.size(); ++head) {
      const int64_t v = order[head];
      aux.assign(adj.begin() + ptr[(size_t)v], adj.begin() + ptr[(size_t)v + 1]);
      std::stable_sort(aux.begin(), aux.end(), [&](int64_t a, int64_t b) { return degree(a) < degree(b); });
      for (int64_t w : aux) {
        if (visited[(size_t)w]) continue;
        visited[(size_t)w] = 1;
        order.push_back(w);
      }
    }
    while (next_unvisited < n_nodes && visited[(size_t)next_unvisited]) ++next_unvisited;
    if (next_unvisited < n_nodes) s = next_unvisited;
  }
  std::reverse(order.begin(), order.end());
  std::vector<int64_t> newpos((size_t)n_nodes);
  for (int64_t k = 0; k < n_nodes; ++k) {
    perm[k] = order[(size_t)k] + index_base;   // new position k holds old node perm[k]
    newpos[(size_t)order[(size_t)k]] = k;
  }
  if (bandwidth_before) *bandwidth_before = jfem::graph_bandwidth(n_nodes, ptr, adj, nullptr);
  if (bandwidth_after) *bandwidth_after = jfem::graph_bandwidth(n_nodes, ptr, adj, newpos.data());
  return JFEM_OK;
  ABI_CATCH(nullptr)
}

}  // extern "C"

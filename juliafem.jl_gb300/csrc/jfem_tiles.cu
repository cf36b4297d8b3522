// jfem_tiles.cu — element tiles for the shared-memory apply.
//
// The two-phase apply (element kernel → per-element results in HBM → node
// gather) moves 2 × 4·3·n_en bytes per element through HBM and gathers them with
// scattered 4-byte loads.  Tiling keeps that traffic on chip: elements are
// ordered along a Morton curve of their centroids and cut into tiles of
// JFEM_TILE consecutive elements; one CTA per tile stages the tile's nodes in
// shared memory, computes the element vectors into shared memory, sums them per
// local node in a fixed order, writes the nodes owned entirely by the tile to y
// and only the tile-boundary partial sums to HBM (one float4 per (node, tile),
// grouped by node).  A second kernel adds the boundary partials of each shared
// node in ascending tile order.  Results are deterministic (fixed summation
// orders) and independent of scheduling.  Padding elements exist only past E
// (in the last tile), so a tile position is valid iff its index is below E.
//
// Built once per mesh on the host from the caller's arrays (O(E log E)).
#include <algorithm>
#include <cstring>
#include <numeric>
#include <type_traits>
#include <vector>

#include "jfem_common.cuh"

namespace jfem {

static inline uint64_t spread3(uint64_t v) {   // 21 bits → every third bit
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}

int tiles_build(Ctx* c, const double* X, const int64_t* conn_h, int base) {
  const int64_t N = c->N, E = c->E;
  const int nn = c->nn;
  const int T = JFEM_TILE;
  // Morton order of element centroids
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int64_t i = 0; i < N; ++i)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], X[3 * i + d]);
      hi[d] = std::max(hi[d], X[3 * i + d]);
    }
  double span = 0.0;
  for (int d = 0; d < 3; ++d) span = std::max(span, hi[d] - lo[d]);
  if (!(span > 0.0)) span = 1.0;
  std::vector<std::pair<uint64_t, int64_t>> key((size_t)E);
  for (int64_t e = 0; e < E; ++e) {
    double cen[3] = {0, 0, 0};
    for (int a = 0; a < nn; ++a)
      for (int d = 0; d < 3; ++d) cen[d] += X[3 * (conn_h[e * nn + a] - base) + d];
    uint64_t code = 0;
    for (int d = 0; d < 3; ++d) {
      const double q = (cen[d] / nn - lo[d]) / span * 2097151.0;
      code |= spread3((uint64_t)std::max(0.0, std::min(2097151.0, q))) << d;
    }
    key[(size_t)e] = {code, e};
  }
  std::sort(key.begin(), key.end());
  const int64_t ntiles = (E + T - 1) / T;
  const int64_t Epad = ntiles * T;
  std::vector<int> perm((size_t)Epad, -1);
  for (int64_t k = 0; k < E; ++k) perm[(size_t)k] = (int)key[(size_t)k].second;
  // elements per global node
  std::vector<int> cntg((size_t)N, 0);
  for (int64_t t = 0; t < E * nn; ++t) cntg[(size_t)(conn_h[t] - base)]++;

  std::vector<uint16_t> tconn((size_t)nn * Epad, 0);
  std::vector<int> tnode_ptr((size_t)ntiles + 1, 0), tnodes, tout;
  std::vector<uint16_t> tadj_ptr, tadj((size_t)ntiles * T * nn, 0);
  std::vector<std::pair<int64_t, int64_t>> brec;   // (node, slot), slots ascend with tile
  tnodes.reserve((size_t)E * 2);
  int Lmax = 0;
  int64_t nslots = 0;
  std::vector<int> loc;     // (node) of the tile, sorted unique
  std::vector<int> lcnt;
  for (int64_t t = 0; t < ntiles; ++t) {
    loc.clear();
    for (int k = 0; k < T; ++k) {
      const int e = perm[(size_t)(t * T + k)];
      if (e < 0) continue;
      for (int a = 0; a < nn; ++a) loc.push_back((int)(conn_h[(int64_t)e * nn + a] - base));
    }
    std::sort(loc.begin(), loc.end());
    loc.erase(std::unique(loc.begin(), loc.end()), loc.end());
    const int L = (int)loc.size();
    if (L > 65535) return set_err(c, JFEM_ERR_INVALID, "tile has too many nodes");
    Lmax = std::max(Lmax, L);
    tnode_ptr[(size_t)t + 1] = tnode_ptr[(size_t)t] + L;
    lcnt.assign((size_t)L + 1, 0);
    // local connectivity and counts
    for (int k = 0; k < T; ++k) {
      const int e = perm[(size_t)(t * T + k)];
      if (e < 0) continue;
      for (int a = 0; a < nn; ++a) {
        const int g = (int)(conn_h[(int64_t)e * nn + a] - base);
        const int li = (int)(std::lower_bound(loc.begin(), loc.end(), g) - loc.begin());
        tconn[(size_t)a * Epad + t * T + k] = (uint16_t)li;
        lcnt[(size_t)li + 1]++;
      }
    }
    for (int j = 0; j < L; ++j) lcnt[(size_t)j + 1] += lcnt[(size_t)j];
    for (int j = 0; j <= L; ++j) tadj_ptr.push_back((uint16_t)lcnt[(size_t)j]);
    // local adjacency, ascending local element then local node index
    std::vector<int> cur(lcnt.begin(), lcnt.end() - 1);
    for (int k = 0; k < T; ++k) {
      const int e = perm[(size_t)(t * T + k)];
      if (e < 0) continue;
      for (int a = 0; a < nn; ++a) {
        const int li = tconn[(size_t)a * Epad + t * T + k];
        tadj[(size_t)t * T * nn + cur[(size_t)li]++] = (uint16_t)(a * T + k);   // slot of (k, a) in [n_en][T]
      }
    }
    for (int j = 0; j < L; ++j) {
      const int g = loc[(size_t)j];
      tnodes.push_back(g);
      const int here = lcnt[(size_t)j + 1] - lcnt[(size_t)j];
      if (here == cntg[(size_t)g]) {
        tout.push_back(g);
      } else {
        tout.push_back(-1 - (int)nslots);
        brec.push_back({g, nslots});
        ++nslots;
      }
    }
  }
  // boundary nodes: partial-sum slots grouped by node, ascending tile within a
  // node, so the boundary pass reads each node's partials as one contiguous run
  std::stable_sort(brec.begin(), brec.end(),
                   [](const std::pair<int64_t, int64_t>& a, const std::pair<int64_t, int64_t>& b) {
                     return a.first < b.first;
                   });
  std::vector<int> bnodes, bptr(1, 0), pos_of_slot((size_t)nslots, 0);
  for (size_t i = 0; i < brec.size(); ++i) {
    if (i == 0 || brec[i].first != brec[i - 1].first) {
      if (i) bptr.push_back((int)i);
      bnodes.push_back((int)brec[i].first);
    }
    pos_of_slot[(size_t)brec[i].second] = (int)i;
  }
  bptr.push_back((int)brec.size());
  if (bnodes.empty()) bptr.assign(1, 0);
  for (int& o : tout)
    if (o < 0) o = -1 - pos_of_slot[(size_t)(-1 - o)];

  // upload
  int rc = 0;
  auto up = [&](auto** dst, const auto& src) -> int {
    using T_ = std::remove_reference_t<decltype(src[0])>;
    int r = dalloc(c, dst, std::max<size_t>(src.size(), 1));
    if (r) return r;
    if (!src.empty())
      cudaMemcpyAsync(*dst, src.data(), src.size() * sizeof(T_), cudaMemcpyHostToDevice, c->stream);
    return 0;
  };
  if ((rc = up(&c->tperm, perm))) return rc;
  if ((rc = up(&c->tconn, tconn))) return rc;
  if ((rc = up(&c->tnode_ptr, tnode_ptr))) return rc;
  if ((rc = up(&c->tnodes, tnodes))) return rc;
  if ((rc = up(&c->tadj_ptr, tadj_ptr))) return rc;
  if ((rc = up(&c->tadj, tadj))) return rc;
  if ((rc = up(&c->tout, tout))) return rc;
  if ((rc = up(&c->bnodes, bnodes))) return rc;
  if ((rc = up(&c->bptr, bptr))) return rc;
  if ((rc = dalloc(c, &c->bpart, std::max<int64_t>(nslots, 1)))) return rc;
  c->ntiles = ntiles;
  c->Epad = Epad;
  c->tile_Lmax = Lmax;
  c->n_bnodes = (int64_t)bnodes.size();
  c->n_bslots = nslots;
  return sync_and_check(c, "tile upload");
}

}  // namespace jfem

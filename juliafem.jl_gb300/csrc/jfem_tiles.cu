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
#include <thread>
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
  host_parallel(E, [&](int64_t e0, int64_t e1) {
    for (int64_t e = e0; e < e1; ++e) {
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
  });
  // keys are unique (element index in the low half), so any sort gives the
  // same order: sort contiguous chunks on host threads, then merge pairwise
  {
    const int64_t hw = std::max<int64_t>(1, std::min<int64_t>(16, std::thread::hardware_concurrency()));
    const int64_t nchunk = std::max<int64_t>(1, std::min<int64_t>(hw, E / 4096));
    std::vector<int64_t> cut((size_t)nchunk + 1);
    for (int64_t k = 0; k <= nchunk; ++k) cut[(size_t)k] = E * k / nchunk;
    host_tasks(nchunk, [&](int64_t k) {
      std::sort(key.begin() + cut[(size_t)k], key.begin() + cut[(size_t)k + 1]);
    });
    for (int64_t w = 1; w < nchunk; w *= 2) {
      host_tasks((nchunk - w + 2 * w - 1) / (2 * w), [&](int64_t m) {
        const int64_t k = 2 * w * m;
        const int64_t lo = cut[(size_t)k], mid = cut[(size_t)(k + w)], hi = cut[(size_t)std::min(k + 2 * w, nchunk)];
        std::inplace_merge(key.begin() + lo, key.begin() + mid, key.begin() + hi);
      });
    }
  }
  const int64_t ntiles = (E + T - 1) / T;
  const int64_t Epad = ntiles * T;
  std::vector<int> perm((size_t)Epad, -1);
  for (int64_t k = 0; k < E; ++k) perm[(size_t)k] = (int)key[(size_t)k].second;
  // elements per global node
  std::vector<int> cntg((size_t)N, 0);   // elements per node (relaxed atomic counts: order-free)
  host_parallel(E * nn, [&](int64_t t0, int64_t t1) {
    for (int64_t t = t0; t < t1; ++t) __atomic_fetch_add(&cntg[(size_t)(conn_h[t] - base)], 1, __ATOMIC_RELAXED);
  });

  std::vector<uint16_t> tconn((size_t)nn * Epad, 0);
  std::vector<uint16_t> tadj((size_t)ntiles * T * nn, 0);
  // Per tile (independent, built on host threads): its sorted unique nodes,
  // their adjacency offsets, and which of them other tiles share.
  struct TileNodes {
    std::vector<int> asc;            // global nodes of the tile, ascending (the staging order)
    std::vector<uint16_t> asc_loc;   // local index of each of them
    std::vector<int> loc;            // global nodes of the tile (element slots descending, then ascending)
    std::vector<uint16_t> ptr;       // L + 1 offsets into the tile's adjacency block
    std::vector<uint8_t> shared;     // node also in another tile
    int nshared = 0;
  };
  std::vector<TileNodes> tn((size_t)ntiles);
  // per-thread scratch, reused across the thread's tiles (no allocation per tile)
  // open-addressing table of a tile's nodes (power of two ≥ 2·T·n_en slots)
  int HB = 1;
  while (HB < 2 * T * nn) HB <<= 1;
  struct Scratch {
    std::vector<int> lcnt, cnt, order, newidx, hkey, hval;
    std::vector<unsigned> used;   // table slots filled by the current tile
  };
  auto build_tile = [&](int64_t t, Scratch& sc) {
    TileNodes& o = tn[(size_t)t];
    std::vector<int>& hkey = sc.hkey;
    std::vector<int>& hval = sc.hval;
    if (hkey.size() != (size_t)HB) {
      hkey.assign((size_t)HB, -1);
      hval.assign((size_t)HB, 0);
    }
    auto slot_of = [&](int g) {
      unsigned h = ((unsigned)g * 2654435761u) & (unsigned)(HB - 1);
      while (hkey[h] != -1 && hkey[h] != g) h = (h + 1) & (unsigned)(HB - 1);
      return h;
    };
    // the tile's distinct global nodes (hash table), then ascending
    std::vector<int>& asc = o.asc;
    asc.clear();
    sc.used.clear();
    for (int k = 0; k < T; ++k) {
      const int e = perm[(size_t)(t * T + k)];
      if (e < 0) continue;
      for (int a = 0; a < nn; ++a) {
        const int g = (int)(conn_h[(int64_t)e * nn + a] - base);
        const unsigned h = slot_of(g);
        if (hkey[h] == -1) {
          hkey[h] = g;
          sc.used.push_back(h);
          asc.push_back(g);
        }
      }
    }
    std::sort(asc.begin(), asc.end());
    const int L = (int)asc.size();
    for (int j = 0; j < L; ++j) hval[slot_of(asc[(size_t)j])] = j;
    // ascending index of every (element, node) slot; element slots per node
    std::vector<int>& cnt = sc.cnt;
    cnt.assign((size_t)L, 0);
    for (int k = 0; k < T; ++k) {
      const int e = perm[(size_t)(t * T + k)];
      if (e < 0) continue;
      for (int a = 0; a < nn; ++a) {
        const int g = (int)(conn_h[(int64_t)e * nn + a] - base);
        const int ai = hval[slot_of(g)];
        tconn[(size_t)a * Epad + t * T + k] = (uint16_t)ai;
        cnt[(size_t)ai]++;
      }
    }
    for (const unsigned h : sc.used) hkey[h] = -1;   // empty again for the thread's next tile
    // local order: element slots per node descending (ties: ascending global
    // node), so the 32 nodes a warp sums have similar loop lengths
    std::vector<int>& order = sc.order;
    std::vector<int>& newidx = sc.newidx;
    order.resize((size_t)L);
    newidx.resize((size_t)L);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cnt[(size_t)x] > cnt[(size_t)y]; });
    std::vector<int>& loc = o.loc;
    loc.resize((size_t)L);
    for (int j = 0; j < L; ++j) {
      newidx[(size_t)order[(size_t)j]] = j;
      loc[(size_t)j] = asc[(size_t)order[(size_t)j]];
    }
    o.asc_loc.assign(newidx.begin(), newidx.end());
    std::vector<int>& lcnt = sc.lcnt;
    lcnt.assign((size_t)L + 1, 0);
    // local connectivity (ascending index → local index) and counts
    for (int k = 0; k < T; ++k) {
      const int e = perm[(size_t)(t * T + k)];
      if (e < 0) continue;
      for (int a = 0; a < nn; ++a) {
        uint16_t& slot = tconn[(size_t)a * Epad + t * T + k];
        const int li = newidx[slot];
        slot = (uint16_t)li;
        lcnt[(size_t)li + 1]++;
      }
    }
    for (int j = 0; j < L; ++j) lcnt[(size_t)j + 1] += lcnt[(size_t)j];
    o.ptr.assign(lcnt.begin(), lcnt.end());
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
    o.shared.assign((size_t)L, 0);
    o.nshared = 0;
    for (int j = 0; j < L; ++j)
      if (lcnt[(size_t)j + 1] - lcnt[(size_t)j] != cntg[(size_t)loc[(size_t)j]]) {
        o.shared[(size_t)j] = 1;
        ++o.nshared;
      }
  };
  host_parallel(ntiles, [&](int64_t t0, int64_t t1) {
    Scratch sc;
    for (int64_t t = t0; t < t1; ++t) build_tile(t, sc);
  });
  // tile offsets (serial prefix sums in tile order)
  std::vector<int> tnode_ptr((size_t)ntiles + 1, 0);
  std::vector<int64_t> slot_base((size_t)ntiles + 1, 0);
  int Lmax = 0;
  for (int64_t t = 0; t < ntiles; ++t) {
    const int L = (int)tn[(size_t)t].loc.size();
    if (L > 65535) return set_err(c, JFEM_ERR_INVALID, "tile has too many nodes");
    Lmax = std::max(Lmax, L);
    tnode_ptr[(size_t)t + 1] = tnode_ptr[(size_t)t] + L;
    slot_base[(size_t)t + 1] = slot_base[(size_t)t] + tn[(size_t)t].nshared;
  }
  const int64_t total = tnode_ptr[(size_t)ntiles];
  const int64_t nslots = slot_base[(size_t)ntiles];
  // Shared nodes: one partial-sum slot per (node, tile), numbered in tile order;
  // the boundary pass reads each node's partials as one contiguous run in
  // ascending tile order, so positions are grouped by node (counting sort over
  // the slots in tile order keeps tiles ascending within a node).
  std::vector<int> slot_node((size_t)nslots);
  std::vector<int> tnodes((size_t)total), tout((size_t)total);
  std::vector<uint16_t> tloc((size_t)total);
  std::vector<uint16_t> tadj_ptr((size_t)(total + ntiles));
  host_parallel(ntiles, [&](int64_t t0, int64_t t1) {
    for (int64_t t = t0; t < t1; ++t) {
      const TileNodes& o = tn[(size_t)t];
      const int64_t n0 = tnode_ptr[(size_t)t];
      int64_t sl = slot_base[(size_t)t];
      for (size_t j = 0; j < o.loc.size(); ++j) {
        tnodes[(size_t)(n0 + j)] = o.asc[j];
        tloc[(size_t)(n0 + j)] = o.asc_loc[j];
        if (o.shared[j]) slot_node[(size_t)sl++] = o.loc[j];
      }
      for (size_t j = 0; j < o.ptr.size(); ++j) tadj_ptr[(size_t)(n0 + t + j)] = o.ptr[j];
    }
  });
  std::vector<int> bcnt((size_t)N + 1, 0);   // slots per node (relaxed atomic counts)
  host_parallel(nslots, [&](int64_t s0, int64_t s1) {
    for (int64_t s2 = s0; s2 < s1; ++s2)
      __atomic_fetch_add(&bcnt[(size_t)slot_node[(size_t)s2] + 1], 1, __ATOMIC_RELAXED);
  });
  std::vector<int> bnodes, bptr(1, 0), bidx((size_t)N, -1);
  for (int64_t g = 0; g < N; ++g)
    if (bcnt[(size_t)g + 1] > 0) {
      bidx[(size_t)g] = (int)bnodes.size();
      bnodes.push_back((int)g);
      bptr.push_back(bptr.back() + bcnt[(size_t)g + 1]);
    }
  std::vector<int> pos_of_slot((size_t)nslots, 0), fill(bptr.begin(), bptr.end() - 1);
  for (int64_t s2 = 0; s2 < nslots; ++s2) pos_of_slot[(size_t)s2] = fill[(size_t)bidx[(size_t)slot_node[(size_t)s2]]]++;
  host_parallel(ntiles, [&](int64_t t0, int64_t t1) {
    for (int64_t t = t0; t < t1; ++t) {
      const TileNodes& o = tn[(size_t)t];
      const int64_t n0 = tnode_ptr[(size_t)t];
      int64_t sl = slot_base[(size_t)t];
      for (size_t j = 0; j < o.loc.size(); ++j)
        tout[(size_t)(n0 + j)] = o.shared[j] ? -1 - pos_of_slot[(size_t)sl++] : o.loc[j];
    }
  });
  std::vector<TileNodes>().swap(tn);

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
  if ((rc = up(&c->tloc, tloc))) return rc;
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

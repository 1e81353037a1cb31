// Host-side setup (H1): sparsity pattern, distance-2 colouring, element colouring,
// node incidence and the element-block plan used by the assembly kernels.
//
// Reference: tatva/sparse/_extraction.py _create_sparse_structure (:37-87) and
// pattern_from_mesh (:90-102); tatva/sparse/_coloring.py get_distance2_adjacency
// (:27-48), greedy_coloring (:136-153), distance2_colors (:270-283).  The reference
// pins tatva_coloring.distance2_colors (external, tatva/sparse/base.py:32,66); the
// in-repo natural-order greedy restated here is the one this project reproduces
// bit for bit.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <numeric>
#include <thread>
#include <vector>

#include "tatva_gb300.h"

namespace tg {
int set_error(int code, const char* fmt, ...);
}
using tg::set_error;

namespace {

template <class F>
void parallel_for(int64_t n, F&& f) {
  unsigned hc = std::thread::hardware_concurrency();
  int nt = (int)(hc == 0 ? 1 : (hc > 32 ? 32 : hc));
  if (n < 8192 || nt <= 1) {
    f(0, n, 0);
    return;
  }
  const int64_t chunk = (n + nt - 1) / nt;
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t) {
    const int64_t a = t * chunk, b = std::min<int64_t>(n, a + chunk);
    if (a >= b) break;
    th.emplace_back([&, a, b, t] { f(a, b, t); });
  }
  for (auto& x : th) x.join();
}

int nthreads() {
  unsigned hc = std::thread::hardware_concurrency();
  return (int)(hc == 0 ? 1 : (hc > 32 ? 32 : hc));
}

int check_conn(const int32_t* conn, int64_t n_elems, int npe, int64_t n_nodes) {
  if (!conn && n_elems > 0) return set_error(TG_ERR_VALUE, "conn must not be NULL");
  if (n_elems < 0 || n_nodes < 0 || npe <= 0) return set_error(TG_ERR_VALUE, "bad mesh sizes");
  if (n_nodes > INT32_MAX || n_elems * npe > INT32_MAX)
    return set_error(TG_ERR_VALUE, "mesh too large for int32 indexing");
  for (int64_t k = 0; k < n_elems * npe; ++k) {
    if (conn[k] < 0) return set_error(TG_ERR_VALUE, "Mesh element connectivity contains negative node indices.");
    if (conn[k] >= n_nodes)
      return set_error(TG_ERR_VALUE,
                       "Mesh element connectivity references nodes outside the mesh coordinates array.");
  }
  return TG_OK;
}

// node -> incident (e*npe + a), ascending e
void incidence(const int32_t* conn, int64_t n_elems, int npe, int64_t n_nodes,
               std::vector<int32_t>& ptr, std::vector<int32_t>& idx) {
  ptr.assign(n_nodes + 1, 0);
  for (int64_t k = 0; k < n_elems * npe; ++k) ptr[conn[k] + 1]++;
  for (int64_t i = 0; i < n_nodes; ++i) ptr[i + 1] += ptr[i];
  idx.resize(n_elems * npe);
  std::vector<int32_t> pos(ptr.begin(), ptr.end() - 1);
  for (int64_t k = 0; k < n_elems * npe; ++k) idx[pos[conn[k]]++] = (int32_t)k;
}

struct Pattern {
  int64_t n_rows = 0;
  std::vector<int32_t> indptr;
  std::vector<int32_t> indices;
};

struct Plan {
  int32_t n_blocks = 0, n_elems = 0, npad = 4, max_local = 0, max_colors = 0, n_affine = 0,
          n_diag = 0, max_elems = 0, n_lattice = 0;
  std::vector<int32_t> blk_elem_ptr, blk_color_ptr, color_ofs, blk_node_ptr, elem_id, lnode_gid,
      lnode_slot, lnode_smem, shared_node, shared_ptr, shared_slots;
  std::vector<uint16_t> lconn;
};

uint64_t spread3(uint64_t x) {  // 21 bits -> every third bit
  x &= 0x1fffff;
  x = (x | x << 32) & 0x1f00000000ffffULL;
  x = (x | x << 16) & 0x1f0000ff0000ffULL;
  x = (x | x << 8) & 0x100f00f00f00f00fULL;
  x = (x | x << 4) & 0x10c30c30c30c30c3ULL;
  x = (x | x << 2) & 0x1249249249249249ULL;
  return x;
}
uint64_t spread2(uint64_t x) {  // 31 bits -> every second bit
  x &= 0x7fffffff;
  x = (x | x << 16) & 0x0000ffff0000ffffULL;
  x = (x | x << 8) & 0x00ff00ff00ff00ffULL;
  x = (x | x << 4) & 0x0f0f0f0f0f0f0f0fULL;
  x = (x | x << 2) & 0x3333333333333333ULL;
  x = (x | x << 1) & 0x5555555555555555ULL;
  return x;
}

// Exact parallelepiped test of a Hex8 element in precision T, replaying the
// device's 8-point butterfly on the coordinates (additions only, so the host and
// the GPU produce identical bits): the bilinear and trilinear modes must vanish.
template <class T>
bool hex_affine_exact(const double* coords, const int32_t* nodes) {
  static const int tmap[8] = {0, 1, 3, 2, 4, 5, 7, 6};
  for (int k = 0; k < 3; ++k) {
    volatile T m[8];
    for (int a = 0; a < 8; ++a) m[tmap[a]] = (T)coords[(int64_t)nodes[a] * 3 + k];
    for (int h = 1; h < 8; h <<= 1)
      for (int t = 0; t < 8; ++t)
        if (!(t & h)) {
          const T a = m[t], b = m[t | h];
          m[t] = b + a;
          m[t | h] = b - a;
        }
    if (m[3] != T(0) || m[5] != T(0) || m[6] != T(0) || m[7] != T(0)) return false;
  }
  return true;
}

// Axis-aligned box test in precision T: the edge vectors at node 0 (x1 - x0, x3 - x0,
// x4 - x0, one subtraction each, as on the device) have exact zeros off their axis.
template <class T>
bool hex_box_exact(const double* coords, const int32_t* nodes) {
  const int ed[3] = {1, 3, 4};
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) {
      if (k == i) continue;
      const T a = (T)coords[(int64_t)nodes[ed[i]] * 3 + k];
      const T b = (T)coords[(int64_t)nodes[0] * 3 + k];
      if (a - b != T(0)) return false;
    }
  return true;
}

// Lattice blocks: 8 x 8 x 8 Hex8 boxes on a 9 x 9 x 9 grid of nodes.
constexpr int LAT_N = 8, LAT_NN = LAT_N + 1, LAT_NODES = LAT_NN * LAT_NN * LAT_NN;

// Grid positions of a block's nodes: lat[l] = ix + 9 iy + 81 iz for node ids[l] when
// the nodes' coordinates take exactly 9 distinct values per axis and fill the 9 x 9 x 9
// grid once; false otherwise.
bool lattice_positions(const double* coords, const std::vector<int32_t>& ids,
                       std::vector<int32_t>& lat) {
  if ((int)ids.size() != LAT_NODES) return false;
  std::vector<double> ax[3];
  for (int d = 0; d < 3; ++d) {
    ax[d].reserve(ids.size());
    for (int32_t g : ids) ax[d].push_back(coords[(int64_t)g * 3 + d]);
    std::sort(ax[d].begin(), ax[d].end());
    ax[d].erase(std::unique(ax[d].begin(), ax[d].end()), ax[d].end());
    if ((int)ax[d].size() != LAT_NN) return false;
  }
  lat.assign(ids.size(), -1);
  std::vector<char> seen(LAT_NODES, 0);
  for (size_t l = 0; l < ids.size(); ++l) {
    int p = 0;
    for (int d = 2; d >= 0; --d) {
      const double x = coords[(int64_t)ids[l] * 3 + d];
      p = p * LAT_NN + (int)(std::lower_bound(ax[d].begin(), ax[d].end(), x) - ax[d].begin());
    }
    if (seen[p]) return false;
    seen[p] = 1;
    lat[l] = p;
  }
  return true;
}

// Lattice test of a Hex8 box block (elements key[k0, k1)): 512 elements whose node a
// sits at grid offset (dx, dy, dz)_a = (0,0,0) (1,0,0) (1,1,0) (0,1,0) (0,0,1) (1,0,1)
// (1,1,1) (0,1,1) from node 0, one element per grid cell.
bool hex_block_lattice(const double* coords, const int32_t* conn,
                       const std::vector<std::pair<uint64_t, int32_t>>& key, int32_t k0,
                       int32_t k1) {
  if (k1 - k0 != LAT_N * LAT_N * LAT_N) return false;
  std::vector<int32_t> ids;
  ids.reserve((size_t)(k1 - k0) * 8);
  for (int32_t k = k0; k < k1; ++k)
    for (int a = 0; a < 8; ++a) ids.push_back(conn[(int64_t)key[k].second * 8 + a]);
  std::sort(ids.begin(), ids.end());
  ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
  std::vector<int32_t> lat;
  if (!lattice_positions(coords, ids, lat)) return false;
  static const int off[8] = {0, 1, 1 + LAT_NN, LAT_NN, LAT_NN * LAT_NN, 1 + LAT_NN * LAT_NN,
                             1 + LAT_NN + LAT_NN * LAT_NN, LAT_NN + LAT_NN * LAT_NN};
  std::vector<char> cell(LAT_N * LAT_N * LAT_N, 0);
  for (int32_t k = k0; k < k1; ++k) {
    const int32_t* nodes = conn + (int64_t)key[k].second * 8;
    int p[8];
    for (int a = 0; a < 8; ++a)
      p[a] = lat[std::lower_bound(ids.begin(), ids.end(), nodes[a]) - ids.begin()];
    const int ix = p[0] % LAT_NN, iy = (p[0] / LAT_NN) % LAT_NN, iz = p[0] / (LAT_NN * LAT_NN);
    if (ix >= LAT_N || iy >= LAT_N || iz >= LAT_N) return false;
    for (int a = 1; a < 8; ++a)
      if (p[a] != p[0] + off[a]) return false;
    char& c = cell[ix + LAT_N * (iy + LAT_N * iz)];
    if (c) return false;
    c = 1;
  }
  return true;
}

// Shared-memory slots of a block's local nodes for the affine Hex8 kernels, whose node
// records are 16 bytes (one vector access per node).  Consecutive element positions run on
// consecutive threads, so every run of 8 positions is one quarter-warp: the nodes it
// reads at one element corner should sit in distinct 16-byte bank quads (slot % 8).
// The same holds for every run of 8 consecutive local nodes, which one warp
// instruction copies into shared memory.  Greedy capacity-constrained 8-colouring of
// both kinds of groups, nodes in order of first use; slot = quad + 8 * (rank within
// quad) < 8 ceil(nl / 8).
void bank_aware_slots(const std::vector<int32_t>& lc_sorted, int npe, int ne, int nl,
                      std::vector<int32_t>& slot) {
  const int ng = ((ne + 7) / 8) * npe;
  std::vector<int32_t> gptr(ng + 1, 0), gidx;
  gidx.reserve((size_t)ne * npe);
  for (int g0 = 0, gi = 0; g0 < ne; g0 += 8)
    for (int c = 0; c < npe; ++c, ++gi) {
      for (int k = g0; k < std::min(ne, g0 + 8); ++k) gidx.push_back(lc_sorted[(size_t)k * npe + c]);
      gptr[gi + 1] = (int32_t)gidx.size();
    }
  std::vector<int32_t> nptr(nl + 1, 0), nidx(gidx.size());
  for (int32_t v : gidx) nptr[v + 1]++;
  for (int i = 0; i < nl; ++i) nptr[i + 1] += nptr[i];
  {
    std::vector<int32_t> pos(nptr.begin(), nptr.end() - 1);
    for (int gi = 0; gi < ng; ++gi)
      for (int k = gptr[gi]; k < gptr[gi + 1]; ++k) nidx[pos[gidx[k]]++] = gi;
  }
  const int cap = (nl + 7) / 8;
  std::vector<int> quad(nl, -1), used(8, 0);
  std::vector<char> seen(nl, 0);
  std::vector<int32_t> order;
  order.reserve(nl);
  for (int32_t v : gidx)
    if (!seen[v]) { seen[v] = 1; order.push_back(v); }
  for (int v = 0; v < nl; ++v)
    if (!seen[v]) order.push_back(v);
  for (int32_t v : order) {
    int cost[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = nptr[v]; k < nptr[v + 1]; ++k) {
      const int gi = nidx[k];
      for (int j = gptr[gi]; j < gptr[gi + 1]; ++j) {
        const int o = gidx[j];
        if (o != v && quad[o] >= 0) cost[quad[o]]++;
      }
    }
    // staging group: the 8 consecutive local nodes that one warp instruction copies
    for (int o = v & ~7; o < std::min(nl, (v & ~7) + 8); ++o)
      if (o != v && quad[o] >= 0) cost[quad[o]]++;
    int best = -1;
    for (int qd = 0; qd < 8; ++qd)
      if (used[qd] < cap && (best < 0 || cost[qd] < cost[best])) best = qd;
    quad[v] = best;
    used[best]++;
  }
  int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  slot.assign(nl, 0);
  for (int v = 0; v < nl; ++v) slot[v] = quad[v] + 8 * cnt[quad[v]]++;
}

// Shared-memory slots for the general block kernel, whose node records are scalar
// words (word d of a node at slot * stride + d, stride 1-3 and odd for every 3-D
// law): the 32 lanes of a warp are one wavefront, free of bank conflicts when their
// slots differ modulo 32.  Groups are every run of 32 element positions at one
// corner (one warp's load or add) and every run of 32 consecutive local nodes (one
// warp's staging or write-back).  Greedy capacity-constrained 32-colouring, the nodes
// in most groups first (ties in order of first use); class r holds the slots
// r, r + 32, ... below 8 ceil(nl / 8), so the shared-memory bound does not change.
void bank_aware_slots32(const std::vector<int32_t>& lc_sorted, int npe, int ne, int nl,
                        std::vector<int32_t>& slot) {
  constexpr int W = 32;
  const int ng_e = ((ne + W - 1) / W) * npe, ng = ng_e + (nl + W - 1) / W;
  std::vector<int32_t> gptr(ng + 1, 0), gidx;
  gidx.reserve((size_t)ne * npe + nl);
  int gi = 0;
  for (int g0 = 0; g0 < ne; g0 += W)
    for (int c = 0; c < npe; ++c, ++gi) {
      for (int k = g0; k < std::min(ne, g0 + W); ++k) gidx.push_back(lc_sorted[(size_t)k * npe + c]);
      gptr[gi + 1] = (int32_t)gidx.size();
    }
  for (int s0 = 0; s0 < nl; s0 += W, ++gi) {
    for (int v = s0; v < std::min(nl, s0 + W); ++v) gidx.push_back(v);
    gptr[gi + 1] = (int32_t)gidx.size();
  }
  std::vector<int32_t> nptr(nl + 1, 0), nidx(gidx.size());
  for (int32_t v : gidx) nptr[v + 1]++;
  for (int i = 0; i < nl; ++i) nptr[i + 1] += nptr[i];
  {
    std::vector<int32_t> pos(nptr.begin(), nptr.end() - 1);
    for (int g = 0; g < ng; ++g)
      for (int k = gptr[g]; k < gptr[g + 1]; ++k) nidx[pos[gidx[k]]++] = g;
  }
  std::vector<int32_t> order;
  order.reserve(nl);
  {
    std::vector<char> seen(nl, 0);
    for (int32_t v : gidx)
      if (!seen[v]) { seen[v] = 1; order.push_back(v); }
  }
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
    return nptr[a + 1] - nptr[a] > nptr[b + 1] - nptr[b];
  });
  const int nl8 = (nl + 7) & ~7;
  int cap[W], used[W] = {};
  for (int r = 0; r < W; ++r) cap[r] = r < nl8 ? (nl8 - r + W - 1) / W : 0;
  std::vector<int> cls(nl, -1);
  // hist[g * W + r]: members of group g already placed in class r (a node listed twice
  // in a group counts twice, as it would when the members were walked)
  std::vector<int32_t> hist((size_t)ng * W, 0);
  for (int32_t v : order) {
    int cost[W] = {};
    for (int k = nptr[v]; k < nptr[v + 1]; ++k) {
      const int32_t* h = hist.data() + (size_t)nidx[k] * W;
      for (int r = 0; r < W; ++r) cost[r] += h[r];
    }
    int best = -1;
    for (int r = 0; r < W; ++r)
      if (used[r] < cap[r] && (best < 0 || cost[r] < cost[best])) best = r;
    cls[v] = best;
    used[best]++;
    for (int k = nptr[v]; k < nptr[v + 1]; ++k) hist[(size_t)nidx[k] * W + best]++;
  }
  int cnt[W] = {};
  slot.assign(nl, 0);
  for (int v = 0; v < nl; ++v) slot[v] = cls[v] + W * cnt[cls[v]]++;
}

}  // namespace

// ============================================================================ pattern
extern "C" int tg_pattern_build(const int32_t* conn, int64_t n_elems, int npe, int64_t n_nodes,
                                int ndpn, void** handle) {
  if (!handle) return set_error(TG_ERR_VALUE, "handle must not be NULL");
  *handle = nullptr;
  if (ndpn <= 0) return set_error(TG_ERR_VALUE, "n_dofs_per_node must be positive");
  int rc = check_conn(conn, n_elems, npe, n_nodes);
  if (rc) return rc;
  try {
    std::vector<int32_t> iptr, iidx;
    incidence(conn, n_elems, npe, n_nodes, iptr, iidx);
    // node adjacency (sorted, unique, includes the node itself)
    std::vector<int64_t> cnt(n_nodes + 1, 0);
    const int nt = nthreads();
    std::vector<std::vector<int32_t>> marks(nt);
    parallel_for(n_nodes, [&](int64_t a, int64_t b, int t) {
      auto& mark = marks[t];
      mark.assign(n_nodes, -1);
      for (int64_t p = a; p < b; ++p) {
        int64_t c = 0;
        for (int k = iptr[p]; k < iptr[p + 1]; ++k) {
          const int64_t e = iidx[k] / npe;
          for (int j = 0; j < npe; ++j) {
            const int32_t q = conn[e * npe + j];
            if (mark[q] != (int32_t)p) { mark[q] = (int32_t)p; ++c; }
          }
        }
        cnt[p + 1] = c;
      }
    });
    std::vector<int64_t> nptr(n_nodes + 1, 0);
    for (int64_t p = 0; p < n_nodes; ++p) nptr[p + 1] = nptr[p] + cnt[p + 1];
    std::vector<int32_t> nadj(nptr[n_nodes]);
    parallel_for(n_nodes, [&](int64_t a, int64_t b, int t) {
      auto& mark = marks[t];
      std::fill(mark.begin(), mark.end(), -1);
      for (int64_t p = a; p < b; ++p) {
        int64_t o = nptr[p];
        for (int k = iptr[p]; k < iptr[p + 1]; ++k) {
          const int64_t e = iidx[k] / npe;
          for (int j = 0; j < npe; ++j) {
            const int32_t q = conn[e * npe + j];
            if (mark[q] != (int32_t)p) { mark[q] = (int32_t)p; nadj[o++] = q; }
          }
        }
        std::sort(nadj.begin() + nptr[p], nadj.begin() + nptr[p + 1]);
      }
    });
    marks.clear();
    const int64_t n_rows = n_nodes * ndpn;
    int64_t nnz = 0;
    for (int64_t p = 0; p < n_nodes; ++p) nnz += (nptr[p + 1] - nptr[p]) * ndpn * ndpn;
    if (nnz > INT32_MAX || n_rows > INT32_MAX)
      return set_error(TG_ERR_VALUE, "pattern has more than 2^31-1 entries");
    auto* P = new Pattern();
    P->n_rows = n_rows;
    P->indptr.resize(n_rows + 1);
    P->indices.resize(nnz);
    P->indptr[0] = 0;
    for (int64_t p = 0; p < n_nodes; ++p) {
      const int32_t len = (int32_t)((nptr[p + 1] - nptr[p]) * ndpn);
      for (int c = 0; c < ndpn; ++c) P->indptr[p * ndpn + c + 1] = P->indptr[p * ndpn + c] + len;
    }
    parallel_for(n_nodes, [&](int64_t a, int64_t b, int) {
      for (int64_t p = a; p < b; ++p)
        for (int c = 0; c < ndpn; ++c) {
          int64_t o = P->indptr[p * ndpn + c];
          for (int64_t k = nptr[p]; k < nptr[p + 1]; ++k)
            for (int d = 0; d < ndpn; ++d) P->indices[o++] = (int32_t)((int64_t)nadj[k] * ndpn + d);
        }
    });
    *handle = P;
  } catch (const std::bad_alloc&) {
    return set_error(TG_ERR_VALUE, "tg_pattern_build: out of host memory");
  }
  return TG_OK;
}

extern "C" int tg_pattern_nnz(const void* handle, int64_t* nnz) {
  if (!handle || !nnz) return set_error(TG_ERR_VALUE, "NULL argument");
  *nnz = (int64_t)static_cast<const Pattern*>(handle)->indices.size();
  return TG_OK;
}

extern "C" int tg_pattern_export(const void* handle, int32_t* indptr, int32_t* indices) {
  if (!handle) return set_error(TG_ERR_VALUE, "NULL handle");
  const Pattern* P = static_cast<const Pattern*>(handle);
  if (indptr) std::memcpy(indptr, P->indptr.data(), P->indptr.size() * sizeof(int32_t));
  if (indices) std::memcpy(indices, P->indices.data(), P->indices.size() * sizeof(int32_t));
  return TG_OK;
}

extern "C" void tg_pattern_free(void* handle) { delete static_cast<Pattern*>(handle); }

// ============================================================================ colouring
// Natural-order greedy over A @ A neighbourhoods.  Rows with identical column lists
// ("groups", e.g. the ndpn dofs of one node) share their distance-2 neighbourhood;
// each neighbourhood is scanned once per group and the group's rows are then
// coloured in order, adding a freshly used colour to the forbidden set exactly when
// that row lies in the neighbourhood -- the same result as scanning row by row.
extern "C" int tg_distance2_colors(const int32_t* indptr, const int32_t* indices, int64_t n,
                                   int32_t* colors, int32_t* n_colors) {
  if (n < 0) return set_error(TG_ERR_VALUE, "negative size");
  if (n == 0) {
    if (n_colors) *n_colors = 0;
    return TG_OK;
  }
  if (!indptr || !indices || !colors) return set_error(TG_ERR_VALUE, "NULL argument");
  for (int64_t i = 0; i < n; ++i)
    if (indptr[i + 1] < indptr[i]) return set_error(TG_ERR_VALUE, "indptr is not monotone");
  const int64_t nnz = indptr[n];
  for (int64_t k = 0; k < nnz; ++k)
    if (indices[k] < 0 || indices[k] >= n) return set_error(TG_ERR_VALUE, "column index out of range");
  try {
    std::vector<int32_t> group_of(n), group_rep;
    group_rep.reserve(n / 2 + 1);
    for (int64_t i = 0; i < n; ++i) {
      bool same = false;
      if (i > 0) {
        const int32_t l0 = indptr[i] - indptr[i - 1], l1 = indptr[i + 1] - indptr[i];
        same = (l0 == l1) && std::memcmp(indices + indptr[i - 1], indices + indptr[i],
                                         sizeof(int32_t) * l1) == 0;
      }
      if (!same) group_rep.push_back((int32_t)i);
      group_of[i] = (int32_t)group_rep.size() - 1;
    }
    const int64_t ng = (int64_t)group_rep.size();
    std::vector<int32_t> gseen(ng, -1), visited(n, -1), used;
    used.reserve(256);
    for (int64_t i = 0; i < n; ++i) colors[i] = -1;
    int32_t maxc = -1;
    for (int64_t g = 0; g < ng; ++g) {
      const int32_t stamp = (int32_t)g;
      const int32_t r0 = group_rep[g];
      const int32_t r1 = (g + 1 < ng) ? group_rep[g + 1] : (int32_t)n;
      for (int32_t k = indptr[r0]; k < indptr[r0 + 1]; ++k) {
        const int32_t j = indices[k];
        const int32_t gj = group_of[j];
        if (gseen[gj] == stamp) continue;
        gseen[gj] = stamp;
        const int32_t rep = group_rep[gj];
        for (int32_t kk = indptr[rep]; kk < indptr[rep + 1]; ++kk) {
          const int32_t m = indices[kk];
          if (visited[m] == stamp) continue;
          visited[m] = stamp;
          const int32_t cm = colors[m];
          if (cm >= 0) {
            if ((size_t)cm >= used.size()) used.resize(cm + 1, -1);
            used[cm] = stamp;
          }
        }
      }
      for (int32_t r = r0; r < r1; ++r) {
        int32_t c = 0;
        while ((size_t)c < used.size() && used[c] == stamp) ++c;
        colors[r] = c;
        if (c > maxc) maxc = c;
        if (visited[r] == stamp) {
          if ((size_t)c >= used.size()) used.resize(c + 1, -1);
          used[c] = stamp;
        }
      }
    }
    if (n_colors) *n_colors = maxc + 1;
  } catch (const std::bad_alloc&) {
    return set_error(TG_ERR_VALUE, "tg_distance2_colors: out of host memory");
  }
  return TG_OK;
}

extern "C" int tg_element_colors(const int32_t* conn, int64_t n_elems, int npe, int64_t n_nodes,
                                 int32_t* colors, int32_t* order, int32_t* color_ptr,
                                 int32_t* n_colors) {
  int rc = check_conn(conn, n_elems, npe, n_nodes);
  if (rc) return rc;
  if (!colors || !order || !color_ptr || !n_colors) return set_error(TG_ERR_VALUE, "NULL argument");
  std::vector<uint64_t> lo(n_nodes, 0), hi(n_nodes, 0);
  int32_t maxc = -1;
  for (int64_t e = 0; e < n_elems; ++e) {
    uint64_t ml = 0, mh = 0;
    for (int a = 0; a < npe; ++a) {
      ml |= lo[conn[e * npe + a]];
      mh |= hi[conn[e * npe + a]];
    }
    int c;
    if (~ml) c = __builtin_ctzll(~ml);
    else if (~mh) c = 64 + __builtin_ctzll(~mh);
    else return set_error(TG_ERR_VALUE, "element colouring needs more than 128 colours");
    colors[e] = c;
    if (c > maxc) maxc = c;
    for (int a = 0; a < npe; ++a) {
      if (c < 64) lo[conn[e * npe + a]] |= (1ULL << c);
      else hi[conn[e * npe + a]] |= (1ULL << (c - 64));
    }
  }
  const int nc = maxc + 1;
  std::vector<int32_t> cnt(nc + 1, 0);
  for (int64_t e = 0; e < n_elems; ++e) cnt[colors[e] + 1]++;
  for (int c = 0; c < nc; ++c) cnt[c + 1] += cnt[c];
  for (int c = 0; c <= nc; ++c) color_ptr[c] = cnt[c];
  for (int64_t e = 0; e < n_elems; ++e) order[cnt[colors[e]]++] = (int32_t)e;
  *n_colors = nc;
  return TG_OK;
}

extern "C" int tg_node_incidence(const int32_t* conn, int64_t n_elems, int npe, int64_t n_nodes,
                                 int32_t* ptr, int32_t* idx) {
  int rc = check_conn(conn, n_elems, npe, n_nodes);
  if (rc) return rc;
  if (!ptr || (!idx && n_elems > 0)) return set_error(TG_ERR_VALUE, "NULL argument");
  std::vector<int32_t> p, i;
  incidence(conn, n_elems, npe, n_nodes, p, i);
  std::memcpy(ptr, p.data(), p.size() * sizeof(int32_t));
  if (!i.empty()) std::memcpy(idx, i.data(), i.size() * sizeof(int32_t));
  return TG_OK;
}

// ============================================================================ block plan
extern "C" int tg_plan_build(int elem, const int32_t* conn, int64_t n_elems, int64_t n_nodes,
                             const double* coords, int dim, int block_elems, int max_local_nodes,
                             void** handle) {
  if (!handle) return set_error(TG_ERR_VALUE, "handle must not be NULL");
  *handle = nullptr;
  int npe, npad;
  switch (elem) {
    case TG_TRI3: npe = 3; npad = 4; break;
    case TG_TET4: npe = 4; npad = 4; break;
    case TG_HEX8: npe = 8; npad = 8; break;
    default: return set_error(TG_ERR_VALUE, "unknown element type %d", elem);
  }
  if (dim != 2 && dim != 3) return set_error(TG_ERR_VALUE, "dim must be 2 or 3");
  if (block_elems <= 0) return set_error(TG_ERR_VALUE, "block_elems must be positive");
  if (max_local_nodes < npe || max_local_nodes > 65535)
    return set_error(TG_ERR_VALUE, "max_local_nodes must be in [nodes_per_elem, 65535]");
  int rc = check_conn(conn, n_elems, npe, n_nodes);
  if (rc) return rc;
  if (!coords && n_elems > 0) return set_error(TG_ERR_VALUE, "coords must not be NULL");
  try {
    auto* P = new Plan();
    P->npad = npad;
    P->n_elems = (int32_t)n_elems;
    // 1. Morton order of element centroids
    std::vector<std::pair<uint64_t, int32_t>> key(n_elems);
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    std::vector<double> cen(n_elems * dim);
    for (int64_t e = 0; e < n_elems; ++e)
      for (int d = 0; d < dim; ++d) {
        double s = 0;
        for (int a = 0; a < npe; ++a) s += coords[(int64_t)conn[e * npe + a] * dim + d];
        s /= npe;
        cen[e * dim + d] = s;
        lo[d] = std::min(lo[d], s);
        hi[d] = std::max(hi[d], s);
      }
    const double bits = (dim == 3) ? 2097151.0 : 2147483647.0;
    // Centroids on a tensor grid (a structured mesh, any spacing per axis): quantize by
    // grid index, so that runs of 8^dim Morton keys are aligned 8 x 8 (x 8) cubes.
    std::vector<double> axis[3];
    bool grid = n_elems > 0;
    {
      int64_t cells = 1;
      for (int d = 0; d < dim && grid; ++d) {
        axis[d].resize(n_elems);
        for (int64_t e = 0; e < n_elems; ++e) axis[d][e] = cen[e * dim + d];
        std::sort(axis[d].begin(), axis[d].end());
        axis[d].erase(std::unique(axis[d].begin(), axis[d].end()), axis[d].end());
        cells *= (int64_t)axis[d].size();
        // the per-axis counts of a tensor grid multiply to n_elems
        if (cells > n_elems || n_elems % cells != 0 || (double)axis[d].size() > bits) grid = false;
      }
      grid = grid && cells == n_elems;
    }
    for (int64_t e = 0; e < n_elems; ++e) {
      uint64_t code = 0;
      for (int d = 0; d < dim; ++d) {
        uint64_t qd;
        if (grid) {
          qd = (uint64_t)(std::lower_bound(axis[d].begin(), axis[d].end(), cen[e * dim + d]) -
                          axis[d].begin());
        } else {
          const double w = hi[d] - lo[d];
          const double t = w > 0 ? (cen[e * dim + d] - lo[d]) / w : 0.0;
          qd = (uint64_t)(t * bits);
        }
        code |= (dim == 3 ? spread3(qd) : spread2(qd)) << d;
      }
      key[e] = {code, (int32_t)e};
    }
    for (auto& a : axis) std::vector<double>().swap(a);
    cen.clear();
    cen.shrink_to_fit();
    std::sort(key.begin(), key.end());
    // 2. chunk into blocks (element count and local-node cap).  On a 3-D tensor grid
    // with 512-element blocks, a block also ends where the 8 x 8 x 8 Morton cube changes
    // (key >> 9), so that every full cube is one block whatever the grid's sides, and
    // the partial cubes at the far faces form blocks of their own.
    const bool cube_cuts = grid && dim == 3 && block_elems == 512;
    std::vector<int32_t> stamp(n_nodes, -1);
    P->blk_elem_ptr.push_back(0);
    std::vector<int32_t> blk_nodes;  // local node count per block
    {
      int32_t b = 0, ne = 0, nl = 0;
      for (int64_t k = 0; k < n_elems; ++k) {
        const int32_t e = key[k].second;
        int add = 0;  // upper bound on the nodes this element brings into block b
        for (int a = 0; a < npe; ++a)
          if (stamp[conn[(int64_t)e * npe + a]] != b) ++add;
        const bool new_cube = cube_cuts && k > 0 && (key[k].first >> 9) != (key[k - 1].first >> 9);
        if (ne > 0 && (ne >= block_elems || nl + add > max_local_nodes || new_cube)) {
          P->blk_elem_ptr.push_back((int32_t)k);
          blk_nodes.push_back(nl);
          ++b;
          ne = 0;
          nl = 0;
        }
        for (int a = 0; a < npe; ++a) {
          const int32_t g = conn[(int64_t)e * npe + a];
          if (stamp[g] != b) {
            stamp[g] = b;
            ++nl;
          }
        }
        ++ne;
      }
      if (ne > 0) {
        P->blk_elem_ptr.push_back((int32_t)n_elems);
        blk_nodes.push_back(nl);
      }
    }
    const int32_t nb = (int32_t)blk_nodes.size();
    P->n_blocks = nb;
    if (elem == TG_HEX8 && dim == 3 && nb > 0) {
      // 3: 8 x 8 x 8 box lattice, 2: all boxes, 1: all parallelepipeds, 0: general
      std::vector<char> kind(nb, 2);
      parallel_for(nb, [&](int64_t b0, int64_t b1, int) {
        for (int64_t b = b0; b < b1; ++b) {
          for (int32_t k = P->blk_elem_ptr[b]; k < P->blk_elem_ptr[b + 1] && kind[b]; ++k) {
            const int32_t* nodes = conn + (int64_t)key[k].second * npe;
            if (!(hex_affine_exact<double>(coords, nodes) && hex_affine_exact<float>(coords, nodes)))
              kind[b] = 0;
            else if (kind[b] == 2 &&
                     !(hex_box_exact<double>(coords, nodes) && hex_box_exact<float>(coords, nodes)))
              kind[b] = 1;
          }
          if (kind[b] == 2 &&
              hex_block_lattice(coords, conn, key, P->blk_elem_ptr[b], P->blk_elem_ptr[b + 1]))
            kind[b] = 3;
        }
      });
      std::vector<int32_t> order;
      for (int want = 3; want >= 0; --want) {
        for (int32_t b = 0; b < nb; ++b)
          if (kind[b] == want) order.push_back(b);
        if (want == 3) P->n_lattice = (int32_t)order.size();
        if (want == 2) P->n_diag = (int32_t)order.size();
        if (want == 1) P->n_affine = (int32_t)order.size();
      }
      std::vector<std::pair<uint64_t, int32_t>> key2;
      key2.reserve(n_elems);
      std::vector<int32_t> ptr2(1, 0), nodes2;
      for (int32_t b : order) {
        for (int32_t k = P->blk_elem_ptr[b]; k < P->blk_elem_ptr[b + 1]; ++k) key2.push_back(key[k]);
        ptr2.push_back((int32_t)key2.size());
        nodes2.push_back(blk_nodes[b]);
      }
      key.swap(key2);
      P->blk_elem_ptr.swap(ptr2);
      blk_nodes.swap(nodes2);
    }
    P->blk_node_ptr.assign(nb + 1, 0);
    for (int32_t b = 0; b < nb; ++b) P->blk_node_ptr[b + 1] = P->blk_node_ptr[b] + blk_nodes[b];
    const int64_t total_local = P->blk_node_ptr[nb];
    P->lnode_gid.assign(total_local, 0);
    P->lnode_slot.assign(total_local, -1);
    P->lnode_smem.assign(total_local, 0);
    P->elem_id.assign(n_elems, 0);
    P->lconn.assign(n_elems * npad, 0);
    // global degree of every node
    std::vector<int32_t> deg(n_nodes, 0);
    for (int64_t k = 0; k < n_elems * npe; ++k) deg[conn[k]]++;
    // 3. per block: local numbering, in-block colouring, shared classification
    std::vector<std::vector<int32_t>> blk_colors(nb);
    std::vector<int32_t> blk_nshared(nb, 0);
    const int nt = nthreads();
    std::vector<std::vector<int32_t>> lid_t(nt), lcnt_t(nt);
    std::vector<char> overflow_t(nt, 0);
    parallel_for(nb, [&](int64_t b0, int64_t b1, int t) {
      auto& lid = lid_t[t];
      auto& lcnt = lcnt_t[t];
      lid.assign(n_nodes, -1);
      lcnt.assign(n_nodes, 0);
      std::vector<int32_t> ids, ecol, tmp_e;
      std::vector<uint16_t> tmp_c;
      std::vector<uint64_t> mlo, mhi;
      for (int64_t b = b0; b < b1; ++b) {
        const int32_t e0 = P->blk_elem_ptr[b], e1 = P->blk_elem_ptr[b + 1];
        ids.clear();
        for (int32_t k = e0; k < e1; ++k) {
          const int32_t e = key[k].second;
          for (int a = 0; a < npe; ++a) {
            const int32_t g = conn[(int64_t)e * npe + a];
            if (lcnt[g]++ == 0) ids.push_back(g);
          }
        }
        std::sort(ids.begin(), ids.end());
        if (b < P->n_lattice) {  // local node = grid position i + 9 j + 81 k
          std::vector<int32_t> lat, by_lat(ids.size());
          lattice_positions(coords, ids, lat);
          for (size_t l = 0; l < ids.size(); ++l) by_lat[lat[l]] = ids[l];
          ids.swap(by_lat);
        }
        const int32_t n0 = P->blk_node_ptr[b];
        for (size_t l = 0; l < ids.size(); ++l) lid[ids[l]] = (int32_t)l;
        // colouring in Morton order
        const int32_t ne = e1 - e0;
        ecol.assign(ne, 0);
        mlo.assign(ids.size(), 0);
        mhi.assign(ids.size(), 0);
        int32_t maxc = -1;
        for (int32_t k = 0; k < ne; ++k) {
          const int32_t e = key[e0 + k].second;
          uint64_t ml = 0, mh = 0;
          for (int a = 0; a < npe; ++a) {
            const int32_t l = lid[conn[(int64_t)e * npe + a]];
            ml |= mlo[l];
            mh |= mhi[l];
          }
          int c;
          if (~ml) c = __builtin_ctzll(~ml);
          else if (~mh) c = 64 + __builtin_ctzll(~mh);
          else { overflow_t[t] = 1; c = 127; }
          ecol[k] = c;
          maxc = std::max(maxc, c);
          for (int a = 0; a < npe; ++a) {
            const int32_t l = lid[conn[(int64_t)e * npe + a]];
            if (c < 64) mlo[l] |= 1ULL << c;
            else mhi[l] |= 1ULL << (c - 64);
          }
        }
        const int nc = maxc + 1;
        std::vector<int32_t> cofs(nc + 1, 0);
        for (int32_t k = 0; k < ne; ++k) cofs[ecol[k] + 1]++;
        for (int c = 0; c < nc; ++c) cofs[c + 1] += cofs[c];
        blk_colors[b] = cofs;
        std::vector<int32_t> pos(cofs.begin(), cofs.end() - 1);
        std::vector<int32_t> lc_sorted((size_t)ne * npe);
        for (int32_t k = 0; k < ne; ++k) {
          const int32_t e = key[e0 + k].second;
          const int32_t r = pos[ecol[k]]++;
          P->elem_id[e0 + r] = e;
          for (int a = 0; a < npe; ++a)
            lc_sorted[(size_t)r * npe + a] = lid[conn[(int64_t)e * npe + a]];
        }
        std::vector<int32_t> smem_slot;
        // affine Hex8 blocks run the kernels with 16-byte node records, every other
        // block the general kernel with scalar records
        if (b < P->n_affine)
          bank_aware_slots(lc_sorted, npe, ne, (int)ids.size(), smem_slot);
        else
          bank_aware_slots32(lc_sorted, npe, ne, (int)ids.size(), smem_slot);
        for (int32_t r = 0; r < ne; ++r) {
          const int32_t dst = e0 + r;
          for (int a = 0; a < npe; ++a)
            P->lconn[(int64_t)dst * npad + a] = (uint16_t)smem_slot[lc_sorted[(size_t)r * npe + a]];
          for (int a = npe; a < npad; ++a) P->lconn[(int64_t)dst * npad + a] = 0;
        }
        for (size_t l = 0; l < ids.size(); ++l) P->lnode_smem[n0 + l] = smem_slot[l];
        int32_t nsh = 0;
        for (size_t l = 0; l < ids.size(); ++l) {
          const int32_t g = ids[l];
          P->lnode_gid[n0 + l] = g;
          if (lcnt[g] != deg[g]) {
            P->lnode_slot[n0 + l] = -2;  // shared: slot assigned below
            ++nsh;
          }
          lcnt[g] = 0;
          lid[g] = -1;
        }
        blk_nshared[b] = nsh;
      }
    });
    lid_t.clear();
    lcnt_t.clear();
    for (char o : overflow_t)
      if (o) {
        delete P;
        return set_error(TG_ERR_VALUE, "block colouring needs more than 128 colours; use smaller blocks");
      }
    // colour offsets
    P->blk_color_ptr.assign(nb + 1, 0);
    for (int32_t b = 0; b < nb; ++b) {
      P->blk_color_ptr[b + 1] = P->blk_color_ptr[b] + (int32_t)blk_colors[b].size();
      P->max_colors = std::max<int32_t>(P->max_colors, (int32_t)blk_colors[b].size() - 1);
      P->max_local = std::max<int32_t>(P->max_local, blk_nodes[b]);
      P->max_elems = std::max<int32_t>(P->max_elems, P->blk_elem_ptr[b + 1] - P->blk_elem_ptr[b]);
    }
    P->color_ofs.reserve(P->blk_color_ptr[nb]);
    for (int32_t b = 0; b < nb; ++b)
      P->color_ofs.insert(P->color_ofs.end(), blk_colors[b].begin(), blk_colors[b].end());
    // 4. partial slots: the slots of one shared node are consecutive (its blocks in
    // block order), so the final sum over a node reads one contiguous run
    int64_t slot = 0;
    std::vector<int32_t> nshare(n_nodes, 0);
    for (int32_t b = 0; b < nb; ++b)
      for (int32_t l = P->blk_node_ptr[b]; l < P->blk_node_ptr[b + 1]; ++l)
        if (P->lnode_slot[l] == -2) {
          ++slot;
          nshare[P->lnode_gid[l]]++;
        }
    if (slot > INT32_MAX) {
      delete P;
      return set_error(TG_ERR_VALUE, "too many partial slots");
    }
    std::vector<int32_t> sidx(n_nodes, -1);
    for (int64_t g = 0; g < n_nodes; ++g)
      if (nshare[g] > 0) {
        sidx[g] = (int32_t)P->shared_node.size();
        P->shared_node.push_back((int32_t)g);
      }
    const int64_t nsh = (int64_t)P->shared_node.size();
    P->shared_ptr.assign(nsh + 1, 0);
    for (int64_t s = 0; s < nsh; ++s) P->shared_ptr[s + 1] = P->shared_ptr[s] + nshare[P->shared_node[s]];
    P->shared_slots.resize(slot);
    for (int64_t k = 0; k < slot; ++k) P->shared_slots[k] = (int32_t)k;
    std::vector<int32_t> fill(P->shared_ptr.begin(), P->shared_ptr.end() - 1);
    for (int32_t b = 0; b < nb; ++b)
      for (int32_t l = P->blk_node_ptr[b]; l < P->blk_node_ptr[b + 1]; ++l)
        if (P->lnode_slot[l] == -2) P->lnode_slot[l] = fill[sidx[P->lnode_gid[l]]]++;
    *handle = P;
  } catch (const std::bad_alloc&) {
    return set_error(TG_ERR_VALUE, "tg_plan_build: out of host memory");
  }
  return TG_OK;
}

extern "C" int tg_plan_sizes(const void* handle, int64_t* s) {
  if (!handle || !s) return set_error(TG_ERR_VALUE, "NULL argument");
  const Plan* P = static_cast<const Plan*>(handle);
  s[0] = P->n_blocks;
  s[1] = P->n_elems;
  s[2] = (int64_t)P->color_ofs.size();
  s[3] = (int64_t)P->lnode_gid.size();
  s[4] = (int64_t)P->shared_node.size();
  s[5] = (int64_t)P->shared_slots.size();
  s[6] = P->max_local;
  s[7] = P->max_colors;
  s[8] = P->npad;
  s[9] = P->n_affine;
  s[10] = P->n_diag;
  s[11] = P->max_elems;
  s[12] = P->n_lattice;
  return TG_OK;
}

extern "C" int tg_plan_export(const void* handle, int32_t* blk_elem_ptr, int32_t* blk_color_ptr,
                              int32_t* color_ofs, int32_t* blk_node_ptr, uint16_t* lconn,
                              int32_t* elem_id, int32_t* lnode_gid, int32_t* lnode_slot,
                              int32_t* lnode_smem, int32_t* shared_node, int32_t* shared_ptr,
                              int32_t* shared_slots) {
  if (!handle) return set_error(TG_ERR_VALUE, "NULL handle");
  const Plan* P = static_cast<const Plan*>(handle);
  auto cp = [](auto* dst, const auto& v) {
    if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(v[0]));
  };
  cp(blk_elem_ptr, P->blk_elem_ptr);
  cp(blk_color_ptr, P->blk_color_ptr);
  cp(color_ofs, P->color_ofs);
  cp(blk_node_ptr, P->blk_node_ptr);
  cp(lconn, P->lconn);
  cp(elem_id, P->elem_id);
  cp(lnode_gid, P->lnode_gid);
  cp(lnode_slot, P->lnode_slot);
  cp(lnode_smem, P->lnode_smem);
  cp(shared_node, P->shared_node);
  cp(shared_ptr, P->shared_ptr);
  cp(shared_slots, P->shared_slots);
  return TG_OK;
}

extern "C" void tg_plan_free(void* handle) { delete static_cast<Plan*>(handle); }

// Structured-brick test of a Hex8 mesh (see tg_grid_detect in the header).
extern "C" int tg_grid_detect(int elem, const int32_t* conn, int64_t n_elems, int64_t n_nodes,
                              const double* coords, int dim, int32_t* nodes, double* h) {
  if (!nodes || !h) return set_error(TG_ERR_VALUE, "tg_grid_detect: NULL output");
  for (int d = 0; d < 3; ++d) {
    nodes[d] = 0;
    h[d] = 0.0;
  }
  if (elem != TG_HEX8 || dim != 3 || n_elems <= 0 || n_nodes < 8 || !conn || !coords)
    return TG_OK;
  // row length: nodes 0, 1, ... share y and z until the first row ends
  const double* c = coords;
  int64_t nx = 1;
  while (nx < n_nodes && c[nx * 3 + 1] == c[1] && c[nx * 3 + 2] == c[2]) ++nx;
  int64_t nxy = nx;
  while (nxy < n_nodes && c[nxy * 3 + 2] == c[2]) nxy += nx;
  if (nx < 2 || nxy % nx != 0 || n_nodes % nxy != 0) return TG_OK;
  const int64_t ny = nxy / nx, nz = n_nodes / nxy;
  if (ny < 2 || nz < 2 || nx > INT32_MAX || ny > INT32_MAX || nz > INT32_MAX) return TG_OK;
  if ((nx - 1) * (ny - 1) * (nz - 1) != n_elems) return TG_OK;
  // grid lines, strictly increasing with uniform spacing (1e-13 relative)
  std::vector<double> X(nx), Y(ny), Z(nz);
  for (int64_t i = 0; i < nx; ++i) X[i] = c[i * 3];
  for (int64_t j = 0; j < ny; ++j) Y[j] = c[j * nx * 3 + 1];
  for (int64_t k = 0; k < nz; ++k) Z[k] = c[k * nxy * 3 + 2];
  double hh[3];
  const std::vector<double>* lines[3] = {&X, &Y, &Z};
  for (int d = 0; d < 3; ++d) {
    const std::vector<double>& L = *lines[d];
    const int64_t n = (int64_t)L.size();
    hh[d] = (L[n - 1] - L[0]) / (double)(n - 1);
    if (!(hh[d] > 0.0)) return TG_OK;
    for (int64_t i = 0; i + 1 < n; ++i)
      if (std::fabs((L[i + 1] - L[i]) - hh[d]) > 1e-13 * hh[d]) return TG_OK;
  }
  // every node on its grid position
  for (int64_t k = 0; k < nz; ++k)
    for (int64_t j = 0; j < ny; ++j)
      for (int64_t i = 0; i < nx; ++i) {
        const double* p = c + 3 * (i + nx * (j + ny * k));
        if (p[0] != X[i] || p[1] != Y[j] || p[2] != Z[k]) return TG_OK;
      }
  // every cell exactly once, corners in the reference order
  const int64_t off[8] = {0, 1, 1 + nx, nx, nxy, 1 + nxy, 1 + nx + nxy, nx + nxy};
  std::vector<char> seen((size_t)n_elems, 0);
  for (int64_t e = 0; e < n_elems; ++e) {
    const int32_t* q = conn + e * 8;
    const int64_t n0 = q[0];
    if (n0 < 0 || n0 >= n_nodes) return TG_OK;
    const int64_t i = n0 % nx, j = (n0 / nx) % ny, k = n0 / nxy;
    if (i >= nx - 1 || j >= ny - 1 || k >= nz - 1) return TG_OK;
    for (int a = 1; a < 8; ++a)
      if ((int64_t)q[a] != n0 + off[a]) return TG_OK;
    const int64_t cell = i + (nx - 1) * (j + (ny - 1) * k);
    if (seen[cell]) return TG_OK;
    seen[cell] = 1;
  }
  nodes[0] = (int32_t)nx;
  nodes[1] = (int32_t)ny;
  nodes[2] = (int32_t)nz;
  for (int d = 0; d < 3; ++d) h[d] = hh[d];
  return TG_OK;
}

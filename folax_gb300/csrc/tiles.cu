// Element tiles of the tile-local fused loss + adjoint.
//
// The reference scatters every element residual into the global vector
// (fol/loss_functions/fe_loss.py:283-310, jax.grad's transpose of the gather
// at :155-164).  The tile-local kernels instead give each thread block a
// compact group of elements (a tile) and sum the element residuals of the
// tile's nodes in shared memory; a node that lies inside one tile is
// finished there, and only the nodes shared by several tiles go through
// global memory, as one partial record per (tile, node), summed afterwards in
// ascending tile order.  Every sum has a fixed order, so results are
// deterministic and no float atomics are used.
//
// Tiles are built once per mesh on the host:
//   1. elements are sorted by the Morton code of their centroid (21 bits per
//      axis over the nodes' bounding box; ties by element id), so consecutive
//      elements are close in space (on a structured box mesh a tile of 128 is
//      an 8 x 4 x 4 brick of cells with 225 distinct nodes);
//   2. tiles are cut greedily along that order: an element joins the current
//      tile unless the tile already has kTileElems elements or the element's
//      new nodes would take it past kTileNodes distinct nodes;
//   3. per tile, its distinct nodes get local entries: nodes that need
//      partial records (they also belong to other tiles, or have more than
//      kTileRecs records in this tile) first, then the tile's own nodes, each
//      group in ascending node id;
//   4. per entry, up to kTileRecs records (a * kTileElems + element-in-tile)
//      of the tile's elements that touch the node, in ascending element then
//      corner order, padded with the index of a zero record; a node with more
//      records gets further entries (all of them partial), its first entry
//      is the one the elements load from; and the node's Dirichlet mask;
//   5. per node with partial records, its slots in ascending tile order.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "folgb_internal.cuh"

namespace folgb {

namespace {

uint64_t spread3(uint64_t v) {  // 21 bits -> every third bit
  v &= 0x1fffffULL;
  v = (v | (v << 32)) & 0x1f00000000ffffULL;
  v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
  v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
  v = (v | (v << 2)) & 0x1249249249249249ULL;
  return v;
}

template <class T>
int upload_vec(T** dst, const std::vector<T>& v) {
  const size_t n = v.empty() ? 1 : v.size();
  FOLGB_CUDA_TRY(cudaMalloc((void**)dst, n * sizeof(T)));
  if (!v.empty()) FOLGB_CUDA_TRY(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return FOLGB_OK;
}

}  // namespace

int build_tile_tables(folgb_plan* p, const std::vector<int>& conn, const double* xyz,
                      const std::vector<unsigned char>& dmask, const std::vector<unsigned char>& elem_bc) {
  const int nen = p->nen;
  const int64_t E = p->E, N = p->N;
  if (nen != 8 || E > (int64_t)INT32_MAX / nen) return FOLGB_OK;  // hex8 only; no tables otherwise
  // 1. Morton order of the element centroids
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int64_t n = 0; n < N; ++n)
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], xyz[3 * n + k]);
      hi[k] = std::max(hi[k], xyz[3 * n + k]);
    }
  std::vector<uint64_t> key(E);
  const double scale = (double)((1u << 21) - 1);
  for (int64_t e = 0; e < E; ++e) {
    double c[3] = {0, 0, 0};
    for (int a = 0; a < nen; ++a)
      for (int k = 0; k < 3; ++k) c[k] += xyz[3 * (int64_t)conn[e * nen + a] + k];
    uint64_t code = 0;
    for (int k = 0; k < 3; ++k) {
      const double ext = hi[k] - lo[k];
      double t = ext > 0 ? (c[k] / nen - lo[k]) / ext : 0.0;
      t = std::min(1.0, std::max(0.0, t));
      code |= spread3((uint64_t)(t * scale)) << k;  // x in the lowest bit
    }
    key[e] = code;
  }
  std::vector<int> order(E);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
  key.clear();
  key.shrink_to_fit();
  // 2. greedy tiles.  A local node has at most kTileRecs records per entry;
  // a node with more records in one tile gets further entries (see 4.), so
  // the cut bounds the entries: sum over nodes of ceil(records / kTileRecs).
  std::vector<int> tile_eptr{0};
  std::vector<int> stamp(N, -1), cnt(N, 0);
  int cur = 0, cur_entries = 0, cur_elems = 0;
  auto entries_added = [&](int e, bool fresh_tile) {
    // entries the element adds: corners in order, counting repeats
    int add = 0;
    int seen_n[8], seen_c[8], ns = 0;
    for (int a = 0; a < nen; ++a) {
      const int n = conn[(int64_t)e * nen + a];
      int j = 0;
      while (j < ns && seen_n[j] != n) ++j;
      if (j == ns) {
        seen_n[ns] = n;
        seen_c[ns++] = (!fresh_tile && stamp[n] == cur) ? cnt[n] : 0;
      }
      if (seen_c[j]++ % kTileRecs == 0) ++add;
    }
    return add;
  };
  for (int64_t i = 0; i < E; ++i) {
    const int e = order[i];
    int add = entries_added(e, false);
    if (cur_elems == kTileElems || cur_entries + add > kTileNodes) {
      tile_eptr.push_back((int)i);
      ++cur;
      cur_entries = 0;
      cur_elems = 0;
      add = entries_added(e, true);
    }
    for (int a = 0; a < nen; ++a) {
      const int n = conn[(int64_t)e * nen + a];
      if (stamp[n] != cur) {
        stamp[n] = cur;
        cnt[n] = 0;
      }
      cnt[n]++;
    }
    cur_entries += add;
    ++cur_elems;
  }
  tile_eptr.push_back((int)E);
  const int T = (int)tile_eptr.size() - 1;
  // tiles touching each node, and whether a node needs partial records
  // (in no tile, in several, or with several entries in its tile)
  std::vector<int> ntiles(N, 0);
  std::vector<unsigned char> partial(N, 0);
  std::fill(stamp.begin(), stamp.end(), -1);
  for (int t = 0; t < T; ++t)
    for (int i = tile_eptr[t]; i < tile_eptr[t + 1]; ++i)
      for (int a = 0; a < nen; ++a) {
        const int n = conn[(int64_t)order[i] * nen + a];
        if (stamp[n] != t) {
          stamp[n] = t;
          cnt[n] = 0;
          ntiles[n]++;
        }
        if (++cnt[n] > kTileRecs) partial[n] = 1;
      }
  for (int64_t n = 0; n < N; ++n)
    if (ntiles[n] != 1) partial[n] = 1;
  // 3.-4. local node entries, local connectivity, record lists
  std::vector<int> tile_nptr{0}, tile_bptr{0}, tn_gid;
  std::vector<unsigned> tn_info;
  std::vector<unsigned short> tn_pos;
  std::vector<unsigned char> t_lconn((size_t)E * nen);
  std::vector<int> local(N, -1), nodes;
  std::fill(stamp.begin(), stamp.end(), -1);
  std::vector<int> node_slot_count(N, 0);
  for (int t = 0; t < T; ++t) {
    nodes.clear();
    const int e0 = tile_eptr[t], ne = tile_eptr[t + 1] - e0;
    for (int j = 0; j < ne; ++j)
      for (int a = 0; a < nen; ++a) {
        const int n = conn[(int64_t)order[e0 + j] * nen + a];
        if (stamp[n] != t) {
          stamp[n] = t;
          nodes.push_back(n);
        }
      }
    std::sort(nodes.begin(), nodes.end(), [&](int a, int b) {
      return partial[a] != partial[b] ? partial[a] > partial[b] : a < b;
    });
    const int nn = (int)nodes.size();
    for (int k = 0; k < nn; ++k) local[nodes[k]] = k;
    // records of each distinct node, ascending element-in-tile then corner
    std::vector<std::vector<unsigned short>> nrec(nn);
    for (int j = 0; j < ne; ++j)
      for (int a = 0; a < nen; ++a) {
        const int k = local[conn[(int64_t)order[e0 + j] * nen + a]];
        nrec[k].push_back((unsigned short)(a * kTileElems + j));
      }
    // entries: a node's records in chunks of kTileRecs; the first entry is
    // the one the elements load from
    std::vector<int> primary(nn);
    int nl = 0, nb = 0;
    for (int k = 0; k < nn; ++k) {
      const int n = nodes[k];
      const int chunks = std::max(1, (int)((nrec[k].size() + kTileRecs - 1) / kTileRecs));
      primary[k] = nl;
      for (int c = 0; c < chunks; ++c) {
        tn_gid.push_back(n);
        tn_info.push_back((unsigned)dmask[n] << 16);
        for (int r = 0; r < kTileRecs; ++r) {
          const size_t q = (size_t)c * kTileRecs + r;
          tn_pos.push_back(q < nrec[k].size() ? nrec[k][q] : (unsigned short)kTileZeroRec);
        }
        ++nl;
        if (partial[n]) {
          ++nb;
          node_slot_count[n]++;
        }
      }
    }
    if (nl > kTileNodes) return FOLGB_ERR_INVALID_ARGUMENT;  // cannot happen: tiles are cut before
    for (int j = 0; j < ne; ++j)
      for (int a = 0; a < nen; ++a)
        t_lconn[(size_t)(e0 + j) * nen + a] =
            (unsigned char)primary[local[conn[(int64_t)order[e0 + j] * nen + a]]];
    tile_nptr.push_back(tile_nptr.back() + nl);
    tile_bptr.push_back(tile_bptr.back() + nb);
  }
  // 5. nodes with partial records, their slots in tile order (entries in order)
  const int64_t S = tile_bptr.back();
  std::vector<int> bn_node, bn_ptr{0}, bn_slot(S), in_node;
  for (int64_t n = 0; n < N; ++n) {
    if (!partial[n]) {
      in_node.push_back((int)n);
    } else {
      bn_node.push_back((int)n);
      bn_ptr.push_back(bn_ptr.back() + node_slot_count[n]);
    }
  }
  std::vector<int> node_pos(N, -1);
  for (size_t i = 0; i < bn_node.size(); ++i) node_pos[bn_node[i]] = bn_ptr[i];
  for (int t = 0; t < T; ++t) {
    const int n0 = tile_nptr[t], nb = tile_bptr[t + 1] - tile_bptr[t];
    for (int k = 0; k < nb; ++k) bn_slot[node_pos[tn_gid[n0 + k]]++] = tile_bptr[t] + k;
  }
  // element ids in tile order; bit 31: the element touches a Dirichlet dof
  std::vector<int> t_elem(E);
  for (int64_t i = 0; i < E; ++i) t_elem[i] = order[i] | (elem_bc[order[i]] ? (int)0x80000000u : 0);
  int rc;
  if ((rc = upload_vec(&p->d_tile_eptr, tile_eptr)) || (rc = upload_vec(&p->d_tile_nptr, tile_nptr)) ||
      (rc = upload_vec(&p->d_tile_bptr, tile_bptr)) || (rc = upload_vec(&p->d_t_elem, t_elem)) ||
      (rc = upload_vec(&p->d_t_lconn, t_lconn)) || (rc = upload_vec(&p->d_tn_pos, tn_pos)) ||
      (rc = upload_vec(&p->d_tn_gid, tn_gid)) || (rc = upload_vec(&p->d_tn_info, tn_info)) ||
      (rc = upload_vec(&p->d_bn_node, bn_node)) || (rc = upload_vec(&p->d_bn_ptr, bn_ptr)) ||
      (rc = upload_vec(&p->d_bn_slot, bn_slot)) || (rc = upload_vec(&p->d_in_node, in_node))) {
    free_tile_tables(p);
    return rc;
  }
  p->tiles = T;
  p->tile_local_nodes = (int64_t)tn_gid.size();
  p->tile_boundary_slots = S;
  p->tile_boundary_nodes = (int64_t)bn_node.size();
  p->tile_interior_nodes = (int64_t)in_node.size();
  return FOLGB_OK;
}

void free_tile_tables(folgb_plan* p) {
  void* ptrs[] = {p->d_tile_eptr, p->d_tile_nptr, p->d_tile_bptr, p->d_t_elem, p->d_t_lconn, p->d_tn_pos,
                  p->d_tn_gid,    p->d_tn_info,   p->d_bn_node,   p->d_bn_ptr, p->d_bn_slot, p->d_in_node};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  p->d_tile_eptr = p->d_tile_nptr = p->d_tile_bptr = p->d_t_elem = nullptr;
  p->d_t_lconn = nullptr;
  p->d_tn_pos = nullptr;
  p->d_tn_info = nullptr;
  p->d_tn_gid = p->d_bn_node = p->d_bn_ptr = p->d_bn_slot = p->d_in_node = nullptr;
  p->tiles = 0;
}

}  // namespace folgb

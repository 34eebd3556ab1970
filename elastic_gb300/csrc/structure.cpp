// Host-side structure of the solve path: node graph, RCM permutation,
// equation numbering and the lower CSRC pattern (all bit-identical to the
// reference's), plus what the GPU kernels need beyond the reference's
// arrays: the tiled transposed index of the SpMV, an element colouring and
// the per-element slot map used by the assembly kernels.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <numeric>
#include <thread>

#include "elx_internal.h"

namespace elx {

namespace {

// Runs f(begin, end) over [0, n) in contiguous chunks on up to 16 threads,
// with at least min_chunk items per thread (small meshes run on the calling
// thread alone).  f must not throw.
template <class F>
void parallel_chunks(int64_t n, int64_t min_chunk, F &&f) {
  int64_t nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  nt = std::min<int64_t>(nt, n / std::max<int64_t>(1, min_chunk));
  if (nt <= 1) {
    if (n > 0) f((int64_t)0, n);
    return;
  }
  const int64_t per = (n + nt - 1) / nt;
  std::vector<std::thread> th;
  for (int64_t w = 1; w < nt; w++) {
    const int64_t b = w * per, e = std::min(n, b + per);
    if (b < e) th.emplace_back([&f, b, e] { f(b, e); });
  }
  f((int64_t)0, std::min(n, per));
  for (auto &t : th) t.join();
}

}  // namespace

int elem_nodes(int iel) {
  switch (iel) {
    case TRIA3_STRAIN:
    case TRIA3_STRESS: return 3;
    case QUAD4_STRAIN:
    case QUAD4_STRESS:
    case TETRA4: return 4;
    case HEXA8: return 8;
    default: return 0;
  }
}

// Node adjacency: for every node the ascending list of distinct other nodes
// that share an element with it.  Same lists as graph/aponta/graph0/graph1
// (mef/src/Graph.f:20-208); node numbers 0 or > nnode are skipped as there.
// Output is 0-based: neighbours of node v are adj[xadj[v] .. xadj[v+1]).
void node_graph(const Mesh &m, std::vector<int32_t> &xadj, std::vector<int32_t> &adj) {
  const int nen1 = m.nen + 1;
  // every element's node pairs scattered into per-node lists (elements in
  // parallel: a list's order depends on the threads, its sorted set does not)
  std::vector<int32_t> cnt(m.nnode + 1, 0);
  parallel_chunks(m.numel, 65536, [&](int64_t e0, int64_t e1) {
    for (int64_t el = e0; el < e1; el++)
      for (int a = 0; a < m.nen; a++) {
        int no = m.ix[(size_t)el * nen1 + a];
        if (no <= 0 || no > m.nnode) continue;
        __atomic_fetch_add(&cnt[no], m.nen - 1, __ATOMIC_RELAXED);
      }
  });
  std::vector<int64_t> start(m.nnode + 1, 0);
  for (int v = 0; v < m.nnode; v++) start[v + 1] = start[v] + cnt[v + 1];
  std::vector<int32_t> raw(start[m.nnode]);
  std::vector<int64_t> fill(start.begin(), start.end() - 1);
  parallel_chunks(m.numel, 65536, [&](int64_t e0, int64_t e1) {
    for (int64_t el = e0; el < e1; el++) {
      const int32_t *c = &m.ix[(size_t)el * nen1];
      for (int a = 0; a < m.nen; a++) {
        int na = c[a];
        if (na <= 0 || na > m.nnode) continue;
        for (int b = 0; b < m.nen; b++) {
          int nb = c[b];
          if (nb <= 0 || nb > m.nnode || nb == na) continue;
          raw[__atomic_fetch_add(&fill[na - 1], (int64_t)1, __ATOMIC_RELAXED)] = nb - 1;
        }
      }
    }
  });
  // each node's list sorted and deduplicated in place, then packed
  std::vector<int32_t> nuniq(m.nnode);
  parallel_chunks(m.nnode, 8192, [&](int64_t v0, int64_t v1) {
    for (int64_t v = v0; v < v1; v++) {
      auto b = raw.begin() + start[v], e = raw.begin() + fill[v];
      std::sort(b, e);
      nuniq[v] = (int32_t)(std::unique(b, e) - b);
    }
  });
  xadj.assign(m.nnode + 1, 0);
  for (int v = 0; v < m.nnode; v++) xadj[v + 1] = xadj[v] + nuniq[v];
  adj.assign(xadj[m.nnode], 0);
  parallel_chunks(m.nnode, 8192, [&](int64_t v0, int64_t v1) {
    for (int64_t v = v0; v < v1; v++)
      std::copy(raw.begin() + start[v], raw.begin() + start[v] + nuniq[v], adj.begin() + xadj[v]);
  });
}

namespace {

// Breadth-first level structure of the masked component containing root
// (rootls, Reord.f:278-354).  Returns the number of levels; ls holds the
// nodes level by level, xls[l] the start of level l (xls[nlvl] = size).
int level_structure(int root, const std::vector<int32_t> &xadj,
                    const std::vector<int32_t> &adj, std::vector<char> &mask,
                    int32_t *ls, std::vector<int32_t> &xls) {
  mask[root] = 0;
  ls[0] = root;
  int nlvl = 0, lvl_end = 0, size = 1;
  for (;;) {
    int lvl_begin = lvl_end;
    lvl_end = size;
    xls[nlvl++] = lvl_begin;
    for (int i = lvl_begin; i < lvl_end; i++) {
      int v = ls[i];
      for (int k = xadj[v]; k < xadj[v + 1]; k++) {
        int w = adj[k];
        if (!mask[w]) continue;
        mask[w] = 0;
        ls[size++] = w;
      }
    }
    if (size == lvl_end) break;
  }
  xls[nlvl] = lvl_end;
  for (int i = 0; i < size; i++) mask[ls[i]] = 1;
  return nlvl;
}

// Pseudo-peripheral node of the masked component of root: the
// Gibbs-Poole-Stockmeyer variant of fnroot (Reord.f:101-169).  Among the
// nodes of the last level it picks the first one of strictly smallest masked
// degree, and repeats while the level count grows.
int pseudo_peripheral(int root, const std::vector<int32_t> &xadj,
                      const std::vector<int32_t> &adj, std::vector<char> &mask,
                      int32_t *ls, std::vector<int32_t> &xls) {
  int nlvl = level_structure(root, xadj, adj, mask, ls, xls);
  int size = xls[nlvl];
  if (nlvl == 1 || nlvl == size) return root;
  for (;;) {
    int first = xls[nlvl - 1];
    int mindeg = size;
    root = ls[first];
    if (size - 1 != first) {
      for (int j = first; j < size; j++) {
        int v = ls[j], deg = 0;
        for (int k = xadj[v]; k < xadj[v + 1]; k++) deg += mask[adj[k]] ? 1 : 0;
        if (deg < mindeg) {
          root = v;
          mindeg = deg;
        }
      }
    }
    int nl = level_structure(root, xadj, adj, mask, ls, xls);
    if (nl <= nlvl) return root;
    nlvl = nl;
    if (nlvl >= size) return root;
  }
}

}  // namespace

// Reverse Cuthill-McKee ordering of every connected component, components in
// the order of their lowest-numbered node, as genrcm/rcm/degree do
// (Reord.f:45-100, 170-277, 355-435): breadth first from a pseudo-peripheral
// root, the unnumbered neighbours of each node appended in adjacency order and
// then stably sorted by increasing masked degree, the component reversed at
// the end.  perm[k] = 0-based old node at new position k.
void rcm_order(int32_t n, const std::vector<int32_t> &xadj,
               const std::vector<int32_t> &adj, std::vector<int32_t> &perm) {
  perm.assign(n, 0);
  std::vector<char> mask(n, 1);
  std::vector<int32_t> xls(n + 2);
  // the masked degree the ordering sorts by (degree, Reord.f:355-435) counts
  // a node's unnumbered neighbours; a component is numbered only once all
  // of it is reached, so while it is being numbered every neighbour of its
  // nodes is unnumbered and the masked degree is the node's full degree
  auto deg = [&](int v) { return xadj[v + 1] - xadj[v]; };
  int num = 0;
  for (int i = 0; i < n && num < n; i++) {
    if (!mask[i]) continue;
    int32_t *ls = perm.data() + num;
    int root = pseudo_peripheral(i, xadj, adj, mask, ls, xls);
    // Cuthill-McKee numbering (rcm, Reord.f:170-265)
    mask[root] = 0;
    ls[0] = root;
    int last = 1;  // one past the last numbered node
    for (int h = 0; h < last; h++) {
      int v = ls[h];
      int first_new = last;
      for (int k = xadj[v]; k < xadj[v + 1]; k++) {
        int w = adj[k];
        if (!mask[w]) continue;
        mask[w] = 0;
        ls[last++] = w;
      }
      // stable insertion sort of the new neighbours by degree
      for (int a = first_new + 1; a < last; a++) {
        int w = ls[a], b = a - 1;
        const int dw = deg(w);
        while (b >= first_new && deg(ls[b]) > dw) {
          ls[b + 1] = ls[b];
          b--;
        }
        ls[b + 1] = w;
      }
    }
    std::reverse(ls, ls + last);  // the component: all `last` nodes reached
    num += last;
  }
}

// Equation numbering (numeq, Numeq.f:139-192): nodes visited in perm order,
// the free dofs of a node numbered consecutively in dof order.
// bc(ndf,nnode): nonzero = constrained.  id gets 1-based numbers, 0 = fixed.
int32_t number_equations(const Mesh &m, const std::vector<int32_t> &perm,
                         const int32_t *bc, std::vector<int32_t> &id) {
  id.assign((size_t)m.ndf * m.nnode, 0);
  int32_t neq = 0;
  for (int k = 0; k < m.nnode; k++) {
    int v = perm[k];
    for (int d = 0; d < m.ndf; d++) {
      size_t q = (size_t)v * m.ndf + d;
      id[q] = bc[q] == 0 ? ++neq : 0;
    }
  }
  return neq;
}

// Lower CSRC pattern (csrstruct/csria/csrja lower-only + sortgraph,
// Csr.f:13-305): row r holds, ascending, every equation c < r of the same
// node or of an adjacent node.  Since a node's free equations are
// consecutive and the blocks of different nodes are disjoint, each row is the
// concatenation of whole blocks of lower adjacent nodes (sorted by their
// first equation) followed by the node's own lower equations.
void csrc_pattern(const Mesh &m, const Structure &s, const std::vector<int32_t> &xadj,
                  const std::vector<int32_t> &adj, std::vector<int32_t> &ia,
                  std::vector<int32_t> &ja) {
  const int ndf = m.ndf;
  const int32_t neq = s.neq;
  std::vector<int32_t> first(m.nnode, 0), nfree(m.nnode, 0);
  for (int v = 0; v < m.nnode; v++) {
    int f = 0, c = 0;
    for (int d = 0; d < ndf; d++) {
      int q = s.id[(size_t)v * ndf + d];
      if (q > 0) {
        if (!c) f = q;
        c++;
      }
    }
    first[v] = f;
    nfree[v] = c;
  }
  ia.assign(neq + 1, 0);
  // row lengths (each node writes its own rows)
  parallel_chunks(m.nnode, 8192, [&](int64_t v0, int64_t v1) {
    for (int64_t v = v0; v < v1; v++) {
      if (!nfree[v]) continue;
      int32_t cnt = 0;
      for (int k = xadj[v]; k < xadj[v + 1]; k++) {
        int w = adj[k];
        if (nfree[w] && first[w] < first[v]) cnt += nfree[w];
      }
      for (int d = 0; d < nfree[v]; d++) ia[first[v] - 1 + d + 1] = cnt + d;
    }
  });
  ia[0] = 1;
  for (int r = 0; r < neq; r++) ia[r + 1] += ia[r];
  ja.assign((size_t)ia[neq] - 1, 0);
  parallel_chunks(m.nnode, 8192, [&](int64_t v0, int64_t v1) {
    std::vector<std::pair<int32_t, int32_t>> blocks;
    for (int64_t v = v0; v < v1; v++) {
      if (!nfree[v]) continue;
      blocks.clear();
      for (int k = xadj[v]; k < xadj[v + 1]; k++) {
        int w = adj[k];
        if (nfree[w] && first[w] < first[v]) blocks.emplace_back(first[w], nfree[w]);
      }
      std::sort(blocks.begin(), blocks.end());
      for (int d = 0; d < nfree[v]; d++) {
        int32_t r = first[v] + d;  // 1-based row
        int64_t p = ia[r - 1] - 1;
        for (auto &b : blocks)
          for (int t = 0; t < b.second; t++) ja[p++] = b.first + t;
        for (int t = 0; t < d; t++) ja[p++] = first[v] + t;
      }
    }
  });
}

// Greedy element colouring: each element, in element order, takes the
// smallest colour none of its vertex nodes has yet, so that the elements of
// one colour share no node (and so no equation): the assembly kernels then
// add element blocks colour by colour without atomics.  Any colouring with
// that property serves (the reference's colormsh, Colormsh.f:9-308, is
// another); returns the number of colours, color[el] 0-based.
int color_elements(const Mesh &m, std::vector<int32_t> &color) {
  const int nen1 = m.nen + 1;
  color.assign(m.numel, -1);
  // per node a bit per colour taken, `words` 64-bit words per node, node-major
  int words = 1;
  std::vector<uint64_t> used((size_t)m.nnode, 0);
  int ncolors = 0;
  for (int el = 0; el < m.numel; el++) {
    const int32_t *c = &m.ix[(size_t)el * nen1];
    int iel = m.ie[c[m.nen] - 1];
    int nv = elem_nodes(iel);
    int chosen = -1;
    for (int w = 0; chosen < 0; w++) {
      if (w == words) {  // more than 64 * words colours: widen every node's set
        std::vector<uint64_t> wider((size_t)m.nnode * (words + 1), 0);
        for (size_t v = 0; v < (size_t)m.nnode; v++)
          std::copy(used.begin() + v * words, used.begin() + (v + 1) * words,
                    wider.begin() + v * (words + 1));
        used.swap(wider);
        words++;
      }
      uint64_t busy = 0;
      for (int a = 0; a < nv; a++) busy |= used[(size_t)(c[a] - 1) * words + w];
      if (~busy) chosen = w * 64 + __builtin_ctzll(~busy);
    }
    color[el] = chosen;
    ncolors = std::max(ncolors, chosen + 1);
    for (int a = 0; a < nv; a++)
      used[(size_t)(c[a] - 1) * words + chosen / 64] |= 1ull << (chosen % 64);
  }
  return ncolors;
}

// What the assembly kernels need beyond ia/ja/id:
//  * a greedy element colouring in which no two elements of a colour share a
//    node (so colour-ordered assembly needs no atomics), elements grouped per
//    colour and element type;
//  * the slot map: for each element and each unordered pair of its nodes
//    {a, b} with free dofs, the offset within the row of the higher node of
//    the lower node's first column (identical for every dof row of that node).
// The SpMV's tiled transposed index is built by build_tiles.
void derive_structure(const Mesh &m, Structure &s) {
  // ---- element colouring
  const int nen1 = m.nen + 1;
  std::vector<int32_t> color;
  s.ncolors = color_elements(m, color);
  // group by (colour, element type), elements ascending inside a group: a
  // counting sort on colour * kTypes + type, scattered in element order
  auto type_of = [&](int el) { return m.ie[m.ix[(size_t)el * nen1 + m.nen] - 1]; };
  constexpr int kTypes = 8;  // element type codes 2..7
  std::vector<int64_t> bucket((size_t)s.ncolors * kTypes + 1, 0);
  for (int el = 0; el < m.numel; el++) {
    const int t = type_of(el);
    ELX_REQUIRE(t >= 0 && t < kTypes, ELX_ERR_BAD_ELEMENT, "unsupported element type");
    bucket[(size_t)color[el] * kTypes + t + 1]++;
  }
  for (size_t k = 1; k < bucket.size(); k++) bucket[k] += bucket[k - 1];
  s.elem_order.resize(m.numel);
  for (int el = 0; el < m.numel; el++)
    s.elem_order[bucket[(size_t)color[el] * kTypes + type_of(el)]++] = el;
  s.segments.clear();
  s.color_of_segment.clear();
  for (int i = 0; i < m.numel;) {
    int el = s.elem_order[i];
    int c = color[el], t = type_of(el), j = i;
    while (j < m.numel && color[s.elem_order[j]] == c && type_of(s.elem_order[j]) == t) j++;
    s.segments.push_back({t, i, j});
    s.color_of_segment.push_back(c);
    i = j;
  }
  // ---- slot map
  const int nen = m.nen;
  s.npairs = nen * (nen - 1) / 2;
  s.slot.assign((size_t)s.npairs * m.numel, -1);
  std::vector<int32_t> first(m.nnode, 0);
  for (int v = 0; v < m.nnode; v++)
    for (int d = m.ndf - 1; d >= 0; d--) {
      int q = s.id[(size_t)v * m.ndf + d];
      if (q > 0) first[v] = q;  // smallest free equation of the node
    }
  std::atomic<bool> missing{false};
  parallel_chunks(m.numel, 16384, [&](int64_t t0, int64_t t1) {
    for (int64_t t = t0; t < t1; t++) {
      int el = s.elem_order[t];
      const int32_t *c = &m.ix[(size_t)el * nen1];
      int nv = elem_nodes(type_of(el));
      int pair = 0;
      for (int a = 0; a < nen; a++)
        for (int b = a + 1; b < nen; b++, pair++) {
          if (a >= nv || b >= nv) continue;
          int va = c[a] - 1, vb = c[b] - 1;
          if (!first[va] || !first[vb] || va == vb) continue;
          int hi = first[va] > first[vb] ? va : vb;
          int lo = hi == va ? vb : va;
          int32_t r = first[hi] - 1;  // 0-based row of the higher node's first dof
          const int32_t *rb = s.ja.data() + (s.ia[r] - 1);
          const int32_t *re = s.ja.data() + (s.ia[r + 1] - 1);
          const int32_t *pos = std::lower_bound(rb, re, first[lo]);
          if (pos == re || *pos != first[lo]) {
            missing = true;
            continue;
          }
          s.slot[(size_t)pair * m.numel + t] = (int32_t)(pos - rb);
        }
    }
  });
  ELX_REQUIRE(!missing, ELX_ERR_ARG, "CSRC pattern does not contain an element's node pair");
}

namespace {

template <class F>
void parallel_for(int n, F &&f) {
  int nt = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  if (n < 64) nt = 1;
  std::vector<std::thread> th;
  for (int w = 0; w < nt; w++)
    th.emplace_back([&, w] {
      for (int i = w; i < n; i += nt) f(i);
    });
  for (auto &t : th) t.join();
}

}  // namespace

// Tiled transposed index for the single-read symmetric SpMV (spmv.cu).
// Rows are cut into tiles of tile_rows consecutive rows.  For tile t its
// entries are the CSRC positions [ia[r0], ia[r1]); every distinct column j
// of those entries is a "target" that receives sum a_k x_row(k) over the
// tile's entries in column j.  Targets are ascending by column, so the ones
// left of the tile (j < r0, whose rows belong to earlier tiles) come first;
// each of those gets a halo slot, and every row lists its halo slots in tile
// order, which fixes the summation order of every y entry.
void build_tiles(Structure &s, int tile_rows) {
  const int32_t neq = s.neq;
  s.tile_rows = tile_rows;
  s.ntiles = (neq + tile_rows - 1) / tile_rows;
  const int nt = s.ntiles;
  // lanes per row from the mean row length
  const double mean_len = neq ? (double)s.nad / neq : 0.0;
  s.lanes = mean_len < 8 ? 1 : 2;  // threads per row in the SpMV row phase
  std::vector<int32_t> ntgt(nt, 0), nout(nt, 0);
  std::vector<std::vector<uint64_t>> keys(nt);
  s.tpos.assign(s.nad, 0);
  int32_t max_nnz = 0;
  for (int t = 0; t < nt; t++) {
    const int r0 = t * tile_rows, r1 = std::min(neq, r0 + tile_rows);
    max_nnz = std::max(max_nnz, s.ia[r1] - s.ia[r0]);
  }
  ELX_REQUIRE(max_nnz <= 65535, ELX_ERR_ARG, "tile too large for 16-bit positions");
  s.max_tile_nnz = max_nnz;
  // per tile: sort (column, position) pairs; count targets
  parallel_for(nt, [&](int t) {
    const int r0 = t * tile_rows, r1 = std::min(neq, r0 + tile_rows);
    const int64_t b0 = s.ia[r0] - 1, b1 = s.ia[r1] - 1;
    std::vector<uint64_t> &kk = keys[t];
    kk.resize(b1 - b0);
    for (int64_t k = b0; k < b1; k++)
      kk[k - b0] = ((uint64_t)(uint32_t)(s.ja[k] - 1) << 16) | (uint64_t)(k - b0);
    std::sort(kk.begin(), kk.end());
    int32_t c = 0, o = 0;
    for (size_t q = 0; q < kk.size(); q++) {
      const int32_t col = (int32_t)(kk[q] >> 16);
      if (q == 0 || col != (int32_t)(kk[q - 1] >> 16)) {
        c++;
        if (col < r0) o++;
      }
    }
    ntgt[t] = c;
    nout[t] = o;
  });
  s.tile_tgt.assign(nt + 1, 0);
  s.tile_out.assign(nt + 1, 0);
  for (int t = 0; t < nt; t++) {
    s.tile_tgt[t + 1] = s.tile_tgt[t] + ntgt[t];
    s.tile_out[t + 1] = s.tile_out[t] + nout[t];
  }
  const int32_t ntargets = s.tile_tgt[nt];
  s.tgt_col.assign(ntargets, 0);
  s.tgt_start.assign(ntargets + 1, 0);
  // Within each class (left of the tile, inside it) the targets are ordered
  // by decreasing entry count, so that the 32 threads of a warp in the
  // column phase run loops of nearly equal length (the FP64 pipe is charged
  // per warp instruction, whatever the number of active lanes).
  parallel_for(nt, [&](int t) {
    const int r0 = t * tile_rows;
    const int64_t b0 = s.ia[r0] - 1;
    const std::vector<uint64_t> &kk = keys[t];
    struct Run { int32_t col, begin, len; };
    std::vector<Run> runs;
    for (size_t q = 0; q < kk.size(); q++) {
      const int32_t col = (int32_t)(kk[q] >> 16);
      if (q == 0 || col != (int32_t)(kk[q - 1] >> 16)) runs.push_back({col, (int32_t)q, 0});
      runs.back().len++;
    }
    const int32_t no = nout[t];
    auto by_len = [](const Run &a, const Run &b) {
      return a.len != b.len ? a.len > b.len : a.col < b.col;
    };
    std::stable_sort(runs.begin(), runs.begin() + no, by_len);
    std::stable_sort(runs.begin() + no, runs.end(), by_len);
    int32_t g = s.tile_tgt[t], q = 0;
    for (const Run &r : runs) {
      s.tgt_col[g] = r.col;
      s.tgt_start[g] = (int32_t)(b0 + q);
      for (int32_t e = 0; e < r.len; e++)
        s.tpos[b0 + q + e] = (uint16_t)(kk[r.begin + e] & 0xffff);
      q += r.len;
      g++;
    }
  });
  s.tgt_start[ntargets] = (int32_t)s.nad;
  s.tile_desc.assign((size_t)8 * nt, 0);
  s.max_tile_tgt = 0;
  for (int t = 0; t < nt; t++) {
    const int r0 = t * tile_rows, r1 = std::min(neq, r0 + tile_rows);
    int32_t *d = &s.tile_desc[(size_t)8 * t];
    d[0] = s.ia[r0] - 1;
    d[1] = s.ia[r1] - s.ia[r0];
    d[2] = s.tile_tgt[t];
    d[3] = ntgt[t];
    d[4] = s.tile_out[t];
    d[5] = nout[t];
    d[6] = r0;
    d[7] = r1 - r0;
    s.max_tile_tgt = std::max(s.max_tile_tgt, ntgt[t]);
  }
  keys.clear();
  keys.shrink_to_fit();
  // halo lists per row, in tile order
  s.halo_ptr.assign(neq + 1, 0);
  for (int t = 0; t < nt; t++)
    for (int32_t g = s.tile_tgt[t]; g < s.tile_tgt[t] + nout[t]; g++) s.halo_ptr[s.tgt_col[g] + 1]++;
  for (int r = 0; r < neq; r++) s.halo_ptr[r + 1] += s.halo_ptr[r];
  s.halo_slot.assign(s.halo_ptr[neq], 0);
  std::vector<int32_t> fill(s.halo_ptr.begin(), s.halo_ptr.end() - 1);
  for (int t = 0; t < nt; t++)
    for (int32_t q = 0; q < nout[t]; q++) {
      const int32_t g = s.tile_tgt[t] + q;
      s.halo_slot[fill[s.tgt_col[g]]++] = s.tile_out[t] + q;
    }
}

// Transposed index of the strict lower part by a counting sort on columns:
// iat/jat is the CSR of the upper part, pt the position in al of each of its
// entries (so that alt = al[pt] is the upper part's value array).
void build_transpose(Structure &s) {
  const int32_t neq = s.neq;
  s.iat.assign(neq + 1, 0);
  for (int64_t k = 0; k < s.nad; k++) s.iat[s.ja[k]]++;  // 1-based column c counts at iat[c]
  for (int c = 0; c < neq; c++) s.iat[c + 1] += s.iat[c];
  s.jat.assign(s.nad, 0);
  s.pt.assign(s.nad, 0);
  std::vector<int32_t> fill(s.iat.begin(), s.iat.end() - 1);
  int32_t bw = 0;
  for (int r = 0; r < neq; r++)
    for (int32_t k = s.ia[r] - 1; k < s.ia[r + 1] - 1; k++) {
      const int c = s.ja[k] - 1;
      const int32_t q = fill[c]++;
      s.jat[q] = r;
      s.pt[q] = k;
      bw = std::max(bw, r - c);
    }
  // 16-bit deltas when every |row - col| fits (typical after RCM)
  s.bw16 = bw <= 65535;
  s.ja16.clear();
  s.jat16.clear();
  if (s.bw16) {
    s.ja16.resize(s.nad);
    s.jat16.resize(s.nad);
    for (int r = 0; r < neq; r++) {
      for (int32_t k = s.ia[r] - 1; k < s.ia[r + 1] - 1; k++)
        s.ja16[k] = (uint16_t)(r - (s.ja[k] - 1));
      for (int32_t q = s.iat[r]; q < s.iat[r + 1]; q++) s.jat16[q] = (uint16_t)(s.jat[q] - r);
    }
  }
}

// Node blocks of the CSRC pattern.  numeq (Numeq.f:139-192) numbers the free
// dofs of each node consecutively in node order, so when no node is only
// partly fixed, equation B I + a is dof a of the I-th free node and the
// lower pattern of row B I + a is: B consecutive columns per lower neighbour
// node J (ascending), then the a columns B I .. B I + a - 1 of the node's own
// block.  Checks exactly that shape; any other pattern leaves s.blocked false
// (the scalar kernels then handle the matrix).
void build_blocks(Structure &s, int bsize) {
  s.blocked = false;
  s.bsize = s.nb = 0;
  s.nnzb = 0;
  s.bia.clear();
  s.bja.clear();
  s.bt.clear();
  s.nslices = 0;
  s.sell_ptr.clear();
  s.sell_col.clear();
  const int B = bsize;
  if (B < 2 || B > 3 || s.neq % B) return;
  const int nb = s.neq / B;
  std::vector<int32_t> nl(nb), nup(nb, 0);
  // every row block I: B rows of whole B x B blocks left of the diagonal
  // block (the same block columns in each row) plus the diagonal block's
  // lower part
  std::atomic<bool> not_blocked{false};
  parallel_chunks(nb, 8192, [&](int64_t I0, int64_t I1) {
    for (int64_t I = I0; I < I1 && !not_blocked.load(std::memory_order_relaxed); I++) {
      const int r0 = B * (int)I;
      const int32_t k0 = s.ia[r0] - 1;
      const int32_t len0 = s.ia[r0 + 1] - s.ia[r0];
      bool ok = len0 % B == 0;
      const int n = len0 / B;
      nl[I] = n;
      for (int a = 0; ok && a < B; a++) {
        const int r = r0 + a;
        const int32_t k = s.ia[r] - 1;
        if (s.ia[r + 1] - s.ia[r] != B * n + a) {
          ok = false;
          break;
        }
        for (int q = 0; ok && q < n; q++) {
          const int c0 = s.ja[k0 + B * q] - 1;
          if (c0 % B || c0 / B >= I) ok = false;
          for (int b = 0; ok && b < B; b++)
            if (s.ja[k + B * q + b] - 1 != c0 + b) ok = false;
        }
        for (int t = 0; ok && t < a; t++)
          if (s.ja[k + B * n + t] - 1 != r0 + t) ok = false;
      }
      if (!ok) not_blocked = true;
    }
  });
  if (not_blocked) return;
  for (int I = 0; I < nb; I++) {
    const int32_t k0 = s.ia[B * I] - 1;
    for (int q = 0; q < nl[I]; q++) nup[(s.ja[k0 + B * q] - 1) / B]++;
  }
  s.bia.assign(nb + 1, 0);
  for (int I = 0; I < nb; I++) s.bia[I + 1] = s.bia[I] + nl[I] + 1 + nup[I];
  const int64_t nnzb = s.bia[nb];
  s.bja.assign(nnzb, 0);
  s.bt.assign(nnzb, 0);
  std::vector<int32_t> upos(nb);
  for (int I = 0; I < nb; I++) upos[I] = s.bia[I] + nl[I] + 1;
  for (int I = 0; I < nb; I++) {
    const int32_t k0 = s.ia[B * I] - 1;
    const int32_t p0 = s.bia[I];
    for (int q = 0; q < nl[I]; q++) {
      const int J = (s.ja[k0 + B * q] - 1) / B;
      s.bja[p0 + q] = J;
      s.bt[p0 + q] = -1 - I;
      // the mirror (I above J) goes to the next upper slot of row J; rows I
      // arrive in ascending order, so the upper blocks come out sorted
      const int32_t u = upos[J]++;
      s.bja[u] = I;
      s.bt[u] = p0 + q;
    }
    s.bja[p0 + nl[I]] = I;
    s.bt[p0 + nl[I]] = -1 - I;
  }
  s.blocked = true;
  s.bsize = B;
  s.nb = nb;
  s.nnzb = nnzb;
  // the sliced copy's pattern: each slice as wide as its longest block row
  const int R = kSliceRows;
  s.nslices = (nb + R - 1) / R;
  s.sell_ptr.assign(s.nslices + 1, 0);
  for (int sl = 0; sl < s.nslices; sl++) {
    int w = 0;
    for (int I = sl * R; I < std::min(nb, sl * R + R); I++) w = std::max(w, s.bia[I + 1] - s.bia[I]);
    s.sell_ptr[sl + 1] = s.sell_ptr[sl] + w;
  }
  s.sell_col.assign((size_t)s.sell_ptr[s.nslices] * R, 0);
  parallel_chunks(s.nslices, 1024, [&](int64_t sl0, int64_t sl1) {
    for (int64_t sl = sl0; sl < sl1; sl++)
      for (int t = 0; t < R; t++) {
        const int I = (int)sl * R + t;
        const int n = I < nb ? s.bia[I + 1] - s.bia[I] : 0;
        for (int g = s.sell_ptr[sl]; g < s.sell_ptr[sl + 1]; g++) {
          const int k = g - s.sell_ptr[sl];
          s.sell_col[(size_t)g * R + t] = k < n ? s.bja[s.bia[I] + k] : (I < nb ? I : 0);
        }
      }
  });
}

}  // namespace elx

namespace elx {

// Row-block partitions of the RCM-ordered equations for a multi-GPU run, one
// partition per GPU, in the layout of the reference's overlapping MPI
// partitions (csrstruct with lower = right = .true., Csr.f:13-305).
//
// Cuts fall on node boundaries -- on multiples of kSliceRows nodes when the
// matrix has node blocks, so that a partition's rows are whole slices of the
// sliced copy -- and balance the full-row nonzeros (each owned row's lower,
// diagonal and upper entries), as Matrix_partition.f:98-150 balances rows
// between threads.  Returns the nparts + 1 cut equations (0-based), or an
// empty vector if there are fewer cut units than partitions.
std::vector<int32_t> partition_bounds(const Structure &s, int ndf, int nparts) {
  const int32_t neq = s.neq;
  // the first equation of every node that has equations, ascending
  std::vector<int32_t> starts;
  const int nnode = (int)(s.id.size() / ndf);
  for (int n = 0; n < nnode; n++) {
    int32_t first = INT32_MAX;
    for (int j = 0; j < ndf; j++)
      if (s.id[(size_t)n * ndf + j] > 0) first = std::min(first, s.id[(size_t)n * ndf + j] - 1);
    if (first != INT32_MAX) starts.push_back(first);
  }
  std::sort(starts.begin(), starts.end());
  // node blocks: every node with equations has all ndf of them
  bool blocked = neq % ndf == 0 && (int64_t)starts.size() * ndf == neq;
  const int unit = blocked ? kSliceRows : 1;
  std::vector<int32_t> cuts;  // candidate cut equations (unit starts)
  for (size_t k = 0; k < starts.size(); k += unit) cuts.push_back(starts[k]);
  if ((int)cuts.size() < nparts || nparts < 1) return {};
  // prefix sums of full-row counts: lower + diagonal + upper entries
  std::vector<int64_t> w(neq + 1, 0);
  for (int i = 0; i < neq; i++) w[i + 1] = (s.ia[i + 1] - s.ia[i]) + 1;
  for (int64_t k = 0; k < s.nad; k++) w[s.ja[k]] += 1;  // column c: upper entry of row c
  for (int i = 0; i < neq; i++) w[i + 1] += w[i];
  std::vector<int32_t> b(1, 0);
  size_t c = 1;
  for (int p = 1; p < nparts; p++) {
    const int64_t target = w[neq] * p / nparts;
    // the first candidate at or past the target, leaving room for the rest
    while (c < cuts.size() && w[cuts[c]] < target) c++;
    const size_t limit = cuts.size() - (size_t)(nparts - p);
    if (c > limit) c = limit;
    b.push_back(cuts[c]);
    c++;
  }
  b.push_back(neq);
  return b;
}

void build_partition(const Structure &s, int32_t eq0, int32_t eq1, Partition &p) {
  p.eq0 = eq0;
  p.neq = eq1 - eq0;
  p.halo.clear();
  // the rectangular entries of each owned row: (global column, al position)
  std::vector<std::vector<std::pair<int32_t, int64_t>>> right(p.neq);
  p.ia.assign(p.neq + 1, 1);
  p.ja.clear();
  p.pos.clear();
  for (int32_t i = eq0; i < eq1; i++) {
    for (int32_t k = s.ia[i] - 1; k < s.ia[i + 1] - 1; k++) {
      const int32_t col = s.ja[k] - 1;
      if (col >= eq0) {
        p.ja.push_back(col - eq0 + 1);
        p.pos.push_back(k);
      } else {
        right[i - eq0].push_back({col, k});
      }
    }
    p.ia[i - eq0 + 1] = (int32_t)p.ja.size() + 1;
  }
  // upper entries of owned rows outside the block: rows past it whose
  // lower part has an owned column
  for (int32_t r = eq1; r < s.neq; r++)
    for (int32_t k = s.ia[r] - 1; k < s.ia[r + 1] - 1; k++) {
      const int32_t col = s.ja[k] - 1;
      if (col >= eq0 && col < eq1) right[col - eq0].push_back({r, k});
    }
  for (auto &r : right)
    for (auto &e : r) p.halo.push_back(e.first);
  std::sort(p.halo.begin(), p.halo.end());
  p.halo.erase(std::unique(p.halo.begin(), p.halo.end()), p.halo.end());
  p.ia1.assign(p.neq + 1, 1);
  p.ja1.clear();
  p.pos1.clear();
  for (int32_t r = 0; r < p.neq; r++) {
    auto &e = right[r];
    std::sort(e.begin(), e.end());
    for (auto &q : e) {
      const int32_t h = (int32_t)(std::lower_bound(p.halo.begin(), p.halo.end(), q.first) -
                                  p.halo.begin());
      p.ja1.push_back(p.neq + 1 + h);
      p.pos1.push_back(q.second);
    }
    p.ia1[r + 1] = (int32_t)p.ja1.size() + 1;
  }
}

}  // namespace elx

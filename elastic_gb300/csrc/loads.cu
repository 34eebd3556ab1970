// Loads on the GPU: pload_mec (mef/src/Pload.f:2-58) for evaluated nodal
// loads and the 2-D distributed edge loads of pform_mec isw = 4
// (Elmlib02.f:260-314 TRIA3, 856-910 QUAD4), written into the resident b0
// and u so that a load step needs no host copy of b.
//
// pload: one thread per (dof, node): b0(id) = f for a free dof, u = f for a
// prescribed one (a free dof's u keeps its value, as in the reference).
//
// Edge loads: the reference forms, per loaded element in element order, the
// element vector p (every loaded side j, in side order, subtracts
// traction * length / 2 from each of its two nodes) and assembles
// b(k) = b(k) - p(i).  Here one thread per loaded node replays exactly that
// sequence for its node -- its (element, sides) entries in ascending element
// order, each side in side order -- with unfused multiply and subtract, so
// b0 is bitwise the reference's (no colours, no atomics).  The host builds
// only the integer lists (which node, which element, which sides); every
// floating-point operation runs here.
#include <algorithm>
#include <climits>

#include "elx_internal.h"

namespace elx {
namespace {

__global__ void pload_kernel(int64_t n, const int32_t *__restrict__ eq,
                             const double *__restrict__ f, double *__restrict__ u,
                             double *__restrict__ b0) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k = eq[q];
    if (k >= 0)
      b0[k] = f[q];
    else
      u[q] = f[q];
  }
}

// ent (kEdgeEntryInts, nent): element (1-based), number of loaded sides of
// the element through this node (1 or 2), then per side its two nodes
// (0-based) and its load number (1-based).
__global__ void edge_load_kernel(int nnodes, const int32_t *__restrict__ node,
                                 const int32_t *__restrict__ ptr,
                                 const int32_t *__restrict__ ent, const double *__restrict__ x,
                                 const int32_t *__restrict__ eq,
                                 const double *__restrict__ loadvec, double *__restrict__ b0,
                                 int32_t *bad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnodes; i += gridDim.x * blockDim.x) {
    const int no = node[i];
    for (int d = 0; d < 2; d++) {
      const int32_t k = eq[2 * no + d];
      if (k < 0) continue;
      double acc = b0[k];
      for (int e = ptr[i]; e < ptr[i + 1]; e++) {
        const int32_t *en = ent + (size_t)e * kEdgeEntryInts;
        double pa = 0.0;
        for (int s = 0; s < en[1]; s++) {
          const int na = en[2 + 3 * s], nb = en[3 + 3 * s], lc = en[4 + 3 * s];
          const double dx = __dsub_rn(x[2 * nb], x[2 * na]);
          const double dy = __dsub_rn(x[2 * nb + 1], x[2 * na + 1]);
          const double det = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
          if (!(det > 0.0)) {
            atomicMin(bad, en[0]);
            continue;
          }
          const double wt1 = __dmul_rn(0.5, __dsqrt_rn(det));
          pa = __dsub_rn(pa, __dmul_rn(loadvec[(size_t)(lc - 1) * 2 + d], wt1));
        }
        acc = __dsub_rn(acc, pa);
      }
      b0[k] = acc;
    }
  }
}

int grid_for(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, grid_cap(8)));
}

}  // namespace

// The loaded nodes of a 2-D mesh and their (element, sides) entries, in the
// reference's order: elements ascending, within an element the sides in
// side order.  Returns false if a load number is outside 1..nload or a
// loaded element is not a TRIA3/QUAD4; `bad_el` is then its 1-based number.
bool build_edge_lists(const Mesh &m, const int32_t *eload, int32_t nload,
                      std::vector<int32_t> &node, std::vector<int32_t> &ptr,
                      std::vector<int32_t> &ent, int32_t &bad_el) {
  static const int tri_side[3][2] = {{0, 1}, {1, 2}, {2, 0}};
  static const int quad_side[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
  node.clear();
  ptr.assign(1, 0);
  ent.clear();
  const int nen1 = m.nen + 1;
  // per node, its entries (a node appears in few loaded elements)
  std::vector<std::vector<int32_t>> at;
  std::vector<int32_t> slot_of(m.nnode, -1);
  for (int el = 0; el < m.numel; el++) {
    const int32_t *iq = eload + (size_t)el * 7;
    const int32_t *ixe = &m.ix[(size_t)el * nen1];
    const int iel = m.ie[ixe[m.nen] - 1];
    const int nside = (iel == TRIA3_STRAIN || iel == TRIA3_STRESS)   ? 3
                      : (iel == QUAD4_STRAIN || iel == QUAD4_STRESS) ? 4
                                                                     : 0;
    int tp = 0;
    for (int j = 0; j < 7; j++) {
      if (iq[j] < 0 || iq[j] > nload || (iq[j] > 0 && j >= nside)) {
        bad_el = el + 1;
        return false;
      }
      tp += iq[j];
    }
    if (tp == 0) continue;
    for (int a = 0; a < nside; a++) {
      int32_t rec[kEdgeEntryInts] = {el + 1, 0, 0, 0, 0, 0, 0, 0};
      for (int j = 0; j < nside; j++) {
        if (iq[j] <= 0) continue;
        const int *sn = nside == 3 ? tri_side[j] : quad_side[j];
        if (sn[0] != a && sn[1] != a) continue;
        const int s = rec[1]++;
        rec[2 + 3 * s] = ixe[sn[0]] - 1;
        rec[3 + 3 * s] = ixe[sn[1]] - 1;
        rec[4 + 3 * s] = iq[j];
      }
      if (rec[1] == 0) continue;
      const int no = ixe[a] - 1;
      if (slot_of[no] < 0) {
        slot_of[no] = (int32_t)at.size();
        at.emplace_back();
        node.push_back(no);
      }
      at[slot_of[no]].insert(at[slot_of[no]].end(), rec, rec + kEdgeEntryInts);
    }
  }
  for (const auto &v : at) {
    ent.insert(ent.end(), v.begin(), v.end());
    ptr.push_back((int32_t)(ent.size() / kEdgeEntryInts));
  }
  return true;
}

void launch_pload(int64_t n, const int32_t *eq, const double *f, double *u, double *b0,
                  cudaStream_t st) {
  if (n <= 0) return;
  pload_kernel<<<grid_for(n), 256, 0, st>>>(n, eq, f, u, b0);
  ELX_CUDA(cudaGetLastError());
}

void launch_edge_loads(int nnodes, const int32_t *node, const int32_t *ptr, const int32_t *ent,
                       const double *x, const int32_t *eq, const double *loadvec, double *b0,
                       int32_t *bad, cudaStream_t st) {
  if (nnodes <= 0) return;
  edge_load_kernel<<<grid_for(nnodes), 256, 0, st>>>(nnodes, node, ptr, ent, x, eq, loadvec, b0,
                                                     bad);
  ELX_CUDA(cudaGetLastError());
}

}  // namespace elx

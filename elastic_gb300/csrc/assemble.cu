// Element stiffness integration and CSRC assembly on the GPU:
// pform_mec(isw=2, lhs=.true., rhs=.true.) of mef/src/Pform.f:1-254 with the
// element routines of Elmlib02.f (elmt02..07_mec, isw=2) and the CSR
// scatter of Assbly.f:66-146.
//
// One thread per element.  Elements are processed colour by colour (no two
// elements of a colour share a node), so every read-modify-write of ad, al
// and b is race free without atomics, and the summation order of each entry
// is fixed by the colour order: results are deterministic.
//
// Scatter without search: the reference finds the column of each entry by a
// linear search of the row (Assbly.f:124-128).  Here a node's free equations
// are consecutive and the blocks of two nodes are disjoint, so inside the
// rows of the higher node the lower node's columns form one contiguous run at
// an offset that is the same for every dof row; the host precomputes that
// offset per element and node pair (the slot map).  A node's own lower
// columns are the last entries of its rows.
//
// Stiffness blocks.  For the isotropic 3-D law of elmt06/07_mec the 3x3 block
// of nodes (i, j) at one integration point is
//   wt1 * ( b * g_i g_j^T + c * g_j g_i^T + c * (g_i . g_j) I ),
// using b + 2c = 1 with a, b, c of Elmlib02.f:1697-1705.  Summed over the
// points it only needs M_ij = sum_gp wt1 g_i g_j^T, so each block costs 9
// FMAs per point instead of the ~36 operations of the reference's expanded
// form (Elmlib02.f:1747-1772).  The 2-D laws use the same M_ij with
// d11, d12, d22, d33 (Elmlib02.f:781-795).  Rounding differs from the
// reference's operand order by a few ulps; the assembled values agree to
// well below 1e-13 relative.
#include <cstdlib>
#include <mutex>

#include "elx_internal.h"

namespace elx {
namespace {

// Gauss-Legendre 2-point abscissa (Elmlib.f:2987), weights 1 (Elmlib.f:3018).
__device__ __constant__ double kPg2[2] = {-.577350269189626e0, .577350269189626e0};

struct Law {
  double d11, d12, d22, d33;  // 2-D constitutive terms
  double a, b, c;             // 3-D factors of elmt06/07_mec
  double thic;                // QUAD4 plane-stress thickness
};

// Constitutive constants of the element routines (Elmlib02.f:179-186 plane
// strain, 469-476 plane stress, 1331-1338 / 1697-1705 3-D).
__device__ Law make_law(int iel, const double *e) {
  Law L{};
  const double ym = e[0], ps = e[1];
  if (iel == TRIA3_STRESS || iel == QUAD4_STRESS) {
    const double a1 = 1.0 - ps, a2 = 1.0 - ps * ps;
    const double a = ym / a2, b = ps, c = 0.5 * a1;
    L.d11 = a; L.d12 = a * b; L.d22 = a; L.d33 = a * c;
    L.thic = e[2] == 0.0 ? 1.0 : e[2];
  } else {
    const double a1 = 1.0 - ps, a2 = 1.0 - 2.0 * ps, a3 = 1.0 + ps;
    const double a = (ym * a1) / (a3 * a2), b = ps / a1, c = 0.5 * (a2 / a1);
    L.d11 = a; L.d12 = a * b; L.d22 = a; L.d33 = a * c;
    L.a = a; L.b = b; L.c = c;
    L.thic = 1.0;
  }
  return L;
}

// Everything one thread needs to scatter blocks of its element.
template <int NEN, int NDF>
struct Elem {
  int eq[NEN][NDF];  // 0-based equation or -1
  int first[NEN];    // smallest equation of the node, -1 if none free
  double u[NEN][NDF];
  double p[NEN][NDF];  // p = K_e u_e (lku_m, Elmlib.f:336-368)
};

// Pair index of local nodes lo < hi in the host's slot-map order (pairs
// enumerated lo-major over the mesh's nen nodes per element).
__device__ __forceinline__ int pair_index(int nen, int lo, int hi) {
  return lo * (nen - 1) - (lo * (lo - 1)) / 2 + (hi - lo - 1);
}

// Adds the block K_ab (rows = dofs of local node a, columns = dofs of b) of a
// node pair a != b into al, and both directions of K u into p.
template <int NEN, int NDF>
__device__ __forceinline__ void scatter_pair(Elem<NEN, NDF> &E, const CsrcDev &k,
                                             const MeshDev &m, int t, int a, int b,
                                             const double (&K)[NDF][NDF], bool with_u) {
  if (with_u) {
#pragma unroll
    for (int r = 0; r < NDF; r++)
#pragma unroll
      for (int c = 0; c < NDF; c++) {
        E.p[a][r] += K[r][c] * E.u[b][c];
        E.p[b][c] += K[r][c] * E.u[a][r];
      }
  }
  const int fa = E.first[a], fb = E.first[b];
  if (fa < 0 || fb < 0) return;
  const int lo = a < b ? a : b, hi = a < b ? b : a;
  const int off = m.slot[(size_t)pair_index(m.nen, lo, hi) * m.numel + t];
  if (fa > fb) {  // rows of a, columns of b
#pragma unroll
    for (int r = 0; r < NDF; r++) {
      const int row = E.eq[a][r];
      if (row < 0) continue;
      const int base = k.ia[row] + off - fb;
#pragma unroll
      for (int c = 0; c < NDF; c++)
        if (E.eq[b][c] >= 0) k.al[base + E.eq[b][c]] += K[r][c];
    }
  } else {  // rows of b, columns of a: entry (b c, a r) = K_ab[r][c]
#pragma unroll
    for (int c = 0; c < NDF; c++) {
      const int row = E.eq[b][c];
      if (row < 0) continue;
      const int base = k.ia[row] + off - fa;
#pragma unroll
      for (int r = 0; r < NDF; r++)
        if (E.eq[a][r] >= 0) k.al[base + E.eq[a][r]] += K[r][c];
    }
  }
}

// Diagonal block of node a: ad and the node's own lower entries, which are
// the last entries of each of its rows (column c of row r at ia[r+1]-(r-c)).
template <int NEN, int NDF>
__device__ __forceinline__ void scatter_diag(Elem<NEN, NDF> &E, const CsrcDev &k, int a,
                                             const double (&K)[NDF][NDF], bool with_u) {
  if (with_u) {
#pragma unroll
    for (int r = 0; r < NDF; r++)
#pragma unroll
      for (int c = 0; c < NDF; c++) E.p[a][r] += K[r][c] * E.u[a][c];
  }
#pragma unroll
  for (int r = 0; r < NDF; r++) {
    const int row = E.eq[a][r];
    if (row < 0) continue;
    k.ad[row] += K[r][r];
    const int end = k.ia[row + 1];
#pragma unroll
    for (int c = 0; c < r; c++) {
      const int col = E.eq[a][c];
      if (col >= 0) k.al[end - (row - col)] += K[r][c];
    }
  }
}

template <int NEN, int NDF>
__device__ __forceinline__ void load_elem(Elem<NEN, NDF> &E, const MeshDev &m, int t,
                                          const int (&node)[NEN], const double *u) {
#pragma unroll
  for (int a = 0; a < NEN; a++) {
    int f = -1;
#pragma unroll
    for (int d = NDF - 1; d >= 0; d--) {
      const int q = m.eq[(size_t)node[a] * NDF + d];
      E.eq[a][d] = q;
      if (q >= 0) f = q;
      E.u[a][d] = u ? u[(size_t)node[a] * NDF + d] : 0.0;
      E.p[a][d] = 0.0;
    }
    E.first[a] = f;
  }
}

// b(k) = b(k) - p(i) for free dofs (Assbly.f:118).
template <int NEN, int NDF>
__device__ __forceinline__ void finish_rhs(const Elem<NEN, NDF> &E, double *b) {
  if (b == nullptr) return;
#pragma unroll
  for (int a = 0; a < NEN; a++)
#pragma unroll
    for (int d = 0; d < NDF; d++)
      if (E.eq[a][d] >= 0) b[E.eq[a][d]] -= E.p[a][d];
}

__device__ __forceinline__ void mark_bad(int32_t *bad, int elnum) { atomicMin(bad, elnum); }

// 2-D block from M = sum wt g_i g_j^T (rows x, y).
__device__ __forceinline__ void block2d(const Law &L, const double (&M)[2][2],
                                        double (&K)[2][2]) {
  K[0][0] = L.d11 * M[0][0] + L.d33 * M[1][1];
  K[0][1] = L.d12 * M[0][1] + L.d33 * M[1][0];
  K[1][0] = L.d12 * M[1][0] + L.d33 * M[0][1];
  K[1][1] = L.d22 * M[1][1] + L.d33 * M[0][0];
}

// 3-D block from M = sum wt1 g_i g_j^T: b M + c M^T + c tr(M) I.
__device__ __forceinline__ void block3d(const Law &L, const double (&M)[3][3],
                                        double (&K)[3][3]) {
  const double tr = L.c * (M[0][0] + M[1][1] + M[2][2]);
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) K[r][c] = L.b * M[r][c] + L.c * M[c][r] + (r == c ? tr : 0.0);
}

// ---------------------------------------------------------------- TRIA3
// elmt02_mec / elmt03_mec (Elmlib02.f:50-627): constant-strain triangle,
// wt1 = det/2; the plane-stress thickness is not applied to K (as there).
__global__ void tria3_kernel(MeshDev m, CsrcDev k, int begin, int end, int iel,
                             const double *__restrict__ u, double *__restrict__ b,
                             int32_t *bad) {
  const int t = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= end) return;
  int node[3];
#pragma unroll
  for (int a = 0; a < 3; a++) node[a] = m.conn[(size_t)a * m.numel + t];
  double xl[3][2];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    xl[a][0] = m.x[(size_t)node[a] * m.ndm + 0];
    xl[a][1] = m.x[(size_t)node[a] * m.ndm + 1];
  }
  const double xj11 = xl[0][0] - xl[2][0], xj12 = xl[0][1] - xl[2][1];
  const double xj21 = xl[1][0] - xl[2][0], xj22 = xl[1][1] - xl[2][1];
  const double det = xj11 * xj22 - xj12 * xj21;
  if (det <= 0.0) { mark_bad(bad, m.elnum[t]); return; }
  const double xji11 = xj22 / det, xji12 = -xj12 / det;
  const double xji21 = -xj21 / det, xji22 = xj11 / det;
  const double g[3][2] = {{xji11, xji21}, {xji12, xji22},
                          {-xji11 - xji12, -xji21 - xji22}};
  const Law L = make_law(iel, m.e + (size_t)m.mat[t] * m.prop);
  const double wt1 = 0.5 * det;
  Elem<3, 2> E;
  load_elem<3, 2>(E, m, t, node, u);
  const bool with_u = u != nullptr;
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int bb = 0; bb <= a; bb++) {
      double M[2][2], K[2][2];
#pragma unroll
      for (int r = 0; r < 2; r++)
#pragma unroll
        for (int c = 0; c < 2; c++) M[r][c] = wt1 * g[a][r] * g[bb][c];
      block2d(L, M, K);
      if (a == bb) scatter_diag<3, 2>(E, k, a, K, with_u);
      else scatter_pair<3, 2>(E, k, m, t, a, bb, K, with_u);
    }
  finish_rhs<3, 2>(E, b);
}

// ---------------------------------------------------------------- QUAD4
// elmt04_mec / elmt05_mec (Elmlib02.f:629-1230): 2x2 Gauss with sfquad4_m
// (Elmlib.f:815-886) and jacob2d_m (Elmlib.f:1769-1852).
__global__ void quad4_kernel(MeshDev m, CsrcDev k, int begin, int end, int iel,
                             const double *__restrict__ u, double *__restrict__ b,
                             int32_t *bad) {
  const int t = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= end) return;
  int node[4];
#pragma unroll
  for (int a = 0; a < 4; a++) node[a] = m.conn[(size_t)a * m.numel + t];
  double xl[4][2];
#pragma unroll
  for (int a = 0; a < 4; a++) {
    xl[a][0] = m.x[(size_t)node[a] * m.ndm + 0];
    xl[a][1] = m.x[(size_t)node[a] * m.ndm + 1];
  }
  const Law L = make_law(iel, m.e + (size_t)m.mat[t] * m.prop);
  double g[4][4][2];  // [gp][node][x,y]
  double wt[4];
#pragma unroll
  for (int ly = 0; ly < 2; ly++)
#pragma unroll
    for (int lx = 0; lx < 2; lx++) {
      const int gp = ly * 2 + lx;
      const double r = kPg2[lx], s = kPg2[ly];
      const double opr = 1.0 + r, ops = 1.0 + s, omr = 1.0 - r, oms = 1.0 - s;
      const double hr[4] = {ops * 0.25, -(ops * 0.25), -(oms * 0.25), oms * 0.25};
      const double hs[4] = {opr * 0.25, omr * 0.25, -(omr * 0.25), -(opr * 0.25)};
      double j11 = 0, j12 = 0, j21 = 0, j22 = 0;
#pragma unroll
      for (int a = 0; a < 4; a++) {
        j11 += hr[a] * xl[a][0];
        j12 += hr[a] * xl[a][1];
        j21 += hs[a] * xl[a][0];
        j22 += hs[a] * xl[a][1];
      }
      const double det = j11 * j22 - j21 * j12;
      if (det <= 1.e-14) { mark_bad(bad, m.elnum[t]); return; }
      const double i11 = j22 / det, i12 = -j12 / det, i21 = -j21 / det, i22 = j11 / det;
#pragma unroll
      for (int a = 0; a < 4; a++) {
        g[gp][a][0] = i11 * hr[a] + i12 * hs[a];
        g[gp][a][1] = i21 * hr[a] + i22 * hs[a];
      }
      wt[gp] = det * L.thic;  // wg(lx)*wg(ly) = 1
    }
  Elem<4, 2> E;
  load_elem<4, 2>(E, m, t, node, u);
  const bool with_u = u != nullptr;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int bb = 0; bb <= a; bb++) {
      double M[2][2] = {{0, 0}, {0, 0}}, K[2][2];
#pragma unroll
      for (int gp = 0; gp < 4; gp++) {
        const double s0 = wt[gp] * g[gp][a][0], s1 = wt[gp] * g[gp][a][1];
        M[0][0] += s0 * g[gp][bb][0];
        M[0][1] += s0 * g[gp][bb][1];
        M[1][0] += s1 * g[gp][bb][0];
        M[1][1] += s1 * g[gp][bb][1];
      }
      block2d(L, M, K);
      if (a == bb) scatter_diag<4, 2>(E, k, a, K, with_u);
      else scatter_pair<4, 2>(E, k, m, t, a, bb, K, with_u);
    }
  finish_rhs<4, 2>(E, b);
}

// --------------------------------------------------------------- TETRA4
// elmt06_mec (Elmlib02.f:1232-1573) with jtetra4 (Elmlib.f:2636-2713):
// constant strain, wt1 = a * det * div6 with the literal div6.
__global__ void tetra4_kernel(MeshDev m, CsrcDev k, int begin, int end,
                              const double *__restrict__ u, double *__restrict__ b,
                              int32_t *bad) {
  const int t = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= end) return;
  int node[4];
#pragma unroll
  for (int a = 0; a < 4; a++) node[a] = m.conn[(size_t)a * m.numel + t];
  double xl[4][3];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int d = 0; d < 3; d++) xl[a][d] = m.x[(size_t)node[a] * 3 + d];
  double xj[3][3];
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int d = 0; d < 3; d++) xj[r][d] = xl[r][d] - xl[3][d];
  const double det = xj[0][0] * xj[1][1] * xj[2][2] + xj[0][1] * xj[1][2] * xj[2][0] +
                     xj[0][2] * xj[1][0] * xj[2][1] - xj[2][0] * xj[1][1] * xj[0][2] -
                     xj[0][1] * xj[1][0] * xj[2][2] - xj[0][0] * xj[2][1] * xj[1][2];
  if (det <= 1.e-14) { mark_bad(bad, m.elnum[t]); return; }
  const double deti = 1.0 / det;
  double g[4][3];
  g[0][0] = (xj[1][1] * xj[2][2] - xj[1][2] * xj[2][1]) * deti;
  g[1][0] = (xj[0][2] * xj[2][1] - xj[0][1] * xj[2][2]) * deti;
  g[2][0] = (xj[0][1] * xj[1][2] - xj[0][2] * xj[1][1]) * deti;
  g[0][1] = (xj[1][2] * xj[2][0] - xj[1][0] * xj[2][2]) * deti;
  g[1][1] = (xj[0][0] * xj[2][2] - xj[0][2] * xj[2][0]) * deti;
  g[2][1] = (xj[0][2] * xj[1][0] - xj[0][0] * xj[1][2]) * deti;
  g[0][2] = (xj[1][0] * xj[2][1] - xj[1][1] * xj[2][0]) * deti;
  g[1][2] = (xj[0][1] * xj[2][0] - xj[0][0] * xj[2][1]) * deti;
  g[2][2] = (xj[0][0] * xj[1][1] - xj[0][1] * xj[1][0]) * deti;
#pragma unroll
  for (int d = 0; d < 3; d++) g[3][d] = -g[0][d] - g[1][d] - g[2][d];
  const Law L = make_law(TETRA4, m.e + (size_t)m.mat[t] * m.prop);
  const double div6 = 0.166666666666667e+00;
  const double wt1 = L.a * det * div6;
  Elem<4, 3> E;
  load_elem<4, 3>(E, m, t, node, u);
  const bool with_u = u != nullptr;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int bb = 0; bb <= a; bb++) {
      double M[3][3], K[3][3];
#pragma unroll
      for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) M[r][c] = wt1 * g[a][r] * g[bb][c];
      block3d(L, M, K);
      if (a == bb) scatter_diag<4, 3>(E, k, a, K, with_u);
      else scatter_pair<4, 3>(E, k, m, t, a, bb, K, with_u);
    }
  finish_rhs<4, 3>(E, b);
}

// ---------------------------------------------------------------- HEXA8
// elmt07_mec (Elmlib02.f:1577-2023): 2x2x2 Gauss with sfhexa8_m
// (Elmlib.f:1151-1258) and jacob3d_m (Elmlib.f:1942-2036).  The shape
// function gradients of the 8 points are kept in shared memory, one column
// per thread ([gp][node][xyz][thread]) so that accesses are bank-conflict free.
constexpr int kHexThreads = 64;
constexpr size_t kHexSmem = sizeof(double) * 8 * 8 * 3 * kHexThreads;

__global__ void __launch_bounds__(kHexThreads)
hexa8_kernel(MeshDev m, CsrcDev k, int begin, int end, const double *__restrict__ u,
             double *__restrict__ b, int32_t *bad) {
  extern __shared__ double sg[];
  const int tid = threadIdx.x;
  const int t = begin + blockIdx.x * kHexThreads + tid;
  if (t >= end) return;
#define SG(gp, a, d) sg[(((gp) * 8 + (a)) * 3 + (d)) * kHexThreads + tid]
  int node[8];
#pragma unroll
  for (int a = 0; a < 8; a++) node[a] = m.conn[(size_t)a * m.numel + t];
  double xl[8][3];
#pragma unroll
  for (int a = 0; a < 8; a++)
#pragma unroll
    for (int d = 0; d < 3; d++) xl[a][d] = m.x[(size_t)node[a] * 3 + d];
  const Law L = make_law(HEXA8, m.e + (size_t)m.mat[t] * m.prop);
  double wt[8];
  // natural-coordinate signs of the nodes (Elmlib.f:1177-1184)
  const double rn[8] = {1, -1, -1, 1, 1, -1, -1, 1};
  const double sn[8] = {1, 1, -1, -1, 1, 1, -1, -1};
  const double tn[8] = {1, 1, 1, 1, -1, -1, -1, -1};
  for (int lz = 0; lz < 2; lz++)
    for (int ly = 0; ly < 2; ly++)
      for (int lx = 0; lx < 2; lx++) {
        const int gp = (lz * 2 + ly) * 2 + lx;
        const double r = kPg2[lx], s = kPg2[ly], tt = kPg2[lz];
        double hr[8], hs[8], ht[8];
#pragma unroll
        for (int a = 0; a < 8; a++) {
          const double fr = 1.0 + rn[a] * r, fs = 1.0 + sn[a] * s, ft = 1.0 + tn[a] * tt;
          hr[a] = rn[a] * (fs * ft * 0.125);
          hs[a] = sn[a] * (fr * ft * 0.125);
          ht[a] = tn[a] * (fr * fs * 0.125);
        }
        double xj[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
        for (int a = 0; a < 8; a++)
#pragma unroll
          for (int d = 0; d < 3; d++) {
            xj[0][d] += hr[a] * xl[a][d];
            xj[1][d] += hs[a] * xl[a][d];
            xj[2][d] += ht[a] * xl[a][d];
          }
        const double det = xj[0][0] * xj[1][1] * xj[2][2] + xj[0][1] * xj[1][2] * xj[2][0] +
                           xj[0][2] * xj[1][0] * xj[2][1] - xj[2][0] * xj[1][1] * xj[0][2] -
                           xj[1][0] * xj[0][1] * xj[2][2] - xj[0][0] * xj[2][1] * xj[1][2];
        if (det <= 1.e-14) { mark_bad(bad, m.elnum[t]); return; }
        double ji[3][3];
        ji[0][0] = (xj[1][1] * xj[2][2] - xj[1][2] * xj[2][1]) / det;
        ji[1][0] = -(xj[1][0] * xj[2][2] - xj[1][2] * xj[2][0]) / det;
        ji[2][0] = (xj[1][0] * xj[2][1] - xj[1][1] * xj[2][0]) / det;
        ji[0][1] = -(xj[0][1] * xj[2][2] - xj[0][2] * xj[2][1]) / det;
        ji[1][1] = (xj[0][0] * xj[2][2] - xj[0][2] * xj[2][0]) / det;
        ji[2][1] = -(xj[0][0] * xj[2][1] - xj[0][1] * xj[2][0]) / det;
        ji[0][2] = (xj[0][1] * xj[1][2] - xj[0][2] * xj[1][1]) / det;
        ji[1][2] = -(xj[0][0] * xj[1][2] - xj[0][2] * xj[1][0]) / det;
        ji[2][2] = (xj[0][0] * xj[1][1] - xj[0][1] * xj[1][0]) / det;
#pragma unroll
        for (int a = 0; a < 8; a++)
#pragma unroll
          for (int d = 0; d < 3; d++)
            SG(gp, a, d) = ji[d][0] * hr[a] + ji[d][1] * hs[a] + ji[d][2] * ht[a];
        wt[gp] = det * L.a;  // wg^3 = 1
      }
  Elem<8, 3> E;
  load_elem<8, 3>(E, m, t, node, u);
  const bool with_u = u != nullptr;
  for (int a = 0; a < 8; a++) {
    double sa[8][3];
#pragma unroll
    for (int gp = 0; gp < 8; gp++)
#pragma unroll
      for (int d = 0; d < 3; d++) sa[gp][d] = wt[gp] * SG(gp, a, d);
    for (int bb = 0; bb <= a; bb++) {
      double M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, K[3][3];
#pragma unroll
      for (int gp = 0; gp < 8; gp++) {
        const double g0 = SG(gp, bb, 0), g1 = SG(gp, bb, 1), g2 = SG(gp, bb, 2);
#pragma unroll
        for (int r = 0; r < 3; r++) {
          M[r][0] += sa[gp][r] * g0;
          M[r][1] += sa[gp][r] * g1;
          M[r][2] += sa[gp][r] * g2;
        }
      }
      block3d(L, M, K);
      if (a == bb) scatter_diag<8, 3>(E, k, a, K, with_u);
      else scatter_pair<8, 3>(E, k, m, t, a, bb, K, with_u);
    }
  }
  finish_rhs<8, 3>(E, b);
#undef SG
}

// HEXA8 with a team of 8 threads per element.  One thread per element
// (hexa8_kernel, ELX_HEX_TEAM=0) left each colour's launch with 32,768 long
// serial threads on the 64^3 cube: 8.45 ms per assembly, latency bound.
// Here thread g of a team first forms integration point g (Jacobian, one
// reciprocal of its determinant, the 8 nodes' gradients and weighted
// gradients into shared memory; the natural derivatives come from a table)
// and stages node g's equations and displacements, then the team splits the
// 36 node pairs (lane i: pairs i, i+8, ...), each pair's block formed as in
// hexa8_kernel; the element vector K u is summed over the team by a fixed
// shuffle tree and lane g subtracts node g's part from b.  5.30 ms per
// assembly, the FP64 pipe 77 % busy (FP64-bound: ~7,000 FP64 operations per
// element).
constexpr int kTeamElems = 8;  // elements per 64-thread block

// Natural derivatives (d/dr, d/ds, d/dt) of the 8 shape functions at the 8
// points (sfhexa8_m, Elmlib.f:1151-1258; point g = lx + 2 ly + 4 lz), the
// same for every element: filled once from the host with the kernel's own
// expressions (exact: the node signs are +-1 and 0.125 a power of two).
__device__ __constant__ double kHexDh[8][3][8];

__device__ __constant__ unsigned char kPairA[36] = {0, 1, 1, 2, 2, 2, 3, 3, 3, 3, 4, 4,
                                                    4, 4, 4, 5, 5, 5, 5, 5, 5, 6, 6, 6,
                                                    6, 6, 6, 6, 7, 7, 7, 7, 7, 7, 7, 7};
__device__ __constant__ unsigned char kPairB[36] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3, 0, 1,
                                                    2, 3, 4, 0, 1, 2, 3, 4, 5, 0, 1, 2,
                                                    3, 4, 5, 6, 0, 1, 2, 3, 4, 5, 6, 7};

__global__ void __launch_bounds__(64)
hexa8_team_kernel(MeshDev m, CsrcDev k, int begin, int end, const double *__restrict__ u,
                  double *__restrict__ b, int32_t *bad) {
  __shared__ double sg[kTeamElems][8][8][3];   // [element][point][node][d]: gradients
  __shared__ double swg[kTeamElems][8][8][3];  // the same times the point's weight
  __shared__ double su[kTeamElems][8][3];
  __shared__ int seq[kTeamElems][8][3];
  __shared__ int sfirst[kTeamElems][8];
  const int le = threadIdx.x >> 3, lane = threadIdx.x & 7;
  const int t = begin + blockIdx.x * kTeamElems + le;
  const bool active = t < end;
  const int te = active ? t : begin;  // inactive teams read a valid element, write nothing
  int node[8];
#pragma unroll
  for (int a = 0; a < 8; a++) node[a] = m.conn[(size_t)a * m.numel + te];
  const Law L = make_law(HEXA8, m.e + (size_t)m.mat[te] * m.prop);
  {
    // integration point `lane`
    double hr[8], hs[8], ht[8];
#pragma unroll
    for (int a = 0; a < 8; a++) {
      hr[a] = kHexDh[lane][0][a];
      hs[a] = kHexDh[lane][1][a];
      ht[a] = kHexDh[lane][2][a];
    }
    double xj[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
    for (int a = 0; a < 8; a++)
#pragma unroll
      for (int d = 0; d < 3; d++) {
        const double xa = m.x[(size_t)node[a] * 3 + d];
        xj[0][d] += hr[a] * xa;
        xj[1][d] += hs[a] * xa;
        xj[2][d] += ht[a] * xa;
      }
    const double det = xj[0][0] * xj[1][1] * xj[2][2] + xj[0][1] * xj[1][2] * xj[2][0] +
                       xj[0][2] * xj[1][0] * xj[2][1] - xj[2][0] * xj[1][1] * xj[0][2] -
                       xj[1][0] * xj[0][1] * xj[2][2] - xj[0][0] * xj[2][1] * xj[1][2];
    if (active && det <= 1.e-14) mark_bad(bad, m.elnum[t]);
    // the inverse Jacobian through one reciprocal of det (one FP64 division
    // instead of nine; the FP64 pipe bounds this kernel)
    const double rd = 1.0 / det;
    double ji[3][3];
    ji[0][0] = (xj[1][1] * xj[2][2] - xj[1][2] * xj[2][1]) * rd;
    ji[1][0] = -(xj[1][0] * xj[2][2] - xj[1][2] * xj[2][0]) * rd;
    ji[2][0] = (xj[1][0] * xj[2][1] - xj[1][1] * xj[2][0]) * rd;
    ji[0][1] = -(xj[0][1] * xj[2][2] - xj[0][2] * xj[2][1]) * rd;
    ji[1][1] = (xj[0][0] * xj[2][2] - xj[0][2] * xj[2][0]) * rd;
    ji[2][1] = -(xj[0][0] * xj[2][1] - xj[0][1] * xj[2][0]) * rd;
    ji[0][2] = (xj[0][1] * xj[1][2] - xj[0][2] * xj[1][1]) * rd;
    ji[1][2] = -(xj[0][0] * xj[1][2] - xj[0][2] * xj[1][0]) * rd;
    ji[2][2] = (xj[0][0] * xj[1][1] - xj[0][1] * xj[1][0]) * rd;
    const double w = det * L.a;  // wg^3 = 1
#pragma unroll
    for (int a = 0; a < 8; a++)
#pragma unroll
      for (int d = 0; d < 3; d++) {
        const double g = ji[d][0] * hr[a] + ji[d][1] * hs[a] + ji[d][2] * ht[a];
        sg[le][lane][a][d] = g;
        swg[le][lane][a][d] = w * g;
      }
    // node `lane`: its equations, the smallest of them, its displacements
    int f = -1;
#pragma unroll
    for (int d = 2; d >= 0; d--) {
      const int q = m.eq[(size_t)node[lane] * 3 + d];
      seq[le][lane][d] = q;
      if (q >= 0) f = q;
      su[le][lane][d] = u ? u[(size_t)node[lane] * 3 + d] : 0.0;
    }
    sfirst[le][lane] = f;
  }
  __syncthreads();
  // K u only where the element has a non-zero displacement (an element with
  // u = 0 adds nothing to b; the first solvm pass has u = 0 away from
  // prescribed values): decided per team, from its 8 lanes' nodes
  const unsigned team_mask = 0xffu << (threadIdx.x & 24);
  const bool nz = su[le][lane][0] != 0.0 || su[le][lane][1] != 0.0 || su[le][lane][2] != 0.0;
  const bool with_u = u != nullptr && (__ballot_sync(0xffffffffu, nz) & team_mask) != 0u;
  double p[8][3];
#pragma unroll
  for (int a = 0; a < 8; a++)
#pragma unroll
    for (int d = 0; d < 3; d++) p[a][d] = 0.0;
  for (int q = lane; q < 36; q += 8) {
    const int a = kPairA[q], bb = kPairB[q];
    double M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, K[3][3];
#pragma unroll
    for (int gp = 0; gp < 8; gp++) {
      const double s0 = swg[le][gp][a][0], s1 = swg[le][gp][a][1], s2 = swg[le][gp][a][2];
      const double g0 = sg[le][gp][bb][0], g1 = sg[le][gp][bb][1], g2 = sg[le][gp][bb][2];
      M[0][0] += s0 * g0; M[0][1] += s0 * g1; M[0][2] += s0 * g2;
      M[1][0] += s1 * g0; M[1][1] += s1 * g1; M[1][2] += s1 * g2;
      M[2][0] += s2 * g0; M[2][1] += s2 * g1; M[2][2] += s2 * g2;
    }
    block3d(L, M, K);
    if (with_u) {
#pragma unroll
      for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
          p[a][r] += K[r][c] * su[le][bb][c];
          if (a != bb) p[bb][c] += K[r][c] * su[le][a][r];
        }
    }
    if (!active) continue;
    if (a == bb) {
#pragma unroll
      for (int r = 0; r < 3; r++) {
        const int row = seq[le][a][r];
        if (row < 0) continue;
        k.ad[row] += K[r][r];
        const int endr = k.ia[row + 1];
#pragma unroll
        for (int c = 0; c < r; c++) {
          const int col = seq[le][a][c];
          if (col >= 0) k.al[endr - (row - col)] += K[r][c];
        }
      }
    } else {
      const int fa = sfirst[le][a], fb = sfirst[le][bb];
      if (fa < 0 || fb < 0) continue;
      const int off = m.slot[(size_t)pair_index(m.nen, bb, a) * m.numel + t];
      if (fa > fb) {  // rows of a, columns of bb
#pragma unroll
        for (int r = 0; r < 3; r++) {
          const int row = seq[le][a][r];
          if (row < 0) continue;
          const int base = k.ia[row] + off - fb;
#pragma unroll
          for (int c = 0; c < 3; c++)
            if (seq[le][bb][c] >= 0) k.al[base + seq[le][bb][c]] += K[r][c];
        }
      } else {  // rows of bb, columns of a: entry (bb c, a r) = K[r][c]
#pragma unroll
        for (int c = 0; c < 3; c++) {
          const int row = seq[le][bb][c];
          if (row < 0) continue;
          const int base = k.ia[row] + off - fa;
#pragma unroll
          for (int r = 0; r < 3; r++)
            if (seq[le][a][r] >= 0) k.al[base + seq[le][a][r]] += K[r][c];
        }
      }
    }
  }
  if (!with_u || b == nullptr) return;
  // K u over the team: fixed shuffle tree within the team's 8 lanes (other
  // teams of the warp may have left above)
#pragma unroll
  for (int off = 4; off > 0; off >>= 1)
#pragma unroll
    for (int a = 0; a < 8; a++)
#pragma unroll
      for (int d = 0; d < 3; d++) p[a][d] += __shfl_xor_sync(team_mask, p[a][d], off, 8);
  if (!active) return;
#pragma unroll
  for (int a = 0; a < 8; a++)
    if (a == lane)
#pragma unroll
      for (int d = 0; d < 3; d++)
        if (seq[le][a][d] >= 0) b[seq[le][a][d]] -= p[a][d];
}

// kHexDh for the current device, once per device.
void fill_hex_table(cudaStream_t st) {
  static std::mutex mu;
  static bool done[64] = {};
  int dev = 0;
  ELX_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  if (dev < 0 || dev >= 64 || done[dev]) return;
  static const double rn[8] = {1, -1, -1, 1, 1, -1, -1, 1};
  static const double sn[8] = {1, 1, -1, -1, 1, 1, -1, -1};
  static const double tn[8] = {1, 1, 1, 1, -1, -1, -1, -1};
  static const double pg[2] = {-.577350269189626e0, .577350269189626e0};
  static double h[8][3][8];
  for (int g = 0; g < 8; g++) {
    const double r = pg[g & 1], s = pg[(g >> 1) & 1], t = pg[g >> 2];
    for (int a = 0; a < 8; a++) {
      const double fr = 1.0 + rn[a] * r, fs = 1.0 + sn[a] * s, ft = 1.0 + tn[a] * t;
      h[g][0][a] = rn[a] * (fs * ft * 0.125);
      h[g][1][a] = sn[a] * (fr * ft * 0.125);
      h[g][2][a] = tn[a] * (fr * fs * 0.125);
    }
  }
  ELX_CUDA(cudaMemcpyToSymbolAsync(kHexDh, h, sizeof(h), 0, cudaMemcpyHostToDevice, st));
  ELX_CUDA(cudaStreamSynchronize(st));
  done[dev] = true;
}

}  // namespace

void launch_assembly(const MeshDev &m, const CsrcDev &k, const Segment &seg,
                     const double *u, double *b, int32_t *bad, cudaStream_t st) {
  const int n = seg.end - seg.begin;
  if (n <= 0) return;
  switch (seg.iel) {
    case TRIA3_STRAIN:
    case TRIA3_STRESS:
      tria3_kernel<<<(n + 127) / 128, 128, 0, st>>>(m, k, seg.begin, seg.end, seg.iel, u, b, bad);
      break;
    case QUAD4_STRAIN:
    case QUAD4_STRESS:
      quad4_kernel<<<(n + 127) / 128, 128, 0, st>>>(m, k, seg.begin, seg.end, seg.iel, u, b, bad);
      break;
    case TETRA4:
      tetra4_kernel<<<(n + 127) / 128, 128, 0, st>>>(m, k, seg.begin, seg.end, u, b, bad);
      break;
    case HEXA8: {
      static const bool team = !getenv("ELX_HEX_TEAM") || atoi(getenv("ELX_HEX_TEAM")) != 0;
      if (team) {
        fill_hex_table(st);
        hexa8_team_kernel<<<(n + kTeamElems - 1) / kTeamElems, 8 * kTeamElems, 0, st>>>(
            m, k, seg.begin, seg.end, u, b, bad);
      } else {
        ELX_CUDA(cudaFuncSetAttribute(hexa8_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kHexSmem));
        hexa8_kernel<<<(n + kHexThreads - 1) / kHexThreads, kHexThreads, kHexSmem, st>>>(
            m, k, seg.begin, seg.end, u, b, bad);
      }
      break;
    }
    default:
      throw Error{ELX_ERR_BAD_ELEMENT, "unsupported element type"};
  }
  ELX_CUDA(cudaGetLastError());
}

}  // namespace elx

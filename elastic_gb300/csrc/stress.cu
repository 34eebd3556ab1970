// Stress recovery on the GPU: tform_mec (mef/src/Pform.f:258-421) with the
// elements' isw = 3 (Elmlib02.f: TRIA3 235-250 / 525-540, QUAD4 836-846 /
// 1138-1148, TETRA4 1412-1437, HEXA8 1798-1812).
//
// One thread per element computes the stresses at its nodes -- constant
// for TRIA3 and TETRA4, at each node's natural coordinates for QUAD4 and
// HEXA8 (shape-function derivatives, Jacobian, strain, stress) -- and adds
// them to its nodes' sums, colour by colour (the colours of the assembly: no
// two elements of a colour share a node, so the adds need no atomics and the
// sums are deterministic).  A node pass then divides by the number of
// elements at the node and adds the initial stresses tx0.
// ntn = 4 (sxx, syy, szz, sxy) in 2-D, 6 (sxx, syy, szz, sxy, syz, sxz) in 3-D.
#include "elx_internal.h"

namespace elx {
namespace {

struct Law3 {
  double a, b, c, ps;
  bool plane_strain;
};

// Constitutive constants of elmt02-07_mec (Elmlib02.f:179-186, 469-476,
// 819-832, 1124-1134, 1402-1408, 1697-1705).
__device__ Law3 law_of(int iel, const double *e) {
  Law3 L;
  const double ym = e[0], ps = e[1];
  L.ps = ps;
  if (iel == TRIA3_STRESS || iel == QUAD4_STRESS) {
    L.a = ym / (1.0 - ps * ps);
    L.b = ps;
    L.c = 0.5 * (1.0 - ps);
    L.plane_strain = false;
  } else {
    const double a1 = 1.0 - ps, a2 = 1.0 - 2.0 * ps, a3 = 1.0 + ps;
    L.a = (ym * a1) / (a3 * a2);
    L.b = ps / a1;
    L.c = 0.5 * (a2 / a1);
    L.plane_strain = true;
  }
  return L;
}

// deform2d + stress2d_m (Elmlib.f:2368-2411, 2502-2538)
template <int N>
__device__ __forceinline__ void stress2d(const Law3 &L, const double (&hx)[N],
                                         const double (&hy)[N], const double (&u)[N][2],
                                         double *t) {
  double ux = 0.0, uy = 0.0, vx = 0.0, vy = 0.0;
#pragma unroll
  for (int i = 0; i < N; i++) {
    ux = ux + hx[i] * u[i][0];
    uy = uy + hy[i] * u[i][0];
    vx = vx + hx[i] * u[i][1];
    vy = vy + hy[i] * u[i][1];
  }
  const double e1 = ux, e2 = vy, e3 = uy + vx;
  const double d11 = L.a, d12 = L.a * L.b, d22 = L.a, d33 = L.a * L.c;
  t[0] = d11 * e1 + d12 * e2;
  t[1] = d12 * e1 + d22 * e2;
  t[2] = L.plane_strain ? L.ps * (t[0] + t[1]) : 0.0;
  t[3] = d33 * e3;
}

// deform3d + stress3d (Elmlib.f:2413-2471, 2540-2571)
template <int N>
__device__ __forceinline__ void stress3d(const Law3 &L, const double (&hx)[N],
                                         const double (&hy)[N], const double (&hz)[N],
                                         const double (&u)[N][3], double *t) {
  double ux = 0, uy = 0, uz = 0, vx = 0, vy = 0, vz = 0, wx = 0, wy = 0, wz = 0;
#pragma unroll
  for (int i = 0; i < N; i++) {
    ux = ux + hx[i] * u[i][0];
    uy = uy + hy[i] * u[i][0];
    uz = uz + hz[i] * u[i][0];
    vx = vx + hx[i] * u[i][1];
    vy = vy + hy[i] * u[i][1];
    vz = vz + hz[i] * u[i][1];
    wx = wx + hx[i] * u[i][2];
    wy = wy + hy[i] * u[i][2];
    wz = wz + hz[i] * u[i][2];
  }
  const double e1 = ux, e2 = vy, e3 = wz, e4 = uy + vx, e5 = vz + wy, e6 = uz + wx;
  const double a = L.a, b = L.b, c = L.c;
  t[0] = (e1 + b * e2 + b * e3) * a;
  t[1] = (b * e1 + e2 + b * e3) * a;
  t[2] = (b * e1 + b * e2 + e3) * a;
  t[3] = e4 * c * a;
  t[4] = e5 * c * a;
  t[5] = e6 * c * a;
}

template <int NEN, int NDM>
__device__ __forceinline__ void load_xu(const MeshDev &m, int t, const double *u, int (&node)[NEN],
                                        double (&xl)[NEN][NDM], double (&ul)[NEN][NDM]) {
#pragma unroll
  for (int a = 0; a < NEN; a++) {
    node[a] = m.conn[(size_t)a * m.numel + t];
#pragma unroll
    for (int d = 0; d < NDM; d++) {
      xl[a][d] = m.x[(size_t)node[a] * NDM + d];
      ul[a][d] = u[(size_t)node[a] * NDM + d];
    }
  }
}

template <int NEN, int NTN>
__device__ __forceinline__ void add_nodal(double *ts, const int (&node)[NEN],
                                          const double (&p)[NEN][NTN]) {
#pragma unroll
  for (int a = 0; a < NEN; a++)
#pragma unroll
    for (int j = 0; j < NTN; j++) ts[(size_t)node[a] * NTN + j] += p[a][j];
}

__global__ void tria3_stress_kernel(MeshDev m, int begin, int end, int iel,
                                    const double *__restrict__ u, double *ts, int32_t *bad) {
  const int t = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= end) return;
  int node[3];
  double xl[3][2], ul[3][2];
  load_xu<3, 2>(m, t, u, node, xl, ul);
  const Law3 L = law_of(iel, m.e + (size_t)m.mat[t] * m.prop);
  const double xj11 = xl[0][0] - xl[2][0], xj12 = xl[0][1] - xl[2][1];
  const double xj21 = xl[1][0] - xl[2][0], xj22 = xl[1][1] - xl[2][1];
  const double det = xj11 * xj22 - xj12 * xj21;
  if (det <= 0.0) {
    atomicMin(bad, m.elnum[t]);
    return;
  }
  const double i11 = xj22 / det, i12 = -xj12 / det, i21 = -xj21 / det, i22 = xj11 / det;
  const double hx[3] = {i11, i12, -i11 - i12}, hy[3] = {i21, i22, -i21 - i22};
  double p[3][4];
  stress2d<3>(L, hx, hy, ul, p[0]);
#pragma unroll
  for (int a = 1; a < 3; a++)
#pragma unroll
    for (int j = 0; j < 4; j++) p[a][j] = p[0][j];
  add_nodal<3, 4>(ts, node, p);
}

__global__ void quad4_stress_kernel(MeshDev m, int begin, int end, int iel,
                                    const double *__restrict__ u, double *ts, int32_t *bad) {
  const int t = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= end) return;
  int node[4];
  double xl[4][2], ul[4][2];
  load_xu<4, 2>(m, t, u, node, xl, ul);
  const Law3 L = law_of(iel, m.e + (size_t)m.mat[t] * m.prop);
  const double rn[4] = {1, -1, -1, 1}, sn[4] = {1, 1, -1, -1};
  double p[4][4];
#pragma unroll
  for (int n = 0; n < 4; n++) {
    // sfquad4_m derivatives (Elmlib.f:815-886) at the node, jacob2d_m (1769-1852)
    const double r = rn[n], s = sn[n];
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
    if (det <= 1.e-14) {
      atomicMin(bad, m.elnum[t]);
      return;
    }
    const double i11 = j22 / det, i12 = -j12 / det, i21 = -j21 / det, i22 = j11 / det;
    double hx[4], hy[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      hx[a] = i11 * hr[a] + i12 * hs[a];
      hy[a] = i21 * hr[a] + i22 * hs[a];
    }
    stress2d<4>(L, hx, hy, ul, p[n]);
  }
  add_nodal<4, 4>(ts, node, p);
}

__global__ void tetra4_stress_kernel(MeshDev m, int begin, int end, int iel,
                                     const double *__restrict__ u, double *ts, int32_t *bad) {
  const int t = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= end) return;
  int node[4];
  double xl[4][3], ul[4][3];
  load_xu<4, 3>(m, t, u, node, xl, ul);
  const Law3 L = law_of(iel, m.e + (size_t)m.mat[t] * m.prop);
  // jtetra4 (Elmlib.f:2636-2713)
  const double xj11 = xl[0][0] - xl[3][0], xj12 = xl[0][1] - xl[3][1], xj13 = xl[0][2] - xl[3][2];
  const double xj21 = xl[1][0] - xl[3][0], xj22 = xl[1][1] - xl[3][1], xj23 = xl[1][2] - xl[3][2];
  const double xj31 = xl[2][0] - xl[3][0], xj32 = xl[2][1] - xl[3][1], xj33 = xl[2][2] - xl[3][2];
  const double det = xj11 * xj22 * xj33 + xj12 * xj23 * xj31 + xj13 * xj21 * xj32 -
                     xj31 * xj22 * xj13 - xj12 * xj21 * xj33 - xj11 * xj32 * xj23;
  if (det <= 1.e-14) {
    atomicMin(bad, m.elnum[t]);
    return;
  }
  const double di = 1.0 / det;
  double hx[4], hy[4], hz[4];
  hx[0] = (xj22 * xj33 - xj23 * xj32) * di;
  hx[1] = (xj13 * xj32 - xj12 * xj33) * di;
  hx[2] = (xj12 * xj23 - xj13 * xj22) * di;
  hy[0] = (xj23 * xj31 - xj21 * xj33) * di;
  hy[1] = (xj11 * xj33 - xj13 * xj31) * di;
  hy[2] = (xj13 * xj21 - xj11 * xj23) * di;
  hz[0] = (xj21 * xj32 - xj22 * xj31) * di;
  hz[1] = (xj12 * xj31 - xj11 * xj32) * di;
  hz[2] = (xj11 * xj22 - xj12 * xj21) * di;
  hx[3] = -hx[0] - hx[1] - hx[2];
  hy[3] = -hy[0] - hy[1] - hy[2];
  hz[3] = -hz[0] - hz[1] - hz[2];
  double p[4][6];
  stress3d<4>(L, hx, hy, hz, ul, p[0]);
#pragma unroll
  for (int a = 1; a < 4; a++)
#pragma unroll
    for (int j = 0; j < 6; j++) p[a][j] = p[0][j];
  add_nodal<4, 6>(ts, node, p);
}

// Eight threads per element, thread n for the element's node n (the nodes'
// stresses are independent): the same per-node arithmetic as one thread per
// element, so the sums are bitwise the same, with 8x the threads per colour
// (elx_stress on the 64^3 cube, its 13 MB copy back included: 2.24 against
// 2.40 ms).
__global__ void __launch_bounds__(128)
hexa8_stress_kernel(MeshDev m, int begin, int end, int iel, const double *__restrict__ u,
                    double *ts, int32_t *bad) {
  const int t = begin + (blockIdx.x * blockDim.x + threadIdx.x) / 8;
  const int n = threadIdx.x % 8;
  if (t >= end) return;
  int node[8];
  double xl[8][3], ul[8][3];
  load_xu<8, 3>(m, t, u, node, xl, ul);
  const Law3 L = law_of(iel, m.e + (size_t)m.mat[t] * m.prop);
  const double rn[8] = {1, -1, -1, 1, 1, -1, -1, 1};
  const double sn[8] = {1, 1, -1, -1, 1, 1, -1, -1};
  const double tn[8] = {1, 1, 1, 1, -1, -1, -1, -1};
  {
    // sfhexa8_m derivatives (Elmlib.f:1151-1258) at the node, jacob3d_m (1942-2036)
    const double pR = 1.0 + rn[n], pS = 1.0 + sn[n], pT = 1.0 + tn[n];
    const double mR = 1.0 - rn[n], mS = 1.0 - sn[n], mT = 1.0 - tn[n];
    const double hr[8] = {pS * pT * 0.125, -(pS * pT * 0.125), -(mS * pT * 0.125),
                          mS * pT * 0.125, pS * mT * 0.125,    -(pS * mT * 0.125),
                          -(mS * mT * 0.125), mS * mT * 0.125};
    const double hs[8] = {pR * pT * 0.125, mR * pT * 0.125,    -(mR * pT * 0.125),
                          -(pR * pT * 0.125), pR * mT * 0.125, mR * mT * 0.125,
                          -(mR * mT * 0.125), -(pR * mT * 0.125)};
    const double ht[8] = {pR * pS * 0.125,    mR * pS * 0.125,    mR * mS * 0.125,
                          pR * mS * 0.125,    -(pR * pS * 0.125), -(mR * pS * 0.125),
                          -(mR * mS * 0.125), -(pR * mS * 0.125)};
    double xj[3][3];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      xj[0][j] = 0.0;
      xj[1][j] = 0.0;
      xj[2][j] = 0.0;
#pragma unroll
      for (int a = 0; a < 8; a++) {
        xj[0][j] = xj[0][j] + hr[a] * xl[a][j];
        xj[1][j] = xj[1][j] + hs[a] * xl[a][j];
        xj[2][j] = xj[2][j] + ht[a] * xl[a][j];
      }
    }
    const double det = xj[0][0] * xj[1][1] * xj[2][2] + xj[0][1] * xj[1][2] * xj[2][0] +
                       xj[0][2] * xj[1][0] * xj[2][1] - xj[2][0] * xj[1][1] * xj[0][2] -
                       xj[1][0] * xj[0][1] * xj[2][2] - xj[0][0] * xj[2][1] * xj[1][2];
    if (det <= 1.e-14) {
      atomicMin(bad, m.elnum[t]);
      return;
    }
    double xi[3][3];
    xi[0][0] = (xj[1][1] * xj[2][2] - xj[1][2] * xj[2][1]) / det;
    xi[1][0] = -(xj[1][0] * xj[2][2] - xj[1][2] * xj[2][0]) / det;
    xi[2][0] = (xj[1][0] * xj[2][1] - xj[1][1] * xj[2][0]) / det;
    xi[0][1] = -(xj[0][1] * xj[2][2] - xj[0][2] * xj[2][1]) / det;
    xi[1][1] = (xj[0][0] * xj[2][2] - xj[0][2] * xj[2][0]) / det;
    xi[2][1] = -(xj[0][0] * xj[2][1] - xj[0][1] * xj[2][0]) / det;
    xi[0][2] = (xj[0][1] * xj[1][2] - xj[0][2] * xj[1][1]) / det;
    xi[1][2] = -(xj[0][0] * xj[1][2] - xj[0][2] * xj[1][0]) / det;
    xi[2][2] = (xj[0][0] * xj[1][1] - xj[0][1] * xj[1][0]) / det;
    double hx[8], hy[8], hz[8];
#pragma unroll
    for (int a = 0; a < 8; a++) {
      hx[a] = xi[0][0] * hr[a] + xi[0][1] * hs[a] + xi[0][2] * ht[a];
      hy[a] = xi[1][0] * hr[a] + xi[1][1] * hs[a] + xi[1][2] * ht[a];
      hz[a] = xi[2][0] * hr[a] + xi[2][1] * hs[a] + xi[2][2] * ht[a];
    }
    double p[6];
    stress3d<8>(L, hx, hy, hz, ul, p);
#pragma unroll
    for (int j = 0; j < 6; j++) ts[(size_t)node[n] * 6 + j] += p[j];
  }
}

// t = t / ic + tx0 per node (the average of Pform.f:411-415).
__global__ void stress_average_kernel(int nnode, int ntn, const int32_t *__restrict__ count,
                                      const double *__restrict__ tx0, double *__restrict__ ts) {
  const int64_t n = (int64_t)nnode * ntn;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x)
    ts[q] = ts[q] / count[q / ntn] + (tx0 ? tx0[q] : 0.0);
}

// update_mec on the device (Predict.f:183-209): u(j,i) = x(id(j,i)) for the
// free dofs; eq is id - 1 (-1 for fixed dofs, whose u stays as prescribed).
__global__ void update_kernel(int64_t n, const int32_t *__restrict__ eq,
                              const double *__restrict__ x, double *__restrict__ u) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int e = eq[q];
    if (e >= 0) u[q] = x[e];
  }
}

}  // namespace

void launch_update(int64_t n, const int32_t *eq, const double *x, double *u, cudaStream_t st) {
  const int grid = (int)std::min<int64_t>((n + 255) / 256, grid_cap(8));
  update_kernel<<<std::max(grid, 1), 256, 0, st>>>(n, eq, x, u);
  ELX_CUDA(cudaGetLastError());
}

void launch_stress(const MeshDev &m, const Segment &seg, const double *u, double *ts,
                   int32_t *bad, cudaStream_t st) {
  const int n = seg.end - seg.begin;
  if (n <= 0) return;
  switch (seg.iel) {
    case TRIA3_STRAIN:
    case TRIA3_STRESS:
      tria3_stress_kernel<<<(n + 127) / 128, 128, 0, st>>>(m, seg.begin, seg.end, seg.iel, u, ts,
                                                           bad);
      break;
    case QUAD4_STRAIN:
    case QUAD4_STRESS:
      quad4_stress_kernel<<<(n + 127) / 128, 128, 0, st>>>(m, seg.begin, seg.end, seg.iel, u, ts,
                                                           bad);
      break;
    case TETRA4:
      tetra4_stress_kernel<<<(n + 127) / 128, 128, 0, st>>>(m, seg.begin, seg.end, seg.iel, u,
                                                            ts, bad);
      break;
    case HEXA8:
      hexa8_stress_kernel<<<(8 * n + 127) / 128, 128, 0, st>>>(m, seg.begin, seg.end, seg.iel, u,
                                                               ts, bad);
      break;
    default:
      throw Error{ELX_ERR_BAD_ELEMENT, "unsupported element type"};
  }
  ELX_CUDA(cudaGetLastError());
}

void launch_stress_average(int nnode, int ntn, const int32_t *count, const double *tx0,
                           double *ts, cudaStream_t st) {
  const int64_t n = (int64_t)nnode * ntn;
  const int grid = (int)std::min<int64_t>((n + 255) / 256, grid_cap(8));
  stress_average_kernel<<<std::max(grid, 1), 256, 0, st>>>(nnode, ntn, count, tx0, ts);
  ELX_CUDA(cudaGetLastError());
}

}  // namespace elx

// The result file of write_mesh_res_mec (mef/src/Write_vtk.f:742-985, with
// the record writers of Vtk.f) formatted on the GPU from the resident mesh,
// displacements and nodal stresses.
//
// Every data record of the file has a fixed width -- a coordinate line is
// three E15.5 fields and a newline, a stress line nine E15.5E3 fields, a
// connectivity line nnoel I10 fields, a binary record a fixed number of
// big-endian words -- so the file is laid out on the host (header strings
// and the offset of each section) and one thread per node or element writes
// its record at offset + index * width.  The host copies the finished buffer
// back once and writes it with one fwrite.
//
// Numbers are printed as gfortran prints the reference's edit descriptors:
// Ew.d[Ee] as [-]0.ddddd followed by the exponent, digits correctly rounded
// (ties to even).  The rounding is exact for every double: the digits are
// first estimated in floating point, then fixed by comparing the value with
// the decimal boundaries N * 10^s and (N + 1/2) * 10^s in integer
// arithmetic (a double is m * 2^q; 10^s = 5^s * 2^s, so each comparison is
// between two integers of at most ~830 bits).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <string>

#include "elx_internal.h"

namespace elx {
namespace {

// ---------------------------------------------------------------- integers
constexpr int kLimbs = 36;  // 1152 bits: the largest comparison needs ~830

struct Big {
  uint32_t w[kLimbs];
  int n;
};

__device__ void big_set(Big &b, uint64_t v) {
  b.w[0] = (uint32_t)v;
  b.w[1] = (uint32_t)(v >> 32);
  b.n = b.w[1] ? 2 : 1;
}

__device__ void big_mul(Big &b, uint32_t f) {
  uint64_t carry = 0;
  for (int i = 0; i < b.n; i++) {
    const uint64_t t = (uint64_t)b.w[i] * f + carry;
    b.w[i] = (uint32_t)t;
    carry = t >> 32;
  }
  if (carry && b.n < kLimbs) b.w[b.n++] = (uint32_t)carry;
}

__device__ void big_pow5(Big &b, int k) {
  // 5^13 is the largest power of 5 below 2^32
  const uint32_t p5[13] = {1u,      5u,       25u,       125u,       625u,
                           3125u,   15625u,   78125u,    390625u,    1953125u,
                           9765625u, 48828125u, 244140625u};
  for (; k >= 13; k -= 13) big_mul(b, 1220703125u);
  if (k) big_mul(b, p5[k]);
}

__device__ void big_shl(Big &b, int s) {
  const int limbs = s >> 5, bits = s & 31;
  if (s <= 0) return;
  int n = b.n + limbs + 1;
  if (n > kLimbs) n = kLimbs;
  for (int i = n - 1; i >= 0; i--) {
    const int src = i - limbs;
    uint32_t hi = src >= 0 && src < b.n ? b.w[src] : 0u;
    uint32_t lo = src - 1 >= 0 && src - 1 < b.n ? b.w[src - 1] : 0u;
    b.w[i] = bits ? (hi << bits) | (lo >> (32 - bits)) : hi;
  }
  b.n = n;
  while (b.n > 1 && b.w[b.n - 1] == 0) b.n--;
}

__device__ int big_cmp(const Big &a, const Big &b) {
  if (a.n != b.n) return a.n < b.n ? -1 : 1;
  for (int i = a.n - 1; i >= 0; i--)
    if (a.w[i] != b.w[i]) return a.w[i] < b.w[i] ? -1 : 1;
  return 0;
}

// sign of m * 2^q - c * 10^s
__device__ int cmp_scaled(uint64_t m, int q, uint64_t c, int s) {
  Big L, R;
  big_set(L, m);
  big_set(R, c);
  if (s >= 0)
    big_pow5(R, s);
  else
    big_pow5(L, -s);
  const int t = q - s;  // L * 2^q vs R * 2^s
  if (t >= 0)
    big_shl(L, t);
  else
    big_shl(R, -t);
  return big_cmp(L, R);
}

// a > 0 finite: the d-digit N (10^(d-1) <= N < 10^d) and E with
// a = 0.N * 10^E, N correctly rounded (ties to even).
__device__ void dec_round(double a, int d, uint32_t &N_out, int &E) {
  int e2;
  const double f = frexp(a, &e2);
  const uint64_t m = (uint64_t)ldexp(f, 53);
  const int q = e2 - 53;
  E = (int)floor(log10(a)) + 1;
  while (cmp_scaled(m, q, 1, E - 1) < 0) E--;  // a < 10^(E-1)
  while (cmp_scaled(m, q, 1, E) >= 0) E++;     // a >= 10^E
  const int s = E - d;
  uint64_t lo = 1, hi;
  for (int i = 1; i < d; i++) lo *= 10;
  hi = lo * 10 - 1;
  const int h = -s / 2;
  double est = floor(a * pow(10.0, (double)h) * pow(10.0, (double)(-s - h)));
  uint64_t N = est < (double)lo ? lo : est > (double)hi ? hi : (uint64_t)est;
  while (N > lo && cmp_scaled(m, q, N, s) < 0) N--;           // a < N 10^s
  while (N < hi && cmp_scaled(m, q, N + 1, s) >= 0) N++;      // a >= (N+1) 10^s
  const int r = cmp_scaled(m, q + 1, 2 * N + 1, s);           // a vs (N + 1/2) 10^s
  if (r > 0 || (r == 0 && (N & 1))) N++;
  if (N > hi) {
    N = lo;
    E++;
  }
  N_out = (uint32_t)N;
}

// ---------------------------------------------------------------- fields
// Ew.d (e = 0) / Ew.dEe, as gfortran writes them (see the oracle's
// orc_fmt_e for the same rules on the host).
__device__ void put_e(char *out, double x, int w, int d, int e) {
  char body[40];
  int n = 0;
  bool ok = true;
  if (isnan(x)) {
    body[0] = 'N', body[1] = 'a', body[2] = 'N';
    n = 3;
  } else if (isinf(x)) {
    const char *s = x < 0 ? (w >= 9 ? "-Infinity" : "-Inf") : (w >= 8 ? "Infinity" : "Inf");
    while (s[n]) body[n] = s[n], n++;
  } else {
    uint32_t N = 0;
    int E = 0;
    const double a = fabs(x);
    if (a != 0.0) dec_round(a, d, N, E);
    if (signbit(x)) body[n++] = '-';
    body[n++] = '0';
    body[n++] = '.';
    char dig[12];
    for (int i = d - 1; i >= 0; i--) dig[i] = (char)('0' + N % 10), N /= 10;
    for (int i = 0; i < d; i++) body[n++] = dig[i];
    const int ae = E < 0 ? -E : E;
    int ed;
    if (e == 0) {
      if (ae <= 99) {
        body[n++] = 'E';
        ed = 2;
      } else if (ae <= 999) {
        ed = 3;
      } else {
        ok = false;
        ed = 0;
      }
    } else {
      int lim = 1;
      for (int i = 0; i < e; i++) lim *= 10;
      ok = ae < lim;
      body[n++] = 'E';
      ed = e;
    }
    if (ok) {
      body[n++] = E < 0 ? '-' : '+';
      int v = ae;
      for (int i = ed - 1; i >= 0; i--) body[n + i] = (char)('0' + v % 10), v /= 10;
      n += ed;
    }
    if (ok && n == w + 1) {  // drop the optional leading zero
      const int z = body[0] == '-' ? 1 : 0;
      for (int i = z; i < n - 1; i++) body[i] = body[i + 1];
      n--;
    }
  }
  if (!ok || n > w) {
    for (int i = 0; i < w; i++) out[i] = '*';
    return;
  }
  for (int i = 0; i < w - n; i++) out[i] = ' ';
  for (int i = 0; i < n; i++) out[w - n + i] = body[i];
}

__device__ void put_i(char *out, long long v, int w) {
  char body[24];
  int n = 0;
  unsigned long long u = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  do {
    body[n++] = (char)('0' + u % 10);
    u /= 10;
  } while (u);
  if (v < 0) body[n++] = '-';
  if (n > w) {
    for (int i = 0; i < w; i++) out[i] = '*';
    return;
  }
  for (int i = 0; i < w - n; i++) out[i] = ' ';
  for (int i = 0; i < n; i++) out[w - 1 - i] = body[i];
}

__device__ void put_be32(char *out, uint32_t v) {
  out[0] = (char)(v >> 24);
  out[1] = (char)(v >> 16);
  out[2] = (char)(v >> 8);
  out[3] = (char)v;
}

__device__ void put_be64(char *out, double x) {
  const uint64_t v = (uint64_t)__double_as_longlong(x);
  for (int i = 0; i < 8; i++) out[i] = (char)(v >> (56 - 8 * i));
}

// make_full_tensor (Write_vtk.f:1166-1226): component j of node i's tensor.
__device__ double tensor9(const double *tx, int ntn, int i, int j) {
  const double *s = tx + (size_t)i * ntn;
  const int map4[9] = {0, 3, -1, 3, 1, -1, -1, -1, 2};
  const int map6[9] = {0, 3, 5, 3, 1, 4, 5, 4, 2};
  const int k = ntn == 4 ? map4[j] : map6[j];
  return k < 0 ? 0.0 : s[k];
}

struct Sec {
  int kind;
  int64_t off;
};

// Record kinds (one thread per node or element).
enum {
  kCoordA,    // 3 x E15.5 + '\n'                     (node)
  kConnA,     // nnoel x I10 + '\n'                   (element)
  kOffsA,     // I20 + '\n'                           (element)
  kTypesA,    // I3 + '\n'                            (element)
  kMatA,      // I9 + '\n'                            (element)
  kElIdA,     // I9 + '\n'                            (element)
  kNodeIdA,   // I10 + '\n'                           (node)
  kDeslocA,   // ndf x E15.5E3 + '\n'                 (node)
  kStressA,   // 9 x E15.5E3 + '\n'                   (node)
  kCoordB,    // 3 big-endian doubles                 (node)
  kConnB,     // (nnoel + 1) big-endian int32         (element)
  kTypesB,    // int32                                (element)
  kMatB,      // int32                                (element)
  kElIdB,     // int32                                (element)
  kNodeIdB,   // int32                                (node)
  kDeslocB,   // 3 big-endian doubles                 (node)
  kStressB,   // 9 big-endian doubles                 (node)
};

struct VtkArgs {
  char *buf;
  int nnode, numel, ndm, ndf, ntn, nnoel, ctype;
  const double *x, *u, *tx;
  const int32_t *conn, *mat, *elnum;
};

__device__ int record_width(int kind, const VtkArgs &A) {
  switch (kind) {
    case kCoordA: return 46;
    case kConnA: return 10 * A.nnoel + 1;
    case kOffsA: return 21;
    case kTypesA: return 4;
    case kMatA: case kElIdA: return 10;
    case kNodeIdA: return 11;
    case kDeslocA: return 15 * A.ndf + 1;
    case kStressA: return 136;
    case kCoordB: case kDeslocB: return 24;
    case kConnB: return 4 * (A.nnoel + 1);
    case kTypesB: case kMatB: case kElIdB: case kNodeIdB: return 4;
    case kStressB: return 72;
  }
  return 0;
}

__global__ void vtk_section_kernel(VtkArgs A, Sec sec, int count) {
  const int w = record_width(sec.kind, A);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < count; t += gridDim.x * blockDim.x) {
    // element records go to the element's place in the reference's order
    int r = t;
    const bool by_elem = sec.kind == kConnA || sec.kind == kMatA || sec.kind == kConnB ||
                         sec.kind == kMatB;
    if (by_elem) r = A.elnum[t] - 1;
    char *o = A.buf + sec.off + (int64_t)r * w;
    switch (sec.kind) {
      case kCoordA:
        for (int j = 0; j < 3; j++)
          put_e(o + 15 * j, j < A.ndm ? A.x[(size_t)t * A.ndm + j] : 0.0, 15, 5, 0);
        o[45] = '\n';
        break;
      case kConnA:
        for (int a = 0; a < A.nnoel; a++) put_i(o + 10 * a, A.conn[(size_t)a * A.numel + t], 10);
        o[10 * A.nnoel] = '\n';
        break;
      case kOffsA:
        put_i(o, (long long)(t + 1) * A.nnoel, 20);
        o[20] = '\n';
        break;
      case kTypesA:
        put_i(o, A.ctype, 3);
        o[3] = '\n';
        break;
      case kMatA:
        put_i(o, A.mat[t] + 1, 9);
        o[9] = '\n';
        break;
      case kElIdA:
        put_i(o, t + 1, 9);
        o[9] = '\n';
        break;
      case kNodeIdA:
        put_i(o, t + 1, 10);
        o[10] = '\n';
        break;
      case kDeslocA:
        for (int j = 0; j < A.ndf; j++) put_e(o + 15 * j, A.u[(size_t)t * A.ndf + j], 15, 5, 3);
        o[15 * A.ndf] = '\n';
        break;
      case kStressA:
        for (int j = 0; j < 9; j++) put_e(o + 15 * j, tensor9(A.tx, A.ntn, t, j), 15, 5, 3);
        o[135] = '\n';
        break;
      case kCoordB:
        for (int j = 0; j < 3; j++) put_be64(o + 8 * j, j < A.ndm ? A.x[(size_t)t * A.ndm + j] : 0.0);
        break;
      case kConnB:
        put_be32(o, (uint32_t)A.nnoel);
        for (int a = 0; a < A.nnoel; a++)
          put_be32(o + 4 + 4 * a, (uint32_t)A.conn[(size_t)a * A.numel + t]);
        break;
      case kTypesB:
        put_be32(o, (uint32_t)A.ctype);
        break;
      case kMatB:
        put_be32(o, (uint32_t)(A.mat[t] + 1));
        break;
      case kElIdB:
        put_be32(o, (uint32_t)(t + 1));
        break;
      case kNodeIdB:
        put_be32(o, (uint32_t)(t + 1));
        break;
      case kDeslocB:
        for (int j = 0; j < 3; j++)
          put_be64(o + 8 * j, j < A.ndm ? A.u[(size_t)t * A.ndf + j] : 0.0);
        break;
      case kStressB:
        for (int j = 0; j < 9; j++) put_be64(o + 8 * j, tensor9(A.tx, A.ntn, t, j));
        break;
    }
  }
}

// Formatter test hook: n fields Ew.d[Ee] of x into out (n * w chars).
__global__ void fortran_e_kernel(const double *x, int n, int w, int d, int e, char *out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    put_e(out + (size_t)i * w, x[i], w, d, e);
}

int host_width(int kind, int nnoel, int ndf) {
  switch (kind) {
    case kCoordA: return 46;
    case kConnA: return 10 * nnoel + 1;
    case kOffsA: return 21;
    case kTypesA: return 4;
    case kMatA: case kElIdA: return 10;
    case kNodeIdA: return 11;
    case kDeslocA: return 15 * ndf + 1;
    case kStressA: return 136;
    case kCoordB: case kDeslocB: return 24;
    case kConnB: return 4 * (nnoel + 1);
    case kTypesB: case kMatB: case kElIdB: case kNodeIdB: return 4;
    case kStressB: return 72;
  }
  return 0;
}

bool node_kind(int kind) {
  return kind == kCoordA || kind == kNodeIdA || kind == kDeslocA || kind == kStressA ||
         kind == kCoordB || kind == kNodeIdB || kind == kDeslocB || kind == kStressB;
}

std::string fmt(const char *f, ...) __attribute__((format(printf, 1, 2)));
std::string fmt(const char *f, ...) {
  char b[512];
  va_list ap;
  va_start(ap, f);
  vsnprintf(b, sizeof b, f, ap);
  va_end(ap);
  return b;
}

}  // namespace

// The file as pieces: host strings and device sections, in file order.
void VtkLayout::add_text(const std::string &s) {
  texts.push_back({size, s});
  size += (int64_t)s.size();
}
void VtkLayout::add_section(int kind, int count, int nnoel, int ndf) {
  sections.push_back({kind, size, count});
  size += (int64_t)count * host_width(kind, nnoel, ndf);
}

// write_mesh_res_mec's record sequence (format 0: VTU ASCII, 1: legacy
// binary); fields & 1: desloc, fields & 2: stress.
VtkLayout vtk_layout(int format, int fields, int nnode, int numel, int ndf, int nnoel,
                     int ctype) {
  VtkLayout L;
  if (format == 0) {
    L.add_text("<?xml version=\"1.0\"?>\n"
               "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"BigEndian\">\n"
               "<UnstructuredGrid>\n");
    L.add_text(fmt("<Piece NumberOfPoints=\"%15d\" NumberOfCells=\"%15d\">\n", nnode, numel));
    L.add_text("<Points>\n"
               "<DataArray type=\"Float64\" NumberOfComponents =\"3\" format=\"ascii\">\n");
    L.add_section(kCoordA, nnode, nnoel, ndf);
    L.add_text("</DataArray>\n</Points>\n<Cells> \n"
               "<DataArray type=\"Int32\" Name=\"connectivity\" format=\"ascii\">\n");
    L.add_section(kConnA, numel, nnoel, ndf);
    L.add_text("</DataArray>\n<DataArray type=\"Int64\" Name=\"offsets\" format=\"ascii\">\n");
    L.add_section(kOffsA, numel, nnoel, ndf);
    L.add_text("</DataArray>\n<DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n");
    L.add_section(kTypesA, numel, nnoel, ndf);
    L.add_text("</DataArray>\n</Cells>\n<CellData Scalars=\"scalars\">\n"
               "<DataArray type=\"Int32\" NumberOfComponents=\"1\" Name=\"mat\" "
               "format=\"ascii\">\n");
    L.add_section(kMatA, numel, nnoel, ndf);
    L.add_text("</DataArray>\n<DataArray type=\"Int32\" NumberOfComponents=\"1\" "
               "Name=\"elIdG\" format=\"ascii\">\n");
    L.add_section(kElIdA, numel, nnoel, ndf);
    L.add_text("</DataArray>\n</CellData>\n<PointData>\n"
               "<DataArray type=\"Int32\" NumberOfComponents=\" 1\" Name=\"noIdG\" "
               "format=\"ascii\">\n");
    L.add_section(kNodeIdA, nnode, nnoel, ndf);
    L.add_text("</DataArray>\n");
    if (fields & 1) {
      L.add_text(fmt("<DataArray type=\"Float64\" NumberOfComponents=\"%2d\" Name=\"desloc\" "
                     "format=\"ascii\">\n",
                     ndf));
      L.add_section(kDeslocA, nnode, nnoel, ndf);
      L.add_text("</DataArray>\n");
    }
    if (fields & 2) {
      L.add_text("<DataArray type=\"Float64\" NumberOfComponents=\"9\" Name=\"stress\" "
                 "format=\"ascii\">\n");
      L.add_section(kStressA, nnode, nnoel, ndf);
      L.add_text("</DataArray>\n");
    }
    L.add_text("</PointData>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n");
  } else {
    L.add_text(fmt("# vtk DataFile Version 3.0\n%-30s\nBINARY\nDATASET UNSTRUCTURED_GRID\n",
                   "Malha Res"));
    L.add_text(fmt("POINTS %15d double\n", nnode));
    L.add_section(kCoordB, nnode, nnoel, ndf);
    L.add_text(fmt("\nCELLS %15d%15d\n", numel, (nnoel + 1) * numel));
    L.add_section(kConnB, numel, nnoel, ndf);
    L.add_text(fmt("\nCELL_TYPES %15d\n", numel));
    L.add_section(kTypesB, numel, nnoel, ndf);
    L.add_text(fmt("\nCELL_DATA %8d\n", numel));
    L.add_text(fmt("SCALARS %-15s int%8d\nLOOKUP_TABLE default\n", "mat", 1));
    L.add_section(kMatB, numel, nnoel, ndf);
    L.add_text(fmt("SCALARS %-15s int%8d\nLOOKUP_TABLE default\n", "elIdG", 1));
    L.add_section(kElIdB, numel, nnoel, ndf);
    L.add_text(fmt("\n POINT_DATA %8d\n", nnode));
    L.add_text(fmt(" SCALARS %-15s int %6d\n LOOKUP_TABLE default \n", "noIdG", 1));
    L.add_section(kNodeIdB, nnode, nnoel, ndf);
    if (fields & 1) {
      L.add_text(fmt(" VECTORS %-15s double\n", "desloc"));
      L.add_section(kDeslocB, nnode, nnoel, ndf);
    }
    if (fields & 2) {
      L.add_text(fmt(" TENSORS %-15s double\n", "stress"));
      L.add_section(kStressB, nnode, nnoel, ndf);
    }
  }
  (void)ctype;
  return L;
}

void launch_vtk(const VtkLayout &L, char *dbuf, const MeshDev &m, int ntn, int nnoel, int ctype,
                const double *u, const double *tx, cudaStream_t st) {
  VtkArgs A;
  A.buf = dbuf;
  A.nnode = m.nnode;
  A.numel = m.numel;
  A.ndm = m.ndm;
  A.ndf = m.ndf;
  A.ntn = ntn;
  A.nnoel = nnoel;
  A.ctype = ctype;
  A.x = m.x;
  A.u = u;
  A.tx = tx;
  A.conn = m.conn;
  A.mat = m.mat;
  A.elnum = m.elnum;
  for (const VtkLayout::Text &t : L.texts)
    ELX_CUDA(cudaMemcpyAsync(dbuf + t.off, t.s.data(), t.s.size(), cudaMemcpyHostToDevice, st));
  for (const VtkLayout::Section &s : L.sections) {
    if (s.count <= 0) continue;
    const int grid = std::max(1, std::min((s.count + 255) / 256, grid_cap(8)));
    vtk_section_kernel<<<grid, 256, 0, st>>>(A, Sec{s.kind, s.off}, s.count);
    ELX_CUDA(cudaGetLastError());
  }
  (void)node_kind;
}

void launch_fortran_e(const double *x, int n, int w, int d, int e, char *out, cudaStream_t st) {
  if (n <= 0) return;
  fortran_e_kernel<<<std::max(1, std::min((n + 255) / 256, grid_cap(8))), 256, 0, st>>>(x, n, w, d, e,
                                                                                 out);
  ELX_CUDA(cudaGetLastError());
}

}  // namespace elx

/*
 * elx_oracle.c -- CPU restatement of Elastic's linear-elasticity solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle: the tests,
 * the smoke check and the CPU-baseline leg of the benchmark call it to check
 * (or time, as the reference's CPU path) the CUDA library in elastic_gb300/.
 * The product never links, loads or calls it.
 *
 * Every routine restates one Fortran routine of the reference (lmn-labest/
 * Elastic, directory mef/src) and cites it.  Arrays keep the reference's
 * conventions: 1-based *contents* (node numbers, equation numbers, ia/ja
 * positions), column-major multi-dimensional arrays, 4-byte integers and
 * real*8.  The C arrays themselves are 0-based, so the accessor macros below
 * subtract one.  Floating-point expressions keep the reference's operand order;
 * the build passes -ffp-contract=off so that no FMA contraction changes the
 * rounding on either host architecture.
 *
 * Sorting: the reference sorts adjacency lists and CSR rows with a bubble sort
 * (Graph.f:235-257).  The sorted result of distinct integers does not depend on
 * the algorithm, so an insertion sort with the same ascending order is used.
 */
#include <math.h>
#include <stdio.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_ERR_ZERO_DIAG 1
#define ORC_ERR_NO_CONVERGENCE 2
#define ORC_ERR_BAD_DET 3
#define ORC_ERR_OOM 4
#define ORC_ERR_ARG 6
#define ORC_ERR_BAD_ELEMENT 7

static double wall(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ---------------------------------------------------------------------- */
/* Graph.f:20-257 -- node adjacency                                        */
/* ---------------------------------------------------------------------- */

/* Graph.f:235-257 bubblesort (same ascending result, see header). */
static void sort_asc(int *a, int n) {
  for (int i = 1; i < n; i++) {
    int v = a[i], j = i - 1;
    while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; j--; }
    a[j + 1] = v;
  }
}

/* Graph.f:20-71 graph (aponta + graph0 + graph1).
 * ix is (nen+1, numel) column-major with 1-based node numbers.
 * Outputs malloc'ed 1-based arrays: ip[1..nnode+1] (ip[0] unused) and
 * ips[0..] holding the adjacency (positions ip[i]..ip[i+1]-1, 1-based). */
static int graph(const int *ix, int nnode, int numel, int nen, int **ip_out,
                 int **ips_out) {
  const int nen1 = nen + 1;
#define IX(j, i) ix[(size_t)((i) - 1) * nen1 + ((j) - 1)]
  int *ip = (int *)calloc((size_t)nnode + 2, sizeof(int));
  if (!ip) return ORC_ERR_OOM;
  /* aponta (Graph.f:72-108) */
  ip[1] = 1;
  for (int i = 1; i <= numel; i++)
    for (int j = 1; j <= nen; j++) {
      int no = IX(j, i);
      if (no == 0 || no > nnode) continue;
      ip[no + 1] += nen - 1;
    }
  for (int i = 2; i <= nnode + 1; i++) ip[i] += ip[i - 1];
  int ipos = ip[nnode + 1] - 1;
  size_t cap = (size_t)(ipos > nnode ? ipos : nnode) + 2;
  int *ips = (int *)calloc(cap, sizeof(int));   /* 1-based */
  int *noviz = (int *)calloc(cap, sizeof(int)); /* 1-based */
  if (!ips || !noviz) { free(ip); free(ips); free(noviz); return ORC_ERR_OOM; }
  /* graph0 (Graph.f:109-149) */
  for (int i = 1; i <= numel; i++)
    for (int j = 1; j <= nen; j++) {
      int noj = IX(j, i);
      if (noj == 0 || noj > nnode) continue;
      for (int k = 1; k <= nen; k++) {
        int nok = IX(k, i);
        if (nok == 0 || nok > nnode) continue;
        if (nok == noj) continue;
        int pos = ip[noj] + ips[noj];
        ips[noj] += 1;
        noviz[pos] = nok;
      }
    }
  /* graph1 (Graph.f:150-208) */
  for (int i = 1; i <= nnode; i++) sort_asc(&noviz[ip[i]], ip[i + 1] - ip[i]);
  for (int i = 1; i <= nnode; i++) {
    int l = ip[i], k = ip[i + 1] - 2;
    for (int j = l; j <= k; j++) {
      int no = noviz[j];
      if (no != 0 && noviz[j + 1] == no) { noviz[j] = 0; ips[i] -= 1; }
    }
  }
  for (int i = 1; i <= nnode; i++) ip[i + 1] = ip[i] + ips[i];
  int j = 1;
  for (int i = 1; i <= ipos; i++)
    if (noviz[i] != 0) ips[j++] = noviz[i];
  free(noviz);
  /* shift ips to a 0-based array whose element p-1 is adjacency entry p */
  int total = ip[nnode + 1] - 1;
  int *adj = (int *)malloc(((size_t)total + 1) * sizeof(int));
  if (!adj) { free(ip); free(ips); return ORC_ERR_OOM; }
  for (int p = 1; p <= total; p++) adj[p - 1] = ips[p];
  free(ips);
  *ip_out = ip;
  *ips_out = adj;
  return ORC_OK;
#undef IX
}

/* Exported for tests: node graph as (ip[nnode+1], adjacency[]) 1-based. */
int orc_graph(const int *ix, int nnode, int numel, int nen, int *ip_out,
              int *adj_out, int adj_cap) {
  int *ip, *adj;
  int st = graph(ix, nnode, numel, nen, &ip, &adj);
  if (st) return -st;
  int total = ip[nnode + 1] - 1;
  for (int i = 1; i <= nnode + 1; i++) ip_out[i - 1] = ip[i];
  if (total <= adj_cap) memcpy(adj_out, adj, (size_t)total * sizeof(int));
  free(ip);
  free(adj);
  return total;
}

/* ---------------------------------------------------------------------- */
/* Reord.f -- George-Liu reverse Cuthill-McKee (SPARSPAK)                  */
/* All arrays below are 1-based: xadj[1..n+1], adjncy[1..], mask[1..n].    */
/* ---------------------------------------------------------------------- */

/* Reord.f:355-435 degree (uses the sign of xadj as a visited marker). */
static void rcm_degree(int root, int *xadj, const int *adjncy, const int *mask,
                       int *deg, int *ccsize_out, int *ls) {
  ls[1] = root;
  xadj[root] = -xadj[root];
  int lvlend = 0, ccsize = 1;
  for (;;) {
    int lbegin = lvlend + 1;
    lvlend = ccsize;
    for (int i = lbegin; i <= lvlend; i++) {
      int node = ls[i];
      int jstrt = -xadj[node];
      int jstop = abs(xadj[node + 1]) - 1;
      int ideg = 0;
      for (int j = jstrt; j <= jstop; j++) {
        int nbr = adjncy[j];
        if (mask[nbr] == 0) continue;
        ideg++;
        if (xadj[nbr] < 0) continue;
        xadj[nbr] = -xadj[nbr];
        ccsize++;
        ls[ccsize] = nbr;
      }
      deg[node] = ideg;
    }
    if (ccsize - lvlend <= 0) break;
  }
  for (int i = 1; i <= ccsize; i++) {
    int node = ls[i];
    xadj[node] = -xadj[node];
  }
  *ccsize_out = ccsize;
}

/* Reord.f:278-354 rootls */
static void rcm_rootls(int root, const int *xadj, const int *adjncy, int *mask,
                       int *nlvl_out, int *xls, int *ls) {
  mask[root] = 0;
  ls[1] = root;
  int nlvl = 0, lvlend = 0, ccsize = 1;
  for (;;) {
    int lbegin = lvlend + 1;
    lvlend = ccsize;
    nlvl++;
    xls[nlvl] = lbegin;
    for (int i = lbegin; i <= lvlend; i++) {
      int node = ls[i];
      int jstrt = xadj[node], jstop = xadj[node + 1] - 1;
      for (int j = jstrt; j <= jstop; j++) {
        int nbr = adjncy[j];
        if (mask[nbr] == 0) continue;
        ccsize++;
        ls[ccsize] = nbr;
        mask[nbr] = 0;
      }
    }
    if (ccsize - lvlend <= 0) break;
  }
  xls[nlvl + 1] = lvlend + 1;
  for (int i = 1; i <= ccsize; i++) mask[ls[i]] = 1;
  *nlvl_out = nlvl;
}

/* Reord.f:101-169 fnroot (Gibbs-Poole-Stockmeyer pseudo-peripheral node). */
static void rcm_fnroot(int *root, const int *xadj, const int *adjncy, int *mask,
                       int *nlvl_out, int *xls, int *ls) {
  int nlvl, nunlvl;
  rcm_rootls(*root, xadj, adjncy, mask, &nlvl, xls, ls);
  int ccsize = xls[nlvl + 1] - 1;
  if (nlvl == 1 || nlvl == ccsize) { *nlvl_out = nlvl; return; }
  for (;;) {
    int jstrt = xls[nlvl];
    int mindeg = ccsize;
    *root = ls[jstrt];
    if (ccsize != jstrt) {
      for (int j = jstrt; j <= ccsize; j++) {
        int node = ls[j], ndeg = 0;
        for (int k = xadj[node]; k <= xadj[node + 1] - 1; k++)
          if (mask[adjncy[k]] > 0) ndeg++;
        if (ndeg < mindeg) { *root = node; mindeg = ndeg; }
      }
    }
    rcm_rootls(*root, xadj, adjncy, mask, &nunlvl, xls, ls);
    if (nunlvl <= nlvl) break;
    nlvl = nunlvl;
    if (nlvl >= ccsize) break;
  }
  *nlvl_out = nlvl;
}

/* Reord.f:170-277 rcm */
static void rcm_rcm(int root, int *xadj, const int *adjncy, int *mask,
                    int *perm, int *ccsize_out, int *deg) {
  int ccsize;
  rcm_degree(root, xadj, adjncy, mask, deg, &ccsize, perm);
  mask[root] = 0;
  *ccsize_out = ccsize;
  if (ccsize <= 1) return;
  int lvlend = 0, lnbr = 1;
  do {
    int lbegin = lvlend + 1;
    lvlend = lnbr;
    for (int i = lbegin; i <= lvlend; i++) {
      int node = perm[i];
      int jstrt = xadj[node], jstop = xadj[node + 1] - 1;
      int fnbr = lnbr + 1;
      for (int j = jstrt; j <= jstop; j++) {
        int nbr = adjncy[j];
        if (mask[nbr] == 0) continue;
        lnbr++;
        mask[nbr] = 0;
        perm[lnbr] = nbr;
      }
      if (fnbr >= lnbr) continue;
      /* linear insertion by increasing degree (Reord.f:253-261) */
      int k = fnbr;
      do {
        int l = k;
        k++;
        int nbr = perm[k];
        while (l >= fnbr) {
          int lperm = perm[l];
          if (deg[lperm] <= deg[nbr]) break;
          perm[l + 1] = lperm;
          l--;
        }
        perm[l + 1] = nbr;
      } while (k < lnbr);
    }
  } while (lnbr > lvlend);
  /* reverse (Reord.f:266-273) */
  int k = ccsize / 2, l = ccsize;
  for (int i = 1; i <= k; i++) {
    int t = perm[l];
    perm[l] = perm[i];
    perm[i] = t;
    l--;
  }
}

/* Reord.f:45-100 genrcm.  perm is 1-based of size neq+1. */
static void rcm_genrcm(int neq, int *xadj, const int *adjncy, int *perm,
                       int *mask, int *xls) {
  for (int i = 1; i <= neq; i++) mask[i] = 1;
  int num = 1;
  for (int i = 1; i <= neq; i++) {
    if (mask[i] == 0) continue;
    int root = i, nlvl, ccsize;
    rcm_fnroot(&root, xadj, adjncy, mask, &nlvl, xls, &perm[num - 1]);
    rcm_rcm(root, xadj, adjncy, mask, &perm[num - 1], &ccsize, xls);
    num += ccsize;
    if (num > neq) return;
  }
}

/* Reord.f:1-44 reord with afl = .true. and nnodei = nnode.
 * perm_out[k-1] = old node number (1-based) at new position k. */
int orc_reord(const int *ix, int nnode, int numel, int nen, int *perm_out) {
  int *ip, *adj;
  int st = graph(ix, nnode, numel, nen, &ip, &adj);
  if (st) return st;
  int total = ip[nnode + 1] - 1;
  int *adjncy = (int *)malloc(((size_t)total + 2) * sizeof(int));
  int *perm = (int *)calloc((size_t)nnode + 2, sizeof(int));
  int *mask = (int *)calloc((size_t)nnode + 2, sizeof(int));
  int *xls = (int *)calloc((size_t)nnode + 2, sizeof(int));
  if (!adjncy || !perm || !mask || !xls) {
    free(ip); free(adj); free(adjncy); free(perm); free(mask); free(xls);
    return ORC_ERR_OOM;
  }
  for (int p = 1; p <= total; p++) adjncy[p] = adj[p - 1];
  rcm_genrcm(nnode, ip, adjncy, perm, mask, xls);
  for (int k = 1; k <= nnode; k++) perm_out[k - 1] = perm[k];
  free(ip); free(adj); free(adjncy); free(perm); free(mask); free(xls);
  return ORC_OK;
}

/* ---------------------------------------------------------------------- */
/* Numeq.f:139-192 numeq (id used as both input and output, as Main.f:427) */
/* ---------------------------------------------------------------------- */
int orc_numeq(int *id, const int *num, int nnode, int ndf) {
  int neq = 0;
  for (int i = 1; i <= nnode; i++) {
    int n = num[i - 1];
    for (int j = 1; j <= ndf; j++) {
      int *p = &id[(size_t)(n - 1) * ndf + (j - 1)];
      if (*p == 0) { neq++; *p = neq; }
      else *p = 0;
    }
  }
  return neq;
}

/* ---------------------------------------------------------------------- */
/* Csr.f:13-305 csrstruct / csria / csrja, called lower-only               */
/* (Datastruct.f:80-83: lower=.true., diag=.false., upper=.false.)        */
/* ---------------------------------------------------------------------- */
#define ID(j, n) id[(size_t)((n) - 1) * ndf + ((j) - 1)]

/* Csr.f:87-191 csria with lower only.  ia is 1-based contents, size neq+1. */
static long long csria_lower(const int *id, const int *num, const int *ip,
                             const int *adj, int *ia, int nnode, int ndf,
                             int neq) {
  /* ia_[1..neq+1] */
  int *c = (int *)calloc((size_t)neq + 2, sizeof(int));
  if (!c) return -ORC_ERR_OOM;
  for (int no = 1; no <= nnode; no++) {
    int i = num[no - 1];
    for (int ii = 1; ii <= ndf; ii++) {
      int neqi = ID(ii, i);
      if (!(neqi > 0 && neqi <= neq)) continue;
      for (int kk = 1; kk <= ndf; kk++) {
        int neqj = ID(kk, i);
        if (neqj <= 0) continue;
        if (neqj < neqi) c[neqi]++;
      }
      for (int k = ip[i]; k <= ip[i + 1] - 1; k++) {
        int j = adj[k - 1];
        for (int jj = 1; jj <= ndf; jj++) {
          int neqj = ID(jj, j);
          if (neqj <= 0) continue;
          if (neqj < neqi) c[neqi]++;
        }
      }
    }
  }
  for (int i = neq; i >= 1; i--) c[i + 1] = c[i];
  c[1] = 1;
  for (int i = 1; i <= neq; i++) c[i + 1] += c[i];
  for (int i = 1; i <= neq + 1; i++) ia[i - 1] = c[i];
  long long nad = (long long)c[neq + 1] - 1;
  free(c);
  return nad;
}

/* Csr.f:192-305 csrja with lower only, then sortgraph (Csr.f:81). */
static void csrja_lower(const int *id, const int *num, const int *ip,
                        const int *adj, const int *ia, int *ja, int nnode,
                        int ndf, int neq) {
  long long n = 0;
  for (int no = 1; no <= nnode; no++) {
    int i = num[no - 1];
    for (int ii = 1; ii <= ndf; ii++) {
      int neqi = ID(ii, i);
      if (!(neqi > 0 && neqi <= neq)) continue;
      for (int kk = 1; kk <= ndf; kk++) {
        int neqj = ID(kk, i);
        if (neqj <= 0) continue;
        if (neqj < neqi) ja[n++] = neqj;
      }
      for (int k = ip[i]; k <= ip[i + 1] - 1; k++) {
        int j = adj[k - 1];
        for (int jj = 1; jj <= ndf; jj++) {
          int neqj = ID(jj, j);
          if (neqj <= 0) continue;
          if (neqj < neqi) ja[n++] = neqj;
        }
      }
    }
  }
  /* ia is 1-based contents in a 0-based array; sortgraph wants ia[1..] */
  for (int i = 0; i < neq; i++) sort_asc(&ja[ia[i] - 1], ia[i + 1] - ia[i]);
}

/* Csr.f:87-305 csria / csrja with lower = right = .true. (an overlapping
 * MPI partition: equations > neq are the halo).  ia gets 2 (neq + 1)
 * entries: ia(1..neq+1) for the lower part, ia(neq+2..2neq+2) for the
 * rectangular part (1-based positions from 1 into ja(nad+1..)); ja gets nad
 * + nad1 columns; both parts sorted per row (sortgraph, Csr.f:81-84).
 * With ja == NULL only the counts are returned. */
int orc_csr_right(const int *id, const int *num, const int *ix, int nnode, int numel,
                  int nen, int ndf, int neq, int *ia, int *ja, long long *nad_out,
                  long long *nad1_out) {
  int *ip, *adj;
  int st = graph(ix, nnode, numel, nen, &ip, &adj);
  if (st) return st;
  int *c = (int *)calloc((size_t)2 * neq + 4, sizeof(int)); /* c[1..2neq+2] */
  if (!c) return ORC_ERR_OOM;
  for (int no = 1; no <= nnode; no++) {
    int i = num[no - 1];
    for (int ii = 1; ii <= ndf; ii++) {
      int neqi = ID(ii, i);
      if (!(neqi > 0 && neqi <= neq)) continue;
      for (int kk = 1; kk <= ndf; kk++) {
        int neqj = ID(kk, i);
        if (neqj <= 0) continue;
        if (neqj < neqi) c[neqi]++;
      }
      for (int k = ip[i]; k <= ip[i + 1] - 1; k++) {
        int j = adj[k - 1];
        for (int jj = 1; jj <= ndf; jj++) {
          int neqj = ID(jj, j);
          if (neqj <= 0) continue;
          if (neqj < neqi) c[neqi]++;
          else if (neqj > neq) c[neq + 1 + neqi]++;
        }
      }
    }
  }
  for (int i = neq; i >= 1; i--) {
    c[i + 1] = c[i];
    c[i + neq + 2] = c[i + neq + 1];
  }
  c[1] = 1;
  c[neq + 2] = 1;
  for (int i = 1; i <= neq; i++) {
    c[i + 1] += c[i];
    c[i + neq + 2] += c[i + neq + 1];
  }
  const long long nad = (long long)c[neq + 1] - 1, nad1 = (long long)c[2 * neq + 2] - 1;
  if (nad_out) *nad_out = nad;
  if (nad1_out) *nad1_out = nad1;
  if (ia)
    for (int i = 1; i <= 2 * neq + 2; i++) ia[i - 1] = c[i];
  if (ja) {
    long long n = 0, m = 0;
    for (int no = 1; no <= nnode; no++) {
      int i = num[no - 1];
      for (int ii = 1; ii <= ndf; ii++) {
        int neqi = ID(ii, i);
        if (!(neqi > 0 && neqi <= neq)) continue;
        for (int kk = 1; kk <= ndf; kk++) {
          int neqj = ID(kk, i);
          if (neqj <= 0) continue;
          if (neqj < neqi) ja[n++] = neqj;
        }
        for (int k = ip[i]; k <= ip[i + 1] - 1; k++) {
          int j = adj[k - 1];
          for (int jj = 1; jj <= ndf; jj++) {
            int neqj = ID(jj, j);
            if (neqj <= 0) continue;
            if (neqj < neqi) ja[n++] = neqj;
            else if (neqj > neq) ja[nad + m++] = neqj;
          }
        }
      }
    }
    for (int i = 1; i <= neq; i++) {
      sort_asc(&ja[c[i] - 1], c[i + 1] - c[i]);
      sort_asc(&ja[nad + c[neq + 1 + i] - 1], c[neq + 2 + i] - c[neq + 1 + i]);
    }
  }
  free(c);
  free(ip);
  free(adj);
  return ORC_OK;
}

/* csrstruct phase 1: ia (neq+1 ints).  Returns nad (>= 0) or -status. */
long long orc_csr_ia(const int *id, const int *num, const int *ix, int nnode,
                     int numel, int nen, int ndf, int neq, int *ia) {
  int *ip, *adj;
  int st = graph(ix, nnode, numel, nen, &ip, &adj);
  if (st) return -st;
  long long nad = csria_lower(id, num, ip, adj, ia, nnode, ndf, neq);
  free(ip);
  free(adj);
  return nad;
}

/* csrstruct phase 2: ja (nad ints), given ia from phase 1. */
int orc_csr_ja(const int *id, const int *num, const int *ix, int nnode,
               int numel, int nen, int ndf, int neq, const int *ia, int *ja) {
  int *ip, *adj;
  int st = graph(ix, nnode, numel, nen, &ip, &adj);
  if (st) return st;
  csrja_lower(id, num, ip, adj, ia, ja, nnode, ndf, neq);
  free(ip);
  free(adj);
  return ORC_OK;
}
#undef ID

/* ---------------------------------------------------------------------- */
/* Element library (Elmlib.f, Elmlib02.f), isw = 2 and 2-D isw = 4          */
/* ---------------------------------------------------------------------- */

/* Elmlib.f:2985-2988, 3016-3018: 2-point Gauss-Legendre row of pg/wg. */
static const double PG2[2] = {-.577350269189626e0, .577350269189626e0};
static const double WG2[2] = {1.e0, 1.e0};

/* Elmlib.f:336-368 lku_m: p = s.u sweeping columns.  s is (nst,nst) col-major */
static void lku_m(const double *s, const double *u, double *p, int nst) {
  for (int i = 0; i < nst; i++) p[i] = 0.0;
  for (int j = 0; j < nst; j++)
    for (int i = 0; i < nst; i++) p[i] = p[i] + s[(size_t)j * nst + i] * u[j];
}

/* Elmlib.f:815-886 sfquad4_m (derivatives only: afl=.false., bfl=.true.) */
static void sfquad4_m(double *hx, double *hy, double r, double s) {
  double opr = 1.0 + r, ops = 1.0 + s, omr = 1.0 - r, oms = 1.0 - s;
  hx[0] = ops * 0.25;
  hx[1] = -(ops * 0.25);
  hx[2] = -(oms * 0.25);
  hx[3] = oms * 0.25;
  hy[0] = opr * 0.25;
  hy[1] = omr * 0.25;
  hy[2] = -(omr * 0.25);
  hy[3] = -(opr * 0.25);
}

/* Elmlib.f:1151-1258 sfhexa8_m (derivatives only) */
static void sfhexa8_m(double *hx, double *hy, double *hz, double r, double s,
                      double t) {
  double pR = 1.0 + r, pS = 1.0 + s, pT = 1.0 + t;
  double mR = 1.0 - r, mS = 1.0 - s, mT = 1.0 - t;
  hx[0] = pS * pT * 0.125;  hx[1] = -(pS * pT * 0.125);
  hx[2] = -(mS * pT * 0.125); hx[3] = mS * pT * 0.125;
  hx[4] = pS * mT * 0.125;  hx[5] = -(pS * mT * 0.125);
  hx[6] = -(mS * mT * 0.125); hx[7] = mS * mT * 0.125;
  hy[0] = pR * pT * 0.125;  hy[1] = mR * pT * 0.125;
  hy[2] = -(mR * pT * 0.125); hy[3] = -(pR * pT * 0.125);
  hy[4] = pR * mT * 0.125;  hy[5] = mR * mT * 0.125;
  hy[6] = -(mR * mT * 0.125); hy[7] = -(pR * mT * 0.125);
  hz[0] = pR * pS * 0.125;  hz[1] = mR * pS * 0.125;
  hz[2] = mR * mS * 0.125;  hz[3] = pR * mS * 0.125;
  hz[4] = -(pR * pS * 0.125); hz[5] = -(mR * pS * 0.125);
  hz[6] = -(mR * mS * 0.125); hz[7] = -(pR * mS * 0.125);
}

/* Elmlib.f:1769-1852 jacob2d_m (afl=.true.).  x is (ndm,nen) col-major.
 * Returns nonzero when det <= 1e-14 (the reference stops there). */
static int jacob2d_m(double *hx, double *hy, const double *x, int nen, int ndm,
                     double *det_out) {
  double xj[2][2];
  for (int j = 0; j < 2; j++) {
    xj[0][j] = 0.0;
    xj[1][j] = 0.0;
    for (int k = 0; k < nen; k++) {
      xj[0][j] = xj[0][j] + hx[k] * x[(size_t)k * ndm + j];
      xj[1][j] = xj[1][j] + hy[k] * x[(size_t)k * ndm + j];
    }
  }
  double det = xj[0][0] * xj[1][1] - xj[1][0] * xj[0][1];
  if (det <= 1.e-14) return 1;
  double xji11 = xj[1][1] / det, xji12 = -xj[0][1] / det;
  double xji21 = -xj[1][0] / det, xji22 = xj[0][0] / det;
  for (int k = 0; k < nen; k++) {
    double hxk = hx[k], hyk = hy[k];
    hx[k] = xji11 * hxk + xji12 * hyk;
    hy[k] = xji21 * hxk + xji22 * hyk;
  }
  *det_out = det;
  return 0;
}

/* Elmlib.f:1942-2036 jacob3d_m (afl=.true.).  x is (3,nen) col-major. */
static int jacob3d_m(double *hx, double *hy, double *hz, const double *x,
                     int nen, double *det_out) {
  double xj[3][3]; /* xj[a][b] = xj(a+1,b+1) */
  for (int j = 0; j < 3; j++) {
    xj[0][j] = 0.0; xj[1][j] = 0.0; xj[2][j] = 0.0;
    for (int k = 0; k < nen; k++) {
      xj[0][j] = xj[0][j] + hx[k] * x[(size_t)k * 3 + j];
      xj[1][j] = xj[1][j] + hy[k] * x[(size_t)k * 3 + j];
      xj[2][j] = xj[2][j] + hz[k] * x[(size_t)k * 3 + j];
    }
  }
  double det = xj[0][0] * xj[1][1] * xj[2][2] + xj[0][1] * xj[1][2] * xj[2][0] +
               xj[0][2] * xj[1][0] * xj[2][1] - xj[2][0] * xj[1][1] * xj[0][2] -
               xj[1][0] * xj[0][1] * xj[2][2] - xj[0][0] * xj[2][1] * xj[1][2];
  if (det <= 1.e-14) return 1;
  double xji[3][3];
  xji[0][0] = (xj[1][1] * xj[2][2] - xj[1][2] * xj[2][1]) / det;
  xji[1][0] = -(xj[1][0] * xj[2][2] - xj[1][2] * xj[2][0]) / det;
  xji[2][0] = (xj[1][0] * xj[2][1] - xj[1][1] * xj[2][0]) / det;
  xji[0][1] = -(xj[0][1] * xj[2][2] - xj[0][2] * xj[2][1]) / det;
  xji[1][1] = (xj[0][0] * xj[2][2] - xj[0][2] * xj[2][0]) / det;
  xji[2][1] = -(xj[0][0] * xj[2][1] - xj[0][1] * xj[2][0]) / det;
  xji[0][2] = (xj[0][1] * xj[1][2] - xj[0][2] * xj[1][1]) / det;
  xji[1][2] = -(xj[0][0] * xj[1][2] - xj[0][2] * xj[1][0]) / det;
  xji[2][2] = (xj[0][0] * xj[1][1] - xj[0][1] * xj[1][0]) / det;
  for (int k = 0; k < nen; k++) {
    double hxk = hx[k], hyk = hy[k], hzk = hz[k];
    hx[k] = xji[0][0] * hxk + xji[0][1] * hyk + xji[0][2] * hzk;
    hy[k] = xji[1][0] * hxk + xji[1][1] * hyk + xji[1][2] * hzk;
    hz[k] = xji[2][0] * hxk + xji[2][1] * hyk + xji[2][2] * hzk;
  }
  *det_out = det;
  return 0;
}

/* Elmlib.f:2636-2713 jtetra4 (afl=.true.) */
static int jtetra4(const double *x, double *hx, double *hy, double *hz,
                   double *det_out) {
#define X3(a, n) x[(size_t)((n) - 1) * 3 + ((a) - 1)]
  double xj11 = X3(1, 1) - X3(1, 4), xj12 = X3(2, 1) - X3(2, 4),
         xj13 = X3(3, 1) - X3(3, 4);
  double xj21 = X3(1, 2) - X3(1, 4), xj22 = X3(2, 2) - X3(2, 4),
         xj23 = X3(3, 2) - X3(3, 4);
  double xj31 = X3(1, 3) - X3(1, 4), xj32 = X3(2, 3) - X3(2, 4),
         xj33 = X3(3, 3) - X3(3, 4);
#undef X3
  double det = xj11 * xj22 * xj33 + xj12 * xj23 * xj31 + xj13 * xj21 * xj32 -
               xj31 * xj22 * xj13 - xj12 * xj21 * xj33 - xj11 * xj32 * xj23;
  if (det <= 1.e-14) return 1;
  double deti = 1.0 / det;
  hx[0] = (xj22 * xj33 - xj23 * xj32) * deti;
  hx[1] = (xj13 * xj32 - xj12 * xj33) * deti;
  hx[2] = (xj12 * xj23 - xj13 * xj22) * deti;
  hy[0] = (xj23 * xj31 - xj21 * xj33) * deti;
  hy[1] = (xj11 * xj33 - xj13 * xj31) * deti;
  hy[2] = (xj13 * xj21 - xj11 * xj23) * deti;
  hz[0] = (xj21 * xj32 - xj22 * xj31) * deti;
  hz[1] = (xj12 * xj31 - xj11 * xj32) * deti;
  hz[2] = (xj11 * xj22 - xj12 * xj21) * deti;
  hx[3] = -hx[0] - hx[1] - hx[2];
  hy[3] = -hy[0] - hy[1] - hy[2];
  hz[3] = -hz[0] - hz[1] - hz[2];
  *det_out = det;
  return 0;
}

/* 2-D stiffness block shared by TRIA3/QUAD4 (Elmlib02.f:211-225, 773-795). */
static void k2d_add(double *s, int nst, int nn, const double *hx,
                    const double *hy, double d11, double d12, double d22,
                    double d33, double wt1, int accumulate) {
#define S(r, c) s[(size_t)((c) - 1) * nst + ((r) - 1)]
  for (int jj = 1; jj <= nn; jj++) {
    int k1 = 2 * jj - 1, k2 = k1 + 1;
    for (int ii = 1; ii <= nn; ii++) {
      int l1 = 2 * ii - 1, l2 = l1 + 1;
      const int i = ii - 1, j = jj - 1;
      double v11 = (hx[i] * d11 * hx[j] + hy[i] * d33 * hy[j]) * wt1;
      double v12 = (hx[i] * d12 * hy[j] + hy[i] * d33 * hx[j]) * wt1;
      double v21 = (hy[i] * d12 * hx[j] + hx[i] * d33 * hy[j]) * wt1;
      double v22 = (hy[i] * d22 * hy[j] + hx[i] * d33 * hx[j]) * wt1;
      if (accumulate) {
        S(l1, k1) = S(l1, k1) + v11;
        S(l1, k2) = S(l1, k2) + v12;
        S(l2, k1) = S(l2, k1) + v21;
        S(l2, k2) = S(l2, k2) + v22;
      } else {
        S(l1, k1) = v11;
        S(l1, k2) = v12;
        S(l2, k1) = v21;
        S(l2, k2) = v22;
      }
    }
  }
#undef S
}

/* Elmlib02.f:50-337 elmt02_mec (plane strain) and 339-627 elmt03_mec
 * (plane stress), isw = 2.  TRIA3: thickness is read but not used in K
 * (Elmlib02.f:463-464 vs 492). */
static int elmt_tria3(const double *e, const double *x, int ndm,
                      double *s, int plane_stress) {
  const int nst = 6;
#define XX(a, n) x[(size_t)((n) - 1) * ndm + ((a) - 1)]
  double xj11 = XX(1, 1) - XX(1, 3), xj12 = XX(2, 1) - XX(2, 3);
  double xj21 = XX(1, 2) - XX(1, 3), xj22 = XX(2, 2) - XX(2, 3);
#undef XX
  double det = xj11 * xj22 - xj12 * xj21;
  if (det <= 0.0) return ORC_ERR_BAD_DET;
  double xji11 = xj22 / det, xji12 = -xj12 / det;
  double xji21 = -xj21 / det, xji22 = xj11 / det;
  double hx[3], hy[3];
  hx[0] = xji11; hx[1] = xji12; hx[2] = -xji11 - xji12;
  hy[0] = xji21; hy[1] = xji22; hy[2] = -xji21 - xji22;
  double ym = e[0], ps = e[1], a, b, c;
  if (!plane_stress) {
    double a1 = 1.0 - ps, a2 = 1.0 - 2.0 * ps, a3 = 1.0 + ps;
    a = (ym * a1) / (a3 * a2);
    b = ps / a1;
    c = 0.5 * (a2 / a1);
  } else {
    double a1 = 1.0 - ps, a2 = 1.0 - ps * ps;
    a = ym / a2;
    b = ps;
    c = 0.5 * a1;
  }
  double d11 = a, d12 = a * b, d22 = a, d33 = a * c;
  for (int i = 0; i < nst * nst; i++) s[i] = 0.0;
  double wt1 = 0.5 * det;
  k2d_add(s, nst, 3, hx, hy, d11, d12, d22, d33, wt1, 0);
  return ORC_OK;
}

/* Elmlib02.f:629-929 elmt04_mec (plane strain) and 931-1230 elmt05_mec
 * (plane stress, weight times thickness at 1071), isw = 2. */
static int elmt_quad4(const double *e, const double *x, int ndm, double *s,
                      int plane_stress) {
  const int nst = 8;
  double ym = e[0], ps = e[1], thic = 1.0, a, b, c;
  if (!plane_stress) {
    double a1 = 1.0 - ps, a2 = 1.0 - 2.0 * ps, a3 = 1.0 + ps;
    a = (ym * a1) / (a3 * a2);
    b = ps / a1;
    c = 0.5 * (a2 / a1);
  } else {
    thic = e[2];
    if (thic == 0.0) thic = 1.0;
    double a1 = 1.0 - ps, a2 = 1.0 - ps * ps;
    a = ym / a2;
    b = ps;
    c = 0.5 * a1;
  }
  double d11 = a, d12 = a * b, d22 = a, d33 = a * c;
  for (int i = 0; i < nst * nst; i++) s[i] = 0.0;
  for (int ly = 0; ly < 2; ly++) {
    double si = PG2[ly];
    for (int lx = 0; lx < 2; lx++) {
      double ri = PG2[lx], hx[4], hy[4], det;
      sfquad4_m(hx, hy, ri, si);
      if (jacob2d_m(hx, hy, x, 4, ndm, &det)) return ORC_ERR_BAD_DET;
      double w = plane_stress ? WG2[lx] * WG2[ly] * det * thic
                              : WG2[lx] * WG2[ly] * det;
      k2d_add(s, nst, 4, hx, hy, d11, d12, d22, d33, w, 1);
    }
  }
  return ORC_OK;
}

/* Elmlib02.f:1232-1573 elmt06_mec TETRA4, isw = 2 (div6 literal at 1278). */
static int elmt_tetra4(const double *e, const double *x, double *s) {
  const int nst = 12;
  const double div6 = 0.166666666666667e+00;
  double ym = e[0], ps = e[1];
  double a1 = 1.0 - ps, a2 = 1.0 - 2.0 * ps, a3 = 1.0 + ps;
  double a = (ym * a1) / (a3 * a2), b = ps / a1, c = 0.5 * (a2 / a1);
  for (int i = 0; i < nst * nst; i++) s[i] = 0.0;
  double hx[4], hy[4], hz[4], det;
  if (jtetra4(x, hx, hy, hz, &det)) return ORC_ERR_BAD_DET;
  double wt1 = a * det * div6;
#define S(r, cc) s[(size_t)((cc) - 1) * nst + ((r) - 1)]
  for (int ii = 1; ii <= 4; ii++) {
    int l1 = 3 * ii - 2, l2 = l1 + 1, l3 = l2 + 1, i = ii - 1;
    for (int jj = 1; jj <= 4; jj++) {
      int k1 = 3 * jj - 2, k2 = k1 + 1, k3 = k2 + 1, j = jj - 1;
      S(l1, k1) = (hx[i] * hx[j] + c * hy[i] * hy[j] + c * hz[i] * hz[j]) * wt1;
      S(l1, k2) = (b * hx[i] * hy[j] + c * hy[i] * hx[j]) * wt1;
      S(l1, k3) = (b * hx[i] * hz[j] + c * hz[i] * hx[j]) * wt1;
      S(l2, k1) = (b * hy[i] * hx[j] + c * hx[i] * hy[j]) * wt1;
      S(l2, k2) = (hy[i] * hy[j] + c * hx[i] * hx[j] + c * hz[i] * hz[j]) * wt1;
      S(l2, k3) = (b * hy[i] * hz[j] + c * hz[i] * hy[j]) * wt1;
      S(l3, k1) = (b * hz[i] * hx[j] + c * hx[i] * hz[j]) * wt1;
      S(l3, k2) = (b * hz[i] * hy[j] + c * hy[i] * hz[j]) * wt1;
      S(l3, k3) = (hz[i] * hz[j] + c * hy[i] * hy[j] + c * hx[i] * hx[j]) * wt1;
    }
  }
#undef S
  return ORC_OK;
}

/* Elmlib02.f:1577-2023 elmt07_mec HEXA8, isw = 2 (2x2x2 Gauss, 1714-1777). */
static int elmt_hexa8(const double *e, const double *x, double *s) {
  const int nst = 24;
  double ym = e[0], ps = e[1];
  double a1 = 1.0 - ps, a2 = 1.0 - 2.0 * ps, a3 = 1.0 + ps;
  double a = (ym * a1) / (a3 * a2), b = ps / a1, c = 0.5 * (a2 / a1);
  for (int i = 0; i < nst * nst; i++) s[i] = 0.0;
#define S(r, cc) s[(size_t)((cc) - 1) * nst + ((r) - 1)]
  for (int lz = 0; lz < 2; lz++) {
    double ti = PG2[lz];
    for (int ly = 0; ly < 2; ly++) {
      double si = PG2[ly];
      for (int lx = 0; lx < 2; lx++) {
        double ri = PG2[lx], hx[8], hy[8], hz[8], det;
        sfhexa8_m(hx, hy, hz, ri, si, ti);
        if (jacob3d_m(hx, hy, hz, x, 8, &det)) return ORC_ERR_BAD_DET;
        double w = WG2[lx] * WG2[ly] * WG2[lz] * det;
        double wt1 = w * a;
        for (int ii = 1; ii <= 8; ii++) {
          int l1 = 3 * ii - 2, l2 = l1 + 1, l3 = l2 + 1, i = ii - 1;
          for (int jj = 1; jj <= 8; jj++) {
            int k1 = 3 * jj - 2, k2 = k1 + 1, k3 = k2 + 1, j = jj - 1;
            S(l1, k1) = S(l1, k1) + (hx[i] * hx[j] + c * (hy[i] * hy[j] + hz[i] * hz[j])) * wt1;
            S(l1, k2) = S(l1, k2) + (b * hx[i] * hy[j] + c * hy[i] * hx[j]) * wt1;
            S(l1, k3) = S(l1, k3) + (b * hx[i] * hz[j] + c * hz[i] * hx[j]) * wt1;
            S(l2, k1) = S(l2, k1) + (b * hy[i] * hx[j] + c * hx[i] * hy[j]) * wt1;
            S(l2, k2) = S(l2, k2) + (hy[i] * hy[j] + c * (hx[i] * hx[j] + hz[i] * hz[j])) * wt1;
            S(l2, k3) = S(l2, k3) + (b * hy[i] * hz[j] + c * hz[i] * hy[j]) * wt1;
            S(l3, k1) = S(l3, k1) + (b * hz[i] * hx[j] + c * hx[i] * hz[j]) * wt1;
            S(l3, k2) = S(l3, k2) + (b * hz[i] * hy[j] + c * hy[i] * hz[j]) * wt1;
            S(l3, k3) = S(l3, k3) + (hz[i] * hz[j] + c * (hy[i] * hy[j] + hx[i] * hx[j])) * wt1;
          }
        }
      }
    }
  }
#undef S
  return ORC_OK;
}

/* Element matrix for reference element type iel (Elmlib.f:43-144). */
static int elmlib_k(int iel, const double *e, const double *xl, int ndm,
                    double *s, int *nst_out) {
  switch (iel) {
    case 2: *nst_out = 6; return elmt_tria3(e, xl, ndm, s, 0);
    case 3: *nst_out = 6; return elmt_tria3(e, xl, ndm, s, 1);
    case 4: *nst_out = 8; return elmt_quad4(e, xl, ndm, s, 0);
    case 5: *nst_out = 8; return elmt_quad4(e, xl, ndm, s, 1);
    case 6: *nst_out = 12; return elmt_tetra4(e, xl, s);
    case 7: *nst_out = 24; return elmt_hexa8(e, xl, s);
    default: return ORC_ERR_BAD_ELEMENT;
  }
}

/* Exported for tests: one element stiffness matrix, s (nst,nst) col-major. */
int orc_element_stiffness(int iel, const double *e, const double *xl, int ndm,
                          double *s) {
  int nst;
  return elmlib_k(iel, e, xl, ndm, s, &nst);
}

/* Assbly.f:66-146 csr (lower storage, symmetric: unsym = .false.). */
static void assbly_csr(const double *s, const double *p, const int *ld,
                       const int *ia, const int *ja, double *al, double *ad,
                       double *b, int nst, int neq, int lhs, int rhs) {
  for (int i = 1; i <= nst; i++) {
    int k = ld[i - 1];
    if (k <= 0 || k > neq) continue;
    if (rhs) b[k - 1] = b[k - 1] - p[i - 1];
    if (lhs) {
      ad[k - 1] = ad[k - 1] + s[(size_t)(i - 1) * nst + (i - 1)];
      for (int j = 1; j <= nst; j++) {
        int l = ld[j - 1];
        if (l <= 0) continue;
        for (int kk = ia[k - 1]; kk <= ia[k] - 1; kk++)
          if (l == ja[kk - 1])
            al[kk - 1] = al[kk - 1] + s[(size_t)(j - 1) * nst + (i - 1)];
      }
    }
  }
}

/* Pform.f:1-254 pform_mec, sequential element loop (Pform.f:190-247), with
 * isw = 2 (K and p = K u).  ix (nen+1,numel); ie(numat) element type per
 * material; e(prop,numat); x(ndm,nnode); id(ndf,nnode); u(ndf,nnode).
 * Returns 0, or ORC_ERR_BAD_DET with *bad_el = element number. */
int orc_pform_k(const int *ix, const int *ie, const double *e, int prop,
                const double *x, const int *id, const int *ia, const int *ja,
                double *al, double *ad, double *b, const double *u, int numel,
                int nen, int nenv, int ndf, int ndm, int neq, long long nad,
                int lhs, int rhs, int *bad_el) {
  const int nen1 = nen + 1;
  double xl[3 * 8], ul[24], pl[24], sl[24 * 24];
  int ld[24];
  if (nen > 8 || ndf > 3 || ndm > 3) return ORC_ERR_ARG;
  if (lhs) {
    memset(al, 0, (size_t)nad * sizeof(double));
    memset(ad, 0, (size_t)neq * sizeof(double));
  }
  for (int nel = 1; nel <= numel; nel++) {
    const int *ixe = &ix[(size_t)(nel - 1) * nen1];
    int kk = 0;
    for (int i = 1; i <= nen; i++) {
      int no = ixe[i - 1];
      for (int j = 1; j <= ndf; j++) {
        ld[kk] = id[(size_t)(no - 1) * ndf + (j - 1)];
        pl[kk] = 0.0;
        ul[kk] = u[(size_t)(no - 1) * ndf + (j - 1)];
        kk++;
      }
    }
    for (int i = 1; i <= nenv; i++) {
      int no = ixe[i - 1];
      for (int j = 1; j <= ndm; j++)
        xl[(size_t)(i - 1) * ndm + (j - 1)] = x[(size_t)(no - 1) * ndm + (j - 1)];
    }
    int ma = ixe[nen];
    int iel = ie[ma - 1];
    const double *el = &e[(size_t)(ma - 1) * prop];
    int nst;
    int st = elmlib_k(iel, el, xl, ndm, sl, &nst);
    if (st) { if (bad_el) *bad_el = nel; return st; }
    lku_m(sl, ul, pl, nst);
    assbly_csr(sl, pl, ld, ia, ja, al, ad, b, nst, neq, lhs, rhs);
  }
  return ORC_OK;
}

/* ---------------------------------------------------------------------- */
/* Stress recovery: elmt02-07_mec isw = 3 and tform_mec (Pform.f:258-421)  */
/* ---------------------------------------------------------------------- */

/* Elmlib.f:2368-2411 deform2d */
static void deform2d(const double *hx, const double *hy, const double *u, double *eps,
                     int nen) {
  double ux = 0.0, uy = 0.0, vx = 0.0, vy = 0.0;
  for (int i = 0; i < nen; i++) {
    ux = ux + hx[i] * u[2 * i];
    uy = uy + hy[i] * u[2 * i];
    vx = vx + hx[i] * u[2 * i + 1];
    vy = vy + hy[i] * u[2 * i + 1];
  }
  eps[0] = ux;
  eps[1] = vy;
  eps[2] = uy + vx;
}

/* Elmlib.f:2413-2471 deform3d */
static void deform3d(const double *hx, const double *hy, const double *hz, const double *u,
                     double *eps, int nen) {
  double ux = 0, uy = 0, uz = 0, vx = 0, vy = 0, vz = 0, wx = 0, wy = 0, wz = 0;
  for (int i = 0; i < nen; i++) {
    ux = ux + hx[i] * u[3 * i];
    uy = uy + hy[i] * u[3 * i];
    uz = uz + hz[i] * u[3 * i];
    vx = vx + hx[i] * u[3 * i + 1];
    vy = vy + hy[i] * u[3 * i + 1];
    vz = vz + hz[i] * u[3 * i + 1];
    wx = wx + hx[i] * u[3 * i + 2];
    wy = wy + hy[i] * u[3 * i + 2];
    wz = wz + hz[i] * u[3 * i + 2];
  }
  eps[0] = ux;
  eps[1] = vy;
  eps[2] = wz;
  eps[3] = uy + vx;
  eps[4] = vz + wy;
  eps[5] = uz + wx;
}

/* Elmlib.f:2502-2538 stress2d_m: sxx, syy, szz (ps (sxx + syy) in plane
 * strain, 0 in plane stress), sxy */
static void stress2d_m(double d11, double d12, double d22, double d33, double ps, int ept,
                       const double *eps, double *t) {
  t[0] = d11 * eps[0] + d12 * eps[1];
  t[1] = d12 * eps[0] + d22 * eps[1];
  t[2] = ept ? ps * (t[0] + t[1]) : 0.0;
  t[3] = d33 * eps[2];
}

/* Elmlib.f:2540-2571 stress3d */
static void stress3d(double a, double b, double c, const double *eps, double *t) {
  t[0] = (eps[0] + b * eps[1] + b * eps[2]) * a;
  t[1] = (b * eps[0] + eps[1] + b * eps[2]) * a;
  t[2] = (b * eps[0] + b * eps[1] + eps[2]) * a;
  t[3] = eps[3] * c * a;
  t[4] = eps[4] * c * a;
  t[5] = eps[5] * c * a;
}

/* Constitutive constants of elmt02-07 (plane strain / 3-D: a, b, c of
 * Elmlib02.f:179-186, 819-832, 1402-1408, 1697-1705; plane stress:
 * Elmlib02.f:469-476, 1124-1134). */
static void law(int plane_stress, double ym, double ps, double *a, double *b, double *c) {
  if (!plane_stress) {
    double a1 = 1.0 - ps, a2 = 1.0 - 2.0 * ps, a3 = 1.0 + ps;
    *a = (ym * a1) / (a3 * a2);
    *b = ps / a1;
    *c = 0.5 * (a2 / a1);
  } else {
    double a1 = 1.0 - ps, a2 = 1.0 - ps * ps;
    *a = ym / a2;
    *b = ps;
    *c = 0.5 * a1;
  }
}

/* isw = 3 of elmt02-07_mec: stresses at the element's nodes, p(ntn, nen)
 * col-major (ntn = 4 in 2-D, 6 in 3-D).  TRIA3 Elmlib02.f:235-250 (plane
 * strain) / 525-540 (plane stress): constant, copied to the 3 nodes; QUAD4
 * 836-846 / 1138-1148: at each node (rn, sn); TETRA4 1412-1437: constant;
 * HEXA8 1798-1812: at each node (rn, sn, tn). */
static int elmt_stress(int iel, const double *e, const double *x, int ndm, const double *u,
                       double *p) {
  static const double rn[8] = {1, -1, -1, 1, 1, -1, -1, 1};
  static const double sn[8] = {1, 1, -1, -1, 1, 1, -1, -1};
  static const double tn[8] = {1, 1, 1, 1, -1, -1, -1, -1};
  const double ym = e[0], ps = e[1];
  double a, b, c, eps[6];
  switch (iel) {
    case 2:
    case 3: {
      const int pstress = iel == 3;
      law(pstress, ym, ps, &a, &b, &c);
#define XX(q, n) x[(size_t)((n) - 1) * ndm + ((q) - 1)]
      double xj11 = XX(1, 1) - XX(1, 3), xj12 = XX(2, 1) - XX(2, 3);
      double xj21 = XX(1, 2) - XX(1, 3), xj22 = XX(2, 2) - XX(2, 3);
#undef XX
      double det = xj11 * xj22 - xj12 * xj21;
      if (det <= 0.0) return ORC_ERR_BAD_DET;
      double xji11 = xj22 / det, xji12 = -xj12 / det;
      double xji21 = -xj21 / det, xji22 = xj11 / det;
      double hx[3] = {xji11, xji12, -xji11 - xji12};
      double hy[3] = {xji21, xji22, -xji21 - xji22};
      deform2d(hx, hy, u, eps, 3);
      stress2d_m(a, a * b, a, a * c, ps, !pstress, eps, p);
      for (int n = 1; n < 3; n++)
        for (int j = 0; j < 4; j++) p[4 * n + j] = p[j];
      return ORC_OK;
    }
    case 4:
    case 5: {
      const int pstress = iel == 5;
      law(pstress, ym, ps, &a, &b, &c);
      for (int n = 0; n < 4; n++) {
        double hx[4], hy[4], det;
        sfquad4_m(hx, hy, rn[n], sn[n]);
        if (jacob2d_m(hx, hy, x, 4, ndm, &det)) return ORC_ERR_BAD_DET;
        deform2d(hx, hy, u, eps, 4);
        stress2d_m(a, a * b, a, a * c, ps, !pstress, eps, p + 4 * n);
      }
      return ORC_OK;
    }
    case 6: {
      law(0, ym, ps, &a, &b, &c);
      double hx[4], hy[4], hz[4], det;
      if (jtetra4(x, hx, hy, hz, &det)) return ORC_ERR_BAD_DET;
      deform3d(hx, hy, hz, u, eps, 4);
      stress3d(a, b, c, eps, p);
      for (int n = 1; n < 4; n++)
        for (int j = 0; j < 6; j++) p[6 * n + j] = p[j];
      return ORC_OK;
    }
    case 7: {
      law(0, ym, ps, &a, &b, &c);
      for (int n = 0; n < 8; n++) {
        double hx[8], hy[8], hz[8], det;
        sfhexa8_m(hx, hy, hz, rn[n], sn[n], tn[n]);
        if (jacob3d_m(hx, hy, hz, x, 8, &det)) return ORC_ERR_BAD_DET;
        deform3d(hx, hy, hz, u, eps, 8);
        stress3d(a, b, c, eps, p + 6 * n);
      }
      return ORC_OK;
    }
    default:
      return ORC_ERR_BAD_ELEMENT;
  }
}

/* Pform.f:258-421 tform_mec (isw = 3, every element node counted):
 * t(ntn, nnode) = average over the elements of a node of their nodal
 * stresses, + tx0 (may be NULL: zero).  ic(nnode) work array.  On a bad
 * element returns its status and the element number in *bad_el. */
int orc_tform(const int *ix, const int *ie, const double *e, int prop, const double *x,
              const double *u, const double *tx0, int nnode, int numel, int nen, int ndm,
              int ndf, double *t, int *ic, int *bad_el) {
  const int nen1 = nen + 1, ntn = ndm == 2 ? 4 : 6;
  double xl[3 * 8], ul[24], pl[6 * 8];
  if (nen > 8 || ndf > 3 || ndm > 3) return ORC_ERR_ARG;
  for (int i = 0; i < nnode; i++) {
    ic[i] = 0;
    for (int j = 0; j < ntn; j++) t[(size_t)i * ntn + j] = 0.0;
  }
  for (int nel = 1; nel <= numel; nel++) {
    const int *ixe = &ix[(size_t)(nel - 1) * nen1];
    int kk = 0;
    for (int i = 0; i < nen; i++) {
      const int no = ixe[i];
      for (int j = 0; j < ndf; j++) ul[kk++] = u[(size_t)(no - 1) * ndf + j];
    }
    for (int i = 0; i < nen; i++)
      for (int j = 0; j < ndm; j++) xl[i * ndm + j] = x[(size_t)(ixe[i] - 1) * ndm + j];
    const int ma = ixe[nen];
    int st = elmt_stress(ie[ma - 1], &e[(size_t)(ma - 1) * prop], xl, ndm, ul, pl);
    if (st) {
      if (bad_el) *bad_el = nel;
      return st;
    }
    for (int i = 0; i < nen; i++) {
      const int no = ixe[i];
      if (no <= 0) continue;
      ic[no - 1] += 1;
      for (int j = 0; j < ntn; j++) t[(size_t)(no - 1) * ntn + j] += pl[i * ntn + j];
    }
  }
  for (int i = 0; i < nnode; i++)
    for (int j = 0; j < ntn; j++)
      t[(size_t)i * ntn + j] = t[(size_t)i * ntn + j] / ic[i] + (tx0 ? tx0[(size_t)i * ntn + j] : 0.0);
  return ORC_OK;
}

/* Colormsh.f:9-308 coloredmesh with omp_elmt = .true.: nodegrade +
 * elmincid + colormsh (greedy, at most 200 colours) + setcolor.
 * elcolor (numel) receives the elements colour by colour (1-based),
 * colorg (2, ncolors) the first/last position of each colour (1-based).
 * Returns the number of colours, or -status. */
int orc_colormsh(const int *ix, int nnode, int numel, int nen, int nenv,
                 int *elcolor, int *colorg, int maxcolors_out) {
  const int nen1 = nen + 1;
  int *nincid = calloc((size_t)nnode + 1, sizeof(int));
  int *icolor = calloc((size_t)numel + 1, sizeof(int));
  if (!nincid || !icolor) { free(nincid); free(icolor); return -ORC_ERR_OOM; }
  int maxgrade = 0;
  for (int i = 1; i <= numel; i++)
    for (int j = 1; j <= nenv; j++) {
      int node = ix[(size_t)(i - 1) * nen1 + (j - 1)];
      if (node > 0) {
        nincid[node]++;
        if (nincid[node] > maxgrade) maxgrade = nincid[node];
      }
    }
  int *incid = calloc((size_t)maxgrade * (nnode + 1), sizeof(int));
  if (!incid) { free(nincid); free(icolor); return -ORC_ERR_OOM; }
#define INCID(m, node) incid[(size_t)((node) - 1) * maxgrade + ((m) - 1)]
  for (int i = 1; i <= nnode; i++) nincid[i] = 0;
  for (int i = 1; i <= numel; i++)
    for (int j = 1; j <= nenv; j++) {
      int node = ix[(size_t)(i - 1) * nen1 + (j - 1)];
      if (node > 0) {
        nincid[node]++;
        INCID(nincid[node], node) = i;
      }
    }
  const int maxcolors = 200;
  int numcolors = 0, quit = 0;
  for (int c = 1; c <= maxcolors && !quit; c++) {
    for (int node = 1; node <= nnode; node++) {
      int found = 0, l = nincid[node];
      for (int m = 1; m <= l; m++)
        if (icolor[INCID(m, node)] == c) found = 1;
      if (found) continue;
      int ielfirst = 0;
      for (int m = 1; m <= l; m++)
        if (icolor[INCID(m, node)] == 0) ielfirst = INCID(m, node);
      if (ielfirst == 0) continue;
      icolor[ielfirst] = c;
      for (int j = 1; j <= nenv; j++) {
        int ixj = ix[(size_t)(ielfirst - 1) * nen1 + (j - 1)];
        if (ixj <= 0) continue;
        for (int k = 1; k <= nincid[ixj]; k++) {
          int ik = INCID(k, ixj);
          if (icolor[ik] == 0) icolor[ik] = -1;
        }
      }
    }
    quit = 1;
    for (int n = 1; n <= numel; n++)
      if (icolor[n] == -1) { icolor[n] = 0; quit = 0; }
    numcolors = c;
  }
#undef INCID
  free(incid);
  free(nincid);
  if (!quit || numcolors > maxcolors_out) { free(icolor); return -ORC_ERR_ARG; }
  /* setcolor (Colormsh.f:255-308) */
  int ipos = 1;
  for (int c = 1; c <= numcolors; c++) {
    int count = 0, first = 1;
    for (int j = 1; j <= numel; j++)
      if (icolor[j] == c) {
        elcolor[ipos - 1] = j;
        if (first) colorg[(size_t)(c - 1) * 2] = ipos;
        first = 0;
        ipos++;
        count++;
      }
    colorg[(size_t)(c - 1) * 2 + 1] = colorg[(size_t)(c - 1) * 2] + count - 1;
  }
  free(icolor);
  return numcolors;
}

/* Pform.f:108-183: the OpenMP element loop over colours (omp_elmt), each
 * thread with private element arrays; same element and assembly routines as
 * the sequential loop.  elcolor/colorg from orc_colormsh. */
int orc_pform_k_omp(const int *ix, const int *ie, const double *e, int prop,
                    const double *x, const int *id, const int *ia, const int *ja,
                    double *al, double *ad, double *b, const double *u, int numel,
                    int nen, int nenv, int ndf, int ndm, int neq, long long nad,
                    const int *elcolor, const int *colorg, int numcolors, int nth,
                    int *bad_el) {
  const int nen1 = nen + 1;
  if (nen > 8 || ndf > 3 || ndm > 3) return ORC_ERR_ARG;
  memset(al, 0, (size_t)nad * sizeof(double));
  memset(ad, 0, (size_t)neq * sizeof(double));
  int status = ORC_OK, bad = 0;
#pragma omp parallel num_threads(nth)
  {
    double xl[3 * 8], ul[24], pl[24], sl[24 * 24];
    int ld[24];
    for (int ic = 1; ic <= numcolors; ic++) {
#pragma omp for schedule(static)
      for (int jc = colorg[(ic - 1) * 2]; jc <= colorg[(ic - 1) * 2 + 1]; jc++) {
        int nel = elcolor[jc - 1];
        const int *ixe = &ix[(size_t)(nel - 1) * nen1];
        int kk = 0;
        for (int i = 1; i <= nen; i++) {
          int no = ixe[i - 1];
          for (int j = 1; j <= ndf; j++) {
            ld[kk] = id[(size_t)(no - 1) * ndf + (j - 1)];
            ul[kk] = u[(size_t)(no - 1) * ndf + (j - 1)];
            pl[kk] = 0.0;
            kk++;
          }
        }
        for (int i = 1; i <= nenv; i++) {
          int no = ixe[i - 1];
          for (int j = 1; j <= ndm; j++)
            xl[(size_t)(i - 1) * ndm + (j - 1)] = x[(size_t)(no - 1) * ndm + (j - 1)];
        }
        int ma = ixe[nen], iel = ie[ma - 1], nst;
        int st = elmlib_k(iel, &e[(size_t)(ma - 1) * prop], xl, ndm, sl, &nst);
        if (st) {
#pragma omp critical
          { if (!status || nel < bad) { status = st; bad = nel; } }
          continue;
        }
        lku_m(sl, ul, pl, nst);
        assbly_csr(sl, pl, ld, ia, ja, al, ad, b, nst, neq, 1, 1);
      }
    }
  }
  if (status && bad_el) *bad_el = bad;
  return status;
}

/* Pform.f isw = 4 for 2-D elements: distributed edge tractions of TRIA3
 * (Elmlib02.f:214-314) and QUAD4 (Elmlib02.f:856-910).  eload(7,numel) gives
 * per side the load number; loadvec(2,numload) the type-40 traction vector
 * (Pload.f:246-249, tload).  Only the rhs is formed: b(k) -= p(i). */
int orc_pform_edge_loads(const int *ix, const int *ie, const double *x,
                         const int *id, const int *eload,
                         const double *loadvec, double *b, int numel, int nen,
                         int ndf, int ndm, int neq, int *bad_el) {
  static const int tri_side[3][2] = {{1, 2}, {2, 3}, {3, 1}};
  static const int quad_side[4][2] = {{1, 2}, {2, 3}, {3, 4}, {4, 1}};
  const int nen1 = nen + 1;
  if (ndm != 2 || ndf != 2) return ORC_ERR_ARG;
  for (int nel = 1; nel <= numel; nel++) {
    const int *ixe = &ix[(size_t)(nel - 1) * nen1];
    const int *iq = &eload[(size_t)(nel - 1) * 7];
    int ma = ixe[nen], iel = ie[ma - 1];
    int nside = (iel == 2 || iel == 3) ? 3 : (iel == 4 || iel == 5) ? 4 : 0;
    if (nside == 0) return ORC_ERR_BAD_ELEMENT;
    int tp = 0;
    for (int i = 0; i < nside; i++) tp += iq[i];
    if (tp <= 0) continue;
    double p[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int j = 1; j <= nside; j++) {
      if (iq[j - 1] <= 0) continue;
      const int *sn = nside == 3 ? tri_side[j - 1] : quad_side[j - 1];
      double xf[2][2];
      for (int i = 0; i < 2; i++) {
        int no = ixe[sn[i] - 1];
        xf[i][0] = x[(size_t)(no - 1) * ndm + 0];
        xf[i][1] = x[(size_t)(no - 1) * ndm + 1];
      }
      double det = (xf[1][0] - xf[0][0]) * (xf[1][0] - xf[0][0]) +
                   (xf[1][1] - xf[0][1]) * (xf[1][1] - xf[0][1]);
      if (det <= 0.0) { if (bad_el) *bad_el = nel; return ORC_ERR_BAD_DET; }
      det = sqrt(det);
      const double *face_f = &loadvec[(size_t)(iq[j - 1] - 1) * 2];
      double wt1 = 0.5 * det;
      for (int i = 0; i < 2; i++) {
        int no = sn[i], l1 = 2 * no - 1, l2 = l1 + 1;
        p[l1 - 1] = p[l1 - 1] - face_f[0] * wt1;
        p[l2 - 1] = p[l2 - 1] - face_f[1] * wt1;
      }
    }
    /* assbly with lhs = .false., rhs = .true. */
    for (int i = 1; i <= 2 * nside; i++) {
      int node = ixe[(i - 1) / 2];
      int k = id[(size_t)(node - 1) * ndf + ((i - 1) % 2)];
      if (k <= 0 || k > neq) continue;
      b[k - 1] = b[k - 1] - p[i - 1];
    }
  }
  return ORC_OK;
}

/* Pload.f:2-58 pload_mec with f(ndf,nnode) already evaluated:
 * b(k) = f for a free dof, u = f for a prescribed one. */
void orc_pload(const int *id, const double *f, double *u, double *b, int nnode,
               int ndf) {
  for (int i = 1; i <= nnode; i++)
    for (int j = 1; j <= ndf; j++) {
      size_t q = (size_t)(i - 1) * ndf + (j - 1);
      int k = id[q];
      if (k > 0) b[k - 1] = f[q];
      else u[q] = f[q];
    }
}

/* Predict.f:183-209 update_mec: u(j,i) = x(id(j,i)) for free dofs. */
void orc_update(const int *id, const double *xsol, double *u, int nnode,
                int ndf) {
  for (size_t q = 0; q < (size_t)nnode * ndf; q++)
    if (id[q] > 0) u[q] = xsol[id[q] - 1];
}

/* ---------------------------------------------------------------------- */
/* Matvec.f / Iters.f -- CSRC SpMV, dot, Jacobi PCG, BiCGSTAB, GMRES        */
/* ---------------------------------------------------------------------- */

/* Matvec.f:528-621 matvec_csrcsym1: y = (D + L + L^T) x, 2-way unrolled. */
void orc_matvec_csrcsym1(int neq, const int *ia, const int *ja,
                         const double *ad, const double *al, const double *x,
                         double *y) {
  for (int i = 1; i <= neq; i++) {
    double xi = x[i - 1];
    double t = ad[i - 1] * xi;
    int k1 = ia[i - 1], k2 = ia[i];
    if (k2 != k1) {
      int n = (k2 - k1) % 2;
      if (n != 0) {
        int jak1 = ja[k1 - 1];
        t = t + al[k1 - 1] * x[jak1 - 1];
        y[jak1 - 1] = y[jak1 - 1] + al[k1 - 1] * xi;
        k1 = k1 + 1;
      }
      for (int k = k1; k <= k2 - 1; k += 2) {
        int jak = ja[k - 1], jak1 = ja[k];
        double s = al[k - 1], s1 = al[k];
        t = t + s * x[jak - 1] + s1 * x[jak1 - 1];
        y[jak - 1] = y[jak - 1] + s * xi;
        y[jak1 - 1] = y[jak1 - 1] + s1 * xi;
      }
    }
    y[i - 1] = t;
  }
}

/* Matvec.f:1090-1191 matvec_csrcrsym1: y = A x on an overlapping
 * partition -- the lower CSRC part with its mirror as matvec_csrcsym1, then
 * each owned row times the halo values through the rectangular part (ia1,
 * ja1, ar), 2-way unrolled; x holds the owned then the halo values (the
 * exchange, communicate(), has filled the halo). */
void orc_matvec_csrcrsym1(int neq, const int *ia, const int *ja, const int *ia1,
                          const int *ja1, const double *ad, const double *al,
                          const double *ar, const double *x, double *y) {
  for (int i = 1; i <= neq; i++) {
    double xi = x[i - 1];
    double t = ad[i - 1] * xi;
    int k1 = ia[i - 1], k2 = ia[i];
    if (k2 != k1) {
      if ((k2 - k1) % 2 != 0) {
        int jak1 = ja[k1 - 1];
        t = t + al[k1 - 1] * x[jak1 - 1];
        y[jak1 - 1] = y[jak1 - 1] + al[k1 - 1] * xi;
        k1 = k1 + 1;
      }
      for (int k = k1; k <= k2 - 1; k += 2) {
        int jak = ja[k - 1], jak1 = ja[k];
        double s = al[k - 1], s1 = al[k];
        t = t + s * x[jak - 1] + s1 * x[jak1 - 1];
        y[jak - 1] = y[jak - 1] + s * xi;
        y[jak1 - 1] = y[jak1 - 1] + s1 * xi;
      }
    }
    k1 = ia1[i - 1];
    k2 = ia1[i];
    if (k2 != k1) {
      if ((k2 - k1) % 2 != 0) {
        t = t + ar[k1 - 1] * x[ja1[k1 - 1] - 1];
        k1 = k1 + 1;
      }
      for (int k = k1; k <= k2 - 1; k += 2)
        t = t + ar[k - 1] * x[ja1[k - 1] - 1] + ar[k] * x[ja1[k] - 1];
    }
    y[i - 1] = t;
  }
}

/* Matvec.f:1237-1266 dot_par (single rank) */
double orc_dot(const double *a, const double *b, int n) {
  double tmp = 0.0;
  for (int i = 0; i < n; i++) tmp = tmp + a[i] * b[i];
  return tmp;
}

/* Matvec.f:1470-1531 flop_csrc / flop_cg (icod = 2, PCG) */
double orc_flop_cg(int neq, long long nad, int it) {
  double fmatvec = (double)neq + 4.0 * (double)nad;
  double fdot = 2.0 * (double)neq; /* flop_dot = 2*neq */
  return (fmatvec + 2.0 * fdot + 7.0 * neq + 2.0) * it;
}

/* Solver diagnostics; mirrors the fields PCG prints (Iters.f:473-490). */
typedef struct {
  int iters;
  int status;
  double xkx, norm_x, norm_r, norm_m_r, conv, seconds, mflops;
} orc_info;

/* Precond.f:22-45 pre_diag (pd = .false.): m = 1/ad. */
void orc_pre_diag(const double *ad, double *m, int neq) {
  for (int i = 0; i < neq; i++) m[i] = 1.0 / ad[i];
}

/* Iters.f:252-524 pcg (fnew = .true.), with Solv.f:65-69 building m. */
int orc_pcg(int neq, long long nad, const int *ia, const int *ja,
            const double *ad, const double *al, const double *b, double *x,
            double tol, int maxit, orc_info *info) {
  double t0 = wall();
  for (int i = 0; i < neq; i++)
    if (ad[i] == 0.0) { if (info) info->status = ORC_ERR_ZERO_DIAG; return ORC_ERR_ZERO_DIAG; }
  double *m = (double *)malloc((size_t)neq * sizeof(double));
  double *z = (double *)malloc((size_t)neq * sizeof(double));
  double *r = (double *)malloc((size_t)neq * sizeof(double));
  double *p = (double *)malloc((size_t)neq * sizeof(double));
  if (!m || !z || !r || !p) { free(m); free(z); free(r); free(p); return ORC_ERR_OOM; }
  orc_pre_diag(ad, m, neq);
  for (int i = 0; i < neq; i++) x[i] = 0.0;
  for (int i = 0; i < neq; i++) z[i] = b[i] * m[i];
  double d = orc_dot(b, z, neq);
  double conv = tol * sqrt(fabs(d));
  orc_matvec_csrcsym1(neq, ia, ja, ad, al, x, z);
  for (int i = 0; i < neq; i++) {
    r[i] = b[i] - z[i];
    z[i] = r[i] * m[i];
    p[i] = z[i];
  }
  d = orc_dot(r, z, neq);
  int j, converged = 0;
  for (j = 1; j <= maxit; j++) {
    orc_matvec_csrcsym1(neq, ia, ja, ad, al, p, z);
    double alpha = d / orc_dot(z, p, neq);
    for (int i = 0; i < neq; i++) {
      x[i] = x[i] + alpha * p[i];
      r[i] = r[i] - alpha * z[i];
      z[i] = r[i] * m[i];
    }
    double di = orc_dot(r, z, neq);
    double beta = di / d;
    for (int i = 0; i < neq; i++) p[i] = z[i] + beta * p[i];
    d = di;
    if (sqrt(fabs(d)) < conv) { converged = 1; break; }
  }
  int status = ORC_OK;
  if (!converged) { status = ORC_ERR_NO_CONVERGENCE; j = maxit; }
  orc_matvec_csrcsym1(neq, ia, ja, ad, al, x, z);
  double xkx = orc_dot(x, z, neq);
  double norm = sqrt(orc_dot(x, x, neq));
  for (int i = 0; i < neq; i++) {
    r[i] = b[i] - z[i];
    z[i] = r[i] * m[i];
  }
  double norm_m_r = sqrt(fabs(orc_dot(r, z, neq)));
  double norm_r = sqrt(orc_dot(r, r, neq));
  double time = wall() - t0;
  if (info) {
    info->iters = j;
    info->status = status;
    info->xkx = xkx;
    info->norm_x = norm;
    info->norm_r = norm_r;
    info->norm_m_r = norm_m_r;
    info->conv = conv;
    info->seconds = time;
    info->mflops = time > 0 ? orc_flop_cg(neq, nad, j) * 1e-6 / time : 0.0;
  }
  free(m); free(z); free(r); free(p);
  return status;
}

/* Iters.f:1079-1349 pbicgstab: right-Jacobi BiCGSTAB, 2-norm test. */
int orc_pbicgstab(int neq, long long nad, const int *ia, const int *ja,
                  const double *ad, const double *al, const double *b,
                  double *x, double tol, int maxit, orc_info *info) {
  double t0 = wall();
  for (int i = 0; i < neq; i++)
    if (ad[i] == 0.0) { if (info) info->status = ORC_ERR_ZERO_DIAG; return ORC_ERR_ZERO_DIAG; }
  size_t sz = (size_t)neq * sizeof(double);
  double *m = malloc(sz), *t = malloc(sz), *v = malloc(sz), *r = malloc(sz),
         *p = malloc(sz), *z = malloc(sz), *r0 = malloc(sz);
  if (!m || !t || !v || !r || !p || !z || !r0) {
    free(m); free(t); free(v); free(r); free(p); free(z); free(r0);
    return ORC_ERR_OOM;
  }
  orc_pre_diag(ad, m, neq);
  for (int i = 0; i < neq; i++) x[i] = 0.0;
  double d = orc_dot(b, b, neq);
  double conv = tol * sqrt(fabs(d));
  orc_matvec_csrcsym1(neq, ia, ja, ad, al, x, z);
  for (int i = 0; i < neq; i++) {
    r0[i] = b[i] - z[i];
    p[i] = r0[i];
    r[i] = r0[i];
    z[i] = p[i] * m[i];
  }
  int j, converged = 0;
  for (j = 1; j <= maxit; j++) {
    orc_matvec_csrcsym1(neq, ia, ja, ad, al, z, v);
    double rr0 = orc_dot(r, r0, neq);
    double alpha = rr0 / orc_dot(v, r0, neq);
    for (int i = 0; i < neq; i++) {
      x[i] = x[i] + alpha * z[i];
      r[i] = r[i] - alpha * v[i];
      z[i] = r[i] * m[i];
    }
    d = orc_dot(r, r, neq);
    if (sqrt(fabs(d)) < conv) { converged = 1; break; }
    orc_matvec_csrcsym1(neq, ia, ja, ad, al, z, t);
    double w = orc_dot(t, r, neq) / orc_dot(t, t, neq);
    for (int i = 0; i < neq; i++) {
      x[i] = x[i] + w * z[i];
      r[i] = r[i] - w * t[i];
    }
    d = orc_dot(r, r, neq);
    if (sqrt(fabs(d)) < conv) { converged = 1; break; }
    double beta = (orc_dot(r, r0, neq) / rr0) * (alpha / w);
    for (int i = 0; i < neq; i++) {
      p[i] = r[i] + beta * (p[i] - w * v[i]);
      z[i] = p[i] * m[i];
    }
  }
  int status = ORC_OK;
  if (!converged) { status = ORC_ERR_NO_CONVERGENCE; j = maxit; }
  orc_matvec_csrcsym1(neq, ia, ja, ad, al, x, z);
  double xkx = orc_dot(x, z, neq);
  double norm = sqrt(orc_dot(x, x, neq));
  for (int i = 0; i < neq; i++) r[i] = b[i] - z[i];
  double norm_r = sqrt(orc_dot(r, r, neq));
  for (int i = 0; i < neq; i++) z[i] = r[i] * m[i];
  double norm_m_r = sqrt(fabs(orc_dot(r, z, neq)));
  if (info) {
    info->iters = j;
    info->status = status;
    info->xkx = xkx;
    info->norm_x = norm;
    info->norm_r = norm_r;
    info->norm_m_r = norm_m_r;
    info->conv = conv;
    info->seconds = wall() - t0;
    info->mflops = 0.0;
  }
  free(m); free(t); free(v); free(r); free(p); free(z); free(r0);
  return status;
}

/* Iters.f:812-1075 bicgstab: BiCGSTAB without a preconditioner, x0 = 0
 * (fnew), stopping on the 2-norm, sqrt|(r, r)| < tol sqrt|(b, b)|, after
 * each half step.  Its beta takes (r, b) where the method has (r, r0)
 * (Iters.f:987); with x0 = 0, r0 = b - K 0 = b exactly, so the two agree.
 * Unreachable from the reference's decks (its only call is commented out,
 * Solv.f:334); norm_m_r is reported as ||b - K x|| (no M). */
int orc_bicgstab(int neq, long long nad, const int *ia, const int *ja,
                 const double *ad, const double *al, const double *b,
                 double *x, double tol, int maxit, orc_info *info) {
  double t0 = wall();
  (void)nad;
  for (int i = 0; i < neq; i++)
    if (ad[i] == 0.0) { if (info) info->status = ORC_ERR_ZERO_DIAG; return ORC_ERR_ZERO_DIAG; }
  size_t sz = (size_t)neq * sizeof(double);
  double *t = malloc(sz), *v = malloc(sz), *r = malloc(sz), *p = malloc(sz), *r0 = malloc(sz);
  if (!t || !v || !r || !p || !r0) {
    free(t); free(v); free(r); free(p); free(r0);
    return ORC_ERR_OOM;
  }
  for (int i = 0; i < neq; i++) x[i] = 0.0;
  double d = orc_dot(b, b, neq);
  double conv = tol * sqrt(fabs(d));
  orc_matvec_csrcsym1(neq, ia, ja, ad, al, x, p);
  for (int i = 0; i < neq; i++) {
    r0[i] = b[i] - p[i];
    r[i] = r0[i];
    p[i] = r0[i];
  }
  int j, converged = 0;
  for (j = 1; j <= maxit; j++) {
    orc_matvec_csrcsym1(neq, ia, ja, ad, al, p, v);
    double rr0 = orc_dot(r, r0, neq);
    double alpha = rr0 / orc_dot(v, r0, neq);
    for (int i = 0; i < neq; i++) {
      x[i] = x[i] + alpha * p[i];
      r[i] = r[i] - alpha * v[i];
    }
    d = orc_dot(r, r, neq);
    if (sqrt(fabs(d)) < conv) { converged = 1; break; }
    orc_matvec_csrcsym1(neq, ia, ja, ad, al, r, t);
    double w = orc_dot(t, r, neq) / orc_dot(t, t, neq);
    for (int i = 0; i < neq; i++) {
      x[i] = x[i] + w * r[i];
      r[i] = r[i] - w * t[i];
    }
    d = orc_dot(r, r, neq);
    if (sqrt(fabs(d)) < conv) { converged = 1; break; }
    double beta = (orc_dot(r, b, neq) / rr0) * (alpha / w);
    for (int i = 0; i < neq; i++) p[i] = r[i] + beta * (p[i] - w * v[i]);
  }
  int status = ORC_OK;
  if (!converged) { status = ORC_ERR_NO_CONVERGENCE; j = maxit; }
  orc_matvec_csrcsym1(neq, ia, ja, ad, al, x, p);
  double xkx = orc_dot(x, p, neq);
  double norm = sqrt(orc_dot(x, x, neq));
  for (int i = 0; i < neq; i++) r[i] = b[i] - p[i];
  double norm_r = sqrt(orc_dot(r, r, neq));
  if (info) {
    info->iters = j;
    info->status = status;
    info->xkx = xkx;
    info->norm_x = norm;
    info->norm_r = norm_r;
    info->norm_m_r = norm_r;
    info->conv = conv;
    info->seconds = wall() - t0;
    info->mflops = 0.0;
  }
  free(t); free(v); free(r); free(p); free(r0);
  return status;
}

/* Iters.f:528-808 gmres: left-Jacobi GMRES(k), modified Gram-Schmidt,
 * Givens rotations; maxit counts restart cycles; iters = total inner steps. */
int orc_gmres(int neq, long long nad, const int *ia, const int *ja,
              const double *ad, const double *al, const double *b, double *x,
              int k, double tol, int maxit, orc_info *info) {
  double t0 = wall();
  for (int i = 0; i < neq; i++)
    if (ad[i] == 0.0) { if (info) info->status = ORC_ERR_ZERO_DIAG; return ORC_ERR_ZERO_DIAG; }
  double *m = malloc((size_t)neq * sizeof(double));
  double *g = malloc((size_t)neq * (k + 1) * sizeof(double));
  double *h = calloc((size_t)(k + 1) * k, sizeof(double));
  double *y = calloc((size_t)k + 1, sizeof(double));
  double *c = calloc((size_t)k + 1, sizeof(double));
  double *s = calloc((size_t)k + 1, sizeof(double));
  double *e = calloc((size_t)k + 2, sizeof(double));
  if (!m || !g || !h || !y || !c || !s || !e) {
    free(m); free(g); free(h); free(y); free(c); free(s); free(e);
    return ORC_ERR_OOM;
  }
  orc_pre_diag(ad, m, neq);
#define G(i, j) g[(size_t)((j) - 1) * neq + ((i) - 1)]
#define H(i, j) h[(size_t)((j) - 1) * (k + 1) + ((i) - 1)]
  for (int i = 1; i <= neq; i++) {
    x[i - 1] = 0.0;
    G(i, 1) = b[i - 1] * m[i - 1];
  }
  double norm = sqrt(orc_dot(&G(1, 1), &G(1, 1), neq));
  double econv = tol * norm;
  int nit = 0, ni = 0, l, converged = 0;
  for (l = 1; l <= maxit; l++) {
    orc_matvec_csrcsym1(neq, ia, ja, ad, al, x, &G(1, 1));
    for (int i = 1; i <= neq; i++) G(i, 1) = (b[i - 1] - G(i, 1)) * m[i - 1];
    e[1] = sqrt(orc_dot(&G(1, 1), &G(1, 1), neq));
    for (int i = 1; i <= neq; i++) G(i, 1) = G(i, 1) / e[1];
    ni = 0;
    for (int i = 1; i <= k; i++) {
      nit++;
      ni++;
      orc_matvec_csrcsym1(neq, ia, ja, ad, al, &G(1, i), &G(1, i + 1));
      for (int jj = 1; jj <= neq; jj++) G(jj, i + 1) = G(jj, i + 1) * m[jj - 1];
      for (int jj = 1; jj <= i; jj++) {
        double beta = orc_dot(&G(1, i + 1), &G(1, jj), neq);
        for (int ic = 1; ic <= neq; ic++) G(ic, i + 1) = G(ic, i + 1) - beta * G(ic, jj);
        H(jj, i) = beta;
      }
      norm = sqrt(orc_dot(&G(1, i + 1), &G(1, i + 1), neq));
      H(i + 1, i) = norm;
      for (int ic = 1; ic <= neq; ic++) G(ic, i + 1) = G(ic, i + 1) / norm;
      for (int jj = 1; jj <= i - 1; jj++) {
        double aux1 = c[jj] * H(jj, i) + s[jj] * H(jj + 1, i);
        double aux2 = -s[jj] * H(jj, i) + c[jj] * H(jj + 1, i);
        H(jj, i) = aux1;
        H(jj + 1, i) = aux2;
      }
      double rr = sqrt(H(i, i) * H(i, i) + H(i + 1, i) * H(i + 1, i));
      c[i] = H(i, i) / rr;
      s[i] = H(i + 1, i) / rr;
      H(i, i) = rr;
      H(i + 1, i) = 0.0;
      e[i + 1] = -s[i] * e[i];
      e[i] = c[i] * e[i];
      if (fabs(e[i + 1]) <= econv) break;
    }
    y[ni] = e[ni] / H(ni, ni);
    for (int i = ni - 1; i >= 1; i--) {
      y[i] = 0.0;
      for (int jj = i + 1; jj <= ni; jj++) y[i] = y[i] - H(i, jj) * y[jj];
      y[i] = (y[i] + e[i]) / H(i, i);
    }
    for (int i = 1; i <= neq; i++)
      for (int jj = 1; jj <= ni; jj++) x[i - 1] = x[i - 1] + y[jj] * G(i, jj);
    if (fabs(e[ni + 1]) <= econv) { converged = 1; break; }
  }
  orc_matvec_csrcsym1(neq, ia, ja, ad, al, x, &G(1, 1));
  double xkx = orc_dot(x, &G(1, 1), neq);
  double normx = sqrt(orc_dot(x, x, neq));
  for (int i = 1; i <= neq; i++) G(i, 2) = b[i - 1] - G(i, 1);
  double norm_r = sqrt(orc_dot(&G(1, 2), &G(1, 2), neq));
  /* ||b - Ax||_M is not printed by the reference's GMRES; it is added here
   * so that every solver reports the same diagnostics. */
  double norm_m_r = 0.0;
  for (int i = 1; i <= neq; i++) norm_m_r += G(i, 2) * G(i, 2) * m[i - 1];
  norm_m_r = sqrt(fabs(norm_m_r));
#undef G
#undef H
  int status = converged ? ORC_OK : ORC_ERR_NO_CONVERGENCE;
  if (info) {
    info->iters = nit;
    info->status = status;
    info->xkx = xkx;
    info->norm_x = normx;
    info->norm_r = norm_r;
    info->norm_m_r = norm_m_r;
    info->conv = econv;
    info->seconds = wall() - t0;
    info->mflops = 0.0;
  }
  free(m); free(g); free(h); free(y); free(c); free(s); free(e);
  return status;
}

/* ---------------------------------------------------------------------- */
/* OpenMP CPU path: Matrix_partition.f, Matvec_omp.f, Iters_omp.f          */
/* ---------------------------------------------------------------------- */

typedef struct {
  int nth;
  int *begin, *end, *height; /* 1-based rows, per thread (0-based index) */
} orc_part;

/* Matrix_partition.f:98-150 partition_csrc_bynonzeros (ovlp = .false.) and
 * Matrix_partition.f:196-231 compute_effective_work. */
static int partition_matrix(const int *ia, const int *ja, int neq, int nth,
                            orc_part *pt) {
  pt->nth = nth;
  pt->begin = calloc((size_t)nth, sizeof(int));
  pt->end = calloc((size_t)nth, sizeof(int));
  pt->height = calloc((size_t)nth, sizeof(int));
  int *size = calloc((size_t)nth, sizeof(int));
  if (!pt->begin || !pt->end || !pt->height || !size) { free(size); return ORC_ERR_OOM; }
  long long nad = (long long)ia[neq] - 1;
  long long mean_variables = (2 * nad + neq) / nth + 1;
  int line = 2;
  pt->begin[0] = 1;
  for (int i = 0; i < nth - 1; i++) {
    size[i] = 0;
    for (;;) {
      if (line > neq + 1) break; /* guard: the Fortran reads past ia here */
      int tam = 2 * (ia[line - 1] - ia[line - 2]) + 1;
      if (size[i] + tam <= mean_variables) {
        size[i] += tam;
        pt->end[i] = line - 1;
        pt->begin[i + 1] = line;
        line++;
      } else break;
    }
  }
  pt->end[nth - 1] = neq;
  for (int t = 0; t < nth; t++) {
    int h = pt->begin[t];
    for (int i = pt->begin[t]; i <= pt->end[t]; i++) {
      int c = ja[ia[i - 1] - 1]; /* ja(ia(i)); reads the next row when empty */
      if (ia[i - 1] - 1 < nad && c < h) h = c;
    }
    pt->height[t] = h;
  }
  free(size);
  for (int t = 0; t < nth; t++)
    if (pt->height[t] <= 0 || pt->begin[t] <= 0 || pt->end[t] <= 0) return ORC_ERR_ARG;
  return ORC_OK;
}

static void part_free(orc_part *pt) {
  free(pt->begin); free(pt->end); free(pt->height);
}

/* Matvec_omp.f:150-245 matvec_csrcsym_omp, called inside a parallel region.
 * thread_y is (neq, nth). */
static void matvec_csrcsym_omp_body(int neq, const int *ia, const int *ja,
                                    const double *ad, const double *al,
                                    const double *x, double *y,
                                    double *thread_y, const orc_part *pt) {
#ifdef _OPENMP
  int tid = omp_get_thread_num();
#else
  int tid = 0;
#endif
  for (int t = 0; t < pt->nth; t++) {
    size_t inc = (size_t)t * neq;
#pragma omp for schedule(static)
    for (int j = pt->height[t]; j <= pt->begin[t] - 1; j++) thread_y[j - 1 + inc] = 0.0;
  }
  size_t inc = (size_t)tid * neq;
#pragma omp barrier
  for (int i = pt->begin[tid]; i <= pt->end[tid]; i++) {
    y[i - 1] = 0.0;
    double xi = x[i - 1];
    double t = ad[i - 1] * xi;
    for (int k = ia[i - 1]; k <= ia[i] - 1; k++) {
      int jak = ja[k - 1];
      double s = al[k - 1];
      t = t + s * x[jak - 1];
      thread_y[jak - 1 + inc] = thread_y[jak - 1 + inc] + s * xi;
    }
    thread_y[i - 1 + inc] = t;
  }
#pragma omp barrier
  for (int t = 0; t < pt->nth; t++) {
    size_t inc2 = (size_t)t * neq;
#pragma omp for schedule(static)
    for (int j = pt->height[t]; j <= pt->end[t]; j++) y[j - 1] = y[j - 1] + thread_y[j - 1 + inc2];
  }
}

/* Standalone OpenMP SpMV (for timing the CPU baseline SpMV). */
int orc_matvec_csrcsym_omp(int neq, const int *ia, const int *ja,
                           const double *ad, const double *al, const double *x,
                           double *y, int nth, int reps, double *seconds) {
  orc_part pt;
  int st = partition_matrix(ia, ja, neq, nth, &pt);
  if (st) { part_free(&pt); return st; }
  double *thread_y = calloc((size_t)neq * nth, sizeof(double));
  if (!thread_y) { part_free(&pt); return ORC_ERR_OOM; }
  double t0 = wall();
  for (int r = 0; r < reps; r++) {
#pragma omp parallel num_threads(nth)
    matvec_csrcsym_omp_body(neq, ia, ja, ad, al, x, y, thread_y, &pt);
  }
  if (seconds) *seconds = wall() - t0;
  free(thread_y);
  part_free(&pt);
  return ORC_OK;
}

/* Iters_omp.f:17-334 pcg_omp with matvec_csrcsym_omp and dot_par_omp.
 * maxit bounds the iterations; when stop_at_maxit is nonzero, reaching maxit
 * without convergence is reported as status 0 (a bounded timing sample). */
int orc_pcg_omp(int neq, long long nad, const int *ia, const int *ja,
                const double *ad, const double *al, const double *b, double *x,
                double tol, int maxit, int nth, int stop_at_maxit,
                orc_info *info) {
  for (int i = 0; i < neq; i++)
    if (ad[i] == 0.0) { if (info) info->status = ORC_ERR_ZERO_DIAG; return ORC_ERR_ZERO_DIAG; }
  orc_part pt;
  int st = partition_matrix(ia, ja, neq, nth, &pt);
  if (st) { part_free(&pt); return st; }
  size_t sz = (size_t)neq * sizeof(double);
  double *m = malloc(sz), *z = malloc(sz), *r = malloc(sz), *p = malloc(sz);
  double *thread_y = calloc((size_t)neq * nth, sizeof(double));
  if (!m || !z || !r || !p || !thread_y) {
    free(m); free(z); free(r); free(p); free(thread_y); part_free(&pt);
    return ORC_ERR_OOM;
  }
  orc_pre_diag(ad, m, neq);
  double t0 = wall();
  double omp_dot = 0.0;
  int it_out = 0, conv_out = 0;
  double xkx_o = 0, norm_o = 0, norm_r_o = 0, norm_m_r_o = 0, conv_o = 0;
#pragma omp parallel num_threads(nth)
  {
    double d, di, conv, alpha, beta;
    int j, converged = 0;
#pragma omp for schedule(static)
    for (int i = 0; i < neq; i++) x[i] = 0.0;
#pragma omp for schedule(static)
    for (int i = 0; i < neq; i++) z[i] = b[i] * m[i];
    /* dot_par_omp (Matvec_omp.f:438-490) */
#define OMP_DOT(A, B, OUT)                                \
  do {                                                    \
    _Pragma("omp single") omp_dot = 0.0;                  \
    _Pragma("omp for schedule(static) reduction(+:omp_dot)") \
    for (int i_ = 0; i_ < neq; i_++) omp_dot = omp_dot + (A)[i_] * (B)[i_]; \
    (OUT) = omp_dot;                                      \
    _Pragma("omp barrier")                                \
  } while (0)
    OMP_DOT(b, z, d);
    conv = tol * sqrt(fabs(d));
    matvec_csrcsym_omp_body(neq, ia, ja, ad, al, x, z, thread_y, &pt);
#pragma omp for schedule(static)
    for (int i = 0; i < neq; i++) {
      r[i] = b[i] - z[i];
      z[i] = r[i] * m[i];
      p[i] = z[i];
    }
    OMP_DOT(r, z, d);
    for (j = 1; j <= maxit; j++) {
      matvec_csrcsym_omp_body(neq, ia, ja, ad, al, p, z, thread_y, &pt);
      double zp;
      OMP_DOT(z, p, zp);
      alpha = d / zp;
#pragma omp for schedule(static)
      for (int i = 0; i < neq; i++) {
        x[i] = x[i] + alpha * p[i];
        r[i] = r[i] - alpha * z[i];
        z[i] = r[i] * m[i];
      }
      OMP_DOT(r, z, di);
      beta = di / d;
#pragma omp for schedule(static)
      for (int i = 0; i < neq; i++) p[i] = z[i] + beta * p[i];
      d = di;
      if (sqrt(fabs(d)) < conv) { converged = 1; break; }
    }
    if (!converged) j = maxit;
    matvec_csrcsym_omp_body(neq, ia, ja, ad, al, x, z, thread_y, &pt);
    double xkx, nx, nmr, nr;
    OMP_DOT(x, z, xkx);
    OMP_DOT(x, x, nx);
#pragma omp for schedule(static)
    for (int i = 0; i < neq; i++) {
      r[i] = b[i] - z[i];
      z[i] = r[i] * m[i];
    }
    OMP_DOT(r, z, nmr);
    OMP_DOT(r, r, nr);
#undef OMP_DOT
#pragma omp single
    {
      it_out = j;
      conv_out = converged;
      xkx_o = xkx;
      norm_o = sqrt(nx);
      norm_m_r_o = sqrt(fabs(nmr));
      norm_r_o = sqrt(nr);
      conv_o = conv;
    }
  }
  double time = wall() - t0;
  int status = (conv_out || stop_at_maxit) ? ORC_OK : ORC_ERR_NO_CONVERGENCE;
  if (info) {
    info->iters = it_out;
    info->status = status;
    info->xkx = xkx_o;
    info->norm_x = norm_o;
    info->norm_r = norm_r_o;
    info->norm_m_r = norm_m_r_o;
    info->conv = conv_o;
    info->seconds = time;
    info->mflops = time > 0 ? orc_flop_cg(neq, nad, it_out) * 1e-6 / time : 0.0;
  }
  free(m); free(z); free(r); free(p); free(thread_y); part_free(&pt);
  return status;
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---------------------------------------------------------------------- */
/* Write_vtk.f / Vtk.f -- the result file of write_mesh_res_mec            */
/* ---------------------------------------------------------------------- */

/* The Fortran edit descriptors the writer uses, as gfortran prints them:
 * Ew.d / Ew.dEe -> [-]0.d1..dd followed by E+xx (Ee: E+ and e digits; no
 * Ee and 99 < |x| <= 999: +xxx without the E), right-justified in w;
 * digits correctly rounded (glibc's exact conversion, ties to even); zero
 * prints exponent 0; NaN / Infinity right-justified; a field that does not
 * fit is w asterisks.  Iw -> right-justified, asterisks on overflow. */
static void orc_fmt_e(char *out, double x, int w, int d, int e) {
  char body[64];
  int n = 0;
  if (isnan(x)) {
    n = snprintf(body, sizeof body, "NaN");
  } else if (isinf(x)) {
    n = snprintf(body, sizeof body, "%s", x < 0 ? (w >= 9 ? "-Infinity" : "-Inf")
                                                : (w >= 8 ? "Infinity" : "Inf"));
  } else {
    char dig[40];
    int ex = 0;
    const double a = fabs(x);
    if (a == 0.0) {
      for (int i = 0; i < d; i++) dig[i] = '0';
      dig[d] = 0;
    } else {
      char tmp[64];
      snprintf(tmp, sizeof tmp, "%.*e", d - 1, a); /* D.DDDDe+XX */
      int k = 0;
      for (const char *p = tmp; *p && *p != 'e'; p++)
        if (*p != '.') dig[k++] = *p;
      dig[k] = 0;
      ex = atoi(strchr(tmp, 'e') + 1) + 1;
    }
    const int aex = ex < 0 ? -ex : ex;
    char expo[16];
    if (e == 0) {
      if (aex <= 99) snprintf(expo, sizeof expo, "E%c%02d", ex < 0 ? '-' : '+', aex);
      else if (aex <= 999) snprintf(expo, sizeof expo, "%c%03d", ex < 0 ? '-' : '+', aex);
      else expo[0] = 0, n = -1;
    } else {
      int lim = 1;
      for (int i = 0; i < e; i++) lim *= 10;
      if (aex < lim) snprintf(expo, sizeof expo, "E%c%0*d", ex < 0 ? '-' : '+', e, aex);
      else expo[0] = 0, n = -1;
    }
    if (n == 0)
      n = snprintf(body, sizeof body, "%s0.%s%s", signbit(x) ? "-" : "", dig, expo);
    if (n > w && n - 1 == w) { /* drop the optional leading zero */
      char *z = strstr(body, "0.");
      memmove(z, z + 1, strlen(z));
      n -= 1;
    }
  }
  if (n < 0 || n > w) {
    memset(out, '*', w);
    return;
  }
  memset(out, ' ', w - n);
  memcpy(out + w - n, body, n);
}

static void orc_fmt_i(char *out, long long v, int w) {
  char body[32];
  int n = snprintf(body, sizeof body, "%lld", v);
  if (n > w) {
    memset(out, '*', w);
    return;
  }
  memset(out, ' ', w - n);
  memcpy(out + w - n, body, n);
}

/* Writes E15.5 / E15.5E3 / Iw fields for the tests of the device formatter:
 * out gets n fields of width w (kind 0: Ew.d with e = 0; 1: Ew.dEe). */
void orc_fortran_e(const double *x, int n, int w, int d, int e, char *out) {
  for (int i = 0; i < n; i++) orc_fmt_e(out + (size_t)i * w, x[i], w, d, e);
}

static void put_be(FILE *f, const void *p, int bytes) {
  unsigned char b[8];
  memcpy(b, p, bytes);
  for (int i = bytes - 1; i >= 0; i--) fputc(b[i], f);
}
static void put_be_i32(FILE *f, int32_t v) { put_be(f, &v, 4); }
static void put_be_f64(FILE *f, double v) { put_be(f, &v, 8); }

/* VTK cell type and node count of the reference's element types
 * (elm_vtk / elm_vtu: TRIA3 5, QUAD4 9, TETRA4 10, HEXA8 12). */
static int vtk_cell(int iel, int *nnoel) {
  switch (iel) {
    case 2: case 3: *nnoel = 3; return 5;
    case 4: case 5: *nnoel = 4; return 9;
    case 6: *nnoel = 4; return 10;
    case 7: *nnoel = 8; return 12;
  }
  return -1;
}

/* make_full_tensor (Write_vtk.f:1166-1226): the 9 components of node i. */
static void full_tensor(const double *tx, int ntn, int i, double *t9) {
  const double *s = tx + (size_t)i * ntn;
  if (ntn == 4) {
    t9[0] = s[0]; t9[1] = s[3]; t9[2] = 0.0;
    t9[3] = s[3]; t9[4] = s[1]; t9[5] = 0.0;
    t9[6] = 0.0;  t9[7] = 0.0;  t9[8] = s[2];
  } else {
    t9[0] = s[0]; t9[1] = s[3]; t9[2] = s[5];
    t9[3] = s[3]; t9[4] = s[1]; t9[5] = s[4];
    t9[6] = s[5]; t9[7] = s[4]; t9[8] = s[2];
  }
}

/* write_mesh_res_mec (Write_vtk.f:742-985) with fprint(2) = u != NULL and
 * fprint(3) = tx != NULL: format 0 = the XML VTU ASCII file (legacy =
 * .false., bvtk = .false.: head_vtu, coor_vtu, elm_vtu, cell_prop_vtu,
 * point_prop_vtu), format 1 = the legacy binary file (legacy = .true.,
 * bvtk = .true.: head_vtk, coor_vtk, elm_vtk, cell_prop_vtk,
 * point_prop_vtk, big-endian stream).  All elements must be of one VTK
 * cell type (the reference's offsets loop assumes it, Vtk.f:1051). */
int orc_write_mesh_res(const char *path, int format, const int *ix, const int *ie,
                       const double *x, const double *u, const double *tx, int nnode,
                       int numel, int nen, int ndm, int ndf, int ntn) {
  int nnoel = 0, ctype = -1;
  for (int el = 0; el < numel; el++) {
    int nn, ct = vtk_cell(ie[ix[(size_t)el * (nen + 1) + nen] - 1], &nn);
    if (ct < 0 || (ctype >= 0 && ct != ctype)) return ORC_ERR_ARG;
    ctype = ct;
    nnoel = nn;
  }
  FILE *f = fopen(path, "wb");
  if (!f) return ORC_ERR_ARG;
  char fld[32];
  if (format == 0) {
    fputs("<?xml version=\"1.0\"?>\n", f);
    fputs("<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"BigEndian\">\n", f);
    fputs("<UnstructuredGrid>\n", f);
    fprintf(f, "<Piece NumberOfPoints=\"%15d\" NumberOfCells=\"%15d\">\n", nnode, numel);
    fputs("<Points>\n", f);
    fputs("<DataArray type=\"Float64\" NumberOfComponents =\"3\" format=\"ascii\">\n", f);
    for (int i = 0; i < nnode; i++) {
      for (int j = 0; j < 3; j++) {
        orc_fmt_e(fld, j < ndm ? x[(size_t)i * ndm + j] : 0.0, 15, 5, 0);
        fwrite(fld, 1, 15, f);
      }
      fputc('\n', f);
    }
    fputs("</DataArray>\n</Points>\n", f);
    fputs("<Cells> \n", f);
    fputs("<DataArray type=\"Int32\" Name=\"connectivity\" format=\"ascii\">\n", f);
    for (int el = 0; el < numel; el++) {
      for (int a = 0; a < nnoel; a++) {
        orc_fmt_i(fld, ix[(size_t)el * (nen + 1) + a] - 1, 10);
        fwrite(fld, 1, 10, f);
      }
      fputc('\n', f);
    }
    fputs("</DataArray>\n", f);
    fputs("<DataArray type=\"Int64\" Name=\"offsets\" format=\"ascii\">\n", f);
    for (long long el = 1; el <= numel; el++) {
      orc_fmt_i(fld, el * nnoel, 20);
      fwrite(fld, 1, 20, f);
      fputc('\n', f);
    }
    fputs("</DataArray>\n", f);
    fputs("<DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n", f);
    for (int el = 0; el < numel; el++) {
      orc_fmt_i(fld, ctype, 3);
      fwrite(fld, 1, 3, f);
      fputc('\n', f);
    }
    fputs("</DataArray>\n</Cells>\n", f);
    fputs("<CellData Scalars=\"scalars\">\n", f);
    for (int pass = 0; pass < 2; pass++) {
      fprintf(f, "<DataArray type=\"Int32\" NumberOfComponents=\"1\" Name=\"%s\" format=\"ascii\">\n",
              pass == 0 ? "mat" : "elIdG");
      for (int el = 0; el < numel; el++) {
        orc_fmt_i(fld, pass == 0 ? ix[(size_t)el * (nen + 1) + nen] : el + 1, 9);
        fwrite(fld, 1, 9, f);
        fputc('\n', f);
      }
      fputs("</DataArray>\n", f);
    }
    fputs("</CellData>\n", f);
    fputs("<PointData>\n", f);
    fputs("<DataArray type=\"Int32\" NumberOfComponents=\" 1\" Name=\"noIdG\" format=\"ascii\">\n", f);
    for (int i = 0; i < nnode; i++) {
      orc_fmt_i(fld, i + 1, 10);
      fwrite(fld, 1, 10, f);
      fputc('\n', f);
    }
    fputs("</DataArray>\n", f);
    if (u) {
      fprintf(f, "<DataArray type=\"Float64\" NumberOfComponents=\"%2d\" Name=\"desloc\" format=\"ascii\">\n",
              ndf);
      for (int i = 0; i < nnode; i++) {
        for (int j = 0; j < ndf; j++) {
          orc_fmt_e(fld, u[(size_t)i * ndf + j], 15, 5, 3);
          fwrite(fld, 1, 15, f);
        }
        fputc('\n', f);
      }
      fputs("</DataArray>\n", f);
    }
    if (tx) {
      fputs("<DataArray type=\"Float64\" NumberOfComponents=\"9\" Name=\"stress\" format=\"ascii\">\n", f);
      for (int i = 0; i < nnode; i++) {
        double t9[9];
        full_tensor(tx, ntn, i, t9);
        for (int j = 0; j < 9; j++) {
          orc_fmt_e(fld, t9[j], 15, 5, 3);
          fwrite(fld, 1, 15, f);
        }
        fputc('\n', f);
      }
      fputs("</DataArray>\n", f);
    }
    fputs("</PointData>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n", f);
  } else {
    fputs("# vtk DataFile Version 3.0\n", f);
    fprintf(f, "%-30s", "Malha Res");
    fputs("\nBINARY\n", f);
    fputs("DATASET UNSTRUCTURED_GRID\n", f);
    fprintf(f, "POINTS %15d double\n", nnode);
    for (int i = 0; i < nnode; i++)
      for (int j = 0; j < 3; j++) put_be_f64(f, j < ndm ? x[(size_t)i * ndm + j] : 0.0);
    fprintf(f, "\nCELLS %15d%15d\n", numel, (nnoel + 1) * numel);
    for (int el = 0; el < numel; el++) {
      put_be_i32(f, nnoel);
      for (int a = 0; a < nnoel; a++) put_be_i32(f, ix[(size_t)el * (nen + 1) + a] - 1);
    }
    fprintf(f, "\nCELL_TYPES %15d\n", numel);
    for (int el = 0; el < numel; el++) put_be_i32(f, ctype);
    fprintf(f, "\nCELL_DATA %8d\n", numel);
    for (int pass = 0; pass < 2; pass++) {
      fprintf(f, "SCALARS %-15s int%8d\n", pass == 0 ? "mat" : "elIdG", 1);
      fputs("LOOKUP_TABLE default\n", f);
      for (int el = 0; el < numel; el++)
        put_be_i32(f, pass == 0 ? ix[(size_t)el * (nen + 1) + nen] : el + 1);
    }
    fprintf(f, "\n POINT_DATA %8d\n", nnode);
    fprintf(f, " SCALARS %-15s int %6d\n", "noIdG", 1);
    fputs(" LOOKUP_TABLE default \n", f);
    for (int i = 0; i < nnode; i++) put_be_i32(f, i + 1);
    if (u) {
      fprintf(f, " VECTORS %-15s double\n", "desloc");
      for (int i = 0; i < nnode; i++)
        for (int j = 0; j < 3; j++) put_be_f64(f, j < ndm ? u[(size_t)i * ndf + j] : 0.0);
    }
    if (tx) {
      fprintf(f, " TENSORS %-15s double\n", "stress");
      for (int i = 0; i < nnode; i++) {
        double t9[9];
        full_tensor(tx, ntn, i, t9);
        for (int j = 0; j < 9; j++) put_be_f64(f, t9[j]);
      }
    }
  }
  fclose(f);
  return ORC_OK;
}

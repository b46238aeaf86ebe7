/* CPU oracle for the libEMMI_MGFD hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates, in plain C with complex double arithmetic, the algorithm of the
 * reference's src/gmg.c (multigrid curl-curl solve), src/inject_extract.c
 * and src/find_index.c (injection/extraction) and src/build_gradient.c.
 * Every function cites the reference lines it follows.  It is the checker
 * for the CUDA path and the CPU baseline of the benchmark; it is never part
 * of the product path.  Pinned against the reference: see emmi_oracle.h.
 *
 * Structure (ours, not the reference's): every stencil operation is driven by
 * one generic edge-equation evaluator (edge_row) written for a component c
 * and its cyclic partners p=(c+1)%3, q=(c+2)%3.  The residual, the line block
 * relaxation and the node-patch block relaxation all assemble from it.
 */
#include "emmi_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef double complex zc;

#define EO_PI 3.14159265358979323846264
#define EO_MU0 (4. * EO_PI * 1e-7) /* include/cstd.h:38-40 */

/* ------------------------------------------------------------------------ */
/* level state                                                               */
/* ------------------------------------------------------------------------ */
typedef struct {
  int n[3];
  double *x[3], *xs[3], *d[3], *ds[3]; /* n+1 each (gmg.c:26-29)          */
  double *sig[3], *imu;                /* volume weighted, cells          */
  zc *u, *f, *r;                       /* 3 components of slots           */
  int sc[3];
  int own_cells;                       /* sig/imu allocated here          */
} lev_t;

static inline long nslots(const int n[3]) {
  return (long)(n[0] + 1) * (n[1] + 1) * (n[2] + 1);
}
static inline long slot_of(const int n[3], const int P[3]) {
  return P[0] + (long)(n[0] + 1) * (P[1] + (long)(n[1] + 1) * P[2]);
}
static inline long cell_of(const int n[3], const int P[3]) {
  return P[0] + (long)n[0] * (P[1] + (long)n[1] * P[2]);
}

/* x -> xs, d, ds: gmg.c:1672-1685 (and regrid_init_free.c:21-34) */
static void stagger(int n, const double *x, double *xs, double *d, double *ds) {
  for (int i = 0; i < n; i++) {
    ds[i] = x[i + 1] - x[i];
    xs[i] = 0.5 * (x[i] + x[i + 1]);
  }
  xs[n] = x[n] + 0.5 * ds[n - 1];
  ds[n] = xs[n] - x[n];
  for (int i = 1; i <= n; i++) d[i] = xs[i] - xs[i - 1];
  d[0] = xs[0] - x[0];
}

/* Is edge (c, P) an unknown?  E_c lives at c-index [0,n_c-1] and interior
 * transverse node indices (tangential E = 0 on the boundary, gmg.c:1365). */
static inline int is_unknown(const int n[3], int c, const int P[3]) {
  int p = (c + 1) % 3, q = (c + 2) % 3;
  return P[c] >= 0 && P[c] < n[c] && P[p] >= 1 && P[p] < n[p] && P[q] >= 1 &&
         P[q] < n[q];
}

/* ------------------------------------------------------------------------ */
/* generic edge equation                                                     */
/* ------------------------------------------------------------------------ */
typedef struct {
  int comp;
  int P[3];
  double coef;
} nbr_t;

/* Row of the discrete operator for the unknown E_c at P.  Follows the
 * finite-integration stencil of gmg.c:1365-1404 (and the matrix rows of
 * gmg.c:199-318): with p=(c+1)%3, q=(c+2)%3 and a,b,g the c-,p-,q-indices,
 *   (A E)_c = (m1 T1/ds_p[b] - m2 T2/ds_p[b-1]) - (m3 T3/ds_q[g] - m4 T4/ds_q[g-1])
 *             - i w mu0 sbar_c E_c
 * where T1,T2 are the H_q face curls at p=b, b-1 and T3,T4 the H_p face curls
 * at q=g, g-1; m1..m4 average the volume-weighted inverse permeability over
 * the two cells sharing each face; sbar_c is the 4-cell average of sigma_c.
 * Expanded into coefficients: one complex diagonal and 12 real neighbours. */
static void edge_row(const lev_t *L, zc iwmu, int c, const int P[3],
                     zc *diag, nbr_t nb[12]) {
  const int p = (c + 1) % 3, q = (c + 2) % 3;
  const int a = P[c], b = P[p], g = P[q];
  const int *n = L->n;
  int C[3];
  /* cells sharing the edge: (p,q) in {b-1,b} x {g-1,g}, c-index a */
  double s = 0, m1, m2, m3, m4;
  double im[2][2]; /* im[dp][dq] = imu at p=b-1+dp, q=g-1+dq */
  for (int dp = 0; dp < 2; dp++)
    for (int dq = 0; dq < 2; dq++) {
      C[c] = a;
      C[p] = b - 1 + dp;
      C[q] = g - 1 + dq;
      long id = cell_of(n, C);
      s += L->sig[c][id];
      im[dp][dq] = L->imu[id];
    }
  s *= 0.25;
  m1 = 0.5 * (im[1][1] + im[1][0]); /* H_q face at p=b   */
  m2 = 0.5 * (im[0][1] + im[0][0]); /* H_q face at p=b-1 */
  m3 = 0.5 * (im[1][1] + im[0][1]); /* H_p face at q=g   */
  m4 = 0.5 * (im[1][0] + im[0][0]); /* H_p face at q=g-1 */
  const double dc = L->ds[c][a];
  const double dpp = L->ds[p][b], dpm = L->ds[p][b - 1];
  const double dqp = L->ds[q][g], dqm = L->ds[q][g - 1];

  *diag = (m1 / (dpp * dpp) + m2 / (dpm * dpm)) + (m3 / (dqp * dqp) + m4 / (dqm * dqm)) -
          iwmu * s;
  int k = 0;
#define NB(cc, oc, op, oq, val)                                                \
  do {                                                                         \
    nb[k].comp = (cc);                                                         \
    nb[k].P[0] = P[0]; nb[k].P[1] = P[1]; nb[k].P[2] = P[2];                   \
    nb[k].P[c] += (oc); nb[k].P[p] += (op); nb[k].P[q] += (oq);                \
    nb[k].coef = (val);                                                        \
    k++;                                                                       \
  } while (0)
  NB(c, 0, +1, 0, -m1 / (dpp * dpp));
  NB(c, 0, -1, 0, -m2 / (dpm * dpm));
  NB(c, 0, 0, +1, -m3 / (dqp * dqp));
  NB(c, 0, 0, -1, -m4 / (dqm * dqm));
  NB(p, +1, 0, 0, m1 / (dc * dpp));
  NB(p, 0, 0, 0, -m1 / (dc * dpp));
  NB(p, +1, -1, 0, -m2 / (dc * dpm));
  NB(p, 0, -1, 0, m2 / (dc * dpm));
  NB(q, +1, 0, 0, m3 / (dc * dqp));
  NB(q, 0, 0, 0, -m3 / (dc * dqp));
  NB(q, +1, 0, -1, -m4 / (dc * dqm));
  NB(q, 0, 0, -1, m4 / (dc * dqm));
#undef NB
}

static inline zc field_at(const lev_t *L, const zc *u, int comp, const int P[3]) {
  return u[comp * nslots(L->n) + slot_of(L->n, P)];
}

/* ------------------------------------------------------------------------ */
/* residual: gmg.c:1316-1410                                                 */
/* ------------------------------------------------------------------------ */
static void residual_lev(const lev_t *L, zc iwmu, const zc *u, const zc *f,
                         zc *r) {
  const long S = nslots(L->n);
  memcpy(r, f, 3 * S * sizeof(zc));
  nbr_t nb[12];
  zc dg;
  int P[3];
  for (int c = 0; c < 3; c++)
    for (P[2] = 0; P[2] <= L->n[2]; P[2]++)
      for (P[1] = 0; P[1] <= L->n[1]; P[1]++)
        for (P[0] = 0; P[0] <= L->n[0]; P[0]++) {
          if (!is_unknown(L->n, c, P)) continue;
          edge_row(L, iwmu, c, P, &dg, nb);
          zc au = dg * field_at(L, u, c, P);
          for (int t = 0; t < 12; t++)
            au += nb[t].coef * field_at(L, u, nb[t].comp, nb[t].P);
          r[c * S + slot_of(L->n, P)] -= au;
        }
}

/* ------------------------------------------------------------------------ */
/* banded / dense direct solvers (no pivoting, as gmg.c:39-112)             */
/* ------------------------------------------------------------------------ */
/* band row-major: A[i*11 + 5 + off], off in [-5,5]; solved in place into b */
static void band_solve(zc *A, zc *b, int m) {
  for (int k = 0; k < m - 1; k++) {
    const zc piv = A[k * 11 + 5];
    const int last = (k + 5 < m - 1) ? k + 5 : m - 1;
    for (int i = k + 1; i <= last; i++) {
      zc *ri = A + i * 11 + 5 - i; /* ri[col] = A(i,col) */
      const zc *rk = A + k * 11 + 5 - k;
      zc l = ri[k] / piv;
      ri[k] = l;
      for (int j = k + 1; j <= last; j++) ri[j] -= l * rk[j];
    }
  }
  for (int i = 0; i < m; i++) {
    const zc *ri = A + i * 11 + 5 - i;
    zc s = 0;
    for (int j = (i - 5 > 0 ? i - 5 : 0); j < i; j++) s += ri[j] * b[j];
    b[i] -= s;
  }
  for (int i = m - 1; i >= 0; i--) {
    const zc *ri = A + i * 11 + 5 - i;
    zc s = 0;
    for (int j = i + 1; j < (i + 6 < m ? i + 6 : m); j++) s += ri[j] * b[j];
    b[i] = (b[i] - s) / ri[i];
  }
}

static void dense_solve(zc *A, zc *b, int n) {
  for (int k = 0; k < n - 1; k++) {
    for (int i = k + 1; i < n; i++) A[i * n + k] /= A[k * n + k];
    for (int i = k + 1; i < n; i++)
      for (int j = k + 1; j < n; j++) A[i * n + j] -= A[i * n + k] * A[k * n + j];
  }
  for (int i = 0; i < n; i++) {
    zc s = 0;
    for (int j = 0; j < i; j++) s += A[i * n + j] * b[j];
    b[i] -= s;
  }
  for (int i = n - 1; i >= 0; i--) {
    zc s = 0;
    for (int j = i + 1; j < n; j++) s += A[i * n + j] * b[j];
    b[i] = (b[i] - s) / A[i * n + i];
  }
}

/* ------------------------------------------------------------------------ */
/* line block relaxation: gmg.c:340-1298                                     */
/* ------------------------------------------------------------------------ */
/* Unknowns of the line along d through transverse nodes (ta,tb), a<b the
 * other directions, in the reference's row order: at node s = 1..n_d-1
 *   5(s-1)+0: E_d(s-1)   +1: E_a(ta-1)  +2: E_a(ta)  +3: E_b(tb-1)  +4: E_b(tb)
 * plus E_d(n_d-1) last, m = 5 n_d - 4 rows.  Returns -1 if not on the line. */
static inline int line_pos(int d, int a, int b, int ta, int tb, const int n[3],
                           int comp, const int P[3]) {
  if (comp == d) {
    if (P[a] == ta && P[b] == tb && P[d] >= 0 && P[d] < n[d]) return 5 * P[d];
    return -1;
  }
  if (P[d] < 1 || P[d] >= n[d]) return -1;
  if (comp == a) {
    if (P[b] == tb && (P[a] == ta - 1 || P[a] == ta))
      return 5 * (P[d] - 1) + 1 + (P[a] - ta + 1);
    return -1;
  }
  if (P[a] == ta && (P[b] == tb - 1 || P[b] == tb))
    return 5 * (P[d] - 1) + 3 + (P[b] - tb + 1);
  return -1;
}

static void line_unknown(int d, int a, int b, int ta, int tb, int pos,
                         int *comp, int P[3]) {
  int s = pos / 5, o = pos % 5;
  if (o == 0) {
    *comp = d; P[d] = s; P[a] = ta; P[b] = tb;
  } else if (o <= 2) {
    *comp = a; P[d] = s + 1; P[a] = ta - 2 + o; P[b] = tb;
  } else {
    *comp = b; P[d] = s + 1; P[a] = ta; P[b] = tb - 4 + o;
  }
}

static void solve_line(const lev_t *L, zc iwmu, int d, int ta, int tb, zc *u,
                       const zc *f, zc *A, zc *rhs) {
  const int a = (d == 0) ? 1 : 0, b = (d == 2) ? 1 : 2;
  const int m = 5 * L->n[d] - 4;
  const long S = nslots(L->n);
  nbr_t nb[12];
  zc dg;
  int comp, P[3];
  memset(A, 0, (size_t)m * 11 * sizeof(zc));
  for (int row = 0; row < m; row++) {
    line_unknown(d, a, b, ta, tb, row, &comp, P);
    edge_row(L, iwmu, comp, P, &dg, nb);
    zc acc = f[comp * S + slot_of(L->n, P)];
    A[row * 11 + 5] = dg;
    for (int t = 0; t < 12; t++) {
      int pos = line_pos(d, a, b, ta, tb, L->n, nb[t].comp, nb[t].P);
      if (pos >= 0)
        A[row * 11 + 5 + (pos - row)] += nb[t].coef;
      else
        acc -= nb[t].coef * field_at(L, u, nb[t].comp, nb[t].P);
    }
    rhs[row] = acc;
  }
  band_solve(A, rhs, m);
  for (int row = 0; row < m; row++) {
    line_unknown(d, a, b, ta, tb, row, &comp, P);
    u[comp * S + slot_of(L->n, P)] = rhs[row];
  }
}

static void line_sweep_lev(const lev_t *L, zc iwmu, int d, int ordering,
                           int iter, zc *u, const zc *f) {
  const int a = (d == 0) ? 1 : 0, b = (d == 2) ? 1 : 2;
  const int na = L->n[a], nbb = L->n[b];
  const int m = 5 * L->n[d] - 4;
  zc *A = malloc((size_t)m * 11 * sizeof(zc));
  zc *rhs = malloc((size_t)m * sizeof(zc));
  const int rev = iter % 2 == 1;
  if (ordering == EO_ORDER_LEX) {
    /* outer loop over the higher transverse direction, gmg.c:380-391 */
    for (int ib = 0; ib < nbb - 1; ib++) {
      int tb = rev ? nbb - 1 - ib : 1 + ib;
      for (int ia = 0; ia < na - 1; ia++) {
        int ta = rev ? na - 1 - ia : 1 + ia;
        solve_line(L, iwmu, d, ta, tb, u, f, A, rhs);
      }
    }
  } else {
    /* four colours by transverse parity; same-colour lines are independent */
    for (int cc = 0; cc < 4; cc++) {
      int col = rev ? 3 - cc : cc;
      int pa = col & 1, pb = col >> 1;
      for (int tb = 1; tb < nbb; tb++) {
        if ((tb & 1) != pb) continue;
        for (int ta = 1; ta < na; ta++) {
          if ((ta & 1) != pa) continue;
          solve_line(L, iwmu, d, ta, tb, u, f, A, rhs);
        }
      }
    }
  }
  free(A);
  free(rhs);
}

/* ------------------------------------------------------------------------ */
/* node-patch block relaxation: gmg.c:116-336                                */
/* ------------------------------------------------------------------------ */
static void solve_patch(const lev_t *L, zc iwmu, const int N[3], zc *u,
                        const zc *f) {
  const long S = nslots(L->n);
  zc A[36], rhs[6], dg;
  nbr_t nb[12];
  int P[3];
  for (int row = 0; row < 6; row++) {
    int c = row / 2;
    P[0] = N[0]; P[1] = N[1]; P[2] = N[2];
    P[c] -= 1 - (row & 1);
    edge_row(L, iwmu, c, P, &dg, nb);
    zc acc = f[c * S + slot_of(L->n, P)];
    for (int j = 0; j < 6; j++) A[row * 6 + j] = 0;
    A[row * 6 + row] = dg;
    for (int t = 0; t < 12; t++) {
      int cn = nb[t].comp;
      int off = nb[t].P[cn] - N[cn];
      int in = (off == -1 || off == 0);
      for (int e = 0; e < 3 && in; e++)
        if (e != cn && nb[t].P[e] != N[e]) in = 0;
      if (in)
        A[row * 6 + 2 * cn + (off + 1)] += nb[t].coef;
      else
        acc -= nb[t].coef * field_at(L, u, cn, nb[t].P);
    }
    rhs[row] = acc;
  }
  dense_solve(A, rhs, 6);
  for (int row = 0; row < 6; row++) {
    int c = row / 2;
    P[0] = N[0]; P[1] = N[1]; P[2] = N[2];
    P[c] -= 1 - (row & 1);
    u[c * S + slot_of(L->n, P)] = rhs[row];
  }
}

static void point_sweep_lev(const lev_t *L, zc iwmu, int ordering, int iter,
                            zc *u, const zc *f) {
  const int rev = iter % 2 == 1;
  int N[3];
  if (ordering == EO_ORDER_LEX) {
    for (int kk = 0; kk < L->n[2] - 1; kk++) {
      N[2] = rev ? L->n[2] - 1 - kk : 1 + kk;
      for (int jj = 0; jj < L->n[1] - 1; jj++) {
        N[1] = rev ? L->n[1] - 1 - jj : 1 + jj;
        for (int ii = 0; ii < L->n[0] - 1; ii++) {
          N[0] = rev ? L->n[0] - 1 - ii : 1 + ii;
          solve_patch(L, iwmu, N, u, f);
        }
      }
    }
  } else {
    for (int cc = 0; cc < 8; cc++) {
      int col = rev ? 7 - cc : cc;
      for (N[2] = 1; N[2] < L->n[2]; N[2]++) {
        if ((N[2] & 1) != ((col >> 2) & 1)) continue;
        for (N[1] = 1; N[1] < L->n[1]; N[1]++) {
          if ((N[1] & 1) != ((col >> 1) & 1)) continue;
          for (N[0] = 1; N[0] < L->n[0]; N[0]++) {
            if ((N[0] & 1) != (col & 1)) continue;
            solve_patch(L, iwmu, N, u, f);
          }
        }
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* transfers: gmg.c:1463-1573                                                */
/* ------------------------------------------------------------------------ */
/* weight of the upper coarse node for fine node index ii along direction */
static inline double wright(const double *xf, const double *xc, int ii, int ic) {
  return (xf[ii] - xc[ic]) / (xc[ic + 1] - xc[ic]);
}

static void restrict_op(const int nf[3], const double *const xf[3],
                        const int nc[3], const double *const xc[3],
                        const int sc[3], const zc *rf, zc *fc) {
  const long Sf = nslots(nf), Sc = nslots(nc);
  memset(fc, 0, 3 * Sc * sizeof(zc));
  int F[3], Cn[3];
  double wr[3], wl[3];
  for (F[2] = 0; F[2] < nf[2]; F[2]++)
    for (F[1] = 0; F[1] < nf[1]; F[1]++)
      for (F[0] = 0; F[0] < nf[0]; F[0]++) {
        for (int e = 0; e < 3; e++) {
          Cn[e] = sc[e] == 2 ? F[e] / 2 : F[e];
          wr[e] = wright(xf[e], xc[e], F[e], Cn[e]);
          wl[e] = 1. - wr[e];
        }
        for (int c = 0; c < 3; c++) {
          int p = (c + 1) % 3, q = (c + 2) % 3;
          /* the two transverse directions in increasing order */
          int t1 = p < q ? p : q, t2 = p < q ? q : p;
          if (F[t1] == 0 || F[t2] == 0) continue;
          zc v = rf[c * Sf + slot_of(nf, F)];
          for (int o2 = 0; o2 < 2; o2++)
            for (int o1 = 0; o1 < 2; o1++) {
              int C[3] = {Cn[0], Cn[1], Cn[2]};
              C[t1] += o1;
              C[t2] += o2;
              double w = (o1 ? wr[t1] : wl[t1]) * (o2 ? wr[t2] : wl[t2]);
              fc[c * Sc + slot_of(nc, C)] += w * v;
            }
        }
      }
}

static void prolong_op(const int nf[3], const double *const xf[3],
                       const int nc[3], const double *const xc[3],
                       const int sc[3], const zc *uc, zc *uf) {
  const long Sf = nslots(nf), Sc = nslots(nc);
  int F[3], Cn[3];
  double wr[3], wl[3];
  for (F[2] = 0; F[2] < nf[2]; F[2]++)
    for (F[1] = 0; F[1] < nf[1]; F[1]++)
      for (F[0] = 0; F[0] < nf[0]; F[0]++) {
        for (int e = 0; e < 3; e++) {
          Cn[e] = sc[e] == 2 ? F[e] / 2 : F[e];
          wr[e] = wright(xf[e], xc[e], F[e], Cn[e]);
          wl[e] = 1. - wr[e];
        }
        for (int c = 0; c < 3; c++) {
          int p = (c + 1) % 3, q = (c + 2) % 3;
          int t1 = p < q ? p : q, t2 = p < q ? q : p;
          if (F[t1] == 0 || F[t2] == 0) continue;
          /* bilinear in (t1,t2), evaluated as wl2*(wl1 u00 + wr1 u10) + ...
           * in the reference's grouping (outer weight on the lower
           * transverse direction, gmg.c:1496-1500) */
          int C[3] = {Cn[0], Cn[1], Cn[2]};
          zc u00 = uc[c * Sc + slot_of(nc, C)];
          C[t2] += 1;
          zc u01 = uc[c * Sc + slot_of(nc, C)];
          C[t2] -= 1; C[t1] += 1;
          zc u10 = uc[c * Sc + slot_of(nc, C)];
          C[t2] += 1;
          zc u11 = uc[c * Sc + slot_of(nc, C)];
          uf[c * Sf + slot_of(nf, F)] +=
              wl[t1] * (wl[t2] * u00 + wr[t2] * u01) +
              wr[t1] * (wl[t2] * u10 + wr[t2] * u11);
        }
      }
}

/* gmg.c:1803-1858 */
static void coarsen_cells(const int nf[3], const int sc[3], const double *cf,
                          int nc0, int nc1, int nc2, double *cc) {
  const int repeat = 8 / (sc[0] * sc[1] * sc[2]);
  for (int k = 0; k < nc2; k++) {
    int k0 = sc[2] == 2 ? 2 * k : k, k1 = sc[2] == 2 ? 2 * k + 1 : k;
    for (int j = 0; j < nc1; j++) {
      int j0 = sc[1] == 2 ? 2 * j : j, j1 = sc[1] == 2 ? 2 * j + 1 : j;
      for (int i = 0; i < nc0; i++) {
        int i0 = sc[0] == 2 ? 2 * i : i, i1 = sc[0] == 2 ? 2 * i + 1 : i;
#define CF(ii, jj, kk) cf[(ii) + (long)nf[0] * ((jj) + (long)nf[1] * (kk))]
        double v = CF(i0, j0, k0) + CF(i1, j0, k0) + CF(i0, j1, k0) +
                   CF(i1, j1, k0) + CF(i0, j0, k1) + CF(i1, j0, k1) +
                   CF(i0, j1, k1) + CF(i1, j1, k1);
#undef CF
        cc[i + (long)nc0 * (j + (long)nc1 * k)] = v / repeat;
      }
    }
  }
}

/* H = curl E / (i w mu0): gmg.c:1414-1460 */
static void curl_h_lev(const lev_t *L, zc iwmu, const zc *u, zc *h) {
  const int *n = L->n;
  const long S = nslots(n);
  memset(h, 0, 3 * S * sizeof(zc));
#define U(c, i, j, k) u[(c) * S + (i) + (long)(n[0] + 1) * ((j) + (long)(n[1] + 1) * (k))]
  for (int k = 0; k < n[2]; k++)
    for (int j = 0; j < n[1]; j++)
      for (int i = 0; i < n[0]; i++) {
        long s = i + (long)(n[0] + 1) * (j + (long)(n[1] + 1) * k);
        zc t1 = (U(2, i, j + 1, k) - U(2, i, j, k)) / L->ds[1][j] -
                (U(1, i, j, k + 1) - U(1, i, j, k)) / L->ds[2][k];
        zc t2 = (U(0, i, j, k + 1) - U(0, i, j, k)) / L->ds[2][k] -
                (U(2, i + 1, j, k) - U(2, i, j, k)) / L->ds[0][i];
        zc t3 = (U(1, i + 1, j, k) - U(1, i, j, k)) / L->ds[0][i] -
                (U(0, i, j + 1, k) - U(0, i, j, k)) / L->ds[1][j];
        h[s] = t1 / iwmu;
        h[S + s] = t2 / iwmu;
        h[2 * S + s] = t3 / iwmu;
      }
#undef U
}

/* ------------------------------------------------------------------------ */
/* multigrid hierarchy and cycles: gmg.c:1586-1932                          */
/* ------------------------------------------------------------------------ */
typedef struct {
  int lmax;
  lev_t *lev; /* lmax levels; lev[0] persistent, coarse levels per hierarchy */
  lev_t *hier[3]; /* coarse levels for icycle%3 = 0,1,2 (lazily built) */
  zc iwmu;
  eo_params prm;
  int icycle;
  double rnorm0, rnorm;
  int stop;
  double *hist;
} mg_t;

/* gmg.c:1688-1699 */
static int depth_of(int n) {
  int l = 0, nn = n;
  while (nn % 2 == 0 && nn > 1) {
    l++;
    nn >>= 1;
  }
  if (nn > 2) l++;
  return l;
}

static void lev_alloc_fields(lev_t *L) {
  long S = nslots(L->n);
  L->u = calloc(3 * S, sizeof(zc));
  L->f = calloc(3 * S, sizeof(zc));
  L->r = calloc(3 * S, sizeof(zc));
}

static void lev_alloc_grid(lev_t *L) {
  for (int e = 0; e < 3; e++) {
    L->x[e] = calloc(L->n[e] + 1, sizeof(double));
    L->xs[e] = calloc(L->n[e] + 1, sizeof(double));
    L->d[e] = calloc(L->n[e] + 1, sizeof(double));
    L->ds[e] = calloc(L->n[e] + 1, sizeof(double));
  }
}

static void lev_free(lev_t *L) {
  for (int e = 0; e < 3; e++) {
    free(L->x[e]); free(L->xs[e]); free(L->d[e]); free(L->ds[e]);
  }
  if (L->own_cells) {
    for (int e = 0; e < 3; e++) free(L->sig[e]);
    free(L->imu);
  }
  free(L->u); free(L->f); free(L->r);
}

/* coarse levels of hierarchy h (= icycle%3), grid_init gmg.c:1751-1858 */
static lev_t *build_hierarchy(const mg_t *M, int h) {
  lev_t *H = calloc(M->lmax, sizeof(lev_t));
  H[0] = M->lev[0];
  for (int l = 1; l < M->lmax; l++) {
    const lev_t *F = &H[l - 1];
    lev_t *C = &H[l];
    for (int e = 0; e < 3; e++)
      C->sc[e] = (F->n[e] % 2 == 0 && F->n[e] > 2) ? 2 : 1;
    if (M->prm.isemicoarsen) C->sc[h] = 1;
    for (int e = 0; e < 3; e++) C->n[e] = F->n[e] / C->sc[e];
    lev_alloc_grid(C);
    for (int e = 0; e < 3; e++) {
      for (int i = 0; i <= C->n[e]; i++) C->x[e][i] = F->x[e][C->sc[e] * i];
      stagger(C->n[e], C->x[e], C->xs[e], C->d[e], C->ds[e]);
    }
    long nc = (long)C->n[0] * C->n[1] * C->n[2];
    for (int e = 0; e < 3; e++) {
      C->sig[e] = malloc(nc * sizeof(double));
      coarsen_cells(F->n, C->sc, F->sig[e], C->n[0], C->n[1], C->n[2], C->sig[e]);
    }
    C->imu = malloc(nc * sizeof(double));
    coarsen_cells(F->n, C->sc, F->imu, C->n[0], C->n[1], C->n[2], C->imu);
    C->own_cells = 1;
    lev_alloc_fields(C);
  }
  return H;
}

static void smooth(mg_t *M, lev_t *H, int l, int iter) {
  lev_t *L = &H[l];
  if (M->prm.isemicoarsen && l < M->lmax - 1) {
    for (int d = 0; d < 3; d++)
      if (H[l + 1].sc[d] == 2)
        line_sweep_lev(L, M->iwmu, d, M->prm.ordering, iter, L->u, L->f);
  } else {
    point_sweep_lev(L, M->iwmu, M->prm.ordering, iter, L->u, L->f);
  }
}

static double norm_of(const lev_t *L, const zc *r) {
  long n3 = 3 * nslots(L->n);
  double s = 0;
  for (long i = 0; i < n3; i++) s += creal(conj(r[i]) * r[i]);
  return sqrt(s);
}

/* level-0 norm test shared by the three cycle types (gmg.c:1593-1600,
 * 1624-1631, 1650-1657).  Returns 1 if the solve has converged. */
static int norm_test(mg_t *M, lev_t *L) {
  M->rnorm = norm_of(L, L->r);
  if (M->prm.verb) printf("icycle=%d rnorm=%e\n", M->icycle, M->rnorm);
  if (M->hist) M->hist[M->icycle] = M->rnorm;
  if (M->icycle == 0)
    M->rnorm0 = M->rnorm;
  else if (M->rnorm < M->rnorm0 * M->prm.tol) {
    M->stop = 1;
    return 1;
  }
  return 0;
}

static int can_descend(const mg_t *M, const lev_t *H, int l) {
  return l < M->lmax - 1 && H[l + 1].sc[0] * H[l + 1].sc[1] * H[l + 1].sc[2] > 1;
}

static void to_coarse(mg_t *M, lev_t *H, int l) {
  lev_t *F = &H[l], *C = &H[l + 1];
  restrict_op(F->n, (const double *const *)F->x, C->n,
              (const double *const *)C->x, C->sc, F->r, C->f);
  memset(C->u, 0, 3 * nslots(C->n) * sizeof(zc));
  (void)M;
}

static void to_fine(lev_t *H, int l) {
  lev_t *F = &H[l], *C = &H[l + 1];
  prolong_op(F->n, (const double *const *)F->x, C->n,
             (const double *const *)C->x, C->sc, C->u, F->u);
}

/* gmg.c:1586-1612 */
static void v_cycle(mg_t *M, lev_t *H, int l) {
  for (int i = 0; i < M->prm.v1; i++) smooth(M, H, l, i);
  if (can_descend(M, H, l)) {
    residual_lev(&H[l], M->iwmu, H[l].u, H[l].f, H[l].r);
    if (M->prm.cycleopt == 1 && l == 0 && norm_test(M, &H[0])) return;
    to_coarse(M, H, l);
    v_cycle(M, H, l + 1);
    to_fine(H, l);
  }
  for (int i = 0; i < M->prm.v2; i++) smooth(M, H, l, i);
}

/* gmg.c:1615-1640 */
static void f_cycle(mg_t *M, lev_t *H, int l) {
  if (l == M->lmax - 1) {
    memset(H[l].u, 0, 3 * nslots(H[l].n) * sizeof(zc));
  } else if (can_descend(M, H, l)) {
    residual_lev(&H[l], M->iwmu, H[l].u, H[l].f, H[l].r);
    if (M->prm.cycleopt == 2 && l == 0 && norm_test(M, &H[0])) return;
    to_coarse(M, H, l);
    f_cycle(M, H, l + 1);
    to_fine(H, l);
  }
  v_cycle(M, H, l);
}

/* gmg.c:1643-1668 */
static void w_cycle(mg_t *M, lev_t *H, int l) {
  for (int i = 0; i < M->prm.v1; i++) smooth(M, H, l, i);
  if (can_descend(M, H, l)) {
    residual_lev(&H[l], M->iwmu, H[l].u, H[l].f, H[l].r);
    if (M->prm.cycleopt == 3 && l == 0 && norm_test(M, &H[0])) return;
    to_coarse(M, H, l);
    w_cycle(M, H, l + 1);
    w_cycle(M, H, l + 1);
    to_fine(H, l);
  }
  for (int i = 0; i < M->prm.v2; i++) smooth(M, H, l, i);
}

static double wall_seconds(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t.tv_sec + 1e-9 * t.tv_nsec;
}

int eo_gmg_solve(int n1, int n2, int n3, const float *x1, const float *x2,
                 const float *x3, const float *sigma11, const float *sigma22,
                 const float *sigma33, const float *invmur, double omega,
                 const eo_params *prm, double *b, double *x,
                 double *rnorm_hist) {
  return eo_gmg_solve_timed(n1, n2, n3, x1, x2, x3, sigma11, sigma22, sigma33, invmur, omega,
                            prm, b, x, rnorm_hist, NULL);
}

int eo_gmg_solve_timed(int n1, int n2, int n3, const float *x1, const float *x2,
                       const float *x3, const float *sigma11, const float *sigma22,
                       const float *sigma33, const float *invmur, double omega,
                       const eo_params *prm, double *b, double *x,
                       double *rnorm_hist, double *seconds) {
  const double t0 = wall_seconds();
  mg_t M;
  memset(&M, 0, sizeof(M));
  M.prm = *prm;
  M.hist = rnorm_hist;
  /* I*omega*mu0 as the reference forms it (gmg.c:1710) */
  M.iwmu = I * (omega * EO_MU0);
  M.lmax = depth_of(n1);
  if (depth_of(n2) > M.lmax) M.lmax = depth_of(n2);
  if (depth_of(n3) > M.lmax) M.lmax = depth_of(n3);

  lev_t L0;
  memset(&L0, 0, sizeof(L0));
  L0.n[0] = n1; L0.n[1] = n2; L0.n[2] = n3;
  L0.sc[0] = L0.sc[1] = L0.sc[2] = 1;
  lev_alloc_grid(&L0);
  const float *xin[3] = {x1, x2, x3};
  for (int e = 0; e < 3; e++) {
    for (int i = 0; i <= L0.n[e]; i++) L0.x[e][i] = xin[e][i];
    stagger(L0.n[e], L0.x[e], L0.xs[e], L0.d[e], L0.ds[e]);
  }
  long nc = (long)n1 * n2 * n3;
  for (int e = 0; e < 3; e++) L0.sig[e] = malloc(nc * sizeof(double));
  L0.imu = malloc(nc * sizeof(double));
  L0.own_cells = 1;
  const float *sin_[3] = {sigma11, sigma22, sigma33};
  for (int k = 0; k < n3; k++)
    for (int j = 0; j < n2; j++)
      for (int i = 0; i < n1; i++) {
        long id = i + (long)n1 * (j + (long)n2 * k);
        double vol = L0.ds[0][i] * L0.ds[1][j] * L0.ds[2][k]; /* gmg.c:1795 */
        for (int e = 0; e < 3; e++) L0.sig[e][id] = sin_[e][id] * vol;
        L0.imu[id] = invmur[id] * vol;
      }
  lev_alloc_fields(&L0);
  const long S = nslots(L0.n);
  zc *bz = (zc *)b;
  memcpy(L0.f, bz, 3 * S * sizeof(zc));
  /* scale by dual volumes, gmg.c:1901-1910 */
  for (int k = 0; k <= n3; k++)
    for (int j = 0; j <= n2; j++)
      for (int i = 0; i <= n1; i++) {
        long s = i + (long)(n1 + 1) * (j + (long)(n2 + 1) * k);
        L0.f[s] *= L0.ds[0][i] * L0.d[1][j] * L0.d[2][k];
        L0.f[S + s] *= L0.d[0][i] * L0.ds[1][j] * L0.d[2][k];
        L0.f[2 * S + s] *= L0.d[0][i] * L0.d[1][j] * L0.ds[2][k];
      }
  M.lev = &L0;

  int ncycles = prm->ncycle;
  const double t1 = wall_seconds();
  for (M.icycle = 0; M.icycle < prm->ncycle; M.icycle++) {
    int h = M.icycle % 3;
    if (!M.hier[h]) M.hier[h] = build_hierarchy(&M, h);
    lev_t *H = M.hier[h];
    H[0] = L0; /* level 0 shared */
    if (prm->cycleopt == 1) v_cycle(&M, H, 0);
    if (prm->cycleopt == 2) f_cycle(&M, H, 0);
    if (prm->cycleopt == 3) w_cycle(&M, H, 0);
    L0 = H[0];
    if (M.stop) {
      ncycles = M.icycle;
      break;
    }
  }
  if (seconds) {
    seconds[0] = t1 - t0;
    seconds[1] = wall_seconds() - t1;
  }
  memcpy(x, L0.u, 3 * S * sizeof(zc));
  curl_h_lev(&L0, M.iwmu, L0.u, bz);

  for (int h = 0; h < 3; h++) {
    if (!M.hier[h]) continue;
    for (int l = 1; l < M.lmax; l++) lev_free(&M.hier[h][l]);
    free(M.hier[h]);
  }
  lev_free(&L0);
  return ncycles;
}

/* ------------------------------------------------------------------------ */
/* single-level wrappers                                                     */
/* ------------------------------------------------------------------------ */
static void wrap_level(const eo_level_desc *D, lev_t *L) {
  memset(L, 0, sizeof(*L));
  for (int e = 0; e < 3; e++) L->n[e] = D->n[e];
  lev_alloc_grid(L);
  for (int e = 0; e < 3; e++) {
    memcpy(L->x[e], D->x[e], (L->n[e] + 1) * sizeof(double));
    stagger(L->n[e], L->x[e], L->xs[e], L->d[e], L->ds[e]);
    L->sig[e] = (double *)D->sig[e];
  }
  L->imu = (double *)D->imu;
  L->own_cells = 0;
}

static zc iwmu_of(double omega) { return I * (omega * EO_MU0); }

void eo_residual(const eo_level_desc *D, const double *u, const double *f,
                 double *r) {
  lev_t L;
  wrap_level(D, &L);
  residual_lev(&L, iwmu_of(D->omega), (const zc *)u, (const zc *)f, (zc *)r);
  lev_free(&L);
}

void eo_apply(const eo_level_desc *D, const double *u, double *au) {
  lev_t L;
  wrap_level(D, &L);
  const long S = nslots(L.n);
  zc *z = calloc(3 * S, sizeof(zc));
  residual_lev(&L, iwmu_of(D->omega), (const zc *)u, z, (zc *)au);
  zc *o = (zc *)au;
  int P[3];
  for (int c = 0; c < 3; c++)
    for (P[2] = 0; P[2] <= L.n[2]; P[2]++)
      for (P[1] = 0; P[1] <= L.n[1]; P[1]++)
        for (P[0] = 0; P[0] <= L.n[0]; P[0]++) {
          long s = c * S + slot_of(L.n, P);
          o[s] = is_unknown(L.n, c, P) ? -o[s] : 0;
        }
  free(z);
  lev_free(&L);
}

void eo_line_sweep(const eo_level_desc *D, int dir, int ordering, int iter,
                   double *u, const double *f) {
  lev_t L;
  wrap_level(D, &L);
  line_sweep_lev(&L, iwmu_of(D->omega), dir, ordering, iter, (zc *)u,
                 (const zc *)f);
  lev_free(&L);
}

void eo_point_sweep(const eo_level_desc *D, int ordering, int iter, double *u,
                    const double *f) {
  lev_t L;
  wrap_level(D, &L);
  point_sweep_lev(&L, iwmu_of(D->omega), ordering, iter, (zc *)u,
                  (const zc *)f);
  lev_free(&L);
}

void eo_restrict(const int nf[3], const double *const xf[3], const int nc[3],
                 const double *const xc[3], const int sc[3], const double *rf,
                 double *fc) {
  restrict_op(nf, xf, nc, xc, sc, (const zc *)rf, (zc *)fc);
}

void eo_prolong(const int nf[3], const double *const xf[3], const int nc[3],
                const double *const xc[3], const int sc[3], const double *uc,
                double *uf) {
  prolong_op(nf, xf, nc, xc, sc, (const zc *)uc, (zc *)uf);
}

void eo_coarsen_cells(const int nf[3], const int sc[3], const double *cf,
                      double *cc) {
  coarsen_cells(nf, sc, cf, nf[0] / sc[0], nf[1] / sc[1], nf[2] / sc[2], cc);
}

void eo_curl_h(const eo_level_desc *D, const double *u, double *h) {
  lev_t L;
  wrap_level(D, &L);
  curl_h_lev(&L, iwmu_of(D->omega), (const zc *)u, (zc *)h);
  lev_free(&L);
}

/* ------------------------------------------------------------------------ */
/* injection / extraction / gradient                                         */
/* ------------------------------------------------------------------------ */
/* find_index.c:9-30: binary search for x[k] <= val < x[k+1] */
int eo_find_index(int n, const float *x, float val) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi) / 2;
    if (x[mid] <= val) lo = mid;
    if (x[mid] > val) hi = mid;
    if (lo == hi || lo == hi - 1) break;
  }
  return lo;
}

/* Rotation of a unit dipole / channel vector into grid axes,
 * inject_extract.c:40-55 (and :139-154, :220-235).  ch: 0/3 -> x', 1/4 -> y',
 * 2/5 -> z'.  Adds amp * direction to F. */
static void rotate_in(int chx, float phi, float theta, zc amp, zc F[3]) {
  if (chx == 0) {
    F[0] += amp * cos(phi);
    F[1] += amp * sin(phi);
  } else if (chx == 1) {
    F[0] -= amp * sin(phi) * cos(theta);
    F[1] += amp * cos(phi) * cos(theta);
    F[2] += amp * sin(theta);
  } else if (chx == 2) {
    F[0] += amp * sin(phi) * sin(theta);
    F[1] -= amp * cos(phi) * sin(theta);
    F[2] += amp * cos(theta);
  }
}

/* Staggered-grid coordinate arrays of a component: E/J component c lives
 * on (xs if axis==c else x); H/M component c on (x if axis==c else xs). */
static const float *axis_grid(const eo_grid *g, int axis, int half) {
  if (axis == 0) return half ? g->x1s : g->x1;
  if (axis == 1) return half ? g->x2s : g->x2;
  return half ? g->x3s : g->x3;
}

typedef struct {
  int i[3];
  float w[3];
  float vol;
} tri_t;

/* Trilinear stencil of a point on the grid of one staggered component,
 * inject_extract.c:57-65 */
static tri_t trilin(const eo_grid *g, const int half[3], float px, float py,
                    float pz) {
  tri_t t;
  const int n[3] = {g->n1, g->n2, g->n3};
  const float pv[3] = {px, py, pz};
  t.vol = 1.f;
  for (int e = 0; e < 3; e++) {
    const float *ax = axis_grid(g, e, half[e]);
    t.i[e] = eo_find_index(n[e] + 1, ax, pv[e]);
    t.w[e] = (pv[e] - ax[t.i[e]]) / (ax[t.i[e] + 1] - ax[t.i[e]]);
  }
  /* vol is a float product in the reference's order (x)(y)(z) */
  const float *a0 = axis_grid(g, 0, half[0]), *a1 = axis_grid(g, 1, half[1]),
              *a2 = axis_grid(g, 2, half[2]);
  t.vol = (a0[t.i[0] + 1] - a0[t.i[0]]) * (a1[t.i[1] + 1] - a1[t.i[1]]) *
          (a2[t.i[2] + 1] - a2[t.i[2]]);
  return t;
}

static inline long gidx(const eo_grid *g, int c, int i, int j, int k) {
  long S = (long)(g->n1 + 1) * (g->n2 + 1) * (g->n3 + 1);
  return c * S + i + (long)(g->n1 + 1) * (j + (long)(g->n2 + 1) * k);
}

/* scatter val with trilinear weights onto component c of y (8 corners, in
 * the reference's corner order, inject_extract.c:68-75) */
static void scatter8(const eo_grid *g, int c, const tri_t *t, zc val, zc *y) {
  const float w1 = t->w[0], w2 = t->w[1], w3 = t->w[2];
  const int i = t->i[0], j = t->i[1], k = t->i[2];
  y[gidx(g, c, i, j, k)] += val * (1. - w1) * (1. - w2) * (1. - w3);
  y[gidx(g, c, i + 1, j, k)] += val * w1 * (1. - w2) * (1. - w3);
  y[gidx(g, c, i, j + 1, k)] += val * (1. - w1) * w2 * (1. - w3);
  y[gidx(g, c, i + 1, j + 1, k)] += val * w1 * w2 * (1. - w3);
  y[gidx(g, c, i, j, k + 1)] += val * (1. - w1) * (1. - w2) * w3;
  y[gidx(g, c, i + 1, j, k + 1)] += val * w1 * (1. - w2) * w3;
  y[gidx(g, c, i, j + 1, k + 1)] += val * (1. - w1) * w2 * w3;
  y[gidx(g, c, i + 1, j + 1, k + 1)] += val * w1 * w2 * w3;
}

void eo_inject_source(const eo_grid *g, int nsrc, const float *sx,
                      const float *sy, const float *sz, const float *azim,
                      const float *dip, int nch, const int *chsrc, float omega,
                      double *bd) {
  zc *b = (zc *)bd;
  long S = (long)(g->n1 + 1) * (g->n2 + 1) * (g->n3 + 1);
  memset(b, 0, 3 * S * sizeof(zc));
  const zc src_fd = 1;
  for (int is = 0; is < nsrc; is++) {
    zc F[3] = {0, 0, 0};
    for (int ic = 0; ic < nch; ic++)
      if (chsrc[ic] <= 2) rotate_in(chsrc[ic], azim[is], dip[is], src_fd, F);
    for (int c = 0; c < 3; c++) {
      int half[3] = {c == 0, c == 1, c == 2};
      tri_t t = trilin(g, half, sx[is], sy[is], sz[is]);
      /* I*omega (complex float) * mu0 * F / vol, inject_extract.c:66 */
      float complex iw = I * omega;
      zc v = (zc)iw * EO_MU0 * F[c] / t.vol;
      scatter8(g, c, &t, v, b);
    }
  }
}

void eo_inject_adj_source(const eo_grid *g, int nrec, const float *rx,
                          const float *ry, const float *rz, const float *azim,
                          const float *dip, int nch, const int *chrec,
                          const float *dres, float omega, double *xd,
                          double *bd) {
  zc *b = (zc *)bd, *x = (zc *)xd;
  long S = (long)(g->n1 + 1) * (g->n2 + 1) * (g->n3 + 1);
  memset(b, 0, 3 * S * sizeof(zc));
  memset(x, 0, 3 * S * sizeof(zc));
  const float complex *dr = (const float complex *)dres;
  for (int ir = 0; ir < nrec; ir++) {
    zc F[3] = {0, 0, 0};
    for (int ic = 0; ic < nch; ic++)
      if (chrec[ic] <= 2)
        rotate_in(chrec[ic], azim[ir], dip[ir], (zc)dr[(long)ic * nrec + ir], F);
    for (int c = 0; c < 3; c++) {
      int half[3] = {c == 0, c == 1, c == 2};
      tri_t t = trilin(g, half, rx[ir], ry[ir], rz[ir]);
      float complex iw = I * omega;
      zc v = (zc)iw * EO_MU0 * F[c] / t.vol;
      scatter8(g, c, &t, v, b);
    }
    /* magnetic channels -> M on the H grids, inject_extract.c:220-301 */
    zc G[3] = {0, 0, 0};
    for (int ic = 0; ic < nch; ic++)
      if (chrec[ic] >= 3)
        rotate_in(chrec[ic] - 3, azim[ir], dip[ir], (zc)dr[(long)ic * nrec + ir], G);
    for (int c = 0; c < 3; c++) {
      int half[3] = {c != 0, c != 1, c != 2};
      tri_t t = trilin(g, half, rx[ir], ry[ir], rz[ir]);
      zc v = G[c] / t.vol;
      scatter8(g, c, &t, v, x);
    }
  }
  /* b += curl M with the node spacings d1,d2,d3, inject_extract.c:303-312 */
  for (int k = 1; k <= g->n3; k++)
    for (int j = 1; j <= g->n2; j++)
      for (int i = 1; i <= g->n1; i++) {
        b[gidx(g, 0, i, j, k)] +=
            (x[gidx(g, 2, i, j, k)] - x[gidx(g, 2, i, j - 1, k)]) / g->d2[j] -
            (x[gidx(g, 1, i, j, k)] - x[gidx(g, 1, i, j, k - 1)]) / g->d3[k];
        b[gidx(g, 1, i, j, k)] +=
            (x[gidx(g, 0, i, j, k)] - x[gidx(g, 0, i, j, k - 1)]) / g->d3[k] -
            (x[gidx(g, 2, i, j, k)] - x[gidx(g, 2, i - 1, j, k)]) / g->d1[i];
        b[gidx(g, 2, i, j, k)] +=
            (x[gidx(g, 1, i, j, k)] - x[gidx(g, 1, i - 1, j, k)]) / g->d1[i] -
            (x[gidx(g, 0, i, j, k)] - x[gidx(g, 0, i, j - 1, k)]) / g->d2[j];
      }
}

/* gather with trilinear weights (inject_extract.c:339-346); if sig != NULL
 * each corner is weighted by the cell value sig at the same (i,j,k) (Jz) */
static zc gather8(const eo_grid *g, int c, const tri_t *t, const zc *y,
                  const float *sig) {
  const float w1 = t->w[0], w2 = t->w[1], w3 = t->w[2];
  const int i = t->i[0], j = t->i[1], k = t->i[2];
  zc F = 0;
#define SG(ii, jj, kk) (sig ? (double)sig[(ii) + (long)g->n1 * ((jj) + (long)g->n2 * (kk))] : 1.0)
#define TERM(ii, jj, kk, w)                                                    \
  do {                                                                         \
    if (sig)                                                                   \
      F += sig[(ii) + (long)g->n1 * ((jj) + (long)g->n2 * (kk))] *            \
           y[gidx(g, c, ii, jj, kk)] * w;                                      \
    else                                                                       \
      F += y[gidx(g, c, ii, jj, kk)] * w;                                      \
  } while (0)
  /* weights grouped left to right as in the reference: v*(a)*(b)*(c) */
  if (sig) {
    F += SG(i, j, k) * y[gidx(g, c, i, j, k)] * (1. - w1) * (1. - w2) * (1. - w3);
    F += SG(i + 1, j, k) * y[gidx(g, c, i + 1, j, k)] * w1 * (1. - w2) * (1. - w3);
    F += SG(i, j + 1, k) * y[gidx(g, c, i, j + 1, k)] * (1. - w1) * w2 * (1. - w3);
    F += SG(i + 1, j + 1, k) * y[gidx(g, c, i + 1, j + 1, k)] * w1 * w2 * (1. - w3);
    F += SG(i, j, k + 1) * y[gidx(g, c, i, j, k + 1)] * (1. - w1) * (1. - w2) * w3;
    F += SG(i + 1, j, k + 1) * y[gidx(g, c, i + 1, j, k + 1)] * w1 * (1. - w2) * w3;
    F += SG(i, j + 1, k + 1) * y[gidx(g, c, i, j + 1, k + 1)] * (1. - w1) * w2 * w3;
    F += SG(i + 1, j + 1, k + 1) * y[gidx(g, c, i + 1, j + 1, k + 1)] * w1 * w2 * w3;
  } else {
    F += y[gidx(g, c, i, j, k)] * (1. - w1) * (1. - w2) * (1. - w3);
    F += y[gidx(g, c, i + 1, j, k)] * w1 * (1. - w2) * (1. - w3);
    F += y[gidx(g, c, i, j + 1, k)] * (1. - w1) * w2 * (1. - w3);
    F += y[gidx(g, c, i + 1, j + 1, k)] * w1 * w2 * (1. - w3);
    F += y[gidx(g, c, i, j, k + 1)] * (1. - w1) * (1. - w2) * w3;
    F += y[gidx(g, c, i + 1, j, k + 1)] * w1 * (1. - w2) * w3;
    F += y[gidx(g, c, i, j + 1, k + 1)] * (1. - w1) * w2 * w3;
    F += y[gidx(g, c, i + 1, j + 1, k + 1)] * w1 * w2 * w3;
  }
#undef TERM
#undef SG
  return F;
}

/* receiver-frame rotation, inject_extract.c:391-399 */
static zc rotate_out(int chx, float phi, float theta, const zc F[3]) {
  if (chx == 0) return cos(phi) * F[0] + sin(phi) * F[1];
  if (chx == 1)
    return -sin(phi) * cos(theta) * F[0] + cos(phi) * cos(theta) * F[1] -
           sin(theta) * F[2];
  return sin(phi) * sin(theta) * F[0] - cos(phi) * sin(theta) * F[1] +
         cos(theta) * F[2];
}

void eo_extract_emf_data(const eo_grid *g, int nrec, const float *rx,
                         const float *ry, const float *rz, const float *azim,
                         const float *dip, int nch, const int *chrec,
                         const double *xd, const double *bd, float *dcal) {
  const zc *x = (const zc *)xd, *b = (const zc *)bd;
  float complex *out = (float complex *)dcal;
  for (int ir = 0; ir < nrec; ir++) {
    zc E[3], H[3];
    for (int c = 0; c < 3; c++) {
      int half[3] = {c == 0, c == 1, c == 2};
      tri_t t = trilin(g, half, rx[ir], ry[ir], rz[ir]);
      E[c] = gather8(g, c, &t, x, c == 2 ? g->sigma33 : NULL);
    }
    E[2] *= g->rho_water; /* Jz -> Ez, inject_extract.c:386 */
    for (int c = 0; c < 3; c++) {
      int half[3] = {c != 0, c != 1, c != 2};
      tri_t t = trilin(g, half, rx[ir], ry[ir], rz[ir]);
      H[c] = gather8(g, c, &t, b, NULL);
    }
    for (int ic = 0; ic < nch; ic++) {
      int ch = chrec[ic];
      zc v = ch <= 2 ? rotate_out(ch, azim[ir], dip[ir], E)
                     : rotate_out(ch - 3, azim[ir], dip[ir], H);
      out[(long)ic * nrec + ir] = (float complex)v;
    }
  }
}

/* per-axis interpolation tables for input cell centres,
 * inject_extract.c:505-546 */
static void centre_tables(int nn, float o, float dd, int ng, const float *ax,
                          int *idx, float *w) {
  for (int i = 0; i < nn; i++) {
    float xc = o + (i + 0.5) * dd;
    int ii = eo_find_index(ng + 1, ax, xc);
    w[i] = (xc - ax[ii]) / (ax[ii + 1] - ax[ii]);
    idx[i] = ii;
  }
}

void eo_extract_electric_field(const eo_grid *g, int nx, int ny, int nz,
                               float ox, float oy, float oz, float dx,
                               float dy, float dz, const float *rho33,
                               const double *xd, float *E1, float *E2,
                               float *E3) {
  const zc *x = (const zc *)xd;
  int *i1 = malloc(nx * sizeof(int)), *i1s = malloc(nx * sizeof(int));
  int *i2 = malloc(ny * sizeof(int)), *i2s = malloc(ny * sizeof(int));
  int *i3 = malloc(nz * sizeof(int)), *i3s = malloc(nz * sizeof(int));
  float *w1 = malloc(nx * sizeof(float)), *w1s = malloc(nx * sizeof(float));
  float *w2 = malloc(ny * sizeof(float)), *w2s = malloc(ny * sizeof(float));
  float *w3 = malloc(nz * sizeof(float)), *w3s = malloc(nz * sizeof(float));
  centre_tables(nx, ox, dx, g->n1, g->x1, i1, w1);
  centre_tables(nx, ox, dx, g->n1, g->x1s, i1s, w1s);
  centre_tables(ny, oy, dy, g->n2, g->x2, i2, w2);
  centre_tables(ny, oy, dy, g->n2, g->x2s, i2s, w2s);
  centre_tables(nz, oz, dz, g->n3, g->x3, i3, w3);
  centre_tables(nz, oz, dz, g->n3, g->x3s, i3s, w3s);
  float complex *o1 = (float complex *)E1, *o2 = (float complex *)E2,
                *o3 = (float complex *)E3;
  const float *s33 = g->sigma33;
  const int n1 = g->n1, n2 = g->n2;
#define S33(ii, jj, kk) s33[(ii) + (long)n1 * ((jj) + (long)n2 * (kk))]
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        long o = i + (long)nx * (j + (long)ny * k);
        tri_t t;
        t.i[0] = i1s[i]; t.w[0] = w1s[i];
        t.i[1] = i2[j];  t.w[1] = w2[j];
        t.i[2] = i3[k];  t.w[2] = w3[k];
        o1[o] = (float complex)gather8(g, 0, &t, x, NULL);
        t.i[0] = i1[i];  t.w[0] = w1[i];
        t.i[1] = i2s[j]; t.w[1] = w2s[j];
        o2[o] = (float complex)gather8(g, 1, &t, x, NULL);
        /* Ez through Jz with 4-cell-averaged sigma33, :598-617 */
        int ii = i1[i], jj = i2[j], kk = i3s[k];
        float wx = w1[i], wy = w2[j], wz = w3s[k];
        zc s = 0;
        float sg;
        for (int dk = 0; dk < 2; dk++)
          for (int dj = 0; dj < 2; dj++)
            for (int di = 0; di < 2; di++) {
              int a = ii + di, bb = jj + dj, cc = kk + dk;
              sg = 0.25 * (S33(a, bb, cc) + S33(a, bb - 1, cc) +
                           S33(a - 1, bb, cc) + S33(a - 1, bb - 1, cc));
              double fx = di ? wx : (1. - wx), fy = dj ? wy : (1. - wy),
                     fz = dk ? wz : (1. - wz);
              s += sg * x[gidx(g, 2, a, bb, cc)] * fx * fy * fz;
            }
        o3[o] = (float complex)(s * rho33[o]);
      }
#undef S33
  free(i1); free(i1s); free(i2); free(i2s); free(i3); free(i3s);
  free(w1); free(w1s); free(w2); free(w2s); free(w3); free(w3s);
}

void eo_extract_magnetic_field(const eo_grid *g, int nx, int ny, int nz,
                               float ox, float oy, float oz, float dx,
                               float dy, float dz, const double *bd, float *H1,
                               float *H2, float *H3) {
  const zc *b = (const zc *)bd;
  int *i1 = malloc(nx * sizeof(int)), *i1s = malloc(nx * sizeof(int));
  int *i2 = malloc(ny * sizeof(int)), *i2s = malloc(ny * sizeof(int));
  int *i3 = malloc(nz * sizeof(int)), *i3s = malloc(nz * sizeof(int));
  float *w1 = malloc(nx * sizeof(float)), *w1s = malloc(nx * sizeof(float));
  float *w2 = malloc(ny * sizeof(float)), *w2s = malloc(ny * sizeof(float));
  float *w3 = malloc(nz * sizeof(float)), *w3s = malloc(nz * sizeof(float));
  centre_tables(nx, ox, dx, g->n1, g->x1, i1, w1);
  centre_tables(nx, ox, dx, g->n1, g->x1s, i1s, w1s);
  centre_tables(ny, oy, dy, g->n2, g->x2, i2, w2);
  centre_tables(ny, oy, dy, g->n2, g->x2s, i2s, w2s);
  centre_tables(nz, oz, dz, g->n3, g->x3, i3, w3);
  centre_tables(nz, oz, dz, g->n3, g->x3s, i3s, w3s);
  float complex *o1 = (float complex *)H1, *o2 = (float complex *)H2,
                *o3 = (float complex *)H3;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        long o = i + (long)nx * (j + (long)ny * k);
        tri_t t;
        t.i[0] = i1[i];  t.w[0] = w1[i];
        t.i[1] = i2s[j]; t.w[1] = w2s[j];
        t.i[2] = i3s[k]; t.w[2] = w3s[k];
        o1[o] = (float complex)gather8(g, 0, &t, b, NULL);
        t.i[0] = i1s[i]; t.w[0] = w1s[i];
        t.i[1] = i2[j];  t.w[1] = w2[j];
        o2[o] = (float complex)gather8(g, 1, &t, b, NULL);
        t.i[1] = i2s[j]; t.w[1] = w2s[j];
        t.i[2] = i3[k];  t.w[2] = w3[k];
        o3[o] = (float complex)gather8(g, 2, &t, b, NULL);
      }
  free(i1); free(i1s); free(i2); free(i2s); free(i3); free(i3s);
  free(w1); free(w1s); free(w2); free(w2s); free(w3); free(w3s);
}

/* build_gradient.c:13-113 */
void eo_build_gradient(int nx, int ny, int nz, float ox, float oy, float oz,
                       float dx, float dy, float dz, int nfreq, int npar,
                       const int *idxpar, int preco, const float *E1f,
                       const float *E2f, const float *E3f, const float *E1a,
                       const float *E2a, const float *E3a, const float *rho11,
                       const float *rho33, const float *bathy, int nsrc,
                       const float *sx, const float *sy, const float *sz,
                       float dsmute, int nrec, const float *rx, const float *ry,
                       const float *rz, float drmute, float *grad,
                       float *phess) {
  const long nxyz = (long)nx * ny * nz;
  const float s = dx * dy * dz;
  const float complex *e1f = (const float complex *)E1f,
                      *e2f = (const float complex *)E2f,
                      *e3f = (const float complex *)E3f,
                      *e1a = (const float complex *)E1a,
                      *e2a = (const float complex *)E2a,
                      *e3a = (const float complex *)E3a;
  for (int kp = 0; kp < npar; kp++)
    for (int i3 = 0; i3 < nz; i3++)
      for (int i2 = 0; i2 < ny; i2++)
        for (int i1 = 0; i1 < nx; i1++) {
          long c = i1 + (long)nx * (i2 + (long)ny * i3);
          float *gp = &grad[kp * nxyz + c];
          *gp = 0;
          for (int f = 0; f < nfreq; f++) {
            long o = f * nxyz + c;
            if (idxpar[kp] == 1) {
              *gp += crealf(e1f[o] * e1a[o]);
              *gp += crealf(e2f[o] * e2a[o]);
            }
            if (idxpar[kp] == 2) *gp += crealf(e3f[o] * e3a[o]);
          }
          if (idxpar[kp] == 1) *gp *= s / rho11[c];
          if (idxpar[kp] == 2) *gp *= s / rho33[c];
          if (oz + (i3 + 0.5) * dz <= bathy[i1 + (long)nx * i2] + dz) *gp = 0.;
          if (preco == 1) {
            float *hp = &phess[kp * nxyz + c];
            *hp = 0.;
            for (int f = 0; f < nfreq; f++) {
              long o = f * nxyz + c;
              if (idxpar[kp] == 1) {
                *hp += cabs(e1f[o]) * cabs(e1f[o]);
                *hp += cabs(e2f[o]) * cabs(e2f[o]);
              }
              if (idxpar[kp] == 2) *hp += cabs(e3f[o]) * cabs(e3f[o]);
            }
            if (idxpar[kp] == 1) *hp *= s / rho11[c];
            if (idxpar[kp] == 2) *hp *= s / rho33[c];
          }
        }
  /* zero boxes around sources and receivers, build_gradient.c:63-111 */
  for (int pass = 0; pass < 2; pass++) {
    int np = pass ? nrec : nsrc;
    const float *px = pass ? rx : sx, *py = pass ? ry : sy, *pz = pass ? rz : sz;
    float rad = pass ? drmute : dsmute;
    for (int is = 0; is < np; is++) {
      int lo[3], hi[3];
      const int nn[3] = {nx, ny, nz};
      lo[0] = (px[is] - rad - ox) / dx; hi[0] = (px[is] + rad - ox) / dx;
      lo[1] = (py[is] - rad - oy) / dy; hi[1] = (py[is] + rad - oy) / dy;
      lo[2] = (pz[is] - rad - oz) / dz; hi[2] = (pz[is] + rad - oz) / dz;
      for (int e = 0; e < 3; e++) {
        lo[e] = lo[e] < 0 ? 0 : lo[e];
        lo[e] = lo[e] > nn[e] - 1 ? nn[e] - 1 : lo[e];
        hi[e] = hi[e] < 0 ? 0 : hi[e];
        hi[e] = hi[e] > nn[e] - 1 ? nn[e] - 1 : hi[e];
      }
      for (int kp = 0; kp < npar; kp++)
        for (int i3 = lo[2]; i3 <= hi[2]; i3++)
          for (int i2 = lo[1]; i2 <= hi[1]; i2++)
            for (int i1 = lo[0]; i1 <= hi[0]; i1++)
              grad[kp * nxyz + i1 + (long)nx * (i2 + (long)ny * i3)] = 0.;
    }
  }
}

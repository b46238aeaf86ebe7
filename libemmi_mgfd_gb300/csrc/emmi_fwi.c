/* Host side of the inversion mode: l-BFGS, the Wolfe line search, model
 * regularization and triangle smoothing, in the reference's float arithmetic
 * (functions cite the reference lines they restate in include/emmi_fwi.h). */
#include "emmi_fwi.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

float ef_l2norm(int n, const float *a) {
  float s = 0.;
  for (int i = 0; i < n; i++) s += a[i] * a[i];
  return sqrtf(s);
}

float ef_dotprod(int n, const float *a, const float *b) {
  float s = 0.;
  for (int i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

void ef_flipsign(int n, const float *a, float *b) {
  for (int i = 0; i < n; i++) b[i] = -a[i];
}

void ef_lbfgs_save(int n, const float *x, const float *g, ef_opt *o) {
  if (o->kpair < o->npair) {
    memcpy(o->sk[o->kpair], x, n * sizeof(float));
    memcpy(o->yk[o->kpair], g, n * sizeof(float));
    o->kpair++;
    return;
  }
  /* full: shift the pairs down one place, the newest last */
  float *s0 = o->sk[0], *y0 = o->yk[0];
  for (int k = 0; k < o->npair - 1; k++) {
    o->sk[k] = o->sk[k + 1];
    o->yk[k] = o->yk[k + 1];
  }
  o->sk[o->npair - 1] = s0;
  o->yk[o->npair - 1] = y0;
  memcpy(s0, x, n * sizeof(float));
  memcpy(y0, g, n * sizeof(float));
}

void ef_lbfgs_update(int n, const float *x, const float *g, ef_opt *o) {
  float *s = o->sk[o->kpair - 1], *y = o->yk[o->kpair - 1];
  for (int i = 0; i < n; i++) {
    s[i] = x[i] - s[i];
    y[i] = g[i] - y[i];
  }
}

/* first loop of the two-loop recursion on q (q = g on entry) */
static void first_loop(int n, float *q, ef_opt *o) {
  for (int k = o->kpair - 1; k >= 0; k--) {
    const float ys = ef_dotprod(n, o->yk[k], o->sk[k]);
    const float sq = ef_dotprod(n, o->sk[k], q);
    o->rho[k] = 1. / ys;
    o->alp[k] = o->rho[k] * sq;
    for (int j = 0; j < n; j++) q[j] -= o->alp[k] * o->yk[k][j];
  }
}

/* scaled initial Hessian and second loop: d = H q (d may be q) */
static void second_loop(int n, const float *q, float *d, ef_opt *o) {
  const int last = o->kpair - 1;
  const float ys = 1. / o->rho[last];
  const float yy = ef_dotprod(n, o->yk[last], o->yk[last]);
  const float gamma = ys / yy;
  for (int j = 0; j < n; j++) d[j] = gamma * q[j];
  for (int k = 0; k < o->kpair; k++) {
    const float beta = o->rho[k] * ef_dotprod(n, o->yk[k], d);
    const float c = o->alp[k] - beta;
    for (int j = 0; j < n; j++) d[j] += c * o->sk[k][j];
  }
}

void ef_lbfgs_descent(int n, const float *g, float *d, ef_opt *o) {
  const float s = o->kpair > 0 ? ef_l2norm(n, o->sk[o->kpair - 1]) : 0;
  const float y = o->kpair > 0 ? ef_l2norm(n, o->yk[o->kpair - 1]) : 0;
  if (!(s > 0. && y > 0.)) { /* no usable pair: steepest descent */
    ef_flipsign(n, g, d);
    return;
  }
  memcpy(o->q, g, n * sizeof(float));
  first_loop(n, o->q, o);
  second_loop(n, o->q, d, o);
  for (int j = 0; j < n; j++) d[j] = -d[j];
}

void ef_lbfgs_descent1(int n, const float *g, ef_opt *o) {
  memcpy(o->q, g, n * sizeof(float));
  o->loop1 = 0;
  const float s = ef_l2norm(n, o->sk[o->kpair - 1]);
  const float y = ef_l2norm(n, o->yk[o->kpair - 1]);
  if (!(s > 0. && y > 0.)) return;
  first_loop(n, o->q, o);
  o->loop1 = 1;
}

void ef_lbfgs_descent2(int n, ef_opt *o) {
  second_loop(n, o->q, o->q, o);
  ef_flipsign(n, o->q, o->d);
}

void ef_boundx(int n, float *x, const float *xmin, const float *xmax) {
  for (int i = 0; i < n; i++) {
    if (x[i] < xmin[i]) x[i] = xmin[i];
    if (x[i] > xmax[i]) x[i] = xmax[i];
  }
}

void ef_line_search(int n, float *x, float *g, const float *d, ef_fg fg, void *ctx, ef_opt *o) {
  const float inf = 0x3f3f3f3f; /* the reference's "infinity" */
  float a1 = 0, a2 = inf, fcost = 0;
  o->alpha = 1.;
  float *xk = malloc(n * sizeof(float));
  memcpy(xk, x, n * sizeof(float));
  float gxd = ef_dotprod(n, g, d);
  const float c1_gxd = o->c1 * gxd, c2_gxd = o->c2 * gxd;
  for (o->ils = 0; o->ils < o->nls; o->ils++) {
    for (int j = 0; j < n; j++) x[j] = xk[j] + o->alpha * d[j];
    if (o->bound == 1) ef_boundx(n, x, o->xmin, o->xmax);
    fcost = fg(ctx, x, g);
    o->igrad++;
    gxd = ef_dotprod(n, g, d);
    const float fxx = o->fk + o->alpha * c1_gxd;
    if (fcost > fxx) { /* sufficient decrease fails: shrink */
      if (o->verb) printf("Wolfe condition 1 fails: insufficient misfit decrease!\n");
      a2 = o->alpha;
      o->alpha = 0.5 * (a1 + a2);
    } else if (gxd < c2_gxd) { /* curvature fails: the step is too short */
      if (o->verb) printf("Wolfe condition 2 fails: stepsize is too small!\n");
      a1 = o->alpha;
      if (a2 < inf) o->alpha = 0.5 * (a1 + a2);
      else o->alpha *= 2.0;
    } else {
      break;
    }
    if (o->verb) {
      printf("#line search %d, alp1=%f alp2=%f alp=%f\n", o->ils, a1, a2, o->alpha);
      printf("------------------------------------------------\n");
    }
  }
  if (fcost <= o->fk) {
    o->ls_fail = 0;
    o->fk = fcost;
  } else {
    o->ls_fail = 1;
  }
  free(xk);
}

float ef_tikhonov(const float *x, float *g, int n1, int n2, int n3) {
  const float ch = 1, cv = 0.03; /* horizontal and vertical weights */
  memset(g, 0, (size_t)n1 * n2 * n3 * sizeof(float));
  float s1 = 0., s2 = 0., s3 = 0.;
  const long st[3] = {1, n1, (long)n1 * n2};
  for (int i3 = 1; i3 < n3 - 1; i3++)
    for (int i2 = 1; i2 < n2 - 1; i2++)
      for (int i1 = 1; i1 < n1 - 1; i1++) {
        const long k = i1 + n1 * ((long)i2 + (long)n2 * i3);
        float t[3];
        for (int e = 0; e < 3; e++) {
          t[e] = -(x[k - st[e]] - 2.0 * x[k] + x[k + st[e]]);
          const float dd = x[k + st[e]] - x[k];
          if (e == 0) s1 += dd * dd;
          else if (e == 1) s2 += dd * dd;
          else s3 += dd * dd;
        }
        g[k] = ch * (t[0] + t[1]) + cv * t[2];
      }
  return ch * (s1 + s2) + cv * s3;
}

float ef_tv(const float *x, float *g, int n1, int n2, int n3) {
  const float eps = 1e-14;
  const size_t nn = (size_t)n1 * n2 * n3;
  float *q = calloc(3 * nn, sizeof(float)); /* grad x / |grad x| */
  memset(g, 0, nn * sizeof(float));
  float cost = 0;
  const long st[3] = {1, n1, (long)n1 * n2};
  for (int i3 = 0; i3 < n3 - 1; i3++)
    for (int i2 = 0; i2 < n2 - 1; i2++)
      for (int i1 = 0; i1 < n1 - 1; i1++) {
        const long k = i1 + n1 * ((long)i2 + (long)n2 * i3);
        const float s1 = x[k + st[0]] - x[k], s2 = x[k + st[1]] - x[k], s3 = x[k + st[2]] - x[k];
        const float t = sqrt(s1 * s1 + s2 * s2 + s3 * s3 + eps);
        cost += t;
        q[k] = s1 / t;
        q[nn + k] = s2 / t;
        q[2 * nn + k] = s3 / t;
      }
  for (int i3 = 1; i3 < n3; i3++)
    for (int i2 = 1; i2 < n2; i2++)
      for (int i1 = 1; i1 < n1; i1++) {
        const long k = i1 + n1 * ((long)i2 + (long)n2 * i3);
        const float a = q[k] - q[k - st[0]];
        const float b = q[nn + k] - q[nn + k - st[1]];
        const float c = q[2 * nn + k] - q[2 * nn + k - st[2]];
        g[k] = -(a + b + c); /* -div(grad x / |grad x|) */
      }
  free(q);
  return cost;
}

/* y = box(x) of length nx + nbox - 1 through the running sum (the box
 * filter of triangle_smoothing.c:34-48) */
static void box(int nbox, int nx, const float *x, float *y, float *run) {
  const int ny = nx + nbox - 1;
  run[0] = x[0];
  for (int i = 1; i < nx; i++) run[i] = run[i - 1] + x[i];
  for (int i = nx; i < ny; i++) run[i] = run[i - 1];
  for (int i = 0; i < nbox; i++) y[i] = run[i];
  for (int i = nbox; i < ny; i++) y[i] = run[i] - run[i - nbox];
  for (int i = 0; i < ny; i++) y[i] /= nbox;
}

/* triangle filter of one line in place, the two ends folded back
 * (triangle_smoothing.c:51-59) */
static void triangle(int nbox, int nd, float *x, float *w) {
  const int np = nbox + nd - 1, nq = nbox + np - 1;
  float *p = w, *q = p + np, *r1 = q + nq, *r2 = r1 + np, *y = r2 + nq;
  box(nbox, nd, x, p, r1);
  box(nbox, np, p, q, r2);
  for (int i = 0; i < nd; i++) y[i] = q[i + nbox - 1];
  for (int i = 0; i < nbox - 1; i++) y[i] += q[nbox - 2 - i];
  for (int i = 0; i < nbox - 1; i++) y[nd - i - 1] += q[nd + (nbox - 1) + i];
  memcpy(x, y, nd * sizeof(float));
}

void ef_triangle_smoothing(float *mod, int n1, int n2, int n3, int r1, int r2, int r3,
                           int repeat) {
  const int nmax = n1 > n2 ? (n1 > n3 ? n1 : n3) : (n2 > n3 ? n2 : n3);
  const int rmax = r1 > r2 ? (r1 > r3 ? r1 : r3) : (r2 > r3 ? r2 : r3);
  float *w = malloc((size_t)(5 * (nmax + 2 * rmax) + 8) * sizeof(float));
  float *line = malloc((size_t)nmax * sizeof(float));
  for (int it = 0; it < repeat; it++) {
    for (int i3 = 0; i3 < n3; i3++)
      for (int i2 = 0; i2 < n2; i2++) triangle(r1, n1, mod + (size_t)n1 * (i2 + (size_t)n2 * i3), w);
    for (int i3 = 0; i3 < n3; i3++)
      for (int i1 = 0; i1 < n1; i1++) {
        for (int i2 = 0; i2 < n2; i2++) line[i2] = mod[i1 + (size_t)n1 * (i2 + (size_t)n2 * i3)];
        triangle(r2, n2, line, w);
        for (int i2 = 0; i2 < n2; i2++) mod[i1 + (size_t)n1 * (i2 + (size_t)n2 * i3)] = line[i2];
      }
    if (n3 > 1)
      for (int i2 = 0; i2 < n2; i2++)
        for (int i1 = 0; i1 < n1; i1++) {
          for (int i3 = 0; i3 < n3; i3++) line[i3] = mod[i1 + (size_t)n1 * (i2 + (size_t)n2 * i3)];
          triangle(r3, n3, line, w);
          for (int i3 = 0; i3 < n3; i3++) mod[i1 + (size_t)n1 * (i2 + (size_t)n2 * i3)] = line[i3];
        }
  }
  free(w);
  free(line);
}

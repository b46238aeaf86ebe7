/* Host front end of the GB300 hot path: regridding and homogenization.
 *
 * Float-for-float restatement of the reference's regrid stage so the mesh
 * and conductivities fed to the solver are the reference's bit for bit
 * (checked against tests/golden by tests/test_host_frontend.py):
 *   create_nugrid   src/create_nugrid.c:13-36
 *   find_index      src/find_index.c:9-30
 *   staggering      src/regrid_init_free.c:21-34
 *   homogenization  src/homogenization.c:15-111
 *   regrid          src/regrid_init_free.c:37-232
 */
#include "emmi_host.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

float eh_create_nugrid(int n, float len, float dx, float *x) {
  if (n * dx >= len) {
    for (int i = 0; i <= n; i++) x[i] = i * dx;
    return 1;
  }
  /* ratio q with dx (q^n - 1)/(q - 1) = len by fixed-point iteration in
   * float, each step evaluated in double (create_nugrid.c:24-33).  The
   * reference loops until two iterates are equal; where the iteration has
   * no fixed point (n = 1 and len > dx: q runs off to infinity, then NaN)
   * it never returns.  Here the loop is capped and that case returns 0. */
  float q = 1.1f, qq;
  const float eps = 1e-15f;
  int done = 0;
  for (int it = 0; it < 100000; it++) {
    qq = pow(len * (q - 1.) / dx + 1., 1. / n);
    if (fabs(qq - q) < eps) {
      done = 1;
      break;
    }
    q = qq;
  }
  if (!done || !isfinite(q)) {
    for (int i = 0; i <= n; i++) x[i] = i * dx;
    return 0;
  }
  x[0] = 0;
  for (int i = 1; i <= n; i++) x[i] = (pow(q, i) - 1.) * dx / (q - 1.);
  return q;
}

int eh_find_index(int n, const float *x, float val) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi) / 2;
    if (x[mid] <= val) lo = mid;
    if (x[mid] > val) hi = mid;
    if (lo == hi || lo == hi - 1) break;
  }
  return lo;
}

/* the same search with a bound on the readable length of x; returns -1 if
 * a probe would fall outside x[0..len-1] */
static int find_index_checked(int n, const float *x, int len, float val) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi) / 2;
    if (mid >= len) return -1;
    if (x[mid] <= val) lo = mid;
    if (x[mid] > val) hi = mid;
    if (lo == hi || lo == hi - 1) break;
  }
  return lo;
}

void eh_stagger(int n, const float *x, float *xs, float *d, float *ds) {
  for (int i = 0; i < n; i++) {
    ds[i] = x[i + 1] - x[i];
    xs[i] = 0.5 * (x[i] + x[i + 1]);
  }
  xs[n] = x[n] + 0.5 * ds[n - 1];
  ds[n] = xs[n] - x[n];
  for (int i = 1; i <= n; i++) d[i] = xs[i] - xs[i - 1];
  d[0] = xs[0] - x[0];
}

/* one 1D conservative average along an axis: source cells [src[k],src[k+1])
 * (ns cells) onto target cells [dst[j],dst[j+1]) (nd cells).  `in` and
 * `out` are read/written with strides. */
static void average_axis(const float *in, long in_stride, int ns, const float *src, float *out,
                         long out_stride, int nd, const float *dst) {
  int i = 0;
  for (int j = 0; j < nd; j++) {
    const float a = dst[j], b = dst[j + 1];
    float s = 0.0;
    while (i < ns && src[i + 1] <= a) i++;
    for (int k = i; k < ns && src[k] < b; k++) {
      const float left = (src[k] > a) ? src[k] : a;
      const float right = (src[k + 1] < b) ? src[k + 1] : b;
      const float overlap = right - left;
      if (overlap > 0.0) s += in[k * in_stride] * overlap;
    }
    out[j * out_stride] = s / (b - a);
  }
}

int eh_homogenize(const float *in, float *out, int nx, int ny, int nz, const float *xx,
                  const float *yy, const float *zz, int n1, int n2, int n3, const float *x1,
                  const float *x2, const float *x3) {
  float *t1 = malloc((size_t)n1 * ny * nz * sizeof(float));
  float *t2 = malloc((size_t)n1 * n2 * nz * sizeof(float));
  if (!t1 || !t2) {
    free(t1);
    free(t2);
    return EH_EINVAL;
  }
  /* x, then y, then z: homogenization.c:24-48, 51-76, 79-103 */
  for (int iz = 0; iz < nz; iz++)
    for (int iy = 0; iy < ny; iy++)
      average_axis(in + (size_t)nx * (iy + (size_t)ny * iz), 1, nx, xx,
                   t1 + (size_t)n1 * (iy + (size_t)ny * iz), 1, n1, x1);
  for (int iz = 0; iz < nz; iz++)
    for (int ix = 0; ix < n1; ix++)
      average_axis(t1 + ix + (size_t)n1 * ny * iz, n1, ny, yy, t2 + ix + (size_t)n1 * n2 * iz, n1,
                   n2, x2);
  for (int iy = 0; iy < n2; iy++)
    for (int ix = 0; ix < n1; ix++)
      average_axis(t2 + ix + (size_t)n1 * iy, (long)n1 * n2, nz, zz, out + ix + (size_t)n1 * iy,
                   (long)n1 * n2, n3, x3);
  free(t1);
  free(t2);
  return EH_OK;
}

float eh_rho_water(const eh_model *m) {
  const long n = (long)m->nx * m->ny * m->nz;
  float vmin = m->rho11[0];
  for (long i = 0; i < n; i++) {
    if (m->rho11[i] < vmin) vmin = m->rho11[i];
    if (m->rho22[i] < vmin) vmin = m->rho22[i];
    if (m->rho33[i] < vmin) vmin = m->rho33[i];
  }
  return vmin;
}

/* padded axis: nb geometric cells on each side of n uniform cells
 * (regrid_init_free.c:47-70) */
static int padded_axis(int n, float d, float o, int nb, float lextend, float *ax) {
  float *x = malloc((nb + 1) * sizeof(float));
  for (int i = 0; i <= n; i++) ax[i + nb] = o + i * d;
  const float q = eh_create_nugrid(nb, lextend, d, x);
  for (int i = 0; i <= nb; i++) {
    ax[i] = o - x[nb - i];
    ax[i + n + nb] = o + n * d + x[i];
  }
  free(x);
  return q == 0 ? EH_ENUGRID : EH_OK;
}

/* stretched mesh axis centred on the source: n/2 cells to the low side and
 * the rest to the high side (regrid_init_free.c:156-187) */
static int centred_axis(int n, float src, float lo, float hi, float dmin, float *out) {
  const int np1 = n / 2, np2 = n - np1;
  float *x = malloc((n + 1) * sizeof(float));
  const float q1 = eh_create_nugrid(np1, src - lo, dmin, x);
  for (int i = 0; i <= np1; i++) out[np1 - i] = src - x[i];
  const float q2 = eh_create_nugrid(np2, hi - src, dmin, x);
  for (int i = 0; i <= np2; i++) out[np1 + i] = src + x[i];
  free(x);
  return (q1 == 0 || q2 == 0) ? EH_ENUGRID : EH_OK;
}

int eh_pad_dims(const eh_model *m, int *nxp, int *nyp, int *nzp) {
  if (!m || m->nx < 1 || m->ny < 1 || m->nz < 1 || m->nb < 0) return EH_EINVAL;
  *nxp = m->nx + 2 * m->nb;
  *nyp = m->ny + 2 * m->nb;
  *nzp = m->nz + 2 * m->nb;
  return EH_OK;
}

/* padded model: interior copied (sigma = 1/rho for 11/22, rho for 33),
 * edges replicated, nb air cells on top (regrid_init_free.c:82-141); the
 * padded node axes (regrid_init_free.c:47-70) */
int eh_pad_model(const eh_model *m, float *xx, float *yy, float *zz, float *pad) {
  int nxp, nyp, nzp;
  if (eh_pad_dims(m, &nxp, &nyp, &nzp) != EH_OK) return EH_EINVAL;
  const int nb = m->nb;
  if (padded_axis(m->nx, m->dx, m->ox, nb, m->lextend, xx) != EH_OK ||
      padded_axis(m->ny, m->dy, m->oy, nb, m->lextend, yy) != EH_OK ||
      padded_axis(m->nz, m->dz, m->oz, nb, m->lextend, zz) != EH_OK)
    return EH_ENUGRID;
  const size_t np = (size_t)nxp * nyp * nzp;
#define PAD(a, i, j, k) pad[(size_t)(a) * np + (i) + (size_t)nxp * ((j) + (size_t)nyp * (k))]
  for (int k = 0; k < m->nz; k++)
    for (int j = 0; j < m->ny; j++)
      for (int i = 0; i < m->nx; i++) {
        const size_t c = i + (size_t)m->nx * (j + (size_t)m->ny * k);
        PAD(0, i + nb, j + nb, k + nb) = 1. / m->rho11[c];
        PAD(1, i + nb, j + nb, k + nb) = 1. / m->rho22[c];
        PAD(2, i + nb, j + nb, k + nb) = m->rho33[c];
      }
  for (int a = 0; a < 3; a++) {
    for (int k = 0; k < nzp; k++)
      for (int j = 0; j < nyp; j++)
        for (int i = 0; i < nb; i++) {
          PAD(a, i, j, k) = PAD(a, nb, j, k);
          PAD(a, nxp - 1 - i, j, k) = PAD(a, nxp - 1 - nb, j, k);
        }
    for (int k = 0; k < nzp; k++)
      for (int j = 0; j < nb; j++)
        for (int i = 0; i < nxp; i++) {
          PAD(a, i, j, k) = PAD(a, i, nb, k);
          PAD(a, i, nyp - 1 - j, k) = PAD(a, i, nyp - 1 - nb, k);
        }
    for (int k = 0; k < nb; k++)
      for (int j = 0; j < nyp; j++)
        for (int i = 0; i < nxp; i++) {
          PAD(a, i, j, k) = (a < 2) ? (float)(1. / m->rho_air) : m->rho_air;
          PAD(a, i, j, nzp - 1 - k) = PAD(a, i, j, nzp - 1 - nb);
        }
  }
#undef PAD
  return EH_OK;
}

int eh_regrid_axes(const eh_model *m, const float *xx, const float *yy, const float *zz,
                   float sx, float sy, float sz, eh_grid *g) {
  int nxp, nyp, nzp;
  if (!g || eh_pad_dims(m, &nxp, &nyp, &nzp) != EH_OK || m->n1 < 2 || m->n2 < 2 || m->n3 < 2)
    return EH_EINVAL;
  if (centred_axis(m->n1, sx, xx[0], xx[nxp], m->d1min, g->x1) != EH_OK ||
      centred_axis(m->n2, sy, yy[0], yy[nyp], m->d2min, g->x2) != EH_OK)
    return EH_ENUGRID;
  /* z: input-model nodes down to 5 cells below the source, then stretched
   * to the bottom (regrid_init_free.c:190-205).  The reference sizes the
   * source search by nx (its line 194); it is reproduced, with a check that
   * the search stays on the padded z axis. */
  const int k0 = find_index_checked(m->nx + 2 * m->nb, zz, nzp + 1, sz);
  if (k0 < 0) return EH_ESEARCH;
  const int np1 = k0 + 5, np2 = m->n3 - np1;
  if (np1 > nzp || np2 < 1) return EH_EINVAL;
  for (int i = 0; i <= np1; i++) g->x3[i] = zz[i];
  float *x = malloc((np2 + 1) * sizeof(float));
  const float q = eh_create_nugrid(np2, zz[nzp] - g->x3[np1], m->d3min, x);
  for (int i = 0; i <= np2; i++) g->x3[np1 + i] = g->x3[np1] + x[i];
  free(x);
  if (q == 0) return EH_ENUGRID;
  eh_stagger(m->n1, g->x1, g->x1s, g->d1, g->d1s);
  eh_stagger(m->n2, g->x2, g->x2s, g->d2, g->d2s);
  eh_stagger(m->n3, g->x3, g->x3s, g->d3, g->d3s);
  return EH_OK;
}

int eh_regrid(const eh_model *m, float sx, float sy, float sz, eh_grid *g) {
  if (!m || !g || m->nx < 1 || m->ny < 1 || m->nz < 1 || m->nb < 0 || m->n1 < 2 || m->n2 < 2 ||
      m->n3 < 2)
    return EH_EINVAL;
  int nxp, nyp, nzp;
  eh_pad_dims(m, &nxp, &nyp, &nzp);
  float *xx = malloc((nxp + 1) * sizeof(float));
  float *yy = malloc((nyp + 1) * sizeof(float));
  float *zz = malloc((nzp + 1) * sizeof(float));
  const size_t np = (size_t)nxp * nyp * nzp;
  float *pad = malloc(3 * np * sizeof(float));
  int rc = eh_pad_model(m, xx, yy, zz, pad);
  if (rc == EH_OK) rc = eh_regrid_axes(m, xx, yy, zz, sx, sy, sz, g);
  if (rc == EH_OK) {
    float *outs[3] = {g->sigma11, g->sigma22, g->sigma33};
    for (int a = 0; a < 3 && rc == EH_OK; a++)
      rc = eh_homogenize(pad + (size_t)a * np, outs[a], nxp, nyp, nzp, xx, yy, zz, m->n1, m->n2,
                         m->n3, g->x1, g->x2, g->x3);
    const size_t nc = (size_t)m->n1 * m->n2 * m->n3;
    for (size_t c = 0; c < nc; c++) {
      g->sigma33[c] = 1. / g->sigma33[c]; /* rho33 average -> sigma33 */
      g->invmur[c] = 1.;
    }
  }
  free(pad);
  free(xx);
  free(yy);
  free(zz);
  return rc;
}

/* ---- data misfit of the gradient mode --------------------------------- */
/* The arithmetic keeps the reference's types: float data and uncertainty,
 * double trigonometry and absolute values, float accumulation. */
enum { EH_EX = 0, EH_EY = 1, EH_HX = 3, EH_HY = 4 };

static float complex datum(const float *a, long i) { return a[2 * i] + I * a[2 * i + 1]; }

void eh_uncertainty(int nchrec, const int *ch, int nfreq, int nrec, const float *rec_azimuth,
                    float src_azimuth, const float *dobs, float amp_perc, float delta_phi,
                    float noisefloorE, float noisefloorH, float *delta) {
  memset(delta, 0, (size_t)nchrec * nfreq * nrec * sizeof(float));
  for (int ir = 0; ir < nrec; ir++) {
    const float phi = rec_azimuth[ir] - src_azimuth;  /* receiver vs towline */
    for (int f = 0; f < nfreq; f++) {
      /* the horizontal components and their rotation into the towline */
      float complex ex = 0, ey = 0, hx = 0, hy = 0, exc = 0, eyc = 0, hxc = 0, hyc = 0;
      for (int c = 0; c < nchrec; c++) {
        const float complex v = datum(dobs, ((long)c * nfreq + f) * nrec + ir);
        switch (ch[c]) {
          case EH_EX: ex = v; exc += ex * cos(phi); eyc += ex * sin(phi); break;
          case EH_EY: ey = v; exc -= ey * sin(phi); eyc += ey * cos(phi); break;
          case EH_HX: hx = v; hxc += hx * cos(phi); hyc += hx * sin(phi); break;
          case EH_HY: hy = v; hxc -= hy * sin(phi); hyc += hy * cos(phi); break;
          default: break;
        }
      }
      for (int c = 0; c < nchrec; c++) {
        float s1, s2, s3, nf;
        switch (ch[c]) {
          case EH_EX:
            s1 = cabs(amp_perc * ex) * cos(phi);
            s2 = cabs(amp_perc * ey) * sin(phi);
            s3 = delta_phi * cabs(eyc);
            nf = noisefloorE;
            break;
          case EH_EY:
            s1 = cabs(amp_perc * ex) * sin(phi);
            s2 = cabs(amp_perc * ey) * cos(phi);
            s3 = delta_phi * cabs(exc);
            nf = noisefloorE;
            break;
          case EH_HX:
            s1 = cabs(amp_perc * hx) * cos(phi);
            s2 = cabs(amp_perc * hy) * sin(phi);
            s3 = delta_phi * cabs(hyc);
            nf = noisefloorH;
            break;
          case EH_HY:  /* the reference scales inside the modulus here */
            s1 = cabs(amp_perc * hx) * sin(phi);
            s2 = cabs(amp_perc * hy) * cos(phi);
            s3 = cabs(delta_phi * hxc);
            nf = noisefloorH;
            break;
          default:
            continue;
        }
        delta[((long)c * nfreq + f) * nrec + ir] = sqrt(s1 * s1 + s2 * s2 + s3 * s3 + nf * nf);
      }
    }
  }
}

float eh_misfit(int nchrec, int nfreq, int nrec, const float *omegas, float rho_water, float src_x,
                float src_y, const float *rec_x, const float *rec_y, const float *dobs,
                const float *dcal, const float *delta, float *dres, float *rmse) {
  const double mu0 = 4. * 3.14159265358979323846264 * 1e-7;
  memset(dres, 0, (size_t)nchrec * nfreq * nrec * 2 * sizeof(float));
  memset(rmse, 0, (size_t)nchrec * nfreq * nrec * sizeof(float));
  float fcost = 0.f;
  for (int c = 0; c < nchrec; c++)
    for (int f = 0; f < nfreq; f++) {
      const float skin = 5.5 * sqrt(2. * rho_water / (omegas[f] * mu0));
      for (int ir = 0; ir < nrec; ir++) {
        const float ox = rec_x[ir] - src_x, oy = rec_y[ir] - src_y;
        if (!(sqrt(ox * ox + oy * oy) > skin)) continue;
        const long i = ((long)c * nfreq + f) * nrec + ir;
        float complex r = datum(dobs, i) - datum(dcal, i);
        r /= delta[i];
        rmse[i] = cabs(r);
        fcost += r * conj(r);
        r /= delta[i];
        r = conj(r);
        dres[2 * i] = crealf(r);
        dres[2 * i + 1] = cimagf(r);
      }
    }
  fcost *= 0.5;
  return fcost;
}

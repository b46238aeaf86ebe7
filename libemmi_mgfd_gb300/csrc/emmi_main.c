/* emmi_main: the reference's command line on the GB300 hot path.
 *
 *   emmi_main mode=0 freqs=1 chsrc=Ex chrec=Ex,Ey,Hx,Hy nx=.. ny=.. nz=..
 *             dx=.. dy=.. dz=.. ox=.. oy=.. [oz=0] [n1=n2=n3=128]
 *             frho11=.. frho22=.. frho33=.. fsrc=.. frec=.. fsrcrec=..
 *             [shots=1,2,..] [cycleopt ncycle v1 v2 tol isemicoarsen]
 *             [gmg_precision=1] [skip_pre=0 skip_post=0] [verb=1]
 *   emmi_main mode=2 ... fbathy=.. [npar=2 idxpar=1,2 preco=1 addnoise=1
 *             amp_perc=0.03 delta_phi=0 noisefloorE=1e-15 noisefloorH=1e-13
 *             dsmute=800 drmute=200 gamma1=10 gamma2=0 r1=r2=r3=3 repeat=1]
 *   emmi_main mode=1 ... [niter=30 nls=5 npair=5 c1=1e-4 c2=0.9 tol=1e-6
 *             bound=0 minpar=.. maxpar=..]
 *
 * Same parameters (src/emf_init_free.c:19-112, src/acq_init_free.c:27-128,
 * src/gmg.c:1712-1717, src/do_fwi.c:68-72, src/fg_fwi.c:55-63), same input
 * files and the same output files in the reference's formats
 * (src/read_write_data.c).  mode=0 is the frequency loop of
 * src/do_modelling.c:49-67 -> emf_%04d.txt.  mode=2 is one gradient of
 * src/fg_fwi.c:139-290: observed data from emf_%04d.txt, uncertainties,
 * forward modelling (syn_%04d.txt), misfit and adjoint sources
 * (rmse_%04d.txt), adjoint modelling and build_gradient, summed over the
 * shots into gradient_dat_Rv / gradient_dat_Rh (the reference's names: the
 * first holds parameter idxpar[0], the second idxpar[1]).  mode=1 is the
 * inversion of src/do_fwi.c:68-231: x = log of the resistivities named by
 * idxpar, the objective of src/fg_fwi.c (data misfit with the gradient
 * above, plus the model regularization of src/fg_mod_reg.c, with the
 * first-gradient scaling) minimized by l-BFGS with the Wolfe bisection
 * line search and the preconditioners of src/precondition.c (libemmi_host's
 * emmi_fwi.h); iterate.txt, rmse_misfit.txt, Rv_iteration_%02d and
 * Rh_iteration_%02d as the reference writes them.  All modes call the
 * drop-in entry points of libemmi_gpu.  Without MPI the shots listed in
 * shots= run one after another in this process (the reference runs one per
 * rank and sums with MPI_Allreduce).  With addnoise=1 the noise comes from
 * this program's own seeded generator (seed=), not the reference's.
 */
#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "emmi_dropin.h"
#include "emmi_fwi.h"
#include "emmi_gpu.h"
#include "emmi_host.h"

void initargs(int argc, char **argv);
int countparval(const char *name);
int getparint(char *name, int *p);
int getparfloat(char *name, float *p);
int getparstring(char *name, char **p);
int getparstringarray(char *name, char **p);

#define PI_REF 3.14159265358979323846264

static void die(const char *msg, const char *arg) {
  fprintf(stderr, "emmi_main: %s%s\n", msg, arg ? arg : "");
  exit(1);
}

static float *read_floats(const char *path, size_t n) {
  float *a = malloc(n * sizeof(float));
  FILE *fp = fopen(path, "rb");
  if (!fp) die("cannot open ", path);
  if (fread(a, sizeof(float), n, fp) != n) die("size mismatch in ", path);
  fclose(fp);
  return a;
}

/* pointer table over a contiguous block, as the reference's alloc3/alloc4 */
static void ***table3(void *base, size_t esz, int n1, int n2, int n3) {
  void ***t = malloc(n3 * sizeof(void **));
  void **t2 = malloc((size_t)n3 * n2 * sizeof(void *));
  for (int k = 0; k < n3; k++) {
    t[k] = t2 + (size_t)k * n2;
    for (int j = 0; j < n2; j++) t[k][j] = (char *)base + (((size_t)k * n2 + j) * n1) * esz;
  }
  return t;
}

static void ****table4(void *base, size_t esz, int n1, int n2, int n3, int n4) {
  void ****t = malloc(n4 * sizeof(void ***));
  for (int l = 0; l < n4; l++)
    t[l] = table3((char *)base + (size_t)l * n3 * n2 * n1 * esz, esz, n1, n2, n3);
  return t;
}

static int chan_code(const char *c) {
  static const char *names[6] = {"Ex", "Ey", "Ez", "Hx", "Hy", "Hz"};
  for (int i = 0; i < 6; i++)
    if (!strcmp(c, names[i])) return i;
  die("unknown channel ", c);
  return -1;
}

/* complex Gaussian with unit variance (Box-Muller on a 64-bit LCG) */
static unsigned long long rng_state = 1;
static double uniform01(void) {
  rng_state = rng_state * 6364136223846793005ULL + 1442695040888963407ULL;
  return ((rng_state >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
static float complex gauss_c(void) {
  const double r = sqrt(-2.0 * log(uniform01())), t = 2.0 * PI_REF * uniform01();
  return (float)(r * cos(t) / sqrt(2.)) + I * (float)(r * sin(t) / sqrt(2.));
}

typedef struct {
  float x, y, z, hd, pit;
} point_t;

/* acquisition file: header line, then "x y z heading pitch idx" */
static point_t *read_points(const char *path, int *n) {
  FILE *fp = fopen(path, "r");
  if (!fp) die("cannot open ", path);
  int cap = 1024, k = 0, idx;
  point_t *p = malloc(cap * sizeof(point_t));
  if (fscanf(fp, "%*[^\n]\n") < 0) die("empty file ", path);
  point_t q;
  while (fscanf(fp, "%f %f %f %f %f %d", &q.x, &q.y, &q.z, &q.hd, &q.pit, &idx) == 6) {
    if (k == cap) p = realloc(p, (cap *= 2) * sizeof(point_t));
    p[k++] = q;
  }
  fclose(fp);
  *n = k;
  return p;
}

/* the frequency loop of do_modelling (src/do_modelling.c:50-64) and of the
 * two modelling stages of fg_fwi (src/fg_fwi.c:183-202, 237-258): forward
 * sources, or adjoint sources from emf->dres_fd; in the gradient mode the
 * electric field is also interpolated to the input cells (emf->E1..E3) */
static void model_all(emmi_emf_t *emf, emmi_acq_t *acq, double complex *x, double complex *b,
                      long n3s, int shot, int adjoint) {
  for (int f = 0; f < emf->nfreq; f++) {
    gmg_init(emf, f);
    if (adjoint)
      inject_adj_source(acq, emf, (emmi_cf64 *)x, (emmi_cf64 *)b, f);
    else
      inject_source(acq, emf, (emmi_cf64 *)b, f);
    memset(x, 0, n3s * sizeof(double complex));
    gmg_apply((int)n3s, (emmi_cf64 *)b, (emmi_cf64 *)x);
    int cyc;
    double rel;
    const int st = emmi_gpu_last_status(&cyc, &rel);
    if (emf->verb)
      printf("shot %d freq %g%s: %d cycles, relative residual %.3e, status %d\n", shot,
             emf->freqs[f], adjoint ? " (adjoint)" : "", cyc, rel, st);
    extract_emf_data(acq, emf, (emmi_cf64 *)x, (emmi_cf64 *)b, f);
    if (emf->mode != 0) extract_electric_field(acq, emf, (emmi_cf64 *)x, f);
    gmg_free();
  }
}

/* write_data (src/read_write_data.c:14-36): data[nchrec][nfreq][nrec] */
static void write_data(const char *fname, int shot, const emmi_emf_t *emf, int nrec,
                       const emmi_cf32 *data) {
  FILE *out = fopen(fname, "w");
  if (!out) die("cannot write ", fname);
  fprintf(out, "iTx \tiRx    chrec  frequency/Hz    Real{E/H}     Imag{E/H}\n");
  for (int ic = 0; ic < emf->nchrec; ic++)
    for (int f = 0; f < emf->nfreq; f++)
      for (int ir = 0; ir < nrec; ir++) {
        const float *v = (const float *)&data[((size_t)ic * emf->nfreq + f) * nrec + ir];
        fprintf(out, "%d \t %d \t %s \t %g \t %e \t %e\n", shot, ir + 1, emf->chrec[ic],
                emf->freqs[f], v[0], v[1]);
      }
  fclose(out);
}

/* read_data (src/read_write_data.c:39-77): observed data of this shot from
 * emf_%04d.txt, matched by channel name and frequency (within 1e-4 Hz) */
static void read_data(int shot, const emmi_emf_t *emf, int nrec, emmi_cf32 *dobs) {
  char fname[64];
  snprintf(fname, sizeof(fname), "emf_%04d.txt", shot);
  FILE *fp = fopen(fname, "r");
  if (!fp) die("cannot open observed data ", fname);
  if (fscanf(fp, "%*[^\n]\n") < 0) die("empty file ", fname);
  int isrc, irec;
  char ch[16];
  float freq, re, im;
  while (fscanf(fp, "%d %d %15s %g %e %e", &isrc, &irec, ch, &freq, &re, &im) == 6) {
    if (isrc != shot || irec < 1 || irec > nrec) continue;
    for (int ic = 0; ic < emf->nchrec; ic++) {
      if (strcmp(emf->chrec[ic], ch)) continue;
      for (int f = 0; f < emf->nfreq; f++)
        if (fabs(emf->freqs[f] - freq) < 1e-4) {
          dobs[((size_t)ic * emf->nfreq + f) * nrec + irec - 1] = re + I * im;
          break;
        }
      break;
    }
  }
  fclose(fp);
}

/* one shot's acquisition and, in the inversion modes, its observed data
 * with their uncertainties (fg_fwi_init, src/fg_fwi.c:105-114: read once,
 * noise added once) */
typedef struct {
  int shot, nrec;
  float src5[5]; /* x, y, z, azimuth, dip (radians) */
  float *rx, *ry, *rz, *raz, *rdip;
  emmi_cf32 *dobs; /* [nchrec][nfreq][nrec] */
  float *delta;
} shot_t;

/* what one misfit-and-gradient evaluation needs */
typedef struct {
  emmi_emf_t *emf;
  emmi_acq_t *acq;
  emmi_fwi_t *fwi;
  eh_model *M;
  shot_t *sh;
  int nshots, ndata;
  double complex *x, *b;
  long n3s;
  size_t nxyz;
  int *chc;
  emmi_cf32 *Ef, *Ea, *dc;
  float *s11, *s22, *s33, *imu, *gsum, *hsum;
  /* the batched evaluation on the device (batch=1): the padded model and
   * its axes, each shot's misfit, data and rmse [nshot][nchrec][nfreq]
   * [maxrec], solve statistics [2][nshot*nfreq] */
  emmi_fg *fg;
  int nxp, nyp, nzp, maxrec;
  float *pxx, *pyy, *pzz, *pad, *fshot, *rall;
  emmi_cf32 *dall;
  emmi_rhs_stats *stats;
} fg_ctx;

/* point acq at the shot, regrid the current model around its source
 * (regrid_init, the host front end) into emf */
static void set_shot(fg_ctx *c, shot_t *t) {
  emmi_emf_t *emf = c->emf;
  emmi_acq_t *acq = c->acq;
  acq->nsrc = 1;
  acq->nrec = t->nrec;
  acq->src_x1 = &t->src5[0];
  acq->src_x2 = &t->src5[1];
  acq->src_x3 = &t->src5[2];
  acq->src_azimuth = &t->src5[3];
  acq->src_dip = &t->src5[4];
  acq->rec_x1 = t->rx;
  acq->rec_x2 = t->ry;
  acq->rec_x3 = t->rz;
  acq->rec_azimuth = t->raz;
  acq->rec_dip = t->rdip;
  eh_grid G = {emf->x1, emf->x2, emf->x3, emf->x1s, emf->x2s, emf->x3s,
               emf->d1, emf->d2, emf->d3, emf->d1s, emf->d2s, emf->d3s,
               c->s11, c->s22, c->s33, c->imu};
  const int rg = eh_regrid(c->M, t->src5[0], t->src5[1], t->src5[2], &G);
  if (rg == EH_ENUGRID)
    die("no geometric stretching ratio for a mesh axis (too few cells left below the source "
        "for the bottom stretch? raise n3)", NULL);
  if (rg != EH_OK) die("regrid failed", NULL);
}

/* rmse_%04d.txt of a shot: rmse [nchrec][nfreq][nrec] (write_rmse,
 * src/read_write_data.c:80-102) */
static void write_rmse(const emmi_emf_t *emf, const shot_t *t, const float *rmse) {
  char fname[64];
  snprintf(fname, sizeof(fname), "rmse_%04d.txt", t->shot);
  FILE *fp = fopen(fname, "w");
  if (!fp) die("cannot write ", fname);
  fprintf(fp, "iTx iRx chrec frequency/Hz RMSE x y z\n");
  for (int ic = 0; ic < emf->nchrec; ic++)
    for (int f = 0; f < emf->nfreq; f++)
      for (int ir = 0; ir < t->nrec; ir++)
        fprintf(fp, "%d %d %s %g %e %g %g %g\n", t->shot, ir + 1, emf->chrec[ic], emf->freqs[f],
                rmse[((size_t)ic * emf->nfreq + f) * t->nrec + ir], t->rx[ir], t->ry[ir],
                t->rz[ir]);
  fclose(fp);
}

/* forward modelling, misfit and adjoint sources, adjoint modelling and the
 * gradient of one shot (src/fg_fwi.c:183-268); returns its misfit and
 * leaves its data gradient in fwi->grad (fwi->phess with preco=1) */
static float gradient_shot(fg_ctx *c, shot_t *t) {
  emmi_emf_t *emf = c->emf;
  emmi_acq_t *acq = c->acq;
  const int nrec = t->nrec, nr = nrec ? nrec : 1, nf = emf->nfreq;
  const size_t nd = (size_t)emf->nchrec * nf * nr;
  emmi_cf32 *dres = calloc(nd, sizeof(emmi_cf32));
  float *rmse = calloc(nd, sizeof(float));
  memset(c->dc, 0, nd * sizeof(emmi_cf32));
  emf->dcal_fd = (emmi_cf32 ***)table3(c->dc, sizeof(emmi_cf32), nr, nf, emf->nchrec);
  emf->dobs_fd = (emmi_cf32 ***)table3(t->dobs, sizeof(emmi_cf32), nr, nf, emf->nchrec);
  emf->dres_fd = (emmi_cf32 ***)table3(dres, sizeof(emmi_cf32), nr, nf, emf->nchrec);
  emf->delta_emf = (float ***)table3(t->delta, sizeof(float), nr, nf, emf->nchrec);
  emf->rmse = (float ***)table3(rmse, sizeof(float), nr, nf, emf->nchrec);
  const int nx = emf->nx, ny = emf->ny, nz = emf->nz;
  const size_t nfe = c->nxyz * nf;
  emmi_cf32 ****E1f = (emmi_cf32 ****)table4(c->Ef, sizeof(emmi_cf32), nx, ny, nz, nf);
  emmi_cf32 ****E2f = (emmi_cf32 ****)table4(c->Ef + nfe, sizeof(emmi_cf32), nx, ny, nz, nf);
  emmi_cf32 ****E3f = (emmi_cf32 ****)table4(c->Ef + 2 * nfe, sizeof(emmi_cf32), nx, ny, nz, nf);
  emmi_cf32 ****E1a = (emmi_cf32 ****)table4(c->Ea, sizeof(emmi_cf32), nx, ny, nz, nf);
  emmi_cf32 ****E2a = (emmi_cf32 ****)table4(c->Ea + nfe, sizeof(emmi_cf32), nx, ny, nz, nf);
  emmi_cf32 ****E3a = (emmi_cf32 ****)table4(c->Ea + 2 * nfe, sizeof(emmi_cf32), nx, ny, nz, nf);
  emf->E1 = E1f;
  emf->E2 = E2f;
  emf->E3 = E3f;
  model_all(emf, acq, c->x, c->b, c->n3s, t->shot, 0);
  char fname[64];
  snprintf(fname, sizeof(fname), "syn_%04d.txt", t->shot);
  write_data(fname, t->shot, emf, nrec, c->dc);
  /* misfit and adjoint sources, rmse_%04d.txt (write_rmse,
   * src/read_write_data.c:80-102) */
  const float fcost = eh_misfit(emf->nchrec, nf, nrec, emf->omegas, emf->rho_water,
                                acq->src_x1[0], acq->src_x2[0], acq->rec_x1, acq->rec_x2,
                                (const float *)t->dobs, (const float *)c->dc, t->delta,
                                (float *)dres, rmse);
  write_rmse(emf, t, rmse);
  const int ndat = emf->nchrec * nf * nrec;
  if (emf->verb) printf("isrc=%d, fcost=%g, rmse=%g\n", t->shot, fcost, sqrt(2. * fcost / ndat));
  emf->E1 = E1a;
  emf->E2 = E2a;
  emf->E3 = E3a;
  model_all(emf, acq, c->x, c->b, c->n3s, t->shot, 1);
  build_gradient(acq, emf, c->fwi, E1f, E2f, E3f, E1a, E2a, E3a);
  void ****tb[6] = {(void ****)E1f, (void ****)E2f, (void ****)E3f,
                    (void ****)E1a, (void ****)E2a, (void ****)E3a};
  for (int k = 0; k < 6; k++) {
    for (int l = 0; l < nf; l++) {
      free(tb[k][l][0]);
      free(tb[k][l]);
    }
    free(tb[k]);
  }
  void ***t3[5] = {(void ***)emf->dcal_fd, (void ***)emf->dobs_fd, (void ***)emf->dres_fd,
                   (void ***)emf->delta_emf, (void ***)emf->rmse};
  for (int k = 0; k < 5; k++) {
    free(t3[k][0]);
    free(t3[k]);
  }
  free(dres);
  free(rmse);
  return fcost;
}

/* the batched evaluation (batch=1): every shot's mesh axes (the padded
 * model's node axes do not depend on the resistivities), the survey and,
 * with_data, the observed data and the uncertainties go to the device once;
 * without them only the forward modelling of mode=0 runs */
static void fg_batch_init(fg_ctx *c, int with_data) {
  emmi_emf_t *emf = c->emf;
  emmi_fwi_t *fwi = c->fwi;
  const int ns = c->nshots, nf = emf->nfreq, nch = emf->nchrec;
  const int n1 = emf->n1, n2 = emf->n2, n3 = emf->n3;
  if (eh_pad_dims(c->M, &c->nxp, &c->nyp, &c->nzp) != EH_OK) die("eh_pad_dims failed", NULL);
  c->pxx = malloc((c->nxp + 1) * sizeof(float));
  c->pyy = malloc((c->nyp + 1) * sizeof(float));
  c->pzz = malloc((c->nzp + 1) * sizeof(float));
  c->pad = malloc((size_t)3 * c->nxp * c->nyp * c->nzp * sizeof(float));
  if (eh_pad_model(c->M, c->pxx, c->pyy, c->pzz, c->pad) != EH_OK) die("eh_pad_model failed", NULL);
  int maxrec = 1;
  for (int is = 0; is < ns; is++)
    if (c->sh[is].nrec > maxrec) maxrec = c->sh[is].nrec;
  c->maxrec = maxrec;
  float *ax[3] = {malloc((size_t)ns * (n1 + 1) * sizeof(float)),
                  malloc((size_t)ns * (n2 + 1) * sizeof(float)),
                  malloc((size_t)ns * (n3 + 1) * sizeof(float))};
  float *tmp = malloc((size_t)9 * (n1 + n2 + n3 + 3) * sizeof(float));
  float *src = calloc((size_t)ns * 5, sizeof(float));
  float *rec = calloc((size_t)ns * maxrec * 5, sizeof(float));
  int *nrs = malloc(ns * sizeof(int));
  const size_t nper = (size_t)ns * nch * nf * maxrec;
  emmi_cf32 *dobs = calloc(nper, sizeof(emmi_cf32));
  float *delta = calloc(nper, sizeof(float));
  for (int is = 0; is < ns; is++) {
    const shot_t *t = &c->sh[is];
    float *q = tmp;
    eh_grid g;
    memset(&g, 0, sizeof(g));
    g.x1 = ax[0] + (size_t)is * (n1 + 1);
    g.x2 = ax[1] + (size_t)is * (n2 + 1);
    g.x3 = ax[2] + (size_t)is * (n3 + 1);
    float **rest[9] = {&g.x1s, &g.x2s, &g.x3s, &g.d1, &g.d2, &g.d3, &g.d1s, &g.d2s, &g.d3s};
    const int len[3] = {n1 + 1, n2 + 1, n3 + 1};
    for (int k = 0; k < 9; k++) {
      *rest[k] = q;
      q += len[k % 3];
    }
    const int rg = eh_regrid_axes(c->M, c->pxx, c->pyy, c->pzz, t->src5[0], t->src5[1],
                                  t->src5[2], &g);
    if (rg == EH_ENUGRID)
      die("no geometric stretching ratio for a mesh axis (too few cells left below the source "
          "for the bottom stretch? raise n3)", NULL);
    if (rg != EH_OK) die("eh_regrid_axes failed", NULL);
    memcpy(src + (size_t)is * 5, t->src5, 5 * sizeof(float));
    nrs[is] = t->nrec;
    for (int ir = 0; ir < t->nrec; ir++) {
      float *p = rec + ((size_t)is * maxrec + ir) * 5;
      p[0] = t->rx[ir];
      p[1] = t->ry[ir];
      p[2] = t->rz[ir];
      p[3] = t->raz[ir];
      p[4] = t->rdip[ir];
    }
    if (with_data)
      for (int ic = 0; ic < nch; ic++)
        for (int f = 0; f < nf; f++)
          for (int ir = 0; ir < t->nrec; ir++) {
            const size_t from = ((size_t)ic * nf + f) * t->nrec + ir;
            const size_t to = (((size_t)is * nch + ic) * nf + f) * maxrec + ir;
            dobs[to] = t->dobs[from];
            delta[to] = t->delta[from];
          }
  }
  int *src_ch = malloc(emf->nchsrc * sizeof(int));
  for (int k = 0; k < emf->nchsrc; k++) src_ch[k] = chan_code(emf->chsrc[k]);
  int *rec_ch = malloc(nch * sizeof(int));
  for (int k = 0; k < nch; k++) rec_ch[k] = chan_code(emf->chrec[k]);
  emmi_fg_problem P;
  memset(&P, 0, sizeof(P));
  P.nx = emf->nx;
  P.ny = emf->ny;
  P.nz = emf->nz;
  P.o[0] = emf->ox;
  P.o[1] = emf->oy;
  P.o[2] = emf->oz;
  P.d[0] = emf->dx;
  P.d[1] = emf->dy;
  P.d[2] = emf->dz;
  P.n1 = n1;
  P.n2 = n2;
  P.n3 = n3;
  P.nshot = ns;
  P.nfreq = nf;
  P.omega = emf->omegas;
  P.x1 = ax[0];
  P.x2 = ax[1];
  P.x3 = ax[2];
  P.rho_water = emf->rho_water;
  P.nsrc_ch = emf->nchsrc;
  P.src_ch = src_ch;
  P.nrec_ch = nch;
  P.rec_ch = rec_ch;
  P.nrec = maxrec;
  P.nrec_shot = nrs;
  P.src = src;
  P.rec = rec;
  if (with_data) {
    P.dobs = (const float *)dobs;
    P.delta = delta;
    P.npar = fwi->npar;
    P.idxpar = fwi->idxpar;
    P.preco = fwi->preco;
    P.bathy = &emf->bathy[0][0];
    P.dsmute = emf->dsmute;
    P.drmute = emf->drmute;
  }
  emmi_options opt;
  emmi_dropin_options(&opt, 0);
  if (emmi_fg_create(&c->fg, &P, &opt) != EMMI_OK) die("emmi_fg_create failed: ", emmi_last_error());
  c->fshot = malloc(ns * sizeof(float));
  c->rall = malloc(nper * sizeof(float));
  c->dall = malloc(nper * sizeof(emmi_cf32));
  c->stats = malloc((size_t)2 * ns * nf * sizeof(emmi_rhs_stats));
  for (int k = 0; k < 3; k++) free(ax[k]);
  free(tmp);
  free(src);
  free(rec);
  free(nrs);
  free(dobs);
  free(delta);
  free(src_ch);
  free(rec_ch);
}

/* the data part of fg_fwi for every shot in one device evaluation: the
 * shot-summed gradient into c->gsum (pseudo-Hessian into c->hsum), each
 * shot's syn_ and rmse_ files and misfit line; returns the summed misfit */
static float fg_batch(fg_ctx *c) {
  emmi_emf_t *emf = c->emf;
  const int nf = emf->nfreq, nch = emf->nchrec;
  if (eh_pad_model(c->M, c->pxx, c->pyy, c->pzz, c->pad) != EH_OK) die("eh_pad_model failed", NULL);
  if (emmi_fg_eval(c->fg, c->nxp, c->nyp, c->nzp, c->pxx, c->pyy, c->pzz, c->pad,
                   &emf->rho11[0][0][0], &emf->rho33[0][0][0], c->fshot, c->gsum,
                   c->fwi->preco == 1 ? c->hsum : NULL, (float *)c->dall, c->rall,
                   c->stats) != EMMI_OK)
    die("emmi_fg_eval failed: ", emmi_last_error());
  float fcost_dat = 0;
  float *rm = malloc((size_t)nch * nf * c->maxrec * sizeof(float));
  for (int is = 0; is < c->nshots; is++) {
    const shot_t *t = &c->sh[is];
    if (emf->verb)
      for (int a = 0; a < 2; a++)
        for (int f = 0; f < nf; f++) {
          const emmi_rhs_stats *q = &c->stats[((size_t)a * c->nshots + is) * nf + f];
          printf("shot %d freq %g%s: %d cycles, relative residual %.3e, status %d\n", t->shot,
                 emf->freqs[f], a ? " (adjoint)" : "", q->cycles,
                 q->rnorm0 > 0 ? q->rnorm / q->rnorm0 : 0., q->status);
        }
    for (int ic = 0; ic < nch; ic++)
      for (int f = 0; f < nf; f++)
        for (int ir = 0; ir < t->nrec; ir++) {
          const size_t from = (((size_t)is * nch + ic) * nf + f) * c->maxrec + ir;
          const size_t to = ((size_t)ic * nf + f) * t->nrec + ir;
          c->dc[to] = c->dall[from];
          rm[to] = c->rall[from];
        }
    char fname[64];
    snprintf(fname, sizeof(fname), "syn_%04d.txt", t->shot);
    write_data(fname, t->shot, emf, t->nrec, c->dc);
    write_rmse(emf, t, rm);
    const int ndat = nch * nf * t->nrec;
    if (emf->verb)
      printf("isrc=%d, fcost=%g, rmse=%g\n", t->shot, c->fshot[is], sqrt(2. * c->fshot[is] / ndat));
    fcost_dat += c->fshot[is];
  }
  free(rm);
  return fcost_dat;
}

static void write_floats(const char *name, const float *a, size_t n) {
  FILE *fp = fopen(name, "wb");
  if (!fp) die("cannot write ", name);
  fwrite(a, sizeof(float), n, fp);
  fclose(fp);
}

/* is cell (i2, i3) of the input model at or above the sea floor plus one
 * cell: the regularization leaves those cells alone (src/fg_mod_reg.c:36) */
static int above_floor(const emmi_emf_t *emf, int i1, int i2, int i3) {
  return emf->oz + (i3 + 0.5) * emf->dz < emf->bathy[i2][i1] + emf->dz;
}

/* fg_mod_reg (src/fg_mod_reg.c:19-91): Tikhonov (gamma1) and TV (gamma2)
 * terms of x - xref below the sea floor, cooled by 0.8^iter, added to g */
static void fg_mod_reg(fg_ctx *c, const float *x, float *g) {
  emmi_emf_t *emf = c->emf;
  emmi_fwi_t *fwi = c->fwi;
  const int nxyz = (int)c->nxyz;
  const float beta = pow(0.8, fwi->iter);
  fwi->fcost_mod = 0;
  float *xm = malloc(fwi->n * sizeof(float)), *gm = malloc(fwi->n * sizeof(float));
  for (int k = 0; k < fwi->npar; k++)
    for (int i3 = 0; i3 < emf->nz; i3++)
      for (int i2 = 0; i2 < emf->ny; i2++)
        for (int i1 = 0; i1 < emf->nx; i1++) {
          const int i = i1 + emf->nx * (i2 + emf->ny * (i3 + emf->nz * k));
          xm[i] = above_floor(emf, i1, i2, i3) ? 0 : (x[i] - fwi->xref[i]);
        }
  for (int term = 0; term < 2; term++) {
    const float gam = term == 0 ? fwi->gamma1 : fwi->gamma2;
    if (!(gam > 0)) continue;
    memset(gm, 0, fwi->n * sizeof(float));
    const float gb = gam * beta;
    for (int k = 0; k < fwi->npar; k++) {
      const float cost = term == 0
                             ? ef_tikhonov(xm + (size_t)k * nxyz, gm + (size_t)k * nxyz, emf->nx,
                                           emf->ny, emf->nz)
                             : ef_tv(xm + (size_t)k * nxyz, gm + (size_t)k * nxyz, emf->nx,
                                     emf->ny, emf->nz);
      fwi->fcost_mod += 0.5 * gb * cost;
      for (int i = 0; i < nxyz; i++) g[(size_t)k * nxyz + i] += 0.5 * gb * gm[(size_t)k * nxyz + i];
    }
    if (emf->verb) { /* the reference's names: the first parameter's part is "Rh" here */
      write_floats(term == 0 ? "gradient_tikhonov_Rh" : "gradient_tv_Rh", gm, nxyz);
      if (fwi->npar > 1)
        write_floats(term == 0 ? "gradient_tikhonov_Rv" : "gradient_tv_Rv", gm + nxyz, nxyz);
    }
  }
  free(xm);
  free(gm);
}

/* fg_fwi (src/fg_fwi.c:139-290): misfit and gradient at the logarithmic
 * parameters xx, summed over the shots, regularized, scaled */
static float fg_eval(void *ctx, float *xx, float *g) {
  fg_ctx *c = ctx;
  emmi_emf_t *emf = c->emf;
  emmi_fwi_t *fwi = c->fwi;
  const size_t nxyz = c->nxyz;
  emf->rhomin = emf->rhomax = exp(xx[0]);
  for (int j = 0; j < fwi->npar; j++)
    for (size_t i = 0; i < nxyz; i++) {
      const float s = exp(xx[j * nxyz + i]);
      if (fwi->idxpar[j] == 1) {
        (&emf->rho11[0][0][0])[i] = s;
        (&emf->rho22[0][0][0])[i] = s;
      }
      if (fwi->idxpar[j] == 2) (&emf->rho33[0][0][0])[i] = s;
      if (s < emf->rhomin) emf->rhomin = s;
      if (s > emf->rhomax) emf->rhomax = s;
    }
  if (emf->verb) printf("fg_fwi iter=%d: [rhomin,rhomax]=[%g,%g]\n", fwi->iter, emf->rhomin,
                        emf->rhomax);
  memset(c->gsum, 0, fwi->n * sizeof(float));
  memset(c->hsum, 0, fwi->n * sizeof(float));
  float fcost_dat = 0;
  if (c->fg) {
    fcost_dat = fg_batch(c);
  } else {
    for (int is = 0; is < c->nshots; is++) {
      set_shot(c, &c->sh[is]);
      fcost_dat += gradient_shot(c, &c->sh[is]);
      for (long i = 0; i < fwi->n; i++) {
        c->gsum[i] += (&fwi->grad[0][0][0][0])[i];
        if (fwi->preco == 1) c->hsum[i] += (&fwi->phess[0][0][0][0])[i];
      }
    }
  }
  /* the shot sums (the reference's MPI_Allreduce, src/fg_fwi.c:262-268) */
  if (fwi->preco == 1) memcpy(&fwi->phess[0][0][0][0], c->hsum, fwi->n * sizeof(float));
  memcpy(g, c->gsum, fwi->n * sizeof(float));
  fwi->fcost_dat = fcost_dat;
  fwi->mse = sqrt(2. * fcost_dat / c->ndata);
  if (emf->verb) {
    printf("fcost_dat=%g, rmse=%g\n", fcost_dat, fwi->mse);
    /* the summed data gradient before regularization (src/fg_fwi.c:276-283) */
    write_floats("gradient_dat_Rv", g, nxyz);
    if (fwi->npar > 1) write_floats("gradient_dat_Rh", g + nxyz, nxyz);
    if (fwi->preco == 1) write_floats("gradient_phess", c->hsum, fwi->n);
  }
  fg_mod_reg(c, xx, g);
  fwi->fcost = fwi->fcost_dat + fwi->fcost_mod;
  if (emf->verb) {
    printf("fcost_dat=%g\n", fwi->fcost_dat);
    printf("fcost_mod=%g\n", fwi->fcost_mod);
    printf("fcost=%g\n", fwi->fcost);
  }
  /* l-BFGS is not scale invariant: the first gradient of the inversion sets
   * a scale for the objective (src/fg_fwi.c:294-307) */
  if (emf->mode == 1 && fwi->firstgrad) {
    float s1 = 0, s2 = 0;
    for (long k = 0; k < fwi->n; k++) {
      s1 += fabs(xx[k]);
      s2 += fabs(g[k]);
    }
    fwi->alpha = 2e-3 * s1 / s2;
    if (emf->verb) printf("|x|_1=%g, |g|_1=%g, scaling=%g\n", s1, s2, fwi->alpha);
  }
  for (long k = 0; k < fwi->n; k++) g[k] *= fwi->alpha;
  if (fwi->firstgrad) fwi->firstgrad = 0;
  return fwi->fcost * fwi->alpha;
}

/* precondition (src/precondition.c:16-85): 1 = divide by the pseudo-Hessian
 * (regularized by 1e-5 of its largest value below the sea floor) and
 * rescale to the input norm; 2 = depth weighting exp(depth / skin depth at
 * 1 ohm-m); 3 = triangle smoothing */
static void precondition(fg_ctx *c, float *g) {
  emmi_emf_t *emf = c->emf;
  emmi_fwi_t *fwi = c->fwi;
  const int nx = emf->nx, ny = emf->ny, nz = emf->nz;
  if (fwi->preco == 1) {
    float s1 = 0., s2 = 0., z;
    for (int k = 0; k < fwi->npar; k++) {
      z = 0;
      for (int i3 = 0; i3 < nz; i3++)
        for (int i2 = 0; i2 < ny; i2++)
          for (int i1 = 0; i1 < nx; i1++)
            if (emf->oz + (i3 + 0.5) * emf->dz > emf->bathy[i2][i1] &&
                fwi->phess[k][i3][i2][i1] > z)
              z = fwi->phess[k][i3][i2][i1];
      for (int i3 = 0; i3 < nz; i3++)
        for (int i2 = 0; i2 < ny; i2++)
          for (int i1 = 0; i1 < nx; i1++) {
            const int i = i1 + nx * (i2 + ny * (i3 + nz * k));
            s1 += g[i] * g[i];
            g[i] /= (fwi->phess[k][i3][i2][i1] + 1e-5 * z);
            s2 += g[i] * g[i];
          }
    }
    z = sqrt(s1 / s2);
    for (long i = 0; i < fwi->n; i++) g[i] *= z;
  } else if (fwi->preco == 2) {
    const float skin = sqrt(2. / (emf->omegas[0] * 4e-7 * PI_REF));
    for (int k = 0; k < fwi->npar; k++)
      for (int i3 = 0; i3 < nz; i3++)
        for (int i2 = 0; i2 < ny; i2++)
          for (int i1 = 0; i1 < nx; i1++) {
            const int i = i1 + nx * (i2 + ny * (i3 + nz * k));
            float z = emf->oz + (i3 + 0.5) * emf->dz;
            if (z > emf->bathy[i2][i1]) {
              z -= emf->bathy[i2][i1];
              g[i] *= exp(z / skin);
            }
          }
  } else if (fwi->preco == 3) {
    for (int k = 0; k < fwi->npar; k++)
      ef_triangle_smoothing(g + (size_t)k * c->nxyz, nx, ny, nz, fwi->r1, fwi->r2, fwi->r3,
                            fwi->repeat);
  }
}

/* do_fwi (src/do_fwi.c:42-231) with l-BFGS (method=0): the inversion loop,
 * iterate.txt, rmse_misfit.txt and the models of every iteration */
static void do_fwi(fg_ctx *c) {
  emmi_emf_t *emf = c->emf;
  emmi_fwi_t *fwi = c->fwi;
  const size_t nxyz = c->nxyz;
  ef_opt o;
  memset(&o, 0, sizeof(o));
  if (!getparint("niter", &o.niter)) o.niter = 30;
  if (!getparint("nls", &o.nls)) o.nls = 5;
  if (!getparfloat("tol", &o.tol)) o.tol = 1e-6;
  if (!getparint("npair", &o.npair)) o.npair = 5;
  if (!getparfloat("c1", &o.c1)) o.c1 = 1e-4;
  if (!getparfloat("c2", &o.c2)) o.c2 = 0.9;
  if (!getparfloat("alpha", &o.alpha)) o.alpha = 1.;
  if (!getparint("bound", &o.bound)) o.bound = 0;
  if (!getparint("method", &o.method)) o.method = 0;
  if (!getparint("ncg", &o.ncg)) o.ncg = 5;
  o.preco = fwi->preco;
  o.verb = emf->verb;
  if (o.method != 0)
    die("method=1 (Gauss-Newton) needs a Hessian-vector product; the reference's is empty "
        "(src/fg_fwi.c:316-320): use method=0", NULL);
  const int n = fwi->n;
  if (o.bound) {
    if (countparval("minpar") != fwi->npar || countparval("maxpar") != fwi->npar)
      die("bound=1 needs minpar= and maxpar= of length npar", NULL);
    fwi->minpar = malloc(fwi->npar * sizeof(float));
    fwi->maxpar = malloc(fwi->npar * sizeof(float));
    getparfloat("minpar", fwi->minpar);
    getparfloat("maxpar", fwi->maxpar);
  }
  o.x = malloc(n * sizeof(float));
  o.g = malloc(n * sizeof(float));
  o.d = calloc(n, sizeof(float));
  o.q = malloc(n * sizeof(float));
  o.sk = malloc(o.npair * sizeof(float *));
  o.yk = malloc(o.npair * sizeof(float *));
  for (int k = 0; k < o.npair; k++) {
    o.sk[k] = malloc(n * sizeof(float));
    o.yk[k] = malloc(n * sizeof(float));
  }
  o.rho = malloc(o.npair * sizeof(float));
  o.alp = malloc(o.npair * sizeof(float));
  /* x = log of the inverted resistivities (src/do_fwi.c:113-124) */
  for (int j = 0; j < fwi->npar; j++)
    for (size_t i = 0; i < nxyz; i++) {
      if (fwi->idxpar[j] == 1) o.x[j * nxyz + i] = log((&emf->rho11[0][0][0])[i]);
      if (fwi->idxpar[j] == 2) o.x[j * nxyz + i] = log((&emf->rho33[0][0][0])[i]);
    }
  memcpy(fwi->xref, o.x, n * sizeof(float));
  if (o.bound) { /* bounds below the sea floor, the input elsewhere (do_fwi.c:126-146) */
    o.xmin = malloc(n * sizeof(float));
    o.xmax = malloc(n * sizeof(float));
    for (int j = 0; j < fwi->npar; j++)
      for (int i3 = 0; i3 < emf->nz; i3++)
        for (int i2 = 0; i2 < emf->ny; i2++)
          for (int i1 = 0; i1 < emf->nx; i1++) {
            const int i = i1 + emf->nx * (i2 + emf->ny * (i3 + emf->nz * j));
            if (emf->oz + (i3 + 0.5) * emf->dz > emf->bathy[i2][i1] + emf->dz) {
              o.xmin[i] = log(fwi->minpar[j]);
              o.xmax[i] = log(fwi->maxpar[j]);
            } else {
              o.xmin[i] = o.x[i];
              o.xmax[i] = o.x[i];
            }
          }
  }
  float fcost = fg_eval(c, o.x, o.g);
  o.f0 = o.fk = fcost;
  FILE *fp;
  if (o.verb) {
    o.gk_norm = ef_l2norm(n, o.g);
    fp = fopen("iterate.txt", "w");
    if (!fp) die("cannot write iterate.txt", NULL);
    fprintf(fp, "==========================================================\n");
    fprintf(fp, "l-BFGS memory length: %d\n", o.npair);
    fprintf(fp, "Maximum number of iterations: %d\n", o.niter);
    fprintf(fp, "Convergence tolerance: %3.2e\n", o.tol);
    fprintf(fp, "maximum number of line search: %d\n", o.nls);
    fprintf(fp, "initial step length: alpha=%g\n", o.alpha);
    fprintf(fp, "==========================================================\n");
    fprintf(fp, "iter    fk       fk/f0      ||gk||    alpha     nls   ngrad\n");
    fclose(fp);
  }
  for (o.iter = 0; o.iter < o.niter; o.iter++) {
    fwi->iter = o.iter;
    if (o.verb) {
      printf("==========================================================\n");
      printf("# iter=%d  fk/f0=%g\n", o.iter, o.fk / o.f0);
      o.gk_norm = ef_l2norm(n, o.g);
      fp = fopen("iterate.txt", "a");
      fprintf(fp, "%3d   %3.2e  %3.2e   %3.2e  %3.2e  %3d  %4d\n", o.iter, o.fk, o.fk / o.f0,
              o.gk_norm, o.alpha, o.ils, o.igrad);
      fclose(fp);
      fp = fopen("rmse_misfit.txt", o.iter == 0 ? "w" : "a");
      fprintf(fp, "%d \t %g\n", fwi->iter, fwi->mse);
      fclose(fp);
    }
    memcpy(o.q, o.g, n * sizeof(float));
    if (o.iter == 0) {
      if (o.preco) precondition(c, o.q);
      ef_flipsign(n, o.q, o.d);
    } else {
      ef_lbfgs_update(n, o.x, o.g, &o);
      if (o.preco) {
        /* as the reference: without a usable pair the previous direction
         * stays (src/do_fwi.c:193-197) */
        ef_lbfgs_descent1(n, o.g, &o);
        precondition(c, o.q);
        if (o.loop1) ef_lbfgs_descent2(n, &o);
      } else {
        ef_lbfgs_descent(n, o.g, o.d, &o);
      }
    }
    ef_lbfgs_save(n, o.x, o.g, &o);
    ef_line_search(n, o.x, o.g, o.d, fg_eval, c, &o);
    if (o.verb) {
      char fname[32];
      snprintf(fname, sizeof(fname), "Rv_iteration_%02d", o.iter);
      write_floats(fname, &emf->rho33[0][0][0], nxyz);
      snprintf(fname, sizeof(fname), "Rh_iteration_%02d", o.iter);
      write_floats(fname, &emf->rho11[0][0][0], nxyz);
    }
  }
  if (o.verb && o.iter == o.niter) {
    fp = fopen("iterate.txt", "a");
    fprintf(fp, "==>Maximum iteration number reached!\n");
    fclose(fp);
  }
}

int main(int argc, char **argv) {
  initargs(argc, argv);
  emmi_emf_t emf;
  emmi_acq_t acq;
  memset(&emf, 0, sizeof(emf));
  memset(&acq, 0, sizeof(acq));
  if (!getparint("mode", &emf.mode)) emf.mode = 0;
  if (emf.mode < 0 || emf.mode > 2) die("mode must be 0 (modelling), 1 (inversion) or 2 (gradient)", NULL);
  if (!getparint("verb", &emf.verb)) emf.verb = 1;
  if (emf.mode == 1) { /* checked before any work: do_fwi.c:63 */
    int method = 0;
    getparint("method", &method);
    if (method != 0)
      die("method=1 (Gauss-Newton) needs a Hessian-vector product; the reference's is empty "
          "(src/fg_fwi.c:316-320): use method=0", NULL);
  }
  /* ---- emf_init (src/emf_init_free.c:12-128) ---- */
  if (!(emf.nfreq = countparval("freqs"))) die("Need freqs= vector", NULL);
  emf.freqs = malloc(emf.nfreq * sizeof(float));
  emf.omegas = malloc(emf.nfreq * sizeof(float));
  getparfloat("freqs", emf.freqs);
  for (int f = 0; f < emf.nfreq; f++) emf.omegas[f] = 2. * PI_REF * emf.freqs[f];
  static char *defch[] = {"Ex"};
  if ((emf.nchsrc = countparval("chsrc"))) {
    emf.chsrc = malloc(emf.nchsrc * sizeof(char *));
    getparstringarray("chsrc", emf.chsrc);
  } else {
    emf.nchsrc = 1;
    emf.chsrc = defch;
  }
  if ((emf.nchrec = countparval("chrec"))) {
    emf.chrec = malloc(emf.nchrec * sizeof(char *));
    getparstringarray("chrec", emf.chrec);
  } else {
    emf.nchrec = 1;
    emf.chrec = defch;
  }
  if (!getparint("nx", &emf.nx)) die("Need nx=", NULL);
  if (!getparint("ny", &emf.ny)) die("Need ny=", NULL);
  if (!getparint("nz", &emf.nz)) die("Need nz=", NULL);
  if (!getparfloat("dx", &emf.dx)) die("Need dx=", NULL);
  if (!getparfloat("dy", &emf.dy)) die("Need dy=", NULL);
  if (!getparfloat("dz", &emf.dz)) die("Need dz=", NULL);
  if (!getparfloat("ox", &emf.ox)) die("Need ox=", NULL);
  if (!getparfloat("oy", &emf.oy)) die("Need oy=", NULL);
  if (!getparfloat("oz", &emf.oz)) emf.oz = 0;
  if (!getparfloat("d1min", &emf.d1min)) emf.d1min = 100;
  if (!getparfloat("d2min", &emf.d2min)) emf.d2min = 100;
  if (!getparfloat("d3min", &emf.d3min)) emf.d3min = 20;
  if (!getparint("n1", &emf.n1)) emf.n1 = 128;
  if (!getparint("n2", &emf.n2)) emf.n2 = 128;
  if (!getparint("n3", &emf.n3)) emf.n3 = 128;
  char *f11, *f22, *f33;
  if (!getparstring("frho11", &f11)) die("Need frho11=", NULL);
  if (!getparstring("frho22", &f22)) die("Need frho22=", NULL);
  if (!getparstring("frho33", &f33)) die("Need frho33=", NULL);
  const size_t nxyz = (size_t)emf.nx * emf.ny * emf.nz;
  float *r11 = read_floats(f11, nxyz), *r22 = read_floats(f22, nxyz), *r33 = read_floats(f33, nxyz);
  emf.rho11 = (float ***)table3(r11, sizeof(float), emf.nx, emf.ny, emf.nz);
  emf.rho22 = (float ***)table3(r22, sizeof(float), emf.nx, emf.ny, emf.nz);
  emf.rho33 = (float ***)table3(r33, sizeof(float), emf.nx, emf.ny, emf.nz);
  if (!getparfloat("lextend", &emf.lextend)) emf.lextend = 50e3;
  if (!getparfloat("rho_air", &emf.rho_air)) emf.rho_air = 1e8;
  if (!getparint("nb", &emf.nb)) emf.nb = 10;
  eh_model M = {emf.nx, emf.ny, emf.nz, emf.dx, emf.dy, emf.dz, emf.ox, emf.oy, emf.oz,
                r11, r22, r33, emf.nb, emf.lextend, emf.rho_air, emf.d1min, emf.d2min,
                emf.d3min, emf.n1, emf.n2, emf.n3};
  emf.rho_water = eh_rho_water(&M);
  /* mesh arrays of the current shot (regrid_init), reused shot after shot */
  const int n1 = emf.n1, n2 = emf.n2, n3 = emf.n3;
  float **arr[12] = {&emf.x1, &emf.x2, &emf.x3, &emf.x1s, &emf.x2s, &emf.x3s,
                     &emf.d1, &emf.d2, &emf.d3, &emf.d1s, &emf.d2s, &emf.d3s};
  const int len[12] = {n1, n2, n3, n1, n2, n3, n1, n2, n3, n1, n2, n3};
  for (int i = 0; i < 12; i++) *arr[i] = malloc((len[i] + 1) * sizeof(float));
  const size_t nc = (size_t)n1 * n2 * n3;
  fg_ctx c;
  memset(&c, 0, sizeof(c));
  c.s11 = malloc(nc * sizeof(float));
  c.s22 = malloc(nc * sizeof(float));
  c.s33 = malloc(nc * sizeof(float));
  c.imu = malloc(nc * sizeof(float));
  emf.sigma11 = (float ***)table3(c.s11, sizeof(float), n1, n2, n3);
  emf.sigma22 = (float ***)table3(c.s22, sizeof(float), n1, n2, n3);
  emf.sigma33 = (float ***)table3(c.s33, sizeof(float), n1, n2, n3);
  emf.invmur = (float ***)table3(c.imu, sizeof(float), n1, n2, n3);
  /* ---- acquisition (src/acq_init_free.c): the shots of this run ---- */
  char *fsrc, *frec, *fsrcrec;
  if (!getparstring("fsrc", &fsrc)) die("Need fsrc=", NULL);
  if (!getparstring("frec", &frec)) die("Need frec=", NULL);
  if (!getparstring("fsrcrec", &fsrcrec)) die("Need fsrcrec=", NULL);
  int nsrc_all, nrec_all;
  point_t *S = read_points(fsrc, &nsrc_all);
  point_t *R = read_points(frec, &nrec_all);
  int nshots = countparval("shots");
  int *shots = malloc((nshots ? nshots : 1) * sizeof(int));
  if (nshots) {
    char *list[4096];
    nshots = getparstringarray("shots", list);
    for (int i = 0; i < nshots; i++) shots[i] = atoi(list[i]);
  } else {
    nshots = 1;
    shots[0] = 1;
  }
  shot_t *sh = calloc(nshots, sizeof(shot_t));
  for (int is = 0; is < nshots; is++) {
    shot_t *t = &sh[is];
    t->shot = shots[is];
    if (t->shot < 1 || t->shot > nsrc_all) die("shot index out of range", NULL);
    /* receivers of this shot from the source-receiver table */
    FILE *fp = fopen(fsrcrec, "r");
    if (!fp) die("cannot open ", fsrcrec);
    if (fscanf(fp, "%*[^\n]\n") < 0) die("empty file ", fsrcrec);
    int a, b2, cap = 1024;
    int *ridx = malloc(cap * sizeof(int));
    while (fscanf(fp, "%d %d", &a, &b2) == 2)
      if (a == t->shot) {
        if (t->nrec == cap) ridx = realloc(ridx, (cap *= 2) * sizeof(int));
        ridx[t->nrec++] = b2;
      }
    fclose(fp);
    const point_t ps = S[t->shot - 1];
    t->src5[0] = ps.x;
    t->src5[1] = ps.y;
    t->src5[2] = ps.z;
    t->src5[3] = (float)(PI_REF * ps.hd / 180.);
    t->src5[4] = (float)(PI_REF * ps.pit / 180.);
    const int nr = t->nrec ? t->nrec : 1;
    t->rx = malloc(nr * sizeof(float));
    t->ry = malloc(nr * sizeof(float));
    t->rz = malloc(nr * sizeof(float));
    t->raz = malloc(nr * sizeof(float));
    t->rdip = malloc(nr * sizeof(float));
    for (int i = 0; i < t->nrec; i++) {
      const point_t p = R[ridx[i] - 1];
      t->rx[i] = p.x;
      t->ry[i] = p.y;
      t->rz[i] = p.z;
      t->raz[i] = PI_REF * p.hd / 180.;
      t->rdip[i] = PI_REF * p.pit / 180.;
    }
    free(ridx);
  }
  const long n3s = 3L * (n1 + 1) * (n2 + 1) * (n3 + 1);
  c.emf = &emf;
  c.acq = &acq;
  c.M = &M;
  c.sh = sh;
  c.nshots = nshots;
  c.x = malloc(n3s * sizeof(double complex));
  c.b = malloc(n3s * sizeof(double complex));
  c.n3s = n3s;
  c.nxyz = nxyz;
  int maxrec = 1;
  for (int is = 0; is < nshots; is++)
    if (sh[is].nrec > maxrec) maxrec = sh[is].nrec;
  c.dc = calloc((size_t)emf.nchrec * emf.nfreq * maxrec, sizeof(emmi_cf32));

  /* batch=1 (default): all shots and frequencies in one device solver;
   * batch=0: shot by shot through the drop-in entry points */
  int batch = 1;
  getparint("batch", &batch);
  if (emf.mode == 0 && batch) {
    /* ---- do_modelling (src/do_modelling.c:49-67) for every shot at once ---- */
    fg_batch_init(&c, 0);
    const int nf = emf.nfreq, nch = emf.nchrec;
    const size_t nper = (size_t)nshots * nch * nf * c.maxrec;
    emmi_cf32 *dall = malloc(nper * sizeof(emmi_cf32));
    emmi_rhs_stats *st = malloc((size_t)nshots * nf * sizeof(emmi_rhs_stats));
    if (emmi_fg_forward(c.fg, c.nxp, c.nyp, c.nzp, c.pxx, c.pyy, c.pzz, c.pad, (float *)dall,
                        st) != EMMI_OK)
      die("emmi_fg_forward failed: ", emmi_last_error());
    for (int is = 0; is < nshots; is++) {
      shot_t *t = &sh[is];
      for (int ic = 0; ic < nch; ic++)
        for (int f = 0; f < nf; f++) {
          if (emf.verb && ic == 0) {
            const emmi_rhs_stats *q = &st[(size_t)is * nf + f];
            printf("shot %d freq %g: %d cycles, relative residual %.3e, status %d\n", t->shot,
                   emf.freqs[f], q->cycles, q->rnorm0 > 0 ? q->rnorm / q->rnorm0 : 0., q->status);
          }
          for (int ir = 0; ir < t->nrec; ir++)
            c.dc[((size_t)ic * nf + f) * t->nrec + ir] =
                dall[(((size_t)is * nch + ic) * nf + f) * c.maxrec + ir];
        }
      char fname[64];
      snprintf(fname, sizeof(fname), "emf_%04d.txt", t->shot);
      write_data(fname, t->shot, &emf, t->nrec, c.dc);
    }
    free(dall);
    free(st);
    emmi_fg_destroy(c.fg);
    return 0;
  }
  if (emf.mode == 0) {
    /* ---- do_modelling frequency loop (src/do_modelling.c:49-67) ---- */
    for (int is = 0; is < nshots; is++) {
      shot_t *t = &sh[is];
      set_shot(&c, t);
      const int nr = t->nrec ? t->nrec : 1;
      memset(c.dc, 0, (size_t)emf.nchrec * emf.nfreq * nr * sizeof(emmi_cf32));
      emf.dcal_fd = (emmi_cf32 ***)table3(c.dc, sizeof(emmi_cf32), nr, emf.nfreq, emf.nchrec);
      model_all(&emf, &acq, c.x, c.b, n3s, t->shot, 0);
      char fname[64];
      snprintf(fname, sizeof(fname), "emf_%04d.txt", t->shot);
      write_data(fname, t->shot, &emf, t->nrec, c.dc);
      free(emf.dcal_fd[0]);
      free(emf.dcal_fd);
    }
    return 0;
  }

  /* ---- fg_fwi_init (src/fg_fwi.c:42-135) and do_fwi parameters ---- */
  emmi_fwi_t fwi;
  memset(&fwi, 0, sizeof(fwi));
  c.fwi = &fwi;
  char *fbathy;
  if (!getparstring("fbathy", &fbathy)) die("Need fbathy= for CSEM inversion", NULL);
  if (!getparint("addnoise", &emf.addnoise)) emf.addnoise = 1;
  if (!getparfloat("amp_perc", &emf.amp_perc)) emf.amp_perc = 0.03;
  if (!getparfloat("delta_phi", &emf.delta_phi)) emf.delta_phi = 0;
  if (!getparfloat("delta_theta", &emf.delta_theta)) emf.delta_theta = 0;
  if (!getparfloat("noisefloorE", &emf.noisefloorE)) emf.noisefloorE = 1e-15;
  if (!getparfloat("noisefloorH", &emf.noisefloorH)) emf.noisefloorH = 1e-13;
  if (!getparfloat("dsmute", &emf.dsmute)) emf.dsmute = 800;
  if (!getparfloat("drmute", &emf.drmute)) emf.drmute = 200;
  if (!getparfloat("gamma1", &fwi.gamma1)) fwi.gamma1 = 10.;
  if (!getparfloat("gamma2", &fwi.gamma2)) fwi.gamma2 = 0.;
  if (!getparint("r1", &fwi.r1)) fwi.r1 = 3;
  if (!getparint("r2", &fwi.r2)) fwi.r2 = 3;
  if (!getparint("r3", &fwi.r3)) fwi.r3 = 1;
  if (!getparint("repeat", &fwi.repeat)) fwi.repeat = 1;
  int seed = 1;
  getparint("seed", &seed);
  rng_state = (unsigned long long)seed;
  if (!getparint("npar", &fwi.npar)) fwi.npar = 2;
  fwi.idxpar = malloc(fwi.npar * sizeof(int));
  for (int j = 0; j < fwi.npar; j++) fwi.idxpar[j] = j + 1;
  getparint("idxpar", fwi.idxpar);
  if (!getparint("preco", &fwi.preco)) fwi.preco = 1;
  float *bathy = read_floats(fbathy, (size_t)emf.nx * emf.ny);
  emf.bathy = malloc(emf.ny * sizeof(float *));
  for (int j = 0; j < emf.ny; j++) emf.bathy[j] = bathy + (size_t)j * emf.nx;
  fwi.n = (int)(nxyz * fwi.npar);
  fwi.xref = malloc((size_t)fwi.n * sizeof(float));
  fwi.alpha = 1;
  fwi.firstgrad = 1;
  float *gr = malloc((size_t)fwi.n * sizeof(float)), *ph = malloc((size_t)fwi.n * sizeof(float));
  fwi.grad = (float ****)table4(gr, sizeof(float), emf.nx, emf.ny, emf.nz, fwi.npar);
  fwi.phess = (float ****)table4(ph, sizeof(float), emf.nx, emf.ny, emf.nz, fwi.npar);
  c.gsum = calloc((size_t)fwi.n, sizeof(float));
  c.hsum = calloc((size_t)fwi.n, sizeof(float));
  c.Ef = malloc(3 * nxyz * emf.nfreq * sizeof(emmi_cf32));
  c.Ea = malloc(3 * nxyz * emf.nfreq * sizeof(emmi_cf32));
  int *chc = malloc(emf.nchrec * sizeof(int));
  for (int k = 0; k < emf.nchrec; k++) chc[k] = chan_code(emf.chrec[k]);
  c.chc = chc;
  /* observed data (emf_%04d.txt), uncertainties and noise, once per shot;
   * obs_%04d.txt (src/fg_fwi.c:105-114) */
  for (int is = 0; is < nshots; is++) {
    shot_t *t = &sh[is];
    const size_t nd = (size_t)emf.nchrec * emf.nfreq * (t->nrec ? t->nrec : 1);
    t->dobs = calloc(nd, sizeof(emmi_cf32));
    t->delta = calloc(nd, sizeof(float));
    read_data(t->shot, &emf, t->nrec, t->dobs);
    eh_uncertainty(emf.nchrec, chc, emf.nfreq, t->nrec, t->raz, t->src5[3],
                   (const float *)t->dobs, emf.amp_perc, emf.delta_phi, emf.noisefloorE,
                   emf.noisefloorH, t->delta);
    if (emf.addnoise)
      for (size_t i = 0; i < nd; i++) t->dobs[i] += t->delta[i] * gauss_c();
    char fname[64];
    snprintf(fname, sizeof(fname), "obs_%04d.txt", t->shot);
    write_data(fname, t->shot, &emf, t->nrec, t->dobs);
    c.ndata += emf.nchrec * emf.nfreq * t->nrec;
  }
  if (batch) fg_batch_init(&c, 1);
  if (emf.mode == 2) {
    /* one misfit and gradient at the input model (x = log rho, do_fwi.c:113-124) */
    float *xx = malloc((size_t)fwi.n * sizeof(float)), *g = malloc((size_t)fwi.n * sizeof(float));
    for (int j = 0; j < fwi.npar; j++)
      for (size_t i = 0; i < nxyz; i++) {
        if (fwi.idxpar[j] == 1) xx[j * nxyz + i] = log(r11[i]);
        if (fwi.idxpar[j] == 2) xx[j * nxyz + i] = log(r33[i]);
      }
    memcpy(fwi.xref, xx, (size_t)fwi.n * sizeof(float));
    fg_eval(&c, xx, g);
  } else {
    do_fwi(&c);
  }
  if (c.fg) emmi_fg_destroy(c.fg);
  return 0;
}

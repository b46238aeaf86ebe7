/* emmi_main: the reference's command line on the GB300 hot path.
 *
 *   emmi_main mode=0 freqs=1 chsrc=Ex chrec=Ex,Ey,Hx,Hy nx=.. ny=.. nz=..
 *             dx=.. dy=.. dz=.. ox=.. oy=.. [oz=0] [n1=n2=n3=128]
 *             frho11=.. frho22=.. frho33=.. fsrc=.. frec=.. fsrcrec=..
 *             [shots=1,2,..] [cycleopt ncycle v1 v2 tol isemicoarsen]
 *             [gmg_precision=1] [verb=1]
 *   emmi_main mode=2 ... fbathy=.. [npar=2 idxpar=1,2 preco=1 addnoise=1
 *             amp_perc=0.03 delta_phi=0 noisefloorE=1e-15 noisefloorH=1e-13
 *             dsmute=800 drmute=200]
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
 * first holds parameter idxpar[0], the second idxpar[1]).  Both call the
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
    if (emf->mode == 2) extract_electric_field(acq, emf, (emmi_cf64 *)x, f);
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

/* one shot of the gradient mode (src/fg_fwi.c:183-268): returns its misfit
 * and leaves its data gradient in fwi->grad (fwi->phess with preco=1) */
static float gradient_shot(emmi_emf_t *emf, emmi_acq_t *acq, emmi_fwi_t *fwi, double complex *x,
                           double complex *b, long n3s, int shot, int nrec, emmi_cf32 *dcal,
                           const int *chc, emmi_cf32 *Ef, emmi_cf32 *Ea, size_t nxyz) {
  const size_t nd = (size_t)emf->nchrec * emf->nfreq * (nrec ? nrec : 1);
  emmi_cf32 *dobs = calloc(nd, sizeof(emmi_cf32)), *dres = calloc(nd, sizeof(emmi_cf32));
  float *delta = calloc(nd, sizeof(float)), *rmse = calloc(nd, sizeof(float));
  const int nr = nrec ? nrec : 1;
  emf->dobs_fd = (emmi_cf32 ***)table3(dobs, sizeof(emmi_cf32), nr, emf->nfreq, emf->nchrec);
  emf->dres_fd = (emmi_cf32 ***)table3(dres, sizeof(emmi_cf32), nr, emf->nfreq, emf->nchrec);
  emf->delta_emf = (float ***)table3(delta, sizeof(float), nr, emf->nfreq, emf->nchrec);
  emf->rmse = (float ***)table3(rmse, sizeof(float), nr, emf->nfreq, emf->nchrec);
  /* observed data, their uncertainties (and noise), obs_%04d.txt */
  read_data(shot, emf, nrec, dobs);
  eh_uncertainty(emf->nchrec, chc, emf->nfreq, nrec, acq->rec_azimuth, acq->src_azimuth[0],
                 (const float *)dobs, emf->amp_perc, emf->delta_phi, emf->noisefloorE,
                 emf->noisefloorH, delta);
  if (emf->addnoise)
    for (size_t i = 0; i < nd; i++) dobs[i] += delta[i] * gauss_c();
  char fname[64];
  snprintf(fname, sizeof(fname), "obs_%04d.txt", shot);
  write_data(fname, shot, emf, nrec, dobs);
  /* forward modelling */
  const int nx = emf->nx, ny = emf->ny, nz = emf->nz, nf = emf->nfreq;
  const size_t nfe = nxyz * nf;
  emmi_cf32 ****E1f = (emmi_cf32 ****)table4(Ef, sizeof(emmi_cf32), nx, ny, nz, nf);
  emmi_cf32 ****E2f = (emmi_cf32 ****)table4(Ef + nfe, sizeof(emmi_cf32), nx, ny, nz, nf);
  emmi_cf32 ****E3f = (emmi_cf32 ****)table4(Ef + 2 * nfe, sizeof(emmi_cf32), nx, ny, nz, nf);
  emmi_cf32 ****E1a = (emmi_cf32 ****)table4(Ea, sizeof(emmi_cf32), nx, ny, nz, nf);
  emmi_cf32 ****E2a = (emmi_cf32 ****)table4(Ea + nfe, sizeof(emmi_cf32), nx, ny, nz, nf);
  emmi_cf32 ****E3a = (emmi_cf32 ****)table4(Ea + 2 * nfe, sizeof(emmi_cf32), nx, ny, nz, nf);
  emf->E1 = E1f;
  emf->E2 = E2f;
  emf->E3 = E3f;
  model_all(emf, acq, x, b, n3s, shot, 0);
  snprintf(fname, sizeof(fname), "syn_%04d.txt", shot);
  write_data(fname, shot, emf, nrec, dcal);
  /* misfit and adjoint sources, rmse_%04d.txt (write_rmse,
   * src/read_write_data.c:80-102) */
  const float fcost = eh_misfit(emf->nchrec, nf, nrec, emf->omegas, emf->rho_water,
                                acq->src_x1[0], acq->src_x2[0], acq->rec_x1, acq->rec_x2,
                                (const float *)dobs, (const float *)dcal, delta, (float *)dres,
                                rmse);
  snprintf(fname, sizeof(fname), "rmse_%04d.txt", shot);
  FILE *fp = fopen(fname, "w");
  if (!fp) die("cannot write ", fname);
  fprintf(fp, "iTx iRx chrec frequency/Hz RMSE x y z\n");
  for (int ic = 0; ic < emf->nchrec; ic++)
    for (int f = 0; f < nf; f++)
      for (int ir = 0; ir < nrec; ir++)
        fprintf(fp, "%d %d %s %g %e %g %g %g\n", shot, ir + 1, emf->chrec[ic], emf->freqs[f],
                rmse[((size_t)ic * nf + f) * nrec + ir], acq->rec_x1[ir], acq->rec_x2[ir],
                acq->rec_x3[ir]);
  fclose(fp);
  const int ndat = emf->nchrec * nf * nrec;
  if (emf->verb) printf("isrc=%d, fcost=%g, rmse=%g\n", shot, fcost, sqrt(2. * fcost / ndat));
  /* adjoint modelling and the gradient */
  emf->E1 = E1a;
  emf->E2 = E2a;
  emf->E3 = E3a;
  model_all(emf, acq, x, b, n3s, shot, 1);
  build_gradient(acq, emf, fwi, E1f, E2f, E3f, E1a, E2a, E3a);
  void ****t[6] = {(void ****)E1f, (void ****)E2f, (void ****)E3f,
                   (void ****)E1a, (void ****)E2a, (void ****)E3a};
  for (int k = 0; k < 6; k++) {
    for (int l = 0; l < nf; l++) {
      free(t[k][l][0]);
      free(t[k][l]);
    }
    free(t[k]);
  }
  free(dobs); free(dres); free(delta); free(rmse);
  return fcost;
}

int main(int argc, char **argv) {
  initargs(argc, argv);
  emmi_emf_t emf;
  emmi_acq_t acq;
  memset(&emf, 0, sizeof(emf));
  memset(&acq, 0, sizeof(acq));
  if (!getparint("mode", &emf.mode)) emf.mode = 0;
  if (emf.mode != 0 && emf.mode != 2)
    die("mode=1 (the l-BFGS inversion) is the reference's host driver: link it against "
        "libemmi_gpu; this program runs mode=0 and mode=2", NULL);
  if (!getparint("verb", &emf.verb)) emf.verb = 1;
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
  /* ---- acquisition (src/acq_init_free.c) ---- */
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
  const long n3s = 3L * (emf.n1 + 1) * (emf.n2 + 1) * (emf.n3 + 1);
  double complex *x = malloc(n3s * sizeof(double complex));
  double complex *b = malloc(n3s * sizeof(double complex));
  /* ---- gradient mode: fg_fwi_init and do_fwi parameters ---- */
  emmi_fwi_t fwi;
  memset(&fwi, 0, sizeof(fwi));
  int *chc = malloc(emf.nchrec * sizeof(int));
  for (int c = 0; c < emf.nchrec; c++) chc[c] = chan_code(emf.chrec[c]);
  float *gsum = NULL, *hsum = NULL, *bathy = NULL, fcost_all = 0;
  emmi_cf32 *Ef = NULL, *Ea = NULL;
  if (emf.mode == 2) {
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
    int seed = 1;
    getparint("seed", &seed);
    rng_state = (unsigned long long)seed;
    if (!getparint("npar", &fwi.npar)) fwi.npar = 2;
    fwi.idxpar = malloc(fwi.npar * sizeof(int));
    for (int j = 0; j < fwi.npar; j++) fwi.idxpar[j] = j + 1;
    getparint("idxpar", fwi.idxpar);
    if (!getparint("preco", &fwi.preco)) fwi.preco = 1;
    bathy = read_floats(fbathy, (size_t)emf.nx * emf.ny);
    emf.bathy = malloc(emf.ny * sizeof(float *));
    for (int j = 0; j < emf.ny; j++) emf.bathy[j] = bathy + (size_t)j * emf.nx;
    fwi.n = (int)(nxyz * fwi.npar);
    gsum = calloc((size_t)fwi.n, sizeof(float));
    hsum = calloc((size_t)fwi.n, sizeof(float));
    float *gr = malloc((size_t)fwi.n * sizeof(float)), *ph = malloc((size_t)fwi.n * sizeof(float));
    fwi.grad = (float ****)table4(gr, sizeof(float), emf.nx, emf.ny, emf.nz, fwi.npar);
    fwi.phess = (float ****)table4(ph, sizeof(float), emf.nx, emf.ny, emf.nz, fwi.npar);
    Ef = malloc(3 * nxyz * emf.nfreq * sizeof(emmi_cf32));
    Ea = malloc(3 * nxyz * emf.nfreq * sizeof(emmi_cf32));
  }
  for (int is = 0; is < nshots; is++) {
    const int shot = shots[is];
    if (shot < 1 || shot > nsrc_all) die("shot index out of range", NULL);
    /* receivers of this shot from the source-receiver table */
    FILE *fp = fopen(fsrcrec, "r");
    if (!fp) die("cannot open ", fsrcrec);
    if (fscanf(fp, "%*[^\n]\n") < 0) die("empty file ", fsrcrec);
    int a, c, nrec = 0, cap = 1024;
    int *ridx = malloc(cap * sizeof(int));
    while (fscanf(fp, "%d %d", &a, &c) == 2)
      if (a == shot) {
        if (nrec == cap) ridx = realloc(ridx, (cap *= 2) * sizeof(int));
        ridx[nrec++] = c;
      }
    fclose(fp);
    acq.nsrc = 1;
    acq.nrec = nrec;
    float src5[5] = {S[shot - 1].x, S[shot - 1].y, S[shot - 1].z,
                     (float)(PI_REF * S[shot - 1].hd / 180.), (float)(PI_REF * S[shot - 1].pit / 180.)};
    acq.src_x1 = &src5[0];
    acq.src_x2 = &src5[1];
    acq.src_x3 = &src5[2];
    acq.src_azimuth = &src5[3];
    acq.src_dip = &src5[4];
    acq.rec_x1 = malloc(nrec * sizeof(float));
    acq.rec_x2 = malloc(nrec * sizeof(float));
    acq.rec_x3 = malloc(nrec * sizeof(float));
    acq.rec_azimuth = malloc(nrec * sizeof(float));
    acq.rec_dip = malloc(nrec * sizeof(float));
    for (int i = 0; i < nrec; i++) {
      point_t p = R[ridx[i] - 1];
      acq.rec_x1[i] = p.x;
      acq.rec_x2[i] = p.y;
      acq.rec_x3[i] = p.z;
      acq.rec_azimuth[i] = PI_REF * p.hd / 180.;
      acq.rec_dip[i] = PI_REF * p.pit / 180.;
    }
    /* ---- regrid_init (host front end) ---- */
    const int n1 = emf.n1, n2 = emf.n2, n3 = emf.n3;
    eh_grid G;
    float **arr[12] = {&emf.x1, &emf.x2, &emf.x3, &emf.x1s, &emf.x2s, &emf.x3s,
                       &emf.d1, &emf.d2, &emf.d3, &emf.d1s, &emf.d2s, &emf.d3s};
    const int len[12] = {n1, n2, n3, n1, n2, n3, n1, n2, n3, n1, n2, n3};
    for (int i = 0; i < 12; i++) *arr[i] = malloc((len[i] + 1) * sizeof(float));
    G.x1 = emf.x1; G.x2 = emf.x2; G.x3 = emf.x3;
    G.x1s = emf.x1s; G.x2s = emf.x2s; G.x3s = emf.x3s;
    G.d1 = emf.d1; G.d2 = emf.d2; G.d3 = emf.d3;
    G.d1s = emf.d1s; G.d2s = emf.d2s; G.d3s = emf.d3s;
    const size_t nc = (size_t)n1 * n2 * n3;
    float *s11 = malloc(nc * sizeof(float)), *s22 = malloc(nc * sizeof(float)),
          *s33 = malloc(nc * sizeof(float)), *imu = malloc(nc * sizeof(float));
    G.sigma11 = s11; G.sigma22 = s22; G.sigma33 = s33; G.invmur = imu;
    if (eh_regrid(&M, src5[0], src5[1], src5[2], &G) != EH_OK) die("regrid failed", NULL);
    emf.sigma11 = (float ***)table3(s11, sizeof(float), n1, n2, n3);
    emf.sigma22 = (float ***)table3(s22, sizeof(float), n1, n2, n3);
    emf.sigma33 = (float ***)table3(s33, sizeof(float), n1, n2, n3);
    emf.invmur = (float ***)table3(imu, sizeof(float), n1, n2, n3);
    /* dcal_fd[nchrec][nfreq][nrec] */
    emmi_cf32 *dc = calloc((size_t)emf.nchrec * emf.nfreq * (nrec ? nrec : 1), sizeof(emmi_cf32));
    emf.dcal_fd = (emmi_cf32 ***)table3(dc, sizeof(emmi_cf32), nrec ? nrec : 1, emf.nfreq,
                                        emf.nchrec);
    char fname[64];
    if (emf.mode == 0) {
      /* ---- do_modelling frequency loop (src/do_modelling.c:50-64) ---- */
      model_all(&emf, &acq, x, b, n3s, shot, 0);
      snprintf(fname, sizeof(fname), "emf_%04d.txt", shot);
      write_data(fname, shot, &emf, nrec, dc);
    } else {
      fcost_all += gradient_shot(&emf, &acq, &fwi, x, b, n3s, shot, nrec, dc, chc, Ef, Ea, nxyz);
      for (long i = 0; i < fwi.n; i++) {
        gsum[i] += (&fwi.grad[0][0][0][0])[i];
        if (fwi.preco == 1) hsum[i] += (&fwi.phess[0][0][0][0])[i];
      }
    }
    for (int i = 0; i < 12; i++) free(*arr[i]);
    free(s11); free(s22); free(s33); free(imu); free(dc); free(ridx);
    free(acq.rec_x1); free(acq.rec_x2); free(acq.rec_x3); free(acq.rec_azimuth); free(acq.rec_dip);
  }
  if (emf.mode == 2) {
    /* the reference writes the summed data gradient before regularization
     * (src/fg_fwi.c:276-283) */
    FILE *fp = fopen("gradient_dat_Rv", "wb");
    if (!fp) die("cannot write gradient_dat_Rv", NULL);
    fwrite(gsum, nxyz * sizeof(float), 1, fp);
    fclose(fp);
    if (fwi.npar > 1) {
      fp = fopen("gradient_dat_Rh", "wb");
      if (!fp) die("cannot write gradient_dat_Rh", NULL);
      fwrite(gsum + nxyz, nxyz * sizeof(float), 1, fp);
      fclose(fp);
    }
    if (fwi.preco == 1) {
      fp = fopen("gradient_phess", "wb");
      if (fp) {
        fwrite(hsum, (size_t)fwi.n * sizeof(float), 1, fp);
        fclose(fp);
      }
    }
    if (emf.verb) printf("fcost_dat=%g\n", fcost_all);
  }
  free(x);
  free(b);
  return 0;
}

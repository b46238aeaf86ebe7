/* emmi_main: the reference's modelling command line on the GB300 hot path.
 *
 *   emmi_main mode=0 freqs=1 chsrc=Ex chrec=Ex,Ey,Hx,Hy nx=.. ny=.. nz=..
 *             dx=.. dy=.. dz=.. ox=.. oy=.. [oz=0] [n1=n2=n3=128]
 *             frho11=.. frho22=.. frho33=.. fsrc=.. frec=.. fsrcrec=..
 *             [shots=1,2,..] [cycleopt ncycle v1 v2 tol isemicoarsen]
 *             [gmg_precision=1] [icheck=0] [verb=1]
 *
 * Same parameters (src/emf_init_free.c:19-112, src/acq_init_free.c:27-128,
 * src/gmg.c:1712-1717), same input files and the same output file
 * emf_%04d.txt in the reference's format (src/read_write_data.c:14-36).
 * The frequency loop is src/do_modelling.c:49-67 and calls the drop-in
 * entry points of libemmi_gpu (gmg_init, inject_source, gmg_apply,
 * extract_emf_data, gmg_free).  Without MPI the shots listed in shots= run
 * one after another in this process (the reference runs one per rank).
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

int main(int argc, char **argv) {
  initargs(argc, argv);
  emmi_emf_t emf;
  emmi_acq_t acq;
  memset(&emf, 0, sizeof(emf));
  memset(&acq, 0, sizeof(acq));
  if (!getparint("mode", &emf.mode)) emf.mode = 0;
  if (emf.mode != 0) die("only mode=0 (forward modelling) is driven by this program", NULL);
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
    /* ---- do_modelling frequency loop (src/do_modelling.c:50-64) ---- */
    for (int f = 0; f < emf.nfreq; f++) {
      gmg_init(&emf, f);
      inject_source(&acq, &emf, (emmi_cf64 *)b, f);
      memset(x, 0, n3s * sizeof(double complex));
      gmg_apply((int)n3s, (emmi_cf64 *)b, (emmi_cf64 *)x);
      int cyc;
      double rel;
      const int st = emmi_gpu_last_status(&cyc, &rel);
      if (emf.verb)
        printf("shot %d freq %g: %d cycles, relative residual %.3e, status %d\n", shot,
               emf.freqs[f], cyc, rel, st);
      extract_emf_data(&acq, &emf, (emmi_cf64 *)x, (emmi_cf64 *)b, f);
      gmg_free();
    }
    /* ---- write_data (src/read_write_data.c:14-36) ---- */
    char fname[64];
    snprintf(fname, sizeof(fname), "emf_%04d.txt", shot);
    FILE *out = fopen(fname, "w");
    if (!out) die("cannot write ", fname);
    fprintf(out, "iTx \tiRx    chrec  frequency/Hz    Real{E/H}     Imag{E/H}\n");
    for (int ic = 0; ic < emf.nchrec; ic++)
      for (int f = 0; f < emf.nfreq; f++)
        for (int ir = 0; ir < nrec; ir++) {
          const float *v = (const float *)&dc[((size_t)ic * emf.nfreq + f) * nrec + ir];
          fprintf(out, "%d \t %d \t %s \t %g \t %e \t %e\n", shot, ir + 1, emf.chrec[ic],
                  emf.freqs[f], v[0], v[1]);
        }
    fclose(out);
    for (int i = 0; i < 12; i++) free(*arr[i]);
    free(s11); free(s22); free(s33); free(imu); free(dc); free(ridx);
    free(acq.rec_x1); free(acq.rec_x2); free(acq.rec_x3); free(acq.rec_azimuth); free(acq.rec_dip);
  }
  free(x);
  free(b);
  return 0;
}

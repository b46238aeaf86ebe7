/* Golden-vector dump driver for the reference -- TEST INFRASTRUCTURE ONLY.
 *
 * Linked against oracle/_ref/libemmi_ref.so (the reference compiled from its
 * own sources).  Runs the reference's own chain for one shot,
 *   emf_init -> acq_init -> regrid_init -> per frequency:
 *     gmg_init, inject_source, gmg_apply, extract_emf_data,
 *     extract_electric_field, extract_magnetic_field, gmg_free
 *   [adjoint=1: inject_adj_source, gmg_apply, extract_electric_field,
 *    then build_gradient]
 * and writes every intermediate array as raw little-endian binary into
 * dumpdir=<dir>.  Parameters are the reference's key=value parameters plus
 * dumpdir, adjoint, npar (1|2), preco, bathy (constant seafloor depth).
 * The call sequence follows src/do_modelling.c:49-67 and src/fg_fwi.c:183-263.
 */
#include "cstd.h"
#include "acq.h"
#include "emf.h"
#include "fwi.h"

void emf_init(emf_t *emf);
void acq_init(acq_t *acq, emf_t *emf);
void regrid_init(acq_t *acq, emf_t *emf);
void gmg_init(emf_t *emf, int ifreq);
void gmg_free();
void gmg_apply(int n, complex *b, complex *x);
void inject_source(acq_t *acq, emf_t *emf, complex *b, int ifreq);
void inject_adj_source(acq_t *acq, emf_t *emf, complex *x, complex *b, int ifreq);
void extract_emf_data(acq_t *acq, emf_t *emf, complex *x, complex *b, int ifreq);
void extract_electric_field(acq_t *acq, emf_t *emf, complex *x, int ifreq);
void extract_magnetic_field(acq_t *acq, emf_t *emf, complex *b, int ifreq);
void build_gradient(acq_t *acq, emf_t *emf, fwi_t *fwi,
                    _Complex float ****E1f, _Complex float ****E2f,
                    _Complex float ****E3f, _Complex float ****E1a,
                    _Complex float ****E2a, _Complex float ****E3a);

static char *outdir = ".";

static void dump(const char *name, const void *p, size_t bytes) {
  char path[4096];
  snprintf(path, sizeof(path), "%s/%s", outdir, name);
  FILE *fp = fopen(path, "wb");
  if (!fp) {
    fprintf(stderr, "ref_dump: cannot write %s\n", path);
    exit(2);
  }
  fwrite(p, 1, bytes, fp);
  fclose(fp);
}

int main(int argc, char **argv) {
  initargs(argc, argv);
  getparstring("dumpdir", &outdir);
  int adjoint = 0, npar = 2, preco = 1;
  float bathy = 1000.f;
  getparint("adjoint", &adjoint);
  getparint("npar", &npar);
  getparint("preco", &preco);
  getparfloat("bathy", &bathy);

  emf_t *emf = calloc(1, sizeof(emf_t));
  acq_t *acq = calloc(1, sizeof(acq_t));
  emf->mode = 0;
  if (!getparint("verb", &emf->verb)) emf->verb = 0;
  emf_init(emf);
  acq_init(acq, emf);
  regrid_init(acq, emf);

  const int n1 = emf->n1, n2 = emf->n2, n3 = emf->n3;
  dump("x1", emf->x1, (n1 + 1) * sizeof(float));
  dump("x2", emf->x2, (n2 + 1) * sizeof(float));
  dump("x3", emf->x3, (n3 + 1) * sizeof(float));
  dump("x1s", emf->x1s, (n1 + 1) * sizeof(float));
  dump("x2s", emf->x2s, (n2 + 1) * sizeof(float));
  dump("x3s", emf->x3s, (n3 + 1) * sizeof(float));
  dump("d1", emf->d1, (n1 + 1) * sizeof(float));
  dump("d2", emf->d2, (n2 + 1) * sizeof(float));
  dump("d3", emf->d3, (n3 + 1) * sizeof(float));
  dump("d1s", emf->d1s, (n1 + 1) * sizeof(float));
  dump("d2s", emf->d2s, (n2 + 1) * sizeof(float));
  dump("d3s", emf->d3s, (n3 + 1) * sizeof(float));
  const size_t ncell = (size_t)n1 * n2 * n3;
  dump("sigma11", &emf->sigma11[0][0][0], ncell * sizeof(float));
  dump("sigma22", &emf->sigma22[0][0][0], ncell * sizeof(float));
  dump("sigma33", &emf->sigma33[0][0][0], ncell * sizeof(float));
  dump("invmur", &emf->invmur[0][0][0], ncell * sizeof(float));
  dump("omegas", emf->omegas, emf->nfreq * sizeof(float));
  dump("rho_water", &emf->rho_water, sizeof(float));
  float srcrec[5 + 5 * 4096];
  srcrec[0] = acq->src_x1[0];
  srcrec[1] = acq->src_x2[0];
  srcrec[2] = acq->src_x3[0];
  srcrec[3] = acq->src_azimuth[0];
  srcrec[4] = acq->src_dip[0];
  int nrec = acq->nrec;
  for (int i = 0; i < nrec && i < 4096; i++) {
    srcrec[5 + 5 * i + 0] = acq->rec_x1[i];
    srcrec[5 + 5 * i + 1] = acq->rec_x2[i];
    srcrec[5 + 5 * i + 2] = acq->rec_x3[i];
    srcrec[5 + 5 * i + 3] = acq->rec_azimuth[i];
    srcrec[5 + 5 * i + 4] = acq->rec_dip[i];
  }
  dump("srcrec", srcrec, (5 + 5 * nrec) * sizeof(float));

  const int n = 3 * (n1 + 1) * (n2 + 1) * (n3 + 1);
  const int nfreq = emf->nfreq, nch = emf->nchrec;
  const size_t nxyz = (size_t)emf->nx * emf->ny * emf->nz;
  complex *x = alloc1complex(n), *b = alloc1complex(n);
  emf->dcal_fd = alloc3complexf(nrec, nfreq, nch);
  _Complex float ****E1f = alloc4complexf(emf->nx, emf->ny, emf->nz, nfreq);
  _Complex float ****E2f = alloc4complexf(emf->nx, emf->ny, emf->nz, nfreq);
  _Complex float ****E3f = alloc4complexf(emf->nx, emf->ny, emf->nz, nfreq);
  emf->H1 = alloc4complexf(emf->nx, emf->ny, emf->nz, nfreq);
  emf->H2 = alloc4complexf(emf->nx, emf->ny, emf->nz, nfreq);
  emf->H3 = alloc4complexf(emf->nx, emf->ny, emf->nz, nfreq);
  emf->E1 = E1f;
  emf->E2 = E2f;
  emf->E3 = E3f;
  char name[64];
  for (int f = 0; f < nfreq; f++) {
    gmg_init(emf, f);
    inject_source(acq, emf, b, f);
    snprintf(name, sizeof(name), "b_f%d", f);
    dump(name, b, n * sizeof(complex));
    memset(x, 0, n * sizeof(complex));
    gmg_apply(n, b, x);
    snprintf(name, sizeof(name), "x_f%d", f);
    dump(name, x, n * sizeof(complex));
    snprintf(name, sizeof(name), "h_f%d", f);
    dump(name, b, n * sizeof(complex));
    extract_emf_data(acq, emf, x, b, f);
    extract_electric_field(acq, emf, x, f);
    extract_magnetic_field(acq, emf, b, f);
    gmg_free();
  }
  dump("dcal", &emf->dcal_fd[0][0][0], (size_t)nch * nfreq * nrec * sizeof(_Complex float));
  dump("E1", &E1f[0][0][0][0], nfreq * nxyz * sizeof(_Complex float));
  dump("E2", &E2f[0][0][0][0], nfreq * nxyz * sizeof(_Complex float));
  dump("E3", &E3f[0][0][0][0], nfreq * nxyz * sizeof(_Complex float));
  dump("H1", &emf->H1[0][0][0][0], nfreq * nxyz * sizeof(_Complex float));
  dump("H2", &emf->H2[0][0][0][0], nfreq * nxyz * sizeof(_Complex float));
  dump("H3", &emf->H3[0][0][0][0], nfreq * nxyz * sizeof(_Complex float));

  if (adjoint) {
    /* deterministic data residual standing in for conj(W^2 (dobs-dcal)),
     * fg_fwi.c:208-226 */
    emf->dres_fd = alloc3complexf(nrec, nfreq, nch);
    for (int ic = 0; ic < nch; ic++)
      for (int f = 0; f < nfreq; f++)
        for (int ir = 0; ir < nrec; ir++)
          emf->dres_fd[ic][f][ir] =
              (1.0f + 0.1f * ir - 0.3f * ic) + I * (0.5f - 0.05f * ir + 0.2f * f);
    dump("dres", &emf->dres_fd[0][0][0], (size_t)nch * nfreq * nrec * sizeof(_Complex float));
    _Complex float ****E1a = alloc4complexf(emf->nx, emf->ny, emf->nz, nfreq);
    _Complex float ****E2a = alloc4complexf(emf->nx, emf->ny, emf->nz, nfreq);
    _Complex float ****E3a = alloc4complexf(emf->nx, emf->ny, emf->nz, nfreq);
    emf->E1 = E1a;
    emf->E2 = E2a;
    emf->E3 = E3a;
    for (int f = 0; f < nfreq; f++) {
      gmg_init(emf, f);
      inject_adj_source(acq, emf, x, b, f);
      snprintf(name, sizeof(name), "badj_f%d", f);
      dump(name, b, n * sizeof(complex));
      snprintf(name, sizeof(name), "madj_f%d", f);
      dump(name, x, n * sizeof(complex));
      memset(x, 0, n * sizeof(complex));
      gmg_apply(n, b, x);
      snprintf(name, sizeof(name), "xa_f%d", f);
      dump(name, x, n * sizeof(complex));
      extract_electric_field(acq, emf, x, f);
      gmg_free();
    }
    dump("E1a", &E1a[0][0][0][0], nfreq * nxyz * sizeof(_Complex float));
    dump("E2a", &E2a[0][0][0][0], nfreq * nxyz * sizeof(_Complex float));
    dump("E3a", &E3a[0][0][0][0], nfreq * nxyz * sizeof(_Complex float));

    fwi_t *fwi = calloc(1, sizeof(fwi_t));
    fwi->npar = npar;
    fwi->n = npar * (int)nxyz;
    fwi->preco = preco;
    fwi->idxpar = alloc1int(npar);
    fwi->idxpar[0] = 1;
    if (npar > 1) fwi->idxpar[1] = 2;
    fwi->grad = alloc4float(emf->nx, emf->ny, emf->nz, npar);
    fwi->phess = alloc4float(emf->nx, emf->ny, emf->nz, npar);
    memset(&fwi->phess[0][0][0][0], 0, npar * nxyz * sizeof(float));
    emf->bathy = alloc2float(emf->nx, emf->ny);
    for (int j = 0; j < emf->ny; j++)
      for (int i = 0; i < emf->nx; i++) emf->bathy[j][i] = bathy;
    if (!getparfloat("dsmute", &emf->dsmute)) emf->dsmute = 800;
    if (!getparfloat("drmute", &emf->drmute)) emf->drmute = 200;
    build_gradient(acq, emf, fwi, E1f, E2f, E3f, E1a, E2a, E3a);
    dump("grad", &fwi->grad[0][0][0][0], npar * nxyz * sizeof(float));
    dump("phess", &fwi->phess[0][0][0][0], npar * nxyz * sizeof(float));
  }
  return 0;
}

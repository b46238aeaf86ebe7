/* emmi_dropin.h -- drop-in replacements for the reference's hot-path
 * functions, with the reference's names and signatures.
 *
 * The struct layouts below restate, member for member, the reference's
 * emf_t (include/emf.h:4-48), acq_t (include/acq.h:4-19) and fwi_t
 * (include/fwi.h:4-28), so a host program compiled against the reference's
 * headers passes its structs unchanged.  N-d arrays are the reference's
 * pointer tables over one contiguous block (src/cstd.c:297-330): &a[0][0][0]
 * is a dense C-order buffer.
 *
 * Replaced entry points (prototypes as redeclared by the reference's callers,
 * src/do_modelling.c:17-24, src/fg_fwi.c:28-40):
 *   gmg_init / gmg_apply / gmg_free         src/gmg.c:1704, 1894, 1887
 *   inject_source / inject_adj_source       src/inject_extract.c:26, 124
 *   extract_emf_data                        src/inject_extract.c:317
 *   extract_electric_field / _magnetic_     src/inject_extract.c:477, 638
 *   build_gradient                          src/build_gradient.c:13
 * Solver knobs are read through the host's getpar functions when present
 * (cycleopt, ncycle, v1, v2, tol, isemicoarsen as gmg.c:1712-1717), plus
 * gmg_precision (0 = complex128 cycles, 1 = complex64 cycles with FP64
 * refinement, default 1) and sigma_floor.  The reference reports no solver
 * status; emmi_gpu_last_status() does.
 */
#ifndef EMMI_DROPIN_H
#define EMMI_DROPIN_H

/* complex element types: C99 _Complex in C; interleaved (re, im) pairs of
 * the same size and alignment in C++ (only pointers to them appear here) */
#ifdef __cplusplus
typedef struct { float re, im; } emmi_cf32;
typedef struct { double re, im; } emmi_cf64;
extern "C" {
#else
typedef _Complex float emmi_cf32;
typedef double _Complex emmi_cf64;
#endif

typedef struct {
  int mode, verb, reciprocity;
  int nfreq;
  float *freqs, *omegas;
  float rho_air, rho_water, lextend;
  int nchsrc, nchrec;
  char **chsrc, **chrec;
  float x1min, x1max, x2min, x2max, x3min, x3max;
  float *xx, *yy, *zz;
  int n1, n2, n3;
  float d1min, d2min, d3min;
  float *x1, *x2, *x3;
  float *x1s, *x2s, *x3s;
  float *d1, *d2, *d3;
  float *d1s, *d2s, *d3s;
  float ***sigma11, ***sigma22, ***sigma33, ***invmur;
  emmi_cf32 ***dcal_fd, ***dobs_fd, ***dres_fd;
  emmi_cf32 ****E1, ****E2, ****E3;
  emmi_cf32 ****H1, ****H2, ****H3;
  float ***mur, ***rho11, ***rho22, ***rho33;
  float **bathy;
  float rhomin, rhomax, depthmax;
  float ox, oy, oz;
  float dx, dy, dz;
  int nx, ny, nz, nb;
  int addnoise;
  float amp_perc, delta_phi, delta_theta;
  float noisefloorE, noisefloorH;
  float ***delta_emf;
  float ***rmse;
  float dsmute, drmute;
} emmi_emf_t;

typedef struct {
  int nsrc, nrec, nsubsrc, nsubrec;
  float lensrc, lenrec;
  float *src_x1, *src_x2, *src_x3, *src_azimuth, *src_dip;
  float *rec_x1, *rec_x2, *rec_x3, *rec_azimuth, *rec_dip;
  float x1min, x1max, x2min, x2max, x3min, x3max;
  int nsrc_total, nrec_total;
  int *shot_idx;
} emmi_acq_t;

typedef struct {
  int npar, n, preco;
  int r1, r2, r3, repeat;
  int *idxpar;
  float *minpar, *maxpar;
  int iter, niter;
  float *xref;
  float gamma1, gamma2;
  int firstgrad;
  float alpha;
  float fcost_dat, fcost_mod, fcost;
  float *fcost_list;
  float ****grad, ****phess, ***Hv;
  float mse;
} emmi_fwi_t;

void gmg_init(emmi_emf_t *emf, int ifreq);
void gmg_apply(int n, emmi_cf64 *b, emmi_cf64 *x);
void gmg_free(void);
void inject_source(emmi_acq_t *acq, emmi_emf_t *emf, emmi_cf64 *b, int ifreq);
void inject_adj_source(emmi_acq_t *acq, emmi_emf_t *emf, emmi_cf64 *x,
                       emmi_cf64 *b, int ifreq);
void extract_emf_data(emmi_acq_t *acq, emmi_emf_t *emf, emmi_cf64 *x,
                      emmi_cf64 *b, int ifreq);
void extract_electric_field(emmi_acq_t *acq, emmi_emf_t *emf, emmi_cf64 *x, int ifreq);
void extract_magnetic_field(emmi_acq_t *acq, emmi_emf_t *emf, emmi_cf64 *b, int ifreq);
void build_gradient(emmi_acq_t *acq, emmi_emf_t *emf, emmi_fwi_t *fwi,
                    emmi_cf32 ****E1f, emmi_cf32 ****E2f, emmi_cf32 ****E3f,
                    emmi_cf32 ****E1a, emmi_cf32 ****E2a, emmi_cf32 ****E3a);

/* status of the last gmg_apply: EMMI_SOLVE_* of emmi_gpu.h, cycles, and the
 * final relative residual; returns the status */
int emmi_gpu_last_status(int *cycles, double *rel_residual);
/* set a solver knob for callers without getpar (same keys as above) */
int emmi_gpu_set_param(const char *key, double value);

#ifdef __cplusplus
}
#endif
#endif

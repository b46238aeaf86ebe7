/* emmi_host.h -- host front end (C) that prepares the hot path's inputs.
 *
 * Restates, in float arithmetic identical to the reference, the regridding
 * stage that runs before the multigrid solve: padding of the input model,
 * the source-centred power-law stretched mesh and volume-averaging
 * homogenization (src/regrid_init_free.c:37-232, src/create_nugrid.c:13-36,
 * src/homogenization.c:15-111).  All functions are pure: caller-owned
 * arrays in, caller-owned arrays out.
 */
#ifndef EMMI_HOST_H
#define EMMI_HOST_H

#ifdef __cplusplus
extern "C" {
#endif

#define EH_OK 0
#define EH_EINVAL -1
#define EH_ESEARCH -2 /* the reference's source-depth search would read past
                         the padded z axis (src/regrid_init_free.c:194 sizes
                         it by nx); the reference's result is undefined there */
#define EH_ENUGRID -3 /* a stretched axis has no geometric ratio: the
                         reference's fixed-point loop (src/create_nugrid.c:
                         24-31) never ends there, e.g. one cell left below
                         the source for the bottom stretch (n3 too small) */

typedef struct {
  int nx, ny, nz;           /* input model cells                         */
  float dx, dy, dz;
  float ox, oy, oz;
  const float *rho11, *rho22, *rho33; /* [nz][ny][nx] resistivity        */
  int nb;                   /* padding cells per side (default 10)        */
  float lextend;            /* padding extent (default 5e4 m)             */
  float rho_air;            /* default 1e8                                */
  float d1min, d2min, d3min;/* smallest stretched cells (100, 100, 20)    */
  int n1, n2, n3;           /* multigrid mesh cells                       */
} eh_model;

typedef struct {
  /* node, staggered and spacing arrays, n+1 floats each (emf->x1 ...) */
  float *x1, *x2, *x3, *x1s, *x2s, *x3s, *d1, *d2, *d3, *d1s, *d2s, *d3s;
  /* homogenized conductivities and inverse permeability, n3*n2*n1 floats */
  float *sigma11, *sigma22, *sigma33, *invmur;
} eh_grid;

/* create_nugrid.c:13-36: x[0..n] of a geometric progression with first cell
 * dx spanning len; returns the ratio (1 for a uniform grid), or 0 where the
 * fixed-point iteration has no fixed point (the reference never returns) */
float eh_create_nugrid(int n, float len, float dx, float *x);

/* find_index.c:9-30 */
int eh_find_index(int n, const float *x, float val);

/* regrid_init_free.c:21-34 */
void eh_stagger(int n, const float *x, float *xs, float *d, float *ds);

/* homogenization.c:15-111: volume averages of in[nz][ny][nx] (on the node
 * axes xx,yy,zz) over the cells of x1,x2,x3 into out[n3][n2][n1] */
int eh_homogenize(const float *in, float *out, int nx, int ny, int nz,
                  const float *xx, const float *yy, const float *zz, int n1,
                  int n2, int n3, const float *x1, const float *x2,
                  const float *x3);

/* regrid_init (regrid_init_free.c:37-232) for a source at (sx,sy,sz);
 * out arrays preallocated by the caller. */
int eh_regrid(const eh_model *m, float sx, float sy, float sz, eh_grid *out);

/* The two halves of eh_regrid, for a batch of shots over one model:
 * eh_pad_dims gives the padded model's cells (nx + 2 nb, ...);
 * eh_pad_model the padded node axes xx[nxp+1], yy[nyp+1], zz[nzp+1] and the
 * padded model pad[3][nzp][nyp][nxp] (sigma11, sigma22, rho33) once per
 * model (regrid_init_free.c:47-141); eh_regrid_axes the shot's mesh axes
 * and their staggered copies in g (regrid_init_free.c:156-214; the
 * conductivity arrays of g are not touched).  Homogenizing pad onto the
 * axes (eh_homogenize, or the GPU library's emmi_homogenize_batch) gives
 * eh_regrid's conductivities. */
int eh_pad_dims(const eh_model *m, int *nxp, int *nyp, int *nzp);
int eh_pad_model(const eh_model *m, float *xx, float *yy, float *zz, float *pad);
int eh_regrid_axes(const eh_model *m, const float *xx, const float *yy,
                   const float *zz, float sx, float sy, float sz, eh_grid *g);

/* emf_init_free.c:114-128: the smallest resistivity of the three cubes */
float eh_rho_water(const eh_model *m);

/* ---- data misfit of the gradient mode (mode=2) ---------------------------
 * Arrays of receiver data are [nchrec][nfreq][nrec], complex values as
 * interleaved (re, im) floats; ch[] holds channel codes 0..5 = Ex, Ey, Ez,
 * Hx, Hy, Hz. */

/* cal_uncertainty_noise.c:17-97 without its noise: the standard deviation
 * delta of every datum from the amplitude uncertainty amp_perc, the azimuth
 * uncertainty delta_phi and the noise floors (Ez, Hz: 0, as the reference
 * leaves them). */
void eh_uncertainty(int nchrec, const int *ch, int nfreq, int nrec,
                    const float *rec_azimuth, float src_azimuth,
                    const float *dobs, float amp_perc, float delta_phi,
                    float noisefloorE, float noisefloorH, float *delta);

/* fg_fwi.c:208-226: for receivers farther than 5.5 skin depths of water from
 * the source (horizontal offset), res = (dobs - dcal)/delta, rmse = |res|,
 * the adjoint source dres = conj(res/delta); nearer receivers get dres = 0
 * and rmse = 0.  Returns fcost = 0.5 * sum |res|^2. */
float eh_misfit(int nchrec, int nfreq, int nrec, const float *omegas,
                float rho_water, float src_x, float src_y, const float *rec_x,
                const float *rec_y, const float *dobs, const float *dcal,
                const float *delta, float *dres, float *rmse);

#ifdef __cplusplus
}
#endif
#endif

/* CPU oracle for the libEMMI_MGFD hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's geometric-multigrid curl-curl
 * solve (src/gmg.c), source injection / receiver extraction
 * (src/inject_extract.c, src/find_index.c) and adjoint gradient accumulation
 * (src/build_gradient.c).  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py may load it, and only as the checker: the product
 * path never calls it.
 *
 * Pinned against the reference: tests/golden/ holds vectors produced by the
 * reference compiled from its own sources (oracle/_ref) on the same inputs,
 * and tests/test_oracle_golden.py checks this library against them.
 *
 * Layout (same as the reference): a field has 3 components, each on an
 * (n1+1)*(n2+1)*(n3+1) slot array, component-major, i fastest:
 *   u[c*S + i + (n1+1)*(j + (n2+1)*k)],  S = (n1+1)(n2+1)(n3+1).
 * Cell arrays (conductivity, inverse permeability) are n3*n2*n1, i fastest.
 */
#ifndef EMMI_ORACLE_H
#define EMMI_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* smoother orderings */
#define EO_ORDER_LEX 0      /* the reference's lexicographic sweeps        */
#define EO_ORDER_COLOR 1    /* multicolour: 4-colour lines, 8-colour nodes */

typedef struct {
  int cycleopt;      /* 1=V, 2=F, 3=W                       (gmg.c:1712) */
  int ncycle;        /* maximum number of cycles              (gmg.c:1713) */
  int v1, v2;        /* pre/post smoothing counts             (gmg.c:1714) */
  double tol;        /* relative residual tolerance           (gmg.c:1716) */
  int isemicoarsen;  /* 1=semi-coarsening                     (gmg.c:1717) */
  int ordering;      /* EO_ORDER_LEX or EO_ORDER_COLOR                     */
  int verb;
} eo_params;

/* Full solve, following gmg_apply (gmg.c:1894-1932).
 * x1,x2,x3: node coordinates (float, n+1 each, as emf->x1..x3);
 * sigma11/22/33, invmur: float cell arrays (as emf->sigma11.. after regrid);
 * b: in = i*omega*mu0*J on the slots, out = H (gmg.c:1929);
 * x: out = E.  rnorm_hist (optional, length >= ncycle+1) receives the
 * level-0 residual norm of every cycle.  Returns the number of cycles run
 * (the cycle index at which the tolerance was met, or ncycle). */
int eo_gmg_solve(int n1, int n2, int n3,
                 const float *x1, const float *x2, const float *x3,
                 const float *sigma11, const float *sigma22,
                 const float *sigma33, const float *invmur,
                 double omega, const eo_params *prm,
                 double *b, double *x, double *rnorm_hist);
/* The same with wall-clock timing: seconds[0] = set-up before the first
 * cycle (level-0 arrays, volume scaling), seconds[1] = the cycles (each
 * hierarchy built at its first use inside them). */
int eo_gmg_solve_timed(int n1, int n2, int n3,
                       const float *x1, const float *x2, const float *x3,
                       const float *sigma11, const float *sigma22,
                       const float *sigma33, const float *invmur,
                       double omega, const eo_params *prm,
                       double *b, double *x, double *rnorm_hist, double *seconds);

/* ---- single-level operators, for kernel parity ------------------------- */
/* A level is described by double node coordinates x[d] (n_d+1 values) and
 * volume-weighted cell arrays sig[3], imu (double, n3*n2*n1).              */
typedef struct {
  int n[3];
  const double *x[3];
  const double *sig[3];
  const double *imu;
  double omega;
} eo_level_desc;

/* r = f - A u over all slots (r = f where no equation applies), gmg.c:1316 */
void eo_residual(const eo_level_desc *L, const double *u, const double *f,
                 double *r);
/* r = A u on unknown slots, 0 elsewhere (the operator itself) */
void eo_apply(const eo_level_desc *L, const double *u, double *au);
/* one line-relaxation sweep along direction dir (0=x,1=y,2=z), gmg.c:340-1298 */
void eo_line_sweep(const eo_level_desc *L, int dir, int ordering, int iter,
                   double *u, const double *f);
/* one node-patch block relaxation sweep, gmg.c:116-336 */
void eo_point_sweep(const eo_level_desc *L, int ordering, int iter,
                    double *u, const double *f);
/* restriction fine r -> coarse f (gmg.c:1510); sc[3] are the coarsening
 * factors of the coarse level; xf/xc node coordinates */
void eo_restrict(const int nf[3], const double *const xf[3],
                 const int nc[3], const double *const xc[3], const int sc[3],
                 const double *rf, double *fc);
/* prolongation u_f += P u_c (gmg.c:1463) */
void eo_prolong(const int nf[3], const double *const xf[3],
                const int nc[3], const double *const xc[3], const int sc[3],
                const double *uc, double *uf);
/* coarse-cell conductivity sums / repeat (gmg.c:1803-1858) */
void eo_coarsen_cells(const int nf[3], const int sc[3], const double *cf,
                      double *cc);
/* H = curl E / (i omega mu0) on faces (gmg.c:1414) */
void eo_curl_h(const eo_level_desc *L, const double *u, double *h);

/* ---- injection / extraction / gradient ---------------------------------- */
/* Grid description as in emf_t after regrid_init (float arrays, n+1 each). */
typedef struct {
  int n1, n2, n3;
  const float *x1, *x2, *x3, *x1s, *x2s, *x3s, *d1, *d2, *d3;
  const float *sigma33;   /* homogenized sigma33, n3*n2*n1 (not weighted) */
  float rho_water;
} eo_grid;

/* channel codes: 0..2 = Ex,Ey,Ez ; 3..5 = Hx,Hy,Hz */
int eo_find_index(int n, const float *x, float val);          /* find_index.c */
void eo_inject_source(const eo_grid *g, int nsrc, const float *sx,
                      const float *sy, const float *sz, const float *azim,
                      const float *dip, int nch, const int *chsrc,
                      float omega, double *b);               /* :26-120  */
void eo_inject_adj_source(const eo_grid *g, int nrec, const float *rx,
                          const float *ry, const float *rz, const float *azim,
                          const float *dip, int nch, const int *chrec,
                          const float *dres /* [nch][nrec] complex float */,
                          float omega, double *x, double *b); /* :124-314 */
void eo_extract_emf_data(const eo_grid *g, int nrec, const float *rx,
                         const float *ry, const float *rz, const float *azim,
                         const float *dip, int nch, const int *chrec,
                         const double *x, const double *b,
                         float *dcal /* [nch][nrec] complex float */); /* :317 */
void eo_extract_electric_field(const eo_grid *g, int nx, int ny, int nz,
                               float ox, float oy, float oz, float dx,
                               float dy, float dz, const float *rho33,
                               const double *x, float *E1, float *E2,
                               float *E3);                   /* :477-635 */
void eo_extract_magnetic_field(const eo_grid *g, int nx, int ny, int nz,
                               float ox, float oy, float oz, float dx,
                               float dy, float dz, const double *b,
                               float *H1, float *H2, float *H3); /* :638 */
void eo_build_gradient(int nx, int ny, int nz, float ox, float oy, float oz,
                       float dx, float dy, float dz, int nfreq, int npar,
                       const int *idxpar, int preco,
                       const float *E1f, const float *E2f, const float *E3f,
                       const float *E1a, const float *E2a, const float *E3a,
                       const float *rho11, const float *rho33,
                       const float *bathy, int nsrc, const float *sx,
                       const float *sy, const float *sz, float dsmute,
                       int nrec, const float *rx, const float *ry,
                       const float *rz, float drmute,
                       float *grad, float *phess);   /* build_gradient.c */

#ifdef __cplusplus
}
#endif
#endif

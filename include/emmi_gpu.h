/* emmi_gpu.h -- C ABI of the GB300 hot path of libEMMI_MGFD.
 *
 * Two layers:
 *  1. Drop-in entry points with the reference's own names and signatures
 *     (declared in include/emmi_dropin.h), replacing src/gmg.c,
 *     src/inject_extract.c and src/build_gradient.c of the reference.
 *  2. The batched solver below, which the drop-in layer is built on and
 *     which a caller can use directly to solve many right-hand sides
 *     (shots x frequencies x forward/adjoint) in one launch sequence.
 *
 * Conventions: a field is 3 components of (n1+1)(n2+1)(n3+1) complex slots,
 * component-major, i fastest (the reference's layout, src/gmg.c:1780);
 * complex numbers are interleaved (re, im) doubles.  Cell arrays are
 * [n3][n2][n1] floats.  All entry points return 0 on success and a negative
 * EMMI_E* code on failure; emmi_last_error() describes the last failure.
 */
#ifndef EMMI_GPU_H
#define EMMI_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* error codes */
#define EMMI_OK 0
#define EMMI_EINVAL -1   /* bad argument                          */
#define EMMI_ECUDA -2    /* CUDA runtime failure                  */
#define EMMI_ENOMEM -3   /* device allocation failed              */
#define EMMI_ESTATE -4   /* call out of order                     */

/* per-RHS solve status (gmg.c never reports non-convergence; this does) */
#define EMMI_SOLVE_OK 0        /* reached tol                        */
#define EMMI_SOLVE_MAXIT 1     /* ncycle cycles without reaching tol */
#define EMMI_SOLVE_STALL 2     /* residual stopped decreasing        */
#define EMMI_SOLVE_NONFINITE 3 /* NaN/Inf in the residual            */

/* precision modes */
#define EMMI_PREC_FP64 0   /* complex128 cycles: the reference's arithmetic  */
#define EMMI_PREC_MIXED 1  /* complex64 cycles + FP64 residual refinement    */

typedef struct {
  int n1, n2, n3;   /* cells per direction, equal for every RHS           */
  int nop;          /* operators: distinct (grid, conductivity) pairs      */
  int nrhs;         /* right-hand sides                                    */
  const float *x1;  /* [nop][n1+1] node coordinates (emf->x1 after regrid)  */
  const float *x2;  /* [nop][n2+1]                                         */
  const float *x3;  /* [nop][n3+1]                                         */
  const float *cells; /* [nop][4][n3][n2][n1]: sigma11, sigma22, sigma33,
                         invmur (emf->sigma11.. after regrid, S/m)          */
  const int *op;    /* [nrhs] operator of each RHS (NULL: rhs i uses op i)  */
  const float *omega; /* [nrhs] angular frequency 2*pi*f (emf->omegas)      */
} emmi_problem;

typedef struct {
  int cycleopt;     /* 1=V 2=F 3=W                  (gmg.c:1712, default 2) */
  int ncycle;       /* max cycles                   (gmg.c:1713, default 30)*/
  int v1, v2;       /* pre/post smoothing           (gmg.c:1714-1715)      */
  double tol;       /* relative residual tolerance  (gmg.c:1716, 1e-6)     */
  int isemicoarsen; /* 1 = rotating semi-coarsening (gmg.c:1717, 1)        */
  int precision;    /* EMMI_PREC_*                                         */
  double sigma_floor; /* MIXED: conductivity floor (S/m) inside the complex64
                         preconditioner only; the FP64 residual keeps the true
                         operator.  <=0 selects 1e-4 * max(1, 2*pi/omega).  */
  int refine_every; /* MIXED: FP64 refinement at least every k cycles (3)  */
  int use_graphs;   /* capture the cycle into CUDA graphs (1)              */
  int verb;         /* print "icycle=%d rnorm=%e" like gmg.c:1627          */
} emmi_options;

typedef struct {
  int cycles;       /* cycles run                                         */
  int status;       /* EMMI_SOLVE_*                                       */
  double rnorm0;    /* |b_vol|                                            */
  double rnorm;     /* final |b_vol - A x| (FP64)                         */
  int refinements;  /* MIXED: FP64 residual evaluations                   */
} emmi_rhs_stats;

typedef struct emmi_solver emmi_solver;

/* fill opts with the reference's defaults (gmg.c:1712-1717) */
void emmi_default_options(emmi_options *opts);

/* Build a solver for a batch: uploads grids/conductivities, precomputes the
 * three semi-coarsening hierarchies and captures the cycle graphs. */
int emmi_solver_create(emmi_solver **out, const emmi_problem *prob,
                       const emmi_options *opts);

/* Solve A x = b for every RHS.  b: [nrhs][3*S] complex (i*omega*mu0*J, as
 * inject_source builds it); x: [nrhs][3*S] complex E out; h (optional):
 * [nrhs][3*S] complex H = curl E/(i omega mu0) out, like gmg_apply
 * (gmg.c:1927-1929).  device != 0: b, x, h are device pointers; else host
 * pointers (copies inside).  stats (optional): [nrhs]. */
int emmi_solver_solve(emmi_solver *s, const double *b, double *x, double *h,
                      int device, emmi_rhs_stats *stats);

/* Seconds of device time of the last solve (CUDA events on its stream). */
double emmi_solver_last_time(const emmi_solver *s);
/* Number of kernel launches in the last solve. */
long emmi_solver_last_launches(const emmi_solver *s);
/* Device bytes held by the solver. */
size_t emmi_solver_device_bytes(const emmi_solver *s);
void emmi_solver_destroy(emmi_solver *s);

const char *emmi_last_error(void);

/* ---- single-operator entry points for parity checks ------------------ */
/* Each works on one level described by node coordinates (double, n+1 per
 * direction) and volume-weighted cells (double [4][n3][n2][n1]), on host
 * arrays, in FP64 (prec=EMMI_PREC_FP64) or complex64 (EMMI_PREC_MIXED). */
int emmi_level_residual(const int n[3], const double *x1, const double *x2,
                        const double *x3, const double *cells, double omega,
                        int prec, const double *u, const double *f, double *r,
                        double *norm);
/* one multicolour sweep: dir 0..2 = line relaxation along x/y/z,
 * dir 3 = node-patch relaxation; iter%2==1 reverses the colour order */
int emmi_level_smooth(const int n[3], const double *x1, const double *x2,
                      const double *x3, const double *cells, double omega,
                      int prec, int dir, int iter, double *u, const double *f);

#ifdef __cplusplus
}
#endif
#endif

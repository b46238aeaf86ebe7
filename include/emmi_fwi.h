/* emmi_fwi.h -- the host side of the inversion mode (mode=1): l-BFGS with a
 * bisection line search on the Wolfe conditions, model regularization and
 * gradient smoothing.  Restates, in the reference's float arithmetic, the
 * optimizer and the regularization that drive the GPU gradient
 * (src/opt.c, src/regularization.c, src/triangle_smoothing.c; the driver
 * loop src/do_fwi.c:151-231 lives in emmi_main).  Plain arrays in and out. */
#ifndef EMMI_FWI_H
#define EMMI_FWI_H

#ifdef __cplusplus
extern "C" {
#endif

/* optimizer state (the fields of the reference's opt_t that l-BFGS uses) */
typedef struct {
  int niter, nls, npair, bound, method, ncg, preco, verb;
  float tol, c1, c2, alpha;
  int iter, kpair, ils, igrad, ls_fail, loop1;
  float f0, fk, gk_norm;
  float *x, *g, *d, *q, *xmin, *xmax;
  float **sk, **yk; /* [npair][n] */
  float *rho, *alp; /* [npair] */
} ef_opt;

/* misfit and gradient at x (the caller's fg_fwi) */
typedef float (*ef_fg)(void *ctx, float *x, float *g);

float ef_l2norm(int n, const float *a);              /* opt.c:27-35  */
float ef_dotprod(int n, const float *a, const float *b); /* opt.c:38-45 */
void ef_flipsign(int n, const float *a, float *b);   /* opt.c:48-52  */
/* store (x, g) as the newest pair, dropping the oldest when full
 * (opt.c:56-74); then, one iteration later, turn it into (s, y) = (x_new -
 * x_old, g_new - g_old) (opt.c:77-86) */
void ef_lbfgs_save(int n, const float *x, const float *g, ef_opt *o);
void ef_lbfgs_update(int n, const float *x, const float *g, ef_opt *o);
/* two-loop recursion: d = -H g (opt.c:89-128); the first loop into o->q
 * (opt.c:131-152) and the second loop from o->q into o->d (opt.c:155-175)
 * for a preconditioner applied in between */
void ef_lbfgs_descent(int n, const float *g, float *d, ef_opt *o);
void ef_lbfgs_descent1(int n, const float *g, ef_opt *o);
void ef_lbfgs_descent2(int n, ef_opt *o);
void ef_boundx(int n, float *x, const float *xmin, const float *xmax); /* opt.c:179-187 */
/* bisection line search on the Wolfe conditions along d from x with
 * gradient g (opt.c:190-252): x, g and o->fk, o->alpha, o->ils, o->igrad,
 * o->ls_fail updated */
void ef_line_search(int n, float *x, float *g, const float *d, ef_fg fg, void *ctx, ef_opt *o);

/* regularization.c:12-56 (Tikhonov, horizontal weight 1, vertical 0.03)
 * and :59-128 (total variation): g = gradient, returns the cost */
float ef_tikhonov(const float *x, float *g, int n1, int n2, int n3);
float ef_tv(const float *x, float *g, int n1, int n2, int n3);
/* triangle_smoothing.c:62-106 on mod[n3][n2][n1], in place */
void ef_triangle_smoothing(float *mod, int n1, int n2, int n3, int r1, int r2, int r3,
                           int repeat);

#ifdef __cplusplus
}
#endif
#endif

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
  const float *rho_water; /* [nop] smallest model resistivity (emf->rho_water),
                             used by the Ez receiver conversion; may be NULL
                             when no extraction is requested                */
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
                         operator.  <=0 selects 1e-5 * max(1, 2*pi/omega).  */
  int refine_every; /* MIXED: FP64 refinement at least every k cycles (4)  */
  int use_graphs;   /* capture the cycle into CUDA graphs (1)              */
  int verb;         /* print "icycle=%d rnorm=%e" like gmg.c:1627          */
  int krylov;       /* MIXED: 0 = stationary FP64 refinement of complex64
                       cycles; k > 0 = FP64 FGMRES(k) (k <= 12) with one
                       complex64 cycle as its preconditioner (0)           */
  int line_factors; /* MIXED: factor every line once per (operator,
                       frequency) at set-up and keep the factors, when they
                       fit in half the free device memory: 2 = L in fp16,
                       1/d in fp32 (fp32 throughout if an L value leaves
                       the fp16 range), 1 = fp32; 0 = factor in every
                       sweep (2)                                           */
  int autotune;     /* MIXED with stored fp16 factors: time the level-0
                       line sweep of each direction at set-up for a few
                       block shapes and keep the fastest; cached for the
                       process per (grid, RHS, direction); no shape changes
                       any result (1); 0 = default shapes; -k (k = 1..10)
                       forces shape k in every direction (checks)          */
  int line_sweep;   /* 1 = one launch per colour: each thread assembles,
                       factors and solves one line, keeping the multipliers
                       only between its two substitutions (fp16 when
                       line_factors = 2, else working precision); no stored
                       factors.  0 = three launches per colour (residual
                       rows, substitution, update) with the stored factors
                       of line_factors (default)                          */
  int fused_level;  /* with line_sweep = 0: levels l >= fused_level use the
                       one-launch sweep (their data sit in L2 and their
                       launches are short); levels above it the three-launch
                       sweep.  A value >= the number of levels keeps the
                       three-launch sweep everywhere                      */
  int staged;       /* MIXED: 1 = the complex64 residual stages each plane's
                       halo in shared memory with tensor copies (default);
                       0 = the plain residual                              */
  int skip_pre;     /* bit l set: level l leaves out its pre-smoothing (0:
                       every level smooths v1 times, as the reference)     */
  int skip_post;    /* bit l set: level l leaves out its post-smoothing (0:
                       every level smooths v2 times, as the reference);
                       bit 0 makes the learned correction, applied after
                       every cycle, take the place of the last level-0
                       post-smoothing (collect its training residuals with
                       the same setting)                                   */
} emmi_options;

typedef struct {
  int cycles;       /* cycles run                                         */
  int status;       /* EMMI_SOLVE_*                                       */
  double rnorm0;    /* |b_vol|                                            */
  double rnorm;     /* final |b_vol - A x| (FP64)                         */
  int refinements;  /* MIXED: FP64 residual evaluations                   */
  int fallback;     /* 1 if the learned correction was switched off for
                       this RHS because its residual stalled               */
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
/* Multiplier format of the one-launch line sweep: 1 = fp16, 0 = working
 * precision (an fp16 multiplier out of range during a solve switches the
 * solver to 0 and restarts its inner cycles), -1 = no level uses it. */
int emmi_solver_line_format(const emmi_solver *s);
/* 1 when every operator's invmur is exactly 1 (as the host front end
 * writes it) and the complex64 operator therefore forms its coefficients
 * from the mesh spacings (the cell weights being the cell volumes), 0 when
 * it reads the volume-weighted invmur cells; the FP64 operator always reads
 * them (the reference's arithmetic). */
int emmi_solver_geometric_weights(const emmi_solver *s);
/* 1 when the complex64 level-0 residual of s stages its halos by tensor
 * copies (emmi_options.staged and a tile that fits shared memory). */
int emmi_solver_staged(const emmi_solver *s);
/* Test hook of the staged residual's bounded waits (no counterpart in the
 * reference): the staged residuals launched after the call give up a wait
 * for a plane's copies after wait_cycles clocks (0: the default, about a
 * second), and with stall_from >= 0 no copy of a plane at or beyond that
 * index is issued, so the first wait for one runs out: the CTA records the
 * failure, waits (with the full limit) for the copies it did issue and
 * returns, the launches after it return at once, and the solve reports
 * EMMI_ECUDA at its next norm check; stall_from = -1 issues every copy.
 * Launches captured in the cycle graphs keep the settings of their capture:
 * create s with use_graphs = 0 for the hook to reach its cycles. */
int emmi_stencil_wait_hook(emmi_solver *s, long long wait_cycles, int stall_from);
/* Number of kernel launches in the last solve. */
long emmi_solver_last_launches(const emmi_solver *s);
/* Device bytes held by the solver. */
size_t emmi_solver_device_bytes(const emmi_solver *s);
/* The stored line factors of a MIXED solver: 1 = L in fp16 with 1/d in
 * fp32, 0 = fp32 (asked for, or after an L value left the fp16 range),
 * -1 = none (factoring in every sweep).  No counterpart in the reference. */
int emmi_solver_line_factor_format(const emmi_solver *s);
/* The CUDA stream (cudaStream_t) every launch of this solver goes to. */
void *emmi_solver_stream(const emmi_solver *s);
/* the level-0 sweep shapes in use per direction d: shapes[d] = {lines per
 * block and ring depth of the fp16 substitution, threads per block of the
 * right-hand-side kernel}; *tuned = 1 when this solver's set-up timed them
 * (0: defaults or the process cache).  No counterpart in the reference. */
int emmi_solver_sweep_shapes(const emmi_solver *s, int shapes[3][3], int *tuned);
/* Time `reps` full level-0 line-relaxation sweeps (4 colours, all RHS) along
 * direction dir with CUDA events on the solver's stream, on the solver's
 * current fields.  ms: average milliseconds per sweep; launches: kernel
 * launches per sweep; bytes: algorithmic bytes per sweep,
 * S*(9c+12)*nrhs with c the complex size (u, f read and u written for three
 * components, three conductivities per cell). */
int emmi_solver_time_smoother(emmi_solver *s, int dir, int reps, double *ms,
                              int *launches, double *bytes);
void emmi_solver_destroy(emmi_solver *s);
/* emmi_solver_create with P->cells in device memory (the rest of P on the
 * host), e.g. from emmi_homogenize_batch: no host round trip of the cells.
 * No counterpart in the reference. */
int emmi_solver_create_dc(emmi_solver **out, const emmi_problem *P,
                          const emmi_options *opts);
/* The homogenization of the reference's regrid stage on the device for
 * nshots shots over one model (src/homogenization.c:15-111,
 * src/regrid_init_free.c:206-226): the padded model pad[3][nzp][nyp][nxp]
 * (sigma11, sigma22, rho33) on the node axes xx, yy, zz (eh_pad_model of
 * the host library) averaged onto each shot's cells x1[nshots][n1+1], x2,
 * x3 (eh_regrid_axes), written as cells[nshots][4][n3][n2][n1] (sigma11,
 * sigma22, sigma33 = 1 / rho33 average, invmur = 1) in device memory; every
 * other pointer is host memory.  Bit for bit the host front end's
 * (eh_regrid).  Synchronises the stream. */
int emmi_homogenize_batch(int nxp, int nyp, int nzp, const float *xx,
                          const float *yy, const float *zz, const float *pad,
                          int nshots, int n1, int n2, int n3, const float *x1,
                          const float *x2, const float *x3, float *cells,
                          void *stream);
/* Solver memory comes from the device's stream-ordered memory pool and goes
 * back to it on destroy, where it stays for the next solver; this returns
 * the pool's unused memory to the device.  No counterpart in the reference. */
int emmi_trim_memory(void);

const char *emmi_last_error(void);

/* ---- learned correction (no counterpart in the reference) -------------- */
/* A small linear 3x3x3 convolutional network (8 -> 8 -> 8 channels, bf16
 * tcgen05 tensor-core forward, 2 x 1728 fp32 weights [layer][tap][cin][cout],
 * tap = (dk+1)*9+(dj+1)*3+(di+1); the hidden layer is zero on the last slot
 * plane of each direction) that corrects the level-0 complex64 iterate after
 * every cycle of a MIXED solver: u += N(D^-1 (f - A u)) on unknown edges.
 * Levels whose rows are too wide for the convolution's shared-memory window
 * (more than about 1600 slots) are refused with EMMI_EINVAL.
 * Training minimises sum_b |r_b - A N(D^-1 r_b)|^2 / |r_b|^2 over residual
 * samples r_b of plain cycles.  A RHS whose FP64 residual does not halve
 * between refinements (restarts with krylov) with the correction on falls
 * back to plain cycles (emmi_rhs_stats.fallback). */
/* Solve b (as emmi_solver_solve, solution discarded) with plain cycles and
 * keep the level-0 residual after each of the first per_rhs cycles of every
 * RHS as training samples (stationary MIXED solvers). */
int emmi_learned_collect(emmi_solver *s, const double *b, int device,
                         int per_rhs, emmi_rhs_stats *stats);
/* Add ns samples r ([ns][3*S] complex float, host) of the operators of RHS
 * rhs[k] to the training set. */
int emmi_learned_add_samples(emmi_solver *s, int ns, const float *r,
                             const int *rhs);
int emmi_learned_samples(const emmi_solver *s);
/* steps full-batch Adam steps (rate lr) on the GPU from W (in/out); loss
 * (optional, [steps]): mean normalised loss before each step. */
int emmi_learned_train(emmi_solver *s, int steps, float lr, float *W,
                       float *loss);
/* loss (mean over samples) and dLoss_sum/dW ([2][1728], sum over samples of
 * the normalised losses) at W, without updating */
int emmi_learned_grad(emmi_solver *s, const float *W, float *loss,
                      float *grad);
/* use W in the following solves; W = NULL switches the correction off */
int emmi_learned_set(emmi_solver *s, const float *W);
/* One application of the correction set by emmi_learned_set to complex64
 * level-0 iterates: u += N(D^-1 (f - A u)), f and u device arrays
 * [nrhs][3][S] of the solver's operators (synchronises the stream). */
int emmi_learned_apply(emmi_solver *s, const void *f, void *u);
/* Test hook of the convolution's bounded waits (no counterpart in the
 * reference): the following emmi_learned_apply calls of s give up a wait
 * after wait_cycles clocks (0: the default, about a second), and with
 * stall = 1 the producer issues no copy and no MMA, so the first wait of
 * the epilogue runs out: the kernel records the failure, frees its tensor
 * memory and returns, and emmi_learned_apply reports EMMI_ECUDA.  Solves
 * never use these settings. */
int emmi_learned_wait_hook(emmi_solver *s, long long wait_cycles, int stall);

/* ---- survey: injection, extraction, gradient (src/inject_extract.c,
 *      src/build_gradient.c) ------------------------------------------- */
/* channel codes: 0..2 = Ex,Ey,Ez ; 3..5 = Hx,Hy,Hz */
typedef struct {
  int nsrc_ch;        /* source channels (chsrc)                            */
  const int *src_ch;
  int nrec_ch;        /* receiver channels (chrec)                          */
  const int *rec_ch;
  int nrec;           /* receivers per RHS                                  */
  const float *src;   /* [nrhs][5]: x, y, z, azimuth (rad), dip (rad)       */
  const float *rec;   /* [nrhs][nrec][5]                                    */
} emmi_survey;

/* End-to-end forward modelling of a batch (do_modelling,
 * src/do_modelling.c:49-67): inject each RHS's source, solve, extract the
 * receiver data.  Host arrays in and out; dcal: [nrhs][nrec_ch][nrec]
 * complex float (interleaved).  h2d/d2h (optional) receive the bytes
 * copied host->device and device->host. */
int emmi_modelling_batch(emmi_solver *s, const emmi_survey *sv, float *dcal,
                         emmi_rhs_stats *stats, size_t *h2d, size_t *d2h);

/* Device-resident variants used by the batch path and the drop-in layer.
 * Data pointers are device pointers (fields [nrhs][3*S] complex double);
 * the channel lists ch (codes 0..5, at most 6) are host arrays. */
int emmi_inject_sources_dev(emmi_solver *s, const float *src_dev, int nch,
                            const int *ch, double *b_dev);
/* adjoint sources from receiver residuals dres_dev [nrhs][nch][nrec]
 * complex float; m_dev: [nrhs][3*S] complex scratch that receives the
 * magnetic part M before b += curl M (inject_extract.c:124-314) */
int emmi_inject_adjoint_dev(emmi_solver *s, const float *rec_dev, int nrec,
                            int nch, const int *ch, const float *dres_dev,
                            double *b_dev, double *m_dev);
/* solve with b already injected into the solver's input buffer (the
 * buffer emmi_modelling_batch injects into); E stays resident, H is formed
 * on the device; x_dev/h_dev (optional) receive copies */
int emmi_solver_solve_resident(emmi_solver *s, double *x_dev, double *h_dev,
                               emmi_rhs_stats *stats);
int emmi_extract_receivers_dev(emmi_solver *s, const float *rec_dev, int nrec,
                               int nch, const int *ch, const double *e_dev,
                               const double *h_dev, float *dcal_dev);

/* Gradient of the data misfit w.r.t. ln(rho) summed over shots
 * (build_gradient.c:13-113 and the MPI_Allreduce of fg_fwi.c:265-268, as a
 * device reduction).  Host arrays: E fields [nshot][nfreq][nz][ny][nx]
 * complex float for the forward (Ef*) and adjoint (Ea*) solves; rho11,
 * rho33 [nz][ny][nx]; bathy [ny][nx]; src [nshot][3]; rec [nshot][nrec][3];
 * idxpar [npar] (1 = rho11/22, 2 = rho33); grad, phess out [npar][nz][ny][nx]
 * (phess when preco == 1, may be NULL otherwise). */
int emmi_build_gradient(int nx, int ny, int nz, const float o[3],
                        const float d[3], int nshot, int nfreq, int npar,
                        const int *idxpar, int preco, const float *E1f,
                        const float *E2f, const float *E3f, const float *E1a,
                        const float *E2a, const float *E3a, const float *rho11,
                        const float *rho33, const float *bathy, const float *src,
                        float dsmute, int nrec, const float *rec, float drmute,
                        float *grad, float *phess);

/* ---- one objective evaluation of the inversion for a batch of shots ----
 * fg_fwi (src/fg_fwi.c:139-290) with every shot and frequency in one
 * solver: the homogenization of the current model for every shot, forward
 * modelling, receiver data, data misfit and adjoint sources (the
 * arithmetic of the host library's eh_misfit), adjoint modelling, and the
 * gradient w.r.t. ln(rho) summed over shots and frequencies
 * (build_gradient.c:13-113 with the MPI_Allreduce of fg_fwi.c:262-268), all
 * on the device; per evaluation only the padded model and the input-grid
 * resistivities go in and the gradient, misfits and data come out.  The
 * model regularization, scaling and optimizer stay with the caller. */
typedef struct {
  int nx, ny, nz;       /* input model cells                                 */
  float o[3], d[3];     /* its origin and cell sizes (emf->ox.., emf->dx..)  */
  int n1, n2, n3;       /* multigrid mesh cells of every shot                */
  int nshot, nfreq;     /* nshot * nfreq <= 65535 right-hand sides           */
  const float *omega;   /* [nfreq] 2*pi*f (emf->omegas)                      */
  const float *x1, *x2, *x3; /* [nshot][n+1] each shot's mesh axes
                           (eh_regrid_axes of the host library)              */
  float rho_water;      /* emf->rho_water of the start model                 */
  int nsrc_ch;          /* source channels, codes 0..5 (Ex..Hz)              */
  const int *src_ch;
  int nrec_ch;          /* receiver channels                                 */
  const int *rec_ch;
  int nrec;             /* receivers per shot, the largest count             */
  const int *nrec_shot; /* [nshot] each shot's receivers (<= nrec)           */
  const float *src;     /* [nshot][5] x, y, z, azimuth, dip (radians)        */
  const float *rec;     /* [nshot][nrec][5]                                  */
  const float *dobs;    /* [nshot][nrec_ch][nfreq][nrec] complex, interleaved*/
  const float *delta;   /* [nshot][nrec_ch][nfreq][nrec] uncertainties       */
  int npar;             /* 1 or 2 parameters                                 */
  const int *idxpar;    /* [npar] 1 = rho11/rho22, 2 = rho33                 */
  int preco;            /* 1: also the pseudo-Hessian                        */
  const float *bathy;   /* [ny][nx] sea-floor depth                          */
  float dsmute, drmute; /* gradient mute half-widths around sources and
                           receivers (fwi->dsmute, fwi->drmute)              */
} emmi_fg_problem;

/* the solver options gmg_init of the drop-in layer takes from the host's
 * key=value parameters (cycleopt ncycle v1 v2 tol isemicoarsen gmg_precision
 * sigma_floor, gmg.c:1712-1717, through getpar or emmi_gpu_set_param) */
void emmi_dropin_options(emmi_options *o, int verb);

typedef struct emmi_fg emmi_fg;
/* copies the survey, data and masks to the device once per inversion; with
 * dobs and delta NULL only emmi_fg_forward may run (npar, idxpar, bathy
 * and the mutes are then not read) */
int emmi_fg_create(emmi_fg **out, const emmi_fg_problem *P,
                   const emmi_options *opts);
/* Forward modelling of every shot and frequency in one solver
 * (do_modelling, src/do_modelling.c:49-67, for all shots at once): the
 * homogenization of the padded model, injection, solve, receiver data
 * dcal [nshot][nrec_ch][nfreq][nrec] (complex, interleaved); stats (may be
 * NULL) [nshot*nfreq].  Host arrays; synchronises. */
int emmi_fg_forward(emmi_fg *f, int nxp, int nyp, int nzp, const float *xx,
                    const float *yy, const float *zz, const float *pad,
                    float *dcal, emmi_rhs_stats *stats);
/* One evaluation at the model whose padded form is xx, yy, zz, pad
 * (eh_pad_model) and whose input-grid resistivities are rho11, rho33
 * [nz][ny][nx]: fcost [nshot] each shot's 0.5*|W(dobs - dcal)|^2, grad and
 * phess (preco == 1; may be NULL) [npar][nz][ny][nx] summed over shots;
 * dcal (complex, interleaved) and rmse (may be NULL) [nshot][nrec_ch]
 * [nfreq][nrec]; stats (may be NULL) [2][nshot*nfreq], forward solves then
 * adjoint.  Host arrays; synchronises. */
int emmi_fg_eval(emmi_fg *f, int nxp, int nyp, int nzp, const float *xx,
                 const float *yy, const float *zz, const float *pad,
                 const float *rho11, const float *rho33, float *fcost,
                 float *grad, float *phess, float *dcal, float *rmse,
                 emmi_rhs_stats *stats);
/* milliseconds of the last evaluation's phases: [0] front end
 * (homogenization), [1] solver set-up (host clock), [2] forward solves,
 * [3] receiver data and forward fields on the model grid, [4] misfit,
 * [5] adjoint sources, [6] adjoint solves, [7] adjoint fields, gradient and
 * copies out (CUDA events on the solver's stream) */
int emmi_fg_phases(const emmi_fg *f, double ms[8]);
void emmi_fg_destroy(emmi_fg *f);
/* The device misfit alone on host arrays (parity checks): per-shot arrays
 * dobs, dcal, dres (complex, interleaved), delta, rmse [nshot][nch][nfreq]
 * [nrec]; src [nshot][5], rec [nshot][nrec][5]; fcost [nshot]. */
int emmi_misfit_batch(int nshot, int nch, int nfreq, int nrec,
                      const int *nrec_shot, const float *omega, float rho_water,
                      const float *src, const float *rec, const float *dobs,
                      const float *delta, const float *dcal, float *dres,
                      float *rmse, float *fcost);

/* Interpolation of E (from x) or H (from h) to the input model's cell
 * centres (extract_electric_field / extract_magnetic_field,
 * inject_extract.c:477-785) for one RHS; host arrays, out [3][nz][ny][nx]
 * complex float.  rho33 is needed for E (the Ez conversion). */
int emmi_extract_volume(emmi_solver *s, int rhs, int which /*0=E 1=H*/,
                        int nx, int ny, int nz, const float o[3],
                        const float d[3], const float *rho33, const double *field,
                        float *out);

/* ---- single-operator entry points for parity checks ------------------ */
/* Each works on one level described by node coordinates (double, n+1 per
 * direction) and volume-weighted cells (double [4][n3][n2][n1]), on host
 * arrays, in FP64 (prec=EMMI_PREC_FP64) or complex64 (EMMI_PREC_MIXED). */
int emmi_level_residual(const int n[3], const double *x1, const double *x2,
                        const double *x3, const double *cells, double omega,
                        int prec, const double *u, const double *f, double *r,
                        double *norm);
/* one grid transfer between a level of nf cells (node coordinates x1..x3)
 * and the level coarsened by sc (1 or 2 per direction, coordinates
 * sub-sampled as gmg.c:1784-1786 builds them): dir 0 restricts the fine
 * complex field in ([3][S_f]) to out ([3][S_c], gmg.c:1510-1573); dir 1 adds
 * the prolongation of the coarse in ([3][S_c]) to out ([3][S_f],
 * gmg.c:1463-1505) */
int emmi_level_transfer(const int nf[3], const double *x1, const double *x2,
                        const double *x3, const int sc[3], int prec, int dir,
                        const double *in, double *out);
/* one multicolour sweep: dir 0..2 = line relaxation along x/y/z,
 * dir 3 = node-patch relaxation; iter%2==1 reverses the colour order */
int emmi_level_smooth(const int n[3], const double *x1, const double *x2,
                      const double *x3, const double *cells, double omega,
                      int prec, int dir, int iter, double *u, const double *f);

/* ---- allocation-free line sweep --------------------------------------- */
/* No counterpart in the reference.  The same sweep as emmi_level_smooth
 * with dir 0..2, for callers that cannot allocate device memory: a program
 * whose memory pool already owns the GPU's HBM, or one whose streams must not
 * be stalled by the device-wide synchronization of cudaMalloc/cudaFree.  It
 * allocates nothing: its scratch (the sweep's band records and the level's
 * geometry) is one static device array of EMMI_NOALLOC_SCRATCH_BYTES that
 * every GPU loading this library holds until the process exits.
 *   cells  device, [4][n3][n2][n1] volume-weighted, double for EMMI_PREC_FP64,
 *          float for EMMI_PREC_MIXED
 *   u, f   device, [3][(n3+1)(n2+1)(n1+1)] complex double / complex float;
 *          u is updated in place
 *   x1..x3 host node coordinates (n_d+1 each); stream may be NULL
 * Levels whose sweep needs more scratch than the maximum, or with n_d
 * outside [2, EMMI_NOALLOC_MAX_N], return EMMI_EINVAL (see emmi_last_error).
 * CUDA loads device code lazily by default, so the array is reserved on a
 * device by the first call there: make one call on each device before the
 * caller's pool takes its HBM (or set CUDA_MODULE_LOADING=EAGER); later calls
 * reserve nothing.  The first call also looks up the array's address on that
 * device and keeps it: do not use the call across cudaDeviceReset.  Each call
 * stages the geometry from host memory, so a call on a stream that is being
 * captured is refused with EMMI_EINVAL.  All calls share the array: calls
 * that overlap on the GPU race, calls ordered on one stream do not. */
#define EMMI_NOALLOC_SCRATCH_BYTES (32u << 20)
#define EMMI_NOALLOC_MAX_N 1024
int emmi_level_line_sweep_noalloc(const int n[3], const double *x1,
                                  const double *x2, const double *x3,
                                  const void *cells, double omega, int prec,
                                  int dir, int iter, void *u, const void *f,
                                  void *stream);

#ifdef __cplusplus
}
#endif
#endif

// Host-side launchers for the multigrid kernels (emmi_kernels.cu).
#pragma once
#include <cuda.h>

#include "emmi_common.cuh"

namespace emmi {

// once per process, before any capture: kernel attributes of the line
// relaxation (shared-memory carveout of the line solve)
void init_line_kernels();

template <typename T, typename TO>
void launch_residual(const LevelView<T>& L, C_t<TO>* rout, double* norm2, cudaStream_t st);

// stored FP64 edge coefficients of level-0 operators (L.nrhs operators,
// L.op unused): coef64_elems doubles per operator; launch_residual_coef is
// launch_residual<double, TO> reading them, bit for bit the same result
long coef64_elems(const int n[3]);
void launch_coef64(const LevelView<double>& L, double* coef, cudaStream_t st);
template <typename TO>
void launch_residual_coef(const LevelView<double>& L, const double* coef, C_t<TO>* rout,
                          double* norm2, cudaStream_t st);

// r = f - A u on level L but only norm (no store)
template <typename T>
void launch_norm(const C_t<T>* v, long n3s, int nrhs, const int* active, double* norm2,
                 cudaStream_t st);

// one colour of line relaxation along direction d; scratch must hold
// (5*n_d-4)*6*lines complex values where lines = nrhs*lines_per_colour.
template <typename T>
void launch_line_sweep(const LevelView<T>& L, int d, int color, C_t<T>* scratch, cudaStream_t st);
long line_count(const int n[3], int d, int color);
long line_scratch_elems(const int n[3], int d, int nrhs);

// stored LDL^T factors of the lines of one colour along d: T values per
// operator group in format fmt (0: fp32 records, 12 values per row; 1: fp16
// L and fp32 1/d, 7 values per row); launch_line_factor fills them for the
// L.nrhs groups of L (L.op / L.wmu per group, u and f unused), the band rows
// assembled in registers, into fac + g * line_factor_elems and sets *ovf
// when an L value does not fit fp16 (format 1); launch_line_sweep_fac then sweeps RHS
// r with the factors of group grp[r], rb holding (5 n_d - 4) * lines complex
// values per RHS
constexpr int kFacF32 = 0, kFacF16 = 1;
long line_factor_elems(const int n[3], int d, int color, int fmt);
template <typename T>
void launch_line_factor(const LevelView<T>& L, int d, int color, T* fac, int fmt, int* ovf,
                        cudaStream_t st);
// block shapes of a stored-factor sweep: the fp16 substitution's variant
// (subst_variant_threads lines per block, a cp.async ring of
// subst_variant_ring rows; 0 = 64 x 6) and the right-hand-side kernel's
// threads per block (256 or 128).  No shape changes any thread's arithmetic.
constexpr int kSubstVariants = 5;
struct SweepShape {
  int subst = 0;
  int rhs_threads = 256;
};
int subst_variant_threads(int v);
int subst_variant_ring(int v);
template <typename T>
void launch_line_sweep_fac(const LevelView<T>& L, int d, int color, const T* fac, const int* grp,
                           C_t<T>* rb, int fmt, cudaStream_t st, SweepShape sh = SweepShape());

// one colour of line relaxation along d in one launch (k_line_fused): each
// thread assembles, factors and solves one line; z waits in L.r (the
// level's residual buffer, dead while the level smooths) at each row's slot
// and the line's multipliers in lbuf, line_l_bytes per RHS: lf = kLExact
// keeps them in T precision, kLHalf (T = float) in fp16 (both substitutions
// use the rounded values; *ovf set when one leaves the fp16 range).  nt:
// lines per block (32, 64 or 128; no value changes any thread's arithmetic)
constexpr int kLExact = 0, kLHalf = 1;
long line_l_bytes(const int n[3], int d, int color, int lf, int tsize);
template <typename T>
void launch_line_fused(const LevelView<T>& L, int d, int color, void* lbuf, int lf, int nt,
                       int* ovf, cudaStream_t st);

// complex64 residual with its halos staged by tensor copies (emmi_stencil.cu):
// tiles of TY rows x KZ planes, plane windows in a ring of shared-memory
// slots.  stencil_prepare sizes the tiles and encodes the tensor maps of a
// level's u (u_elems complex values) and cells (cell_elems floats), both
// allocated in whole 256-byte rows (stencil_pad); false when the level
// cannot be staged, and the plain residual is used.  stencil_err: the word a
// staged launch whose wait ran out sets (nonzero).
struct StencilArgs {
  int TY, KZ;       // rows and planes of a tile
  int ntj, ntk;     // tiles along y and z
  int Ru, Rc;       // 256-byte rows of a u window and of a cell window
  int ncarr;        // cell arrays staged: 3 (sigma) or 4 (+ inverse permeability)
  unsigned uwin, cwin, slot;  // bytes: one u window, one cell window, one slot
  long long wait;   // clocks a wait for a plane's copies gives up after
  int stall = -1;   // test hook: thread 0 issues no copy from this plane on
};
struct StencilPlan {
  CUtensorMap tu, tc;
  StencilArgs args;
  bool ok = false;
};
long stencil_pad(long elems, int esize);
// the wait limit (clocks, 0 = the default) and the test stall of a plan
void stencil_hook(StencilPlan* P, long long wait, int stall);
bool stencil_prepare(const LevelView<float>& V, long u_elems, long cell_elems, StencilPlan* out);
void launch_residual_staged(const LevelView<float>& L, const StencilPlan& P, C_t<float>* rout,
                            double* norm2, cudaStream_t st);
int* stencil_err();

template <typename T>
void launch_point_sweep(const LevelView<T>& L, int color, cudaStream_t st);

// coarse.f = R fine.r ; coarse.u = 0
// LevelView::xw of the transfer F -> Cc for every operator (set-up)
template <typename T>
void launch_xfer_weights(const LevelView<T>& F, const LevelView<T>& Cc, const int sc[3], int nop,
                         T* out, cudaStream_t st);
template <typename T>
void launch_restrict(const LevelView<T>& F, const LevelView<T>& Cc, const int sc[3], cudaStream_t st);
// fine.u += P coarse.u
template <typename T>
void launch_prolong(const LevelView<T>& F, const LevelView<T>& Cc, const int sc[3], cudaStream_t st);

template <typename T>
void launch_coarsen_cells(const T* fine, const int nf[3], T* coarse, const int sc[3], int nrhs,
                          cudaStream_t st);

template <typename T>
void launch_zero(C_t<T>* p, long n, cudaStream_t st);

}  // namespace emmi

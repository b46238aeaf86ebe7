// Internal state of an emmi_solver, shared by the solver and survey units.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "emmi_gpu.h"
#include "emmi_kernels.cuh"

namespace emmi {
constexpr int kMaxLev = 24;
constexpr double kMu0 = 4. * 3.14159265358979323846264 * 1e-7;  // include/cstd.h:38-40

struct HLev {
  int n[3];
  int sc[3];
  long S, ncell;
};

void set_err(const char* fmt, ...);
constexpr int kMaxKrylov = 12;
}  // namespace emmi

struct emmi_solver {
  emmi_options opt;
  int n[3];
  int nop, nrhs, lmax;
  int gmax1, gstride;
  emmi::HLev hier[3][emmi::kMaxLev];
  bool has_norm;  // the cycle has a level-0 norm test
  // block shapes of the stored-factor sweeps per (level, direction): the
  // level-0 ones picked at set-up by timing (opt.autotune), the rest the
  // defaults
  emmi::SweepShape shape[emmi::kMaxLev][3];
  bool tuned_now = false;  // set-up timed shapes (not taken from the cache)

  // device memory
  std::vector<void*> allocs;
  std::vector<size_t> alloc_bytes;  // sizes of allocs, same order
  size_t bytes = 0;
  int* d_op = nullptr;
  int* d_active = nullptr;  // cycling RHS
  int* d_refine = nullptr;  // RHS refining now (MIXED)
  double* d_wmu64 = nullptr;
  float* d_wmu32 = nullptr;
  double* d_norm = nullptr;    // level-0 norm^2 per RHS (cycle)
  double* d_norm64 = nullptr;  // FP64 refinement norm^2 per RHS
  double* geo64[3][emmi::kMaxLev] = {};
  float* geo32[3][emmi::kMaxLev] = {};
  // transfer weights of level l to l+1 per hierarchy (LevelView::xw)
  double* xw64[3][emmi::kMaxLev] = {};
  float* xw32[3][emmi::kMaxLev] = {};
  double* cells64[3][emmi::kMaxLev] = {};
  float* cells32[3][emmi::kMaxLev] = {};
  double2 *u64[emmi::kMaxLev] = {}, *f64[emmi::kMaxLev] = {}, *r64[emmi::kMaxLev] = {};
  float2 *u32[emmi::kMaxLev] = {}, *f32[emmi::kMaxLev] = {}, *r32[emmi::kMaxLev] = {};
  long u32_elems[emmi::kMaxLev] = {};  // complex values of u32[l] (before padding)
  // staged residual (opt.staged, MIXED): tile plans and tensor maps per
  // (hierarchy, level); ok false where a level cannot be staged
  emmi::StencilPlan plan[3][emmi::kMaxLev];
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  int chunk = 1;  // RHS per line-sweep launch (scratch bound)

  // survey data: float grids as emf_t holds them after regrid_init
  // ([nop][9][gmax1]: x1 x2 x3 x1s x2s x3s d1 d2 d3), the raw float cells
  // ([nop][4][ncell]) and rho_water per operator
  float* sgeo = nullptr;
  float* raw_cells = nullptr;
  float* d_rho_water = nullptr;
  float* d_omega = nullptr;  // [nrhs] float omega as the reference stores it
  std::vector<float> h_omega;
  std::vector<int> h_op;

  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // side stream of the set-up work no step needs at once (the stored FP64
  // coefficients), and the event the first use waits for
  cudaStream_t st2 = nullptr;
  cudaEvent_t ev_coef = nullptr;
  bool coef_pending = false;
  cudaGraphExec_t gA[3] = {}, gB[3] = {};
  long nodesA[3] = {}, nodesB[3] = {};
  double last_time = 0;
  long last_launches = 0;
  long launch_counter = 0;

  std::vector<int> h_active, h_refine;

  // stored line factors (opt.line_factors): RHS sharing an operator and a
  // frequency form a group; d_fac holds the LDL^T factors of every line per
  // group, in blocks per (hierarchy, level, direction, colour) at offsets
  // fac_off in elements of the working precision (-1: none; level 0 is
  // shared by the hierarchies)
  bool fac_on = false;
  int fac_fmt = 0;          // 0: records in working precision; 1: fp16 L with fp32 1/d
  int ngroups = 0;
  int* d_grp = nullptr;     // [nrhs] group of each RHS
  int* d_gop = nullptr;     // [ngroups] operator of each group
  void* d_gwmu = nullptr;   // [ngroups] omega*mu0 of each group (working precision)
  void* d_fac = nullptr;
  size_t fac_bytes = 0;
  long fac_off[3][emmi::kMaxLev][3][4];

  // one-launch line sweep (opt.line_sweep): multiplier format (kLHalf only
  // for MIXED with line_factors = 2), the device flag an fp16 multiplier out
  // of range sets, and lines per block per (level, direction)
  int lfmt = 0;
  // every operator's input invmur is exactly 1: the complex64 operator takes
  // its coefficients from the spacings (LevelView::imu_vol)
  bool imu_vol = false;
  int* d_lovf = nullptr;
  int fused_nt[emmi::kMaxLev][3];

  // stored FP64 edge coefficients of the level-0 true operators (MIXED):
  // the refinement residual reads them instead of recomputing (null: off)
  double* d_coef64 = nullptr;

  // FGMRES (MIXED, opt.krylov > 0): basis kv [m+1][nrhs][3S] FP64,
  // preconditioned directions kz [m][nrhs][3S] complex64, FP64 temporaries
  // kt (-z) and kw (A z) [nrhs][3S]; per RHS: Hessenberg column d_kh
  // [nrhs][kMaxKrylov+1], solution weights d_ky [nrhs][kMaxKrylov], basis
  // scale d_kscale and basis index d_kj
  int kry_m = 0;
  double2* kv = nullptr;
  float2* kz = nullptr;
  double2 *kt = nullptr, *kw = nullptr;
  double2 *d_kh = nullptr, *d_ky = nullptr;
  double* d_kscale = nullptr;
  int* d_kj = nullptr;

  // learned correction after each complex64 cycle (level 0): fp32 master
  // weights and their tensor-core B operands, bf16 input/hidden slots
  // [nrhs][S][8] between zero guards, per-RHS enable mask (cleared for a RHS
  // that falls back to plain cycles)
  bool learned_on = false;
  // emmi_learned_apply's wait limit (clocks, 0 = default) and test stall
  long long ls_wait = 0;
  int ls_stall = 0;
  float* d_lsW = nullptr;
  uint4* d_lsWt = nullptr;
  uint32_t *d_lsX = nullptr, *d_lsH = nullptr;
  int* d_learn = nullptr;
  std::vector<int> h_learn, h_fallback;
  // training set: complex64 level-0 residuals [cap][3][S], their |r|^2,
  // operator and omega*mu0 per sample; snapshots are taken after each cycle
  // of a solve while ls_collect is set, at most ls_per_rhs per RHS
  bool ls_collect = false;
  int ls_cap = 0, ls_count = 0, ls_per_rhs = 0;
  float2* d_samples = nullptr;
  double* d_srn2 = nullptr;
  int* d_sop = nullptr;
  float* d_swmu = nullptr;
  std::vector<int> h_sop, h_taken;

  template <typename T> emmi::LevelView<T> view(int h, int l) const;
  template <typename T> void emit_smooth(int h, int l, int iter);
  template <typename T>
  void resid(int h, int l, const emmi::LevelView<T>& V, emmi::C_t<T>* rout, double* norm2);
  template <typename T> void emit_cycle(int h, int l, int kind, int want, int& cur);
  template <typename T> void emit_residual0(int want, int& cur);
  template <typename T> int build_graphs();
  int alloc(void** p, size_t b);
  void release(void* p);  // frees one allocation made by alloc
};

// one part of a cycle on hierarchy h (graph launch or direct emission)
int run_part(emmi_solver* s, int h, int part);
// the one-launch line sweep with fp16 multipliers saw one out of range
// (reads the device flag; synchronizes the solver's stream): from then on
// it keeps working-precision multipliers and the cycle graphs are
// recaptured.  Returns 1 when it switched, 0 when nothing happened, <0 on a
// CUDA error
int line_format_fallback(emmi_solver* s);

// FP64 r = f - A u on level 0 with the true operator (V a level-0 FP64
// view): from the stored coefficients when the solver keeps them
template <typename TO>
inline void true_residual64(emmi_solver* s, const emmi::LevelView<double>& V, emmi::C_t<TO>* rout,
                            double* norm2) {
  if (s->coef_pending) {  // the coefficients come from the side stream
    cudaStreamWaitEvent(s->st, s->ev_coef, 0);
    s->coef_pending = false;
  }
  if (s->d_coef64)
    emmi::launch_residual_coef<TO>(V, s->d_coef64, rout, norm2, s->st);
  else
    emmi::launch_residual<double, TO>(V, rout, norm2, s->st);
}

namespace emmi {
// FGMRES workspace for opt.krylov > 0 (called by emmi_solver_create)
int krylov_alloc(emmi_solver* s);
// FP64 FGMRES around complex64 cycles; expects f64[0] = b*vol and u64[0] = 0
// on the solver's stream; fills the per-RHS statistics
int krylov_solve(emmi_solver* s, std::vector<int>& cycles, std::vector<int>& status,
                 std::vector<int>& nref, std::vector<double>& rnorm0, std::vector<double>& rn);
// after a cycle on hierarchy h: the learned correction of the RHS that are
// active and enabled (act = host copy of d_active)
int learned_after_cycle(emmi_solver* s, int h, const std::vector<int>& act);
// after a cycle: snapshot the level-0 complex64 residuals into the training set
int learned_snapshot(emmi_solver* s, int h, const std::vector<int>& act);
// a RHS that stalls with the learned correction drops back to plain cycles;
// returns true when it did
bool learned_fallback(emmi_solver* s, int r);
// nonzero when a learned-correction convolution gave up waiting since the
// last call (synchronises the stream; clears the record)
int learned_check(cudaStream_t st);
}  // namespace emmi

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
}  // namespace emmi

struct emmi_solver {
  emmi_options opt;
  int n[3];
  int nop, nrhs, lmax;
  int gmax1, gstride;
  emmi::HLev hier[3][emmi::kMaxLev];
  bool has_norm;  // the cycle has a level-0 norm test

  // device memory
  std::vector<void*> allocs;
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
  double* cells64[3][emmi::kMaxLev] = {};
  float* cells32[3][emmi::kMaxLev] = {};
  double2 *u64[emmi::kMaxLev] = {}, *f64[emmi::kMaxLev] = {}, *r64[emmi::kMaxLev] = {};
  float2 *u32[emmi::kMaxLev] = {}, *f32[emmi::kMaxLev] = {}, *r32[emmi::kMaxLev] = {};
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
  cudaGraphExec_t gA[3] = {}, gB[3] = {};
  long nodesA[3] = {}, nodesB[3] = {};
  double last_time = 0;
  long last_launches = 0;
  long launch_counter = 0;

  std::vector<int> h_active, h_refine;

  template <typename T> emmi::LevelView<T> view(int h, int l) const;
  template <typename T> void emit_smooth(int h, int l, int iter);
  template <typename T> void emit_cycle(int h, int l, int kind, int want, int& cur);
  template <typename T> void emit_residual0(int want, int& cur);
  template <typename T> int build_graphs();
  int alloc(void** p, size_t b);
};

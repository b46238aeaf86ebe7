// Host-side launchers for the multigrid kernels (emmi_kernels.cu).
#pragma once
#include "emmi_common.cuh"

namespace emmi {

// line-relaxation band table: for direction D, row type t (0: E_D(s-1),
// 1: E_a(ta-1), 2: E_a(ta), 3: E_b(tb-1), 4: E_b(tb)) and neighbour k of the
// row's edge equation, the band offset of that neighbour on the line, or
// 127 if it is not a line unknown.  Filled once per process.
void init_line_tables();

template <typename T, typename TO>
void launch_residual(const LevelView<T>& L, C_t<TO>* rout, double* norm2, cudaStream_t st);

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

template <typename T>
void launch_point_sweep(const LevelView<T>& L, int color, cudaStream_t st);

// coarse.f = R fine.r ; coarse.u = 0
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

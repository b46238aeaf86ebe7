// Batched multigrid solver for the curl-curl Maxwell system on GB300.
//
// A batch holds nrhs right-hand sides over nop operators (grid +
// conductivity); all share n1 x n2 x n3.  The cycle structure is the
// reference's (src/gmg.c:1586-1668, 1894-1932): F/V/W cycles, the level-0
// residual-norm stopping test, and semi-coarsening whose uncoarsened
// direction rotates with the cycle index (gmg.c:1755).  The three rotation
// states give three fixed level hierarchies, built once at setup instead of
// per cycle (gmg.c:1912), each captured into CUDA graphs:
//   part A  = the work up to and including the level-0 residual and its norm
//   part B  = the rest of the cycle
// so the host can stop a right-hand side exactly where the reference would
// (before the cycle's work) with one small device-to-host read per cycle.
//
// EMMI_PREC_FP64 runs the cycles in complex128 (the reference's arithmetic).
// EMMI_PREC_MIXED runs them in complex64 on a preconditioner operator whose
// conductivity is floored at sigma_floor (the air layer at 1e-8 S/m makes the
// complex64 block solves unstable), and refines in FP64: x += e,
// r = b - A x with the true operator in FP64, until |r| <= tol |b|.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <map>
#include <mutex>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "emmi_gpu.h"
#include "emmi_solver_impl.cuh"

using namespace emmi;

static thread_local std::string g_err;

void emmi::set_err(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
}

namespace {


#define CK(x)                                                                     \
  do {                                                                            \
    cudaError_t e_ = (x);                                                         \
    if (e_ != cudaSuccess) {                                                      \
      set_err("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_));   \
      return EMMI_ECUDA;                                                          \
    }                                                                             \
  } while (0)


// gmg.c:1688-1699
int depth_of(int n) {
  int l = 0, nn = n;
  while (nn % 2 == 0 && nn > 1) {
    l++;
    nn >>= 1;
  }
  if (nn > 2) l++;
  return l;
}

// x -> xs, d, ds (gmg.c:1672-1685)
void stagger(int n, const double* x, double* xs, double* d, double* ds) {
  for (int i = 0; i < n; i++) {
    ds[i] = x[i + 1] - x[i];
    xs[i] = 0.5 * (x[i] + x[i + 1]);
  }
  xs[n] = x[n] + 0.5 * ds[n - 1];
  ds[n] = xs[n] - x[n];
  for (int i = 1; i <= n; i++) d[i] = xs[i] - xs[i - 1];
  d[0] = xs[0] - x[0];
}


// ------------------------------------------------------------ setup kernels
// cells64 = raw * vol, vol = d1s*d2s*d3s (gmg.c:1795-1799); sigmas floored at
// `floor` (invmur untouched); also writes a float copy when c32 != null.
// *flag = 1 where an operator's raw invmur (array 3 of [op][4][ncell]) is not
// exactly 1
__global__ void k_not_one(const float* __restrict__ raw, long ncell, int* __restrict__ flag) {
  const float* imu = raw + ((long)blockIdx.y * 4 + 3) * ncell;
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < ncell;
       c += (long)gridDim.x * blockDim.x)
    if (imu[c] != 1.0f) *flag = 1;
}

__global__ void k_weight_cells(const float* __restrict__ raw, const double* __restrict__ geo,
                               int gstride, int gmax1, int n0, int n1, int n2, double floor,
                               double* __restrict__ c64, float* __restrict__ c32) {
  const long ncell = (long)n0 * n1 * n2;
  const long id = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (id >= ncell) return;
  const int op = blockIdx.y;
  // 32-bit decode (a level has fewer than 2^31 cells)
  const unsigned t = (unsigned)id / (unsigned)n0;
  const int i = (int)((unsigned)id - t * (unsigned)n0);
  const int j = (int)(t % (unsigned)n1), k = (int)(t / (unsigned)n1);
  const double* g = geo + (long)op * gstride;
  const double vol = g[3 * gmax1 + i] * g[4 * gmax1 + j] * g[5 * gmax1 + k];
  for (int a = 0; a < 4; a++) {
    double s = raw[((long)op * 4 + a) * ncell + id];
    if (a < 3 && s < floor) s = floor;
    const double v = s * vol;
    if (c64) c64[((long)op * 4 + a) * ncell + id] = v;
    if (c32) c32[((long)op * 4 + a) * ncell + id] = (float)v;
  }
}

__global__ void k_d2f(const double* __restrict__ a, float* __restrict__ b, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// f = b * dual volume (gmg.c:1901-1910)
__global__ void k_scale_dual(const double2* __restrict__ b, double2* __restrict__ f,
                             const double* __restrict__ geo, const int* __restrict__ op, int gstride,
                             int gmax1, int n0, int n1, int n2) {
  const long S = (long)(n0 + 1) * (n1 + 1) * (n2 + 1);
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= S) return;
  const int rhs = blockIdx.y;
  const int o = op ? op[rhs] : rhs;
  const int i = (int)(s % (n0 + 1)), j = (int)((s / (n0 + 1)) % (n1 + 1)),
            k = (int)(s / ((long)(n0 + 1) * (n1 + 1)));
  const double* g = geo + (long)o * gstride;
  const double d1s = g[3 * gmax1 + i], d2s = g[4 * gmax1 + j], d3s = g[5 * gmax1 + k];
  const double d1 = g[6 * gmax1 + i], d2 = g[7 * gmax1 + j], d3 = g[8 * gmax1 + k];
  const long base = (long)rhs * 3 * S;
  const double w[3] = {d1s * d2 * d3, d1 * d2s * d3, d1 * d2 * d3s};
  for (int c = 0; c < 3; c++) {
    const double2 v = b[base + c * S + s];
    f[base + c * S + s] = make_double2(v.x * w[c], v.y * w[c]);
  }
}

// The first residual of a mixed solve, where x = 0: r = b*vol exactly, so
// f32 = (float) f64, u32 = 0 and |r|^2 need no operator application
__global__ void __launch_bounds__(256) k_first_residual(const double2* __restrict__ f64,
                                                        float2* __restrict__ f32,
                                                        float2* __restrict__ u32, long n3s,
                                                        const int* __restrict__ mask,
                                                        double* __restrict__ norm2) {
  const int rhs = blockIdx.y;
  if (mask && !mask[rhs]) return;
  double acc = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n3s; i += (long)gridDim.x * blockDim.x) {
    const double2 v = f64[(long)rhs * n3s + i];
    f32[(long)rhs * n3s + i] = make_float2((float)v.x, (float)v.y);
    u32[(long)rhs * n3s + i] = make_float2(0.f, 0.f);
    acc += v.x * v.x + v.y * v.y;
  }
  __shared__ double red[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) v += red[k];
    atomicAdd(norm2 + rhs, v);
  }
}

// x64 += e32 on masked RHS
__global__ void k_accumulate(double2* __restrict__ x, const float2* __restrict__ e, long n3s,
                             const int* __restrict__ mask) {
  const int rhs = blockIdx.y;
  if (mask && !mask[rhs]) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n3s; i += (long)gridDim.x * blockDim.x) {
    const float2 v = e[(long)rhs * n3s + i];
    double2 a = x[(long)rhs * n3s + i];
    a.x += (double)v.x;
    a.y += (double)v.y;
    x[(long)rhs * n3s + i] = a;
  }
}

__global__ void k_zero_masked(float2* __restrict__ p, long n3s, const int* __restrict__ mask) {
  const int rhs = blockIdx.y;
  if (mask && !mask[rhs]) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n3s; i += (long)gridDim.x * blockDim.x)
    p[(long)rhs * n3s + i] = make_float2(0.f, 0.f);
}

// H = curl E / (i wmu) on faces (gmg.c:1414-1460)
__global__ void k_curl_h(const double2* __restrict__ E, double2* __restrict__ H,
                         const double* __restrict__ geo, const int* __restrict__ op,
                         const double* __restrict__ wmu, int gstride, int gmax1, int n0, int n1,
                         int n2) {
  const long S = (long)(n0 + 1) * (n1 + 1) * (n2 + 1);
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= S) return;
  const int rhs = blockIdx.y;
  const int o = op ? op[rhs] : rhs;
  const int i = (int)(s % (n0 + 1)), j = (int)((s / (n0 + 1)) % (n1 + 1)),
            k = (int)(s / ((long)(n0 + 1) * (n1 + 1)));
  const long base = (long)rhs * 3 * S;
  if (i >= n0 || j >= n1 || k >= n2) {
    for (int c = 0; c < 3; c++) H[base + c * S + s] = make_double2(0, 0);
    return;
  }
  const double* g = geo + (long)o * gstride;
  const double d1s = g[3 * gmax1 + i], d2s = g[4 * gmax1 + j], d3s = g[5 * gmax1 + k];
  const long si = 1, sj = n0 + 1, sk = (long)(n0 + 1) * (n1 + 1);
  const double2* Ex = E + base;
  const double2* Ey = E + base + S;
  const double2* Ez = E + base + 2 * S;
  auto sub = [](double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); };
  auto sc = [](double2 a, double d) { return make_double2(a.x / d, a.y / d); };
  const double2 t1 = sub(sc(sub(Ez[s + sj], Ez[s]), d2s), sc(sub(Ey[s + sk], Ey[s]), d3s));
  const double2 t2 = sub(sc(sub(Ex[s + sk], Ex[s]), d3s), sc(sub(Ez[s + si], Ez[s]), d1s));
  const double2 t3 = sub(sc(sub(Ey[s + si], Ey[s]), d1s), sc(sub(Ex[s + sj], Ex[s]), d2s));
  // t / (i w) = (t.y/w, -t.x/w)
  const double w = wmu[rhs];
  H[base + s] = make_double2(t1.y / w, -t1.x / w);
  H[base + S + s] = make_double2(t2.y / w, -t2.x / w);
  H[base + 2 * S + s] = make_double2(t3.y / w, -t3.x / w);
}

inline unsigned blocks_for(long n, int bs = 256, long cap = 65535) {
  long b = (n + bs - 1) / bs;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace


// Solver memory comes from the device's stream-ordered pool on the solver's
// stream; freed memory stays in the pool (release threshold raised once per
// device) so that destroying and creating solvers does not map and unmap
// device memory each time.  emmi_trim_memory gives it back.
static void keep_pool_memory() {
  static std::once_flag once[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
  std::call_once(once[dev], [dev] {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess) return;
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  });
}

// device memory a new allocation can have: free memory plus what the pool
// holds unused
static size_t device_avail() {
  size_t freeb = 0, totb = 0;
  if (cudaMemGetInfo(&freeb, &totb) != cudaSuccess) return 0;
  int dev = 0;
  cudaMemPool_t pool;
  if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t res = 0, used = 0;
    cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &res);
    cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used);
    if (res > used) freeb += (size_t)(res - used);
  }
  return freeb;
}

int emmi_solver::alloc(void** p, size_t b) {
  if (b == 0) b = 16;
  cudaError_t e = cudaMallocAsync(p, b, st);
  if (e != cudaSuccess) {
    set_err("cudaMalloc(%zu) failed: %s", b, cudaGetErrorString(e));
    return EMMI_ENOMEM;
  }
  allocs.push_back(*p);
  alloc_bytes.push_back(b);
  bytes += b;
  return EMMI_OK;
}

void emmi_solver::release(void* p) {
  for (size_t i = 0; i < allocs.size(); i++)
    if (allocs[i] == p) {
      cudaFreeAsync(p, st);
      bytes -= alloc_bytes[i];
      allocs.erase(allocs.begin() + i);
      alloc_bytes.erase(alloc_bytes.begin() + i);
      return;
    }
}

template <>
LevelView<double> emmi_solver::view<double>(int h, int l) const {
  LevelView<double> V;
  const HLev& H = hier[h][l];
  for (int e = 0; e < 3; e++) V.n[e] = H.n[e];
  V.nrhs = nrhs;
  V.S = H.S;
  V.ncell = H.ncell;
  V.gstride = gstride;
  V.gmax1 = gmax1;
  V.geo = geo64[h][l];
  V.xw = xw64[h][l];
  V.cells = cells64[h][l];
  V.u = u64[l];
  V.f = f64[l];
  V.r = r64[l];
  V.wmu = d_wmu64;
  V.active = d_active;
  V.op = d_op;
  set_slot_divs(V);
  return V;
}

template <>
LevelView<float> emmi_solver::view<float>(int h, int l) const {
  LevelView<float> V;
  const HLev& H = hier[h][l];
  for (int e = 0; e < 3; e++) V.n[e] = H.n[e];
  V.nrhs = nrhs;
  V.S = H.S;
  V.ncell = H.ncell;
  V.gstride = gstride;
  V.gmax1 = gmax1;
  V.geo = geo32[h][l];
  V.xw = xw32[h][l];
  V.cells = cells32[h][l];
  V.u = u32[l];
  V.f = f32[l];
  V.r = r32[l];
  V.wmu = d_wmu32;
  V.active = d_active;
  V.op = d_op;
  V.imu_vol = imu_vol ? 1 : 0;
  set_slot_divs(V);
  return V;
}

// one colour of line relaxation along d on level l of hierarchy h for the
// RHS chunk W starting at r0: with the stored factors of the colour when the
// complex64 solver keeps them, else factoring in the sweep
template <typename T>
static void line_colour(emmi_solver* s, int h, int l, int d, int col, const LevelView<T>& W,
                        int r0) {
  if (s->opt.line_sweep || l >= s->opt.fused_level) {
    const int lf = std::is_same<T, float>::value ? s->lfmt : kLExact;
    launch_line_fused<T>(W, d, col, s->scratch, lf, s->fused_nt[l][d], s->d_lovf, s->st);
    return;
  }
  if (s->fac_on) {
    const long off = s->fac_off[l == 0 ? 0 : h][l][d][col];
    if (off >= 0) {
      launch_line_sweep_fac<T>(W, d, col, static_cast<const T*>(s->d_fac) + off, s->d_grp + r0,
                               (C_t<T>*)s->scratch, s->fac_fmt, s->st, s->shape[l][d]);
      return;
    }
  }
  launch_line_sweep<T>(W, d, col, (C_t<T>*)s->scratch, s->st);
}

// kernel launches of one colour of line relaxation along d on level l of
// hierarchy h (what line_colour emits per RHS chunk)
static int line_launches(const emmi_solver* s, int h, int l, int d) {
  if (s->opt.line_sweep || l >= s->opt.fused_level) return 1;  // k_line_fused
  if (s->fac_on && s->fac_off[l == 0 ? 0 : h][l][d][0] >= 0)
    return (s->fac_fmt == kFacF16 && d != 0) ? 2 : 3;  // update in the substitution
  return 3;
}

// smoothing (gmg.c:1301-1313): line relaxation along every direction the
// next level coarsens, else node-patch relaxation; odd iter reverses colours
template <typename T>
void emmi_solver::emit_smooth(int h, int l, int iter) {
  LevelView<T> V = view<T>(h, l);
  const bool rev = iter % 2 == 1;
  if (opt.isemicoarsen && l < lmax - 1) {
    for (int d = 0; d < 3; d++) {
      if (hier[h][l + 1].sc[d] != 2) continue;
      for (int cc = 0; cc < 4; cc++) {
        const int col = rev ? 3 - cc : cc;
        for (int r0 = 0; r0 < nrhs; r0 += chunk) {
          LevelView<T> W = V;
          const int nr = std::min(chunk, nrhs - r0);
          W.nrhs = nr;
          W.u += (long)r0 * 3 * V.S;
          W.f += (long)r0 * 3 * V.S;
          W.r += (long)r0 * 3 * V.S;
          W.wmu += r0;
          W.active += r0;
          W.op += r0;
          line_colour<T>(this, h, l, d, col, W, r0);
          launch_counter += line_launches(this, h, l, d);
        }
      }
    }
  } else {
    for (int cc = 0; cc < 8; cc++) {
      launch_point_sweep<T>(V, rev ? 7 - cc : cc, st);
      launch_counter++;
    }
  }
}

// r = f - A u of level l of hierarchy h (view V): the staged kernel where
// the level has a plan, else the plain one
template <typename T>
void emmi_solver::resid(int h, int l, const LevelView<T>& V, C_t<T>* rout, double* norm2) {
  if constexpr (std::is_same<T, float>::value) {
    if (plan[h][l].ok) {
      launch_residual_staged(V, plan[h][l], rout, norm2, st);
      return;
    }
  }
  launch_residual<T, T>(V, rout, norm2, st);
}

// level-0 residual with norm: the point where the cycle tests convergence
template <typename T>
void emmi_solver::emit_residual0(int want, int& cur) {
  if (cur == want) {
    cudaMemsetAsync(d_norm, 0, nrhs * sizeof(double), st);
    LevelView<T> V = view<T>(0, 0);
    resid<T>(0, 0, V, V.r, d_norm);
    launch_counter++;
  }
  cur = 1;
}

// kind: 1 V, 2 F, 3 W (gmg.c:1586-1668).  Emits only the launches of part
// `want` (0 = before/including the level-0 norm, 1 = after it).
template <typename T>
void emmi_solver::emit_cycle(int h, int l, int kind, int want, int& cur) {
  auto can_descend = [&](int lv) {
    return lv < lmax - 1 && hier[h][lv + 1].sc[0] * hier[h][lv + 1].sc[1] * hier[h][lv + 1].sc[2] > 1;
  };
  auto to_coarse = [&](int lv) {
    if (cur == want) {
      launch_restrict<T>(view<T>(h, lv), view<T>(h, lv + 1), hier[h][lv + 1].sc, st);
      launch_counter++;
    }
  };
  auto to_fine = [&](int lv) {
    if (cur == want) {
      launch_prolong<T>(view<T>(h, lv), view<T>(h, lv + 1), hier[h][lv + 1].sc, st);
      launch_counter++;
    }
  };
  auto residual = [&](int lv) {
    if (lv == 0 && kind == opt.cycleopt) {
      emit_residual0<T>(want, cur);
    } else if (cur == want) {
      LevelView<T> V = view<T>(h, lv);
      resid<T>(h, lv, V, V.r, nullptr);
      launch_counter++;
    }
  };
  auto smooth = [&](int lv, int it) {
    if (cur == want) emit_smooth<T>(h, lv, it);
  };
  if (kind == 2) {  // F
    if (l == lmax - 1) {
      if (cur == want) {
        LevelView<T> V = view<T>(h, l);
        launch_zero<T>(V.u, 3 * V.S * nrhs, st);
        launch_counter++;
      }
    } else if (can_descend(l)) {
      residual(l);
      to_coarse(l);
      emit_cycle<T>(h, l + 1, 2, want, cur);
      to_fine(l);
    }
    emit_cycle<T>(h, l, 1, want, cur);
    return;
  }
  // V (kind 1) and W (kind 3); levels whose bit is set in skip_pre /
  // skip_post leave out that smoothing
  if (!((opt.skip_pre >> l) & 1))
    for (int i = 0; i < opt.v1; i++) smooth(l, i);
  if (can_descend(l)) {
    residual(l);
    to_coarse(l);
    emit_cycle<T>(h, l + 1, kind, want, cur);
    if (kind == 3) emit_cycle<T>(h, l + 1, kind, want, cur);
    to_fine(l);
  }
  if (!((opt.skip_post >> l) & 1))
    for (int i = 0; i < opt.v2; i++) smooth(l, i);
}

template <typename T>
int emmi_solver::build_graphs() {
  for (int h = 0; h < 3; h++) {
    for (int part = 0; part < 2; part++) {
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      long before = launch_counter;
      int cur = 0;
      if (opt.cycleopt == 2) {
        // F-cycle: the only level-0 residual of the top call is the norm one
        emit_cycle<T>(h, 0, 2, part, cur);
      } else {
        emit_cycle<T>(h, 0, opt.cycleopt, part, cur);
      }
      CK(cudaStreamEndCapture(st, &g));
      size_t nn = 0;
      cudaGraphGetNodes(g, nullptr, &nn);
      (part ? nodesB : nodesA)[h] = launch_counter - before;
      CK(cudaGraphInstantiate(part ? &gB[h] : &gA[h], g, 0));
      cudaGraphDestroy(g);
    }
  }
  launch_counter = 0;
  return EMMI_OK;
}

// Stored line factors of the complex64 cycle: group the RHS by (operator,
// frequency), size the factor blocks of every (hierarchy, level, direction,
// colour) the smoother relaxes, and factor each group's lines once.  Leaves
// fac_on false (factoring in every sweep) when they would take more than
// half of the free device memory.
template <typename T>
static int build_line_factors(emmi_solver* s) {
  const int nrhs = s->nrhs;
  std::vector<int> grp(nrhs), gop;
  std::vector<T> gw;
  for (int r = 0; r < nrhs; r++) {
    const T w = (T)((double)s->h_omega[r] * kMu0);
    int g = -1;
    for (int k = 0; k < (int)gop.size() && g < 0; k++)
      if (gop[k] == s->h_op[r] && gw[k] == w) g = k;
    if (g < 0) {
      g = (int)gop.size();
      gop.push_back(s->h_op[r]);
      gw.push_back(w);
    }
    grp[r] = g;
  }
  const int ng = (int)gop.size();
  // complex64: fp16 L (the default, line_factors = 2) unless a value leaves
  // its range, then every factor is recomputed in fp32; complex128: records
  // in FP64
  int fmt = (std::is_same<T, float>::value && s->opt.line_factors == 2) ? kFacF16 : kFacF32;
  int* d_ovf = nullptr;
  int rc;
  if ((rc = s->alloc((void**)&d_ovf, sizeof(int))) != EMMI_OK) return rc;
  for (;;) {
    for (int h = 0; h < 3; h++)
      for (int l = 0; l < emmi::kMaxLev; l++)
        for (int d = 0; d < 3; d++)
          for (int c = 0; c < 4; c++) s->fac_off[h][l][d][c] = -1;
    // level 0 is the same in every hierarchy: its blocks live under h = 0
    long total = 0;
    for (int h = 0; h < 3; h++)
      for (int l = 0; l + 1 < s->lmax; l++)
        for (int d = 0; d < 3; d++) {
          if (!s->opt.isemicoarsen || s->hier[h][l + 1].sc[d] != 2) continue;
          if (l >= s->opt.fused_level) continue;  // swept by the one-launch kernel
          const int hb = l == 0 ? 0 : h;
          if (s->fac_off[hb][l][d][0] >= 0) continue;
          for (int c = 0; c < 4; c++) {
            s->fac_off[hb][l][d][c] = total;
            total += (long)ng * line_factor_elems(s->hier[h][l].n, d, c, fmt);
          }
        }
    if (total == 0) return EMMI_OK;
    const size_t freeb = device_avail();
    const size_t bytes = (size_t)total * sizeof(T);
    if (bytes > freeb / 2) return EMMI_OK;  // factor in every sweep instead
    if ((rc = s->alloc((void**)&s->d_fac, bytes)) != EMMI_OK) return rc;
    if (!s->d_grp) {
      if ((rc = s->alloc((void**)&s->d_grp, nrhs * sizeof(int))) != EMMI_OK) return rc;
      if ((rc = s->alloc((void**)&s->d_gop, ng * sizeof(int))) != EMMI_OK) return rc;
      if ((rc = s->alloc((void**)&s->d_gwmu, ng * sizeof(T))) != EMMI_OK) return rc;
      CK(cudaMemcpyAsync(s->d_grp, grp.data(), nrhs * sizeof(int), cudaMemcpyHostToDevice,
                         s->st));
      CK(cudaMemcpyAsync(s->d_gop, gop.data(), ng * sizeof(int), cudaMemcpyHostToDevice, s->st));
      CK(cudaMemcpyAsync(s->d_gwmu, gw.data(), ng * sizeof(T), cudaMemcpyHostToDevice, s->st));
    }
    CK(cudaMemsetAsync(d_ovf, 0, sizeof(int), s->st));
    s->ngroups = ng;
    s->fac_bytes = bytes;
    // factor every block once, every group in one launch per colour
    std::vector<long> done;
    for (int h = 0; h < 3; h++)
      for (int l = 0; l + 1 < s->lmax; l++)
        for (int d = 0; d < 3; d++) {
          if (!s->opt.isemicoarsen || s->hier[h][l + 1].sc[d] != 2) continue;
          if (l >= s->opt.fused_level) continue;  // swept by the one-launch kernel
          const int hb = l == 0 ? 0 : h;
          const long off0 = s->fac_off[hb][l][d][0];
          if (std::find(done.begin(), done.end(), off0) != done.end()) continue;
          done.push_back(off0);
          LevelView<T> V = s->view<T>(h, l);
          V.op = s->d_gop;
          V.wmu = static_cast<const T*>(s->d_gwmu);
          V.active = nullptr;
          V.nrhs = ng;
          for (int c = 0; c < 4; c++)
            launch_line_factor<T>(V, d, c, static_cast<T*>(s->d_fac) + s->fac_off[hb][l][d][c], fmt,
                                  d_ovf, s->st);
        }
    CK(cudaGetLastError());
    int ovf = 0;
    CK(cudaMemcpyAsync(&ovf, d_ovf, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    if (fmt == kFacF16 && ovf) {
      s->release(s->d_fac);
      s->d_fac = nullptr;
      fmt = kFacF32;
      continue;
    }
    break;
  }
  s->release(d_ovf);
  s->fac_fmt = fmt;
  s->fac_on = true;
  return EMMI_OK;
}

// ---- autotuning of the level-0 sweep shapes ------------------------------
// The stored-factor line sweep of each direction is timed at set-up on this
// solver's own level-0 operators (zero fields) for a few block shapes -- the
// right-hand-side kernel's threads per block, then the fp16 substitution's
// lines per block and ring depth -- and the fastest is kept when it beats
// the incumbent by more than 2 %.  No shape changes any result.  Choices are
// cached for the process by (grid, RHS per launch, RHS, factor format,
// direction), so later solvers of the same shape take them without timing.
static std::mutex g_tune_mu;
static std::map<std::array<long, 7>, emmi::SweepShape> g_tune;
static bool g_tune_loaded = false;

// The cache persists across processes in the JSON file named by
// EMMI_TUNE_FILE when that is set: read once before the first tuning,
// rewritten whole after every new entry.  Each entry lists, in this order,
// grid (3), chunk, nrhs, fmt, dir, subst, rhs_threads; entries that do not
// read as nine integers are skipped.  Call with g_tune_mu held.
static void tune_file_load() {
  g_tune_loaded = true;
  const char* path = std::getenv("EMMI_TUNE_FILE");
  if (!path || !*path) return;
  FILE* fp = std::fopen(path, "r");
  if (!fp) return;
  std::string text;
  char buf[4096];
  size_t k;
  while ((k = std::fread(buf, 1, sizeof(buf), fp)) > 0) text.append(buf, k);
  std::fclose(fp);
  size_t pos = text.find("\"sweep_shapes\"");
  while (pos != std::string::npos) {
    const size_t a = text.find('{', pos + 1), b = a == std::string::npos ? a : text.find('}', a);
    if (a == std::string::npos || b == std::string::npos) break;
    long v[9];
    int nv = 0;
    for (size_t i = a; i < b && nv < 9;) {
      if (std::isdigit((unsigned char)text[i])) {
        size_t e = i;
        while (e < b && std::isdigit((unsigned char)text[e])) e++;
        v[nv++] = std::strtol(text.substr(i, e - i).c_str(), nullptr, 10);
        i = e;
      } else {
        i++;
      }
    }
    if (nv == 9 && v[7] >= 0 && v[7] < kSubstVariants && (v[8] == 128 || v[8] == 256)) {
      emmi::SweepShape sh;
      sh.subst = (int)v[7];
      sh.rhs_threads = (int)v[8];
      g_tune[{v[0], v[1], v[2], v[3], v[4], v[5], v[6]}] = sh;
    }
    pos = b;
  }
}

static void tune_file_save() {
  const char* path = std::getenv("EMMI_TUNE_FILE");
  if (!path || !*path) return;
  const std::string tmp = std::string(path) + ".tmp";
  FILE* fp = std::fopen(tmp.c_str(), "w");
  if (!fp) return;
  std::fprintf(fp, "{\"sweep_shapes\": [");
  bool first = true;
  for (const auto& kv : g_tune) {
    const auto& q = kv.first;
    std::fprintf(fp,
                 "%s\n  {\"grid\": [%ld, %ld, %ld], \"chunk\": %ld, \"nrhs\": %ld, \"fmt\": %ld, "
                 "\"dir\": %ld, \"subst\": %d, \"rhs_threads\": %d}",
                 first ? "" : ",", q[0], q[1], q[2], q[3], q[4], q[5], q[6], kv.second.subst,
                 kv.second.rhs_threads);
    first = false;
  }
  std::fprintf(fp, "\n]}\n");
  std::fclose(fp);
  std::rename(tmp.c_str(), path);
}

static int autotune_sweeps(emmi_solver* s) {
  if (!s->fac_on || s->fac_fmt != kFacF16 || !s->opt.isemicoarsen || s->lmax < 2) return EMMI_OK;
  bool ready = false;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  for (int d = 0; d < 3; d++) {
    int h = -1;
    for (int c = 0; c < 3 && h < 0; c++)
      if (s->hier[c][1].sc[d] == 2) h = c;
    if (h < 0) continue;
    const HLev& L0 = s->hier[h][0];
    const std::array<long, 7> key = {L0.n[0], L0.n[1], L0.n[2], s->chunk, s->nrhs, s->fac_fmt, d};
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      if (!g_tune_loaded) tune_file_load();
      auto it = g_tune.find(key);
      if (it != g_tune.end()) {
        s->shape[0][d] = it->second;
        continue;
      }
    }
    if (!ready) {
      std::vector<int> all(s->nrhs, 1);
      CK(cudaMemcpyAsync(s->d_active, all.data(), s->nrhs * sizeof(int), cudaMemcpyHostToDevice,
                         s->st));
      const size_t fb = (size_t)3 * s->hier[0][0].S * s->nrhs * sizeof(float2);
      CK(cudaMemsetAsync(s->u32[0], 0, fb, s->st));
      CK(cudaMemsetAsync(s->f32[0], 0, fb, s->st));
      CK(cudaEventCreate(&e0));
      CK(cudaEventCreate(&e1));
      ready = true;
    }
    auto sweep = [&]() {
      for (int cc = 0; cc < 4; cc++)
        for (int r0 = 0; r0 < s->nrhs; r0 += s->chunk) {
          LevelView<float> W = s->view<float>(h, 0);
          W.nrhs = std::min(s->chunk, s->nrhs - r0);
          W.u += (long)r0 * 3 * W.S;
          W.f += (long)r0 * 3 * W.S;
          W.r += (long)r0 * 3 * W.S;
          W.wmu += r0;
          W.active += r0;
          W.op += r0;
          line_colour<float>(s, h, 0, d, cc, W, r0);
        }
    };
    auto time_shape = [&](SweepShape sh) -> float {
      s->shape[0][d] = sh;
      sweep();
      cudaEventRecord(e0, s->st);
      sweep();
      sweep();
      cudaEventRecord(e1, s->st);
      float ms = 0.f;
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
        return 1e30f;
      return ms;
    };
    SweepShape best;
    float best_ms = time_shape(best);
    auto consider = [&](SweepShape c) {
      const float t = time_shape(c);
      if (t < 0.98f * best_ms) {
        best = c;
        best_ms = t;
      }
    };
    SweepShape c = best;
    c.rhs_threads = 128;
    consider(c);
    for (int v = 1; v < kSubstVariants; v++) {
      c = best;
      c.subst = v;
      consider(c);
    }
    s->shape[0][d] = best;
    s->tuned_now = true;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = best;
    tune_file_save();
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  CK(cudaGetLastError());
  return EMMI_OK;
}

// Stored FP64 coefficients of the level-0 true operators for the mixed
// solver's refinement residual, when they fit in half of the free device
// memory (else the residual computes them, as the FP64 solver does)
static int build_coef64(emmi_solver* s) {
  const HLev& L0 = s->hier[0][0];
  const size_t bytes = (size_t)s->nop * coef64_elems(L0.n) * sizeof(double);
  if (bytes > device_avail() / 2) return EMMI_OK;
  int rc;
  if ((rc = s->alloc((void**)&s->d_coef64, bytes)) != EMMI_OK) return rc;
  CK(cudaMemsetAsync(s->d_coef64, 0, bytes, s->st));
  LevelView<double> V = s->view<double>(0, 0);
  V.nrhs = s->nop;
  V.op = nullptr;
  V.active = nullptr;
  // FP64-bound work that no step needs before the first refinement: on a
  // side stream, overlapping the first complex64 cycles (true_residual64
  // waits for ev_coef)
  CK(cudaStreamCreateWithFlags(&s->st2, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&s->ev_coef, cudaEventDisableTiming));
  CK(cudaEventRecord(s->ev_coef, s->st));
  CK(cudaStreamWaitEvent(s->st2, s->ev_coef, 0));
  launch_coef64(V, s->d_coef64, s->st2);
  CK(cudaGetLastError());
  CK(cudaEventRecord(s->ev_coef, s->st2));
  s->coef_pending = true;
  return EMMI_OK;
}

// ============================================================ C ABI
extern "C" {

const char* emmi_last_error(void) { return g_err.c_str(); }

void emmi_default_options(emmi_options* o) {
  o->cycleopt = 2;
  o->ncycle = 30;
  o->v1 = 1;
  o->v2 = 1;
  o->tol = 1e-6;
  o->isemicoarsen = 1;
  o->precision = EMMI_PREC_MIXED;
  o->sigma_floor = 0;
  o->refine_every = 4;
  o->use_graphs = 1;
  o->verb = 0;
  o->krylov = 0;
  o->line_factors = 2;
  o->autotune = 1;
  o->line_sweep = 0;
  o->fused_level = 99;
  o->staged = 1;
  o->skip_pre = 0;
  o->skip_post = 0;
}

static int create_impl(emmi_solver** out, const emmi_problem* P, const emmi_options* opts,
                       bool cells_on_device);

int emmi_solver_create(emmi_solver** out, const emmi_problem* P, const emmi_options* opts) {
  return create_impl(out, P, opts, false);
}

int emmi_solver_create_dc(emmi_solver** out, const emmi_problem* P, const emmi_options* opts) {
  return create_impl(out, P, opts, true);
}

static int create_impl(emmi_solver** out, const emmi_problem* P, const emmi_options* opts,
                       bool cells_on_device) {
  if (!out || !P || !P->x1 || !P->x2 || !P->x3 || !P->cells || !P->omega) {
    set_err("emmi_solver_create: null argument");
    return EMMI_EINVAL;
  }
  if (P->n1 < 2 || P->n2 < 2 || P->n3 < 2 || P->nop < 1 || P->nrhs < 1) {
    set_err("emmi_solver_create: bad sizes n=(%d,%d,%d) nop=%d nrhs=%d", P->n1, P->n2, P->n3,
            P->nop, P->nrhs);
    return EMMI_EINVAL;
  }
  if (P->op)
    for (int r = 0; r < P->nrhs; r++)
      if (P->op[r] < 0 || P->op[r] >= P->nop) {
        set_err("emmi_solver_create: op[%d]=%d out of range", r, P->op[r]);
        return EMMI_EINVAL;
      }
  if (!P->op && P->nop != P->nrhs) {
    set_err("emmi_solver_create: op==NULL needs nop==nrhs");
    return EMMI_EINVAL;
  }
  // the stencil kernels index a level's 3 (n1+1)(n2+1)(n3+1) edge slots
  // with 32-bit offsets
  if (3.0 * (P->n1 + 1.0) * (P->n2 + 1.0) * (P->n3 + 1.0) >= 2147483647.0) {
    set_err("emmi_solver_create: n=(%d,%d,%d) has 2^31 or more edge slots", P->n1, P->n2, P->n3);
    return EMMI_EINVAL;
  }
  emmi_solver* s = new emmi_solver();
  if (opts) s->opt = *opts; else emmi_default_options(&s->opt);
  if (s->opt.refine_every < 1) s->opt.refine_every = 3;
  if (s->opt.cycleopt < 1 || s->opt.cycleopt > 3) s->opt.cycleopt = 2;
  s->n[0] = P->n1;
  s->n[1] = P->n2;
  s->n[2] = P->n3;
  s->nop = P->nop;
  s->nrhs = P->nrhs;
  s->lmax = std::max(depth_of(P->n1), std::max(depth_of(P->n2), depth_of(P->n3)));
  if (s->lmax < 1) s->lmax = 1;
  if (s->lmax > kMaxLev) {
    set_err("too many levels");
    delete s;
    return EMMI_EINVAL;
  }
  const int gmax = std::max(P->n1, std::max(P->n2, P->n3));
  s->gmax1 = gmax + 1;
  s->gstride = 9 * s->gmax1;
  const bool mixed = s->opt.precision == EMMI_PREC_MIXED;
  int rc;
#define TRY(x)                 \
  do {                         \
    rc = (x);                  \
    if (rc != EMMI_OK) {       \
      emmi_solver_destroy(s);  \
      return rc;               \
    }                          \
  } while (0)
#define CKS(x)                                                                   \
  do {                                                                           \
    cudaError_t e_ = (x);                                                        \
    if (e_ != cudaSuccess) {                                                     \
      set_err("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_));  \
      emmi_solver_destroy(s);                                                    \
      return EMMI_ECUDA;                                                         \
    }                                                                            \
  } while (0)
  // set-up phase times on stderr with verb >= 2 (each mark drains the stream)
  auto t_last = std::chrono::steady_clock::now();
  auto mark = [&](const char* what) {
    if (s->opt.verb < 2) return;
    cudaStreamSynchronize(s->st);
    const auto now = std::chrono::steady_clock::now();
    fprintf(stderr, "emmi_solver_create: %-28s %8.2f ms\n", what,
            std::chrono::duration<double, std::milli>(now - t_last).count());
    t_last = now;
  };
  init_line_kernels();
  keep_pool_memory();
  CKS(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking));
  CKS(cudaEventCreate(&s->ev0));
  CKS(cudaEventCreate(&s->ev1));

  // ---- hierarchies (grid_init, gmg.c:1744-1760)
  for (int h = 0; h < 3; h++) {
    HLev& L0 = s->hier[h][0];
    for (int e = 0; e < 3; e++) {
      L0.n[e] = s->n[e];
      L0.sc[e] = 1;
    }
    for (int l = 1; l < s->lmax; l++) {
      const HLev& F = s->hier[h][l - 1];
      HLev& C = s->hier[h][l];
      for (int e = 0; e < 3; e++) C.sc[e] = (F.n[e] % 2 == 0 && F.n[e] > 2) ? 2 : 1;
      if (s->opt.isemicoarsen) C.sc[h] = 1;
      for (int e = 0; e < 3; e++) C.n[e] = F.n[e] / C.sc[e];
    }
    for (int l = 0; l < s->lmax; l++) {
      HLev& L = s->hier[h][l];
      L.S = (long)(L.n[0] + 1) * (L.n[1] + 1) * (L.n[2] + 1);
      L.ncell = (long)L.n[0] * L.n[1] * L.n[2];
    }
  }
  // a non-semicoarsened batch has one hierarchy; keep three identical copies
  s->has_norm = s->lmax > 1 && s->hier[0][1].sc[0] * s->hier[0][1].sc[1] * s->hier[0][1].sc[2] > 1;

  // ---- geometry per (h, l, op) on the host, then upload
  {
    const size_t gsz = (size_t)s->nop * s->gstride;
    std::vector<double> g64(gsz), prev(gsz);
    std::vector<float> g32(gsz);
    std::vector<double> xs_tmp(s->gmax1);
    for (int h = 0; h < 3; h++) {
      for (int l = 0; l < s->lmax; l++) {
        const HLev& L = s->hier[h][l];
        std::fill(g64.begin(), g64.end(), 0.0);
        for (int o = 0; o < s->nop; o++) {
          double* G = g64.data() + (size_t)o * s->gstride;
          const double* Gp = prev.data() + (size_t)o * s->gstride;
          for (int e = 0; e < 3; e++) {
            double* x = G + e * s->gmax1;
            if (l == 0) {
              const float* src = e == 0 ? P->x1 : e == 1 ? P->x2 : P->x3;
              for (int i = 0; i <= L.n[e]; i++) x[i] = (double)src[(size_t)o * (s->n[e] + 1) + i];
            } else {
              // coordinates by sub-sampling the finer level (gmg.c:1784-1786)
              for (int i = 0; i <= L.n[e]; i++) x[i] = Gp[e * s->gmax1 + L.sc[e] * i];
            }
            stagger(L.n[e], x, xs_tmp.data(), G + (6 + e) * s->gmax1, G + (3 + e) * s->gmax1);
          }
        }
        prev = g64;
        if (h > 0 && l == 0) {
          s->geo64[h][0] = s->geo64[0][0];
          s->geo32[h][0] = s->geo32[0][0];
          continue;
        }
        for (size_t i = 0; i < gsz; i++) g32[i] = (float)g64[i];
        TRY(s->alloc((void**)&s->geo64[h][l], gsz * sizeof(double)));
        TRY(s->alloc((void**)&s->geo32[h][l], gsz * sizeof(float)));
        // every upload goes on the solver's stream: a plain cudaMemcpy from
        // pageable memory may return before its DMA lands, and the
        // non-blocking stream does not wait for the legacy stream
        CKS(cudaMemcpyAsync(s->geo64[h][l], g64.data(), gsz * sizeof(double), cudaMemcpyHostToDevice, s->st));
        CKS(cudaMemcpyAsync(s->geo32[h][l], g32.data(), gsz * sizeof(float), cudaMemcpyHostToDevice, s->st));
        CKS(cudaStreamSynchronize(s->st));
      }
    }
    // transfer weights of every level but the coarsest, from the geometry
    const size_t wsz = (size_t)s->nop * 3 * s->gmax1;
    for (int h = 0; h < 3; h++)
      for (int l = 0; l + 1 < s->lmax; l++) {
        TRY(s->alloc((void**)&s->xw64[h][l], wsz * sizeof(double)));
        TRY(s->alloc((void**)&s->xw32[h][l], wsz * sizeof(float)));
        launch_xfer_weights<double>(s->view<double>(h, l), s->view<double>(h, l + 1),
                                    s->hier[h][l + 1].sc, s->nop, s->xw64[h][l], s->st);
        launch_xfer_weights<float>(s->view<float>(h, l), s->view<float>(h, l + 1),
                                   s->hier[h][l + 1].sc, s->nop, s->xw32[h][l], s->st);
      }
    CKS(cudaGetLastError());
  }

  // ---- per-RHS scalars
  {
    std::vector<int> op(s->nrhs);
    std::vector<double> w64(s->nrhs);
    std::vector<float> w32(s->nrhs);
    for (int r = 0; r < s->nrhs; r++) {
      op[r] = P->op ? P->op[r] : r;
      // I*omega*mu0 as gmg_init forms it (gmg.c:1710): imag = (double)omega_f * mu0
      w64[r] = (double)P->omega[r] * kMu0;
      w32[r] = (float)w64[r];
    }
    TRY(s->alloc((void**)&s->d_op, s->nrhs * sizeof(int)));
    TRY(s->alloc((void**)&s->d_active, s->nrhs * sizeof(int)));
    TRY(s->alloc((void**)&s->d_refine, s->nrhs * sizeof(int)));
    TRY(s->alloc((void**)&s->d_wmu64, s->nrhs * sizeof(double)));
    TRY(s->alloc((void**)&s->d_wmu32, s->nrhs * sizeof(float)));
    TRY(s->alloc((void**)&s->d_norm, s->nrhs * sizeof(double)));
    TRY(s->alloc((void**)&s->d_norm64, s->nrhs * sizeof(double)));
    CKS(cudaMemcpyAsync(s->d_op, op.data(), s->nrhs * sizeof(int), cudaMemcpyHostToDevice, s->st));
    CKS(cudaMemcpyAsync(s->d_wmu64, w64.data(), s->nrhs * sizeof(double), cudaMemcpyHostToDevice, s->st));
    CKS(cudaMemcpyAsync(s->d_wmu32, w32.data(), s->nrhs * sizeof(float), cudaMemcpyHostToDevice, s->st));
    CKS(cudaStreamSynchronize(s->st));
    s->h_active.assign(s->nrhs, 1);
    s->h_refine.assign(s->nrhs, 0);
  }

  // ---- cells: level 0 weighted by volume, coarse levels by summation
  {
    const long nc0 = s->hier[0][0].ncell;
    float* raw = nullptr;
    TRY(s->alloc((void**)&raw, (size_t)s->nop * 4 * nc0 * sizeof(float)));
    CKS(cudaMemcpyAsync(raw, P->cells, (size_t)s->nop * 4 * nc0 * sizeof(float),
                        cells_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s->st));
    s->raw_cells = raw;
    if (mixed) {
      // is every operator's invmur exactly 1 (the front end's value)?
      int* d_flag = nullptr;
      TRY(s->alloc((void**)&d_flag, sizeof(int)));
      CKS(cudaMemsetAsync(d_flag, 0, sizeof(int), s->st));
      dim3 gc(blocks_for(nc0), s->nop);
      k_not_one<<<gc, 256, 0, s->st>>>(raw, nc0, d_flag);
      int flag = 1;
      CKS(cudaMemcpyAsync(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, s->st));
      CKS(cudaStreamSynchronize(s->st));
      s->release(d_flag);
      s->imu_vol = flag == 0;
    }
    // survey grids in float as emf_t holds them (regrid_init_free.c:21-34)
    {
      std::vector<float> sg((size_t)s->nop * s->gstride, 0.f);
      for (int o = 0; o < s->nop; o++) {
        float* G = sg.data() + (size_t)o * s->gstride;
        for (int e = 0; e < 3; e++) {
          const int ne = s->n[e];
          const float* src = e == 0 ? P->x1 : e == 1 ? P->x2 : P->x3;
          float* x = G + e * s->gmax1;
          float* xs = G + (3 + e) * s->gmax1;
          float* d = G + (6 + e) * s->gmax1;
          std::vector<float> ds(ne + 1);
          for (int i = 0; i <= ne; i++) x[i] = src[(size_t)o * (ne + 1) + i];
          for (int i = 0; i < ne; i++) {
            ds[i] = x[i + 1] - x[i];
            xs[i] = 0.5 * (x[i] + x[i + 1]);
          }
          xs[ne] = x[ne] + 0.5 * ds[ne - 1];
          for (int i = 1; i <= ne; i++) d[i] = xs[i] - xs[i - 1];
          d[0] = xs[0] - x[0];
        }
      }
      TRY(s->alloc((void**)&s->sgeo, sg.size() * sizeof(float)));
      CKS(cudaMemcpyAsync(s->sgeo, sg.data(), sg.size() * sizeof(float), cudaMemcpyHostToDevice, s->st));
      std::vector<float> rw(s->nop, 0.f);
      if (P->rho_water)
        for (int o = 0; o < s->nop; o++) rw[o] = P->rho_water[o];
      TRY(s->alloc((void**)&s->d_rho_water, s->nop * sizeof(float)));
      CKS(cudaMemcpyAsync(s->d_rho_water, rw.data(), s->nop * sizeof(float), cudaMemcpyHostToDevice, s->st));
      s->h_omega.assign(P->omega, P->omega + s->nrhs);
      TRY(s->alloc((void**)&s->d_omega, s->nrhs * sizeof(float)));
      CKS(cudaMemcpyAsync(s->d_omega, P->omega, s->nrhs * sizeof(float), cudaMemcpyHostToDevice, s->st));
      CKS(cudaStreamSynchronize(s->st));
      s->h_op.resize(s->nrhs);
      for (int r = 0; r < s->nrhs; r++) s->h_op[r] = P->op ? P->op[r] : r;
    }
    // true operator in FP64 at level 0 (both modes)
    TRY(s->alloc((void**)&s->cells64[0][0], (size_t)s->nop * 4 * nc0 * sizeof(double)));
    dim3 g0(blocks_for(nc0), s->nop);
    k_weight_cells<<<g0, 256, 0, s->st>>>(raw, s->geo64[0][0], s->gstride, s->gmax1, s->n[0], s->n[1],
                                          s->n[2], -1.0, s->cells64[0][0], nullptr);
    for (int h = 1; h < 3; h++) s->cells64[h][0] = s->cells64[0][0];
    if (!mixed) {
      for (int h = 0; h < 3; h++)
        for (int l = 1; l < s->lmax; l++) {
          const HLev& C = s->hier[h][l];
          TRY(s->alloc((void**)&s->cells64[h][l], (size_t)s->nop * 4 * C.ncell * sizeof(double)));
          launch_coarsen_cells<double>(s->cells64[h][l - 1], s->hier[h][l - 1].n, s->cells64[h][l],
                                       C.sc, s->nop, s->st);
        }
    } else {
      // preconditioner operator: floored conductivity, summed in FP64, stored f32
      double floor = s->opt.sigma_floor;
      if (floor <= 0) {
        float wmin = P->omega[0];
        for (int r = 1; r < s->nrhs; r++) wmin = std::min(wmin, P->omega[r]);
        // 1e-5 S/m at 1 Hz keeps the complex64 line/patch factorizations
        // stable (1e-6 is not, on a 64^3 1 Hz survey) while changing the
        // preconditioner little enough that cycles stay at the FP64 count
        floor = 1e-5 * std::max(1.0, 2.0 * 3.14159265358979323846 / (double)wmin);
      }
      s->opt.sigma_floor = floor;
      // base: level-0 floored cells in FP64, kept intact for every
      // hierarchy; ping/pong: the coarse levels of the current hierarchy
      double *base = nullptr, *pp[2] = {nullptr, nullptr};
      TRY(s->alloc((void**)&base, (size_t)s->nop * 4 * nc0 * sizeof(double)));
      TRY(s->alloc((void**)&pp[0], (size_t)s->nop * 4 * nc0 * sizeof(double)));
      TRY(s->alloc((void**)&pp[1], (size_t)s->nop * 4 * nc0 * sizeof(double)));
      TRY(s->alloc((void**)&s->cells32[0][0],
                   (size_t)stencil_pad((long)s->nop * 4 * nc0, 4) * sizeof(float)));
      k_weight_cells<<<g0, 256, 0, s->st>>>(raw, s->geo64[0][0], s->gstride, s->gmax1, s->n[0],
                                            s->n[1], s->n[2], floor, base, s->cells32[0][0]);
      for (int h = 1; h < 3; h++) s->cells32[h][0] = s->cells32[0][0];
      for (int h = 0; h < 3; h++) {
        const double* src = base;
        for (int l = 1; l < s->lmax; l++) {
          const HLev& C = s->hier[h][l];
          double* dst = pp[l & 1];
          launch_coarsen_cells<double>(src, s->hier[h][l - 1].n, dst, C.sc, s->nop, s->st);
          TRY(s->alloc((void**)&s->cells32[h][l],
                       (size_t)stencil_pad((long)s->nop * 4 * C.ncell, 4) * sizeof(float)));
          const long nn = (long)s->nop * 4 * C.ncell;
          k_d2f<<<blocks_for(nn), 256, 0, s->st>>>(dst, s->cells32[h][l], nn);
          src = dst;
        }
      }
      CKS(cudaStreamSynchronize(s->st));
    }
    CKS(cudaGetLastError());
    CKS(cudaStreamSynchronize(s->st));
  }
  mark("geometry and cells");

  // ---- fields: level 0 per mode, coarse levels sized by the largest hierarchy
  {
    for (int l = 0; l < s->lmax; l++) {
      long Smax = 0;
      for (int h = 0; h < 3; h++) Smax = std::max(Smax, s->hier[h][l].S);
      const size_t n3 = (size_t)3 * Smax * s->nrhs;
      if (!mixed || l == 0) {
        // FP64 fields; in MIXED mode level 0 holds x (u64) and b*vol (f64)
        TRY(s->alloc((void**)&s->u64[l], n3 * sizeof(double2)));
        TRY(s->alloc((void**)&s->f64[l], n3 * sizeof(double2)));
        if (!mixed) TRY(s->alloc((void**)&s->r64[l], n3 * sizeof(double2)));
      }
      if (mixed) {
        // whole 256-byte rows: the staged residual's tensor maps read them
        const size_t n3p = (size_t)stencil_pad((long)n3, 8);
        TRY(s->alloc((void**)&s->u32[l], n3p * sizeof(float2)));
        TRY(s->alloc((void**)&s->f32[l], n3p * sizeof(float2)));
        TRY(s->alloc((void**)&s->r32[l], n3p * sizeof(float2)));
        s->u32_elems[l] = (long)n3;
      }
    }
    // line-sweep scratch: largest (level, direction) over the hierarchies,
    // chunked over RHS so it stays below ~8 GB
    long per_rhs = 0;
    const size_t esz = mixed ? sizeof(float2) : sizeof(double2);
    for (int h = 0; h < 3; h++)
      for (int l = 0; l + 1 < s->lmax; l++)
        for (int d = 0; d < 3; d++)
          if (s->hier[h][l + 1].sc[d] == 2) {
            per_rhs = std::max(per_rhs, line_scratch_elems(s->hier[h][l].n, d, 1));
            // the one-launch sweep's multipliers (whole elements of esz)
            for (int c = 0; c < 4; c++)
              per_rhs = std::max<long>(
                  per_rhs, (line_l_bytes(s->hier[h][l].n, d, c, kLExact, (int)esz / 2) + esz - 1) /
                               (long)esz);
          }
    const size_t cap = (size_t)8 << 30;
    s->chunk = s->nrhs;
    while (s->chunk > 1 && (size_t)per_rhs * esz * s->chunk > cap) s->chunk = (s->chunk + 1) / 2;
    s->scratch_bytes = std::max<size_t>((size_t)per_rhs * esz * s->chunk, 16);
    TRY(s->alloc(&s->scratch, s->scratch_bytes));
    if (mixed && s->opt.krylov > 0) TRY(krylov_alloc(s));
    TRY(s->alloc((void**)&s->d_lovf, sizeof(int)));
    CKS(cudaMemsetAsync(s->d_lovf, 0, sizeof(int), s->st));
    s->lfmt = (mixed && s->opt.line_factors == 2) ? kLHalf : kLExact;
    for (int l = 0; l < kMaxLev; l++)
      for (int d = 0; d < 3; d++) s->fused_nt[l][d] = 64;
    mark("field buffers");
    if (s->opt.line_factors && !s->opt.line_sweep)
      TRY(mixed ? build_line_factors<float>(s) : build_line_factors<double>(s));
    mark("line factors");
    if (mixed && s->opt.autotune > 0 && !s->opt.line_sweep) TRY(autotune_sweeps(s));
    if (mixed && s->opt.autotune < 0 && !s->opt.line_sweep) {
      // a forced level-0 shape k = -autotune (1..10): substitution variant
      // (k-1) % 5, right-hand-side threads 256 for k <= 5, else 128
      const int k = std::min(-s->opt.autotune, 2 * kSubstVariants) - 1;
      for (int d = 0; d < 3; d++) {
        s->shape[0][d].subst = k % kSubstVariants;
        s->shape[0][d].rhs_threads = k < kSubstVariants ? 256 : 128;
      }
    }
    mark("sweep shapes");
    if (mixed && s->opt.staged) {
      // staged residual on level 0 (shared by the hierarchies); the coarse
      // levels are too small to fill the GPU with plane-marching tiles and
      // sit in L2, where the plain residual is faster
      LevelView<float> V = s->view<float>(0, 0);
      if (stencil_prepare(V, s->u32_elems[0], (long)s->nop * 4 * V.ncell, &s->plan[0][0]))
        for (int h = 1; h < 3; h++) s->plan[h][0] = s->plan[0][0];
    }
    if (mixed) TRY(build_coef64(s));
    mark("FP64 coefficients");
  }

  // ---- graphs
  if (s->opt.use_graphs) {
    rc = mixed ? s->build_graphs<float>() : s->build_graphs<double>();
    if (rc != EMMI_OK) {
      emmi_solver_destroy(s);
      return rc;
    }
  }
  mark("CUDA graphs");
  *out = s;
  return EMMI_OK;
#undef TRY
#undef CKS
}

}  // extern "C"

int line_format_fallback(emmi_solver* s) {
  if (!(s->opt.line_sweep || s->opt.fused_level < s->lmax) || s->lfmt != kLHalf) return 0;
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, s->d_lovf, sizeof(int), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  if (!flag) return 0;
  s->lfmt = kLExact;
  CK(cudaMemsetAsync(s->d_lovf, 0, sizeof(int), s->st));
  if (s->opt.use_graphs) {
    CK(cudaStreamSynchronize(s->st));
    for (int h = 0; h < 3; h++) {
      if (s->gA[h]) cudaGraphExecDestroy(s->gA[h]);
      if (s->gB[h]) cudaGraphExecDestroy(s->gB[h]);
      s->gA[h] = s->gB[h] = nullptr;
    }
    const int rc = s->build_graphs<float>();
    if (rc != EMMI_OK) return rc;
  }
  if (s->opt.verb) printf("line sweep: an fp16 multiplier left its range; fp32 from here on\n");
  return 1;
}

int run_part(emmi_solver* s, int h, int part) {
  if (s->opt.use_graphs) {
    CK(cudaGraphLaunch(part ? s->gB[h] : s->gA[h], s->st));
    s->last_launches += part ? s->nodesB[h] : s->nodesA[h];
    return EMMI_OK;
  }
  const long before = s->launch_counter;
  int cur = 0;
  if (s->opt.precision == EMMI_PREC_MIXED)
    s->emit_cycle<float>(h, 0, s->opt.cycleopt, part, cur);
  else
    s->emit_cycle<double>(h, 0, s->opt.cycleopt, part, cur);
  s->last_launches += s->launch_counter - before;
  CK(cudaGetLastError());
  return EMMI_OK;
}

extern "C" {

static int upload_mask(emmi_solver* s, int* dev, const std::vector<int>& host) {
  CK(cudaMemcpyAsync(dev, host.data(), host.size() * sizeof(int), cudaMemcpyHostToDevice, s->st));
  return EMMI_OK;
}

static int read_norms(emmi_solver* s, const double* dev, std::vector<double>& host) {
  CK(cudaMemcpyAsync(host.data(), dev, host.size() * sizeof(double), cudaMemcpyDeviceToHost, s->st));
  int staged_err = 0;
  if (s->opt.staged)
    CK(cudaMemcpyAsync(&staged_err, stencil_err(), sizeof(int), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  if (staged_err) {
    cudaMemsetAsync(stencil_err(), 0, sizeof(int), s->st);
    cudaStreamSynchronize(s->st);
    set_err("a staged residual's wait for its tensor copies ran out");
    return EMMI_ECUDA;
  }
  return EMMI_OK;
}

// resident: b is already in u64[0]; x/h may be null (E stays in u64[0],
// H is always formed in f64[0] for the extraction that follows)
static int solve_impl(emmi_solver* s, const double* b, double* x, double* h, int device,
                      emmi_rhs_stats* stats, bool resident) {
  if (!s || (!resident && (!b || !x))) {
    set_err("emmi_solver_solve: null argument");
    return EMMI_EINVAL;
  }
  const int nrhs = s->nrhs;
  const long S = s->hier[0][0].S;
  const long n3s = 3 * S;
  const size_t fbytes = (size_t)n3s * nrhs * sizeof(double2);
  const bool mixed = s->opt.precision == EMMI_PREC_MIXED;
  int rc;
  s->last_launches = 0;
  CK(cudaEventRecord(s->ev0, s->st));
  // b -> device (into u64[0] temporarily), then f64[0] = b * dual volume
  double2* bdev = s->u64[0];
  if (!resident) {
    if (device)
      CK(cudaMemcpyAsync(bdev, b, fbytes, cudaMemcpyDeviceToDevice, s->st));
    else
      CK(cudaMemcpyAsync(bdev, b, fbytes, cudaMemcpyHostToDevice, s->st));
  }
  {
    dim3 g(blocks_for(S), nrhs);
    k_scale_dual<<<g, 256, 0, s->st>>>(bdev, s->f64[0], s->geo64[0][0], s->d_op, s->gstride,
                                       s->gmax1, s->n[0], s->n[1], s->n[2]);
    s->last_launches++;
  }
  CK(cudaMemsetAsync(s->u64[0], 0, fbytes, s->st));  // x = 0 (gmg.c:1900)
  std::vector<int>& act = s->h_active;
  std::vector<int>& ref = s->h_refine;
  act.assign(nrhs, 1);
  ref.assign(nrhs, 0);
  std::vector<double> nrm(nrhs), rnorm0(nrhs, 0.0), rn(nrhs, 0.0);
  std::vector<int> cycles(nrhs, 0), status(nrhs, EMMI_SOLVE_MAXIT), nref(nrhs, 0),
      since(nrhs, 0);
  std::vector<double> best(nrhs, INFINITY), last_rel(nrhs, 1.0);
  std::vector<int> stall(nrhs, 0);
  s->h_fallback.assign(nrhs, 0);
  s->h_learn.assign(nrhs, s->learned_on ? 1 : 0);
  if ((rc = upload_mask(s, s->d_active, act)) != EMMI_OK) return rc;
  const double tol = s->opt.tol;
  const int ncycle = s->opt.ncycle;

  if (mixed && s->kry_m > 0) {
    if ((rc = krylov_solve(s, cycles, status, nref, rnorm0, rn)) != EMMI_OK) return rc;
  } else if (mixed) {
    // initial FP64 residual = b*vol (x = 0) -> f32[0]; rnorm0; u32 = 0
    CK(cudaMemsetAsync(s->d_norm64, 0, nrhs * sizeof(double), s->st));
    {
      dim3 g(blocks_for(n3s, 256, 2048), nrhs);
      k_first_residual<<<g, 256, 0, s->st>>>(s->f64[0], s->f32[0], s->u32[0], n3s, s->d_active,
                                             s->d_norm64);
      s->last_launches++;
    }
    if ((rc = read_norms(s, s->d_norm64, nrm)) != EMMI_OK) return rc;
    for (int r = 0; r < nrhs; r++) {
      rnorm0[r] = std::sqrt(nrm[r]);
      rn[r] = rnorm0[r];
      if (!(rnorm0[r] > 0) || !std::isfinite(rnorm0[r])) {
        act[r] = 0;
        status[r] = std::isfinite(rnorm0[r]) ? EMMI_SOLVE_OK : EMMI_SOLVE_NONFINITE;
      }
    }
    if ((rc = upload_mask(s, s->d_active, act)) != EMMI_OK) return rc;
    for (int icycle = 0; icycle < ncycle; icycle++) {
      bool any = false;
      for (int r = 0; r < nrhs; r++) any |= act[r] != 0;
      if (!any) break;
      const int hh = s->opt.isemicoarsen ? icycle % 3 : 0;
      if ((rc = run_part(s, hh, 0)) != EMMI_OK) return rc;
      if (s->has_norm) {
        if ((rc = read_norms(s, s->d_norm, nrm)) != EMMI_OK) return rc;
        if ((rc = line_format_fallback(s)) < 0) return rc;
        if (rc == 1) {
          // the last cycles' corrections carry the out-of-range multipliers:
          // every cycling RHS restarts its inner problem from u = 0, whose
          // level-0 residual (what part B restricts) is f
          dim3 g(blocks_for(n3s, 256, 2048), nrhs);
          k_zero_masked<<<g, 256, 0, s->st>>>(s->u32[0], n3s, s->d_active);
          LevelView<float> R = s->view<float>(hh, 0);
          s->resid<float>(hh, 0, R, R.r, nullptr);
          s->last_launches += 2;
          for (int r = 0; r < nrhs; r++) since[r] = 0;
          rc = EMMI_OK;
        } else {
          // complex64 estimate of |b - A(x+u)|; refine when it says converged
          // or every refine_every cycles
          bool anyref = false;
          for (int r = 0; r < nrhs; r++) {
            ref[r] = 0;
            if (!act[r]) continue;
            const double est = std::sqrt(nrm[r]) / rnorm0[r];
            if (s->opt.verb) printf("icycle=%d rnorm=%e\n", icycle, est * rnorm0[r]);
            if ((est < tol && since[r] > 0) || since[r] >= s->opt.refine_every || !std::isfinite(est)) {
              ref[r] = 1;
              anyref = true;
            }
          }
          if (anyref) {
            if ((rc = upload_mask(s, s->d_refine, ref)) != EMMI_OK) return rc;
            dim3 g(blocks_for(n3s, 256, 2048), nrhs);
            k_accumulate<<<g, 256, 0, s->st>>>(s->u64[0], s->u32[0], n3s, s->d_refine);
            LevelView<double> W = s->view<double>(0, 0);
            W.u = s->u64[0];
            W.f = s->f64[0];
            W.active = s->d_refine;
            CK(cudaMemsetAsync(s->d_norm64, 0, nrhs * sizeof(double), s->st));
            true_residual64<float>(s, W, s->f32[0], s->d_norm64);
            k_zero_masked<<<g, 256, 0, s->st>>>(s->u32[0], n3s, s->d_refine);
            s->last_launches += 3;
            if ((rc = read_norms(s, s->d_norm64, nrm)) != EMMI_OK) return rc;
            for (int r = 0; r < nrhs; r++) {
              if (!ref[r]) continue;
              nref[r]++;
              since[r] = 0;
              rn[r] = std::sqrt(nrm[r]);
              const double rel = rn[r] / rnorm0[r];
              const double prev_rel = last_rel[r];
              last_rel[r] = rel;
              if (!std::isfinite(rel)) {
                act[r] = 0;
                status[r] = EMMI_SOLVE_NONFINITE;
              } else if (rel <= tol) {
                act[r] = 0;
                status[r] = EMMI_SOLVE_OK;
              } else if (rel > 0.5 * prev_rel && learned_fallback(s, r)) {
                // no halving since the last refinement with the learned
                // correction on: continue with plain cycles
                stall[r] = 0;
              } else {
                if (rel < 0.5 * best[r]) {
                  best[r] = rel;
                  stall[r] = 0;
                } else if (++stall[r] >= 4) {
                  act[r] = 0;
                  status[r] = EMMI_SOLVE_STALL;
                }
              }
            }
            if ((rc = upload_mask(s, s->d_active, act)) != EMMI_OK) return rc;
            // the new inner problem starts from u = 0: its level-0 residual
            // (what part B restricts) is f; recompute it for the refined RHS
            for (int r = 0; r < nrhs; r++) ref[r] = ref[r] && act[r];
            if ((rc = upload_mask(s, s->d_refine, ref)) != EMMI_OK) return rc;
            LevelView<float> R = s->view<float>(hh, 0);
            R.active = s->d_refine;
            s->resid<float>(hh, 0, R, R.r, nullptr);
            s->last_launches++;
          }
        }
      }
      if ((rc = run_part(s, hh, 1)) != EMMI_OK) return rc;
      if (s->learned_on && (rc = learned_after_cycle(s, hh, act)) != EMMI_OK) return rc;
      if (s->ls_collect && (rc = learned_snapshot(s, hh, act)) != EMMI_OK) return rc;
      for (int r = 0; r < nrhs; r++)
        if (act[r]) {
          cycles[r]++;
          since[r]++;
        }
    }
    // RHS still cycling at ncycle: fold in the last correction and measure
    bool anyleft = false;
    for (int r = 0; r < nrhs; r++) {
      ref[r] = act[r];
      anyleft |= act[r] != 0;
    }
    if (anyleft) {
      if ((rc = upload_mask(s, s->d_refine, ref)) != EMMI_OK) return rc;
      dim3 g(blocks_for(n3s, 256, 2048), nrhs);
      k_accumulate<<<g, 256, 0, s->st>>>(s->u64[0], s->u32[0], n3s, s->d_refine);
      LevelView<double> W = s->view<double>(0, 0);
      W.u = s->u64[0];
      W.f = s->f64[0];
      W.active = s->d_refine;
      CK(cudaMemsetAsync(s->d_norm64, 0, nrhs * sizeof(double), s->st));
      true_residual64<float>(s, W, s->f32[0], s->d_norm64);
      s->last_launches += 2;
      if ((rc = read_norms(s, s->d_norm64, nrm)) != EMMI_OK) return rc;
      for (int r = 0; r < nrhs; r++)
        if (ref[r]) {
          nref[r]++;
          rn[r] = std::sqrt(nrm[r]);
          status[r] = rn[r] / rnorm0[r] <= tol ? EMMI_SOLVE_OK
                      : std::isfinite(rn[r]) ? EMMI_SOLVE_MAXIT : EMMI_SOLVE_NONFINITE;
        }
    }
    if (s->learned_on) {
      if (const int why = learned_check(s->st)) {
        set_err("emmi_solver_solve: a learned-correction convolution gave up waiting (code %d)",
                why);
        return EMMI_ECUDA;
      }
    }
  } else {
    // plain FP64 cycles on u64/f64 (gmg_apply, gmg.c:1911-1926)
    for (int icycle = 0; icycle < ncycle; icycle++) {
      bool any = false;
      for (int r = 0; r < nrhs; r++) any |= act[r] != 0;
      if (!any) break;
      const int hh = s->opt.isemicoarsen ? icycle % 3 : 0;
      if ((rc = run_part(s, hh, 0)) != EMMI_OK) return rc;
      if (s->has_norm) {
        if ((rc = read_norms(s, s->d_norm, nrm)) != EMMI_OK) return rc;
        bool changed = false;
        for (int r = 0; r < nrhs; r++) {
          if (!act[r]) continue;
          const double rnorm = std::sqrt(nrm[r]);
          if (s->opt.verb) printf("icycle=%d rnorm=%e\n", icycle, rnorm);
          rn[r] = rnorm;
          if (icycle == 0) {
            rnorm0[r] = rnorm;
            if (!(rnorm > 0)) {
              act[r] = 0;
              status[r] = std::isfinite(rnorm) ? EMMI_SOLVE_OK : EMMI_SOLVE_NONFINITE;
              changed = true;
            }
          } else if (!std::isfinite(rnorm)) {
            act[r] = 0;
            status[r] = EMMI_SOLVE_NONFINITE;
            changed = true;
          } else if (rnorm < rnorm0[r] * tol) {
            act[r] = 0;
            status[r] = EMMI_SOLVE_OK;
            changed = true;
          }
        }
        if (changed && (rc = upload_mask(s, s->d_active, act)) != EMMI_OK) return rc;
      }
      if ((rc = run_part(s, hh, 1)) != EMMI_OK) return rc;
      for (int r = 0; r < nrhs; r++)
        if (act[r]) cycles[r]++;
    }
    // final FP64 residual of every RHS for the statistics
    act.assign(nrhs, 1);
    if ((rc = upload_mask(s, s->d_active, act)) != EMMI_OK) return rc;
    LevelView<double> V = s->view<double>(0, 0);
    CK(cudaMemsetAsync(s->d_norm64, 0, nrhs * sizeof(double), s->st));
    launch_residual<double, double>(V, V.r, s->d_norm64, s->st);
    s->last_launches++;
    if ((rc = read_norms(s, s->d_norm64, nrm)) != EMMI_OK) return rc;
    for (int r = 0; r < nrhs; r++) {
      rn[r] = std::sqrt(nrm[r]);
      if (status[r] == EMMI_SOLVE_MAXIT && !std::isfinite(rn[r])) status[r] = EMMI_SOLVE_NONFINITE;
    }
  }
  // outputs: x = E, h = curl E / (i w mu0) (gmg.c:1927-1929)
  if (x) {
    if (device)
      CK(cudaMemcpyAsync(x, s->u64[0], fbytes, cudaMemcpyDeviceToDevice, s->st));
    else
      CK(cudaMemcpyAsync(x, s->u64[0], fbytes, cudaMemcpyDeviceToHost, s->st));
  }
  if (h || resident) {
    // H goes to f64[0] (b*vol is no longer needed) then out
    dim3 g(blocks_for(S), nrhs);
    k_curl_h<<<g, 256, 0, s->st>>>(s->u64[0], s->f64[0], s->geo64[0][0], s->d_op, s->d_wmu64,
                                   s->gstride, s->gmax1, s->n[0], s->n[1], s->n[2]);
    s->last_launches++;
    if (h && device)
      CK(cudaMemcpyAsync(h, s->f64[0], fbytes, cudaMemcpyDeviceToDevice, s->st));
    else if (h)
      CK(cudaMemcpyAsync(h, s->f64[0], fbytes, cudaMemcpyDeviceToHost, s->st));
  }
  CK(cudaEventRecord(s->ev1, s->st));
  CK(cudaStreamSynchronize(s->st));
  CK(cudaGetLastError());
  float ms = 0;
  cudaEventElapsedTime(&ms, s->ev0, s->ev1);
  s->last_time = ms * 1e-3;
  if (stats)
    for (int r = 0; r < nrhs; r++) {
      stats[r].cycles = cycles[r];
      stats[r].status = status[r];
      stats[r].rnorm0 = rnorm0[r];
      stats[r].rnorm = rn[r];
      stats[r].refinements = nref[r];
      stats[r].fallback = s->h_fallback[r];
    }
  return EMMI_OK;
}

int emmi_solver_solve(emmi_solver* s, const double* b, double* x, double* h, int device,
                      emmi_rhs_stats* stats) {
  return solve_impl(s, b, x, h, device, stats, false);
}

int emmi_solver_solve_resident(emmi_solver* s, double* x_dev, double* h_dev,
                               emmi_rhs_stats* stats) {
  return solve_impl(s, nullptr, x_dev, h_dev, 1, stats, true);
}

void* emmi_solver_stream(const emmi_solver* s) { return s ? (void*)s->st : nullptr; }

int emmi_solver_sweep_shapes(const emmi_solver* s, int shapes[3][3], int* tuned) {
  if (!s || !shapes) {
    set_err("emmi_solver_sweep_shapes: bad argument");
    return EMMI_EINVAL;
  }
  for (int d = 0; d < 3; d++) {
    const SweepShape& sh = s->shape[0][d];
    shapes[d][0] = subst_variant_threads(sh.subst);
    shapes[d][1] = subst_variant_ring(sh.subst);
    shapes[d][2] = sh.rhs_threads;
  }
  if (tuned) *tuned = s->tuned_now ? 1 : 0;
  return EMMI_OK;
}

int emmi_solver_time_smoother(emmi_solver* s, int dir, int reps, double* ms, int* launches,
                              double* bytes) {
  if (!s || dir < 0 || dir > 2 || reps < 1 || s->lmax < 2) {
    set_err("emmi_solver_time_smoother: bad argument");
    return EMMI_EINVAL;
  }
  // the hierarchy whose level 1 coarsens `dir` (its uncoarsened direction
  // is another one), so level 0 relaxes lines along dir
  int h = -1;
  for (int c = 0; c < 3 && h < 0; c++)
    if (s->hier[c][1].sc[dir] == 2) h = c;
  if (h < 0) {
    set_err("emmi_solver_time_smoother: direction %d is never coarsened", dir);
    return EMMI_EINVAL;
  }
  const bool mixed = s->opt.precision == EMMI_PREC_MIXED;
  std::vector<int> all(s->nrhs, 1);
  CK(cudaMemcpyAsync(s->d_active, all.data(), s->nrhs * sizeof(int), cudaMemcpyHostToDevice, s->st));
  auto sweep = [&]() {
    for (int cc = 0; cc < 4; cc++)
      for (int r0 = 0; r0 < s->nrhs; r0 += s->chunk) {
        const int nr = std::min(s->chunk, s->nrhs - r0);
        if (mixed) {
          LevelView<float> W = s->view<float>(h, 0);
          W.nrhs = nr;
          W.u += (long)r0 * 3 * W.S;
          W.f += (long)r0 * 3 * W.S;
          W.r += (long)r0 * 3 * W.S;
          W.wmu += r0;
          W.active += r0;
          W.op += r0;
          line_colour<float>(s, h, 0, dir, cc, W, r0);
        } else {
          LevelView<double> W = s->view<double>(h, 0);
          W.nrhs = nr;
          W.u += (long)r0 * 3 * W.S;
          W.f += (long)r0 * 3 * W.S;
          W.r += (long)r0 * 3 * W.S;
          W.wmu += r0;
          W.active += r0;
          W.op += r0;
          line_colour<double>(s, h, 0, dir, cc, W, r0);
        }
      }
  };
  sweep();  // warm
  CK(cudaEventRecord(s->ev0, s->st));
  for (int i = 0; i < reps; i++) sweep();
  CK(cudaEventRecord(s->ev1, s->st));
  CK(cudaStreamSynchronize(s->st));
  CK(cudaGetLastError());
  float t = 0;
  cudaEventElapsedTime(&t, s->ev0, s->ev1);
  const double c = mixed ? 8.0 : 16.0;
  if (ms) *ms = t / reps;
  if (launches) *launches = 4 * line_launches(s, h, 0, dir) * ((s->nrhs + s->chunk - 1) / s->chunk);
  if (bytes) *bytes = (double)s->hier[0][0].S * (9 * c + 12) * s->nrhs;
  return EMMI_OK;
}

double emmi_solver_last_time(const emmi_solver* s) { return s ? s->last_time : 0.0; }
long emmi_solver_last_launches(const emmi_solver* s) { return s ? s->last_launches : 0; }
size_t emmi_solver_device_bytes(const emmi_solver* s) { return s ? s->bytes : 0; }
int emmi_solver_line_factor_format(const emmi_solver* s) {
  return s && s->fac_on ? s->fac_fmt : -1;
}
int emmi_solver_geometric_weights(const emmi_solver* s) { return s && s->imu_vol ? 1 : 0; }
int emmi_solver_staged(const emmi_solver* s) { return s && s->plan[0][0].ok ? 1 : 0; }

int emmi_stencil_wait_hook(emmi_solver* s, long long wait_cycles, int stall_from) {
  if (!s || wait_cycles < 0 || stall_from < -1) {
    set_err("emmi_stencil_wait_hook: bad argument");
    return EMMI_EINVAL;
  }
  for (int h = 0; h < 3; h++)
    for (int l = 0; l < kMaxLev; l++)
      if (s->plan[h][l].ok) stencil_hook(&s->plan[h][l], wait_cycles, stall_from);
  return EMMI_OK;
}
int emmi_solver_line_format(const emmi_solver* s) {
  return s && (s->opt.line_sweep || s->opt.fused_level < s->lmax) ? s->lfmt : -1;
}

void emmi_solver_destroy(emmi_solver* s) {
  if (!s) return;
  if (s->st2) {
    cudaStreamSynchronize(s->st2);
    cudaStreamDestroy(s->st2);
  }
  if (s->ev_coef) cudaEventDestroy(s->ev_coef);
  if (s->st) cudaStreamSynchronize(s->st);
  for (int h = 0; h < 3; h++) {
    if (s->gA[h]) cudaGraphExecDestroy(s->gA[h]);
    if (s->gB[h]) cudaGraphExecDestroy(s->gB[h]);
  }
  if (s->st) {
    for (void* p : s->allocs) cudaFreeAsync(p, s->st);
    cudaStreamSynchronize(s->st);
  }
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->st) cudaStreamDestroy(s->st);
  delete s;
}

int emmi_trim_memory(void) {
  int dev = 0;
  cudaMemPool_t pool;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess) {
    set_err("emmi_trim_memory: no device memory pool");
    return EMMI_ECUDA;
  }
  CK(cudaDeviceSynchronize());
  CK(cudaMemPoolTrimTo(pool, 0));
  return EMMI_OK;
}

}  // extern "C"

// ------------------------------------------------------------ single level
namespace {
struct OneLevel {
  std::vector<void*> ptrs;
  ~OneLevel() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename P> cudaError_t get(P** p, size_t b) {
    cudaError_t e = cudaMalloc((void**)p, b);
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
};

template <typename T>
int level_op(const int n[3], const double* x1, const double* x2, const double* x3,
             const double* cells, double omega, int dir, int iter, double* u, const double* f,
             double* r, double* norm) {
  OneLevel M;
  const int gmax = std::max(n[0], std::max(n[1], n[2]));
  const int gmax1 = gmax + 1, gstride = 9 * gmax1;
  std::vector<double> g(gstride, 0.0), xs(gmax1);
  const double* xin[3] = {x1, x2, x3};
  for (int e = 0; e < 3; e++) {
    for (int i = 0; i <= n[e]; i++) g[e * gmax1 + i] = xin[e][i];
    stagger(n[e], g.data() + e * gmax1, xs.data(), g.data() + (6 + e) * gmax1,
            g.data() + (3 + e) * gmax1);
  }
  std::vector<T> gT(gstride);
  for (int i = 0; i < gstride; i++) gT[i] = (T)g[i];
  const long S = (long)(n[0] + 1) * (n[1] + 1) * (n[2] + 1);
  const long nc = (long)n[0] * n[1] * n[2];
  std::vector<T> cT(4 * nc);
  for (long i = 0; i < 4 * nc; i++) cT[i] = (T)cells[i];
  std::vector<C_t<T>> uT(3 * S), fT(3 * S);
  for (long i = 0; i < 3 * S; i++) {
    uT[i] = mk<T>((T)u[2 * i], (T)u[2 * i + 1]);
    fT[i] = mk<T>((T)f[2 * i], (T)f[2 * i + 1]);
  }
  LevelView<T> V;
  for (int e = 0; e < 3; e++) V.n[e] = n[e];
  set_slot_divs(V);
  V.nrhs = 1;
  V.S = S;
  V.ncell = nc;
  V.gstride = gstride;
  V.gmax1 = gmax1;
  T* dg;
  T* dc;
  T* dw;
  C_t<T>*du, *df, *dr;
  double* dn;
  void* scr = nullptr;
  const T wmu = (T)(omega * kMu0);
  CK(M.get(&dg, gstride * sizeof(T)));
  CK(M.get(&dc, 4 * nc * sizeof(T)));
  CK(M.get(&dw, sizeof(T)));
  CK(M.get(&du, 3 * S * sizeof(C_t<T>)));
  CK(M.get(&df, 3 * S * sizeof(C_t<T>)));
  CK(M.get(&dr, 3 * S * sizeof(C_t<T>)));
  CK(M.get(&dn, sizeof(double)));
  CK(cudaMemcpy(dg, gT.data(), gstride * sizeof(T), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dc, cT.data(), 4 * nc * sizeof(T), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dw, &wmu, sizeof(T), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(du, uT.data(), 3 * S * sizeof(C_t<T>), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(df, fT.data(), 3 * S * sizeof(C_t<T>), cudaMemcpyHostToDevice));
  CK(cudaMemset(dn, 0, sizeof(double)));
  V.geo = dg;
  V.cells = dc;
  V.u = du;
  V.f = df;
  V.r = dr;
  V.wmu = dw;
  V.active = nullptr;
  V.op = nullptr;
  if (r) {
    launch_residual<T, T>(V, dr, dn, 0);
  } else if (dir < 3) {
    CK(M.get((C_t<T>**)&scr, line_scratch_elems(n, dir, 1) * sizeof(C_t<T>) + 16));
    for (int cc = 0; cc < 4; cc++)
      launch_line_sweep<T>(V, dir, iter % 2 ? 3 - cc : cc, (C_t<T>*)scr, 0);
  } else {
    for (int cc = 0; cc < 8; cc++) launch_point_sweep<T>(V, iter % 2 ? 7 - cc : cc, 0);
  }
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  std::vector<C_t<T>> out(3 * S);
  CK(cudaMemcpy(out.data(), r ? dr : du, 3 * S * sizeof(C_t<T>), cudaMemcpyDeviceToHost));
  double* dst = r ? r : u;
  for (long i = 0; i < 3 * S; i++) {
    dst[2 * i] = (double)out[i].x;
    dst[2 * i + 1] = (double)out[i].y;
  }
  if (norm) {
    double nn;
    CK(cudaMemcpy(&nn, dn, sizeof(double), cudaMemcpyDeviceToHost));
    *norm = std::sqrt(nn);
  }
  return EMMI_OK;
}

// one transfer between a level of nf cells and the level coarsened by sc
// (coordinates sub-sampled, as the hierarchy builds them): dir 0 restricts
// the fine in to the coarse out, dir 1 adds the prolongation of the coarse
// in to the fine out
template <typename T>
int level_xfer(const int nf[3], const double* const xf[3], const int sc[3], int dir,
               const double* in, double* out) {
  OneLevel M;
  int nc[3];
  for (int e = 0; e < 3; e++) nc[e] = nf[e] / sc[e];
  const int gmax = std::max(nf[0], std::max(nf[1], nf[2]));
  const int gmax1 = gmax + 1, gstride = 9 * gmax1;
  std::vector<T> gF(gstride, T(0)), gC(gstride, T(0));
  for (int e = 0; e < 3; e++) {
    for (int i = 0; i <= nf[e]; i++) gF[e * gmax1 + i] = (T)xf[e][i];
    for (int i = 0; i <= nc[e]; i++) gC[e * gmax1 + i] = (T)xf[e][sc[e] * i];
  }
  LevelView<T> F, Cc;
  for (int e = 0; e < 3; e++) {
    F.n[e] = nf[e];
    Cc.n[e] = nc[e];
  }
  set_slot_divs(F);
  set_slot_divs(Cc);
  F.nrhs = Cc.nrhs = 1;
  F.S = (long)(nf[0] + 1) * (nf[1] + 1) * (nf[2] + 1);
  Cc.S = (long)(nc[0] + 1) * (nc[1] + 1) * (nc[2] + 1);
  F.ncell = (long)nf[0] * nf[1] * nf[2];
  Cc.ncell = (long)nc[0] * nc[1] * nc[2];
  F.gstride = Cc.gstride = gstride;
  F.gmax1 = Cc.gmax1 = gmax1;
  F.active = Cc.active = nullptr;
  F.op = Cc.op = nullptr;
  T *dgF, *dgC, *dw;
  C_t<T>*dfine, *dcf, *dcu;
  CK(M.get(&dgF, gstride * sizeof(T)));
  CK(M.get(&dgC, gstride * sizeof(T)));
  CK(M.get(&dw, 3 * gmax1 * sizeof(T)));
  CK(M.get(&dfine, 3 * F.S * sizeof(C_t<T>)));
  CK(M.get(&dcf, 3 * Cc.S * sizeof(C_t<T>)));
  CK(M.get(&dcu, 3 * Cc.S * sizeof(C_t<T>)));
  CK(cudaMemcpy(dgF, gF.data(), gstride * sizeof(T), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dgC, gC.data(), gstride * sizeof(T), cudaMemcpyHostToDevice));
  const long nin = 3 * (dir == 0 ? F.S : Cc.S), nout = 3 * (dir == 0 ? Cc.S : F.S);
  std::vector<C_t<T>> hin(nin), hout(nout);
  for (long i = 0; i < nin; i++) hin[i] = mk<T>((T)in[2 * i], (T)in[2 * i + 1]);
  for (long i = 0; i < nout; i++) hout[i] = mk<T>((T)out[2 * i], (T)out[2 * i + 1]);
  F.geo = dgF;
  Cc.geo = dgC;
  F.u = F.r = dfine;
  F.f = nullptr;
  Cc.f = dcf;
  Cc.u = dcu;
  launch_xfer_weights<T>(F, Cc, sc, 1, dw, 0);
  F.xw = dw;
  if (dir == 0) {
    CK(cudaMemcpy(dfine, hin.data(), nin * sizeof(C_t<T>), cudaMemcpyHostToDevice));
    launch_restrict<T>(F, Cc, sc, 0);
  } else {
    CK(cudaMemcpy(dcu, hin.data(), nin * sizeof(C_t<T>), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dfine, hout.data(), nout * sizeof(C_t<T>), cudaMemcpyHostToDevice));
    launch_prolong<T>(F, Cc, sc, 0);
  }
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(hout.data(), dir == 0 ? dcf : dfine, nout * sizeof(C_t<T>), cudaMemcpyDeviceToHost));
  for (long i = 0; i < nout; i++) {
    out[2 * i] = (double)hout[i].x;
    out[2 * i + 1] = (double)hout[i].y;
  }
  return EMMI_OK;
}
}  // namespace

extern "C" {

int emmi_level_residual(const int n[3], const double* x1, const double* x2, const double* x3,
                        const double* cells, double omega, int prec, const double* u,
                        const double* f, double* r, double* norm) {
  if (!n || !x1 || !x2 || !x3 || !cells || !u || !f || !r) {
    set_err("emmi_level_residual: null argument");
    return EMMI_EINVAL;
  }
  double* uc = const_cast<double*>(u);
  return prec == EMMI_PREC_FP64
             ? level_op<double>(n, x1, x2, x3, cells, omega, 0, 0, uc, f, r, norm)
             : level_op<float>(n, x1, x2, x3, cells, omega, 0, 0, uc, f, r, norm);
}

int emmi_level_transfer(const int nf[3], const double* x1, const double* x2, const double* x3,
                        const int sc[3], int prec, int dir, const double* in, double* out) {
  if (!nf || !x1 || !x2 || !x3 || !sc || !in || !out || dir < 0 || dir > 1) {
    set_err("emmi_level_transfer: bad argument");
    return EMMI_EINVAL;
  }
  for (int e = 0; e < 3; e++)
    if ((sc[e] != 1 && sc[e] != 2) || nf[e] < 2 || nf[e] % sc[e] != 0) {
      set_err("emmi_level_transfer: sc must be 1 or 2 and divide n (n >= 2)");
      return EMMI_EINVAL;
    }
  const double* xf[3] = {x1, x2, x3};
  return prec == EMMI_PREC_FP64 ? level_xfer<double>(nf, xf, sc, dir, in, out)
                                : level_xfer<float>(nf, xf, sc, dir, in, out);
}

int emmi_level_smooth(const int n[3], const double* x1, const double* x2, const double* x3,
                      const double* cells, double omega, int prec, int dir, int iter, double* u,
                      const double* f) {
  if (!n || !x1 || !x2 || !x3 || !cells || !u || !f || dir < 0 || dir > 3) {
    set_err("emmi_level_smooth: bad argument");
    return EMMI_EINVAL;
  }
  return prec == EMMI_PREC_FP64
             ? level_op<double>(n, x1, x2, x3, cells, omega, dir, iter, u, f, nullptr, nullptr)
             : level_op<float>(n, x1, x2, x3, cells, omega, dir, iter, u, f, nullptr, nullptr);
}

}  // extern "C"


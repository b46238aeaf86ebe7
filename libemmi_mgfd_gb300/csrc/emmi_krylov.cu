// Outer Krylov loop of the mixed-precision solver: restarted flexible GMRES
// in FP64 with one complex64 multigrid cycle as its right preconditioner.
//
// The reference runs stationary cycles (gmg_apply, src/gmg.c:1911-1926).
// Here, with opt.precision = MIXED and opt.krylov = m > 0, every RHS runs
// FGMRES(m): the basis vectors, their dot products and norms, the Hessenberg
// columns and the accumulated solution are FP64; z_j = M^-1 v_j is one
// complex64 F/V/W cycle from zero on the floored preconditioner operator,
// kept in complex64; A z_j is the FP64 residual kernel with f = 0.  The cycle
// rotates its semi-coarsening direction from one application to the next,
// which the flexible variant allows.  Every RHS keeps its own restart state;
// the kernels index each RHS's basis slot from a per-RHS table, so RHS that
// restart or finish at different times share the launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <vector>

#include "emmi_solver_impl.cuh"

using namespace emmi;

#define CK(x)                                                                      \
  do {                                                                             \
    cudaError_t e_ = (x);                                                          \
    if (e_ != cudaSuccess) {                                                       \
      set_err("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_));     \
      return EMMI_ECUDA;                                                           \
    }                                                                              \
  } while (0)

namespace {

constexpr int kH = kMaxKrylov + 1;  // Hessenberg column stride per RHS

unsigned grid_for(long n, long cap = 1024) {
  long b = (n + 255) / 256;
  return (unsigned)std::max(1L, std::min(b, cap));
}

// v_j *= scale (normalises the basis vector in place), f32 = (float) v_j,
// u32 = 0: the right-hand side and start of one preconditioning cycle
__global__ void k_kry_prep(double2* __restrict__ kv, const int* __restrict__ kj,
                           const double* __restrict__ scale, float2* __restrict__ f32,
                           float2* __restrict__ u32, long n3s, int nrhs,
                           const int* __restrict__ active) {
  const int r = blockIdx.y;
  if (!active[r]) return;
  const double sc = scale[r];
  double2* v = kv + ((long)kj[r] * nrhs + r) * n3s;
  float2* f = f32 + (long)r * n3s;
  float2* u = u32 + (long)r * n3s;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n3s;
       i += (long)gridDim.x * blockDim.x) {
    double2 a = v[i];
    a.x *= sc;
    a.y *= sc;
    v[i] = a;
    f[i] = make_float2((float)a.x, (float)a.y);
    u[i] = make_float2(0.f, 0.f);
  }
}

// z_j = u32 (kept in complex64), t = -(double) u32 for the FP64 product
__global__ void k_kry_store(const float2* __restrict__ u32, float2* __restrict__ kz,
                            double2* __restrict__ kt, const int* __restrict__ kj, long n3s,
                            int nrhs, const int* __restrict__ active) {
  const int r = blockIdx.y;
  if (!active[r]) return;
  const float2* u = u32 + (long)r * n3s;
  float2* z = kz + ((long)kj[r] * nrhs + r) * n3s;
  double2* t = kt + (long)r * n3s;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n3s;
       i += (long)gridDim.x * blockDim.x) {
    const float2 a = u[i];
    z[i] = a;
    t[i] = make_double2(-(double)a.x, -(double)a.y);
  }
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// h[r][i] += sum conj(v_i) w over this block's slots, i = 0..kj[r]; w is
// kw[r] (first Gram-Schmidt pass) or, with kw null, basis slot kj[r]+1
// (the second pass over the vector the first pass left there)
__global__ void __launch_bounds__(256) k_kry_dots(const double2* __restrict__ kv,
                                                  const double2* __restrict__ kw,
                                                  const int* __restrict__ kj, long n3s, int nrhs,
                                                  double2* __restrict__ kh,
                                                  const int* __restrict__ active) {
  const int r = blockIdx.y;
  if (!active[r]) return;
  const int j = kj[r];
  double ax[kMaxKrylov], ay[kMaxKrylov];
#pragma unroll
  for (int i = 0; i < kMaxKrylov; i++) ax[i] = ay[i] = 0.0;
  const double2* w = kw ? kw + (long)r * n3s : kv + ((long)(j + 1) * nrhs + r) * n3s;
  for (long s = blockIdx.x * (long)blockDim.x + threadIdx.x; s < n3s;
       s += (long)gridDim.x * blockDim.x) {
    const double2 b = w[s];
#pragma unroll
    for (int i = 0; i < kMaxKrylov; i++)
      if (i <= j) {
        const double2 a = kv[((long)i * nrhs + r) * n3s + s];
        ax[i] += a.x * b.x + a.y * b.y;
        ay[i] += a.x * b.y - a.y * b.x;
      }
  }
  __shared__ double red[8][2 * kMaxKrylov];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < kMaxKrylov; i++) {
    if (i > j) break;
    const double sx = warp_sum_d(ax[i]), sy = warp_sum_d(ay[i]);
    if (lane == 0) {
      red[wid][2 * i] = sx;
      red[wid][2 * i + 1] = sy;
    }
  }
  __syncthreads();
  if (threadIdx.x < 2 * (j + 1)) {
    double v = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) v += red[k][threadIdx.x];
    double* dst = reinterpret_cast<double*>(kh + (long)r * kH) + threadIdx.x;
    atomicAdd(dst, v);
  }
}

// v_{j+1} = w - sum_i h_i v_i ; norm2[r] += |v_{j+1}|^2 (norm2 may be
// null); w is kw[r], or v_{j+1} itself (in place) with kw null
__global__ void __launch_bounds__(256) k_kry_orth(double2* kv, const double2* kw,
                                                  const int* __restrict__ kj, long n3s, int nrhs,
                                                  const double2* __restrict__ kh,
                                                  double* __restrict__ norm2,
                                                  const int* __restrict__ active) {
  const int r = blockIdx.y;
  if (!active[r]) return;
  const int j = kj[r];
  double hx[kMaxKrylov], hy[kMaxKrylov];
#pragma unroll
  for (int i = 0; i < kMaxKrylov; i++) {
    const double2 h = i <= j ? kh[(long)r * kH + i] : make_double2(0.0, 0.0);
    hx[i] = h.x;
    hy[i] = h.y;
  }
  double2* out = kv + ((long)(j + 1) * nrhs + r) * n3s;
  const double2* w = kw ? kw + (long)r * n3s : out;
  double acc = 0.0;
  for (long s = blockIdx.x * (long)blockDim.x + threadIdx.x; s < n3s;
       s += (long)gridDim.x * blockDim.x) {
    double2 b = w[s];
#pragma unroll
    for (int i = 0; i < kMaxKrylov; i++)
      if (i <= j) {
        const double2 a = kv[((long)i * nrhs + r) * n3s + s];
        b.x -= hx[i] * a.x - hy[i] * a.y;
        b.y -= hx[i] * a.y + hy[i] * a.x;
      }
    out[s] = b;
    acc += b.x * b.x + b.y * b.y;
  }
  if (!norm2) return;
  __shared__ double red[8];
  acc = warp_sum_d(acc);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) v += red[k];
    atomicAdd(norm2 + r, v);
  }
}

// x += sum_{i < kj[r]} y_i z_i  (z complex64, x and y FP64)
__global__ void k_kry_update(double2* __restrict__ x, const float2* __restrict__ kz,
                             const double2* __restrict__ ky, const int* __restrict__ kj,
                             long n3s, int nrhs, const int* __restrict__ mask) {
  const int r = blockIdx.y;
  if (!mask[r]) return;
  const int k = kj[r];
  double yx[kMaxKrylov], yy[kMaxKrylov];
#pragma unroll
  for (int i = 0; i < kMaxKrylov; i++) {
    const double2 y = i < k ? ky[(long)r * kMaxKrylov + i] : make_double2(0.0, 0.0);
    yx[i] = y.x;
    yy[i] = y.y;
  }
  double2* xr = x + (long)r * n3s;
  for (long s = blockIdx.x * (long)blockDim.x + threadIdx.x; s < n3s;
       s += (long)gridDim.x * blockDim.x) {
    double2 a = xr[s];
#pragma unroll
    for (int i = 0; i < kMaxKrylov; i++)
      if (i < k) {
        const float2 z = kz[((long)i * nrhs + r) * n3s + s];
        a.x += yx[i] * (double)z.x - yy[i] * (double)z.y;
        a.y += yx[i] * (double)z.y + yy[i] * (double)z.x;
      }
    xr[s] = a;
  }
}

using cd = std::complex<double>;

// per-RHS restart state on the host
struct Arnoldi {
  int j = 0;              // basis vectors built in this restart
  cd H[kH][kMaxKrylov];   // rotated Hessenberg (upper triangular part used)
  double c[kMaxKrylov];   // Givens cosines
  cd sn[kMaxKrylov];      // Givens sines
  cd g[kH];               // rotated beta e1
  void start(double beta) {
    j = 0;
    for (int i = 0; i < kH; i++) g[i] = 0.0;
    g[0] = beta;
  }
  // append column j (h[0..j] and the new subdiagonal hn); returns |g[j+1]|
  double push(const double2* h, double hn) {
    cd col[kH];
    for (int i = 0; i <= j; i++) col[i] = cd(h[i].x, h[i].y);
    col[j + 1] = hn;
    for (int i = 0; i < j; i++) {  // earlier rotations
      const cd a = col[i], b = col[i + 1];
      col[i] = c[i] * a + sn[i] * b;
      col[i + 1] = -std::conj(sn[i]) * a + c[i] * b;
    }
    const cd a = col[j];
    const double b = hn;
    const double rho = std::hypot(std::abs(a), b);
    if (rho == 0.0) {
      c[j] = 1.0;
      sn[j] = 0.0;
    } else if (std::abs(a) == 0.0) {
      c[j] = 0.0;
      sn[j] = 1.0;
      col[j] = b;
    } else {
      const cd ph = a / std::abs(a);
      c[j] = std::abs(a) / rho;
      sn[j] = ph * b / rho;
      col[j] = ph * rho;
    }
    col[j + 1] = 0.0;
    for (int i = 0; i <= j; i++) H[i][j] = col[i];
    g[j + 1] = -std::conj(sn[j]) * g[j];
    g[j] = c[j] * g[j];
    j++;
    return std::abs(g[j]);
  }
  // y = R^-1 g over the j columns built
  void solve(double2* y) const {
    cd v[kMaxKrylov];
    for (int i = j - 1; i >= 0; i--) {
      cd t = g[i];
      for (int k = i + 1; k < j; k++) t -= H[i][k] * v[k];
      v[i] = H[i][i] != 0.0 ? t / H[i][i] : 0.0;
    }
    for (int i = 0; i < kMaxKrylov; i++)
      y[i] = i < j ? make_double2(v[i].real(), v[i].imag()) : make_double2(0.0, 0.0);
  }
};

}  // namespace

namespace emmi {

int krylov_alloc(emmi_solver* s) {
  const long n3s = 3 * s->hier[0][0].S;
  const size_t fv = (size_t)n3s * s->nrhs * sizeof(double2);
  const size_t zv = (size_t)n3s * s->nrhs * sizeof(float2);
  // keep the workspace below 96 GB: shorten the restart if needed
  int m = std::min(s->opt.krylov, kMaxKrylov);
  const size_t cap = (size_t)96 << 30;
  while (m > 2 && (m + 3) * fv + m * zv > cap) m--;
  s->kry_m = m;
  int rc;
  if ((rc = s->alloc((void**)&s->kv, (m + 1) * fv)) != EMMI_OK) return rc;
  if ((rc = s->alloc((void**)&s->kz, m * zv)) != EMMI_OK) return rc;
  if ((rc = s->alloc((void**)&s->kt, fv)) != EMMI_OK) return rc;
  if ((rc = s->alloc((void**)&s->kw, fv)) != EMMI_OK) return rc;
  if ((rc = s->alloc((void**)&s->d_kh, (size_t)2 * s->nrhs * kH * sizeof(double2))) != EMMI_OK)
    return rc;
  if ((rc = s->alloc((void**)&s->d_ky, (size_t)s->nrhs * kMaxKrylov * sizeof(double2))) !=
      EMMI_OK)
    return rc;
  if ((rc = s->alloc((void**)&s->d_kscale, (size_t)s->nrhs * sizeof(double))) != EMMI_OK)
    return rc;
  return s->alloc((void**)&s->d_kj, (size_t)s->nrhs * sizeof(int));
}

int krylov_solve(emmi_solver* s, std::vector<int>& cycles, std::vector<int>& status,
                 std::vector<int>& nref, std::vector<double>& rnorm0, std::vector<double>& rn) {
  const int nrhs = s->nrhs, m = s->kry_m;
  const long n3s = 3 * s->hier[0][0].S;
  const double tol = s->opt.tol;
  cudaStream_t st = s->st;
  std::vector<int>& act = s->h_active;
  std::vector<int>& fin = s->h_refine;
  std::vector<Arnoldi> ar(nrhs);
  std::vector<int> kj(nrhs, 0), stall(nrhs, 0), since_best(nrhs, 0);
  std::vector<double> scale(nrhs, 1.0), nrm(nrhs), best(nrhs, INFINITY);
  std::vector<double2> hh((size_t)nrhs * kH), hh2((size_t)nrhs * kH),
      yy((size_t)nrhs * kMaxKrylov);
  const dim3 g(grid_for(n3s), nrhs);

  auto up_int = [&](int* d, const std::vector<int>& h) {
    return cudaMemcpyAsync(d, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice, st);
  };
  // FP64 true residual r = b*vol - A x of the masked RHS into basis slot 0,
  // its squared norm into nrm
  auto true_residual = [&](int* mask) -> int {
    LevelView<double> V = s->view<double>(0, 0);
    V.u = s->u64[0];
    V.f = s->f64[0];
    V.active = mask;
    CK(cudaMemsetAsync(s->d_norm64, 0, nrhs * sizeof(double), st));
    true_residual64<double>(s, V, s->kv, s->d_norm64);
    s->last_launches++;
    CK(cudaMemcpyAsync(nrm.data(), s->d_norm64, nrhs * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return EMMI_OK;
  };

  // x = 0: the first residual is b*vol
  act.assign(nrhs, 1);
  CK(up_int(s->d_active, act));
  int rc = true_residual(s->d_active);
  if (rc != EMMI_OK) return rc;
  for (int r = 0; r < nrhs; r++) {
    rnorm0[r] = rn[r] = std::sqrt(nrm[r]);
    nref[r] = 1;
    if (!(rnorm0[r] > 0) || !std::isfinite(rnorm0[r])) {
      act[r] = 0;
      status[r] = std::isfinite(rnorm0[r]) ? EMMI_SOLVE_OK : EMMI_SOLVE_NONFINITE;
      continue;
    }
    ar[r].start(rnorm0[r]);
    scale[r] = 1.0 / rnorm0[r];
    best[r] = 1.0;
  }

  for (int app = 0; app < s->opt.ncycle; app++) {
    bool any = false;
    for (int r = 0; r < nrhs; r++) {
      any |= act[r] != 0;
      kj[r] = ar[r].j;
    }
    if (!any) break;
    CK(up_int(s->d_active, act));
    CK(up_int(s->d_kj, kj));
    CK(cudaMemcpyAsync(s->d_kscale, scale.data(), nrhs * sizeof(double), cudaMemcpyHostToDevice,
                       st));
    // z_j = M^-1 v_j : one complex64 cycle from zero
    k_kry_prep<<<g, 256, 0, st>>>(s->kv, s->d_kj, s->d_kscale, s->f32[0], s->u32[0], n3s, nrhs,
                                  s->d_active);
    s->last_launches++;
    const int hh_ = s->opt.isemicoarsen ? app % 3 : 0;
    if ((rc = run_part(s, hh_, 0)) != EMMI_OK) return rc;
    if ((rc = run_part(s, hh_, 1)) != EMMI_OK) return rc;
    if (s->learned_on && (rc = learned_after_cycle(s, hh_, act)) != EMMI_OK) return rc;
    k_kry_store<<<g, 256, 0, st>>>(s->u32[0], s->kz, s->kt, s->d_kj, n3s, nrhs, s->d_active);
    // w = A z_j = 0 - A (-z_j), FP64
    LevelView<double> V = s->view<double>(0, 0);
    V.u = s->kt;
    V.f = nullptr;
    V.active = s->d_active;
    true_residual64<double>(s, V, s->kw, nullptr);
    // classical Gram-Schmidt against v_0..v_j, twice (the second pass
    // restores the orthogonality the first loses when A M^-1 has clustered
    // eigenvalues), then |v_{j+1}|
    double2* kh2 = s->d_kh + (size_t)nrhs * kH;
    CK(cudaMemsetAsync(s->d_kh, 0, (size_t)2 * nrhs * kH * sizeof(double2), st));
    CK(cudaMemsetAsync(s->d_norm64, 0, nrhs * sizeof(double), st));
    k_kry_dots<<<g, 256, 0, st>>>(s->kv, s->kw, s->d_kj, n3s, nrhs, s->d_kh, s->d_active);
    k_kry_orth<<<g, 256, 0, st>>>(s->kv, s->kw, s->d_kj, n3s, nrhs, s->d_kh, nullptr,
                                  s->d_active);
    k_kry_dots<<<g, 256, 0, st>>>(s->kv, nullptr, s->d_kj, n3s, nrhs, kh2, s->d_active);
    k_kry_orth<<<g, 256, 0, st>>>(s->kv, nullptr, s->d_kj, n3s, nrhs, kh2, s->d_norm64,
                                  s->d_active);
    s->last_launches += 6;
    CK(cudaMemcpyAsync(hh.data(), s->d_kh, hh.size() * sizeof(double2), cudaMemcpyDeviceToHost,
                       st));
    CK(cudaMemcpyAsync(hh2.data(), kh2, hh2.size() * sizeof(double2), cudaMemcpyDeviceToHost,
                       st));
    CK(cudaMemcpyAsync(nrm.data(), s->d_norm64, nrhs * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    // an fp16 multiplier of the line sweep out of range: redo this
    // preconditioner application with working-precision multipliers
    if ((rc = line_format_fallback(s)) < 0) return rc;
    if (rc == 1) {
      rc = EMMI_OK;
      app--;
      continue;
    }
    for (size_t q = 0; q < hh.size(); q++) {
      hh[q].x += hh2[q].x;
      hh[q].y += hh2[q].y;
    }

    bool anyfin = false;
    fin.assign(nrhs, 0);
    for (int r = 0; r < nrhs; r++) {
      if (!act[r]) continue;
      cycles[r]++;
      since_best[r]++;
      const double hn = std::sqrt(nrm[r]);
      const double est = ar[r].push(&hh[(size_t)r * kH], hn);
      if (s->opt.verb) printf("icycle=%d rnorm=%e\n", cycles[r] - 1, est);
      scale[r] = hn > 0 ? 1.0 / hn : 0.0;
      if (!std::isfinite(est) || est <= tol * rnorm0[r] || ar[r].j == m || hn == 0.0 ||
          app + 1 == s->opt.ncycle) {
        fin[r] = 1;
        anyfin = true;
      }
    }
    if (!anyfin) continue;

    // finish the restart of the flagged RHS: x += Z y, then the true residual
    for (int r = 0; r < nrhs; r++) {
      kj[r] = fin[r] ? ar[r].j : 0;
      if (fin[r]) ar[r].solve(&yy[(size_t)r * kMaxKrylov]);
    }
    CK(up_int(s->d_refine, fin));
    CK(up_int(s->d_kj, kj));
    CK(cudaMemcpyAsync(s->d_ky, yy.data(), yy.size() * sizeof(double2), cudaMemcpyHostToDevice,
                       st));
    k_kry_update<<<g, 256, 0, st>>>(s->u64[0], s->kz, s->d_ky, s->d_kj, n3s, nrhs, s->d_refine);
    s->last_launches++;
    if ((rc = true_residual(s->d_refine)) != EMMI_OK) return rc;
    for (int r = 0; r < nrhs; r++) {
      if (!fin[r]) continue;
      nref[r]++;
      rn[r] = std::sqrt(nrm[r]);
      const double rel = rn[r] / rnorm0[r];
      if (!std::isfinite(rel)) {
        act[r] = 0;
        status[r] = EMMI_SOLVE_NONFINITE;
      } else if (rel <= tol) {
        act[r] = 0;
        status[r] = EMMI_SOLVE_OK;
      } else if (rel < 0.5 * best[r]) {
        best[r] = rel;
        stall[r] = 0;
        since_best[r] = 0;
      } else if (learned_fallback(s, r)) {
        stall[r] = 0;  // no halving over a restart with the learned correction
      } else if (++stall[r] >= 3 && since_best[r] >= 12) {
        // three restarts and twelve cycles without halving the residual
        act[r] = 0;
        status[r] = EMMI_SOLVE_STALL;
      }
      if (act[r]) {  // restart from the true residual
        ar[r].start(rn[r]);
        scale[r] = 1.0 / rn[r];
      }
    }
  }
  for (int r = 0; r < nrhs; r++)
    if (act[r]) status[r] = EMMI_SOLVE_MAXIT;
  return EMMI_OK;
}

}  // namespace emmi

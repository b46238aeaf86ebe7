// Learned smoother: a small convolutional correction of the level-0 complex64
// iterate, applied after every multigrid cycle of the mixed-precision solver,
// and the kernels that train it on residuals of plain cycles.
//
// The reference has no counterpart (its smoother is line/patch Gauss-Seidel,
// src/gmg.c:116-1313, which stays the method here); the network only adds a
// correction after each cycle, and a right-hand side whose residual stops
// falling with it switches back to plain cycles.
//
// Network (per level, here level 0): input z = D^-1 r, the residual of the
// complex64 iterate divided by the diagonal of A edge by edge, as 8 channels
// per slot (Ex, Ey, Ez real/imaginary + 2 zero channels) on the
// (n1+1)(n2+1)(n3+1) slot grid; two bias-free linear 3x3x3 convolutions
// 8 -> 8 -> 8 channels (hidden layer bf16); the first 6 output channels are
// the correction, added on unknown edges only.  A linear, bias-free network
// keeps the corrected cycle a fixed linear preconditioner (scale-equivariant),
// so stationary refinement and FGMRES both stay valid.
//
// Forward convolutions run on the tensor cores as an implicit GEMM:
// M = 16 consecutive slots along i, N = 8 output channels, K = tap x channel
// (two taps per k16 step, 14 steps, the 28th tap zero), bf16 operands, fp32
// accumulation (mma.sync m16n8k16; the channel count of 8 is below the
// 64/128-row tiles tcgen05 issues, and the whole network is ~1 % of a cycle).
// Training: loss = sum_b |r_b - A c_b|^2 / |r_b|^2 over residual samples r_b
// (c_b the masked correction), gradients by fp32 CUDA-core kernels.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <type_traits>
#include <vector>

#include "emmi_solver_impl.cuh"

namespace emmi {

namespace {

constexpr int kCh = 8;
constexpr int kTaps = 27;
constexpr int kKSteps = 14;
constexpr int kWLayer = kTaps * kCh * kCh;  // [tap][cin][cout]

// tap t = (dk+1)*9 + (dj+1)*3 + (di+1)
__host__ __device__ constexpr int tap_di(int t) { return t % 3 - 1; }
__host__ __device__ constexpr int tap_dj(int t) { return (t / 3) % 3 - 1; }
__host__ __device__ constexpr int tap_dk(int t) { return t / 9 - 1; }

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat16 a = __float2bfloat16_rn(lo), b = __float2bfloat16_rn(hi);
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}
__device__ __forceinline__ float bf16_lo(uint32_t v) {
  return __bfloat162float(__ushort_as_bfloat16((unsigned short)(v & 0xffffu)));
}
__device__ __forceinline__ float bf16_hi(uint32_t v) {
  return __bfloat162float(__ushort_as_bfloat16((unsigned short)(v >> 16)));
}

template <int C>
__device__ __forceinline__ bool unknown_edge(const int n[3], int i, int j, int k) {
  const int P[3] = {i, j, k};
  constexpr int p = (C + 1) % 3, q = (C + 2) % 3;
  return P[C] < n[C] && P[p] >= 1 && P[p] < n[p] && P[q] >= 1 && P[q] < n[q];
}
__device__ __forceinline__ bool unknown_any(int c, const int n[3], int i, int j, int k) {
  return c == 0 ? unknown_edge<0>(n, i, j, k)
                : (c == 1 ? unknown_edge<1>(n, i, j, k) : unknown_edge<2>(n, i, j, k));
}

// ---------------------------------------------------------------- weights
// B fragments of mma.m16n8k16 (k x n = 16 x 8): lane (g = lane/4, t4 = lane%4)
// holds k = 2*t4, 2*t4+1 (reg 0) and k = 2*t4+8, +9 (reg 1) of column n = g.
// Here k in [0,8) is tap 2*ks, channels 0..7; k in [8,16) tap 2*ks+1.
__global__ void k_ls_pack(const float* __restrict__ W, uint32_t* __restrict__ Wp) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;  // [layer][ks][lane]
  if (id >= 2 * kKSteps * 32) return;
  const int lane = id % 32, ks = (id / 32) % kKSteps, layer = id / (32 * kKSteps);
  const int g = lane >> 2, t4 = lane & 3;
  const float* w = W + layer * kWLayer;
  uint32_t r[2];
  for (int h = 0; h < 2; h++) {
    const int t = 2 * ks + h;
    float lo = 0.f, hi = 0.f;
    if (t < kTaps) {
      lo = w[(t * kCh + 2 * t4) * kCh + g];
      hi = w[(t * kCh + 2 * t4 + 1) * kCh + g];
    }
    r[h] = pack_bf16x2(lo, hi);
  }
  Wp[2 * id] = r[0];
  Wp[2 * id + 1] = r[1];
}

// ---------------------------------------------------------------- input
// X[b][s][8] bf16 = D^-1 r on unknown edges, 0 elsewhere.  r is read from
// rin ([b][3][S] complex64) when given, else formed as f - A u on L.
__global__ void __launch_bounds__(256) k_ls_input(LevelView<float> L, const float2* __restrict__ rin,
                                                  uint32_t* __restrict__ X) {
  const int b = blockIdx.y;
  if (L.active && !L.active[b]) return;
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= L.S) return;
  const int n0 = L.n[0] + 1, n1 = L.n[1] + 1;
  const int P[3] = {(int)(s % n0), (int)((s / n0) % n1), (int)(s / ((long)n0 * n1))};
  const long ss[3] = {1, (long)n0, (long)n0 * n1};
  const float2* u = L.u + (long)b * 3 * L.S;
  const float2* f = L.f ? L.f + (long)b * 3 * L.S : nullptr;
  const float* cells = L.cells + (long)op_of(L, b) * 4 * L.ncell;
  const Geo<float> G{L.geo + (long)op_of(L, b) * L.gstride, L.gmax1};
  const float wmu = L.wmu[b];
  uint32_t out[4] = {0u, 0u, 0u, 0u};
  auto one = [&](auto cc) {
    constexpr int C = decltype(cc)::value;
    if (!unknown_edge<C>(L.n, P[0], P[1], P[2])) return;
    EdgeCoef<float> e;
    float2 r;
    if (rin) {
      edge_coef<float, C>(L.n, P, cells + (long)C * L.ncell, cells + 3 * L.ncell, G, wmu, e);
      r = rin[((long)b * 3 + C) * L.S + s];
    } else {
      const float2 au = apply_row<float, C>(L, u, cells, G, wmu, P, s, ss, e);
      const float2 fv = f ? f[(long)C * L.S + s] : make_float2(0.f, 0.f);
      r = make_float2(fv.x - au.x, fv.y - au.y);
    }
    // z = r / d = r conj(d) / |d|^2
    const float d2 = e.dre * e.dre + e.dim * e.dim;
    const float zr = (r.x * e.dre + r.y * e.dim) / d2;
    const float zi = (r.y * e.dre - r.x * e.dim) / d2;
    out[C] = pack_bf16x2(zr, zi);
  };
  one(std::integral_constant<int, 0>());
  one(std::integral_constant<int, 1>());
  one(std::integral_constant<int, 2>());
  reinterpret_cast<uint4*>(X)[(long)b * L.S + s] = make_uint4(out[0], out[1], out[2], out[3]);
}

// ---------------------------------------------------------------- conv
// One 3x3x3 convolution, 8 -> 8 channels, on the tensor cores.  A block of
// 4 warps owns a brick of 48 x 2 x 2 slots (i, j, k): it stages the brick
// and its one-slot halo (50 x 4 x 4 slots x 16 bytes) in shared memory with
// coalesced loads, then each warp computes 3 of the brick's 12 m-tiles
// (16 consecutive slots along i) with A fragments read from shared memory
// (8 consecutive slots x 4 words per load: conflict-free).
//   MODE 0: out = hidden layer, bf16 [b][S][8]
//   MODE 1: u += channels 0..5 on unknown edges (deployment)
//   MODE 2: c = channels 0..5 on unknown edges, 0 elsewhere ([b][3][S])
struct ConvArgs {
  int n[3];      // cells of the level
  int X, Y, Z;   // slots per direction (n+1)
  long S;
  int tiles;     // bricks per RHS
  const int* mask;
};

constexpr int kBI = 48, kBJ = 2, kBK = 2;
constexpr int kHI = kBI + 2, kHJ = kBJ + 2, kHK = kBK + 2;

template <int MODE>
__global__ void __launch_bounds__(128) k_ls_conv(ConvArgs a, const uint32_t* __restrict__ in,
                                                 const uint32_t* __restrict__ Wp,
                                                 uint32_t* __restrict__ hid,
                                                 float2* __restrict__ out) {
  __shared__ uint4 halo[kHK * kHJ * kHI];
  const int b = blockIdx.y;
  if (a.mask && !a.mask[b]) return;
  const int nbi = (a.X + kBI - 1) / kBI, nbj = (a.Y + kBJ - 1) / kBJ;
  const int brick = blockIdx.x;
  const int bi0 = (brick % nbi) * kBI;
  const int bj0 = ((brick / nbi) % nbj) * kBJ;
  const int bk0 = (brick / (nbi * nbj)) * kBK;
  const uint4* inb = reinterpret_cast<const uint4*>(in) + (long)b * a.S;
  for (int q = threadIdx.x; q < kHK * kHJ * kHI; q += blockDim.x) {
    const int hi = q % kHI, hj = (q / kHI) % kHJ, hk = q / (kHI * kHJ);
    const int i = bi0 + hi - 1, j = bj0 + hj - 1, k = bk0 + hk - 1;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (i >= 0 && i < a.X && j >= 0 && j < a.Y && k >= 0 && k < a.Z)
      v = inb[((long)k * a.Y + j) * a.X + i];
    halo[q] = v;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t4 = lane & 3;
  uint32_t bw[kKSteps][2];
#pragma unroll
  for (int ks = 0; ks < kKSteps; ks++) {
    bw[ks][0] = Wp[(ks * 32 + lane) * 2];
    bw[ks][1] = Wp[(ks * 32 + lane) * 2 + 1];
  }
  __syncthreads();
  const uint32_t* hw = reinterpret_cast<const uint32_t*>(halo);
  for (int tl = warp; tl < (kBI / 16) * kBJ * kBK; tl += blockDim.x >> 5) {
    const int ib = tl % (kBI / 16), jl = (tl / (kBI / 16)) % kBJ, kl = tl / ((kBI / 16) * kBJ);
    const int j = bj0 + jl, k = bk0 + kl;
    if (j >= a.Y || k >= a.Z) continue;  // warp-uniform
    const int iA = bi0 + 16 * ib + g, iB = iA + 8;
    // halo word of the slot at local i offset li, shifted by tap t
    auto ld = [&](int li, int t) -> uint32_t {
      const int hi = li + 1 + tap_di(t), hj = jl + 1 + tap_dj(t), hk = kl + 1 + tap_dk(t);
      return hw[((hk * kHJ + hj) * kHI + hi) * 4 + t4];
    };
    const int liA = 16 * ib + g, liB = liA + 8;
    float c0 = 0.f, c1 = 0.f, c2 = 0.f, c3 = 0.f;
#pragma unroll
    for (int ks = 0; ks < kKSteps; ks++) {
      const int t0 = 2 * ks, t1 = 2 * ks + 1;
      const uint32_t a0 = ld(liA, t0);
      const uint32_t a1 = ld(liB, t0);
      uint32_t a2 = 0u, a3 = 0u;
      if (t1 < kTaps) {
        a2 = ld(liA, t1);
        a3 = ld(liB, t1);
      }
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
          "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
          : "+f"(c0), "+f"(c1), "+f"(c2), "+f"(c3)
          : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(bw[ks][0]), "r"(bw[ks][1]));
    }
    // c0, c1: slot iA, channels 2*t4, 2*t4+1 ; c2, c3: slot iB
    if (MODE == 0) {
      uint32_t* hb = hid + (long)b * a.S * 4;
      if (iA < a.X) hb[(((long)k * a.Y + j) * a.X + iA) * 4 + t4] = pack_bf16x2(c0, c1);
      if (iB < a.X) hb[(((long)k * a.Y + j) * a.X + iB) * 4 + t4] = pack_bf16x2(c2, c3);
    } else if (t4 < 3) {
      const int comp = t4;
      float2* ob = out + ((long)b * 3 + comp) * a.S;
      auto put = [&](int i, float x, float y) {
        if (i >= a.X) return;
        const long s = ((long)k * a.Y + j) * a.X + i;
        const bool unk = unknown_any(comp, a.n, i, j, k);
        if (MODE == 1) {
          if (unk) {
            float2 v = ob[s];
            v.x += x;
            v.y += y;
            ob[s] = v;
          }
        } else {
          ob[s] = unk ? make_float2(x, y) : make_float2(0.f, 0.f);
        }
      };
      put(iA, c0, c1);
      put(iB, c2, c3);
    }
  }
}

// ---------------------------------------------------------------- training
// gc[b][s][8] = dL/dc on unknown edges: t = -A conj(e) gives
// dL/dRe c = 2 t.x / |r_b|^2, dL/dIm c = -2 t.y / |r_b|^2
__global__ void k_ls_grad_c(ConvArgs a, const float2* __restrict__ t,
                            const double* __restrict__ rn2, float4* __restrict__ gc) {
  const int b = blockIdx.y;
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= a.S) return;
  const int i = (int)(s % a.X), j = (int)((s / a.X) % a.Y), k = (int)(s / ((long)a.X * a.Y));
  const float w = (float)(2.0 / rn2[b]);
  float v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int c = 0; c < 3; c++)
    if (unknown_any(c, a.n, i, j, k)) {
      const float2 tv = t[((long)b * 3 + c) * a.S + s];
      v[2 * c] = w * tv.x;
      v[2 * c + 1] = -w * tv.y;
    }
  gc[((long)b * a.S + s) * 2] = make_float4(v[0], v[1], v[2], v[3]);
  gc[((long)b * a.S + s) * 2 + 1] = make_float4(v[4], v[5], v[6], v[7]);
}

// e = conj(e) on unknown edges, 0 elsewhere: the loss only sees unknown rows
// of A c, so the adjoint A^T conj(e) takes e on those rows only
__global__ void k_ls_conj(ConvArgs a, float2* __restrict__ e) {
  const int b = blockIdx.y;
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= a.S) return;
  const int i = (int)(s % a.X), j = (int)((s / a.X) % a.Y), k = (int)(s / ((long)a.X * a.Y));
  for (int c = 0; c < 3; c++) {
    float2& v = e[((long)b * 3 + c) * a.S + s];
    v = unknown_any(c, a.n, i, j, k) ? make_float2(v.x, -v.y) : make_float2(0.f, 0.f);
  }
}

// dW[t][cin][cout] += sum_s g[s][cout] * in[s + off(t)][cin]
// block: 64 slots of one row in shared memory with their 9-row halo; the
// 256 threads are 4 tap groups x 64 (cin, cout) pairs
constexpr int kDwTile = 64;
__global__ void __launch_bounds__(256) k_ls_dw(ConvArgs a, const float4* __restrict__ g,
                                               const uint32_t* __restrict__ in,
                                               float* __restrict__ dW) {
  const int b = blockIdx.y;
  const int mt = (a.X + kDwTile - 1) / kDwTile;
  const int row = blockIdx.x / mt;
  const int i0 = (blockIdx.x % mt) * kDwTile;
  const int j = row % a.Y, k = row / a.Y;
  __shared__ float gs[kDwTile][kCh];
  __shared__ float hs[9][kDwTile + 2][kCh];
  const float4* gb = g + (long)b * a.S * 2;
  const uint32_t* ib = in + (long)b * a.S * 4;
  for (int q = threadIdx.x; q < kDwTile * 2; q += blockDim.x) {
    const int p = q >> 1, h = q & 1, i = i0 + p;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i < a.X) v = gb[((((long)k * a.Y + j) * a.X) + i) * 2 + h];
    gs[p][4 * h] = v.x;
    gs[p][4 * h + 1] = v.y;
    gs[p][4 * h + 2] = v.z;
    gs[p][4 * h + 3] = v.w;
  }
  for (int q = threadIdx.x; q < 9 * (kDwTile + 2) * 4; q += blockDim.x) {
    const int w4 = q & 3, p = (q >> 2) % (kDwTile + 2), r9 = (q >> 2) / (kDwTile + 2);
    const int jj = j + (r9 % 3) - 1, kk = k + (r9 / 3) - 1, ii = i0 + p - 1;
    uint32_t v = 0u;
    if (ii >= 0 && ii < a.X && jj >= 0 && jj < a.Y && kk >= 0 && kk < a.Z)
      v = ib[(((long)kk * a.Y + jj) * a.X + ii) * 4 + w4];
    hs[r9][p][2 * w4] = bf16_lo(v);
    hs[r9][p][2 * w4 + 1] = bf16_hi(v);
  }
  __syncthreads();
  const int pair = threadIdx.x & 63, grp = threadIdx.x >> 6;
  const int cin = pair >> 3, cout = pair & 7;
  const int np = min(kDwTile, a.X - i0);
  for (int t = grp; t < kTaps; t += 4) {
    const int r9 = (tap_dk(t) + 1) * 3 + (tap_dj(t) + 1), di = tap_di(t);
    float acc = 0.f;
    for (int p = 0; p < np; p++) acc += gs[p][cout] * hs[r9][p + 1 + di][cin];
    if (acc != 0.f) atomicAdd(dW + (t * kCh + cin) * kCh + cout, acc);
  }
}

// gh[s][cin] = sum_t sum_cout W[t][cin][cout] * g[s - off(t)][cout], with
// the bf16-rounded weights the forward convolution used
__global__ void __launch_bounds__(256) k_ls_dgrad(ConvArgs a, const float4* __restrict__ g,
                                                  const float* __restrict__ W,
                                                  float4* __restrict__ gh) {
  __shared__ float ws[kWLayer];
  for (int q = threadIdx.x; q < kWLayer; q += blockDim.x)
    ws[q] = __bfloat162float(__float2bfloat16_rn(W[q]));
  __syncthreads();
  const int b = blockIdx.y;
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= a.S) return;
  const int i = (int)(s % a.X), j = (int)((s / a.X) % a.Y), k = (int)(s / ((long)a.X * a.Y));
  const float4* gb = g + (long)b * a.S * 2;
  float acc[kCh] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int t = 0; t < kTaps; t++) {
    const int ii = i - tap_di(t), jj = j - tap_dj(t), kk = k - tap_dk(t);
    if (ii < 0 || ii >= a.X || jj < 0 || jj >= a.Y || kk < 0 || kk >= a.Z) continue;
    const long q = ((long)kk * a.Y + jj) * a.X + ii;
    const float4 v0 = gb[q * 2], v1 = gb[q * 2 + 1];
    const float gv[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
#pragma unroll
    for (int ci = 0; ci < kCh; ci++) {
      float sum = 0.f;
#pragma unroll
      for (int co = 0; co < kCh; co++) sum += ws[(t * kCh + ci) * kCh + co] * gv[co];
      acc[ci] += sum;
    }
  }
  gh[((long)b * a.S + s) * 2] = make_float4(acc[0], acc[1], acc[2], acc[3]);
  gh[((long)b * a.S + s) * 2 + 1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
}

// Adam on the fp32 master weights (grad = dW already summed over samples)
__global__ void k_ls_adam(float* __restrict__ W, const float* __restrict__ dW,
                          float* __restrict__ m1, float* __restrict__ m2, int n, float lr,
                          float b1, float b2, float c1, float c2, float eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gr = dW[i];
  const float a = b1 * m1[i] + (1.f - b1) * gr;
  const float v = b2 * m2[i] + (1.f - b2) * gr * gr;
  m1[i] = a;
  m2[i] = v;
  W[i] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
}

ConvArgs conv_args(const int n[3], int nb, const int* mask) {
  ConvArgs a;
  for (int e = 0; e < 3; e++) a.n[e] = n[e];
  a.X = n[0] + 1;
  a.Y = n[1] + 1;
  a.Z = n[2] + 1;
  a.S = (long)a.X * a.Y * a.Z;
  a.tiles = ((a.X + kBI - 1) / kBI) * ((a.Y + kBJ - 1) / kBJ) * ((a.Z + kBK - 1) / kBK);
  a.mask = mask;
  (void)nb;
  return a;
}

unsigned conv_blocks(const ConvArgs& a) { return (unsigned)a.tiles; }

}  // namespace

// ---------------------------------------------------------------- host API
void learned_pack(const float* dW32, uint32_t* dWp, cudaStream_t st) {
  k_ls_pack<<<(2 * kKSteps * 32 + 127) / 128, 128, 0, st>>>(dW32, dWp);
}

// u += N(D^-1 (f - A u)) on the RHS that mask selects (level-0 view L)
void learned_apply(const LevelView<float>& L, const uint32_t* Wp, uint32_t* X, uint32_t* H,
                   cudaStream_t st) {
  dim3 g1((unsigned)((L.S + 255) / 256), L.nrhs);
  k_ls_input<<<g1, 256, 0, st>>>(L, nullptr, X);
  ConvArgs a = conv_args(L.n, L.nrhs, L.active);
  dim3 g2(conv_blocks(a), L.nrhs);
  k_ls_conv<0><<<g2, 128, 0, st>>>(a, X, Wp, H, nullptr);
  k_ls_conv<1><<<g2, 128, 0, st>>>(a, H, Wp + kKSteps * 32 * 2, nullptr, L.u);
}

size_t learned_scratch_bytes(long S, int nrhs) { return (size_t)2 * S * nrhs * 16; }

// One training step over all samples (LevelView L: u = c buffer, f = r
// samples, r = e buffer, nrhs = samples, op/wmu per sample).  Buffers:
// X, H bf16 [B][S][8]; t complex64 [B][3][S]; gc, gh fp32 [B][S][8];
// loss2 [B] (|e_b|^2 out), rn2 [B] (|r_b|^2 in); W [2][1728] fp32 master,
// dW, m1, m2 same size, Wp packed.
struct TrainBuffers {
  uint32_t *X, *H, *Wp;
  float2 *c, *e, *t;
  float4 *gc, *gh;
  double *loss2, *rn2;
  float *W, *dW, *m1, *m2;
};

int learned_train_step(const LevelView<float>& L, const TrainBuffers& B, int step, float lr,
                       cudaStream_t st) {
  const int nb = L.nrhs;
  ConvArgs a = conv_args(L.n, nb, nullptr);
  dim3 gs((unsigned)((L.S + 255) / 256), nb);
  dim3 gc(conv_blocks(a), nb);
  LevelView<float> V = L;
  V.active = nullptr;
  // forward: X = D^-1 r, H = W1 * X, c = W2 * H (masked)
  k_ls_input<<<gs, 256, 0, st>>>(V, V.f, B.X);
  k_ls_conv<0><<<gc, 128, 0, st>>>(a, B.X, B.Wp, B.H, nullptr);
  k_ls_conv<2><<<gc, 128, 0, st>>>(a, B.H, B.Wp + kKSteps * 32 * 2, nullptr, B.c);
  // e = r - A c and |e|^2
  cudaMemsetAsync(B.loss2, 0, nb * sizeof(double), st);
  LevelView<float> R = V;
  R.u = B.c;
  launch_residual<float, float>(R, B.e, B.loss2, st);
  // t = -A conj(e), gc = dL/dc
  k_ls_conj<<<gs, 256, 0, st>>>(a, B.e);
  LevelView<float> Q = V;
  Q.u = B.e;
  Q.f = nullptr;
  launch_residual<float, float>(Q, B.t, nullptr, st);
  k_ls_grad_c<<<gs, 256, 0, st>>>(a, B.t, B.rn2, B.gc);
  // backward through the two convolutions
  cudaMemsetAsync(B.dW, 0, 2 * kWLayer * sizeof(float), st);
  const int mt = (a.X + kDwTile - 1) / kDwTile;
  dim3 gd((unsigned)(mt * a.Y * a.Z), nb);
  k_ls_dw<<<gd, 256, 0, st>>>(a, B.gc, B.H, B.dW + kWLayer);
  k_ls_dgrad<<<gs, 256, 0, st>>>(a, B.gc, B.W + kWLayer, B.gh);
  k_ls_dw<<<gd, 256, 0, st>>>(a, B.gh, B.X, B.dW);
  if (lr > 0) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)(step + 1)), c2 = 1.f - powf(b2, (float)(step + 1));
    k_ls_adam<<<(2 * kWLayer + 255) / 256, 256, 0, st>>>(B.W, B.dW, B.m1, B.m2, 2 * kWLayer, lr,
                                                        b1, b2, c1, c2, 1e-8f);
    learned_pack(B.W, B.Wp, st);
  }
  return cudaGetLastError() == cudaSuccess ? EMMI_OK : EMMI_ECUDA;
}

}  // namespace emmi

// ---------------------------------------------------------------- solver hooks
namespace emmi {

int learned_after_cycle(emmi_solver* s, int h, const std::vector<int>& act) {
  bool any = false;
  std::vector<int> m(s->nrhs);
  for (int r = 0; r < s->nrhs; r++) {
    m[r] = act[r] && s->h_learn[r];
    any |= m[r] != 0;
  }
  if (!any) return EMMI_OK;
  cudaError_t e =
      cudaMemcpyAsync(s->d_learn, m.data(), m.size() * sizeof(int), cudaMemcpyHostToDevice, s->st);
  if (e != cudaSuccess) {
    set_err("learned correction: %s", cudaGetErrorString(e));
    return EMMI_ECUDA;
  }
  LevelView<float> L = s->view<float>(h, 0);
  L.active = s->d_learn;
  learned_apply(L, s->d_lsWp, s->d_lsX, s->d_lsH, s->st);
  s->last_launches += 3;
  return EMMI_OK;
}

bool learned_fallback(emmi_solver* s, int r) {
  if (!s->learned_on || !s->h_learn[r]) return false;
  s->h_learn[r] = 0;
  s->h_fallback[r] = 1;
  return true;
}

int learned_snapshot(emmi_solver* s, int h, const std::vector<int>& act) {
  const long n3s = 3 * s->hier[0][0].S;
  LevelView<float> R = s->view<float>(h, 0);
  R.active = s->d_active;
  cudaStream_t st = s->st;
  cudaMemsetAsync(s->d_norm, 0, s->nrhs * sizeof(double), st);
  launch_residual<float, float>(R, R.r, s->d_norm, st);
  for (int r = 0; r < s->nrhs && s->ls_count < s->ls_cap; r++) {
    if (!act[r] || s->h_taken[r] >= s->ls_per_rhs) continue;
    const int k = s->ls_count++;
    s->h_taken[r]++;
    s->h_sop[k] = s->h_op[r];
    cudaMemcpyAsync(s->d_samples + (long)k * n3s, R.r + (long)r * n3s, n3s * sizeof(float2),
                    cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(s->d_srn2 + k, s->d_norm + r, sizeof(double), cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(s->d_swmu + k, s->d_wmu32 + r, sizeof(float), cudaMemcpyDeviceToDevice, st);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_err("learned snapshot: %s", cudaGetErrorString(e));
    return EMMI_ECUDA;
  }
  return EMMI_OK;
}

}  // namespace emmi

// ---------------------------------------------------------------- C ABI
using namespace emmi;

#define LCK(x)                                                                     \
  do {                                                                             \
    cudaError_t e_ = (x);                                                          \
    if (e_ != cudaSuccess) {                                                       \
      set_err("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_));     \
      return EMMI_ECUDA;                                                           \
    }                                                                              \
  } while (0)

namespace {

int ensure_training_set(emmi_solver* s, int cap) {
  if (s->d_samples && s->ls_cap >= cap) return EMMI_OK;
  if (s->d_samples) {
    set_err("learned training set: capacity is fixed at its first allocation (%d)", s->ls_cap);
    return EMMI_ESTATE;
  }
  const long n3s = 3 * s->hier[0][0].S;
  int rc;
  if ((rc = s->alloc((void**)&s->d_samples, (size_t)cap * n3s * sizeof(float2))) != EMMI_OK)
    return rc;
  if ((rc = s->alloc((void**)&s->d_srn2, (size_t)cap * sizeof(double))) != EMMI_OK) return rc;
  if ((rc = s->alloc((void**)&s->d_sop, (size_t)cap * sizeof(int))) != EMMI_OK) return rc;
  if ((rc = s->alloc((void**)&s->d_swmu, (size_t)cap * sizeof(float))) != EMMI_OK) return rc;
  s->ls_cap = cap;
  s->ls_count = 0;
  s->h_sop.assign(cap, 0);
  return EMMI_OK;
}

// the level-0 view over the training samples (u, r: the caller's buffers)
LevelView<float> sample_view(emmi_solver* s) {
  LevelView<float> L = s->view<float>(0, 0);
  L.nrhs = s->ls_count;
  L.f = s->d_samples;
  L.wmu = s->d_swmu;
  L.op = s->d_sop;
  L.active = nullptr;
  return L;
}

struct TrainAlloc {
  std::vector<void*> p;
  ~TrainAlloc() {
    for (void* q : p) cudaFree(q);
  }
  template <typename T> cudaError_t get(T** out, size_t bytes) {
    cudaError_t e = cudaMalloc((void**)out, bytes);
    if (e == cudaSuccess) p.push_back(*out);
    return e;
  }
};

int train_impl(emmi_solver* s, int steps, float lr, float* W, float* loss, float* grad) {
  if (!s || !W || steps < 1 || s->opt.precision != EMMI_PREC_MIXED) {
    set_err("emmi_learned_train: bad argument (a MIXED solver, weights and steps >= 1)");
    return EMMI_EINVAL;
  }
  const int ns = s->ls_count;
  if (ns < 1) {
    set_err("emmi_learned_train: the training set is empty");
    return EMMI_ESTATE;
  }
  cudaStream_t st = s->st;
  LCK(cudaMemcpyAsync(s->d_sop, s->h_sop.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st));
  const long S = s->hier[0][0].S;
  TrainAlloc A;
  TrainBuffers B;
  const size_t nw = 2 * kWLayer;
  LCK(A.get(&B.X, (size_t)ns * S * 16));
  LCK(A.get(&B.H, (size_t)ns * S * 16));
  LCK(A.get(&B.c, (size_t)ns * 3 * S * sizeof(float2)));
  LCK(A.get(&B.e, (size_t)ns * 3 * S * sizeof(float2)));
  LCK(A.get(&B.t, (size_t)ns * 3 * S * sizeof(float2)));
  LCK(A.get(&B.gc, (size_t)ns * S * 32));
  LCK(A.get(&B.gh, (size_t)ns * S * 32));
  LCK(A.get(&B.loss2, ns * sizeof(double)));
  B.rn2 = s->d_srn2;
  LCK(A.get(&B.W, nw * sizeof(float)));
  LCK(A.get(&B.dW, nw * sizeof(float)));
  LCK(A.get(&B.m1, nw * sizeof(float)));
  LCK(A.get(&B.m2, nw * sizeof(float)));
  LCK(A.get(&B.Wp, (size_t)2 * kKSteps * 32 * 2 * sizeof(uint32_t)));
  LCK(cudaMemcpyAsync(B.W, W, nw * sizeof(float), cudaMemcpyHostToDevice, st));
  LCK(cudaMemsetAsync(B.m1, 0, nw * sizeof(float), st));
  LCK(cudaMemsetAsync(B.m2, 0, nw * sizeof(float), st));
  learned_pack(B.W, B.Wp, st);
  std::vector<double> rn2(ns), l2(ns);
  LCK(cudaMemcpyAsync(rn2.data(), s->d_srn2, ns * sizeof(double), cudaMemcpyDeviceToHost, st));
  LevelView<float> L = sample_view(s);
  L.u = B.c;
  L.r = B.e;
  for (int it = 0; it < steps; it++) {
    int rc = learned_train_step(L, B, it, grad ? 0.f : lr, st);
    if (rc != EMMI_OK) {
      set_err("emmi_learned_train: launch failed: %s", cudaGetErrorString(cudaGetLastError()));
      return rc;
    }
    LCK(cudaMemcpyAsync(l2.data(), B.loss2, ns * sizeof(double), cudaMemcpyDeviceToHost, st));
    LCK(cudaStreamSynchronize(st));
    double sum = 0;
    for (int k = 0; k < ns; k++) sum += rn2[k] > 0 ? l2[k] / rn2[k] : 0.0;
    if (loss) loss[it] = (float)(sum / ns);
  }
  if (grad) {
    LCK(cudaMemcpyAsync(grad, B.dW, nw * sizeof(float), cudaMemcpyDeviceToHost, st));
  } else {
    LCK(cudaMemcpyAsync(W, B.W, nw * sizeof(float), cudaMemcpyDeviceToHost, st));
  }
  LCK(cudaStreamSynchronize(st));
  return EMMI_OK;
}

}  // namespace

extern "C" {

int emmi_learned_collect(emmi_solver* s, const double* b, int device, int per_rhs,
                         emmi_rhs_stats* stats) {
  if (!s || !b || per_rhs < 1 || s->opt.precision != EMMI_PREC_MIXED || s->kry_m > 0) {
    set_err("emmi_learned_collect: bad argument (a MIXED solver without krylov, b, per_rhs >= 1)");
    return EMMI_EINVAL;
  }
  int rc = ensure_training_set(s, s->ls_count + per_rhs * s->nrhs);
  if (rc != EMMI_OK) return rc;
  const bool was_on = s->learned_on;
  s->learned_on = false;  // residuals of plain cycles
  s->ls_collect = true;
  s->ls_per_rhs = per_rhs;
  s->h_taken.assign(s->nrhs, 0);
  // the solution is not kept: x goes to a scratch buffer on b's side
  const long n3s = 3 * s->hier[0][0].S;
  std::vector<double2> xh;
  TrainAlloc A;
  double* x = nullptr;
  if (device) {
    rc = A.get(&x, (size_t)s->nrhs * n3s * sizeof(double2)) == cudaSuccess ? EMMI_OK : EMMI_ENOMEM;
  } else {
    xh.resize((size_t)s->nrhs * n3s);
    x = reinterpret_cast<double*>(xh.data());
  }
  if (rc == EMMI_OK) rc = emmi_solver_solve(s, b, x, nullptr, device ? 1 : 0, stats);
  s->ls_collect = false;
  s->learned_on = was_on;
  return rc;
}

int emmi_learned_add_samples(emmi_solver* s, int ns, const float* r, const int* rhs) {
  if (!s || ns < 1 || !r || !rhs || s->opt.precision != EMMI_PREC_MIXED) {
    set_err("emmi_learned_add_samples: bad argument");
    return EMMI_EINVAL;
  }
  int rc = ensure_training_set(s, s->ls_count + ns);
  if (rc != EMMI_OK) return rc;
  const long n3s = 3 * s->hier[0][0].S;
  cudaStream_t st = s->st;
  for (int k = 0; k < ns; k++)
    if (rhs[k] < 0 || rhs[k] >= s->nrhs) {
      set_err("emmi_learned_add_samples: rhs index %d out of range", rhs[k]);
      return EMMI_EINVAL;
    }
  const int k0 = s->ls_count;
  LCK(cudaMemcpyAsync(s->d_samples + (long)k0 * n3s, r, (size_t)ns * n3s * sizeof(float2),
                      cudaMemcpyHostToDevice, st));
  for (int k = 0; k < ns; k++) {
    s->h_sop[k0 + k] = s->h_op[rhs[k]];
    LCK(cudaMemcpyAsync(s->d_swmu + k0 + k, s->d_wmu32 + rhs[k], sizeof(float),
                        cudaMemcpyDeviceToDevice, st));
  }
  s->ls_count += ns;
  // |r|^2 of the new samples
  std::vector<double> nn(ns, 0.0);
  for (int k = 0; k < ns; k++) {
    const float* q = r + (size_t)k * n3s * 2;
    double a = 0;
    for (long i = 0; i < 2 * n3s; i++) a += (double)q[i] * q[i];
    nn[k] = a;
  }
  LCK(cudaMemcpyAsync(s->d_srn2 + k0, nn.data(), ns * sizeof(double), cudaMemcpyHostToDevice, st));
  LCK(cudaStreamSynchronize(st));
  return EMMI_OK;
}

int emmi_learned_samples(const emmi_solver* s) { return s ? s->ls_count : 0; }

int emmi_learned_train(emmi_solver* s, int steps, float lr, float* W, float* loss) {
  return train_impl(s, steps, lr, W, loss, nullptr);
}

int emmi_learned_grad(emmi_solver* s, const float* W, float* loss, float* grad) {
  if (!grad) {
    set_err("emmi_learned_grad: null gradient");
    return EMMI_EINVAL;
  }
  std::vector<float> w(W, W + 2 * kWLayer);
  return train_impl(s, 1, 0.f, w.data(), loss, grad);
}

int emmi_learned_set(emmi_solver* s, const float* W) {
  if (!s || s->opt.precision != EMMI_PREC_MIXED) {
    set_err("emmi_learned_set: the learned correction needs a MIXED solver");
    return EMMI_EINVAL;
  }
  if (!W) {
    s->learned_on = false;
    return EMMI_OK;
  }
  const long S = s->hier[0][0].S;
  int rc;
  if (!s->d_lsW) {
    if ((rc = s->alloc((void**)&s->d_lsW, 2 * kWLayer * sizeof(float))) != EMMI_OK) return rc;
    if ((rc = s->alloc((void**)&s->d_lsWp, (size_t)2 * kKSteps * 32 * 2 * sizeof(uint32_t))) !=
        EMMI_OK)
      return rc;
    if ((rc = s->alloc((void**)&s->d_lsX, (size_t)s->nrhs * S * 16)) != EMMI_OK) return rc;
    if ((rc = s->alloc((void**)&s->d_lsH, (size_t)s->nrhs * S * 16)) != EMMI_OK) return rc;
    if ((rc = s->alloc((void**)&s->d_learn, (size_t)s->nrhs * sizeof(int))) != EMMI_OK) return rc;
  }
  LCK(cudaMemcpyAsync(s->d_lsW, W, 2 * kWLayer * sizeof(float), cudaMemcpyHostToDevice, s->st));
  learned_pack(s->d_lsW, s->d_lsWp, s->st);
  LCK(cudaStreamSynchronize(s->st));
  s->learned_on = true;
  return EMMI_OK;
}

}  // extern "C"

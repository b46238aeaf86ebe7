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
// 8 -> 8 -> 8 channels with zero padding; the hidden layer is rounded to
// bf16 and is zero on the last slot plane of each direction (i = n1, j = n2,
// k = n3), where no component has an unknown edge; the first 6 output
// channels are the correction, added on unknown edges only.  A linear,
// bias-free network keeps the corrected cycle a fixed linear preconditioner
// (scale-equivariant), so stationary refinement and FGMRES both stay valid.
//
// The convolutions run on the fifth-generation tensor cores (tcgen05.mma,
// bf16 operands from shared memory, fp32 accumulators in tensor memory) as
// an implicit GEMM over the flattened slot index s = i + X j + X Y k: tap
// (di, dj, dk) reads slot s + di + X dj + X Y dk.  On the flattened index a
// tap that leaves the grid lands on the last plane of a lower direction (or
// on the previous right-hand side's last plane, or a zero guard), and both
// layer inputs are zero there, so the flattened convolution equals the
// zero-padded one on every slot whose output is used.  Training: loss =
// sum_b |r_b - A c_b|^2 / |r_b|^2 over residual samples r_b (c_b the masked
// correction), gradients by fp32 CUDA-core kernels.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <mutex>
#include <type_traits>
#include <vector>

#include "emmi_solver_impl.cuh"

namespace emmi {

namespace {

constexpr int kCh = 8;
constexpr int kTaps = 27;
constexpr int kTcInstr = 15;  // tcgen05.mma per output tile
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
// B operands of the tensor-core convolution, one 16 x 16 bf16 matrix per
// instruction (N = 16 output columns, 8 of them zero; K = 16 = two taps x 8
// input channels), K-major without swizzle: the 8 x 8 core matrix (n-group
// ng, k-group kc) at byte 256 kc + 128 ng, row n % 8 at 16 bytes, element
// k % 8 at 2 bytes.  Instruction q covers plane dk = q / 5 - 1 and the tap
// pair 2 (q % 5), 2 (q % 5) + 1 of that plane's 9 taps (raster (dj, di));
// the fifth pair holds the ninth tap alone (its second half zero).
__global__ void k_ls_pack(const float* __restrict__ W, uint4* __restrict__ Wt) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;  // [layer][q][kc][ng][n8]
  if (id >= 2 * kTcInstr * 32) return;
  const int n8 = id & 7, ng = (id >> 3) & 1, kc = (id >> 4) & 1, q = (id >> 5) % kTcInstr,
            layer = id / (32 * kTcInstr);
  const int dk = q / 5 - 1, pi = q % 5;
  const int r = 2 * pi + kc;  // tap of this k-group within the plane's raster
  const int n = 8 * ng + n8;
  const float* w = W + layer * kWLayer;
  uint32_t v[4];
  for (int e = 0; e < 4; e++) {
    float lo = 0.f, hi = 0.f;
    if (n < kCh && r < 9) {
      const int t = (dk + 1) * 9 + r;
      lo = w[(t * kCh + 2 * e) * kCh + n];
      hi = w[(t * kCh + 2 * e + 1) * kCh + n];
    }
    v[e] = pack_bf16x2(lo, hi);
  }
  Wt[id] = make_uint4(v[0], v[1], v[2], v[3]);
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
  int P[3];
  slot_nodes(s, L, P);
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
      edge_coef<float, C>(L.n, P, cells + (long)C * L.ncell, cells + 3 * L.ncell, G, wmu, e,
                          L.imu_vol);
      r = rin[((long)b * 3 + C) * L.S + s];
    } else {
      const float2 au = apply_row<float, C>(L, u, cells, G, wmu, P, s, ss, e);
      const float2 fv = f ? f[(long)C * L.S + s] : make_float2(0.f, 0.f);
      r = make_float2(fv.x - au.x, fv.y - au.y);
    }
    // z = r / d = r conj(d) / |d|^2
    const float inv = 1.f / (e.dre * e.dre + e.dim * e.dim);
    const float zr = (r.x * e.dre + r.y * e.dim) * inv;
    const float zi = (r.y * e.dre - r.x * e.dim) * inv;
    out[C] = pack_bf16x2(zr, zi);
  };
  one(std::integral_constant<int, 0>());
  one(std::integral_constant<int, 1>());
  one(std::integral_constant<int, 2>());
  reinterpret_cast<uint4*>(X)[(long)b * L.S + s] = make_uint4(out[0], out[1], out[2], out[3]);
}

// ---------------------------------------------------------------- conv
// PTX wrappers: mbarriers, the bulk copy engine, tensor memory, tcgen05.
__device__ __forceinline__ uint32_t su32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}
__device__ __forceinline__ uint32_t mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok;
}
// a wait that gives up after `limit` clocks (false; about a second by
// default): the caller records the failure and leaves without touching the
// data
constexpr long long kWaitCycles = 2000000000LL;
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long limit) {
  const long long t0 = clock64();
  while (!mbar_test(bar, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes,
                                          uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::
          "r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
// shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte
// offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor: D f32, A and B bf16, both K-major, N = 16, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((16u >> 3) << 17) |
                            ((128u >> 4) << 24);
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(kIdesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                   bar)
               : "memory");
}
__device__ __forceinline__ void tc_load8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

// One 3x3x3 convolution, 8 -> 8 channels, bf16 slots [b][S] (16 bytes per
// slot) with kTcGuard(X, Y) zero slots before the first and after the last
// right-hand side.  A CTA owns one column of 128 consecutive in-plane slots
// (p = i + X j) and walks the planes k of one chunk; the tile of plane k is
// D[m][n] = sum_taps X[s_m + off(tap)] W_tap, 15 tcgen05.mma (M = 128 slots,
// N = 16, K = 16) into one of two tensor-memory accumulators.  One thread of
// the producer warp issues the copies and the MMAs; 4 epilogue warps (one
// TMEM lane per thread) read the accumulators back and store; the two sides
// meet only at mbarriers (window landed, accumulator ready, accumulator read
// back), so the MMAs of the next planes run while an epilogue stores.  Each
// plane's window (slots p0 - X - 1 ... p0 + 127 + X + 2 of that plane,
// contiguous) comes in by one bulk copy, kTcAhead planes ahead, into a ring
// of kTcRing windows; the window serves as the A operand of the plane's
// three dk roles directly: tap (di, dj) is the 128-row matrix starting
// X + 1 + X dj + di slots in (rows 16 bytes apart, 8 channels each = one
// core-matrix row).
//   MODE 0: hidden layer, bf16 [b][S] (guarded layout), zero on the planes
//           i = X-1, j = Y-1, k = Z-1
//   MODE 1: u += channels 0..5 on unknown edges (deployment)
//   MODE 2: c = channels 0..5 on unknown edges, 0 elsewhere ([b][3][S])
// Plane k = Z-1 holds no unknown edge: it is never computed (MODE 0 and 2
// write its zeros).  Waits are bounded; a CTA that gives up sets *err,
// drains its copies and MMAs and frees its tensor memory.
struct ConvArgs {
  int n[3];      // cells of the level
  int X, Y, Z;   // slots per direction (n+1)
  long S;
  int XY;        // slots per plane
  int ncol;      // 128-slot columns per plane
  int nchunk;    // plane chunks per column
  int W;         // window slots: 128 + 2X + 3
  int wbytes;    // window stride in shared memory (16 W rounded up to 128)
  const int* mask;
  long long wait;  // clocks a wait gives up after (kWaitCycles)
  int stall;       // test hook: 1 = the producer issues no copy and no MMA, so
                   // the epilogue's first wait has nothing to wait for
};

constexpr int kTcEpiWarps = 4;  // epilogue warps (TMEM lanes 0..127); one producer warp
constexpr int kTcThreads = 32 * (kTcEpiWarps + 1);
constexpr int kTcRing = 7;      // plane windows in shared memory
constexpr int kTcAhead = kTcRing - 3;  // planes loaded ahead of the MMAs
constexpr int kTcPlanes = 32;   // planes per chunk
constexpr int kTcCols = 32;     // tensor memory: 2 accumulators x 16 columns
// dynamic shared memory a CTA may ask for (227 KB less the static part)
constexpr int kConvSmemMax = 227 * 1024 - 1024;
__host__ __device__ inline long kTcGuard(int X, int Y) { return (long)X * Y + X + 129; }
inline size_t conv_smem(const ConvArgs& a) {
  return (size_t)kTcInstr * 512 + (size_t)kTcRing * a.wbytes;
}

template <int MODE>
__global__ void __launch_bounds__(kTcThreads) k_ls_conv(ConvArgs a, const uint4* __restrict__ in,
                                                        const uint4* __restrict__ Wt,
                                                        uint4* __restrict__ hid,
                                                        float2* __restrict__ out,
                                                        int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char dsm[];
  __shared__ __align__(8) uint64_t bar_full[kTcRing];  // window landed (bulk copy)
  __shared__ __align__(8) uint64_t bar_done[2];        // accumulator ready (tcgen05.commit)
  __shared__ __align__(8) uint64_t bar_free[2];        // accumulator read back (4 epilogue warps)
  __shared__ uint32_t tmem_base;
  __shared__ volatile int failed;
  const int b = blockIdx.y;
  if (a.mask && !a.mask[b]) return;
  // an earlier CTA gave up: the launch has failed (one read for the CTA, so
  // that every thread leaves or stays)
  if (threadIdx.x == 0) failed = *(volatile int*)err ? 1 : 0;
  __syncthreads();
  if (failed) return;
  const int col = blockIdx.x % a.ncol, chunk = blockIdx.x / a.ncol;
  const int k0 = chunk * kTcPlanes;
  const int k1 = min(k0 + kTcPlanes, a.Z - 1);  // planes [k0, k1) are computed
  const int tid = threadIdx.x, warp = tid >> 5;
  uint4* sB = reinterpret_cast<uint4*>(dsm);
  unsigned char* ring = dsm + kTcInstr * 512;
  const int p0 = 128 * col;  // first in-plane slot of the column

  for (int q = tid; q < kTcInstr * 32; q += blockDim.x) sB[q] = Wt[q];
  // generic-proxy stores, read below by the tensor core (async proxy)
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  __syncwarp();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     su32(&tmem_base)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    for (int i = 0; i < kTcRing; i++) mbar_init(su32(&bar_full[i]), 1);
    for (int i = 0; i < 2; i++) {
      mbar_init(su32(&bar_done[i]), 1);
      mbar_init(su32(&bar_free[i]), 4);
    }
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  // plane p -> ring slot and the parity of its use of that slot; plane k's
  // accumulator (16 columns) alternates with k, its u-th use has parity u & 1
  auto slot = [&](int p) { return (p - k0 + 1) % kTcRing; };
  auto parity = [&](int p) { return (uint32_t)(((p - k0 + 1) / kTcRing) & 1); };
  auto acc = [&](int k) { return (k - k0) & 1; };
  auto use = [&](int k) { return (uint32_t)(((k - k0) >> 1) & 1); };

  if (warp == kTcEpiWarps) {
    // ---- producer: one thread issues the window copies and the MMAs
    if ((tid & 31) == 0 && !a.stall) {
      const uint4* inb = in + (long)b * a.S;
      int issued = k0 - 2, waited = k0 - 2, committed = k0 - 1;
      auto load = [&](int p) {
        const uint32_t bar = su32(&bar_full[slot(p)]);
        mbar_expect_tx(bar, (uint32_t)a.W * 16u);
        bulk_load(su32(ring + slot(p) * a.wbytes), inb + (long)p * a.XY + p0 - a.X - 1,
                  (uint32_t)a.W * 16u, bar);
        issued = p;
      };
      for (int p = k0 - 1; p <= min(k0 + kTcAhead - 1, k1); p++) load(p);
      const uint32_t ring0 = su32(ring), sB0 = su32(sB);
      for (int k = k0; k < k1; k++) {
        bool ok = true;
        // accumulator acc(k) and the window slot of plane k-3 are free once
        // the epilogue of plane k-2 has read its accumulator back
        if (k - 2 >= k0) ok = mbar_wait(su32(&bar_free[acc(k)]), use(k) ^ 1u, a.wait);
        if (ok && k + kTcAhead <= k1) load(k + kTcAhead);
        for (int p = waited + 1; p <= k + 1 && ok; p++) {
          ok = mbar_wait(su32(&bar_full[slot(p)]), parity(p), a.wait);
          if (ok) waited = p;
        }
        if (!ok || failed) {
          failed = 1;
          atomicExch(err, 1);
          break;
        }
        tc_fence_after();
        const uint32_t d = tmem + 16u * (uint32_t)acc(k);
#pragma unroll
        for (int q = 0; q < kTcInstr; q++) {
          const int dk = q / 5 - 1, pi = q % 5;
          const int r0 = 2 * pi;
          const int off0 = (r0 / 3 - 1) * a.X + (r0 % 3 - 1);
          const int off1 = pi < 4 ? ((r0 + 1) / 3 - 1) * a.X + ((r0 + 1) % 3 - 1) : off0 + 1;
          const uint32_t base = ring0 + slot(k + dk) * a.wbytes;
          const uint64_t ad = smem_desc(base + 16u * (uint32_t)(a.X + 1 + off0),
                                        16u * (uint32_t)(off1 - off0), 128u);
          const uint64_t bd = smem_desc(sB0 + 512u * q, 256u, 128u);
          tc_mma(d, ad, bd, q > 0 ? 1u : 0u);
        }
        tc_commit(su32(&bar_done[acc(k)]));
        committed = k;
      }
      if (failed) {
        // copies and MMAs in flight finish before shared and tensor memory go
        for (int p = waited + 1; p <= issued; p++)
          mbar_wait(su32(&bar_full[slot(p)]), parity(p), a.wait);
        if (committed >= k0) mbar_wait(su32(&bar_done[acc(committed)]), use(committed), a.wait);
      }
    }
  } else {
    // ---- epilogue: 4 warps, thread tid reads TMEM lane tid (output slot p0 + tid)
    const int p = p0 + tid;
    const bool live = p < a.XY;
    const int j = live ? p / a.X : 0, i = p - j * a.X;
    for (int k = k0; k < k1; k++) {
      const bool late = !mbar_wait(su32(&bar_done[acc(k)]), use(k), a.wait);
      // the warp leaves together (tcgen05.ld below is warp-collective)
      if (__any_sync(0xffffffffu, late || failed)) {
        if (late) {
          failed = 1;
          atomicExch(err, 2);
        }
        break;
      }
      tc_fence_after();
      __syncwarp();
      float v[8];
      tc_load8(tmem + 16u * (uint32_t)acc(k) + ((uint32_t)(warp * 32) << 16), v);
      tc_fence_before();
      __syncwarp();
      if ((tid & 31) == 0) mbar_arrive(su32(&bar_free[acc(k)]));
      if (live) {
        const long s = (long)k * a.XY + p;
        if (MODE == 0) {
          uint4 h = make_uint4(0u, 0u, 0u, 0u);
          if (i < a.X - 1 && j < a.Y - 1)
            h = make_uint4(pack_bf16x2(v[0], v[1]), pack_bf16x2(v[2], v[3]),
                           pack_bf16x2(v[4], v[5]), pack_bf16x2(v[6], v[7]));
          hid[(long)b * a.S + s] = h;
        } else {
#pragma unroll
          for (int c = 0; c < 3; c++) {
            float2* ob = out + ((long)b * 3 + c) * a.S + s;
            const bool unk = unknown_any(c, a.n, i, j, k);
            if (MODE == 1) {
              if (unk) {
                float2 w = *ob;
                w.x += v[2 * c];
                w.y += v[2 * c + 1];
                *ob = w;
              }
            } else {
              *ob = unk ? make_float2(v[2 * c], v[2 * c + 1]) : make_float2(0.f, 0.f);
            }
          }
        }
      }
    }
    // the last plane (no unknown edges): zeros for the hidden layer and c
    if (MODE != 1 && !failed && chunk == a.nchunk - 1 && live) {
      const long s = (long)(a.Z - 1) * a.XY + p;
      if (MODE == 0) {
        hid[(long)b * a.S + s] = make_uint4(0u, 0u, 0u, 0u);
      } else {
        for (int c = 0; c < 3; c++) out[((long)b * 3 + c) * a.S + s] = make_float2(0.f, 0.f);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  __syncwarp();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "r"(kTcCols)
                 : "memory");
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
  // the hidden layer is zero on the last plane of each direction
  if (i == a.X - 1 || j == a.Y - 1 || k == a.Z - 1)
    for (int ci = 0; ci < kCh; ci++) acc[ci] = 0.f;
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

ConvArgs conv_args(const int n[3], const int* mask) {
  ConvArgs a;
  for (int e = 0; e < 3; e++) a.n[e] = n[e];
  a.X = n[0] + 1;
  a.Y = n[1] + 1;
  a.Z = n[2] + 1;
  a.S = (long)a.X * a.Y * a.Z;
  a.XY = a.X * a.Y;
  a.ncol = (a.XY + 127) / 128;
  a.nchunk = (a.Z - 1 + kTcPlanes - 1) / kTcPlanes;
  a.W = 128 + 2 * a.X + 3;
  a.wbytes = (16 * a.W + 127) / 128 * 128;
  a.mask = mask;
  a.wait = kWaitCycles;
  a.stall = 0;
  return a;
}

// a waiting tensor-core convolution that gave up records why here (1: a
// window copy, 2: the MMAs); read and cleared by learned_check
__device__ int g_ls_err = 0;

int* conv_err() {
  static int* p = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaGetSymbolAddress((void**)&p, g_ls_err);
    const int lim = kConvSmemMax;
    cudaFuncSetAttribute(k_ls_conv<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_ls_conv<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_ls_conv<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  });
  return p;
}

template <int MODE>
void launch_conv(const ConvArgs& a, int nb, const uint32_t* in, const uint4* Wt, uint32_t* hid,
                 float2* out, cudaStream_t st) {
  int* err = conv_err();
  dim3 g((unsigned)(a.ncol * a.nchunk), nb);
  k_ls_conv<MODE><<<g, kTcThreads, conv_smem(a), st>>>(a, reinterpret_cast<const uint4*>(in), Wt,
                                                reinterpret_cast<uint4*>(hid), out, err);
}

}  // namespace

// ---------------------------------------------------------------- host API
void learned_pack(const float* dW32, uint4* dWt, cudaStream_t st) {
  k_ls_pack<<<(2 * kTcInstr * 32 + 127) / 128, 128, 0, st>>>(dW32, dWt);
}

// u += N(D^-1 (f - A u)) on the RHS that mask selects (level-0 view L);
// wait > 0 / stall: the convolutions' wait limit and test stall (ConvArgs)
void learned_apply(const LevelView<float>& L, const uint4* Wt, uint32_t* X, uint32_t* H,
                   cudaStream_t st, long long wait = 0, int stall = 0) {
  dim3 g1((unsigned)((L.S + 255) / 256), L.nrhs);
  k_ls_input<<<g1, 256, 0, st>>>(L, nullptr, X);
  ConvArgs a = conv_args(L.n, L.active);
  if (wait > 0) a.wait = wait;
  a.stall = stall;
  launch_conv<0>(a, L.nrhs, X, Wt, H, nullptr, st);
  launch_conv<1>(a, L.nrhs, H, Wt + kTcInstr * 32, nullptr, L.u, st);
}

// slots of zero guard before and after a bf16 slot buffer of the level
long learned_guard(const int n[3]) { return kTcGuard(n[0] + 1, n[1] + 1); }

// the shared memory one convolution needs on a level of n cells, or -1 if
// it is more than a CTA can have
long learned_smem(const int n[3]) {
  const ConvArgs a = conv_args(n, nullptr);
  const size_t b = conv_smem(a);
  return b <= (size_t)kConvSmemMax ? (long)b : -1;
}

// a convolution's give-up code since the last check (0: none); clears it
int learned_check(cudaStream_t st) {
  int v = 0;
  int* p = conv_err();
  cudaMemcpyAsync(&v, p, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaMemsetAsync(p, 0, sizeof(int), st);
  cudaStreamSynchronize(st);
  return v;
}

// One training step over all samples (LevelView L: u = c buffer, f = r
// samples, r = e buffer, nrhs = samples, op/wmu per sample).  Buffers:
// X, H bf16 [B][S][8]; t complex64 [B][3][S]; gc, gh fp32 [B][S][8];
// loss2 [B] (|e_b|^2 out), rn2 [B] (|r_b|^2 in); W [2][1728] fp32 master,
// dW, m1, m2 same size, Wp packed.
struct TrainBuffers {
  uint32_t *X, *H;  // guarded: learned_guard slots of zeros on both sides
  uint4* Wt;
  float2 *c, *e, *t;
  float4 *gc, *gh;
  double *loss2, *rn2;
  float *W, *dW, *m1, *m2;
};

int learned_train_step(const LevelView<float>& L, const TrainBuffers& B, int step, float lr,
                       cudaStream_t st) {
  const int nb = L.nrhs;
  ConvArgs a = conv_args(L.n, nullptr);
  dim3 gs((unsigned)((L.S + 255) / 256), nb);
  LevelView<float> V = L;
  V.active = nullptr;
  // forward: X = D^-1 r, H = W1 * X, c = W2 * H (masked)
  k_ls_input<<<gs, 256, 0, st>>>(V, V.f, B.X);
  launch_conv<0>(a, nb, B.X, B.Wt, B.H, nullptr, st);
  launch_conv<2>(a, nb, B.H, B.Wt + kTcInstr * 32, nullptr, B.c, st);
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
    learned_pack(B.W, B.Wt, st);
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
  learned_apply(L, s->d_lsWt, s->d_lsX, s->d_lsH, s->st);
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
  const int* nl0 = s->hier[0][0].n;
  if (learned_smem(nl0) < 0) {
    set_err("emmi_learned_train: rows of %d slots are wider than the convolution's shared-memory "
            "window allows", nl0[0] + 1);
    return EMMI_EINVAL;
  }
  const long gd = learned_guard(nl0);
  const size_t xb = (size_t)(ns * S + 2 * gd) * 16;
  LCK(A.get(&B.X, xb));
  LCK(A.get(&B.H, xb));
  LCK(cudaMemsetAsync(B.X, 0, xb, st));
  LCK(cudaMemsetAsync(B.H, 0, xb, st));
  B.X += 4 * gd;
  B.H += 4 * gd;
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
  LCK(A.get(&B.Wt, (size_t)2 * kTcInstr * 32 * sizeof(uint4)));
  LCK(cudaMemcpyAsync(B.W, W, nw * sizeof(float), cudaMemcpyHostToDevice, st));
  LCK(cudaMemsetAsync(B.m1, 0, nw * sizeof(float), st));
  LCK(cudaMemsetAsync(B.m2, 0, nw * sizeof(float), st));
  learned_pack(B.W, B.Wt, st);
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
  if (const int why = learned_check(st)) {
    set_err("emmi_learned_train: a tensor-core convolution gave up waiting (code %d)", why);
    return EMMI_ECUDA;
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

int emmi_learned_apply(emmi_solver* s, const void* f, void* u) {
  if (!s || !f || !u || !s->learned_on) {
    set_err("emmi_learned_apply: bad argument (a solver with weights set, f and u)");
    return EMMI_EINVAL;
  }
  LevelView<float> L = s->view<float>(0, 0);
  L.f = reinterpret_cast<float2*>(const_cast<void*>(f));
  L.u = reinterpret_cast<float2*>(u);
  L.active = nullptr;
  learned_apply(L, s->d_lsWt, s->d_lsX, s->d_lsH, s->st, s->ls_wait, s->ls_stall);
  LCK(cudaGetLastError());
  if (const int why = learned_check(s->st)) {
    set_err("emmi_learned_apply: a tensor-core convolution gave up waiting (code %d)", why);
    return EMMI_ECUDA;
  }
  return EMMI_OK;
}

int emmi_learned_wait_hook(emmi_solver* s, long long wait_cycles, int stall) {
  if (!s || wait_cycles < 0 || (stall != 0 && stall != 1)) {
    set_err("emmi_learned_wait_hook: bad argument");
    return EMMI_EINVAL;
  }
  s->ls_wait = wait_cycles;
  s->ls_stall = stall;
  return EMMI_OK;
}

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
  const int* nl0 = s->hier[0][0].n;
  if (learned_smem(nl0) < 0) {
    set_err("emmi_learned_set: rows of %d slots are wider than the convolution's shared-memory "
            "window allows", nl0[0] + 1);
    return EMMI_EINVAL;
  }
  int rc;
  if (!s->d_lsW) {
    // X and H: [nrhs][S] bf16 slots between two zero guards
    const long gd = learned_guard(nl0);
    const size_t xb = (size_t)(s->nrhs * S + 2 * gd) * 16;
    uint32_t *rx = nullptr, *rh = nullptr;
    if ((rc = s->alloc((void**)&s->d_lsW, 2 * kWLayer * sizeof(float))) != EMMI_OK) return rc;
    if ((rc = s->alloc((void**)&s->d_lsWt, (size_t)2 * kTcInstr * 32 * sizeof(uint4))) != EMMI_OK)
      return rc;
    if ((rc = s->alloc((void**)&rx, xb)) != EMMI_OK) return rc;
    if ((rc = s->alloc((void**)&rh, xb)) != EMMI_OK) return rc;
    if ((rc = s->alloc((void**)&s->d_learn, (size_t)s->nrhs * sizeof(int))) != EMMI_OK) return rc;
    LCK(cudaMemsetAsync(rx, 0, xb, s->st));
    LCK(cudaMemsetAsync(rh, 0, xb, s->st));
    s->d_lsX = rx + 4 * gd;
    s->d_lsH = rh + 4 * gd;
  }
  LCK(cudaMemcpyAsync(s->d_lsW, W, 2 * kWLayer * sizeof(float), cudaMemcpyHostToDevice, s->st));
  learned_pack(s->d_lsW, s->d_lsWt, s->st);
  LCK(cudaStreamSynchronize(s->st));
  s->learned_on = true;
  return EMMI_OK;
}

}  // extern "C"

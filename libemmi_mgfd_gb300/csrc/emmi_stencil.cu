// Residual r = f - A u of a complex64 level with its halos staged in shared
// memory by the tensor-memory accelerator (src/gmg.c:1316-1410, the same
// edge equations as k_residual).
//
// A CTA owns TY rows of slots (all of x) and marches up KZ planes of z.  A
// plane's neighbourhood -- u of the three components on rows j0-1..j0+TY and
// the conductivities (and, with stored weights, the inverse permeabilities)
// of the cells on rows j0-1..j0+TY-1 -- arrives by cp.async.bulk.tensor into
// a ring of four plane slots, two planes ahead of the plane being computed,
// each slot's copies counted on its mbarrier.  Every u value is read from
// DRAM once per tile (plus a two-row halo) instead of by up to 13 threads
// through the caches.
//
// The field arrays are [rhs][3][S] with S = X*Y*Z slots, rows of X slots;
// X*8 bytes is rarely a multiple of 16, which a tensor map's row stride must
// be, so each array is described as a flat 2D tensor of 256-byte rows
// (32 complex64 or 64 float elements) and a window of consecutive grid rows
// is one box of R such rows, starting at the 256-byte row that holds the
// window's first element; the window's offset inside the box is kept with
// it.  The solver pads the arrays to whole 256-byte rows.
//
// Waits are bounded: a wait that runs out (about a second) records a code
// in the error word, the CTA drains the copies it issued (bounded again) and
// returns; the solver reads the word with the cycle norms.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "emmi_kernels.cuh"

namespace emmi {

namespace {

constexpr int kStRing = 4;  // planes k-1..k+1 in use, k+2 in flight
constexpr int kStThreads = 1024;
constexpr long long kStWait = 2000000000LL;

__device__ int g_stencil_err = 0;

__device__ __forceinline__ uint32_t st_su32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void st_mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void st_mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ uint32_t st_mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok;
}
__device__ __forceinline__ bool st_mbar_wait(uint32_t bar, uint32_t parity, long long limit) {
  const long long t0 = clock64();
  while (!st_mbar_test(bar, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}
// one box {0, row} of a 2D flat tensor map into shared memory
__device__ __forceinline__ void st_tma_2d(uint32_t dst, const CUtensorMap* map, int row,
                                          uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3}], [%4];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(row), "r"(bar)
      : "memory");
}

}  // namespace

namespace {

template <typename TO, int W>
__global__ void __launch_bounds__(kStThreads) k_residual_staged(
    LevelView<float> L, const __grid_constant__ CUtensorMap tu, const __grid_constant__ CUtensorMap tc,
    StencilArgs a, C_t<TO>* __restrict__ rout, double* __restrict__ norm2, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char sm_raw[];
  __shared__ __align__(8) uint64_t bar[kStRing];
  __shared__ volatile int failed;
  const int rhs = blockIdx.y;
  if (L.active && !L.active[rhs]) return;
  const int X = L.n[0] + 1, Y = L.n[1] + 1, Z = L.n[2] + 1;
  const int n0 = L.n[0], n1 = L.n[1], n2 = L.n[2];
  const int XY = X * Y;
  const int S = (int)L.S;
  const int tj = blockIdx.x % a.ntj, tk = blockIdx.x / a.ntj;
  const int j0 = tj * a.TY, k0 = tk * a.KZ;
  const int j1 = min(j0 + a.TY, Y), k1 = min(k0 + a.KZ, Z);
  const int jlo = max(j0 - 1, 0), jclo = max(j0 - 1, 0);
  const int op = op_of(L, rhs);
  const long ncell = L.ncell;
  const int tid = threadIdx.x;

  if (tid == 0) {
    // an earlier CTA gave up: the launch has failed (one read for the CTA,
    // so that every thread leaves or stays)
    failed = *(volatile int*)err ? 1 : 0;
    for (int i = 0; i < kStRing; i++) st_mbar_init(st_su32(&bar[i]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  if (failed) return;

  // element offsets of the windows of plane p (u: component c; cells: array A)
  auto ufirst = [&](int c, int p) -> long {
    return ((long)rhs * 3 + c) * S + (long)p * XY + (long)jlo * X;
  };
  auto cfirst = [&](int A, int p) -> long {
    return ((long)op * 4 + A) * ncell + (long)p * n0 * n1 + (long)jclo * n0;
  };
  // planes pfirst .. plast are staged in order: plane p takes slot
  // (p - pfirst) mod kStRing for the ((p - pfirst) / kStRing)-th time
  const int pfirst = max(k0 - 1, 0), plast = min(k1, Z - 1);
  auto slot_of = [&](int p) { return (p - pfirst) % kStRing; };
  auto use_of = [&](int p) { return (uint32_t)(((p - pfirst) / kStRing) & 1); };
  // tensor copies land on 128-byte boundaries
  unsigned char* slot0 =
      sm_raw + ((128u - (st_su32(sm_raw) & 127u)) & 127u);
  // thread 0: the copies of plane p into its slot; false (nothing issued)
  // from the test hook's stall plane on
  auto issue = [&](int p) -> bool {
    if (a.stall >= 0 && p >= a.stall) return false;
    const int sl = slot_of(p);
    const uint32_t b = st_su32(&bar[sl]);
    unsigned char* base = slot0 + (size_t)sl * a.slot;
    const bool cells = p < n2;
    st_mbar_expect_tx(b, 3 * a.uwin + (cells ? a.ncarr * a.cwin : 0u));
    for (int c = 0; c < 3; c++)
      st_tma_2d(st_su32(base + c * a.uwin), &tu, (int)(ufirst(c, p) >> 5), b);
    if (cells)
      for (int A = 0; A < a.ncarr; A++)
        st_tma_2d(st_su32(base + 3 * a.uwin + A * a.cwin), &tc, (int)(cfirst(A, p) >> 6), b);
    return true;
  };
  // planes k0-1 .. k1 (those inside the grid) are staged; p is computed with
  // p-1..p+1 in the ring
  int issued = pfirst - 1;  // thread 0: the last plane whose copies are in flight or landed
  if (tid == 0)
    for (int p = pfirst; p <= min(pfirst + kStRing - 2, plast) && issue(p); p++) issued = p;
  const float wmu = L.wmu[rhs];
  const Geo<float> G{L.geo + (long)op * L.gstride, L.gmax1};
  const float2* f = L.f ? L.f + (long)rhs * 3 * S : nullptr;
  C_t<TO>* ro = rout ? rout + (long)rhs * 3 * S : nullptr;
  float acc = 0.f;
  int waited = pfirst - 1;
  for (int k = k0; k < k1; k++) {
    // every plane up to k+1 landed; plane k+2 goes into the slot plane k-2 left
    const int need = min(k + 1, plast);
    bool ok = true;
    for (int p = waited + 1; p <= need && ok; p++) {
      ok = st_mbar_wait(st_su32(&bar[slot_of(p)]), use_of(p), a.wait);
      if (ok) waited = p;  // on a failure: waited is the last plane seen landed
    }
    if (!ok) failed = 1;
    __syncthreads();
    if (failed) break;
    if (tid == 0 && k + kStRing - 2 <= plast && k + kStRing - 2 > issued) {
      // the slot's previous contents were read through the generic proxy
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      if (issue(k + kStRing - 2)) issued = k + kStRing - 2;
    }
    // plane pointers: u of component c at plane k+dz, cells of array A at
    // cell plane k+dz, each shifted so that [j*X + i] / [j*n0 + i] address
    // slot (i, j) of the plane
    const float2* up[3][3];
    const float* cp[4][2];
#pragma unroll
    for (int dz = -1; dz <= 1; dz++) {
      const int p = k + dz;
      if (p < 0 || p >= Z) continue;
      const unsigned char* base = slot0 + (size_t)slot_of(p) * a.slot;
#pragma unroll
      for (int c = 0; c < 3; c++)
        up[c][dz + 1] = reinterpret_cast<const float2*>(base + c * a.uwin) + (ufirst(c, p) & 31) -
                        (long)jlo * X;
      if (dz <= 0 && p < n2) {
#pragma unroll
        for (int A = 0; A < 4; A++)
          if (A < a.ncarr)
            cp[A][dz + 1] = reinterpret_cast<const float*>(base + 3 * a.uwin + A * a.cwin) +
                            (cfirst(A, p) & 63) - (long)jclo * n0;
      }
    }
    // slot (i, j, k) with its three edges per item: the columns i < X-1
    // first, row by row, then the last column (boundary edges only)
    const int rows = j1 - j0;
    const int inner = rows * (X - 1);
    for (int it = tid; it < inner + rows; it += kStThreads) {
      int jj, i;
      if (it < inner) {
        jj = it / (X - 1);
        i = it - jj * (X - 1);
      } else {
        jj = it - inner;
        i = X - 1;
      }
      const int j = j0 + jj;
      const int s = i + X * (j + Y * k);
      const int P[3] = {i, j, k};
      // the edge equation of component C (edge_coef / apply_row's order)
      auto row = [&](auto cc) {
        constexpr int C = decltype(cc)::value;
        float2 r = f ? f[C * S + s] : make_float2(0.f, 0.f);
        constexpr int p_ = Cyc<C>::p, q_ = Cyc<C>::q;
        if (P[C] < L.n[C] && P[p_] >= 1 && P[p_] < L.n[p_] && P[q_] >= 1 && P[q_] < L.n[q_]) {
        const int av = P[C], bv = P[p_], gv = P[q_];
        // the four cells around the edge: coordinates along (C, p, q)
        auto cell = [&](int A, int db, int dg) -> float {
          int Q[3];
          Q[C] = av;
          Q[p_] = bv + db;
          Q[q_] = gv + dg;
          return cp[A][Q[2] - k + 1][Q[1] * n0 + Q[0]];
        };
        const float sg = 0.25f * (((cell(C, -1, -1) + cell(C, -1, 0)) + cell(C, 0, -1)) +
                                  cell(C, 0, 0));
        const float dc = ldro(G.ds(C) + av);
        const float dpp = ldro(G.ds(p_) + bv), dpm = ldro(G.ds(p_) + bv - 1);
        const float dqp = ldro(G.ds(q_) + gv), dqm = ldro(G.ds(q_) + gv - 1);
        EdgeCoef<float> e;
        e.dim = -wmu * sg;
        if (W == 1) {
          const float hq = 0.5f * (dqp + dqm), hp = 0.5f * (dpp + dpm);
          const float kpp = qdiv(dc * hq, dpp), kpm = qdiv(dc * hq, dpm);
          const float kqp = qdiv(dc * hp, dqp), kqm = qdiv(dc * hp, dqm);
          e.dre = (kpp + kpm) + (kqp + kqm);
          e.c[0] = -kpp;
          e.c[1] = -kpm;
          e.c[2] = -kqp;
          e.c[3] = -kqm;
          e.c[4] = hq;
          e.c[5] = -hq;
          e.c[6] = -hq;
          e.c[7] = hq;
          e.c[8] = hp;
          e.c[9] = -hp;
          e.c[10] = -hp;
          e.c[11] = hp;
        } else {
          const float i00 = cell(3, -1, -1), i01 = cell(3, -1, 0), i10 = cell(3, 0, -1),
                      i11 = cell(3, 0, 0);
          const float m1 = 0.5f * (i11 + i10), m2 = 0.5f * (i01 + i00);
          const float m3 = 0.5f * (i11 + i01), m4 = 0.5f * (i10 + i00);
          const float kpp = qdiv(m1, dpp * dpp), kpm = qdiv(m2, dpm * dpm);
          const float kqp = qdiv(m3, dqp * dqp), kqm = qdiv(m4, dqm * dqm);
          e.dre = (kpp + kpm) + (kqp + kqm);
          e.c[0] = -kpp;
          e.c[1] = -kpm;
          e.c[2] = -kqp;
          e.c[3] = -kqm;
          const float xp = qdiv(m1, dc * dpp), xm = qdiv(m2, dc * dpm);
          const float yp = qdiv(m3, dc * dqp), ym = qdiv(m4, dc * dqm);
          e.c[4] = xp;
          e.c[5] = -xp;
          e.c[6] = -xm;
          e.c[7] = xm;
          e.c[8] = yp;
          e.c[9] = -yp;
          e.c[10] = -ym;
          e.c[11] = ym;
        }
        auto uat = [&](int comp, int dC, int dp, int dq) -> float2 {
          int Q[3] = {i, j, k};
          Q[C] += dC;
          Q[p_] += dp;
          Q[q_] += dq;
          return up[comp][Q[2] - k + 1][Q[1] * X + Q[0]];
        };
        const float2 uc = uat(C, 0, 0, 0);
        float ar = e.dre * uc.x - e.dim * uc.y;
        float ai = e.dre * uc.y + e.dim * uc.x;
#pragma unroll
        for (int kk = 0; kk < 12; kk++) {
          const NbrOff o = nbr_off(C, kk);
          const float2 v = uat(o.comp, o.dc, o.dp, o.dq);
          ar += e.c[kk] * v.x;
          ai += e.c[kk] * v.y;
        }
        r = make_float2(r.x - ar, r.y - ai);
        }
        if (ro) ro[C * S + s] = mk<TO>((TO)r.x, (TO)r.y);
        acc += r.x * r.x + r.y * r.y;
      };
      row(std::integral_constant<int, 0>());
      row(std::integral_constant<int, 1>());
      row(std::integral_constant<int, 2>());
    }
    __syncthreads();  // plane k-1's slot is free for plane k+3
  }
  if (failed) {
    if (tid == 0) {
      atomicExch(err, 1);
      // copies issued and not yet seen land before the shared memory goes
      // (the full limit: an issued copy does land)
      for (int p = waited + 1; p <= issued; p++)
        st_mbar_wait(st_su32(&bar[slot_of(p)]), use_of(p), kStWait);
    }
    return;
  }
  if (norm2) {
    __shared__ double red[kStThreads / 32];
    float v = acc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    double w = (double)v;
    const int lane = tid & 31, wi = tid >> 5;
    if (lane == 0) red[wi] = w;
    __syncthreads();
    if (wi == 0) {
      w = lane < kStThreads / 32 ? red[lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
      if (lane == 0 && w != 0.0) atomicAdd(norm2 + rhs, w);
    }
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// a flat array of `elems` elements of `esize` bytes as rows of 256 bytes,
// boxes of `box_rows` rows (the allocation holds whole rows)
bool flat_map(CUtensorMap* m, const void* base, long elems, int esize, int box_rows) {
  auto fn = encode_fn();
  if (!fn || box_rows < 1 || box_rows > 256) return false;
  const cuuint64_t per = 256 / esize;
  const cuuint64_t dim[2] = {per, (cuuint64_t)((elems + (long)per - 1) / (long)per)};
  const cuuint64_t stride[1] = {256};
  const cuuint32_t box[2] = {(cuuint32_t)per, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(m, esize == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                        2, const_cast<void*>(base), dim, stride, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace

int* stencil_err() {
  static int* p = nullptr;
  static std::once_flag once;
  std::call_once(once, [] { cudaGetSymbolAddress((void**)&p, g_stencil_err); });
  return p;
}

void stencil_hook(StencilPlan* P, long long wait, int stall) {
  P->args.wait = wait > 0 ? wait : kStWait;
  P->args.stall = stall;
}

long stencil_pad(long elems, int esize) {
  const long per = 256 / esize;
  return (elems + per - 1) / per * per;
}

// tile geometry and tensor maps for the residual of level view V (all of
// its RHS, the arrays V.u and V.cells padded by stencil_pad); false when the
// level is not staged (too wide a row for a tile that keeps every thread
// busy, no encoder)
bool stencil_prepare(const LevelView<float>& V, long u_elems, long cell_elems, StencilPlan* out) {
  const int X = V.n[0] + 1, Y = V.n[1] + 1, Z = V.n[2] + 1;
  const int n0 = V.n[0];
  const int ncarr = V.imu_vol ? 3 : 4;
  const size_t cap = 200 * 1024;
  StencilArgs a{};
  int TY = 0;
  for (int ty : {16, 8, 4, 2, 1}) {
    if (ty > Y) continue;
    const int Ru = (31 + (ty + 2) * X + 31) / 32;
    const int Rc = (63 + (ty + 1) * n0 + 63) / 64;
    if (Ru > 256 || Rc > 256) continue;
    const size_t slot = (size_t)3 * Ru * 256 + (size_t)ncarr * Rc * 256;
    if (slot * kStRing <= cap) {
      TY = ty;
      a.Ru = Ru;
      a.Rc = Rc;
      break;
    }
  }
  // wide rows leave only thin tiles in shared memory: when the tile is cut
  // below 16 rows (or the grid's rows) and no longer gives every thread a
  // slot per plane, the plain kernel does better
  if (!TY || (TY < std::min(16, Y) && (long)TY * (X - 1) < kStThreads)) return false;
  a.TY = TY;
  a.KZ = 32;
  a.ntj = (Y + TY - 1) / TY;
  a.ntk = (Z + a.KZ - 1) / a.KZ;
  a.ncarr = ncarr;
  a.uwin = (unsigned)a.Ru * 256;
  a.cwin = (unsigned)a.Rc * 256;
  a.slot = 3 * a.uwin + ncarr * a.cwin;
  a.wait = kStWait;
  if (!flat_map(&out->tu, V.u, u_elems, 8, a.Ru)) return false;
  if (!flat_map(&out->tc, V.cells, cell_elems, 4, a.Rc)) return false;
  out->args = a;
  out->ok = true;
  return true;
}

template <typename TO, int W>
static void staged_launch(const LevelView<float>& L, const StencilPlan& P, C_t<TO>* rout,
                          double* norm2, cudaStream_t st) {
  static std::once_flag once;
  std::call_once(once, [] {
    cudaFuncSetAttribute(k_residual_staged<TO, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         210 * 1024);
  });
  const size_t smem = (size_t)kStRing * P.args.slot + 128;
  dim3 g((unsigned)(P.args.ntj * P.args.ntk), L.nrhs);
  k_residual_staged<TO, W><<<g, kStThreads, smem, st>>>(L, P.tu, P.tc, P.args, rout, norm2,
                                                        stencil_err());
}

void launch_residual_staged(const LevelView<float>& L, const StencilPlan& P, C_t<float>* rout,
                            double* norm2, cudaStream_t st) {
  if (L.imu_vol)
    staged_launch<float, 1>(L, P, rout, norm2, st);
  else
    staged_launch<float, 0>(L, P, rout, norm2, st);
}

}  // namespace emmi

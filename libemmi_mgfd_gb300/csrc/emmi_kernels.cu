// Multigrid kernels for the finite-integration curl-curl system on sm_103a.
//
// residual      r = f - A u, fused FP64 norm             (src/gmg.c:1316-1410)
// line sweep    zebra (4-colour) line block relaxation,  (src/gmg.c:340-1298)
//               one thread per line, streaming complex-symmetric LDL^T
// point sweep   8-colour node-patch (6x6) block relaxation (src/gmg.c:116-336)
// restrict      f_c = P^T r_f as a gather                (src/gmg.c:1510-1573)
// prolong       u_f += P u_c                              (src/gmg.c:1463-1505)
// coarsen       coarse-cell sums / repeat                 (src/gmg.c:1803-1858)
//
// The smoothers update in correction form: each block solves A_bb d = r_b
// with r_b the current residual of its rows and adds d.  In exact arithmetic
// this equals the reference's zero-then-solve form (src/gmg.c:395-405) and it
// keeps the relative precision of complex64 updates as the solve converges.
// Blocks of one colour neither overlap nor read each other's unknowns: a line
// along d through (ta,tb) reads transverse neighbours at ta+-1 / tb+-1 only
// (checked by tests/test_coloring.py), so a colour is one parallel launch.
#include "emmi_kernels.cuh"

#include <cuda_fp16.h>

#include <cstdio>
#include <mutex>
#include <type_traits>

namespace emmi {

// ------------------------------------------------------------ line tables
// Position of an edge on the line along d through transverse nodes (ta,tb)
// (a<b the other directions), in the reference's row order
// (src/gmg.c:413-603): node s=1..n_d-1 holds E_d(s-1), E_a(ta-1), E_a(ta),
// E_b(tb-1), E_b(tb); the last row is E_d(n_d-1).  -1 when not on the line.
__host__ __device__ constexpr int line_pos(int d, int a, int b, int ta, int tb, int nd, int comp,
                                          int p0, int p1, int p2) {
  const int P[3] = {p0, p1, p2};
  if (comp == d) return (P[a] == ta && P[b] == tb && P[d] >= 0 && P[d] < nd) ? 5 * P[d] : -1;
  if (P[d] < 1 || P[d] >= nd) return -1;
  if (comp == a)
    return (P[b] == tb && (P[a] == ta - 1 || P[a] == ta)) ? 5 * (P[d] - 1) + 1 + (P[a] - ta + 1)
                                                           : -1;
  return (P[a] == ta && (P[b] == tb - 1 || P[b] == tb)) ? 5 * (P[d] - 1) + 3 + (P[b] - tb + 1)
                                                         : -1;
}

// band offset of neighbour k of the row of type t on a line along d (127 if
// the neighbour is not on the line); evaluated on an interior row.
__host__ __device__ constexpr int line_off(int d, int t, int k) {
  const int a = (d == 0) ? 1 : 0, b = (d == 2) ? 1 : 2;
  const int s = 8, ta = 8, tb = 8, nd = 64;
  const int comp = (t == 0) ? d : (t <= 2 ? a : b);
  int P[3] = {0, 0, 0};
  P[d] = (t == 0) ? s - 1 : s;
  P[a] = ta - (t == 1 ? 1 : 0);
  P[b] = tb - (t == 3 ? 1 : 0);
  const int row = 5 * (s - 1) + t;
  const NbrOff o = nbr_off(comp, k);
  const int p = (comp + 1) % 3, q = (comp + 2) % 3;
  int Q[3] = {P[0], P[1], P[2]};
  Q[comp] += o.dc;
  Q[p] += o.dp;
  Q[q] += o.dq;
  const int pos = line_pos(d, a, b, ta, tb, nd, o.comp, Q[0], Q[1], Q[2]);
  return pos < 0 ? 127 : pos - row;
}


long line_count(const int n[3], int d, int color) {
  const int a = (d == 0) ? 1 : 0, b = (d == 2) ? 1 : 2;
  const int pa = color & 1, pb = (color >> 1) & 1;
  const int fa = pa ? 1 : 2, fb = pb ? 1 : 2;
  const long la = (n[a] - 1 >= fa) ? (n[a] - 1 - fa) / 2 + 1 : 0;
  const long lb = (n[b] - 1 >= fb) ? (n[b] - 1 - fb) / 2 + 1 : 0;
  return la * lb;
}

long line_scratch_elems(const int n[3], int d, int nrhs) {
  long mx = 0;
  for (int c = 0; c < 4; c++) mx = line_count(n, d, c) > mx ? line_count(n, d, c) : mx;
  return (long)(5 * n[d] - 4) * 6 * mx * nrhs;
}

// ------------------------------------------------------------ reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
// a thread's partial sum of squares in working precision: complex64
// residuals square and add across the warp in fp32 and widen once per warp
// (conversions to FP64 and FP64 arithmetic are low-rate on this GPU); the
// block and the grid sum in FP64
template <typename T>
__device__ __forceinline__ double warp_partial(T v) {
  if constexpr (sizeof(T) == 4) return (double)warp_sum(v);
  else return warp_sum((double)v);
}

__device__ __forceinline__ void block_add(double v, double* dst) {
  __shared__ double red[32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? red[lane] : 0.0;
    v = warp_sum(v);
    if (lane == 0 && v != 0.0) atomicAdd(dst, v);
  }
}

// block_add for a thread's partial of type T (see warp_partial)
template <typename T>
__device__ __forceinline__ void block_add_t(T v, double* dst) {
  __shared__ double red[32];
  double w = warp_partial<T>(v);
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  if (lane == 0) red[wi] = w;
  __syncthreads();
  if (wi == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    w = lane < nw ? red[lane] : 0.0;
    w = warp_sum(w);
    if (lane == 0 && w != 0.0) atomicAdd(dst, w);
  }
}

// ------------------------------------------------------------ residual
template <int C>
__device__ __forceinline__ bool is_unknown(const int n[3], const int P[3]) {
  constexpr int p = Cyc<C>::p, q = Cyc<C>::q;
  return P[C] < n[C] && P[p] >= 1 && P[p] < n[p] && P[q] >= 1 && P[q] < n[q];
}

template <typename T, typename TO, int C, int W>
__device__ __forceinline__ T residual_comp(const LevelView<T>& L, const C_t<T>* u,
                                                const C_t<T>* f, const T* cells, const Geo<T>& G,
                                                T wmu, const int P[3], long s, const long ss[3],
                                                C_t<TO>* rout) {
  const int o = C * (int)L.S + (int)s;  // 32-bit offset within the RHS's field
  C_t<T> r = f ? f[o] : mk<T>(0, 0);     // f null: r = -A u
  if (is_unknown<C>(L.n, P)) {
    EdgeCoef<T> e;
    const C_t<T> au = apply_row<T, C, W>(L, u, cells, G, wmu, P, s, ss, e);
    r = csub<T>(r, au);
  }
  if (rout) rout[o] = mk<TO>((TO)r.x, (TO)r.y);
  return r.x * r.x + r.y * r.y;
}

// a thread per (component, slot), the component = blockIdx.z: one edge
// equation per thread keeps more independent loads in flight than three
template <typename T, typename TO, int W>
__global__ void __launch_bounds__(256) k_residual(LevelView<T> L, C_t<TO>* __restrict__ rout,
                                                  double* __restrict__ norm2) {
  const int rhs = blockIdx.y;
  if (L.active && !L.active[rhs]) return;
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  T acc = 0;
  if (s < L.S) {
    const int n0 = L.n[0] + 1, n1 = L.n[1] + 1;
    int P[3];
    slot_nodes(s, L, P);
    const long ss[3] = {1, (long)n0, (long)n0 * n1};
    const C_t<T>* u = L.u + (long)rhs * 3 * L.S;
    const C_t<T>* f = L.f ? L.f + (long)rhs * 3 * L.S : nullptr;
    const T* cells = L.cells + (long)op_of(L, rhs) * 4 * L.ncell;
    const Geo<T> G{L.geo + (long)op_of(L, rhs) * L.gstride, L.gmax1};
    const T wmu = L.wmu[rhs];
    C_t<TO>* ro = rout ? rout + (long)rhs * 3 * L.S : nullptr;
    switch (blockIdx.z) {
      case 0: acc = residual_comp<T, TO, 0, W>(L, u, f, cells, G, wmu, P, s, ss, ro); break;
      case 1: acc = residual_comp<T, TO, 1, W>(L, u, f, cells, G, wmu, P, s, ss, ro); break;
      default: acc = residual_comp<T, TO, 2, W>(L, u, f, cells, G, wmu, P, s, ss, ro); break;
    }
  }
  if (norm2) block_add_t<T>(acc, norm2 + rhs);
}

template <typename T, typename TO>
void launch_residual(const LevelView<T>& L, C_t<TO>* rout, double* norm2, cudaStream_t st) {
  dim3 grid((unsigned)((L.S + 255) / 256), L.nrhs, 3);
  if (L.imu_vol)
    k_residual<T, TO, 1><<<grid, 256, 0, st>>>(L, rout, norm2);
  else
    k_residual<T, TO, 0><<<grid, 256, 0, st>>>(L, rout, norm2);
}

// ------------------------------------------------------------ stored FP64 coefficients
// The FP64 refinement residual of the mixed solver recomputes, per edge, 8
// coupling values with 8 divisions at GB300's FP64 rate.  They depend on the
// operator only (the imaginary diagonal on omega too, as -omega*mu0 * sbar),
// so they are stored once per operator: planes [op][10][3][S] of kpp, kpm,
// kqp, kqm (c[0..3]), xp, xm, yp, ym (c[4], c[7], c[8], c[11]), the real
// diagonal and sbar, taken from edge_coef itself.  The residual then applies
// them in edge_coef/apply_row's order: the same result, bit for bit.
constexpr int kCoef = 10;

template <int C>
__device__ __forceinline__ void store_coef(const LevelView<double>& L, const double* cells,
                                           const Geo<double>& G, const int P[3], long s,
                                           double* __restrict__ out) {
  EdgeCoef<double> e;
  // omega*mu0 = -1 gives dim = -(-1)*sbar = sbar exactly
  edge_coef<double, C>(L.n, P, cells + (long)C * L.ncell, cells + 3 * L.ncell, G, -1.0, e);
  const long n3s = 3 * L.S, o = (long)C * L.S + s;
  const double v[kCoef] = {e.c[0], e.c[1], e.c[2], e.c[3], e.c[4], e.c[7], e.c[8], e.c[11],
                           e.dre, e.dim};
#pragma unroll
  for (int k = 0; k < kCoef; k++) out[k * n3s + o] = v[k];
}

// blockIdx.y = operator
__global__ void __launch_bounds__(256) k_coef64(LevelView<double> L, double* __restrict__ coef) {
  const int op = blockIdx.y;
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= L.S) return;
  int P[3];
  slot_nodes(s, L, P);
  const double* cells = L.cells + (long)op * 4 * L.ncell;
  const Geo<double> G{L.geo + (long)op * L.gstride, L.gmax1};
  double* out = coef + (long)op * kCoef * 3 * L.S;
  if (is_unknown<0>(L.n, P)) store_coef<0>(L, cells, G, P, s, out);
  if (is_unknown<1>(L.n, P)) store_coef<1>(L, cells, G, P, s, out);
  if (is_unknown<2>(L.n, P)) store_coef<2>(L, cells, G, P, s, out);
}

template <typename TO, int C>
__device__ __forceinline__ double residual_comp_coef(const LevelView<double>& L,
                                                     const double2* u, const double2* f,
                                                     const double* __restrict__ cf, double wmu,
                                                     const int P[3], long s, const long ss[3],
                                                     C_t<TO>* rout) {
  double2 r = f ? f[(long)C * L.S + s] : make_double2(0.0, 0.0);
  if (is_unknown<C>(L.n, P)) {
    const long n3s = 3 * L.S, o = (long)C * L.S + s;
    double k8[kCoef];
#pragma unroll
    for (int k = 0; k < kCoef; k++) k8[k] = ldro(cf + k * n3s + o);
    const double c[12] = {k8[0], k8[1], k8[2], k8[3], k8[4], -k8[4], -k8[5], k8[5],
                          k8[6], -k8[6], -k8[7], k8[7]};
    const double dre = k8[8], dim = -wmu * k8[9];
    const double2 uc = ldro(u + o);
    double ar = dre * uc.x - dim * uc.y;
    double ai = dre * uc.y + dim * uc.x;
#pragma unroll
    for (int k = 0; k < 12; k++) {
      const double2 v = ldro(u + s + nbr_slot_delta<C>(k, ss, L.S));
      ar += c[k] * v.x;
      ai += c[k] * v.y;
    }
    r = csub<double>(r, mk<double>(ar, ai));
  }
  if (rout) rout[(long)C * L.S + s] = mk<TO>((TO)r.x, (TO)r.y);
  return r.x * r.x + r.y * r.y;
}

template <typename TO>
__global__ void __launch_bounds__(256) k_residual_coef(LevelView<double> L,
                                                       const double* __restrict__ coef,
                                                       C_t<TO>* __restrict__ rout,
                                                       double* __restrict__ norm2) {
  const int rhs = blockIdx.y;
  if (L.active && !L.active[rhs]) return;
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  double acc = 0.0;
  if (s < L.S) {
    const int n0 = L.n[0] + 1, n1 = L.n[1] + 1;
    int P[3];
    slot_nodes(s, L, P);
    const long ss[3] = {1, (long)n0, (long)n0 * n1};
    const double2* u = L.u + (long)rhs * 3 * L.S;
    const double2* f = L.f ? L.f + (long)rhs * 3 * L.S : nullptr;
    const double* cf = coef + (long)op_of(L, rhs) * kCoef * 3 * L.S;
    const double wmu = L.wmu[rhs];
    C_t<TO>* ro = rout ? rout + (long)rhs * 3 * L.S : nullptr;
    acc += residual_comp_coef<TO, 0>(L, u, f, cf, wmu, P, s, ss, ro);
    acc += residual_comp_coef<TO, 1>(L, u, f, cf, wmu, P, s, ss, ro);
    acc += residual_comp_coef<TO, 2>(L, u, f, cf, wmu, P, s, ss, ro);
  }
  if (norm2) block_add(acc, norm2 + rhs);
}

long coef64_elems(const int n[3]) {
  return (long)kCoef * 3 * (n[0] + 1) * (n[1] + 1) * (n[2] + 1);
}

void launch_coef64(const LevelView<double>& L, double* coef, cudaStream_t st) {
  dim3 grid((unsigned)((L.S + 255) / 256), L.nrhs);
  k_coef64<<<grid, 256, 0, st>>>(L, coef);
}

template <typename TO>
void launch_residual_coef(const LevelView<double>& L, const double* coef, C_t<TO>* rout,
                          double* norm2, cudaStream_t st) {
  dim3 grid((unsigned)((L.S + 255) / 256), L.nrhs);
  k_residual_coef<TO><<<grid, 256, 0, st>>>(L, coef, rout, norm2);
}
template void launch_residual_coef<float>(const LevelView<double>&, const double*, C_t<float>*,
                                          double*, cudaStream_t);
template void launch_residual_coef<double>(const LevelView<double>&, const double*,
                                           C_t<double>*, double*, cudaStream_t);

template <typename T>
__global__ void __launch_bounds__(256) k_norm(const C_t<T>* __restrict__ v, long n, const int* active,
                                              double* norm2) {
  const int rhs = blockIdx.y;
  if (active && !active[rhs]) return;
  double acc = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const C_t<T> z = v[(long)rhs * n + i];
    acc += (double)z.x * z.x + (double)z.y * z.y;
  }
  block_add(acc, norm2 + rhs);
}

template <typename T>
void launch_norm(const C_t<T>* v, long n3s, int nrhs, const int* active, double* norm2,
                 cudaStream_t st) {
  long blocks = (n3s + 255) / 256;
  if (blocks > 1216) blocks = 1216;
  dim3 grid((unsigned)blocks, nrhs);
  k_norm<T><<<grid, 256, 0, st>>>(v, n3s, active, norm2);
}

// ------------------------------------------------------------ line sweep
// One colour of line relaxation along D is three launches:
//   assemble  thread per (line, node): for the rows of the node, the lower
//             band entries (offsets -5..-1, real), the complex diagonal and
//             the current residual, into a record buffer [row][line][12];
//             threads run along the contiguous memory direction so every
//             stencil load is coalesced
//   solve     thread per line: streaming complex-symmetric LDL^T over its
//             records (factors written in place), then back substitution;
//             records of one row are contiguous across lines (coalesced)
//   apply     thread per (line, node): u += correction, coalesced like
//             assemble
// Record of one row, T-typed: [0..4] band, [5,6] diagonal, [7,8] residual;
// after the forward pass [0..9] = l_1..l_5 (complex), [10,11] = z; after the
// backward pass [10,11] = the correction x.
// Records are stored as 16-byte planes, [row][plane][line]: plane q of a row
// holds record values [q*L, q*L+L) with L = 16/sizeof(T) (3 planes for float,
// 6 for double), so one warp-wide 16-byte access of consecutive lines reads
// or writes 512 contiguous bytes.
#define WI(i, j) ((i) * ((i) + 1) / 2 + (j))
constexpr int kRec = 12;

__device__ __forceinline__ float4 pack16(const float* v) { return make_float4(v[0], v[1], v[2], v[3]); }
__device__ __forceinline__ double2 pack16(const double* v) { return make_double2(v[0], v[1]); }
__device__ __forceinline__ void unpack16(const float4& w, float* v) {
  v[0] = w.x; v[1] = w.y; v[2] = w.z; v[3] = w.w;
}
__device__ __forceinline__ void unpack16(const double2& w, double* v) { v[0] = w.x; v[1] = w.y; }

template <typename T> struct Vec16 { using V = float4; };
template <> struct Vec16<double> { using V = double2; };
template <typename T> constexpr int kLanes = 16 / (int)sizeof(T);
template <typename T> constexpr int kPlanes = kRec / kLanes<T>;

// p: plane 0 of one (row, line); ps: distance between planes (= lines)
template <typename T>
__device__ __forceinline__ void rec_put(typename Vec16<T>::V* p, long ps, const T (&v)[kRec]) {
#pragma unroll
  for (int q = 0; q < kPlanes<T>; q++) p[q * ps] = pack16(v + q * kLanes<T>);
}
template <typename T>
__device__ __forceinline__ void rec_get(const typename Vec16<T>::V* p, long ps, T (&v)[kRec]) {
#pragma unroll
  for (int q = 0; q < kPlanes<T>; q++) unpack16(p[q * ps], v + q * kLanes<T>);
}
// values [10,11] (z or x) live in the last plane for both types
template <typename T>
__device__ __forceinline__ C_t<T> rec_get_x(const typename Vec16<T>::V* p, long ps) {
  T v[kLanes<T>];
  unpack16(p[(kPlanes<T> - 1) * ps], v);
  return mk<T>(v[kLanes<T> - 2], v[kLanes<T> - 1]);
}

struct LineGeom {
  int la, lb, fa, fb;  // lines per transverse direction and first index
  long nl;             // lines of the colour
  int nd, m;           // nodes along the line, rows
};

template <int D>
__host__ __device__ __forceinline__ LineGeom line_geom(const int n[3], int pa, int pb) {
  constexpr int A = (D == 0) ? 1 : 0, B = (D == 2) ? 1 : 2;
  LineGeom g;
  g.fa = pa ? 1 : 2;
  g.fb = pb ? 1 : 2;
  g.la = (n[A] - 1 >= g.fa) ? (n[A] - 1 - g.fa) / 2 + 1 : 0;
  g.lb = (n[B] - 1 >= g.fb) ? (n[B] - 1 - g.fb) / 2 + 1 : 0;
  g.nl = (long)g.la * g.lb;
  g.nd = n[D];
  g.m = 5 * n[D] - 4;
  return g;
}

// work item -> (line, node s); threads along memory-contiguous direction
template <int D>
__device__ __forceinline__ bool line_item(const LineGeom& g, long id, long& l, int& s) {
  if (id >= g.nl * g.nd) return false;
  if (D == 0) {  // rows of an x-line are contiguous in memory
    const unsigned u = (unsigned)id, nd = (unsigned)g.nd;
    l = u / nd;
    s = 1 + (int)(u - (unsigned)l * nd);
  } else {  // neighbouring lines (consecutive i) are contiguous
    const unsigned u = (unsigned)id, nl = (unsigned)g.nl;
    const unsigned q = u / nl;
    l = u - q * nl;
    s = 1 + (int)q;
  }
  return true;
}

// the divisors of a colour's thread decode (one launch): rows x items
// (x-line residual), the item-per-line divisor of line_item and the lines
// per transverse direction
struct LineDiv {
  unsigned items;
  FastDiv rows, item, la;
};
template <int D>
LineDiv line_div(const int n[3], int pa, int pb) {
  const LineGeom g = line_geom<D>(n, pa, pb);
  LineDiv v;
  v.items = (unsigned)(g.nl * g.nd);
  v.rows = make_fastdiv(v.items > 0 ? v.items : 1);
  v.item = make_fastdiv((unsigned)(D == 0 ? g.nd : (g.nl > 0 ? g.nl : 1)));
  v.la = make_fastdiv((unsigned)(g.la > 0 ? g.la : 1));
  return v;
}
// line_item with the launch's divisor
template <int D>
__device__ __forceinline__ bool line_item_fd(const LineGeom& g, const LineDiv& v, unsigned id,
                                             long& l, int& s) {
  if (id >= v.items) return false;
  const unsigned q = fdiv(id, v.item);
  if (D == 0) {  // rows of an x-line are contiguous in memory
    l = q;
    s = 1 + (int)(id - q * (unsigned)g.nd);
  } else {  // neighbouring lines (consecutive i) are contiguous
    l = id - q * (unsigned)g.nl;
    s = 1 + (int)q;
  }
  return true;
}

// the record of row type TT of node s: band entries, diagonal, residual
template <typename T, int D, int TT, int C>
__device__ __forceinline__ void assemble_row(const LevelView<T>& L, const C_t<T>* u,
                                             const C_t<T>* f, const T* cells, const Geo<T>& G,
                                             T wmu, int ta, int tb, int s, int row,
                                             const long ss[3], typename Vec16<T>::V* rp,
                                             long ps) {
  constexpr int A = (D == 0) ? 1 : 0, B = (D == 2) ? 1 : 2;
  int P[3];
  P[D] = (TT == 0) ? s - 1 : s;
  P[A] = ta - (TT == 1 ? 1 : 0);
  P[B] = tb - (TT == 3 ? 1 : 0);
  const int sl = P[0] + (L.n[0] + 1) * (P[1] + (L.n[1] + 1) * P[2]);  // 32-bit slot
  EdgeCoef<T> e;
  const C_t<T> au = apply_row<T, C>(L, u, cells, G, wmu, P, sl, ss, e);
  const C_t<T> r = csub<T>(f[C * (int)L.S + sl], au);
  T band[5] = {0, 0, 0, 0, 0};
#define LINE_ENTRY(K)                                                         \
  {                                                                           \
    constexpr int off = line_off(D, TT, K);                                   \
    if constexpr (off < 0) {                                                  \
      if (row + off >= 0) band[5 + off] = e.c[K];                             \
    }                                                                         \
  }
  LINE_ENTRY(0) LINE_ENTRY(1) LINE_ENTRY(2) LINE_ENTRY(3) LINE_ENTRY(4) LINE_ENTRY(5)
  LINE_ENTRY(6) LINE_ENTRY(7) LINE_ENTRY(8) LINE_ENTRY(9) LINE_ENTRY(10) LINE_ENTRY(11)
#undef LINE_ENTRY
  T rec[kRec];
#pragma unroll
  for (int i = 0; i < 5; i++) rec[i] = band[i];
  rec[5] = e.dre;
  rec[6] = e.dim;
  rec[7] = r.x;
  rec[8] = r.y;
  rec[9] = rec[10] = rec[11] = 0;
  rec_put<T>(rp, ps, rec);
}

template <int D, int TT>
__device__ __forceinline__ long line_slot(const int n[3], long S, int ta, int tb, int s) {
  constexpr int A = (D == 0) ? 1 : 0, B = (D == 2) ? 1 : 2;
  constexpr int C = (TT == 0) ? D : (TT <= 2 ? A : B);
  int P[3];
  P[D] = (TT == 0) ? s - 1 : s;
  P[A] = ta - (TT == 1 ? 1 : 0);
  P[B] = tb - (TT == 3 ? 1 : 0);
  return (long)C * S + slot_id(n, P[0], P[1], P[2]);
}

// one thread per (line, node) and its five rows: y and z lines, whose
// neighbouring lines are neighbouring slots
template <typename T, int D>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) k_line_assemble(LevelView<T> L,
                                                                              int pa, int pb,
                                                                              T* __restrict__ buf) {
  constexpr int A = (D == 0) ? 1 : 0, B = (D == 2) ? 1 : 2;
  const int rhs = blockIdx.y;
  if (L.active && !L.active[rhs]) return;
  const LineGeom g = line_geom<D>(L.n, pa, pb);
  long l;
  int s;
  if (!line_item<D>(g, blockIdx.x * (long)blockDim.x + threadIdx.x, l, s)) return;
  const unsigned lq = (unsigned)l / (unsigned)g.la;
  const int ta = g.fa + 2 * (int)((unsigned)l - lq * (unsigned)g.la), tb = g.fb + 2 * (int)lq;
  const int n0 = L.n[0] + 1, n1 = L.n[1] + 1;
  const long ss[3] = {1, (long)n0, (long)n0 * n1};
  const C_t<T>* u = L.u + (long)rhs * 3 * L.S;
  const C_t<T>* f = L.f + (long)rhs * 3 * L.S;
  const T* cells = L.cells + (long)op_of(L, rhs) * 4 * L.ncell;
  const Geo<T> G{L.geo + (long)op_of(L, rhs) * L.gstride, L.gmax1};
  const T wmu = L.wmu[rhs];
  using V = typename Vec16<T>::V;
  V* base = reinterpret_cast<V*>(buf) + (long)rhs * g.m * kPlanes<T> * g.nl;
  const long ps = g.nl;
  const int r0 = 5 * (s - 1);
  auto rec = [&](int row) { return base + (long)row * kPlanes<T> * g.nl + l; };
  assemble_row<T, D, 0, D>(L, u, f, cells, G, wmu, ta, tb, s, r0, ss, rec(r0), ps);
  if (s < g.nd) {
    assemble_row<T, D, 1, A>(L, u, f, cells, G, wmu, ta, tb, s, r0 + 1, ss, rec(r0 + 1), ps);
    assemble_row<T, D, 2, A>(L, u, f, cells, G, wmu, ta, tb, s, r0 + 2, ss, rec(r0 + 2), ps);
    assemble_row<T, D, 3, B>(L, u, f, cells, G, wmu, ta, tb, s, r0 + 3, ss, rec(r0 + 3), ps);
    assemble_row<T, D, 4, B>(L, u, f, cells, G, wmu, ta, tb, s, r0 + 4, ss, rec(r0 + 4), ps);
  }
}

// one thread per (row type, line, node), row type slowest: x lines, where a
// thread owning all five rows of a node holds too many registers for the
// latency of its scattered record stores (a warp shares one row type)
template <typename T, int D>
__global__ void __launch_bounds__(256) k_line_assemble_rows(LevelView<T> L, int pa, int pb,
                                                            T* __restrict__ buf) {
  constexpr int A = (D == 0) ? 1 : 0, B = (D == 2) ? 1 : 2;
  const int rhs = blockIdx.y;
  if (L.active && !L.active[rhs]) return;
  const LineGeom g = line_geom<D>(L.n, pa, pb);
  const long items = g.nl * g.nd;
  const long id = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int rt = (int)((unsigned)id / (unsigned)items);
  if (rt >= 5) return;
  long l;
  int s;
  if (!line_item<D>(g, id - rt * items, l, s)) return;
  if (rt > 0 && s == g.nd) return;  // the last node carries only its E_D row
  const unsigned lq = (unsigned)l / (unsigned)g.la;
  const int ta = g.fa + 2 * (int)((unsigned)l - lq * (unsigned)g.la), tb = g.fb + 2 * (int)lq;
  const int n0 = L.n[0] + 1, n1 = L.n[1] + 1;
  const long ss[3] = {1, (long)n0, (long)n0 * n1};
  const C_t<T>* u = L.u + (long)rhs * 3 * L.S;
  const C_t<T>* f = L.f + (long)rhs * 3 * L.S;
  const T* cells = L.cells + (long)op_of(L, rhs) * 4 * L.ncell;
  const Geo<T> G{L.geo + (long)op_of(L, rhs) * L.gstride, L.gmax1};
  const T wmu = L.wmu[rhs];
  using V = typename Vec16<T>::V;
  V* base = reinterpret_cast<V*>(buf) + (long)rhs * g.m * kPlanes<T> * g.nl;
  const long ps = g.nl;
  const int row = 5 * (s - 1) + rt;
  V* rp = base + (long)row * kPlanes<T> * g.nl + l;
  switch (rt) {
    case 0: assemble_row<T, D, 0, D>(L, u, f, cells, G, wmu, ta, tb, s, row, ss, rp, ps); break;
    case 1: assemble_row<T, D, 1, A>(L, u, f, cells, G, wmu, ta, tb, s, row, ss, rp, ps); break;
    case 2: assemble_row<T, D, 2, A>(L, u, f, cells, G, wmu, ta, tb, s, row, ss, rp, ps); break;
    case 3: assemble_row<T, D, 3, B>(L, u, f, cells, G, wmu, ta, tb, s, row, ss, rp, ps); break;
    default: assemble_row<T, D, 4, B>(L, u, f, cells, G, wmu, ta, tb, s, row, ss, rp, ps); break;
  }
}

// Each thread streams its line's records through a private ring of kRing
// rows in shared memory ([slot][plane][thread], conflict-free 16-byte
// accesses), filled by cp.async kRing-1 rows ahead of the elimination: the
// row-to-row dependency of the factorization no longer waits on a memory
// round trip.
constexpr int kRing = 6;
constexpr int kSolveThreads = 64;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <typename T>
__global__ void __launch_bounds__(kSolveThreads) k_line_solve(const int* __restrict__ active,
                                                              long nl, int m,
                                                              T* __restrict__ buf) {
  using V = typename Vec16<T>::V;
  constexpr int NP = kPlanes<T>;
  __shared__ V ring[kRing][NP][kSolveThreads];
  const int rhs = blockIdx.y;
  if (active && !active[rhs]) return;
  const int tid = threadIdx.x;
  const long l = blockIdx.x * (long)blockDim.x + tid;
  if (l >= nl) return;
  V* base = reinterpret_cast<V*>(buf) + (long)rhs * m * NP * nl + l;
  const long rs = NP * nl;  // distance between rows
  auto issue = [&](int row) {
    const V* src = base + (long)row * rs;
    const int slot = row % kRing;
#pragma unroll
    for (int q = 0; q < NP; q++) cp_async16(&ring[slot][q][tid], src + q * nl);
  };
  auto take = [&](int row, T (&v)[kRec]) {
    const int slot = row % kRing;
#pragma unroll
    for (int q = 0; q < NP; q++) unpack16(ring[slot][q][tid], v + q * kLanes<T>);
  };
  C_t<T> W[21], y[6];
#pragma unroll
  for (int i = 0; i < 21; i++) W[i] = mk<T>(0, 0);
#pragma unroll
  for (int i = 0; i < 5; i++) {
    W[WI(i, i)] = mk<T>(1, 0);  // dummy leading rows
    y[i] = mk<T>(0, 0);
  }
  for (int p = 0; p < kRing - 1; p++) {
    if (p < m) issue(p);
    cp_async_commit();
  }
  // forward: arriving row r eliminates pivot r-5
  for (int row = 0; row < m + 5; row++) {
    if (row < m) {
      if (row + kRing - 1 < m) issue(row + kRing - 1);
      cp_async_commit();
      cp_async_wait<kRing - 1>();
      T nxt[kRec];
      take(row, nxt);
#pragma unroll
      for (int j = 0; j < 5; j++) W[WI(5, j)] = mk<T>(nxt[j], 0);
      W[WI(5, 5)] = mk<T>(nxt[5], nxt[6]);
      y[5] = mk<T>(nxt[7], nxt[8]);
    } else {
#pragma unroll
      for (int j = 0; j < 5; j++) W[WI(5, j)] = mk<T>(0, 0);
      W[WI(5, 5)] = mk<T>(1, 0);
      y[5] = mk<T>(0, 0);
    }
    const C_t<T> id = crcp<T>(W[0]);
    C_t<T> lq[6];
#pragma unroll
    for (int i = 1; i < 6; i++) lq[i] = cmul<T>(W[WI(i, 0)], id);
#pragma unroll
    for (int i = 1; i < 6; i++) {
#pragma unroll
      for (int j = 1; j <= i; j++) W[WI(i, j)] = cfms<T>(W[WI(i, j)], lq[i], W[WI(j, 0)]);
      y[i] = cfms<T>(y[i], lq[i], y[0]);
    }
    const int piv = row - 5;
    if (piv >= 0) {
      const C_t<T> z = cmul<T>(y[0], id);
      T o[kRec];
#pragma unroll
      for (int i = 1; i < 6; i++) {
        o[2 * (i - 1)] = lq[i].x;
        o[2 * (i - 1) + 1] = lq[i].y;
      }
      o[10] = z.x;
      o[11] = z.y;
      rec_put<T>(base + (long)piv * rs, nl, o);
    }
#pragma unroll
    for (int i = 0; i < 5; i++) {
#pragma unroll
      for (int j = 0; j <= i; j++) W[WI(i, j)] = W[WI(i + 1, j + 1)];
      y[i] = y[i + 1];
    }
  }
  cp_async_wait<0>();
  __threadfence_block();  // the factors just stored are read back below
  // backward: x_k = z_k - sum_i l_{k+i,k} x_{k+i}
  C_t<T> xw[5];
#pragma unroll
  for (int i = 0; i < 5; i++) xw[i] = mk<T>(0, 0);
  for (int p = 0; p < kRing - 1; p++) {
    if (m - 1 - p >= 0) issue(m - 1 - p);
    cp_async_commit();
  }
  for (int row = m - 1; row >= 0; row--) {
    if (row - (kRing - 1) >= 0) issue(row - (kRing - 1));
    cp_async_commit();
    cp_async_wait<kRing - 1>();
    T v[kRec];
    take(row, v);
    C_t<T> x = mk<T>(v[10], v[11]);
#pragma unroll
    for (int i = 0; i < 5; i++) x = cfms<T>(x, mk<T>(v[2 * i], v[2 * i + 1]), xw[i]);
#pragma unroll
    for (int i = 4; i > 0; i--) xw[i] = xw[i - 1];
    xw[0] = x;
    T last[kLanes<T>];
#pragma unroll
    for (int i = 0; i < kLanes<T>; i++) last[i] = v[kRec - kLanes<T> + i];
    last[kLanes<T> - 2] = x.x;
    last[kLanes<T> - 1] = x.y;
    base[(long)row * rs + (NP - 1) * nl] = pack16(last);
  }
  cp_async_wait<0>();
}

template <typename T, int D>
__global__ void __launch_bounds__(256) k_line_apply(LevelView<T> L, int pa, int pb,
                                                    const T* __restrict__ buf) {
  const int rhs = blockIdx.y;
  if (L.active && !L.active[rhs]) return;
  const LineGeom g = line_geom<D>(L.n, pa, pb);
  long l;
  int s;
  if (!line_item<D>(g, blockIdx.x * (long)blockDim.x + threadIdx.x, l, s)) return;
  const unsigned lq = (unsigned)l / (unsigned)g.la;
  const int ta = g.fa + 2 * (int)((unsigned)l - lq * (unsigned)g.la), tb = g.fb + 2 * (int)lq;
  using V = typename Vec16<T>::V;
  C_t<T>* u = L.u + (long)rhs * 3 * L.S;
  const V* base = reinterpret_cast<const V*>(buf) + (long)rhs * g.m * kPlanes<T> * g.nl + l;
  const int r0 = 5 * (s - 1);
  auto add = [&](long sl, int row) {
    u[sl] = cadd<T>(u[sl], rec_get_x<T>(base + (long)row * kPlanes<T> * g.nl, g.nl));
  };
  add(line_slot<D, 0>(L.n, L.S, ta, tb, s), r0);
  if (s < g.nd) {
    add(line_slot<D, 1>(L.n, L.S, ta, tb, s), r0 + 1);
    add(line_slot<D, 2>(L.n, L.S, ta, tb, s), r0 + 2);
    add(line_slot<D, 3>(L.n, L.S, ta, tb, s), r0 + 3);
    add(line_slot<D, 4>(L.n, L.S, ta, tb, s), r0 + 4);
  }
}

// ---------------------------------------------------------------- stored line factors
// A line's band matrix depends on the operator only, never on the iterate.
// The complex64 solver can therefore keep the LDL^T factors of every line
// (one record per row: L(p+i, p) for i = 1..5 and 1/d_p, the 12 values
// k_line_solve writes in place, as planes [row][plane][line]) and sweep with
// a residual per row and a substitution: the same arithmetic in the same
// order as k_line_solve, so the same result, with 8 instead of 48 bytes per
// row written by the assembly and no complex reciprocal per row.

template <typename T, int D, int TT, int C, int W>
__device__ __forceinline__ C_t<T> row_residual(const LevelView<T>& L, const C_t<T>* u,
                                               const C_t<T>* f, const T* cells,
                                               const Geo<T>& G, T wmu, int ta, int tb, int s,
                                               const long ss[3]) {
  constexpr int A = (D == 0) ? 1 : 0, B = (D == 2) ? 1 : 2;
  int P[3];
  P[D] = (TT == 0) ? s - 1 : s;
  P[A] = ta - (TT == 1 ? 1 : 0);
  P[B] = tb - (TT == 3 ? 1 : 0);
  const int sl = P[0] + (L.n[0] + 1) * (P[1] + (L.n[1] + 1) * P[2]);  // 32-bit slot
  EdgeCoef<T> e;
  const C_t<T> au = apply_row<T, C, W>(L, u, cells, G, wmu, P, sl, ss, e);
  return csub<T>(f[C * (int)L.S + sl], au);
}

// rb[rhs][row][line] = residual of every row of one colour; y and z lines:
// a thread per (line, node) and its five rows; x lines: a thread per
// (row type, line, node), row type slowest
template <typename T, int D, int W>
__global__ void __launch_bounds__(256) k_line_rhs(LevelView<T> L, int pa, int pb, LineDiv dv,
                                                  C_t<T>* __restrict__ rb) {
  constexpr int A = (D == 0) ? 1 : 0, B = (D == 2) ? 1 : 2;
  const int rhs = blockIdx.y;
  if (L.active && !L.active[rhs]) return;
  const LineGeom g = line_geom<D>(L.n, pa, pb);
  unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
  int rt = 0;
  if (D == 0) {
    rt = (int)fdiv(id, dv.rows);
    if (rt >= 5) return;
    id -= (unsigned)rt * dv.items;
  }
  long l;
  int s;
  if (!line_item_fd<D>(g, dv, id, l, s)) return;
  if (D == 0 && rt > 0 && s == g.nd) return;
  const unsigned lq = fdiv((unsigned)l, dv.la);
  const int ta = g.fa + 2 * (int)((unsigned)l - lq * (unsigned)g.la), tb = g.fb + 2 * (int)lq;
  const int n0 = L.n[0] + 1, n1 = L.n[1] + 1;
  const long ss[3] = {1, (long)n0, (long)n0 * n1};
  const C_t<T>* u = L.u + (long)rhs * 3 * L.S;
  const C_t<T>* f = L.f + (long)rhs * 3 * L.S;
  const T* cells = L.cells + (long)op_of(L, rhs) * 4 * L.ncell;
  const Geo<T> G{L.geo + (long)op_of(L, rhs) * L.gstride, L.gmax1};
  const T wmu = L.wmu[rhs];
  C_t<T>* out = rb + (long)rhs * g.m * g.nl + l;
  const int r0 = 5 * (s - 1);
  auto put = [&](int row, C_t<T> v) { out[(long)row * g.nl] = v; };
  if (D == 0) {
    switch (rt) {
      case 0: put(r0, row_residual<T, D, 0, D, W>(L, u, f, cells, G, wmu, ta, tb, s, ss)); break;
      case 1: put(r0 + 1, row_residual<T, D, 1, A, W>(L, u, f, cells, G, wmu, ta, tb, s, ss)); break;
      case 2: put(r0 + 2, row_residual<T, D, 2, A, W>(L, u, f, cells, G, wmu, ta, tb, s, ss)); break;
      case 3: put(r0 + 3, row_residual<T, D, 3, B, W>(L, u, f, cells, G, wmu, ta, tb, s, ss)); break;
      default: put(r0 + 4, row_residual<T, D, 4, B, W>(L, u, f, cells, G, wmu, ta, tb, s, ss)); break;
    }
  } else {
    put(r0, row_residual<T, D, 0, D, W>(L, u, f, cells, G, wmu, ta, tb, s, ss));
    if (s < g.nd) {
      put(r0 + 1, row_residual<T, D, 1, A, W>(L, u, f, cells, G, wmu, ta, tb, s, ss));
      put(r0 + 2, row_residual<T, D, 2, A, W>(L, u, f, cells, G, wmu, ta, tb, s, ss));
      put(r0 + 3, row_residual<T, D, 3, B, W>(L, u, f, cells, G, wmu, ta, tb, s, ss));
      put(r0 + 4, row_residual<T, D, 4, B, W>(L, u, f, cells, G, wmu, ta, tb, s, ss));
    }
  }
}

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
template <typename T>
__device__ __forceinline__ void cp_async_c(C_t<T>* smem, const C_t<T>* gmem) {
  if constexpr (sizeof(C_t<T>) == 8) cp_async8(smem, gmem);
  else cp_async16(smem, gmem);
}

// Stored-factor formats: kFacF32 keeps the 12 fp32 values per row of
// k_line_solve; kFacF16 keeps the five L values per row as fp16 complex
// (20 bytes) and 1/d as fp32 complex (8 bytes), 28 instead of 48 bytes per
// row for the substitution to stream.  A group's kFacF16 block of m rows x
// nl lines: LA [m][nl] uint4 (L1..L4), LB [m][nl] half2 (L5), ID [m][nl]
// float2, each part starting on 16 bytes.
__host__ __device__ inline long round4(long v) { return (v + 3) / 4 * 4; }
__host__ __device__ inline long half_fac_elems(int m, long nl) {
  return round4(4 * m * nl) + round4(m * nl) + round4(2 * m * nl);
}
struct HalfFac {
  uint4* la;
  __half2* lb;
  float2* id;
};
__host__ __device__ inline HalfFac half_fac(const float* g, int m, long nl) {
  float* b = const_cast<float*>(g);
  HalfFac h;
  h.la = reinterpret_cast<uint4*>(b);
  h.lb = reinterpret_cast<__half2*>(b + round4(4 * m * nl));
  h.id = reinterpret_cast<float2*>(b + round4(4 * m * nl) + round4(m * nl));
  return h;
}
__device__ __forceinline__ uint32_t h2u(__half2 h) { return *reinterpret_cast<uint32_t*>(&h); }
__device__ __forceinline__ float2 u2f2(uint32_t u) {
  return __half22float2(*reinterpret_cast<__half2*>(&u));
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}

// band entries (lower, real) and diagonal of row type TT of node s: the
// band part of assemble_row's record
template <typename T, int D, int TT, int C>
__device__ __forceinline__ void band_row(const LevelView<T>& L, const T* cells, const Geo<T>& G,
                                         T wmu, int ta, int tb, int s, int row, T (&band)[5],
                                         C_t<T>& diag) {
  constexpr int A = (D == 0) ? 1 : 0, B = (D == 2) ? 1 : 2;
  int P[3];
  P[D] = (TT == 0) ? s - 1 : s;
  P[A] = ta - (TT == 1 ? 1 : 0);
  P[B] = tb - (TT == 3 ? 1 : 0);
  EdgeCoef<T> e;
  edge_coef<T, C>(L.n, P, cells + (long)C * L.ncell, cells + 3 * L.ncell, G, wmu, e, L.imu_vol);
#pragma unroll
  for (int j = 0; j < 5; j++) band[j] = 0;
#define LINE_ENTRY(K)                                                         \
  {                                                                           \
    constexpr int off = line_off(D, TT, K);                                   \
    if constexpr (off < 0) {                                                  \
      if (row + off >= 0) band[5 + off] = e.c[K];                             \
    }                                                                         \
  }
  LINE_ENTRY(0) LINE_ENTRY(1) LINE_ENTRY(2) LINE_ENTRY(3) LINE_ENTRY(4) LINE_ENTRY(5)
  LINE_ENTRY(6) LINE_ENTRY(7) LINE_ENTRY(8) LINE_ENTRY(9) LINE_ENTRY(10) LINE_ENTRY(11)
#undef LINE_ENTRY
  diag = mk<T>(e.dre, e.dim);
}

// Factors of every line of one colour, for group blockIdx.y of the chunk,
// straight from the operator: a thread assembles a node's band rows in
// registers (band_row) and runs the forward elimination of k_line_solve on
// them -- no band records through memory -- writing factors to
// fac + grp * gstride:
//   FMT 0 (kFacF32): the record layout, 12 values per row, L(p+i, p) for
//   i = 1..5 and 1/d_p;
//   FMT 1 (kFacF16, T = float): L(p+i, p) rounded to fp16 in planes LA
//   (i = 1..4) and LB (i = 5), 1/d_p in fp32 (ID); an L value outside the
//   fp16 range (or not finite) sets *ovf.
// y and z lines: neighbouring lines are neighbouring slots, so a warp's cell
// loads coalesce; x lines read theirs along each thread's line (uncoalesced,
// still faster than assembling records: 15.4 against 23.2 ms for the 128^3
// batch's set-up).
template <typename T, int D, int FMT>
__global__ void __launch_bounds__(kSolveThreads) k_line_factor_direct(LevelView<T> L, int pa,
                                                                      int pb, long gstride,
                                                                      T* __restrict__ fac,
                                                                      int* __restrict__ ovf) {
  constexpr int A = (D == 0) ? 1 : 0, B = (D == 2) ? 1 : 2;
  using V = typename Vec16<T>::V;
  constexpr int NP = kPlanes<T>;
  const int grp = blockIdx.y;
  const LineGeom g = line_geom<D>(L.n, pa, pb);
  const long l = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (l >= g.nl) return;
  const unsigned lq = (unsigned)l / (unsigned)g.la;
  const int ta = g.fa + 2 * (int)((unsigned)l - lq * (unsigned)g.la), tb = g.fb + 2 * (int)lq;
  const T* cells = L.cells + (long)op_of(L, grp) * 4 * L.ncell;
  const Geo<T> G{L.geo + (long)op_of(L, grp) * L.gstride, L.gmax1};
  const T wmu = L.wmu[grp];
  const int m = g.m, nd = g.nd;
  const long nl = g.nl;
  V* fout = reinterpret_cast<V*>(fac + (long)grp * gstride) + l;
  const long rs = NP * nl;
  HalfFac hf{};
  if constexpr (FMT == kFacF16) hf = half_fac(fac + (long)grp * gstride, m, nl);
  bool over = false;
  C_t<T> W[21];
#pragma unroll
  for (int i = 0; i < 21; i++) W[i] = mk<T>(0, 0);
#pragma unroll
  for (int i = 0; i < 5; i++) W[WI(i, i)] = mk<T>(1, 0);
  // the arriving row sits in W[WI(5, .)]: eliminate pivot row - 5 and
  // store its factors
  auto step = [&](int row) {
    const C_t<T> id = crcp<T>(W[0]);
    C_t<T> lqv[6];
#pragma unroll
    for (int i = 1; i < 6; i++) lqv[i] = cmul<T>(W[WI(i, 0)], id);
#pragma unroll
    for (int i = 1; i < 6; i++) {
#pragma unroll
      for (int j = 1; j <= i; j++) W[WI(i, j)] = cfms<T>(W[WI(i, j)], lqv[i], W[WI(j, 0)]);
    }
    const int piv = row - 5;
    if (piv >= 0) {
      if constexpr (FMT == kFacF32) {
        T o[kRec];
#pragma unroll
        for (int i = 1; i < 6; i++) {
          o[2 * (i - 1)] = lqv[i].x;
          o[2 * (i - 1) + 1] = lqv[i].y;
        }
        o[10] = id.x;
        o[11] = id.y;
        rec_put<T>(fout + (long)piv * rs, nl, o);
      } else {
        __half2 h[5];
#pragma unroll
        for (int i = 1; i < 6; i++) {
          over |= !(fabsf(lqv[i].x) <= 65504.f && fabsf(lqv[i].y) <= 65504.f);
          h[i - 1] = __floats2half2_rn(lqv[i].x, lqv[i].y);
        }
        const long o = (long)piv * nl + l;
        hf.la[o] = make_uint4(h2u(h[0]), h2u(h[1]), h2u(h[2]), h2u(h[3]));
        hf.lb[o] = h[4];
        hf.id[o] = make_float2(id.x, id.y);
      }
    }
#pragma unroll
    for (int i = 0; i < 5; i++) {
#pragma unroll
      for (int j = 0; j <= i; j++) W[WI(i, j)] = W[WI(i + 1, j + 1)];
    }
  };
  T bd[5][5];
  C_t<T> dg[5];
  auto assemble = [&](auto tt, int s) {
    constexpr int TT = decltype(tt)::value;
    constexpr int C = (TT == 0) ? D : (TT <= 2 ? A : B);
    band_row<T, D, TT, C>(L, cells, G, wmu, ta, tb, s, 5 * (s - 1) + TT, bd[TT], dg[TT]);
  };
  auto arrive = [&](auto tt, int s) {
    constexpr int TT = decltype(tt)::value;
#pragma unroll
    for (int j = 0; j < 5; j++) W[WI(5, j)] = mk<T>(bd[TT][j], 0);
    W[WI(5, 5)] = dg[TT];
    step(5 * (s - 1) + TT);
  };
  // rows in record order: node s brings row 5(s-1) and, below the last
  // node, its four transverse rows; a node's loads are issued together
  for (int s = 1; s <= nd; s++) {
    assemble(std::integral_constant<int, 0>(), s);
    if (s < nd) {
      assemble(std::integral_constant<int, 1>(), s);
      assemble(std::integral_constant<int, 2>(), s);
      assemble(std::integral_constant<int, 3>(), s);
      assemble(std::integral_constant<int, 4>(), s);
    }
    arrive(std::integral_constant<int, 0>(), s);
    if (s < nd) {
      arrive(std::integral_constant<int, 1>(), s);
      arrive(std::integral_constant<int, 2>(), s);
      arrive(std::integral_constant<int, 3>(), s);
      arrive(std::integral_constant<int, 4>(), s);
    }
  }
  // five unit rows flush the last pivots (rows m..m+4)
  for (int row = m; row < m + 5; row++) {
#pragma unroll
    for (int j = 0; j < 5; j++) W[WI(5, j)] = mk<T>(0, 0);
    W[WI(5, 5)] = mk<T>(1, 0);
    step(row);
  }
  if (over) atomicOr(ovf, 1);
}

// Substitution with stored factors (group grp[rhs]): rb holds the rows'
// residuals in, z between the passes, the correction x out.
template <typename T>
__global__ void __launch_bounds__(kSolveThreads) k_line_subst(const int* __restrict__ active,
                                                              const int* __restrict__ grp,
                                                              long nl, int m,
                                                              const T* __restrict__ fac,
                                                              C_t<T>* __restrict__ rb) {
  using V = typename Vec16<T>::V;
  constexpr int NP = kPlanes<T>;
  __shared__ V ring[kRing][NP][kSolveThreads];
  __shared__ C_t<T> rring[kRing][kSolveThreads];
  const int rhs = blockIdx.y;
  if (active && !active[rhs]) return;
  const int tid = threadIdx.x;
  const long l = blockIdx.x * (long)blockDim.x + tid;
  if (l >= nl) return;
  const long rs = NP * nl;
  const V* fb = reinterpret_cast<const V*>(fac) + (long)grp[rhs] * m * rs + l;
  C_t<T>* rr = rb + (long)rhs * m * nl + l;
  auto issue_f = [&](int row) {
    const V* src = fb + (long)row * rs;
    const int slot = row % kRing;
#pragma unroll
    for (int q = 0; q < NP; q++) cp_async16(&ring[slot][q][tid], src + q * nl);
  };
  auto take_f = [&](int row, T (&v)[kRec]) {
    const int slot = row % kRing;
#pragma unroll
    for (int q = 0; q < NP; q++) unpack16(ring[slot][q][tid], v + q * kLanes<T>);
  };
  // forward: at step `row` the residual of row `row` arrives and pivot
  // row-5 is eliminated with its stored factors (k_line_solve's order)
  C_t<T> y[6];
#pragma unroll
  for (int i = 0; i < 6; i++) y[i] = mk<T>(0, 0);
  for (int p = 0; p < kRing - 1; p++) {
    if (p < m) cp_async_c<T>(&rring[p % kRing][tid], rr + (long)p * nl);
    if (p - 5 >= 0 && p - 5 < m) issue_f(p - 5);
    cp_async_commit();
  }
  for (int row = 0; row < m + 5; row++) {
    {
      const int q = row + kRing - 1;
      if (q < m) cp_async_c<T>(&rring[q % kRing][tid], rr + (long)q * nl);
      if (q - 5 >= 0 && q - 5 < m) issue_f(q - 5);
      cp_async_commit();
    }
    cp_async_wait<kRing - 1>();
    y[5] = row < m ? rring[row % kRing][tid] : mk<T>(0, 0);
    const int piv = row - 5;
    if (piv >= 0) {
      T v[kRec];
      take_f(piv, v);
#pragma unroll
      for (int i = 1; i < 6; i++) y[i] = cfms<T>(y[i], mk<T>(v[2 * (i - 1)], v[2 * (i - 1) + 1]), y[0]);
      rr[(long)piv * nl] = cmul<T>(y[0], mk<T>(v[10], v[11]));  // z
    }
#pragma unroll
    for (int i = 0; i < 5; i++) y[i] = y[i + 1];
  }
  cp_async_wait<0>();
  __threadfence_block();  // z just stored is read back below
  // backward: x_k = z_k - sum_i L(k+i, k) x_{k+i}
  C_t<T> xw[5];
#pragma unroll
  for (int i = 0; i < 5; i++) xw[i] = mk<T>(0, 0);
  for (int p = 0; p < kRing - 1; p++) {
    const int q = m - 1 - p;
    if (q >= 0) {
      issue_f(q);
      cp_async_c<T>(&rring[q % kRing][tid], rr + (long)q * nl);
    }
    cp_async_commit();
  }
  for (int row = m - 1; row >= 0; row--) {
    {
      const int q = row - (kRing - 1);
      if (q >= 0) {
        issue_f(q);
        cp_async_c<T>(&rring[q % kRing][tid], rr + (long)q * nl);
      }
      cp_async_commit();
    }
    cp_async_wait<kRing - 1>();
    T v[kRec];
    take_f(row, v);
    C_t<T> x = rring[row % kRing][tid];
#pragma unroll
    for (int i = 0; i < 5; i++) x = cfms<T>(x, mk<T>(v[2 * i], v[2 * i + 1]), xw[i]);
#pragma unroll
    for (int i = 4; i > 0; i--) xw[i] = xw[i - 1];
    xw[0] = x;
    rr[(long)row * nl] = x;
  }
  cp_async_wait<0>();
}

// The same substitution with kFacF16 factors of group grp[rhs] (gstride
// values per group): the forward pass streams LA, LB and ID, the backward
// pass LA and LB; the fp16 values are widened to fp32 and the arithmetic is
// k_line_subst's.  NT lines per block, a cp.async ring of RING rows per
// line: every thread's arithmetic is the same for every (NT, RING).
//
// D = 1 or 2 (y or z lines, whose neighbouring lines are neighbouring slots):
// the backward pass also adds x to u at each row's slot (k_line_apply_rb's
// work; the old u values ride the cp.async ring with the factors), so the
// colour takes two launches and x never goes through the record buffer.
// D = -1: x goes to rb for k_line_apply_rb.
template <int D>
__device__ __forceinline__ int subst_row_slot(const int n[3], long S, int ta, int tb, int row) {
  const int s = row / 5 + 1, t = row - 5 * (s - 1);
  switch (t) {
    case 0: return (int)line_slot<D, 0>(n, S, ta, tb, s);
    case 1: return (int)line_slot<D, 1>(n, S, ta, tb, s);
    case 2: return (int)line_slot<D, 2>(n, S, ta, tb, s);
    case 3: return (int)line_slot<D, 3>(n, S, ta, tb, s);
    default: return (int)line_slot<D, 4>(n, S, ta, tb, s);
  }
}

template <int NT, int RING, int D>
__global__ void __launch_bounds__(NT) k_line_subst_h(const int* __restrict__ active,
                                                     const int* __restrict__ grp, long nl, int m,
                                                     long gstride, const float* __restrict__ fac,
                                                     float2* __restrict__ rb, LevelView<float> L,
                                                     int pa, int pb, LineDiv dv) {
  constexpr int kRing = RING;
  __shared__ uint4 ra[kRing][NT];
  __shared__ uint32_t rl5[kRing][NT];
  __shared__ float2 rd[kRing][NT];
  __shared__ float2 rring[kRing][NT];
  __shared__ float2 uring[D >= 1 ? kRing : 1][D >= 1 ? NT : 1];
  const int rhs = blockIdx.y;
  if (active && !active[rhs]) return;
  const int tid = threadIdx.x;
  const long l = blockIdx.x * (long)blockDim.x + tid;
  if (l >= nl) return;
  const HalfFac hf = half_fac(fac + (long)grp[rhs] * gstride, m, nl);
  float2* rr = rb + (long)rhs * m * nl + l;
  float2* u = nullptr;
  int ta = 0, tb = 0;
  if constexpr (D >= 1) {
    const LineGeom g = line_geom<D>(L.n, pa, pb);
    const unsigned lq = fdiv((unsigned)l, dv.la);
    ta = g.fa + 2 * (int)((unsigned)l - lq * (unsigned)g.la);
    tb = g.fb + 2 * (int)lq;
    u = L.u + (long)rhs * 3 * L.S;
  }
  auto issue_l = [&](int row) {
    const int slot = row % kRing;
    cp_async16(&ra[slot][tid], hf.la + (long)row * nl + l);
    cp_async4(&rl5[slot][tid], hf.lb + (long)row * nl + l);
  };
  auto take_l = [&](int row, float2 (&v)[5]) {
    const int slot = row % kRing;
    const uint4 a = ra[slot][tid];
    v[0] = u2f2(a.x);
    v[1] = u2f2(a.y);
    v[2] = u2f2(a.z);
    v[3] = u2f2(a.w);
    v[4] = u2f2(rl5[slot][tid]);
  };
  // forward: at step `row` the residual of row `row` arrives and pivot
  // row-5 is eliminated with its stored factors
  float2 y[6];
#pragma unroll
  for (int i = 0; i < 6; i++) y[i] = make_float2(0.f, 0.f);
  auto issue_fwd = [&](int q) {
    if (q < m) cp_async8(&rring[q % kRing][tid], rr + (long)q * nl);
    const int p = q - 5;
    if (p >= 0 && p < m) {
      issue_l(p);
      cp_async8(&rd[p % kRing][tid], hf.id + (long)p * nl + l);
    }
    cp_async_commit();
  };
  for (int p = 0; p < kRing - 1; p++) issue_fwd(p);
  for (int row = 0; row < m + 5; row++) {
    issue_fwd(row + kRing - 1);
    cp_async_wait<kRing - 1>();
    y[5] = row < m ? rring[row % kRing][tid] : make_float2(0.f, 0.f);
    const int piv = row - 5;
    if (piv >= 0) {
      float2 v[5];
      take_l(piv, v);
#pragma unroll
      for (int i = 1; i < 6; i++) y[i] = cfms<float>(y[i], v[i - 1], y[0]);
      rr[(long)piv * nl] = cmul<float>(y[0], rd[piv % kRing][tid]);  // z
    }
#pragma unroll
    for (int i = 0; i < 5; i++) y[i] = y[i + 1];
  }
  cp_async_wait<0>();
  __threadfence_block();  // z just stored is read back below
  // backward: x_k = z_k - sum_i L(k+i, k) x_{k+i}
  float2 xw[5];
#pragma unroll
  for (int i = 0; i < 5; i++) xw[i] = make_float2(0.f, 0.f);
  auto issue_bwd = [&](int q) {
    if (q >= 0) {
      issue_l(q);
      cp_async8(&rring[q % kRing][tid], rr + (long)q * nl);
      if constexpr (D >= 1)
        cp_async8(&uring[q % kRing][tid], u + subst_row_slot<D>(L.n, L.S, ta, tb, q));
    }
    cp_async_commit();
  };
  for (int p = 0; p < kRing - 1; p++) issue_bwd(m - 1 - p);
  for (int row = m - 1; row >= 0; row--) {
    issue_bwd(row - (kRing - 1));
    cp_async_wait<kRing - 1>();
    float2 v[5];
    take_l(row, v);
    float2 x = rring[row % kRing][tid];
#pragma unroll
    for (int i = 0; i < 5; i++) x = cfms<float>(x, v[i], xw[i]);
#pragma unroll
    for (int i = 4; i > 0; i--) xw[i] = xw[i - 1];
    xw[0] = x;
    if constexpr (D >= 1)
      u[subst_row_slot<D>(L.n, L.S, ta, tb, row)] = cadd<float>(uring[row % kRing][tid], x);
    else
      rr[(long)row * nl] = x;
  }
  cp_async_wait<0>();
}

// u += x from rb[rhs][row][line]
template <typename T, int D>
__global__ void __launch_bounds__(256) k_line_apply_rb(LevelView<T> L, int pa, int pb, LineDiv dv,
                                                       const C_t<T>* __restrict__ rb) {
  const int rhs = blockIdx.y;
  if (L.active && !L.active[rhs]) return;
  const LineGeom g = line_geom<D>(L.n, pa, pb);
  long l;
  int s;
  if (!line_item_fd<D>(g, dv, blockIdx.x * blockDim.x + threadIdx.x, l, s)) return;
  const unsigned lq = fdiv((unsigned)l, dv.la);
  const int ta = g.fa + 2 * (int)((unsigned)l - lq * (unsigned)g.la), tb = g.fb + 2 * (int)lq;
  C_t<T>* u = L.u + (long)rhs * 3 * L.S;
  const C_t<T>* x = rb + (long)rhs * g.m * g.nl + l;
  const int r0 = 5 * (s - 1);
  auto add = [&](long sl, int row) { u[sl] = cadd<T>(u[sl], x[(long)row * g.nl]); };
  add(line_slot<D, 0>(L.n, L.S, ta, tb, s), r0);
  if (s < g.nd) {
    add(line_slot<D, 1>(L.n, L.S, ta, tb, s), r0 + 1);
    add(line_slot<D, 2>(L.n, L.S, ta, tb, s), r0 + 2);
    add(line_slot<D, 3>(L.n, L.S, ta, tb, s), r0 + 3);
    add(line_slot<D, 4>(L.n, L.S, ta, tb, s), r0 + 4);
  }
}

template <typename T, int D>
static void line_factor_d(const LevelView<T>& L, int color, T* fac, int fmt, int* ovf,
                          cudaStream_t st) {
  const int pa = color & 1, pb = (color >> 1) & 1;
  const long nl = line_count(L.n, D, color);
  if (nl == 0) return;
  const long gstride = line_factor_elems(L.n, D, color, fmt);
  dim3 g((unsigned)((nl + kSolveThreads - 1) / kSolveThreads), L.nrhs);
  if constexpr (std::is_same<T, float>::value) {
    if (fmt == kFacF16) {
      k_line_factor_direct<T, D, kFacF16><<<g, kSolveThreads, 0, st>>>(L, pa, pb, gstride, fac,
                                                                       ovf);
      return;
    }
  }
  k_line_factor_direct<T, D, kFacF32><<<g, kSolveThreads, 0, st>>>(L, pa, pb, gstride, fac, ovf);
}

// the fp16-factor substitution's block shapes (threads per block, ring
// depth); variant 0 is the default
constexpr int kSubstShape[kSubstVariants][2] = {{64, 6}, {32, 6}, {128, 6}, {64, 4}, {64, 8}};

int subst_variant_threads(int v) { return kSubstShape[v][0]; }
int subst_variant_ring(int v) { return kSubstShape[v][1]; }

struct SubstArgs {
  long nl;
  int nrhs;
  const int* active;
  const int* grp;
  int m;
  long gstride;
  const float* fac;
  float2* rb;
  LevelView<float> L;
  int pa, pb;
  LineDiv dv;
};

template <int NT, int RING, int D>
static void subst_h_launch(const SubstArgs& a, cudaStream_t st) {
  dim3 g((unsigned)((a.nl + NT - 1) / NT), a.nrhs);
  k_line_subst_h<NT, RING, D><<<g, NT, 0, st>>>(a.active, a.grp, a.nl, a.m, a.gstride, a.fac,
                                                a.rb, a.L, a.pa, a.pb, a.dv);
}

template <int D>
static void subst_h_variant(int v, const SubstArgs& a, cudaStream_t st) {
  switch (v) {
    case 1: subst_h_launch<32, 6, D>(a, st); break;
    case 2: subst_h_launch<128, 6, D>(a, st); break;
    case 3: subst_h_launch<64, 4, D>(a, st); break;
    case 4: subst_h_launch<64, 8, D>(a, st); break;
    default: subst_h_launch<64, 6, D>(a, st); break;
  }
}

template <typename T, int D>
static void line_sweep_fac_d(const LevelView<T>& L, int color, const T* fac, const int* grp,
                             C_t<T>* rb, int fmt, SweepShape sh, cudaStream_t st) {
  const int pa = color & 1, pb = (color >> 1) & 1;
  const long nl = line_count(L.n, D, color);
  if (nl == 0) return;
  const long items = nl * L.n[D];
  const int m = 5 * L.n[D] - 4;
  dim3 g1((unsigned)((items + 255) / 256), L.nrhs);
  const int rt = sh.rhs_threads == 128 ? 128 : 256;
  dim3 gr((unsigned)(((D == 0 ? 5 : 1) * items + rt - 1) / rt), L.nrhs);
  const LineDiv dv = line_div<D>(L.n, pa, pb);
  if (L.imu_vol)
    k_line_rhs<T, D, 1><<<gr, rt, 0, st>>>(L, pa, pb, dv, rb);
  else
    k_line_rhs<T, D, 0><<<gr, rt, 0, st>>>(L, pa, pb, dv, rb);
  dim3 g2((unsigned)((nl + kSolveThreads - 1) / kSolveThreads), L.nrhs);
  if constexpr (std::is_same<T, float>::value) {
    if (fmt == kFacF16) {
      const int v = sh.subst >= 0 && sh.subst < kSubstVariants ? sh.subst : 0;
      const SubstArgs a{nl, L.nrhs, L.active, grp, m, line_factor_elems(L.n, D, color, fmt),
                        fac, rb, L, pa, pb, dv};
      if constexpr (D == 0) {
        subst_h_variant<-1>(v, a, st);
      } else {
        subst_h_variant<D>(v, a, st);  // the update rides the backward pass
        return;
      }
      k_line_apply_rb<T, D><<<g1, 256, 0, st>>>(L, pa, pb, dv, rb);
      return;
    }
  }
  k_line_subst<T><<<g2, kSolveThreads, 0, st>>>(L.active, grp, nl, m, fac, rb);
  k_line_apply_rb<T, D><<<g1, 256, 0, st>>>(L, pa, pb, dv, rb);
}

template <typename T, int D>
static void line_sweep_d(const LevelView<T>& L, int color, T* buf, cudaStream_t st) {
  const int pa = color & 1, pb = (color >> 1) & 1;
  const long nl = line_count(L.n, D, color);
  if (nl == 0) return;
  const long items = nl * L.n[D];
  const int m = 5 * L.n[D] - 4;
  dim3 g1((unsigned)((items + 255) / 256), L.nrhs);
  if (D == 0) {
    dim3 g5((unsigned)((5 * items + 255) / 256), L.nrhs);
    k_line_assemble_rows<T, D><<<g5, 256, 0, st>>>(L, pa, pb, buf);
  } else {
    k_line_assemble<T, D><<<g1, 256, 0, st>>>(L, pa, pb, buf);
  }
  dim3 g2((unsigned)((nl + kSolveThreads - 1) / kSolveThreads), L.nrhs);
  k_line_solve<T><<<g2, kSolveThreads, 0, st>>>(L.active, nl, m, buf);
  k_line_apply<T, D><<<g1, 256, 0, st>>>(L, pa, pb, buf);
}

// the line solve keeps a cp.async ring in shared memory: ask for the
// largest shared-memory carveout so 12 blocks fit on an SM
void init_line_kernels() {
  static std::once_flag once;
  std::call_once(once, [] {
    cudaFuncSetAttribute(k_line_solve<float>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
    cudaFuncSetAttribute(k_line_solve<double>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
    cudaFuncSetAttribute(k_line_subst<float>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
    auto carve = [](const void* k) {
      cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                           cudaSharedmemCarveoutMaxShared);
    };
    carve((const void*)k_line_subst_h<64, 6, -1>);
    carve((const void*)k_line_subst_h<32, 6, -1>);
    carve((const void*)k_line_subst_h<128, 6, -1>);
    carve((const void*)k_line_subst_h<64, 4, -1>);
    carve((const void*)k_line_subst_h<64, 8, -1>);
    carve((const void*)k_line_subst_h<64, 6, 1>);
    carve((const void*)k_line_subst_h<32, 6, 1>);
    carve((const void*)k_line_subst_h<128, 6, 1>);
    carve((const void*)k_line_subst_h<64, 4, 1>);
    carve((const void*)k_line_subst_h<64, 8, 1>);
    carve((const void*)k_line_subst_h<64, 6, 2>);
    carve((const void*)k_line_subst_h<32, 6, 2>);
    carve((const void*)k_line_subst_h<128, 6, 2>);
    carve((const void*)k_line_subst_h<64, 4, 2>);
    carve((const void*)k_line_subst_h<64, 8, 2>);
    cudaFuncSetAttribute(k_line_subst<double>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
  });
}

// scratch: m * lines * kRec values of T (see line_scratch_elems)
template <typename T>
void launch_line_sweep(const LevelView<T>& L, int d, int color, C_t<T>* scratch, cudaStream_t st) {
  T* buf = reinterpret_cast<T*>(scratch);
  if (d == 0) line_sweep_d<T, 0>(L, color, buf, st);
  else if (d == 1) line_sweep_d<T, 1>(L, color, buf, st);
  else line_sweep_d<T, 2>(L, color, buf, st);
}

long line_factor_elems(const int n[3], int d, int color, int fmt) {
  const int m = 5 * n[d] - 4;
  const long nl = line_count(n, d, color);
  return fmt == kFacF16 ? half_fac_elems(m, nl) : (long)m * nl * kRec;
}

template <typename T>
void launch_line_factor(const LevelView<T>& L, int d, int color, T* fac, int fmt, int* ovf,
                        cudaStream_t st) {
  if (d == 0) line_factor_d<T, 0>(L, color, fac, fmt, ovf, st);
  else if (d == 1) line_factor_d<T, 1>(L, color, fac, fmt, ovf, st);
  else line_factor_d<T, 2>(L, color, fac, fmt, ovf, st);
}

template <typename T>
void launch_line_sweep_fac(const LevelView<T>& L, int d, int color, const T* fac, const int* grp,
                           C_t<T>* rb, int fmt, cudaStream_t st, SweepShape sh) {
  if (d == 0) line_sweep_fac_d<T, 0>(L, color, fac, grp, rb, fmt, sh, st);
  else if (d == 1) line_sweep_fac_d<T, 1>(L, color, fac, grp, rb, fmt, sh, st);
  else line_sweep_fac_d<T, 2>(L, color, fac, grp, rb, fmt, sh, st);
}

// ---------------------------------------------------------------- fused line relaxation
// One launch per colour and direction.  A thread owns one line and walks it
// twice:
//   forward   node by node it assembles each row -- band entries and the
//             residual of the current iterate, the row arithmetic of
//             assemble_row -- and feeds it to the streaming LDL^T of
//             k_line_solve: the arriving row eliminates pivot row-5, whose
//             z = D^-1 L^-1 r and L(p+i, p), i = 1..5, are set aside;
//   backward  x_p = z_p - sum_i L(p+i, p) x_{p+i}, u += x at the row's slot.
// z_p waits in the level's residual buffer at row p's own slot: no other line
// of the colour reads or writes it, and that buffer is dead while the level
// smooths (the cycle recomputes the residual after smoothing).  L waits in
// the line scratch, [row][line] planes per RHS:
//   kLExact  the T-precision values (k_line_solve's arithmetic, bit for bit
//            the same operations in the same order);
//   kLHalf   (T = float) rounded to fp16 and used rounded by both
//            substitutions while the elimination keeps the unrounded value:
//            each line solve is then exact for a matrix within fp16 rounding
//            of the line's -- the arithmetic of the stored-factor format
//            kFacF16.  An L value outside the fp16 range sets *ovf.
// Against the three-kernel sweep this writes no band records and reads no
// stored factors: per row the neighbourhood of the residual, L (20 or 40
// bytes) and z (8 bytes) out and back, and u read-modify-write.
template <typename T, int LF> struct LineL;
template <> struct LineL<float, kLExact> {
  static constexpr long kBytes = 40;  // per row
  float4* p0;
  float4* p1;
  float2* p2;
  __device__ __forceinline__ LineL(void* base, int m, long nl) {
    p0 = reinterpret_cast<float4*>(base);
    p1 = p0 + (long)m * nl;
    p2 = reinterpret_cast<float2*>(p1 + (long)m * nl);
  }
  __device__ __forceinline__ bool put(long o, const float2 (&l)[6]) {
    p0[o] = make_float4(l[1].x, l[1].y, l[2].x, l[2].y);
    p1[o] = make_float4(l[3].x, l[3].y, l[4].x, l[4].y);
    p2[o] = l[5];
    return false;
  }
  __device__ __forceinline__ void round(float2 (&) [6]) const {}
  __device__ __forceinline__ void get(long o, float2 (&l)[5]) const {
    const float4 a = p0[o], b = p1[o];
    l[0] = make_float2(a.x, a.y);
    l[1] = make_float2(a.z, a.w);
    l[2] = make_float2(b.x, b.y);
    l[3] = make_float2(b.z, b.w);
    l[4] = p2[o];
  }
};
template <> struct LineL<double, kLExact> {
  static constexpr long kBytes = 80;
  double2* p;
  long ps;
  __device__ __forceinline__ LineL(void* base, int m, long nl) {
    p = reinterpret_cast<double2*>(base);
    ps = (long)m * nl;
  }
  __device__ __forceinline__ bool put(long o, const double2 (&l)[6]) {
#pragma unroll
    for (int i = 0; i < 5; i++) p[i * ps + o] = l[i + 1];
    return false;
  }
  __device__ __forceinline__ void round(double2 (&) [6]) const {}
  __device__ __forceinline__ void get(long o, double2 (&l)[5]) const {
#pragma unroll
    for (int i = 0; i < 5; i++) l[i] = p[i * ps + o];
  }
};
template <> struct LineL<float, kLHalf> {
  static constexpr long kBytes = 20;
  uint4* la;
  uint32_t* lb;
  __device__ __forceinline__ LineL(void* base, int m, long nl) {
    la = reinterpret_cast<uint4*>(base);
    lb = reinterpret_cast<uint32_t*>(la + (long)m * nl);
  }
  // l[1..5] rounded to fp16 in place (the values both substitutions use);
  // true when one left the fp16 range
  __device__ __forceinline__ void round(float2 (&l)[6]) const {
#pragma unroll
    for (int i = 1; i < 6; i++) l[i] = __half22float2(__floats2half2_rn(l[i].x, l[i].y));
  }
  __device__ __forceinline__ bool put(long o, const float2 (&l)[6]) {
    __half2 h[5];
    bool over = false;
#pragma unroll
    for (int i = 0; i < 5; i++) {
      h[i] = __floats2half2_rn(l[i + 1].x, l[i + 1].y);
      over |= !(fabsf(l[i + 1].x) <= 65504.f && fabsf(l[i + 1].y) <= 65504.f);
    }
    la[o] = make_uint4(h2u(h[0]), h2u(h[1]), h2u(h[2]), h2u(h[3]));
    lb[o] = h2u(h[4]);
    return over;
  }
  __device__ __forceinline__ void get(long o, float2 (&l)[5]) const {
    const uint4 a = la[o];
    l[0] = u2f2(a.x);
    l[1] = u2f2(a.y);
    l[2] = u2f2(a.z);
    l[3] = u2f2(a.w);
    l[4] = u2f2(lb[o]);
  }
};

long line_l_bytes(const int n[3], int d, int color, int lf, int tsize) {
  const long m = 5 * n[d] - 4, nl = line_count(n, d, color);
  const long b = lf == kLHalf ? 20 : (tsize == 8 ? 80 : 40);
  return (m * nl * b + 255) / 256 * 256;
}

// band entries (lower, real), diagonal and residual of row type TT of node s
template <typename T, int D, int TT, int C>
__device__ __forceinline__ void fused_row(const LevelView<T>& L, const C_t<T>* u, const C_t<T>* f,
                                          const T* cells, const Geo<T>& G, T wmu, int ta, int tb,
                                          int s, int row, const long ss[3], C_t<T> (&wrow)[6],
                                          C_t<T>& r) {
  constexpr int A = (D == 0) ? 1 : 0, B = (D == 2) ? 1 : 2;
  int P[3];
  P[D] = (TT == 0) ? s - 1 : s;
  P[A] = ta - (TT == 1 ? 1 : 0);
  P[B] = tb - (TT == 3 ? 1 : 0);
  const int sl = P[0] + (L.n[0] + 1) * (P[1] + (L.n[1] + 1) * P[2]);  // 32-bit slot
  EdgeCoef<T> e;
  const C_t<T> au = apply_row<T, C>(L, u, cells, G, wmu, P, sl, ss, e);
  r = csub<T>(f[C * (int)L.S + sl], au);
  T band[5] = {0, 0, 0, 0, 0};
#define LINE_ENTRY(K)                                                         \
  {                                                                           \
    constexpr int off = line_off(D, TT, K);                                   \
    if constexpr (off < 0) {                                                  \
      if (row + off >= 0) band[5 + off] = e.c[K];                             \
    }                                                                         \
  }
  LINE_ENTRY(0) LINE_ENTRY(1) LINE_ENTRY(2) LINE_ENTRY(3) LINE_ENTRY(4) LINE_ENTRY(5)
  LINE_ENTRY(6) LINE_ENTRY(7) LINE_ENTRY(8) LINE_ENTRY(9) LINE_ENTRY(10) LINE_ENTRY(11)
#undef LINE_ENTRY
#pragma unroll
  for (int j = 0; j < 5; j++) wrow[j] = mk<T>(band[j], 0);
  wrow[5] = mk<T>(e.dre, e.dim);
}

// one elimination step of the streaming LDL^T (k_line_solve's order): the
// new row sits in W[WI(5, .)], y[5]; pivot W[0] is eliminated.  Returns
// z = y_0 / d_0 and the multipliers l[1..5] (rounded by LS::round for kLHalf,
// the unrounded ones updating the window)
template <typename T, typename LS>
__device__ __forceinline__ C_t<T> fused_eliminate(C_t<T> (&W)[21], C_t<T> (&y)[6],
                                                  C_t<T> (&lr)[6], const LS& ls) {
  const C_t<T> id = crcp<T>(W[0]);
  C_t<T> lq[6];
#pragma unroll
  for (int i = 1; i < 6; i++) lq[i] = cmul<T>(W[WI(i, 0)], id);
#pragma unroll
  for (int i = 1; i < 6; i++) lr[i] = lq[i];
  ls.round(lr);
#pragma unroll
  for (int i = 1; i < 6; i++) {
#pragma unroll
    for (int j = 1; j <= i; j++) W[WI(i, j)] = cfms<T>(W[WI(i, j)], lq[i], W[WI(j, 0)]);
    y[i] = cfms<T>(y[i], lr[i], y[0]);
  }
  const C_t<T> z = cmul<T>(y[0], id);
#pragma unroll
  for (int i = 0; i < 5; i++) {
#pragma unroll
    for (int j = 0; j <= i; j++) W[WI(i, j)] = W[WI(i + 1, j + 1)];
    y[i] = y[i + 1];
  }
  return z;
}

template <typename T, int D, int LF, int NT>
__global__ void __launch_bounds__(NT) k_line_fused(LevelView<T> L, int pa, int pb, LineDiv dv,
                                                   void* __restrict__ lbuf, long lstride,
                                                   int* __restrict__ ovf) {
  constexpr int A = (D == 0) ? 1 : 0, B = (D == 2) ? 1 : 2;
  using LS = LineL<T, LF>;
  const int rhs = blockIdx.y;
  if (L.active && !L.active[rhs]) return;
  const LineGeom g = line_geom<D>(L.n, pa, pb);
  const long l = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (l >= g.nl) return;
  const unsigned lq = fdiv((unsigned)l, dv.la);
  const int ta = g.fa + 2 * (int)((unsigned)l - lq * (unsigned)g.la), tb = g.fb + 2 * (int)lq;
  const int n0 = L.n[0] + 1, n1 = L.n[1] + 1;
  const long ss[3] = {1, (long)n0, (long)n0 * n1};
  C_t<T>* __restrict__ u = L.u + (long)rhs * 3 * L.S;
  const C_t<T>* __restrict__ f = L.f + (long)rhs * 3 * L.S;
  C_t<T>* __restrict__ zr = L.r + (long)rhs * 3 * L.S;
  const T* __restrict__ cells = L.cells + (long)op_of(L, rhs) * 4 * L.ncell;
  const Geo<T> G{L.geo + (long)op_of(L, rhs) * L.gstride, L.gmax1};
  const T wmu = L.wmu[rhs];
  LS ls(static_cast<char*>(lbuf) + (long)rhs * lstride, g.m, g.nl);
  const int nd = g.nd;
  bool over = false;

  C_t<T> W[21], y[6], lr[6];
#pragma unroll
  for (int i = 0; i < 21; i++) W[i] = mk<T>(0, 0);
#pragma unroll
  for (int i = 0; i < 5; i++) {
    W[WI(i, i)] = mk<T>(1, 0);  // dummy leading rows
    y[i] = mk<T>(0, 0);
  }
  // Rows are assembled a node at a time -- the five rows' loads issued
  // together, ahead of the node's five elimination steps -- so a node waits
  // on memory once rather than once per row.  The arriving row (s, TT)
  // eliminates pivot (s-1, TT): same row type, one node back; with s = 1 the
  // pivots are the dummy leading rows.
  C_t<T> rw[5][6], rr[5];
  auto assemble = [&](auto tt, int s) {
    constexpr int TT = decltype(tt)::value;
    constexpr int C = (TT == 0) ? D : (TT <= 2 ? A : B);
    fused_row<T, D, TT, C>(L, u, f, cells, G, wmu, ta, tb, s, 5 * (s - 1) + TT, ss, rw[TT],
                           rr[TT]);
  };
  auto arrive = [&](auto tt, int s) {
    constexpr int TT = decltype(tt)::value;
#pragma unroll
    for (int j = 0; j < 6; j++) W[WI(5, j)] = rw[TT][j];
    y[5] = rr[TT];
    const C_t<T> z = fused_eliminate<T>(W, y, lr, ls);
    if (s >= 2) {
      const int p = 5 * (s - 2) + TT;
      zr[line_slot<D, TT>(L.n, L.S, ta, tb, s - 1)] = z;
      over |= ls.put((long)p * g.nl + l, lr);
    }
  };
  // trailing steps: identity rows flush pivots (s, TT) of the last rows
  auto flush = [&](auto tt, int s) {
    constexpr int TT = decltype(tt)::value;
#pragma unroll
    for (int j = 0; j < 5; j++) W[WI(5, j)] = mk<T>(0, 0);
    W[WI(5, 5)] = mk<T>(1, 0);
    y[5] = mk<T>(0, 0);
    const C_t<T> z = fused_eliminate<T>(W, y, lr, ls);
    const int p = 5 * (s - 1) + TT;
    zr[line_slot<D, TT>(L.n, L.S, ta, tb, s)] = z;
    over |= ls.put((long)p * g.nl + l, lr);
  };
  using I0 = std::integral_constant<int, 0>;
  using I1 = std::integral_constant<int, 1>;
  using I2 = std::integral_constant<int, 2>;
  using I3 = std::integral_constant<int, 3>;
  using I4 = std::integral_constant<int, 4>;
  for (int s = 1; s < nd; s++) {
    assemble(I0{}, s);
    assemble(I1{}, s);
    assemble(I2{}, s);
    assemble(I3{}, s);
    assemble(I4{}, s);
    arrive(I0{}, s);
    arrive(I1{}, s);
    arrive(I2{}, s);
    arrive(I3{}, s);
    arrive(I4{}, s);
  }
  assemble(I0{}, nd);
  arrive(I0{}, nd);
  flush(I1{}, nd - 1);
  flush(I2{}, nd - 1);
  flush(I3{}, nd - 1);
  flush(I4{}, nd - 1);
  flush(I0{}, nd);
  if (over && ovf) atomicOr(ovf, 1);

  // backward: rows m-1 .. 0, i.e. (nd, 0), then (s, 4..0) for s = nd-1 .. 1
  C_t<T> xw[5];
#pragma unroll
  for (int i = 0; i < 5; i++) xw[i] = mk<T>(0, 0);
  // backward a node at a time as well: its rows' multipliers, z and u are
  // loaded together before the five substitution steps
  C_t<T> bl[5][5], bz[5], bu[5];
  long bs[5];
  auto load = [&](auto tt, int s) {
    constexpr int TT = decltype(tt)::value;
    bs[TT] = line_slot<D, TT>(L.n, L.S, ta, tb, s);
    ls.get((long)(5 * (s - 1) + TT) * g.nl + l, bl[TT]);
    bz[TT] = zr[bs[TT]];
    bu[TT] = u[bs[TT]];
  };
  auto back = [&](auto tt) {
    constexpr int TT = decltype(tt)::value;
    C_t<T> x = bz[TT];
#pragma unroll
    for (int i = 0; i < 5; i++) x = cfms<T>(x, bl[TT][i], xw[i]);
#pragma unroll
    for (int i = 4; i > 0; i--) xw[i] = xw[i - 1];
    xw[0] = x;
    u[bs[TT]] = cadd<T>(bu[TT], x);
  };
  load(I0{}, nd);
  back(I0{});
  for (int s = nd - 1; s >= 1; s--) {
    load(I4{}, s);
    load(I3{}, s);
    load(I2{}, s);
    load(I1{}, s);
    load(I0{}, s);
    back(I4{});
    back(I3{});
    back(I2{});
    back(I1{});
    back(I0{});
  }
}

template <typename T, int D, int LF, int NT>
static void fused_launch(const LevelView<T>& L, int pa, int pb, long nl, void* lbuf, long lstride,
                         int* ovf, cudaStream_t st) {
  const LineDiv dv = line_div<D>(L.n, pa, pb);
  dim3 g((unsigned)((nl + NT - 1) / NT), L.nrhs);
  k_line_fused<T, D, LF, NT><<<g, NT, 0, st>>>(L, pa, pb, dv, lbuf, lstride, ovf);
}

template <typename T, int D>
static void line_fused_d(const LevelView<T>& L, int color, void* lbuf, int lf, int nt, int* ovf,
                         cudaStream_t st) {
  const int pa = color & 1, pb = (color >> 1) & 1;
  const long nl = line_count(L.n, D, color);
  if (nl == 0) return;
  const long lstride = line_l_bytes(L.n, D, color, lf, (int)sizeof(T));
  if constexpr (std::is_same<T, float>::value) {
    if (lf == kLHalf) {
      if (nt == 32) fused_launch<T, D, kLHalf, 32>(L, pa, pb, nl, lbuf, lstride, ovf, st);
      else if (nt == 128) fused_launch<T, D, kLHalf, 128>(L, pa, pb, nl, lbuf, lstride, ovf, st);
      else fused_launch<T, D, kLHalf, 64>(L, pa, pb, nl, lbuf, lstride, ovf, st);
      return;
    }
  }
  if (nt == 32) fused_launch<T, D, kLExact, 32>(L, pa, pb, nl, lbuf, lstride, ovf, st);
  else if (nt == 128) fused_launch<T, D, kLExact, 128>(L, pa, pb, nl, lbuf, lstride, ovf, st);
  else fused_launch<T, D, kLExact, 64>(L, pa, pb, nl, lbuf, lstride, ovf, st);
}

template <typename T>
void launch_line_fused(const LevelView<T>& L, int d, int color, void* lbuf, int lf, int nt,
                       int* ovf, cudaStream_t st) {
  if (d == 0) line_fused_d<T, 0>(L, color, lbuf, lf, nt, ovf, st);
  else if (d == 1) line_fused_d<T, 1>(L, color, lbuf, lf, nt, ovf, st);
  else line_fused_d<T, 2>(L, color, lbuf, lf, nt, ovf, st);
}
template void launch_line_fused<float>(const LevelView<float>&, int, int, void*, int, int, int*,
                                       cudaStream_t);
template void launch_line_fused<double>(const LevelView<double>&, int, int, void*, int, int, int*,
                                        cudaStream_t);

// ------------------------------------------------------------ point sweep
// row (C, side): side 0 = E_C(N - e_C), side 1 = E_C(N); patch index 2C+side.
template <typename T, int C, int SIDE>
__device__ __forceinline__ void patch_row(const LevelView<T>& L, const C_t<T>* u, const C_t<T>* f,
                                          const T* cells, const Geo<T>& G, T wmu, const int N[3],
                                          const long ss[3], C_t<T> (&M)[21], C_t<T> (&y)[6]) {
  constexpr int p = Cyc<C>::p, q = Cyc<C>::q;
  constexpr int ri = 2 * C + SIDE;
  int P[3] = {N[0], N[1], N[2]};
  P[C] -= 1 - SIDE;
  const long sl = slot_id(L.n, P[0], P[1], P[2]);
  EdgeCoef<T> e;
  const C_t<T> au = apply_row<T, C>(L, u, cells, G, wmu, P, sl, ss, e);
  y[ri] = csub<T>(f[(long)C * L.S + sl], au);
  M[WI(ri, ri)] = mk<T>(e.dre, e.dim);
  // in-patch neighbours: side 0 -> k=4 (p,1), 6 (p,0), 8 (q,1), 10 (q,0);
  //                      side 1 -> k=5, 7, 9, 11
  constexpr int kp1 = SIDE ? 5 : 4, kp0 = SIDE ? 7 : 6, kq1 = SIDE ? 9 : 8, kq0 = SIDE ? 11 : 10;
  constexpr int ip1 = 2 * p + 1, ip0 = 2 * p, iq1 = 2 * q + 1, iq0 = 2 * q;
  if constexpr (ip1 < ri) M[WI(ri, ip1)] = mk<T>(e.c[kp1], 0);
  if constexpr (ip0 < ri) M[WI(ri, ip0)] = mk<T>(e.c[kp0], 0);
  if constexpr (iq1 < ri) M[WI(ri, iq1)] = mk<T>(e.c[kq1], 0);
  if constexpr (iq0 < ri) M[WI(ri, iq0)] = mk<T>(e.c[kq0], 0);
}

template <typename T>
__global__ void __launch_bounds__(128) k_point_sweep(LevelView<T> L, int color) {
  const int rhs = blockIdx.y;
  if (L.active && !L.active[rhs]) return;
  int cnt[3], first[3];
#pragma unroll
  for (int e = 0; e < 3; e++) {
    const int par = (color >> e) & 1;
    first[e] = par ? 1 : 2;
    cnt[e] = (L.n[e] - 1 >= first[e]) ? (L.n[e] - 1 - first[e]) / 2 + 1 : 0;
  }
  const long tot = (long)cnt[0] * cnt[1] * cnt[2];
  const long id = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (id >= tot) return;
  const int N[3] = {first[0] + 2 * (int)(id % cnt[0]), first[1] + 2 * (int)((id / cnt[0]) % cnt[1]),
                    first[2] + 2 * (int)(id / ((long)cnt[0] * cnt[1]))};
  const int n0 = L.n[0] + 1, n1 = L.n[1] + 1;
  const long ss[3] = {1, (long)n0, (long)n0 * n1};
  C_t<T>* u = L.u + (long)rhs * 3 * L.S;
  const C_t<T>* f = L.f + (long)rhs * 3 * L.S;
  const T* cells = L.cells + (long)op_of(L, rhs) * 4 * L.ncell;
  const Geo<T> G{L.geo + (long)op_of(L, rhs) * L.gstride, L.gmax1};
  const T wmu = L.wmu[rhs];
  C_t<T> M[21], y[6];
#pragma unroll
  for (int i = 0; i < 21; i++) M[i] = mk<T>(0, 0);
  patch_row<T, 0, 0>(L, u, f, cells, G, wmu, N, ss, M, y);
  patch_row<T, 0, 1>(L, u, f, cells, G, wmu, N, ss, M, y);
  patch_row<T, 1, 0>(L, u, f, cells, G, wmu, N, ss, M, y);
  patch_row<T, 1, 1>(L, u, f, cells, G, wmu, N, ss, M, y);
  patch_row<T, 2, 0>(L, u, f, cells, G, wmu, N, ss, M, y);
  patch_row<T, 2, 1>(L, u, f, cells, G, wmu, N, ss, M, y);
  // dense complex-symmetric LDL^T on the lower triangle
  C_t<T> Lm[21], z[6];
#pragma unroll
  for (int k = 0; k < 6; k++) {
    const C_t<T> id = crcp<T>(M[WI(k, k)]);
#pragma unroll
    for (int i = k + 1; i < 6; i++) {
      const C_t<T> l = cmul<T>(M[WI(i, k)], id);
#pragma unroll
      for (int j = k + 1; j <= i; j++) M[WI(i, j)] = cfms<T>(M[WI(i, j)], l, M[WI(j, k)]);
      y[i] = cfms<T>(y[i], l, y[k]);
      Lm[WI(i, k)] = l;
    }
    z[k] = cmul<T>(y[k], id);
  }
#pragma unroll
  for (int k = 5; k >= 0; k--) {
#pragma unroll
    for (int i = k + 1; i < 6; i++) z[k] = cfms<T>(z[k], Lm[WI(i, k)], z[i]);
  }
#pragma unroll
  for (int ri = 0; ri < 6; ri++) {
    const int c = ri / 2;
    int P[3] = {N[0], N[1], N[2]};
    P[c] -= 1 - (ri & 1);
    const long sl = (long)c * L.S + slot_id(L.n, P[0], P[1], P[2]);
    u[sl] = cadd<T>(u[sl], z[ri]);
  }
}

template <typename T>
void launch_point_sweep(const LevelView<T>& L, int color, cudaStream_t st) {
  long cnt = 1;
  for (int e = 0; e < 3; e++) {
    const int par = (color >> e) & 1, first = par ? 1 : 2;
    cnt *= (L.n[e] - 1 >= first) ? (L.n[e] - 1 - first) / 2 + 1 : 0;
  }
  if (cnt == 0) return;
  dim3 grid((unsigned)((cnt + 127) / 128), L.nrhs);
  k_point_sweep<T><<<grid, 128, 0, st>>>(L, color);
}

// ------------------------------------------------------------ transfers
template <typename T>
struct Xfer {
  int nf[3], nc[3], sc[3];
};

// the transfer weights of a level (LevelView::xw), once per set-up: the
// arithmetic the transfers used to repeat in every thread
template <typename T>
__global__ void __launch_bounds__(256) k_xfer_weights(LevelView<T> F, LevelView<T> Cc, int sc0,
                                                      int sc1, int sc2, int nop, T* __restrict__ out) {
  const int g1 = F.gmax1;
  const long id = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (id >= (long)nop * 3 * g1) return;
  const int o = (int)(id / (3 * g1));
  const int e = (int)((id / g1) % 3);
  const int f = (int)(id % g1);
  const int sc = e == 0 ? sc0 : e == 1 ? sc1 : sc2;
  const int c = sc == 2 ? f / 2 : f;
  T w = 0;
  if (f <= F.n[e] && c < Cc.n[e]) {
    const T* xf = F.geo + (long)o * F.gstride + (long)e * g1;
    const T* xc = Cc.geo + (long)o * Cc.gstride + (long)e * g1;
    w = (xf[f] - xc[c]) / (xc[c + 1] - xc[c]);
  }
  out[id] = w;
}

template <typename T>
void launch_xfer_weights(const LevelView<T>& F, const LevelView<T>& Cc, const int sc[3], int nop,
                         T* out, cudaStream_t st) {
  const long n = (long)nop * 3 * F.gmax1;
  k_xfer_weights<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(F, Cc, sc[0], sc[1], sc[2], nop, out);
}
template void launch_xfer_weights<float>(const LevelView<float>&, const LevelView<float>&,
                                         const int*, int, float*, cudaStream_t);
template void launch_xfer_weights<double>(const LevelView<double>&, const LevelView<double>&,
                                          const int*, int, double*, cudaStream_t);

// the fine nodes along axis e restricted to coarse node Ce, in the order of
// src/gmg.c:1510-1573: those whose coarse interval starts at Ce (weight
// 1 - wr), then those whose interval ends at Ce (weight wr), two slots each;
// a slot is used when its node is an interior fine node and its weight is
// not exactly zero (a zero-weight term adds nothing to the sum)
template <typename T>
__device__ __forceinline__ void xfer_slots(int Ce, int sce, int nfe, int nce,
                                           const T* __restrict__ wr, int (&idx)[4], T (&w)[4],
                                           bool (&ok)[4]) {
#pragma unroll
  for (int t = 0; t < 2; t++) {
    const int F = (sce == 2 ? 2 * Ce : Ce) + t;
    idx[t] = F;
    w[t] = T(0);
    if (t < sce && Ce < nce && F >= 1 && F < nfe) w[t] = T(1) - ldro(wr + F);
    ok[t] = w[t] != T(0);
  }
#pragma unroll
  for (int t = 0; t < 2; t++) {
    const int F = (sce == 2 ? 2 * (Ce - 1) : Ce - 1) + t;
    idx[2 + t] = F;
    w[2 + t] = T(0);
    if (t < sce && Ce >= 1 && F >= 1 && F < nfe) w[2 + t] = ldro(wr + F);
    ok[2 + t] = w[2 + t] != T(0);
  }
}

template <typename T, int C>
__device__ __forceinline__ C_t<T> restrict_comp(const LevelView<T>& F, const LevelView<T>& Cc,
                                                const int sc[3], const int Cn[3],
                                                const C_t<T>* __restrict__ rf,
                                                const T* __restrict__ xw) {
  constexpr int p = Cyc<C>::p, q = Cyc<C>::q;
  constexpr int t1 = p < q ? p : q, t2 = p < q ? q : p;
  int i1[4], i2[4];
  T w1[4], w2[4];
  bool o1[4], o2[4];
  xfer_slots<T>(Cn[t1], sc[t1], F.n[t1], Cc.n[t1], xw + t1 * F.gmax1, i1, w1, o1);
  xfer_slots<T>(Cn[t2], sc[t2], F.n[t2], Cc.n[t2], xw + t2 * F.gmax1, i2, w2, o2);
  const int fs[3] = {1, F.n[0] + 1, (F.n[0] + 1) * (F.n[1] + 1)};
  T ar = 0, ai = 0;
  const int f0 = sc[C] == 2 ? 2 * Cn[C] : Cn[C];
#pragma unroll
  for (int t = 0; t < 2; t++) {
    const int fc = f0 + t;
    if (t >= sc[C] || fc >= F.n[C]) continue;
    const int base = C * (int)F.S + fc * fs[C];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      if (!o1[a]) continue;
      const int ba = base + i1[a] * fs[t1];
#pragma unroll
      for (int b = 0; b < 4; b++) {
        if (!o2[b]) continue;
        const C_t<T> v = ldro(rf + (ba + i2[b] * fs[t2]));
        const T w = w1[a] * w2[b];
        ar += w * v.x;
        ai += w * v.y;
      }
    }
  }
  return mk<T>(ar, ai);
}

template <typename T>
__global__ void __launch_bounds__(256) k_restrict(LevelView<T> F, LevelView<T> Cc, int sc0, int sc1,
                                                  int sc2) {
  const int rhs = blockIdx.y;
  if (Cc.active && !Cc.active[rhs]) return;
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= Cc.S) return;
  const int sc[3] = {sc0, sc1, sc2};
  int Cn[3];
  slot_nodes(s, Cc, Cn);
  const C_t<T>* rf = F.r + (long)rhs * 3 * F.S;
  const int c = blockIdx.z;  // one component per thread
  C_t<T>* fc = Cc.f + ((long)rhs * 3 + c) * Cc.S;
  C_t<T>* uc = Cc.u + ((long)rhs * 3 + c) * Cc.S;
  const T* xw = F.xw + (long)op_of(F, rhs) * 3 * F.gmax1;
  C_t<T> v;
  switch (c) {
    case 0: v = restrict_comp<T, 0>(F, Cc, sc, Cn, rf, xw); break;
    case 1: v = restrict_comp<T, 1>(F, Cc, sc, Cn, rf, xw); break;
    default: v = restrict_comp<T, 2>(F, Cc, sc, Cn, rf, xw); break;
  }
  fc[s] = v;
  uc[s] = mk<T>(0, 0);
}

template <typename T>
void launch_restrict(const LevelView<T>& F, const LevelView<T>& Cc, const int sc[3], cudaStream_t st) {
  dim3 grid((unsigned)((Cc.S + 255) / 256), Cc.nrhs, 3);
  k_restrict<T><<<grid, 256, 0, st>>>(F, Cc, sc[0], sc[1], sc[2]);
}

template <typename T, int C>
__device__ __forceinline__ void prolong_comp(const LevelView<T>& F, const LevelView<T>& Cc,
                                             const int sc[3], const int P[3], C_t<T>* uf,
                                             const C_t<T>* __restrict__ uc,
                                             const T* __restrict__ xw, long s) {
  constexpr int p = Cyc<C>::p, q = Cyc<C>::q;
  constexpr int t1 = p < q ? p : q, t2 = p < q ? q : p;
  if (!(P[C] < F.n[C] && P[t1] >= 1 && P[t1] < F.n[t1] && P[t2] >= 1 && P[t2] < F.n[t2])) return;
  int Cn[3];
#pragma unroll
  for (int e = 0; e < 3; e++) Cn[e] = sc[e] == 2 ? P[e] / 2 : P[e];
  const T wr1 = ldro(xw + t1 * F.gmax1 + P[t1]);
  const T wr2 = ldro(xw + t2 * F.gmax1 + P[t2]);
  const T wl1 = T(1) - wr1, wl2 = T(1) - wr2;
  // 32-bit offsets: the four coarse neighbours differ by the strides of t1, t2
  const int cs[3] = {1, Cc.n[0] + 1, (Cc.n[0] + 1) * (Cc.n[1] + 1)};
  const int q00 = C * (int)Cc.S + slot_id32(Cc.n, Cn[0], Cn[1], Cn[2]);
  const C_t<T> u00 = uc[q00];
  const C_t<T> u01 = uc[q00 + cs[t2]];
  const C_t<T> u10 = uc[q00 + cs[t1]];
  const C_t<T> u11 = uc[q00 + cs[t1] + cs[t2]];
  C_t<T> v = uf[C * (int)F.S + (int)s];
  v.x += wl1 * (wl2 * u00.x + wr2 * u01.x) + wr1 * (wl2 * u10.x + wr2 * u11.x);
  v.y += wl1 * (wl2 * u00.y + wr2 * u01.y) + wr1 * (wl2 * u10.y + wr2 * u11.y);
  uf[C * (int)F.S + (int)s] = v;
}

template <typename T>
__global__ void __launch_bounds__(256) k_prolong(LevelView<T> F, LevelView<T> Cc, int sc0, int sc1,
                                                 int sc2) {
  const int rhs = blockIdx.y;
  if (F.active && !F.active[rhs]) return;
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= F.S) return;
  const int sc[3] = {sc0, sc1, sc2};
  int P[3];
  slot_nodes(s, F, P);
  C_t<T>* uf = F.u + (long)rhs * 3 * F.S;
  const C_t<T>* uc = Cc.u + (long)rhs * 3 * Cc.S;
  const T* xw = F.xw + (long)op_of(F, rhs) * 3 * F.gmax1;
  switch (blockIdx.z) {  // one component per thread
    case 0: prolong_comp<T, 0>(F, Cc, sc, P, uf, uc, xw, s); break;
    case 1: prolong_comp<T, 1>(F, Cc, sc, P, uf, uc, xw, s); break;
    default: prolong_comp<T, 2>(F, Cc, sc, P, uf, uc, xw, s); break;
  }
}

template <typename T>
void launch_prolong(const LevelView<T>& F, const LevelView<T>& Cc, const int sc[3], cudaStream_t st) {
  dim3 grid((unsigned)((F.S + 255) / 256), F.nrhs, 3);
  k_prolong<T><<<grid, 256, 0, st>>>(F, Cc, sc[0], sc[1], sc[2]);
}

// ------------------------------------------------------------ coarsening
template <typename T>
__global__ void __launch_bounds__(256) k_coarsen(const T* __restrict__ fine, int nf0, int nf1, int nf2,
                                                 T* __restrict__ coarse, int sc0, int sc1, int sc2) {
  const int nc0 = nf0 / sc0, nc1 = nf1 / sc1, nc2 = nf2 / sc2;
  const long ncc = (long)nc0 * nc1 * nc2, nfc = (long)nf0 * nf1 * nf2;
  const long id = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (id >= ncc) return;
  const long arr = blockIdx.y;  // rhs*4 + which
  // 32-bit decode (a level has fewer than 2^31 cells)
  const unsigned t = (unsigned)id / (unsigned)nc0;
  const int i = (int)((unsigned)id - t * (unsigned)nc0);
  const int j = (int)(t % (unsigned)nc1), k = (int)(t / (unsigned)nc1);
  const int i0 = sc0 == 2 ? 2 * i : i, i1 = sc0 == 2 ? 2 * i + 1 : i;
  const int j0 = sc1 == 2 ? 2 * j : j, j1 = sc1 == 2 ? 2 * j + 1 : j;
  const int k0 = sc2 == 2 ? 2 * k : k, k1 = sc2 == 2 ? 2 * k + 1 : k;
  const T* F = fine + arr * nfc;
#define CF(a, b, c) F[(a) + (long)nf0 * ((b) + (long)nf1 * (c))]
  const T v = CF(i0, j0, k0) + CF(i1, j0, k0) + CF(i0, j1, k0) + CF(i1, j1, k0) + CF(i0, j0, k1) +
              CF(i1, j0, k1) + CF(i0, j1, k1) + CF(i1, j1, k1);
#undef CF
  const int repeat = 8 / (sc0 * sc1 * sc2);
  coarse[arr * ncc + id] = v / (T)repeat;
}

template <typename T>
void launch_coarsen_cells(const T* fine, const int nf[3], T* coarse, const int sc[3], int nrhs,
                          cudaStream_t st) {
  const long ncc = (long)(nf[0] / sc[0]) * (nf[1] / sc[1]) * (nf[2] / sc[2]);
  dim3 grid((unsigned)((ncc + 255) / 256), 4 * nrhs);
  k_coarsen<T><<<grid, 256, 0, st>>>(fine, nf[0], nf[1], nf[2], coarse, sc[0], sc[1], sc[2]);
}

template <typename T>
__global__ void k_zero(C_t<T>* p, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    p[i] = mk<T>(0, 0);
}

template <typename T>
void launch_zero(C_t<T>* p, long n, cudaStream_t st) {
  long blocks = (n + 255) / 256;
  if (blocks > 4864) blocks = 4864;
  if (blocks < 1) blocks = 1;
  k_zero<T><<<(unsigned)blocks, 256, 0, st>>>(p, n);
}

// ------------------------------------------------------------ instantiations
#define EMMI_INST(T)                                                                               \
  template void launch_norm<T>(const C_t<T>*, long, int, const int*, double*, cudaStream_t);        \
  template void launch_line_sweep<T>(const LevelView<T>&, int, int, C_t<T>*, cudaStream_t);         \
  template void launch_point_sweep<T>(const LevelView<T>&, int, cudaStream_t);                      \
  template void launch_restrict<T>(const LevelView<T>&, const LevelView<T>&, const int*,            \
                                   cudaStream_t);                                                   \
  template void launch_prolong<T>(const LevelView<T>&, const LevelView<T>&, const int*,             \
                                  cudaStream_t);                                                    \
  template void launch_coarsen_cells<T>(const T*, const int*, T*, const int*, int, cudaStream_t);   \
  template void launch_zero<T>(C_t<T>*, long, cudaStream_t);
EMMI_INST(float)
EMMI_INST(double)
template void launch_line_factor<float>(const LevelView<float>&, int, int, float*, int, int*,
                                        cudaStream_t);
template void launch_line_sweep_fac<float>(const LevelView<float>&, int, int, const float*,
                                           const int*, C_t<float>*, int, cudaStream_t, SweepShape);
template void launch_line_factor<double>(const LevelView<double>&, int, int, double*, int, int*,
                                         cudaStream_t);
template void launch_line_sweep_fac<double>(const LevelView<double>&, int, int, const double*,
                                            const int*, C_t<double>*, int, cudaStream_t,
                                            SweepShape);
template void launch_residual<float, float>(const LevelView<float>&, C_t<float>*, double*, cudaStream_t);
template void launch_residual<double, double>(const LevelView<double>&, C_t<double>*, double*, cudaStream_t);
template void launch_residual<double, float>(const LevelView<double>&, C_t<float>*, double*, cudaStream_t);

}  // namespace emmi

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

#include <cstdio>
#include <mutex>

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

void init_line_tables() {}

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

// ------------------------------------------------------------ residual
template <typename T, int C>
__device__ __forceinline__ C_t<T> apply_row(const LevelView<T>& L, const C_t<T>* __restrict__ u,
                                            const T* __restrict__ cells, const Geo<T>& G, T wmu,
                                            const int P[3], long s, const long ss[3],
                                            EdgeCoef<T>& e) {
  // u, cells and geometry are not written by any thread while a residual,
  // an assembly or a same-colour block sweep reads them: read-only loads
  edge_coef<T, C>(L.n, P, cells + (long)C * L.ncell, cells + 3 * L.ncell, G, wmu, e);
  const C_t<T> uc = ldro(u + (long)C * L.S + s);
  T ar = e.dre * uc.x - e.dim * uc.y;
  T ai = e.dre * uc.y + e.dim * uc.x;
#pragma unroll
  for (int k = 0; k < 12; k++) {
    const C_t<T> v = ldro(u + s + nbr_slot_delta<C>(k, ss, L.S));
    ar += e.c[k] * v.x;
    ai += e.c[k] * v.y;
  }
  return mk<T>(ar, ai);
}

template <int C>
__device__ __forceinline__ bool is_unknown(const int n[3], const int P[3]) {
  constexpr int p = Cyc<C>::p, q = Cyc<C>::q;
  return P[C] < n[C] && P[p] >= 1 && P[p] < n[p] && P[q] >= 1 && P[q] < n[q];
}

template <typename T, typename TO, int C>
__device__ __forceinline__ double residual_comp(const LevelView<T>& L, const C_t<T>* u,
                                                const C_t<T>* f, const T* cells, const Geo<T>& G,
                                                T wmu, const int P[3], long s, const long ss[3],
                                                C_t<TO>* rout) {
  C_t<T> r = f[(long)C * L.S + s];
  if (is_unknown<C>(L.n, P)) {
    EdgeCoef<T> e;
    const C_t<T> au = apply_row<T, C>(L, u, cells, G, wmu, P, s, ss, e);
    r = csub<T>(r, au);
  }
  if (rout) rout[(long)C * L.S + s] = mk<TO>((TO)r.x, (TO)r.y);
  return (double)r.x * (double)r.x + (double)r.y * (double)r.y;
}

template <typename T, typename TO>
__global__ void __launch_bounds__(256) k_residual(LevelView<T> L, C_t<TO>* __restrict__ rout,
                                                  double* __restrict__ norm2) {
  const int rhs = blockIdx.y;
  if (L.active && !L.active[rhs]) return;
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  double acc = 0.0;
  if (s < L.S) {
    const int n0 = L.n[0] + 1, n1 = L.n[1] + 1;
    const int P[3] = {(int)(s % n0), (int)((s / n0) % n1), (int)(s / ((long)n0 * n1))};
    const long ss[3] = {1, (long)n0, (long)n0 * n1};
    const C_t<T>* u = L.u + (long)rhs * 3 * L.S;
    const C_t<T>* f = L.f + (long)rhs * 3 * L.S;
    const T* cells = L.cells + (long)op_of(L, rhs) * 4 * L.ncell;
    const Geo<T> G{L.geo + (long)op_of(L, rhs) * L.gstride, L.gmax1};
    const T wmu = L.wmu[rhs];
    C_t<TO>* ro = rout ? rout + (long)rhs * 3 * L.S : nullptr;
    acc += residual_comp<T, TO, 0>(L, u, f, cells, G, wmu, P, s, ss, ro);
    acc += residual_comp<T, TO, 1>(L, u, f, cells, G, wmu, P, s, ss, ro);
    acc += residual_comp<T, TO, 2>(L, u, f, cells, G, wmu, P, s, ss, ro);
  }
  if (norm2) block_add(acc, norm2 + rhs);
}

template <typename T, typename TO>
void launch_residual(const LevelView<T>& L, C_t<TO>* rout, double* norm2, cudaStream_t st) {
  dim3 grid((unsigned)((L.S + 255) / 256), L.nrhs);
  k_residual<T, TO><<<grid, 256, 0, st>>>(L, rout, norm2);
}

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
__device__ __forceinline__ LineGeom line_geom(const int n[3], int pa, int pb) {
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
    l = id / g.nd;
    s = 1 + (int)(id % g.nd);
  } else {  // neighbouring lines (consecutive i) are contiguous
    l = id % g.nl;
    s = 1 + (int)(id / g.nl);
  }
  return true;
}

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
  const long sl = slot_id(L.n, P[0], P[1], P[2]);
  EdgeCoef<T> e;
  const C_t<T> au = apply_row<T, C>(L, u, cells, G, wmu, P, sl, ss, e);
  const C_t<T> r = csub<T>(f[(long)C * L.S + sl], au);
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

template <typename T, int D>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) k_line_assemble(LevelView<T> L, int pa, int pb,
                                                       T* __restrict__ buf) {
  constexpr int A = (D == 0) ? 1 : 0, B = (D == 2) ? 1 : 2;
  const int rhs = blockIdx.y;
  if (L.active && !L.active[rhs]) return;
  const LineGeom g = line_geom<D>(L.n, pa, pb);
  long l;
  int s;
  if (!line_item<D>(g, blockIdx.x * (long)blockDim.x + threadIdx.x, l, s)) return;
  const int ta = g.fa + 2 * (int)(l % g.la), tb = g.fb + 2 * (int)(l / g.la);
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

template <typename T>
__global__ void __launch_bounds__(64) k_line_solve(const int* __restrict__ active, long nl, int m,
                                                   T* __restrict__ buf) {
  using V = typename Vec16<T>::V;
  const int rhs = blockIdx.y;
  if (active && !active[rhs]) return;
  const long l = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (l >= nl) return;
  V* base = reinterpret_cast<V*>(buf) + (long)rhs * m * kPlanes<T> * nl + l;
  const long rs = kPlanes<T> * nl;  // distance between rows
  C_t<T> W[21], y[6];
#pragma unroll
  for (int i = 0; i < 21; i++) W[i] = mk<T>(0, 0);
#pragma unroll
  for (int i = 0; i < 5; i++) {
    W[WI(i, i)] = mk<T>(1, 0);  // dummy leading rows
    y[i] = mk<T>(0, 0);
  }
  T nxt[kRec];
  rec_get<T>(base, nl, nxt);
  // forward: arriving row r eliminates pivot r-5
  for (int row = 0; row < m + 5; row++) {
    if (row < m) {
#pragma unroll
      for (int j = 0; j < 5; j++) W[WI(5, j)] = mk<T>(nxt[j], 0);
      W[WI(5, 5)] = mk<T>(nxt[5], nxt[6]);
      y[5] = mk<T>(nxt[7], nxt[8]);
      if (row + 1 < m) rec_get<T>(base + (long)(row + 1) * rs, nl, nxt);  // prefetch
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
  // backward: x_k = z_k - sum_i l_{k+i,k} x_{k+i}
  C_t<T> xw[5];
#pragma unroll
  for (int i = 0; i < 5; i++) xw[i] = mk<T>(0, 0);
  T v[kRec];
  rec_get<T>(base + (long)(m - 1) * rs, nl, v);
  for (int row = m - 1; row >= 0; row--) {
    V* o = base + (long)row * rs;
    C_t<T> x = mk<T>(v[10], v[11]);
#pragma unroll
    for (int i = 0; i < 5; i++) x = cfms<T>(x, mk<T>(v[2 * i], v[2 * i + 1]), xw[i]);
    T last[kLanes<T>];
#pragma unroll
    for (int i = 0; i < kLanes<T>; i++) last[i] = v[kRec - kLanes<T> + i];
    if (row > 0) rec_get<T>(base + (long)(row - 1) * rs, nl, v);  // prefetch
#pragma unroll
    for (int i = 4; i > 0; i--) xw[i] = xw[i - 1];
    xw[0] = x;
    last[kLanes<T> - 2] = x.x;
    last[kLanes<T> - 1] = x.y;
    o[(kPlanes<T> - 1) * nl] = pack16(last);
  }
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
  const int ta = g.fa + 2 * (int)(l % g.la), tb = g.fb + 2 * (int)(l / g.la);
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

template <typename T, int D>
static void line_sweep_d(const LevelView<T>& L, int color, T* buf, cudaStream_t st) {
  const int pa = color & 1, pb = (color >> 1) & 1;
  const long nl = line_count(L.n, D, color);
  if (nl == 0) return;
  const long items = nl * L.n[D];
  const int m = 5 * L.n[D] - 4;
  dim3 g1((unsigned)((items + 255) / 256), L.nrhs);
  k_line_assemble<T, D><<<g1, 256, 0, st>>>(L, pa, pb, buf);
  dim3 g2((unsigned)((nl + 63) / 64), L.nrhs);
  k_line_solve<T><<<g2, 64, 0, st>>>(L.active, nl, m, buf);
  k_line_apply<T, D><<<g1, 256, 0, st>>>(L, pa, pb, buf);
}

// scratch: m * lines * kRec values of T (see line_scratch_elems)
template <typename T>
void launch_line_sweep(const LevelView<T>& L, int d, int color, C_t<T>* scratch, cudaStream_t st) {
  T* buf = reinterpret_cast<T*>(scratch);
  if (d == 0) line_sweep_d<T, 0>(L, color, buf, st);
  else if (d == 1) line_sweep_d<T, 1>(L, color, buf, st);
  else line_sweep_d<T, 2>(L, color, buf, st);
}

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

// fine indices and weights contributing to coarse transverse index Ce along e
template <typename T>
__device__ __forceinline__ int xfer_list(int Ce, int sce, int nfe, int nce, const T* xf, const T* xc,
                                         int (&idx)[4], T (&w)[4]) {
  int cnt = 0;
  // left: map(F) == Ce, weight 1 - wr
  if (Ce < nce) {
    const T x0 = xc[Ce], h = xc[Ce + 1] - xc[Ce];
    const int f0 = sce == 2 ? 2 * Ce : Ce;
    for (int t = 0; t < sce; t++) {
      const int F = f0 + t;
      if (F >= 1 && F < nfe) {
        idx[cnt] = F;
        w[cnt] = T(1) - (xf[F] - x0) / h;
        cnt++;
      }
    }
  }
  // right: map(F) == Ce-1, weight wr
  if (Ce >= 1) {
    const T x0 = xc[Ce - 1], h = xc[Ce] - xc[Ce - 1];
    const int f0 = sce == 2 ? 2 * (Ce - 1) : Ce - 1;
    for (int t = 0; t < sce; t++) {
      const int F = f0 + t;
      if (F >= 1 && F < nfe) {
        idx[cnt] = F;
        w[cnt] = (xf[F] - x0) / h;
        cnt++;
      }
    }
  }
  return cnt;
}

template <typename T, int C>
__device__ __forceinline__ C_t<T> restrict_comp(const LevelView<T>& F, const LevelView<T>& Cc,
                                                const int sc[3], const int Cn[3],
                                                const C_t<T>* rf, const Geo<T>& Gf,
                                                const Geo<T>& Gc) {
  constexpr int p = Cyc<C>::p, q = Cyc<C>::q;
  constexpr int t1 = p < q ? p : q, t2 = p < q ? q : p;
  int i1[4], i2[4];
  T w1[4], w2[4];
  const int n1c = xfer_list<T>(Cn[t1], sc[t1], F.n[t1], Cc.n[t1], Gf.x(t1), Gc.x(t1), i1, w1);
  const int n2c = xfer_list<T>(Cn[t2], sc[t2], F.n[t2], Cc.n[t2], Gf.x(t2), Gc.x(t2), i2, w2);
  T ar = 0, ai = 0;
  const int f0 = sc[C] == 2 ? 2 * Cn[C] : Cn[C];
  for (int t = 0; t < sc[C]; t++) {
    const int fc = f0 + t;
    if (fc >= F.n[C]) continue;
    for (int a = 0; a < n1c; a++)
      for (int b = 0; b < n2c; b++) {
        int P[3];
        P[C] = fc;
        P[t1] = i1[a];
        P[t2] = i2[b];
        const C_t<T> v = rf[(long)C * F.S + slot_id(F.n, P[0], P[1], P[2])];
        const T w = w1[a] * w2[b];
        ar += w * v.x;
        ai += w * v.y;
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
  const int n0 = Cc.n[0] + 1, n1 = Cc.n[1] + 1;
  const int Cn[3] = {(int)(s % n0), (int)((s / n0) % n1), (int)(s / ((long)n0 * n1))};
  const C_t<T>* rf = F.r + (long)rhs * 3 * F.S;
  C_t<T>* fc = Cc.f + (long)rhs * 3 * Cc.S;
  C_t<T>* uc = Cc.u + (long)rhs * 3 * Cc.S;
  const Geo<T> Gf{F.geo + (long)op_of(F, rhs) * F.gstride, F.gmax1};
  const Geo<T> Gc{Cc.geo + (long)op_of(Cc, rhs) * Cc.gstride, Cc.gmax1};
  fc[s] = restrict_comp<T, 0>(F, Cc, sc, Cn, rf, Gf, Gc);
  fc[Cc.S + s] = restrict_comp<T, 1>(F, Cc, sc, Cn, rf, Gf, Gc);
  fc[2 * Cc.S + s] = restrict_comp<T, 2>(F, Cc, sc, Cn, rf, Gf, Gc);
  uc[s] = mk<T>(0, 0);
  uc[Cc.S + s] = mk<T>(0, 0);
  uc[2 * Cc.S + s] = mk<T>(0, 0);
}

template <typename T>
void launch_restrict(const LevelView<T>& F, const LevelView<T>& Cc, const int sc[3], cudaStream_t st) {
  dim3 grid((unsigned)((Cc.S + 255) / 256), Cc.nrhs);
  k_restrict<T><<<grid, 256, 0, st>>>(F, Cc, sc[0], sc[1], sc[2]);
}

template <typename T, int C>
__device__ __forceinline__ void prolong_comp(const LevelView<T>& F, const LevelView<T>& Cc,
                                             const int sc[3], const int P[3], C_t<T>* uf,
                                             const C_t<T>* uc, const Geo<T>& Gf, const Geo<T>& Gc,
                                             long s) {
  constexpr int p = Cyc<C>::p, q = Cyc<C>::q;
  constexpr int t1 = p < q ? p : q, t2 = p < q ? q : p;
  if (!(P[C] < F.n[C] && P[t1] >= 1 && P[t1] < F.n[t1] && P[t2] >= 1 && P[t2] < F.n[t2])) return;
  int Cn[3];
#pragma unroll
  for (int e = 0; e < 3; e++) Cn[e] = sc[e] == 2 ? P[e] / 2 : P[e];
  const T* xf1 = Gf.x(t1);
  const T* xc1 = Gc.x(t1);
  const T* xf2 = Gf.x(t2);
  const T* xc2 = Gc.x(t2);
  const T wr1 = (xf1[P[t1]] - xc1[Cn[t1]]) / (xc1[Cn[t1] + 1] - xc1[Cn[t1]]);
  const T wr2 = (xf2[P[t2]] - xc2[Cn[t2]]) / (xc2[Cn[t2] + 1] - xc2[Cn[t2]]);
  const T wl1 = T(1) - wr1, wl2 = T(1) - wr2;
  int Q[3] = {Cn[0], Cn[1], Cn[2]};
  const long b = (long)C * Cc.S;
  const C_t<T> u00 = uc[b + slot_id(Cc.n, Q[0], Q[1], Q[2])];
  Q[t2] += 1;
  const C_t<T> u01 = uc[b + slot_id(Cc.n, Q[0], Q[1], Q[2])];
  Q[t2] -= 1;
  Q[t1] += 1;
  const C_t<T> u10 = uc[b + slot_id(Cc.n, Q[0], Q[1], Q[2])];
  Q[t2] += 1;
  const C_t<T> u11 = uc[b + slot_id(Cc.n, Q[0], Q[1], Q[2])];
  C_t<T> v = uf[(long)C * F.S + s];
  v.x += wl1 * (wl2 * u00.x + wr2 * u01.x) + wr1 * (wl2 * u10.x + wr2 * u11.x);
  v.y += wl1 * (wl2 * u00.y + wr2 * u01.y) + wr1 * (wl2 * u10.y + wr2 * u11.y);
  uf[(long)C * F.S + s] = v;
}

template <typename T>
__global__ void __launch_bounds__(256) k_prolong(LevelView<T> F, LevelView<T> Cc, int sc0, int sc1,
                                                 int sc2) {
  const int rhs = blockIdx.y;
  if (F.active && !F.active[rhs]) return;
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= F.S) return;
  const int sc[3] = {sc0, sc1, sc2};
  const int n0 = F.n[0] + 1, n1 = F.n[1] + 1;
  const int P[3] = {(int)(s % n0), (int)((s / n0) % n1), (int)(s / ((long)n0 * n1))};
  C_t<T>* uf = F.u + (long)rhs * 3 * F.S;
  const C_t<T>* uc = Cc.u + (long)rhs * 3 * Cc.S;
  const Geo<T> Gf{F.geo + (long)op_of(F, rhs) * F.gstride, F.gmax1};
  const Geo<T> Gc{Cc.geo + (long)op_of(Cc, rhs) * Cc.gstride, Cc.gmax1};
  prolong_comp<T, 0>(F, Cc, sc, P, uf, uc, Gf, Gc, s);
  prolong_comp<T, 1>(F, Cc, sc, P, uf, uc, Gf, Gc, s);
  prolong_comp<T, 2>(F, Cc, sc, P, uf, uc, Gf, Gc, s);
}

template <typename T>
void launch_prolong(const LevelView<T>& F, const LevelView<T>& Cc, const int sc[3], cudaStream_t st) {
  dim3 grid((unsigned)((F.S + 255) / 256), F.nrhs);
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
  const int i = (int)(id % nc0), j = (int)((id / nc0) % nc1), k = (int)(id / ((long)nc0 * nc1));
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
template void launch_residual<float, float>(const LevelView<float>&, C_t<float>*, double*, cudaStream_t);
template void launch_residual<double, double>(const LevelView<double>&, C_t<double>*, double*, cudaStream_t);
template void launch_residual<double, float>(const LevelView<double>&, C_t<float>*, double*, cudaStream_t);

}  // namespace emmi

// Shared device definitions for the GB300 multigrid curl-curl solver.
//
// Field layout (identical to the reference so the C ABI takes its buffers
// as they are): 3 components, each on (n1+1)(n2+1)(n3+1) slots, component-
// major, i fastest (src/gmg.c:1780; index id1..id3 in src/inject_extract.c:18).
// A batch of right-hand sides stores RHS after RHS: field[rhs][3][S].
// Cell arrays (volume-weighted conductivities and inverse permeability) are
// [rhs][4][n3][n2][n1] in the order sigma11, sigma22, sigma33, invmur.
// Per-RHS geometry is packed as 9 arrays of length nmax+1:
//   x1 x2 x3 | ds1 ds2 ds3 | d1 d2 d3     (gmg.c:26-29, generate_xs_dx :1672)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace emmi {

// ---------------------------------------------------------------- complex
template <typename T> struct cplx;
template <> struct cplx<float> { using type = float2; };
template <> struct cplx<double> { using type = double2; };
template <typename T> using C_t = typename cplx<T>::type;

template <typename T> __host__ __device__ __forceinline__ C_t<T> mk(T re, T im) {
  C_t<T> z; z.x = re; z.y = im; return z;
}
template <typename T> __device__ __forceinline__ C_t<T> cadd(C_t<T> a, C_t<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ C_t<T> csub(C_t<T> a, C_t<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ C_t<T> cmul(C_t<T> a, C_t<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T> __device__ __forceinline__ C_t<T> cscale(C_t<T> a, T s) { return mk<T>(a.x * s, a.y * s); }
// a - b*c
template <typename T> __device__ __forceinline__ C_t<T> cfms(C_t<T> a, C_t<T> b, C_t<T> c) {
  return mk<T>(a.x - (b.x * c.x - b.y * c.y), a.y - (b.x * c.y + b.y * c.x));
}
// a - s*b (s real)
template <typename T> __device__ __forceinline__ C_t<T> crfms(C_t<T> a, T s, C_t<T> b) {
  return mk<T>(a.x - s * b.x, a.y - s * b.y);
}
// 1/z by the scaled formula conj(z)/|z|^2 with a power-of-two prescale so
// |z|^2 neither overflows nor underflows (Smith-style range guard).
template <typename T> __device__ __forceinline__ C_t<T> crcp(C_t<T> z) {
  T m = fmax(fabs(z.x), fabs(z.y));
  int e;
  frexp(m, &e);
  T zx = ldexp(z.x, -e), zy = ldexp(z.y, -e);
  T inv = T(1) / (zx * zx + zy * zy);
  return mk<T>(ldexp(zx * inv, -e), ldexp(-zy * inv, -e));
}

// read-only (non-coherent) loads: the data a kernel only reads during its
// launch; lets loads move past the kernel's own stores
template <typename T> __device__ __forceinline__ T ldro(const T* p) { return __ldg(p); }

// Division by a divisor fixed for a launch, for dividends below 2^31, as a
// multiply-high, an add and a shift: with l = ceil(log2 d) and
// m = floor(2^32 (2^l - d) / d) + 1, u / d = (umulhi(u, m) + u) >> l
// (Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994).  Constants come from the host.
struct FastDiv {
  unsigned m, l;
};
inline FastDiv make_fastdiv(unsigned d) {
  unsigned l = 0;
  while ((1ull << l) < d) l++;
  FastDiv f;
  f.l = l;
  f.m = (unsigned)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
  return f;
}
__device__ __forceinline__ unsigned fdiv(unsigned u, const FastDiv& f) {
  return (__umulhi(u, f.m) + u) >> f.l;
}

// ---------------------------------------------------------------- views
// One multigrid level of a batch, in working precision T.
template <typename T> struct LevelView {
  int n[3];          // cells per direction
  int nrhs;
  long S;            // slots per component = (n1+1)(n2+1)(n3+1)
  long ncell;        // n1*n2*n3
  int gstride;       // per-RHS stride of geo (9*(gmax+1))
  int gmax1;         // gmax+1: length of each packed geometry array
  const T* geo;      // [nrhs][9][gmax+1]
  const T* cells;    // [nrhs][4][ncell], volume weighted
  C_t<T>* u;         // [nrhs][3][S]
  C_t<T>* f;
  C_t<T>* r;
  const T* wmu;      // [nrhs] omega*mu0 (the operator's mass term is -i wmu sigma)
  const int* active; // [nrhs] nonzero = work on this RHS (may be null)
  const int* op;     // [nrhs] operator (geo/cells) index of each RHS (null: identity)
  FastDiv d0, d1;    // division by n[0]+1 and n[1]+1 (set_slot_divs)
  // nonzero: every cell's volume-weighted inverse permeability is its volume
  // (the input invmur is exactly 1, as the front end writes it), so the
  // coefficients come from the spacings alone (edge_coef); set only for the
  // complex64 preconditioner operator
  int imu_vol = 0;
  // [op][3][gmax1]: weight wr of every fine node index along each axis for
  // the transfer to the next coarser level, (x_f[F] - x_c[c]) / (x_c[c+1] -
  // x_c[c]) with c the coarse interval of F (k_xfer_weights); null on the
  // coarsest level
  const T* xw = nullptr;
};

// the slot-decode divisors of a view, set on the host wherever a view is built
template <typename T> inline void set_slot_divs(LevelView<T>& V) {
  V.d0 = make_fastdiv((unsigned)(V.n[0] + 1));
  V.d1 = make_fastdiv((unsigned)(V.n[1] + 1));
}

template <typename T> __device__ __forceinline__ int op_of(const LevelView<T>& L, int rhs) {
  return L.op ? L.op[rhs] : rhs;
}

__host__ __device__ __forceinline__ long slot_id(const int n[3], int i, int j, int k) {
  return i + (long)(n[0] + 1) * (j + (long)(n[1] + 1) * k);
}
// 32-bit slot index (a level has fewer than 2^31 edge slots)
__host__ __device__ __forceinline__ int slot_id32(const int n[3], int i, int j, int k) {
  return i + (n[0] + 1) * (j + (n[1] + 1) * k);
}
__host__ __device__ __forceinline__ long cell_id(const int n[3], int i, int j, int k) {
  return i + (long)n[0] * (j + (long)n[1] * k);
}

// geometry accessors: G[0..2]=x, G[3..5]=ds, G[6..8]=d
template <typename T> struct Geo {
  const T* g;
  int len;
  __device__ __forceinline__ const T* x(int e) const { return g + e * len; }
  __device__ __forceinline__ const T* ds(int e) const { return g + (3 + e) * len; }
  __device__ __forceinline__ const T* d(int e) const { return g + (6 + e) * len; }
};

// ---------------------------------------------------------------- stencil
// Coefficients of the finite-integration curl-curl equation of the unknown
// E_C at node indices P (src/gmg.c:1365-1404 in residual form, the matrix
// rows of :199-318).  With p=(C+1)%3, q=(C+2)%3 and a,b,g the C-,p-,q-
// indices:
//   (A E)_C = (m1 T1/ds_p[b] - m2 T2/ds_p[b-1]) - (m3 T3/ds_q[g] - m4 T4/ds_q[g-1])
//             - i wmu sbar E_C
// expanded into one complex diagonal and 12 real neighbour coefficients in
// the fixed order
//   0 E_C(+p)  1 E_C(-p)  2 E_C(+q)  3 E_C(-q)
//   4 E_p(+C)  5 E_p(0)   6 E_p(+C,-p)  7 E_p(-p)
//   8 E_q(+C)  9 E_q(0)  10 E_q(+C,-q) 11 E_q(-q)
// Entries with the same two cells are formed with identical operand order in
// every row, so the assembled operator is exactly (bitwise) complex-symmetric.
struct NbrOff { int comp; int dc, dp, dq; };

template <int C> struct Cyc {
  static constexpr int p = (C + 1) % 3;
  static constexpr int q = (C + 2) % 3;
};

__host__ __device__ constexpr NbrOff nbr_off(int C, int k) {
  // (component, offset along C, along p, along q)
  return k == 0 ? NbrOff{C, 0, 1, 0}
       : k == 1 ? NbrOff{C, 0, -1, 0}
       : k == 2 ? NbrOff{C, 0, 0, 1}
       : k == 3 ? NbrOff{C, 0, 0, -1}
       : k == 4 ? NbrOff{(C + 1) % 3, 1, 0, 0}
       : k == 5 ? NbrOff{(C + 1) % 3, 0, 0, 0}
       : k == 6 ? NbrOff{(C + 1) % 3, 1, -1, 0}
       : k == 7 ? NbrOff{(C + 1) % 3, 0, -1, 0}
       : k == 8 ? NbrOff{(C + 2) % 3, 1, 0, 0}
       : k == 9 ? NbrOff{(C + 2) % 3, 0, 0, 0}
       : k == 10 ? NbrOff{(C + 2) % 3, 1, 0, -1}
       : NbrOff{(C + 2) % 3, 0, 0, -1};
}

template <typename T> struct EdgeCoef {
  T dre;   // real part of the diagonal (curl-curl)
  T dim;   // imaginary part of the diagonal (-wmu * sbar)
  T c[12];
};

// a / b: the hardware's fast single-precision division for the complex64
// operator (the preconditioner: 2 ulp are immaterial there), IEEE for FP64
__device__ __forceinline__ float qdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double qdiv(double a, double b) { return a / b; }

// P[3]: node indices of the edge; strides of the cell array; G geometry.
// W: the cell weights of the inverse permeability -- 0 read from the cells,
// 1 the cell volumes (LevelView::imu_vol), 2 chosen by imu_vol at run time
template <typename T, int C, int W = 2>
__device__ __forceinline__ void edge_coef(const int n[3], const int P[3], const T* __restrict__ sigC,
                                          const T* __restrict__ imu, const Geo<T>& G, T wmu,
                                          EdgeCoef<T>& e, int imu_vol = 0) {
  constexpr int p = Cyc<C>::p, q = Cyc<C>::q;
  const int a = P[C], b = P[p], g = P[q];
  // 32-bit cell offsets (a level has fewer than 2^31 cells)
  const int cs[3] = {1, n[0], n[0] * n[1]};
  const int c11 = a * cs[C] + b * cs[p] + g * cs[q];  // cell (p=b, q=g)
  const int c10 = c11 - cs[q];                         // (b, g-1)
  const int c01 = c11 - cs[p];                         // (b-1, g)
  const int c00 = c01 - cs[q];                         // (b-1, g-1)
  const T s = T(0.25) * (((ldro(sigC + c00) + ldro(sigC + c01)) + ldro(sigC + c10)) + ldro(sigC + c11));
  const T dc = ldro(G.ds(C) + a);
  const T dpp = ldro(G.ds(p) + b), dpm = ldro(G.ds(p) + b - 1);
  const T dqp = ldro(G.ds(q) + g), dqm = ldro(G.ds(q) + g - 1);
  e.dim = -wmu * s;
  if (W == 1 || (W == 2 && imu_vol)) {
    // cell weight = volume: with the four cells' volumes dc*dp*dq the face
    // averages give k_p+ = dc (dq+ + dq-) / (2 dp+) and so on, and the
    // mixed terms reduce to (dq+ + dq-) / 2 and (dp+ + dp-) / 2
    const T hq = T(0.5) * (dqp + dqm), hp = T(0.5) * (dpp + dpm);
    const T kpp = qdiv(dc * hq, dpp), kpm = qdiv(dc * hq, dpm);
    const T kqp = qdiv(dc * hp, dqp), kqm = qdiv(dc * hp, dqm);
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
    return;
  }
  const T i00 = ldro(imu + c00), i01 = ldro(imu + c01), i10 = ldro(imu + c10), i11 = ldro(imu + c11);
  const T m1 = T(0.5) * (i11 + i10);  // H_q face at p=b
  const T m2 = T(0.5) * (i01 + i00);  // H_q face at p=b-1
  const T m3 = T(0.5) * (i11 + i01);  // H_p face at q=g
  const T m4 = T(0.5) * (i10 + i00);  // H_p face at q=g-1
  const T kpp = qdiv(m1, dpp * dpp), kpm = qdiv(m2, dpm * dpm);
  const T kqp = qdiv(m3, dqp * dqp), kqm = qdiv(m4, dqm * dqm);
  e.dre = (kpp + kpm) + (kqp + kqm);
  e.c[0] = -kpp;
  e.c[1] = -kpm;
  e.c[2] = -kqp;
  e.c[3] = -kqm;
  const T xp = qdiv(m1, dc * dpp), xm = qdiv(m2, dc * dpm);
  const T yp = qdiv(m3, dc * dqp), ym = qdiv(m4, dc * dqm);
  e.c[4] = xp;
  e.c[5] = -xp;
  e.c[6] = -xm;
  e.c[7] = xm;
  e.c[8] = yp;
  e.c[9] = -yp;
  e.c[10] = -ym;
  e.c[11] = ym;
}

// slot offset of neighbour k of a component-C edge, in slot units, plus its
// component's base offset (comp*S); 32-bit: a level's 3 S edge slots fit in
// an int (emmi_solver_create refuses larger grids)
template <int C>
__device__ __forceinline__ long nbr_slot_delta(int k, const long ss[3], long S) {
  const NbrOff o = nbr_off(C, k);
  constexpr int p = Cyc<C>::p, q = Cyc<C>::q;
  return (long)o.comp * S + o.dc * ss[C] + o.dp * ss[p] + o.dq * ss[q];
}
template <int C>
__device__ __forceinline__ int nbr_delta32(int k, const int ss[3], int S) {
  const NbrOff o = nbr_off(C, k);
  constexpr int p = Cyc<C>::p, q = Cyc<C>::q;
  return o.comp * S + o.dc * ss[C] + o.dp * ss[p] + o.dq * ss[q];
}

// slot index -> node indices with 32-bit arithmetic (a level holds fewer
// than 2^31 slots per right-hand side): one division and one modulo fewer
// than the 64-bit decomposition, which dominated the index work
__device__ __forceinline__ void slot_nodes(long s, int n0, int n1, int P[3]) {
  const unsigned u = (unsigned)s, a = (unsigned)n0, b = (unsigned)n1;
  const unsigned t = u / a;
  P[0] = (int)(u - t * a);
  P[1] = (int)(t % b);
  P[2] = (int)(t / b);
}
// the same with the view's launch-invariant divisors (multiply-high)
template <typename T>
__device__ __forceinline__ void slot_nodes(long s, const LevelView<T>& L, int P[3]) {
  const unsigned u = (unsigned)s, a = (unsigned)(L.n[0] + 1), b = (unsigned)(L.n[1] + 1);
  const unsigned t = fdiv(u, L.d0);
  const unsigned k = fdiv(t, L.d1);
  P[0] = (int)(u - t * a);
  P[1] = (int)(t - k * b);
  P[2] = (int)k;
}

// (A u) of the edge equation of component C at slot s, and its coefficients
// (W: edge_coef's cell weights)
template <typename T, int C, int W = 2>
__device__ __forceinline__ C_t<T> apply_row(const LevelView<T>& L, const C_t<T>* __restrict__ u,
                                            const T* __restrict__ cells, const Geo<T>& G, T wmu,
                                            const int P[3], long s, const long ss[3],
                                            EdgeCoef<T>& e) {
  // u, cells and geometry are not written by any thread while a residual,
  // an assembly or a same-colour block sweep reads them: read-only loads.
  // Offsets within the RHS's field are 32-bit.
  edge_coef<T, C, W>(L.n, P, cells + (long)C * L.ncell, cells + 3 * L.ncell, G, wmu, e, L.imu_vol);
  const int si = (int)s, Si = (int)L.S;
  const int s3[3] = {1, (int)ss[1], (int)ss[2]};
  const C_t<T> uc = ldro(u + (C * Si + si));
  T ar = e.dre * uc.x - e.dim * uc.y;
  T ai = e.dre * uc.y + e.dim * uc.x;
#pragma unroll
  for (int k = 0; k < 12; k++) {
    const C_t<T> v = ldro(u + (si + nbr_delta32<C>(k, s3, Si)));
    ar += e.c[k] * v.x;
    ai += e.c[k] * v.y;
  }
  return mk<T>(ar, ai);
}

}  // namespace emmi

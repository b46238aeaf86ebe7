// Source injection, receiver extraction, volume interpolation and gradient
// accumulation on the device, batched over right-hand sides.
//
//   inject_source          src/inject_extract.c:26-120
//   inject_adj_source      src/inject_extract.c:124-314
//   extract_emf_data       src/inject_extract.c:317-474
//   extract_*_field        src/inject_extract.c:477-785
//   build_gradient         src/build_gradient.c:13-113 (+ the shot sum of
//                          src/fg_fwi.c:265-268 as a device reduction)
//
// The arithmetic follows the reference's operand types and order (float
// weights and volumes, double complex accumulation); this unit is compiled
// without FMA contraction so the injected right-hand sides and extracted
// samples reproduce the reference's values (tests/test_gpu_survey.py).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "emmi_solver_impl.cuh"

using namespace emmi;

namespace {

#define CK(x)                                                                     \
  do {                                                                            \
    cudaError_t e_ = (x);                                                         \
    if (e_ != cudaSuccess) {                                                      \
      set_err("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_));   \
      return EMMI_ECUDA;                                                          \
    }                                                                             \
  } while (0)

struct SGrid {
  const float* g;  // [9][gmax1]: x1 x2 x3 x1s x2s x3s d1 d2 d3
  int gmax1;
  int n[3];
  __device__ const float* ax(int e, int half) const { return g + (half ? 3 + e : e) * gmax1; }
  __device__ const float* dd(int e) const { return g + (6 + e) * gmax1; }
};

// find_index.c:9-30
__device__ int find_index_dev(int n, const float* x, float val) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi) / 2;
    if (x[mid] <= val) lo = mid;
    if (x[mid] > val) hi = mid;
    if (lo == hi || lo == hi - 1) break;
  }
  return lo;
}

struct Tri {
  int i[3];
  float w[3];
  float vol;
};

// trilinear stencil of a point on one staggered grid (inject_extract.c:57-65)
__device__ Tri trilin(const SGrid& G, int h0, int h1, int h2, float px, float py, float pz) {
  Tri t;
  const int half[3] = {h0, h1, h2};
  const float pv[3] = {px, py, pz};
  for (int e = 0; e < 3; e++) {
    const float* a = G.ax(e, half[e]);
    t.i[e] = find_index_dev(G.n[e] + 1, a, pv[e]);
    t.w[e] = (pv[e] - a[t.i[e]]) / (a[t.i[e] + 1] - a[t.i[e]]);
  }
  const float* a0 = G.ax(0, h0);
  const float* a1 = G.ax(1, h1);
  const float* a2 = G.ax(2, h2);
  t.vol = (a0[t.i[0] + 1] - a0[t.i[0]]) * (a1[t.i[1] + 1] - a1[t.i[1]]) * (a2[t.i[2] + 1] - a2[t.i[2]]);
  return t;
}

__device__ __forceinline__ long gslot(const int n[3], int c, int i, int j, int k) {
  const long S = (long)(n[0] + 1) * (n[1] + 1) * (n[2] + 1);
  return c * S + i + (long)(n[0] + 1) * (j + (long)(n[1] + 1) * k);
}

// complex double helpers with explicit operation order
struct zd {
  double re, im;
};
__device__ __forceinline__ zd zmul(zd a, zd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ zd zscale(zd a, double s) { return {a.re * s, a.im * s}; }
__device__ __forceinline__ zd zdiv_real(zd a, double s) { return {a.re / s, a.im / s}; }

// channel rotation into grid axes (inject_extract.c:40-55): adds amp*dir
__device__ void rotate_in(int chx, float phi, float theta, zd amp, zd F[3]) {
  const double cp = cos((double)phi), sp = sin((double)phi);
  const double ct = cos((double)theta), st = sin((double)theta);
  if (chx == 0) {
    F[0] = {F[0].re + amp.re * cp, F[0].im + amp.im * cp};
    F[1] = {F[1].re + amp.re * sp, F[1].im + amp.im * sp};
  } else if (chx == 1) {
    zd a = zscale(zscale(amp, sp), ct);
    F[0] = {F[0].re - a.re, F[0].im - a.im};
    a = zscale(zscale(amp, cp), ct);
    F[1] = {F[1].re + a.re, F[1].im + a.im};
    a = zscale(amp, st);
    F[2] = {F[2].re + a.re, F[2].im + a.im};
  } else if (chx == 2) {
    zd a = zscale(zscale(amp, sp), st);
    F[0] = {F[0].re + a.re, F[0].im + a.im};
    a = zscale(zscale(amp, cp), st);
    F[1] = {F[1].re - a.re, F[1].im - a.im};
    a = zscale(amp, ct);
    F[2] = {F[2].re + a.re, F[2].im + a.im};
  }
}

// b[corner] += val * weights, corners in the reference's order (:68-75)
__device__ void scatter8(const int n[3], int c, const Tri& t, zd v, double2* y) {
  const double w1 = t.w[0], w2 = t.w[1], w3 = t.w[2];
  const int i = t.i[0], j = t.i[1], k = t.i[2];
  auto add = [&](int a, int b, int cc, double f1, double f2, double f3) {
    const long s = gslot(n, c, a, b, cc);
    zd q = zscale(zscale(zscale(v, f1), f2), f3);
    y[s].x += q.re;
    y[s].y += q.im;
  };
  add(i, j, k, 1. - w1, 1. - w2, 1. - w3);
  add(i + 1, j, k, w1, 1. - w2, 1. - w3);
  add(i, j + 1, k, 1. - w1, w2, 1. - w3);
  add(i + 1, j + 1, k, w1, w2, 1. - w3);
  add(i, j, k + 1, 1. - w1, 1. - w2, w3);
  add(i + 1, j, k + 1, w1, 1. - w2, w3);
  add(i, j + 1, k + 1, 1. - w1, w2, w3);
  add(i + 1, j + 1, k + 1, w1, w2, w3);
}

struct ChanList {
  int n;
  int ch[6];
};

// one thread per RHS over its nsrc sources in order; b zeroed beforehand
__global__ void k_inject_sources(SGrid G0, int gstride, const int* __restrict__ op,
                                 const float* __restrict__ src, int nsrc,
                                 const float* __restrict__ omega, ChanList chs,
                                 double2* __restrict__ b, int nrhs) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrhs) return;
  SGrid G = G0;
  G.g = G0.g + (long)op[r] * gstride;
  const long S = (long)(G.n[0] + 1) * (G.n[1] + 1) * (G.n[2] + 1);
  double2* y = b + (long)r * 3 * S;
  // I*omega (complex float) * mu0 * F / vol (inject_extract.c:66)
  const zd iw = {0.0 * kMu0, (double)omega[r] * kMu0};
  for (int is = 0; is < nsrc; is++) {
    const float* sr = src + 5 * ((long)r * nsrc + is);
    zd F[3] = {{0, 0}, {0, 0}, {0, 0}};
    const zd one = {1.0, 0.0};  // src_fd = 1 (inject_extract.c:33)
    for (int ic = 0; ic < chs.n; ic++)
      if (chs.ch[ic] <= 2) rotate_in(chs.ch[ic], sr[3], sr[4], one, F);
    for (int c = 0; c < 3; c++) {
      const Tri t = trilin(G, c == 0, c == 1, c == 2, sr[0], sr[1], sr[2]);
      const zd v = zdiv_real(zmul(iw, F[c]), (double)t.vol);
      scatter8(G.n, c, t, v, y);
    }
  }
}

// one adjoint-source term: a trilinear stencil on one staggered grid and
// the value it spreads
struct AdjTerm {
  Tri t;
  double2 v;
};

// adjoint-source terms (inject_extract.c:124-301), one thread per (RHS,
// receiver): for each component c the electric term i*omega*mu0*F[c]/vol
// on E's grid (terms 0..2) and the magnetic term M[c]/vol on H's grid
// (terms 3..5), F and M the receiver-frame residuals rotated to the grid
__global__ void k_adjoint_terms(SGrid G0, int gstride, const int* __restrict__ op,
                                const float* __restrict__ rec, int nrec,
                                const float* __restrict__ omega, ChanList chs,
                                const float2* __restrict__ dres, AdjTerm* __restrict__ terms,
                                int nrhs) {
  const long id = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (id >= (long)nrhs * nrec) return;
  const int r = (int)(id / nrec), ir = (int)(id % nrec);
  SGrid G = G0;
  G.g = G0.g + (long)op[r] * gstride;
  const zd iw = {0.0 * kMu0, (double)omega[r] * kMu0};
  const float* p = rec + ((long)r * nrec + ir) * 5;
  zd F[3] = {{0, 0}, {0, 0}, {0, 0}}, M[3] = {{0, 0}, {0, 0}, {0, 0}};
  for (int ic = 0; ic < chs.n; ic++) {
    const float2 d = dres[((long)r * chs.n + ic) * nrec + ir];
    if (chs.ch[ic] <= 2) rotate_in(chs.ch[ic], p[3], p[4], zd{(double)d.x, (double)d.y}, F);
  }
  for (int ic = 0; ic < chs.n; ic++) {
    const float2 d = dres[((long)r * chs.n + ic) * nrec + ir];
    if (chs.ch[ic] >= 3) rotate_in(chs.ch[ic] - 3, p[3], p[4], zd{(double)d.x, (double)d.y}, M);
  }
  AdjTerm* out = terms + id * 6;
  for (int c = 0; c < 3; c++) {
    const Tri t = trilin(G, c == 0, c == 1, c == 2, p[0], p[1], p[2]);
    const zd v = zdiv_real(zmul(iw, F[c]), (double)t.vol);
    out[c] = AdjTerm{t, make_double2(v.re, v.im)};
  }
  for (int c = 0; c < 3; c++) {
    const Tri t = trilin(G, c != 0, c != 1, c != 2, p[0], p[1], p[2]);
    const zd v = zdiv_real(M[c], (double)t.vol);
    out[3 + c] = AdjTerm{t, make_double2(v.re, v.im)};
  }
}

// the adjoint-source terms spread in receiver order, one thread per (RHS,
// field, component): the slots of different components are disjoint, so
// every slot receives its additions in the reference's order; b and m
// zeroed beforehand
__global__ void k_adjoint_scatter(SGrid G0, const AdjTerm* __restrict__ terms, int nrec,
                                  double2* __restrict__ b, double2* __restrict__ m, int nrhs) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= nrhs * 6) return;
  const int r = id / 6, q = id % 6, c = q % 3;
  const long S = (long)(G0.n[0] + 1) * (G0.n[1] + 1) * (G0.n[2] + 1);
  double2* y = (q < 3 ? b : m) + (long)r * 3 * S;
  for (int ir = 0; ir < nrec; ir++) {
    const AdjTerm a = terms[((long)r * nrec + ir) * 6 + q];
    scatter8(G0.n, c, a.t, zd{a.v.x, a.v.y}, y);
  }
}

// b += curl M with the node spacings d1,d2,d3 (inject_extract.c:303-312)
__global__ void k_curl_m(SGrid G0, int gstride, const int* __restrict__ op,
                         const double2* __restrict__ m, double2* __restrict__ b) {
  const int r = blockIdx.y;
  SGrid G = G0;
  G.g = G0.g + (long)op[r] * gstride;
  const int n1 = G.n[0], n2 = G.n[1], n3 = G.n[2];
  const long cnt = (long)n1 * n2 * n3;
  const long id = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (id >= cnt) return;
  const int i = 1 + (int)(id % n1), j = 1 + (int)((id / n1) % n2), k = 1 + (int)(id / ((long)n1 * n2));
  const long S = (long)(n1 + 1) * (n2 + 1) * (n3 + 1);
  const double2* x = m + (long)r * 3 * S;
  double2* y = b + (long)r * 3 * S;
  const float d1 = G.dd(0)[i], d2 = G.dd(1)[j], d3 = G.dd(2)[k];
  auto X = [&](int c, int a, int bb, int cc) { return x[gslot(G.n, c, a, bb, cc)]; };
  auto term = [](double2 a, double2 b2, float d) {
    return make_double2((a.x - b2.x) / (double)d, (a.y - b2.y) / (double)d);
  };
  double2 t1 = term(X(2, i, j, k), X(2, i, j - 1, k), d2), t2 = term(X(1, i, j, k), X(1, i, j, k - 1), d3);
  long s = gslot(G.n, 0, i, j, k);
  y[s].x += t1.x - t2.x;
  y[s].y += t1.y - t2.y;
  t1 = term(X(0, i, j, k), X(0, i, j, k - 1), d3);
  t2 = term(X(2, i, j, k), X(2, i - 1, j, k), d1);
  s = gslot(G.n, 1, i, j, k);
  y[s].x += t1.x - t2.x;
  y[s].y += t1.y - t2.y;
  t1 = term(X(1, i, j, k), X(1, i - 1, j, k), d1);
  t2 = term(X(0, i, j, k), X(0, i, j - 1, k), d2);
  s = gslot(G.n, 2, i, j, k);
  y[s].x += t1.x - t2.x;
  y[s].y += t1.y - t2.y;
}

// trilinear gather (inject_extract.c:339-346); sig (float cells) weights
// each corner by the cell value at the same indices (the Jz path)
__device__ zd gather8(const int n[3], int c, const Tri& t, const double2* y, const float* sig) {
  const double w1 = t.w[0], w2 = t.w[1], w3 = t.w[2];
  const int i = t.i[0], j = t.i[1], k = t.i[2];
  zd F = {0, 0};
  auto add = [&](int a, int b, int cc, double f1, double f2, double f3) {
    const double2 v = y[gslot(n, c, a, b, cc)];
    zd q = {v.x, v.y};
    if (sig) q = zscale(q, (double)sig[a + (long)n[0] * (b + (long)n[1] * cc)]);
    q = zscale(zscale(zscale(q, f1), f2), f3);
    F.re += q.re;
    F.im += q.im;
  };
  add(i, j, k, 1. - w1, 1. - w2, 1. - w3);
  add(i + 1, j, k, w1, 1. - w2, 1. - w3);
  add(i, j + 1, k, 1. - w1, w2, 1. - w3);
  add(i + 1, j + 1, k, w1, w2, 1. - w3);
  add(i, j, k + 1, 1. - w1, 1. - w2, w3);
  add(i + 1, j, k + 1, w1, 1. - w2, w3);
  add(i, j + 1, k + 1, 1. - w1, w2, w3);
  add(i + 1, j + 1, k + 1, w1, w2, w3);
  return F;
}

// receiver-frame rotation (inject_extract.c:391-399)
__device__ zd rotate_out(int chx, float phi, float theta, const zd F[3]) {
  const double cp = cos((double)phi), sp = sin((double)phi);
  const double ct = cos((double)theta), st = sin((double)theta);
  if (chx == 0) return {cp * F[0].re + sp * F[1].re, cp * F[0].im + sp * F[1].im};
  if (chx == 1) {
    const double a = -sp * ct, b = cp * ct;
    return {a * F[0].re + b * F[1].re - st * F[2].re, a * F[0].im + b * F[1].im - st * F[2].im};
  }
  const double a = sp * st, b = cp * st;
  return {a * F[0].re - b * F[1].re + ct * F[2].re, a * F[0].im - b * F[1].im + ct * F[2].im};
}

// one thread per (RHS, receiver)
__global__ void k_extract_receivers(SGrid G0, int gstride, const int* __restrict__ op,
                                    const float* __restrict__ rec, int nrec, ChanList chs,
                                    const double2* __restrict__ x, const double2* __restrict__ h,
                                    const float* __restrict__ raw_cells,
                                    const float* __restrict__ rho_water, float2* __restrict__ dcal,
                                    int nrhs) {
  const long id = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (id >= (long)nrhs * nrec) return;
  const int r = (int)(id / nrec), ir = (int)(id % nrec);
  const int o = op[r];
  SGrid G = G0;
  G.g = G0.g + (long)o * gstride;
  const long S = (long)(G.n[0] + 1) * (G.n[1] + 1) * (G.n[2] + 1);
  const long nc = (long)G.n[0] * G.n[1] * G.n[2];
  const double2* xe = x + (long)r * 3 * S;
  const double2* xh = h + (long)r * 3 * S;
  const float* sig33 = raw_cells + ((long)o * 4 + 2) * nc;
  const float* p = rec + ((long)r * nrec + ir) * 5;
  zd E[3], H[3];
  for (int c = 0; c < 3; c++) {
    const Tri t = trilin(G, c == 0, c == 1, c == 2, p[0], p[1], p[2]);
    E[c] = gather8(G.n, c, t, xe, c == 2 ? sig33 : nullptr);
  }
  E[2] = zscale(E[2], (double)rho_water[o]);  // Jz -> Ez (inject_extract.c:386)
  for (int c = 0; c < 3; c++) {
    const Tri t = trilin(G, c != 0, c != 1, c != 2, p[0], p[1], p[2]);
    H[c] = gather8(G.n, c, t, xh, nullptr);
  }
  for (int ic = 0; ic < chs.n; ic++) {
    const int ch = chs.ch[ic];
    const zd v = ch <= 2 ? rotate_out(ch, p[3], p[4], E) : rotate_out(ch - 3, p[3], p[4], H);
    dcal[((long)r * chs.n + ic) * nrec + ir] = make_float2((float)v.re, (float)v.im);
  }
}

// interpolation to input-model cell centres for one RHS
// (inject_extract.c:477-635 for E, 638-785 for H); component c of the cell
// id goes to out[c * cstride + id]
__global__ void k_extract_volume(SGrid G, int which, int nx, int ny, int nz, float ox, float oy,
                                 float oz, float dx, float dy, float dz,
                                 const float* __restrict__ rho33, const float* __restrict__ sig33,
                                 const double2* __restrict__ fld, float2* __restrict__ out,
                                 long cstride) {
  const long nxyz = (long)nx * ny * nz;
  const long id = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (id >= nxyz) return;
  const int i = (int)(id % nx), j = (int)((id / nx) % ny), k = (int)(id / ((long)nx * ny));
  const float xc[3] = {(float)(ox + (i + 0.5) * dx), (float)(oy + (j + 0.5) * dy),
                       (float)(oz + (k + 0.5) * dz)};
  int idx[3][2];
  float w[3][2];
  for (int e = 0; e < 3; e++)
    for (int hf = 0; hf < 2; hf++) {
      const float* a = G.ax(e, hf);
      const int ii = find_index_dev(G.n[e] + 1, a, xc[e]);
      idx[e][hf] = ii;
      w[e][hf] = (xc[e] - a[ii]) / (a[ii + 1] - a[ii]);
    }
  for (int c = 0; c < 3; c++) {
    // E_c uses the staggered axis along c; H_c the staggered axes across c
    Tri t;
    for (int e = 0; e < 3; e++) {
      const int hf = which == 0 ? (e == c) : (e != c);
      t.i[e] = idx[e][hf];
      t.w[e] = w[e][hf];
    }
    zd s;
    if (which == 0 && c == 2) {
      // Ez through Jz with the 4-cell-averaged sigma33 (:598-617)
      const int ii = t.i[0], jj = t.i[1], kk = t.i[2];
      const float wx = t.w[0], wy = t.w[1], wz = t.w[2];
      const int n1 = G.n[0], n2 = G.n[1];
      auto S33 = [&](int a, int b, int cc) { return sig33[a + (long)n1 * (b + (long)n2 * cc)]; };
      s = {0, 0};
      for (int dk = 0; dk < 2; dk++)
        for (int dj = 0; dj < 2; dj++)
          for (int di = 0; di < 2; di++) {
            const int a = ii + di, b = jj + dj, cc = kk + dk;
            const float sg = 0.25 * (S33(a, b, cc) + S33(a, b - 1, cc) + S33(a - 1, b, cc) +
                                     S33(a - 1, b - 1, cc));
            const double fx = di ? (double)wx : (1. - wx), fy = dj ? (double)wy : (1. - wy),
                         fz = dk ? (double)wz : (1. - wz);
            const double2 v = fld[gslot(G.n, 2, a, b, cc)];
            zd q = zscale(zd{v.x, v.y}, (double)sg);
            q = zscale(zscale(zscale(q, fx), fy), fz);
            s.re += q.re;
            s.im += q.im;
          }
      s = zscale(s, (double)rho33[id]);
    } else {
      s = gather8(G.n, c, t, fld, nullptr);
    }
    out[c * cstride + id] = make_float2((float)s.re, (float)s.im);
  }
}

// gradient w.r.t. ln(rho) summed over shots; mute[shot][cell] != 0 zeroes
// the shot's contribution (bathymetry, source and receiver boxes)
__global__ void k_gradient(int nxyz, int nshot, int nfreq, int npar, const int* __restrict__ idxpar,
                           int preco, float s, const float2* __restrict__ E1f,
                           const float2* __restrict__ E2f, const float2* __restrict__ E3f,
                           const float2* __restrict__ E1a, const float2* __restrict__ E2a,
                           const float2* __restrict__ E3a, const float* __restrict__ rho11,
                           const float* __restrict__ rho33, const unsigned char* __restrict__ mute,
                           const unsigned char* __restrict__ bmute, float* __restrict__ grad,
                           float* __restrict__ phess) {
  const long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= nxyz) return;
  for (int kp = 0; kp < npar; kp++) {
    float gsum = 0.f, hsum = 0.f;
    for (int sh = 0; sh < nshot; sh++) {
      float g = 0.f;
      for (int f = 0; f < nfreq; f++) {
        const long o = ((long)sh * nfreq + f) * nxyz + c;
        if (idxpar[kp] == 1) {
          float2 a = E1f[o], b = E1a[o];
          g += a.x * b.x - a.y * b.y;
          a = E2f[o];
          b = E2a[o];
          g += a.x * b.x - a.y * b.y;
        }
        if (idxpar[kp] == 2) {
          const float2 a = E3f[o], b = E3a[o];
          g += a.x * b.x - a.y * b.y;
        }
      }
      if (idxpar[kp] == 1) g *= s / rho11[c];
      if (idxpar[kp] == 2) g *= s / rho33[c];
      if (bmute[c]) g = 0.f;
      if (mute[(long)sh * nxyz + c]) g = 0.f;
      gsum += g;
      if (preco == 1) {
        float hh = 0.f;
        for (int f = 0; f < nfreq; f++) {
          const long o = ((long)sh * nfreq + f) * nxyz + c;
          auto ab2 = [](float2 z) {
            const double a = hypot((double)z.x, (double)z.y);
            return a * a;
          };
          if (idxpar[kp] == 1) {
            hh = (float)((double)hh + ab2(E1f[o]));
            hh = (float)((double)hh + ab2(E2f[o]));
          }
          if (idxpar[kp] == 2) hh = (float)((double)hh + ab2(E3f[o]));
        }
        if (idxpar[kp] == 1) hh *= s / rho11[c];
        if (idxpar[kp] == 2) hh *= s / rho33[c];
        hsum += hh;
      }
    }
    grad[(long)kp * nxyz + c] = gsum;
    if (preco == 1 && phess) phess[(long)kp * nxyz + c] = hsum;
  }
}

// data misfit and adjoint sources (fg_fwi.c:208-226, in the arithmetic of
// the host library's eh_misfit), one block per shot.  Per datum (channel c,
// frequency f, receiver ir < nrec_shot) farther than skin[f] from the
// source: r = (dobs - dcal) / delta, rmse = |r|, adjoint source
// conj(r / delta), and term = |r|^2 in double: the reference's r * conj(r)
// multiplies by the double-complex conj, so each term is a double and the
// float cost advances by a double addition rounded to float.  The shot's
// cost, 0.5 * the sum in the reference's loop order, by one thread.  Per-shot arrays
// (dobs, delta, rmse, dsyn, term) are [nshot][nch][nfreq][nrec]; per-RHS
// arrays (dcal, dres) [nshot * nfreq][nch][nrec], src [nshot * nfreq][5],
// rec [nshot * nfreq][nrec][5]
__global__ void k_misfit(int nch, int nfreq, int nrec, const int* __restrict__ nrec_shot,
                         const float* __restrict__ skin, const float* __restrict__ src,
                         const float* __restrict__ rec, const float2* __restrict__ dobs,
                         const float* __restrict__ delta, const float2* __restrict__ dcal,
                         float2* __restrict__ dres, float* __restrict__ rmse,
                         float2* __restrict__ dsyn, double* __restrict__ term,
                         float* __restrict__ fcost) {
  const int sh = blockIdx.x;
  const int nr = nrec_shot[sh];
  const long nd = (long)nch * nfreq * nrec;
  for (long i = threadIdx.x; i < nd; i += blockDim.x) {
    const int ir = (int)(i % nrec), f = (int)((i / nrec) % nfreq), c = (int)(i / ((long)nrec * nfreq));
    const long q = (long)sh * nd + i;
    const long rr = (long)sh * nfreq + f;
    const long k = (rr * nch + c) * nrec + ir;
    const float2 dc = dcal[k];
    float2 out = make_float2(0.f, 0.f);
    float rm = 0.f;
    double t = 0.;
    if (ir < nr) {
      const float* p = rec + (rr * nrec + ir) * 5;
      const float* s0 = src + rr * 5;
      const float ox = __fsub_rn(p[0], s0[0]), oy = __fsub_rn(p[1], s0[1]);
      const float r2 = __fadd_rn(__fmul_rn(ox, ox), __fmul_rn(oy, oy));
      if (sqrt((double)r2) > (double)skin[f]) {
        const float dl = delta[q];
        const float2 ob = dobs[q];
        float re = __fdiv_rn(__fsub_rn(ob.x, dc.x), dl);
        float im = __fdiv_rn(__fsub_rn(ob.y, dc.y), dl);
        rm = (float)sqrt(__dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im)));
        t = __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im));
        re = __fdiv_rn(re, dl);
        im = __fdiv_rn(im, dl);
        out = make_float2(re, -im);
      }
    }
    dres[k] = out;
    rmse[q] = rm;
    term[q] = t;
    dsyn[q] = dc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float acc = 0.f;
    for (long i = 0; i < nd; i++) acc = (float)__dadd_rn((double)acc, term[(long)sh * nd + i]);
    fcost[sh] = __fmul_rn(acc, 0.5f);
  }
}

inline unsigned nblk(long n, int bs = 256) { return (unsigned)std::max<long>(1, (n + bs - 1) / bs); }

// gradient masks (build_gradient.c:50-111, with the reference's float-to-int
// truncation): bm[cell] = 1 at and above the sea floor plus one cell;
// mm[shot][cell] = 1 in the boxes of half-width dsmute around the shot's
// source and drmute around each of its receivers.  src: [nshot] points,
// rec: [nshot][nrec] points, stride floats apart (x, y, z first);
// nrec_shot (optional): receivers of each shot
void gradient_masks(int nx, int ny, int nz, const float o[3], const float d[3], const float* bathy,
                    int nshot, const float* src, float dsmute, int nrec, const int* nrec_shot,
                    const float* rec, float drmute, int stride, std::vector<unsigned char>& bm,
                    std::vector<unsigned char>& mm) {
  const long nxyz = (long)nx * ny * nz;
  bm.assign(nxyz, 0);
  mm.assign((size_t)nshot * nxyz, 0);
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++)
        if (o[2] + (k + 0.5) * d[2] <= bathy[i + (long)nx * j] + d[2])
          bm[i + (long)nx * (j + (long)ny * k)] = 1;
  const int nn[3] = {nx, ny, nz};
  auto paint = [&](int sh, const float* p, float rad) {
    int lo[3], hi[3];
    for (int e = 0; e < 3; e++) {
      lo[e] = (int)((p[e] - rad - o[e]) / d[e]);
      hi[e] = (int)((p[e] + rad - o[e]) / d[e]);
      lo[e] = std::min(std::max(lo[e], 0), nn[e] - 1);
      hi[e] = std::min(std::max(hi[e], 0), nn[e] - 1);
    }
    for (int k = lo[2]; k <= hi[2]; k++)
      for (int j = lo[1]; j <= hi[1]; j++)
        for (int i = lo[0]; i <= hi[0]; i++)
          mm[(size_t)sh * nxyz + i + (long)nx * (j + (long)ny * k)] = 1;
  };
  for (int sh = 0; sh < nshot; sh++) {
    paint(sh, src + (long)stride * sh, dsmute);
    const int nr = nrec_shot ? nrec_shot[sh] : nrec;
    for (int ir = 0; ir < nr; ir++) paint(sh, rec + (long)stride * ((long)sh * nrec + ir), drmute);
  }
}

ChanList make_chans(int n, const int* ch) {
  ChanList c;
  c.n = std::min(n, 6);
  for (int i = 0; i < c.n; i++) c.ch[i] = ch[i];
  return c;
}

SGrid sgrid_of(const emmi_solver* s) {
  SGrid G;
  G.g = s->sgeo;
  G.gmax1 = s->gmax1;
  for (int e = 0; e < 3; e++) G.n[e] = s->n[e];
  return G;
}

}  // namespace

extern "C" {

int emmi_inject_sources_multi_dev(emmi_solver* s, const float* src_dev, int nsrc, int nch,
                                  const int* ch, double* b_dev) {
  if (!s || !src_dev || !b_dev || nch < 1 || nch > 6 || !ch || nsrc < 0) {
    set_err("emmi_inject_sources_dev: bad argument");
    return EMMI_EINVAL;
  }
  const long S = s->hier[0][0].S;
  CK(cudaMemsetAsync(b_dev, 0, (size_t)3 * S * s->nrhs * sizeof(double2), s->st));
  k_inject_sources<<<nblk(s->nrhs, 64), 64, 0, s->st>>>(sgrid_of(s), s->gstride, s->d_op, src_dev,
                                                        nsrc, s->d_omega, make_chans(nch, ch),
                                                        (double2*)b_dev, s->nrhs);
  CK(cudaGetLastError());
  return EMMI_OK;
}

int emmi_inject_sources_dev(emmi_solver* s, const float* src_dev, int nch, const int* ch,
                            double* b_dev) {
  return emmi_inject_sources_multi_dev(s, src_dev, 1, nch, ch, b_dev);
}

int emmi_inject_adjoint_dev(emmi_solver* s, const float* rec_dev, int nrec, int nch, const int* ch,
                            const float* dres_dev, double* b_dev, double* m_dev) {
  if (!s || !rec_dev || !b_dev || !m_dev || !dres_dev || nch < 1 || nch > 6 || !ch || nrec < 0) {
    set_err("emmi_inject_adjoint_dev: bad argument");
    return EMMI_EINVAL;
  }
  const long S = s->hier[0][0].S;
  CK(cudaMemsetAsync(b_dev, 0, (size_t)3 * S * s->nrhs * sizeof(double2), s->st));
  CK(cudaMemsetAsync(m_dev, 0, (size_t)3 * S * s->nrhs * sizeof(double2), s->st));
  if (nrec > 0) {
    AdjTerm* terms = nullptr;
    CK(cudaMallocAsync((void**)&terms, (size_t)s->nrhs * nrec * 6 * sizeof(AdjTerm), s->st));
    k_adjoint_terms<<<nblk((long)s->nrhs * nrec, 128), 128, 0, s->st>>>(
        sgrid_of(s), s->gstride, s->d_op, rec_dev, nrec, s->d_omega, make_chans(nch, ch),
        (const float2*)dres_dev, terms, s->nrhs);
    k_adjoint_scatter<<<nblk((long)s->nrhs * 6, 64), 64, 0, s->st>>>(
        sgrid_of(s), terms, nrec, (double2*)b_dev, (double2*)m_dev, s->nrhs);
    CK(cudaFreeAsync(terms, s->st));
  }
  dim3 g(nblk((long)s->n[0] * s->n[1] * s->n[2]), s->nrhs);
  k_curl_m<<<g, 256, 0, s->st>>>(sgrid_of(s), s->gstride, s->d_op, (const double2*)m_dev,
                                 (double2*)b_dev);
  CK(cudaGetLastError());
  return EMMI_OK;
}

int emmi_extract_receivers_dev(emmi_solver* s, const float* rec_dev, int nrec, int nch,
                               const int* ch, const double* e_dev, const double* h_dev,
                               float* dcal_dev) {
  if (!s || !rec_dev || !e_dev || !h_dev || !dcal_dev || nch < 1 || nch > 6 || !ch) {
    set_err("emmi_extract_receivers_dev: bad argument");
    return EMMI_EINVAL;
  }
  if (nrec == 0) return EMMI_OK;
  k_extract_receivers<<<nblk((long)s->nrhs * nrec, 128), 128, 0, s->st>>>(
      sgrid_of(s), s->gstride, s->d_op, rec_dev, nrec, make_chans(nch, ch),
      (const double2*)e_dev, (const double2*)h_dev, s->raw_cells, s->d_rho_water,
      (float2*)dcal_dev, s->nrhs);
  CK(cudaGetLastError());
  return EMMI_OK;
}

// internal: solve with b already in the solver's input buffer
int emmi_solver_solve_resident(emmi_solver* s, double* x_dev, double* h_dev,
                               emmi_rhs_stats* stats);

int emmi_modelling_batch(emmi_solver* s, const emmi_survey* sv, float* dcal,
                         emmi_rhs_stats* stats, size_t* h2d, size_t* d2h) {
  if (!s || !sv || !dcal || !sv->src || (sv->nrec > 0 && !sv->rec)) {
    set_err("emmi_modelling_batch: bad argument");
    return EMMI_EINVAL;
  }
  const size_t srcb = (size_t)s->nrhs * 5 * sizeof(float);
  const size_t recb = (size_t)s->nrhs * sv->nrec * 5 * sizeof(float);
  const size_t outb = (size_t)s->nrhs * sv->nrec_ch * sv->nrec * 2 * sizeof(float);
  float *dsrc = nullptr, *drec = nullptr, *dout = nullptr;
  CK(cudaMallocAsync((void**)&dsrc, srcb + 16, s->st));
  CK(cudaMallocAsync((void**)&drec, recb + 16, s->st));
  CK(cudaMallocAsync((void**)&dout, outb + 16, s->st));
  CK(cudaMemcpyAsync(dsrc, sv->src, srcb, cudaMemcpyHostToDevice, s->st));
  if (recb) CK(cudaMemcpyAsync(drec, sv->rec, recb, cudaMemcpyHostToDevice, s->st));
  // b is injected straight into the solver's input buffer (u64[0])
  int rc = emmi_inject_sources_dev(s, dsrc, sv->nsrc_ch, sv->src_ch, (double*)s->u64[0]);
  if (rc == EMMI_OK) rc = emmi_solver_solve_resident(s, nullptr, nullptr, stats);
  if (rc == EMMI_OK && sv->nrec > 0)
    rc = emmi_extract_receivers_dev(s, drec, sv->nrec, sv->nrec_ch, sv->rec_ch,
                                    (const double*)s->u64[0], (const double*)s->f64[0], dout);
  if (rc == EMMI_OK) {
    cudaMemcpyAsync(dcal, dout, outb, cudaMemcpyDeviceToHost, s->st);
    cudaError_t e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) {
      set_err("emmi_modelling_batch: %s", cudaGetErrorString(e));
      rc = EMMI_ECUDA;
    }
  }
  cudaFreeAsync(dsrc, s->st);
  cudaFreeAsync(drec, s->st);
  cudaFreeAsync(dout, s->st);
  cudaStreamSynchronize(s->st);
  if (h2d) *h2d = srcb + recb;
  if (d2h) *d2h = outb;
  return rc;
}

int emmi_extract_volume(emmi_solver* s, int rhs, int which, int nx, int ny, int nz,
                        const float o[3], const float d[3], const float* rho33,
                        const double* field, float* out) {
  if (!s || rhs < 0 || rhs >= s->nrhs || !field || !out || (which == 0 && !rho33) || nx < 1 ||
      ny < 1 || nz < 1) {
    set_err("emmi_extract_volume: bad argument");
    return EMMI_EINVAL;
  }
  const long nxyz = (long)nx * ny * nz;
  const long S = s->hier[0][0].S;
  const int op = s->h_op[rhs];
  double2* df = nullptr;
  float* drho = nullptr;
  float2* dout = nullptr;
  CK(cudaMallocAsync((void**)&df, 3 * S * sizeof(double2), s->st));
  CK(cudaMallocAsync((void**)&drho, nxyz * sizeof(float), s->st));
  CK(cudaMallocAsync((void**)&dout, 3 * nxyz * sizeof(float2), s->st));
  CK(cudaMemcpyAsync(df, field, 3 * S * sizeof(double2), cudaMemcpyHostToDevice, s->st));
  if (rho33) CK(cudaMemcpyAsync(drho, rho33, nxyz * sizeof(float), cudaMemcpyHostToDevice, s->st));
  SGrid G = sgrid_of(s);
  G.g = s->sgeo + (long)op * s->gstride;
  const long nc = (long)s->n[0] * s->n[1] * s->n[2];
  k_extract_volume<<<nblk(nxyz), 256, 0, s->st>>>(G, which, nx, ny, nz, o[0], o[1], o[2], d[0],
                                                   d[1], d[2], drho,
                                                   s->raw_cells + ((long)op * 4 + 2) * nc, df,
                                                   dout, nxyz);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, dout, 3 * nxyz * sizeof(float2), cudaMemcpyDeviceToHost, s->st));
  cudaFreeAsync(df, s->st);
  cudaFreeAsync(drho, s->st);
  cudaFreeAsync(dout, s->st);
  CK(cudaStreamSynchronize(s->st));
  return EMMI_OK;
}

int emmi_build_gradient(int nx, int ny, int nz, const float o[3], const float d[3], int nshot,
                        int nfreq, int npar, const int* idxpar, int preco, const float* E1f,
                        const float* E2f, const float* E3f, const float* E1a, const float* E2a,
                        const float* E3a, const float* rho11, const float* rho33,
                        const float* bathy, const float* src, float dsmute, int nrec,
                        const float* rec, float drmute, float* grad, float* phess) {
  if (nx < 1 || ny < 1 || nz < 1 || nshot < 1 || nfreq < 1 || npar < 1 || npar > 2 || !idxpar ||
      !E1f || !E2f || !E3f || !E1a || !E2a || !E3a || !rho11 || !rho33 || !bathy || !src ||
      !grad || (nrec > 0 && !rec)) {
    set_err("emmi_build_gradient: bad argument");
    return EMMI_EINVAL;
  }
  const long nxyz = (long)nx * ny * nz;
  std::vector<unsigned char> bm, mm;
  gradient_masks(nx, ny, nz, o, d, bathy, nshot, src, dsmute, nrec, nullptr, rec, drmute, 3, bm,
                 mm);
  const size_t ef = (size_t)nshot * nfreq * nxyz * sizeof(float2);
  cudaStream_t st;
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  void* buf[12] = {};
  const size_t sizes[12] = {ef, ef, ef, ef, ef, ef, nxyz * sizeof(float), nxyz * sizeof(float),
                            (size_t)nxyz, (size_t)nshot * nxyz, npar * nxyz * sizeof(float),
                            npar * nxyz * sizeof(float)};
  const void* srcs[10] = {E1f, E2f, E3f, E1a, E2a, E3a, rho11, rho33, bm.data(), mm.data()};
  int* didx = nullptr;
  int rc = EMMI_OK;
  for (int b = 0; b < 12 && rc == EMMI_OK; b++)
    if (cudaMallocAsync(&buf[b], sizes[b] + 16, st) != cudaSuccess) rc = EMMI_ENOMEM;
  if (rc == EMMI_OK && cudaMallocAsync((void**)&didx, 2 * sizeof(int), st) != cudaSuccess)
    rc = EMMI_ENOMEM;
  if (rc == EMMI_OK) {
    for (int b = 0; b < 10; b++) cudaMemcpyAsync(buf[b], srcs[b], sizes[b], cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(didx, idxpar, npar * sizeof(int), cudaMemcpyHostToDevice, st);
    const float s = d[0] * d[1] * d[2];
    k_gradient<<<nblk(nxyz), 256, 0, st>>>(
        (int)nxyz, nshot, nfreq, npar, didx, preco, s, (const float2*)buf[0], (const float2*)buf[1],
        (const float2*)buf[2], (const float2*)buf[3], (const float2*)buf[4], (const float2*)buf[5],
        (const float*)buf[6], (const float*)buf[7], (const unsigned char*)buf[9],
        (const unsigned char*)buf[8], (float*)buf[10], (float*)buf[11]);
    cudaMemcpyAsync(grad, buf[10], npar * nxyz * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (preco == 1 && phess)
      cudaMemcpyAsync(phess, buf[11], npar * nxyz * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
      set_err("emmi_build_gradient: CUDA failure");
      rc = EMMI_ECUDA;
    }
  } else {
    set_err("emmi_build_gradient: device allocation failed");
  }
  for (int b = 0; b < 12; b++)
    if (buf[b]) cudaFreeAsync(buf[b], st);
  if (didx) cudaFreeAsync(didx, st);
  cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  return rc;
}

}  // extern "C"

// ---- the inversion's misfit-and-gradient evaluation for a batch of shots --

// the skin-depth offset below which data are left out of the misfit,
// 5.5 skin depths in water (fg_fwi.c:212, the arithmetic of eh_misfit)
static float misfit_skin(float omega, float rho_water) {
  const double mu0 = 4. * 3.14159265358979323846264 * 1e-7;
  return 5.5 * sqrt(2. * rho_water / (omega * mu0));
}

// per-RHS copies of each shot's source and receivers: RHS r = shot * nfreq
// + f; receivers past a shot's count repeat its first receiver (their data
// and adjoint sources are zero) so that every interpolation stays inside
static void per_rhs_points(int nshot, int nfreq, int nrec, const int* nrec_shot, const float* src,
                           const float* rec, std::vector<float>& rsrc, std::vector<float>& rrec) {
  const int nrhs = nshot * nfreq;
  rsrc.assign((size_t)nrhs * 5, 0.f);
  rrec.assign((size_t)nrhs * std::max(nrec, 1) * 5, 0.f);
  for (int r = 0; r < nrhs; r++) {
    const int sh = r / nfreq;
    std::memcpy(&rsrc[(size_t)r * 5], src + (size_t)sh * 5, 5 * sizeof(float));
    const int nr = nrec_shot ? nrec_shot[sh] : nrec;
    for (int ir = 0; ir < nrec; ir++) {
      const float* p = ir < nr ? rec + ((size_t)sh * nrec + ir) * 5
                               : (nr > 0 ? rec + (size_t)sh * nrec * 5 : src + (size_t)sh * 5);
      std::memcpy(&rrec[((size_t)r * nrec + ir) * 5], p, 5 * sizeof(float));
    }
  }
}

struct emmi_fg {
  int nx, ny, nz, n1, n2, n3, nshot, nfreq, nrhs, nrec, nch, nsrc_ch, npar, preco;
  bool have_data = true;  // observed data and uncertainties given (else forward only)
  float o[3], d[3], rho_water;
  long nxyz, nc;
  std::vector<float> x1, x2, x3, omega_rhs, rho_water_op;
  std::vector<int> op, src_ch, rec_ch, idxpar;
  emmi_options opt;
  cudaStream_t st = nullptr;
  float *d_src = nullptr, *d_rec = nullptr, *d_delta = nullptr, *d_skin = nullptr;
  float *d_rmse = nullptr, *d_fcost = nullptr, *d_rho11 = nullptr;
  double* d_term = nullptr;
  float *d_rho33 = nullptr, *d_grad = nullptr, *d_phess = nullptr, *d_cells = nullptr;
  float2 *d_dobs = nullptr, *d_dcal = nullptr, *d_dres = nullptr, *d_dsyn = nullptr;
  float2 *d_Ef = nullptr, *d_Ea = nullptr;
  unsigned char *d_bm = nullptr, *d_mm = nullptr;
  int *d_nrec = nullptr, *d_idx = nullptr;
  // milliseconds of the last evaluation's phases: front end, solver set-up,
  // forward solves, receiver data + forward fields, misfit, adjoint sources,
  // adjoint solves, adjoint fields + gradient + copies out
  double phase_ms[8] = {};
  std::vector<void*> owned;
  template <typename T>
  bool alloc(T** p, size_t n) {
    if (cudaMallocAsync((void**)p, n * sizeof(T) + 16, st) != cudaSuccess) return false;
    owned.push_back(*p);
    return true;
  }
};

extern "C" {

void emmi_fg_destroy(emmi_fg* f) {
  if (!f) return;
  for (void* p : f->owned) cudaFreeAsync(p, f->st);
  if (f->st) {
    cudaStreamSynchronize(f->st);
    cudaStreamDestroy(f->st);
  }
  delete f;
}

int emmi_fg_create(emmi_fg** out, const emmi_fg_problem* P, const emmi_options* opts) {
  if (!out || !P || !opts) {
    set_err("emmi_fg_create: bad argument");
    return EMMI_EINVAL;
  }
  *out = nullptr;
  // without observed data (dobs and delta NULL) only emmi_fg_forward runs,
  // and the gradient's parameters and masks are not needed
  const bool data = P->dobs || P->delta;
  bool ok = P->nx > 0 && P->ny > 0 && P->nz > 0 && P->n1 > 0 && P->n2 > 0 && P->n3 > 0 &&
            P->nshot > 0 && P->nfreq > 0 && (long)P->nshot * P->nfreq <= 65535 && P->omega &&
            P->x1 && P->x2 && P->x3 && P->nsrc_ch >= 1 && P->nsrc_ch <= 6 && P->src_ch &&
            P->nrec_ch >= 1 && P->nrec_ch <= 6 && P->rec_ch && P->nrec >= 1 && P->nrec_shot &&
            P->src && P->rec && P->rho_water > 0 &&
            (!data || (P->dobs && P->delta && P->npar >= 1 && P->npar <= 2 && P->idxpar &&
                       P->bathy));
  for (int k = 0; ok && data && k < P->npar; k++) ok = P->idxpar[k] == 1 || P->idxpar[k] == 2;
  for (int k = 0; ok && k < P->nsrc_ch; k++) ok = P->src_ch[k] >= 0 && P->src_ch[k] <= 5;
  for (int k = 0; ok && k < P->nrec_ch; k++) ok = P->rec_ch[k] >= 0 && P->rec_ch[k] <= 5;
  for (int k = 0; ok && k < P->nshot; k++) ok = P->nrec_shot[k] >= 0 && P->nrec_shot[k] <= P->nrec;
  if (!ok) {
    set_err("emmi_fg_create: bad problem description");
    return EMMI_EINVAL;
  }
  emmi_fg* f = new emmi_fg();
  f->nx = P->nx;
  f->ny = P->ny;
  f->nz = P->nz;
  f->n1 = P->n1;
  f->n2 = P->n2;
  f->n3 = P->n3;
  f->nshot = P->nshot;
  f->nfreq = P->nfreq;
  f->nrhs = P->nshot * P->nfreq;
  f->nrec = P->nrec;
  f->nch = P->nrec_ch;
  f->nsrc_ch = P->nsrc_ch;
  f->have_data = data;
  f->npar = data ? P->npar : 1;
  f->preco = data ? P->preco : 0;
  f->rho_water = P->rho_water;
  for (int e = 0; e < 3; e++) {
    f->o[e] = P->o[e];
    f->d[e] = P->d[e];
  }
  f->nxyz = (long)P->nx * P->ny * P->nz;
  f->nc = (long)P->n1 * P->n2 * P->n3;
  f->x1.assign(P->x1, P->x1 + (size_t)P->nshot * (P->n1 + 1));
  f->x2.assign(P->x2, P->x2 + (size_t)P->nshot * (P->n2 + 1));
  f->x3.assign(P->x3, P->x3 + (size_t)P->nshot * (P->n3 + 1));
  f->rho_water_op.assign(P->nshot, P->rho_water);
  f->src_ch.assign(P->src_ch, P->src_ch + P->nsrc_ch);
  f->rec_ch.assign(P->rec_ch, P->rec_ch + P->nrec_ch);
  if (data) f->idxpar.assign(P->idxpar, P->idxpar + P->npar);
  else f->idxpar.assign(1, 1);
  for (int r = 0; r < f->nrhs; r++) {
    f->op.push_back(r / P->nfreq);
    f->omega_rhs.push_back(P->omega[r % P->nfreq]);
  }
  f->opt = *opts;
  std::vector<float> skin(P->nfreq), rsrc, rrec;
  for (int k = 0; k < P->nfreq; k++) skin[k] = misfit_skin(P->omega[k], P->rho_water);
  per_rhs_points(P->nshot, P->nfreq, P->nrec, P->nrec_shot, P->src, P->rec, rsrc, rrec);
  std::vector<unsigned char> bm(1, 0), mm(1, 0);
  if (data)
    gradient_masks(P->nx, P->ny, P->nz, P->o, P->d, P->bathy, P->nshot, P->src, P->dsmute,
                   P->nrec, P->nrec_shot, P->rec, P->drmute, 5, bm, mm);
  const size_t nper = (size_t)P->nshot * f->nch * P->nfreq * P->nrec;
  const size_t nrd = (size_t)f->nrhs * f->nch * P->nrec;
  const size_t ne = data ? (size_t)3 * f->nrhs * f->nxyz : 1;  // volume fields: gradient only
  if (cudaStreamCreateWithFlags(&f->st, cudaStreamNonBlocking) != cudaSuccess ||
      !f->alloc(&f->d_src, rsrc.size()) || !f->alloc(&f->d_rec, rrec.size()) ||
      !f->alloc(&f->d_delta, nper) || !f->alloc(&f->d_skin, P->nfreq) ||
      !f->alloc(&f->d_rmse, nper) || !f->alloc(&f->d_term, nper) ||
      !f->alloc(&f->d_fcost, P->nshot) || !f->alloc(&f->d_rho11, f->nxyz) ||
      !f->alloc(&f->d_rho33, f->nxyz) || !f->alloc(&f->d_grad, (size_t)f->npar * f->nxyz) ||
      !f->alloc(&f->d_phess, (size_t)f->npar * f->nxyz) ||
      !f->alloc(&f->d_cells, (size_t)P->nshot * 4 * f->nc) || !f->alloc(&f->d_dobs, nper) ||
      !f->alloc(&f->d_dcal, nrd) || !f->alloc(&f->d_dres, nrd) || !f->alloc(&f->d_dsyn, nper) ||
      !f->alloc(&f->d_Ef, ne) || !f->alloc(&f->d_Ea, ne) || !f->alloc(&f->d_bm, bm.size()) ||
      !f->alloc(&f->d_mm, mm.size()) || !f->alloc(&f->d_nrec, P->nshot) ||
      !f->alloc(&f->d_idx, f->npar)) {
    set_err("emmi_fg_create: device allocation failed");
    emmi_fg_destroy(f);
    return EMMI_ENOMEM;
  }
  cudaStream_t st = f->st;
  cudaMemcpyAsync(f->d_src, rsrc.data(), rsrc.size() * sizeof(float), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(f->d_rec, rrec.data(), rrec.size() * sizeof(float), cudaMemcpyHostToDevice, st);
  if (data) {
    cudaMemcpyAsync(f->d_delta, P->delta, nper * sizeof(float), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(f->d_dobs, P->dobs, nper * sizeof(float2), cudaMemcpyHostToDevice, st);
  }
  cudaMemcpyAsync(f->d_skin, skin.data(), skin.size() * sizeof(float), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(f->d_bm, bm.data(), bm.size(), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(f->d_mm, mm.data(), mm.size(), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(f->d_nrec, P->nrec_shot, P->nshot * sizeof(int), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(f->d_idx, f->idxpar.data(), f->npar * sizeof(int), cudaMemcpyHostToDevice, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    set_err("emmi_fg_create: %s", cudaGetErrorString(e));
    emmi_fg_destroy(f);
    return EMMI_ECUDA;
  }
  *out = f;
  return EMMI_OK;
}

int emmi_fg_eval(emmi_fg* f, int nxp, int nyp, int nzp, const float* xx, const float* yy,
                 const float* zz, const float* pad, const float* rho11, const float* rho33,
                 float* fcost, float* grad, float* phess, float* dcal, float* rmse,
                 emmi_rhs_stats* stats) {
  if (!f || !xx || !yy || !zz || !pad || !rho11 || !rho33 || !fcost || !grad) {
    set_err("emmi_fg_eval: bad argument");
    return EMMI_EINVAL;
  }
  if (!f->have_data) {
    set_err("emmi_fg_eval: created without observed data (forward modelling only)");
    return EMMI_ESTATE;
  }
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  // the front end: every shot's homogenization of the current model
  int rc = emmi_homogenize_batch(nxp, nyp, nzp, xx, yy, zz, pad, f->nshot, f->n1, f->n2, f->n3,
                                 f->x1.data(), f->x2.data(), f->x3.data(), f->d_cells, f->st);
  if (rc != EMMI_OK) return rc;
  const auto t1 = clk::now();
  emmi_problem P = {f->n1,         f->n2,        f->n3,        f->nshot,
                    f->nrhs,       f->x1.data(), f->x2.data(), f->x3.data(),
                    f->d_cells,    f->op.data(), f->omega_rhs.data(), f->rho_water_op.data()};
  emmi_solver* s = nullptr;
  rc = emmi_solver_create_dc(&s, &P, &f->opt);
  if (rc != EMMI_OK) return rc;
  const cudaStream_t st = s->st;
  cudaEvent_t ev[7] = {};
  for (auto& e : ev) cudaEventCreate(&e);
  cudaEventRecord(ev[0], st);
  const auto t2 = clk::now();
  const long S = s->hier[0][0].S;
  std::vector<emmi_rhs_stats> tmp;
  emmi_rhs_stats* sf = stats;
  if (!sf) {
    tmp.resize(2 * (size_t)f->nrhs);
    sf = tmp.data();
  }
  auto volume = [&](float2* out) {
    for (int r = 0; r < f->nrhs; r++) {
      SGrid G = sgrid_of(s);
      const int o = f->op[r];
      G.g = s->sgeo + (long)o * s->gstride;
      k_extract_volume<<<nblk(f->nxyz), 256, 0, st>>>(
          G, 0, f->nx, f->ny, f->nz, f->o[0], f->o[1], f->o[2], f->d[0], f->d[1], f->d[2],
          f->d_rho33, s->raw_cells + ((long)o * 4 + 2) * f->nc, s->u64[0] + (long)r * 3 * S,
          out + (long)r * f->nxyz, (long)f->nrhs * f->nxyz);
    }
  };
  double* E = (double*)s->u64[0];
  double* H = (double*)s->f64[0];
  cudaMemcpyAsync(f->d_rho11, rho11, f->nxyz * sizeof(float), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(f->d_rho33, rho33, f->nxyz * sizeof(float), cudaMemcpyHostToDevice, st);
  // 1. forward modelling of every shot and frequency
  rc = emmi_inject_sources_dev(s, f->d_src, f->nsrc_ch, f->src_ch.data(), E);
  if (rc == EMMI_OK) rc = emmi_solver_solve_resident(s, nullptr, nullptr, sf);
  cudaEventRecord(ev[1], st);
  if (rc == EMMI_OK)
    rc = emmi_extract_receivers_dev(s, f->d_rec, f->nrec, f->nch, f->rec_ch.data(), E, H,
                                    (float*)f->d_dcal);
  if (rc == EMMI_OK) {
    volume(f->d_Ef);
    cudaEventRecord(ev[2], st);
    // 2. misfit and adjoint sources
    k_misfit<<<f->nshot, 256, 0, st>>>(f->nch, f->nfreq, f->nrec, f->d_nrec, f->d_skin, f->d_src,
                                       f->d_rec, f->d_dobs, f->d_delta, f->d_dcal, f->d_dres,
                                       f->d_rmse, f->d_dsyn, f->d_term, f->d_fcost);
    cudaEventRecord(ev[3], st);
    // 3. adjoint modelling (H's buffer is the scratch of the magnetic part)
    rc = emmi_inject_adjoint_dev(s, f->d_rec, f->nrec, f->nch, f->rec_ch.data(),
                                 (const float*)f->d_dres, E, H);
  }
  cudaEventRecord(ev[4], st);
  if (rc == EMMI_OK) rc = emmi_solver_solve_resident(s, nullptr, nullptr, sf + f->nrhs);
  cudaEventRecord(ev[5], st);
  if (rc == EMMI_OK) {
    volume(f->d_Ea);
    // 4. the gradient, summed over shots and frequencies
    const long ne = (long)f->nrhs * f->nxyz;
    k_gradient<<<nblk(f->nxyz), 256, 0, st>>>(
        (int)f->nxyz, f->nshot, f->nfreq, f->npar, f->d_idx, f->preco, f->d[0] * f->d[1] * f->d[2],
        f->d_Ef, f->d_Ef + ne, f->d_Ef + 2 * ne, f->d_Ea, f->d_Ea + ne, f->d_Ea + 2 * ne,
        f->d_rho11, f->d_rho33, f->d_mm, f->d_bm, f->d_grad, f->d_phess);
    const size_t nper = (size_t)f->nshot * f->nch * f->nfreq * f->nrec;
    cudaMemcpyAsync(fcost, f->d_fcost, f->nshot * sizeof(float), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(grad, f->d_grad, f->npar * f->nxyz * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (phess && f->preco == 1)
      cudaMemcpyAsync(phess, f->d_phess, f->npar * f->nxyz * sizeof(float),
                      cudaMemcpyDeviceToHost, st);
    if (dcal) cudaMemcpyAsync(dcal, f->d_dsyn, nper * sizeof(float2), cudaMemcpyDeviceToHost, st);
    if (rmse) cudaMemcpyAsync(rmse, f->d_rmse, nper * sizeof(float), cudaMemcpyDeviceToHost, st);
    cudaEventRecord(ev[6], st);
    const cudaError_t e = cudaStreamSynchronize(st);
    const cudaError_t e2 = cudaGetLastError();
    if (e != cudaSuccess || e2 != cudaSuccess) {
      set_err("emmi_fg_eval: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
      rc = EMMI_ECUDA;
    }
  }
  if (rc == EMMI_OK) {
    auto ms = [](clk::time_point a, clk::time_point b) {
      return std::chrono::duration<double, std::milli>(b - a).count();
    };
    f->phase_ms[0] = ms(t0, t1);
    f->phase_ms[1] = ms(t1, t2);
    for (int k = 0; k < 6; k++) {
      float v = 0.f;
      cudaEventElapsedTime(&v, ev[k], ev[k + 1]);
      f->phase_ms[2 + k] = v;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  emmi_solver_destroy(s);
  return rc;
}

int emmi_fg_forward(emmi_fg* f, int nxp, int nyp, int nzp, const float* xx, const float* yy,
                    const float* zz, const float* pad, float* dcal, emmi_rhs_stats* stats) {
  if (!f || !xx || !yy || !zz || !pad || !dcal) {
    set_err("emmi_fg_forward: bad argument");
    return EMMI_EINVAL;
  }
  int rc = emmi_homogenize_batch(nxp, nyp, nzp, xx, yy, zz, pad, f->nshot, f->n1, f->n2, f->n3,
                                 f->x1.data(), f->x2.data(), f->x3.data(), f->d_cells, f->st);
  if (rc != EMMI_OK) return rc;
  emmi_problem P = {f->n1,         f->n2,        f->n3,        f->nshot,
                    f->nrhs,       f->x1.data(), f->x2.data(), f->x3.data(),
                    f->d_cells,    f->op.data(), f->omega_rhs.data(), f->rho_water_op.data()};
  emmi_solver* s = nullptr;
  if ((rc = emmi_solver_create_dc(&s, &P, &f->opt)) != EMMI_OK) return rc;
  double* E = (double*)s->u64[0];
  double* H = (double*)s->f64[0];
  std::vector<emmi_rhs_stats> tmp;
  if (!stats) {
    tmp.resize(f->nrhs);
    stats = tmp.data();
  }
  rc = emmi_inject_sources_dev(s, f->d_src, f->nsrc_ch, f->src_ch.data(), E);
  if (rc == EMMI_OK) rc = emmi_solver_solve_resident(s, nullptr, nullptr, stats);
  if (rc == EMMI_OK)
    rc = emmi_extract_receivers_dev(s, f->d_rec, f->nrec, f->nch, f->rec_ch.data(), E, H,
                                    (float*)f->d_dcal);
  if (rc == EMMI_OK) {
    // [shot * nfreq + f][c][ir] on the device -> [shot][c][f][ir]
    const size_t nrd = (size_t)f->nrhs * f->nch * f->nrec;
    std::vector<float2> h(nrd);
    cudaMemcpyAsync(h.data(), f->d_dcal, nrd * sizeof(float2), cudaMemcpyDeviceToHost, s->st);
    const cudaError_t e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) {
      set_err("emmi_fg_forward: %s", cudaGetErrorString(e));
      rc = EMMI_ECUDA;
    } else {
      for (int sh = 0; sh < f->nshot; sh++)
        for (int c = 0; c < f->nch; c++)
          for (int q = 0; q < f->nfreq; q++)
            for (int ir = 0; ir < f->nrec; ir++) {
              const float2 v = h[(((size_t)sh * f->nfreq + q) * f->nch + c) * f->nrec + ir];
              const size_t o = (((size_t)sh * f->nch + c) * f->nfreq + q) * f->nrec + ir;
              dcal[2 * o] = v.x;
              dcal[2 * o + 1] = v.y;
            }
    }
  }
  emmi_solver_destroy(s);
  return rc;
}

int emmi_fg_phases(const emmi_fg* f, double ms[8]) {
  if (!f || !ms) {
    set_err("emmi_fg_phases: bad argument");
    return EMMI_EINVAL;
  }
  for (int k = 0; k < 8; k++) ms[k] = f->phase_ms[k];
  return EMMI_OK;
}

int emmi_misfit_batch(int nshot, int nch, int nfreq, int nrec, const int* nrec_shot,
                      const float* omega, float rho_water, const float* src, const float* rec,
                      const float* dobs, const float* delta, const float* dcal, float* dres,
                      float* rmse, float* fcost) {
  if (nshot < 1 || nch < 1 || nfreq < 1 || nrec < 1 || !nrec_shot || !omega || !src || !rec ||
      !dobs || !delta || !dcal || !dres || !rmse || !fcost) {
    set_err("emmi_misfit_batch: bad argument");
    return EMMI_EINVAL;
  }
  for (int k = 0; k < nshot; k++)
    if (nrec_shot[k] < 0 || nrec_shot[k] > nrec) {
      set_err("emmi_misfit_batch: bad receiver count");
      return EMMI_EINVAL;
    }
  const size_t nper = (size_t)nshot * nch * nfreq * nrec;
  std::vector<float> skin(nfreq), rsrc, rrec;
  for (int k = 0; k < nfreq; k++) skin[k] = misfit_skin(omega[k], rho_water);
  per_rhs_points(nshot, nfreq, nrec, nrec_shot, src, rec, rsrc, rrec);
  // dcal from the per-shot layout [shot][c][f][ir] to the per-RHS one
  // [shot * nfreq + f][c][ir] that receiver extraction writes
  std::vector<float2> rcal(nper), rres(nper);
  auto rhs_index = [&](int sh, int c, int f, int ir) {
    return (((size_t)sh * nfreq + f) * nch + c) * nrec + ir;
  };
  for (int sh = 0; sh < nshot; sh++)
    for (int c = 0; c < nch; c++)
      for (int f = 0; f < nfreq; f++)
        for (int ir = 0; ir < nrec; ir++) {
          const size_t q = (((size_t)sh * nch + c) * nfreq + f) * nrec + ir;
          rcal[rhs_index(sh, c, f, ir)] = make_float2(dcal[2 * q], dcal[2 * q + 1]);
        }
  cudaStream_t st;
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  std::vector<void*> bufs;
  auto dev = [&](size_t bytes, const void* from) -> void* {
    void* p = nullptr;
    if (cudaMallocAsync(&p, bytes + 16, st) != cudaSuccess) return nullptr;
    bufs.push_back(p);
    if (from) cudaMemcpyAsync(p, from, bytes, cudaMemcpyHostToDevice, st);
    return p;
  };
  float* d_skin = (float*)dev(nfreq * sizeof(float), skin.data());
  float* d_src = (float*)dev(rsrc.size() * sizeof(float), rsrc.data());
  float* d_rec = (float*)dev(rrec.size() * sizeof(float), rrec.data());
  float2* d_dobs = (float2*)dev(nper * sizeof(float2), dobs);
  float* d_delta = (float*)dev(nper * sizeof(float), delta);
  float2* d_dcal = (float2*)dev(nper * sizeof(float2), rcal.data());
  float2* d_dres = (float2*)dev(nper * sizeof(float2), nullptr);
  float* d_rmse = (float*)dev(nper * sizeof(float), nullptr);
  float2* d_dsyn = (float2*)dev(nper * sizeof(float2), nullptr);
  double* d_term = (double*)dev(nper * sizeof(double), nullptr);
  float* d_fcost = (float*)dev(nshot * sizeof(float), nullptr);
  int* d_nrec = (int*)dev(nshot * sizeof(int), nrec_shot);
  int rc = EMMI_OK;
  if (bufs.size() != 12) {
    set_err("emmi_misfit_batch: device allocation failed");
    rc = EMMI_ENOMEM;
  } else {
    k_misfit<<<nshot, 256, 0, st>>>(nch, nfreq, nrec, d_nrec, d_skin, d_src, d_rec, d_dobs,
                                    d_delta, d_dcal, d_dres, d_rmse, d_dsyn, d_term, d_fcost);
    cudaMemcpyAsync(rres.data(), d_dres, nper * sizeof(float2), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(rmse, d_rmse, nper * sizeof(float), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(fcost, d_fcost, nshot * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
      set_err("emmi_misfit_batch: CUDA failure");
      rc = EMMI_ECUDA;
    }
  }
  for (void* p : bufs) cudaFreeAsync(p, st);
  cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  if (rc == EMMI_OK)
    for (int sh = 0; sh < nshot; sh++)
      for (int c = 0; c < nch; c++)
        for (int f = 0; f < nfreq; f++)
          for (int ir = 0; ir < nrec; ir++) {
            const size_t q = (((size_t)sh * nch + c) * nfreq + f) * nrec + ir;
            const float2 v = rres[rhs_index(sh, c, f, ir)];
            dres[2 * q] = v.x;
            dres[2 * q + 1] = v.y;
          }
  return rc;
}

}  // extern "C"

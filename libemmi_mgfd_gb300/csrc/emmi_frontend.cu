// Front end on the device: the homogenization of the reference's regrid
// stage (src/homogenization.c:15-111) for a batch of shots over one model.
//
// The host builds the padded model and each shot's mesh axes (1D work,
// eh_pad_model / eh_regrid_axes of the host library); this file averages
// the padded model onto every shot's cells, three separable 1D passes
// (x, then y, then z) as the reference does them.  Every output value is
// the host's, bit for bit: a thread owns one output cell, finds the first
// overlapping source cell by bisection (the host's running index reaches the
// same cell, the axes being increasing), and accumulates in the host's order
// with round-to-nearest operations and no fused multiply-add.
#include <cuda_runtime.h>

#include <cstdint>

#include "emmi_solver_impl.cuh"

namespace emmi {
namespace {

// out = volume average over [dst[j], dst[j+1]) of in[k * stride] on the
// source cells [src[k], src[k+1]), k < ns (homogenization.c:24-48)
__device__ __forceinline__ float average_cell(const float* __restrict__ in, long stride, int ns,
                                              const float* __restrict__ src, float a, float b) {
  int lo = 0, hi = ns;  // first k with src[k+1] > a (ns if none)
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (src[mid + 1] > a) hi = mid;
    else lo = mid + 1;
  }
  float s = 0.f;
  for (int k = lo; k < ns && src[k] < b; k++) {
    const float left = (src[k] > a) ? src[k] : a;
    const float right = (src[k + 1] < b) ? src[k + 1] : b;
    const float overlap = __fsub_rn(right, left);
    if (overlap > 0.f) s = __fadd_rn(s, __fmul_rn(in[k * stride], overlap));
  }
  return __fdiv_rn(s, __fsub_rn(b, a));
}

struct Dims {
  int nxp, nyp, nzp;  // padded model cells
  int n1, n2, n3;     // mesh cells
  int nshots;
};

// pass x: t1[shot][a][z][y][i'] from pad[a][z][y][:] onto x1 of the shot
__global__ void k_avg_x(Dims d, const float* __restrict__ pad, const float* __restrict__ xx,
                        const float* __restrict__ x1, float* __restrict__ t1) {
  const long per = (long)d.n1 * d.nyp * d.nzp;
  const long id = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (id >= per) return;
  const int a = blockIdx.y, shot = blockIdx.z;
  const int i = (int)(id % d.n1);
  const long yz = id / d.n1;  // y + nyp z
  const float* X = x1 + (long)shot * (d.n1 + 1);
  const float* in = pad + (long)a * d.nxp * d.nyp * d.nzp + yz * d.nxp;
  t1[((long)shot * 3 + a) * per + id] = average_cell(in, 1, d.nxp, xx, X[i], X[i + 1]);
}

// pass y: t2[shot][a][z][j'][i'] from t1 along y onto x2
__global__ void k_avg_y(Dims d, const float* __restrict__ t1, const float* __restrict__ yy,
                        const float* __restrict__ x2, float* __restrict__ t2) {
  const long per = (long)d.n1 * d.n2 * d.nzp;
  const long id = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (id >= per) return;
  const int a = blockIdx.y, shot = blockIdx.z;
  const int i = (int)(id % d.n1);
  const int j = (int)((id / d.n1) % d.n2);
  const int z = (int)(id / ((long)d.n1 * d.n2));
  const float* X = x2 + (long)shot * (d.n2 + 1);
  const long per1 = (long)d.n1 * d.nyp * d.nzp;
  const float* in = t1 + ((long)shot * 3 + a) * per1 + i + (long)d.n1 * d.nyp * z;
  t2[((long)shot * 3 + a) * per + id] = average_cell(in, d.n1, d.nyp, yy, X[j], X[j + 1]);
}

// pass z: cells[shot][a][k'][j'][i'] from t2 along z onto x3; the third
// array is the rho33 average, stored as its inverse (regrid_init_free.c:
// 222-226, in double like the reference's 1./x); invmur = 1
__global__ void k_avg_z(Dims d, const float* __restrict__ t2, const float* __restrict__ zz,
                        const float* __restrict__ x3, float* __restrict__ cells) {
  const long nc = (long)d.n1 * d.n2 * d.n3;
  const long id = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (id >= nc) return;
  const int shot = blockIdx.z;
  float* out = cells + (long)shot * 4 * nc;
  if (blockIdx.y == 3) {
    out[3 * nc + id] = 1.f;
    return;
  }
  const int a = blockIdx.y;
  const int ij = (int)(id % ((long)d.n1 * d.n2));
  const int k = (int)(id / ((long)d.n1 * d.n2));
  const float* X = x3 + (long)shot * (d.n3 + 1);
  const long per2 = (long)d.n1 * d.n2 * d.nzp;
  const float* in = t2 + ((long)shot * 3 + a) * per2 + ij;
  float v = average_cell(in, (long)d.n1 * d.n2, d.nzp, zz, X[k], X[k + 1]);
  if (a == 2) v = (float)(1.0 / (double)v);
  out[(long)a * nc + id] = v;
}

unsigned blocks_of(long n) { return (unsigned)((n + 255) / 256); }

}  // namespace
}  // namespace emmi

using namespace emmi;

extern "C" int emmi_homogenize_batch(int nxp, int nyp, int nzp, const float* xx, const float* yy,
                                     const float* zz, const float* pad, int nshots, int n1,
                                     int n2, int n3, const float* x1, const float* x2,
                                     const float* x3, float* cells, void* stream) {
  if (nxp < 1 || nyp < 1 || nzp < 1 || nshots < 1 || n1 < 1 || n2 < 1 || n3 < 1 || !xx || !yy ||
      !zz || !pad || !x1 || !x2 || !x3 || !cells || nshots > 65535) {
    set_err("emmi_homogenize_batch: bad argument");
    return EMMI_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Dims d{nxp, nyp, nzp, n1, n2, n3, nshots};
  const long np = (long)nxp * nyp * nzp;
  const long per1 = (long)n1 * nyp * nzp, per2 = (long)n1 * n2 * nzp, nc = (long)n1 * n2 * n3;
  float *dpad = nullptr, *dax = nullptr, *t1 = nullptr, *t2 = nullptr;
  const long nax = (nxp + 1) + (nyp + 1) + (nzp + 1) + (long)nshots * (n1 + n2 + n3 + 3);
  auto fail = [&](cudaError_t e) {
    set_err("emmi_homogenize_batch: %s", cudaGetErrorString(e));
    cudaFreeAsync(dpad, st);
    cudaFreeAsync(dax, st);
    cudaFreeAsync(t1, st);
    cudaFreeAsync(t2, st);
    cudaStreamSynchronize(st);
    return EMMI_ECUDA;
  };
  cudaError_t e;
  if ((e = cudaMallocAsync((void**)&dpad, 3 * np * sizeof(float), st)) != cudaSuccess) return fail(e);
  if ((e = cudaMallocAsync((void**)&dax, nax * sizeof(float), st)) != cudaSuccess) return fail(e);
  if ((e = cudaMallocAsync((void**)&t1, (size_t)nshots * 3 * per1 * sizeof(float), st)) !=
      cudaSuccess)
    return fail(e);
  if ((e = cudaMallocAsync((void**)&t2, (size_t)nshots * 3 * per2 * sizeof(float), st)) !=
      cudaSuccess)
    return fail(e);
  float* dxx = dax;
  float* dyy = dxx + (nxp + 1);
  float* dzz = dyy + (nyp + 1);
  float* dx1 = dzz + (nzp + 1);
  float* dx2 = dx1 + (long)nshots * (n1 + 1);
  float* dx3 = dx2 + (long)nshots * (n2 + 1);
  cudaMemcpyAsync(dpad, pad, 3 * np * sizeof(float), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dxx, xx, (nxp + 1) * sizeof(float), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dyy, yy, (nyp + 1) * sizeof(float), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dzz, zz, (nzp + 1) * sizeof(float), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dx1, x1, (size_t)nshots * (n1 + 1) * sizeof(float), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dx2, x2, (size_t)nshots * (n2 + 1) * sizeof(float), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dx3, x3, (size_t)nshots * (n3 + 1) * sizeof(float), cudaMemcpyHostToDevice, st);
  k_avg_x<<<dim3(blocks_of(per1), 3, nshots), 256, 0, st>>>(d, dpad, dxx, dx1, t1);
  k_avg_y<<<dim3(blocks_of(per2), 3, nshots), 256, 0, st>>>(d, t1, dyy, dx2, t2);
  k_avg_z<<<dim3(blocks_of(nc), 4, nshots), 256, 0, st>>>(d, t2, dzz, dx3, cells);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
  cudaFreeAsync(dpad, st);
  cudaFreeAsync(dax, st);
  cudaFreeAsync(t1, st);
  cudaFreeAsync(t2, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) {
    set_err("emmi_homogenize_batch: %s", cudaGetErrorString(e));
    return EMMI_ECUDA;
  }
  return EMMI_OK;
}

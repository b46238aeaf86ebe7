// Line relaxation of one level on caller-owned device buffers, with no device
// allocation at all: the sweep's record buffer (and the level's staggered
// geometry) live in one file-scope device array instead of cudaMalloc'd
// scratch.
//
// Who needs this: a caller whose device memory is fully owned by its own
// pool or arena (it reserved the HBM up front and has nothing left for a
// library to cudaMalloc), and a caller on a latency-critical stream that
// cannot let a library's cudaMalloc/cudaFree synchronize the whole device in
// the middle of its work.  Such a caller already holds u, f and the cells in
// its own device memory and only needs the sweep.
//
// Contract:
//  * the scratch array is EMMI_NOALLOC_SCRATCH_BYTES per GPU.  CUDA loads a
//    library's device code lazily by default (CUDA_MODULE_LOADING=LAZY), so
//    the array is reserved on a device by the first call there, not when the
//    library is loaded: make one call on each device before the caller's
//    pool reserves its HBM, or run with CUDA_MODULE_LOADING=EAGER.  From then
//    on the device holds the array until the process exits and no call
//    reserves anything more;
//  * the first call on a device looks up the array's device address for that
//    device (cudaGetSymbolAddress, with that device current) and keeps it for
//    the life of the process: do not use the call across cudaDeviceReset,
//    which unloads the module the address belongs to;
//  * each call stages the level's geometry from host memory with
//    cudaMemcpyAsync; a call on a stream that is being captured is refused
//    with EMMI_EINVAL, because the copy's host source does not outlive the
//    call;
//  * every call on a device shares the one array and leaves its contents
//    behind; nothing in it needs to start at zero (the assemble launch writes
//    every record the solve then reads), and two calls whose work overlaps on
//    the GPU (different streams, no ordering between them) race on it;
//  * a level whose sweep needs more scratch than the maximum is rejected with
//    EMMI_EINVAL and a message naming the bytes needed;
//  * no cudaMalloc, cudaFree or other allocating routine is called; the host
//    staging arrays are ordinary heap memory sized to the level.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "emmi_solver_impl.cuh"

using namespace emmi;

// layout per call: [geometry (9*(nmax+1) values of T)][omega*mu0][records]
static __device__ __align__(256) unsigned char g_noalloc_scratch[EMMI_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
constexpr int kMaxN = EMMI_NOALLOC_MAX_N;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_addr[kMaxDevices];  // device address of the array, per device

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// node coordinates x[0..n] -> staggered spacings, the same arithmetic as the
// solver's set-up: ds (primary spacing, last one mirrored), d (dual spacing)
void stagger_axis(int n, const double* x, double* d, double* ds) {
  std::vector<double> xs(n + 1);
  for (int i = 0; i < n; i++) {
    ds[i] = x[i + 1] - x[i];
    xs[i] = 0.5 * (x[i] + x[i + 1]);
  }
  xs[n] = x[n] + 0.5 * ds[n - 1];
  ds[n] = xs[n] - x[n];
  for (int i = 1; i <= n; i++) d[i] = xs[i] - xs[i - 1];
  d[0] = xs[0] - x[0];
}

int scratch_on_current_device(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_err("emmi_level_line_sweep_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    return EMMI_ECUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    set_err("emmi_level_line_sweep_noalloc: device %d beyond the %d supported", dev, kMaxDevices);
    return EMMI_EINVAL;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_err("emmi_level_line_sweep_noalloc: cudaGetSymbolAddress on device %d: %s", dev,
              cudaGetErrorString(e));
      return EMMI_ECUDA;
    }
    g_noalloc_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_noalloc_addr[dev];
  return EMMI_OK;
}

template <typename T>
int sweep_noalloc(const int n[3], const double* const xin[3], const void* cells, double omega,
                  int dir, int iter, void* u, const void* f, cudaStream_t st) {
  const int gmax = std::max(n[0], std::max(n[1], n[2]));
  const int gmax1 = gmax + 1, gstride = 9 * gmax1;
  const size_t geo_bytes = align256((size_t)gstride * sizeof(T));
  const size_t rec_bytes = (size_t)line_scratch_elems(n, dir, 1) * sizeof(C_t<T>);
  const size_t need = geo_bytes + 256 + rec_bytes;
  if (need > (size_t)EMMI_NOALLOC_SCRATCH_BYTES) {
    set_err("emmi_level_line_sweep_noalloc: a %s sweep along %d of a %dx%dx%d level needs %zu "
            "bytes of scratch; the maximum is %zu",
            sizeof(T) == 8 ? "complex128" : "complex64", dir, n[0], n[1], n[2], need,
            (size_t)EMMI_NOALLOC_SCRATCH_BYTES);
    return EMMI_EINVAL;
  }
  unsigned char* base = nullptr;
  int rc = scratch_on_current_device(&base);
  if (rc != EMMI_OK) return rc;

  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(st, &cap);
  if (e != cudaSuccess) {
    set_err("emmi_level_line_sweep_noalloc: cudaStreamIsCapturing: %s", cudaGetErrorString(e));
    return EMMI_ECUDA;
  }
  if (cap != cudaStreamCaptureStatusNone) {
    set_err("emmi_level_line_sweep_noalloc: the stream is being captured; the call stages its "
            "geometry from host memory that does not outlive the call");
    return EMMI_EINVAL;
  }

  // geometry rows: 0-2 node coordinates, 3-5 primary spacings, 6-8 dual spacings
  std::vector<T> g((size_t)gstride, (T)0);
  std::vector<double> d(gmax1), ds(gmax1);
  for (int ax = 0; ax < 3; ax++) {
    stagger_axis(n[ax], xin[ax], d.data(), ds.data());
    for (int i = 0; i <= n[ax]; i++) {
      g[ax * gmax1 + i] = (T)xin[ax][i];
      g[(3 + ax) * gmax1 + i] = (T)ds[i];
      g[(6 + ax) * gmax1 + i] = (T)d[i];
    }
  }
  const T wmu = (T)(omega * kMu0);
  T* dgeo = reinterpret_cast<T*>(base);
  T* dwmu = reinterpret_cast<T*>(base + geo_bytes);
  C_t<T>* drec = reinterpret_cast<C_t<T>*>(base + geo_bytes + 256);
  // pageable sources: each copy returns once g / wmu have been staged
  e = cudaMemcpyAsync(dgeo, g.data(), (size_t)gstride * sizeof(T), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dwmu, &wmu, sizeof(T), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) {
    set_err("emmi_level_line_sweep_noalloc: geometry upload: %s", cudaGetErrorString(e));
    return EMMI_ECUDA;
  }

  LevelView<T> V;
  for (int k = 0; k < 3; k++) V.n[k] = n[k];
  set_slot_divs(V);
  V.nrhs = 1;
  V.S = (long)(n[0] + 1) * (n[1] + 1) * (n[2] + 1);
  V.ncell = (long)n[0] * n[1] * n[2];
  V.gstride = gstride;
  V.gmax1 = gmax1;
  V.geo = dgeo;
  V.cells = static_cast<const T*>(cells);
  V.u = static_cast<C_t<T>*>(u);
  V.f = const_cast<C_t<T>*>(static_cast<const C_t<T>*>(f));  // read only
  V.r = nullptr;
  V.wmu = dwmu;
  V.active = nullptr;
  V.op = nullptr;
  for (int cc = 0; cc < 4; cc++) launch_line_sweep<T>(V, dir, iter % 2 ? 3 - cc : cc, drec, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_err("emmi_level_line_sweep_noalloc: launch: %s", cudaGetErrorString(e));
    return EMMI_ECUDA;
  }
  return EMMI_OK;
}

}  // namespace

extern "C" int emmi_level_line_sweep_noalloc(const int n[3], const double* x1, const double* x2,
                                             const double* x3, const void* cells, double omega,
                                             int prec, int dir, int iter, void* u, const void* f,
                                             void* stream) {
  if (!n || !x1 || !x2 || !x3 || !cells || !u || !f || dir < 0 || dir > 2 ||
      (prec != EMMI_PREC_FP64 && prec != EMMI_PREC_MIXED)) {
    set_err("emmi_level_line_sweep_noalloc: bad argument");
    return EMMI_EINVAL;
  }
  for (int k = 0; k < 3; k++)
    if (n[k] < 2 || n[k] > kMaxN) {
      set_err("emmi_level_line_sweep_noalloc: n[%d] = %d outside [2, %d]", k, n[k], kMaxN);
      return EMMI_EINVAL;
    }
  const double* xin[3] = {x1, x2, x3};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return prec == EMMI_PREC_FP64 ? sweep_noalloc<double>(n, xin, cells, omega, dir, iter, u, f, st)
                                : sweep_noalloc<float>(n, xin, cells, omega, dir, iter, u, f, st);
}

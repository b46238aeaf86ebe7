// Drop-in entry points with the reference's names and signatures, built on
// the batched solver and the survey kernels (one right-hand side per call,
// host buffers in and out, as the reference's callers use them).
//
// Call pattern of the reference (src/do_modelling.c:49-67, src/fg_fwi.c:
// 183-263): gmg_init -> inject_* -> gmg_apply -> extract_* -> gmg_free per
// frequency.  gmg_init builds the device solver for (emf, ifreq); inject_*,
// gmg_apply and extract_* reuse it; gmg_free releases it.  Errors end the
// process with a message, as the reference's err() does (src/cstd.c).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "emmi_dropin.h"
#include "emmi_gpu.h"
#include "emmi_solver_impl.cuh"

// the host program's SU-style parameter readers (src/cstd.c), when linked
extern "C" int getparint(char* name, int* p) __attribute__((weak));
extern "C" int getpardouble(char* name, double* p) __attribute__((weak));

extern "C" int emmi_inject_sources_multi_dev(emmi_solver* s, const float* src_dev, int nsrc,
                                             int nch, const int* ch, double* b_dev);

namespace {

struct DropinState {
  emmi_emf_t* emf = nullptr;
  int ifreq = 0;
  emmi_solver* s = nullptr;
  emmi_options opt;
  bool have_opt = false;
  int last_status = EMMI_SOLVE_OK, last_cycles = 0;
  double last_rel = 0;
  std::map<std::string, double> params;
};
DropinState g;

[[noreturn]] void die(const char* what) {
  fprintf(stderr, "libemmi_gpu: %s: %s\n", what, emmi_last_error());
  exit(1);
}

double param(const char* key, double def, bool integer) {
  auto it = g.params.find(key);
  if (it != g.params.end()) return it->second;
  if (integer && getparint) {
    int v;
    if (getparint(const_cast<char*>(key), &v)) return v;
  } else if (!integer && getpardouble) {
    double v;
    if (getpardouble(const_cast<char*>(key), &v)) return v;
  }
  return def;
}

int channel_code(const char* name) {
  static const char* names[6] = {"Ex", "Ey", "Ez", "Hx", "Hy", "Hz"};
  for (int i = 0; i < 6; i++)
    if (strcmp(name, names[i]) == 0) return i;
  return -1;
}

std::vector<int> channels(int n, char** names) {
  std::vector<int> c;
  for (int i = 0; i < n; i++) {
    const int k = channel_code(names[i]);
    if (k >= 0) c.push_back(k);
  }
  return c;
}

long nslots(const emmi_emf_t* e) { return (long)(e->n1 + 1) * (e->n2 + 1) * (e->n3 + 1); }

emmi_solver* solver_for(emmi_emf_t* emf, int ifreq) {
  if (g.s && g.emf == emf && g.ifreq == ifreq) return g.s;
  if (g.s) {
    emmi_solver_destroy(g.s);
    g.s = nullptr;
  }
  if (!g.have_opt) {
    emmi_default_options(&g.opt);
    g.have_opt = true;
  }
  g.emf = emf;
  g.ifreq = ifreq;
  const long nc = (long)emf->n1 * emf->n2 * emf->n3;
  std::vector<float> cells(4 * nc);
  float*** src[4] = {emf->sigma11, emf->sigma22, emf->sigma33, emf->invmur};
  for (int a = 0; a < 4; a++) memcpy(cells.data() + a * nc, &src[a][0][0][0], nc * sizeof(float));
  const float om = emf->omegas[ifreq];
  const float rw = emf->rho_water;
  emmi_problem P;
  P.n1 = emf->n1;
  P.n2 = emf->n2;
  P.n3 = emf->n3;
  P.nop = 1;
  P.nrhs = 1;
  P.x1 = emf->x1;
  P.x2 = emf->x2;
  P.x3 = emf->x3;
  P.cells = cells.data();
  P.op = nullptr;
  P.omega = &om;
  P.rho_water = &rw;
  if (emmi_solver_create(&g.s, &P, &g.opt) != EMMI_OK) die("gmg_init");
  return g.s;
}

template <typename T>
T* dev_copy(const T* h, size_t n, cudaStream_t st) {
  T* d = nullptr;
  if (cudaMallocAsync((void**)&d, n * sizeof(T) + 16, st) != cudaSuccess) die("device allocation");
  if (n && cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, st) != cudaSuccess)
    die("host to device copy");
  return d;
}

void sync(cudaStream_t st, const char* what) {
  if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) die(what);
}

std::vector<float> receivers(const emmi_acq_t* acq) {
  std::vector<float> r((size_t)acq->nrec * 5);
  for (int i = 0; i < acq->nrec; i++) {
    r[5 * i + 0] = acq->rec_x1[i];
    r[5 * i + 1] = acq->rec_x2[i];
    r[5 * i + 2] = acq->rec_x3[i];
    r[5 * i + 3] = acq->rec_azimuth[i];
    r[5 * i + 4] = acq->rec_dip[i];
  }
  return r;
}

}  // namespace

extern "C" {

// gmg.c:1712-1717: the multigrid knobs from the host's parameters
void emmi_dropin_options(emmi_options* o, int verb) {
  emmi_default_options(o);
  o->cycleopt = (int)param("cycleopt", 2, true);
  o->ncycle = (int)param("ncycle", 30, true);
  o->v1 = (int)param("v1", 1, true);
  o->v2 = (int)param("v2", 1, true);
  o->tol = param("tol", 1e-6, false);
  o->isemicoarsen = (int)param("isemicoarsen", 1, true);
  o->precision = (int)param("gmg_precision", EMMI_PREC_MIXED, true);
  o->sigma_floor = param("sigma_floor", 0.0, false);
  // level masks of left-out smoothing (0: the reference's cycle)
  o->skip_pre = (int)param("skip_pre", 0, true);
  o->skip_post = (int)param("skip_post", 0, true);
  o->verb = verb;
}

// gmg.c:1704-1733: knobs from the host's parameters, solver built here
void gmg_init(emmi_emf_t* emf, int ifreq) {
  if (g.s) {
    emmi_solver_destroy(g.s);
    g.s = nullptr;
  }
  emmi_dropin_options(&g.opt, emf->verb);
  g.have_opt = true;
  if (emf->verb) {
    printf("----------- gmg_init (GB300) ---------------\n");
    printf("cycleopt=%d ncycle=%d v1=%d v2=%d tol=%g isemicoarsen=%d precision=%s\n",
           g.opt.cycleopt, g.opt.ncycle, g.opt.v1, g.opt.v2, g.opt.tol, g.opt.isemicoarsen,
           g.opt.precision == EMMI_PREC_FP64 ? "complex128" : "complex64+fp64");
  }
  g.emf = nullptr;
  solver_for(emf, ifreq);
}

// gmg.c:1894-1932: x = E, b overwritten with H
void gmg_apply(int n, emmi_cf64* b, emmi_cf64* x) {
  if (!g.emf) {
    fprintf(stderr, "libemmi_gpu: gmg_apply before gmg_init\n");
    exit(1);
  }
  emmi_solver* s = solver_for(g.emf, g.ifreq);
  if ((long)n != 3 * nslots(g.emf)) {
    fprintf(stderr, "libemmi_gpu: gmg_apply: n=%d != 3*(n1+1)(n2+1)(n3+1)\n", n);
    exit(1);
  }
  emmi_rhs_stats st;
  if (emmi_solver_solve(s, (const double*)b, (double*)x, (double*)b, 0, &st) != EMMI_OK)
    die("gmg_apply");
  g.last_status = st.status;
  g.last_cycles = st.cycles;
  g.last_rel = st.rnorm0 > 0 ? st.rnorm / st.rnorm0 : 0;
}

void gmg_free(void) {
  if (g.s) emmi_solver_destroy(g.s);
  g.s = nullptr;
  g.emf = nullptr;
}

// inject_extract.c:26-120
void inject_source(emmi_acq_t* acq, emmi_emf_t* emf, emmi_cf64* b, int ifreq) {
  emmi_solver* s = solver_for(emf, ifreq);
  std::vector<float> src((size_t)acq->nsrc * 5);
  for (int i = 0; i < acq->nsrc; i++) {
    src[5 * i + 0] = acq->src_x1[i];
    src[5 * i + 1] = acq->src_x2[i];
    src[5 * i + 2] = acq->src_x3[i];
    src[5 * i + 3] = acq->src_azimuth[i];
    src[5 * i + 4] = acq->src_dip[i];
  }
  const std::vector<int> ch = channels(emf->nchsrc, emf->chsrc);
  const long n3s = 3 * nslots(emf);
  float* dsrc = dev_copy(src.data(), src.size(), s->st);
  double* db = nullptr;
  if (cudaMallocAsync((void**)&db, n3s * 2 * sizeof(double), s->st) != cudaSuccess) die("inject_source");
  if (ch.empty()) {
    cudaMemsetAsync(db, 0, n3s * 2 * sizeof(double), s->st);
  } else if (emmi_inject_sources_multi_dev(s, dsrc, acq->nsrc, (int)ch.size(), ch.data(), db) !=
             EMMI_OK) {
    die("inject_source");
  }
  cudaMemcpyAsync(b, db, n3s * 2 * sizeof(double), cudaMemcpyDeviceToHost, s->st);
  cudaFreeAsync(dsrc, s->st);
  cudaFreeAsync(db, s->st);
  sync(s->st, "inject_source");
}

// inject_extract.c:124-314 (x receives the magnetic-source scratch M)
void inject_adj_source(emmi_acq_t* acq, emmi_emf_t* emf, emmi_cf64* x, emmi_cf64* b, int ifreq) {
  emmi_solver* s = solver_for(emf, ifreq);
  const std::vector<int> ch = channels(emf->nchrec, emf->chrec);
  const long n3s = 3 * nslots(emf);
  const std::vector<float> rec = receivers(acq);
  // residual slice of this frequency: dres_fd[ic][ifreq][irec]
  std::vector<float> dres((size_t)std::max<size_t>(ch.size(), 1) * acq->nrec * 2, 0.f);
  const float* all = (const float*)&emf->dres_fd[0][0][0];
  int k = 0;
  for (int ic = 0; ic < emf->nchrec; ic++) {
    if (channel_code(emf->chrec[ic]) < 0) continue;
    memcpy(dres.data() + (size_t)k * acq->nrec * 2,
           all + ((size_t)ic * emf->nfreq + ifreq) * acq->nrec * 2, acq->nrec * 2 * sizeof(float));
    k++;
  }
  float* drec = dev_copy(rec.data(), rec.size(), s->st);
  float* dd = dev_copy(dres.data(), dres.size(), s->st);
  double *db = nullptr, *dm = nullptr;
  if (cudaMallocAsync((void**)&db, n3s * 2 * sizeof(double), s->st) != cudaSuccess ||
      cudaMallocAsync((void**)&dm, n3s * 2 * sizeof(double), s->st) != cudaSuccess)
    die("inject_adj_source");
  if (ch.empty()) {
    cudaMemsetAsync(db, 0, n3s * 2 * sizeof(double), s->st);
    cudaMemsetAsync(dm, 0, n3s * 2 * sizeof(double), s->st);
  } else if (emmi_inject_adjoint_dev(s, drec, acq->nrec, (int)ch.size(), ch.data(), dd, db, dm) !=
             EMMI_OK) {
    die("inject_adj_source");
  }
  cudaMemcpyAsync(b, db, n3s * 2 * sizeof(double), cudaMemcpyDeviceToHost, s->st);
  cudaMemcpyAsync(x, dm, n3s * 2 * sizeof(double), cudaMemcpyDeviceToHost, s->st);
  cudaFreeAsync(drec, s->st);
  cudaFreeAsync(dd, s->st);
  cudaFreeAsync(db, s->st);
  cudaFreeAsync(dm, s->st);
  sync(s->st, "inject_adj_source");
}

// inject_extract.c:317-474 -> emf->dcal_fd[ic][ifreq][irec]
void extract_emf_data(emmi_acq_t* acq, emmi_emf_t* emf, emmi_cf64* x, emmi_cf64* b, int ifreq) {
  emmi_solver* s = solver_for(emf, ifreq);
  const long n3s = 3 * nslots(emf);
  const std::vector<float> rec = receivers(acq);
  std::vector<int> ch;
  std::vector<int> slot;  // dcal channel index of each extracted channel
  for (int ic = 0; ic < emf->nchrec; ic++) {
    const int k = channel_code(emf->chrec[ic]);
    if (k >= 0) {
      ch.push_back(k);
      slot.push_back(ic);
    }
  }
  if (ch.empty() || acq->nrec == 0) return;
  float* drec = dev_copy(rec.data(), rec.size(), s->st);
  double* dx = dev_copy((const double*)x, n3s * 2, s->st);
  double* dh = dev_copy((const double*)b, n3s * 2, s->st);
  float* dout = nullptr;
  if (cudaMallocAsync((void**)&dout, ch.size() * acq->nrec * 2 * sizeof(float), s->st) != cudaSuccess)
    die("extract_emf_data");
  if (emmi_extract_receivers_dev(s, drec, acq->nrec, (int)ch.size(), ch.data(), dx, dh, dout) !=
      EMMI_OK)
    die("extract_emf_data");
  std::vector<float> out(ch.size() * acq->nrec * 2);
  cudaMemcpyAsync(out.data(), dout, out.size() * sizeof(float), cudaMemcpyDeviceToHost, s->st);
  cudaFreeAsync(drec, s->st);
  cudaFreeAsync(dx, s->st);
  cudaFreeAsync(dh, s->st);
  cudaFreeAsync(dout, s->st);
  sync(s->st, "extract_emf_data");
  float* dc = (float*)&emf->dcal_fd[0][0][0];
  for (size_t k = 0; k < ch.size(); k++)
    memcpy(dc + ((size_t)slot[k] * emf->nfreq + ifreq) * acq->nrec * 2,
           out.data() + k * acq->nrec * 2, acq->nrec * 2 * sizeof(float));
}

static void extract_volume(emmi_emf_t* emf, int ifreq, int which, const emmi_cf64* field,
                           emmi_cf32**** o1, emmi_cf32**** o2, emmi_cf32**** o3) {
  emmi_solver* s = solver_for(emf, ifreq);
  const long nxyz = (long)emf->nx * emf->ny * emf->nz;
  std::vector<float> out(3 * nxyz * 2);
  const float o[3] = {emf->ox, emf->oy, emf->oz};
  const float d[3] = {emf->dx, emf->dy, emf->dz};
  if (emmi_extract_volume(s, 0, which, emf->nx, emf->ny, emf->nz, o, d,
                          which == 0 ? &emf->rho33[0][0][0] : nullptr, (const double*)field,
                          out.data()) != EMMI_OK)
    die(which == 0 ? "extract_electric_field" : "extract_magnetic_field");
  emmi_cf32**** dst[3] = {o1, o2, o3};
  for (int c = 0; c < 3; c++)
    memcpy(&dst[c][ifreq][0][0][0], out.data() + (size_t)c * nxyz * 2, nxyz * 2 * sizeof(float));
}

// inject_extract.c:477-635
void extract_electric_field(emmi_acq_t* acq, emmi_emf_t* emf, emmi_cf64* x, int ifreq) {
  (void)acq;
  extract_volume(emf, ifreq, 0, x, emf->E1, emf->E2, emf->E3);
}

// inject_extract.c:638-785
void extract_magnetic_field(emmi_acq_t* acq, emmi_emf_t* emf, emmi_cf64* b, int ifreq) {
  (void)acq;
  extract_volume(emf, ifreq, 1, b, emf->H1, emf->H2, emf->H3);
}

// build_gradient.c:13-113 (one shot per process, as the reference)
void build_gradient(emmi_acq_t* acq, emmi_emf_t* emf, emmi_fwi_t* fwi, emmi_cf32**** E1f,
                    emmi_cf32**** E2f, emmi_cf32**** E3f, emmi_cf32**** E1a, emmi_cf32**** E2a,
                    emmi_cf32**** E3a) {
  const float o[3] = {emf->ox, emf->oy, emf->oz};
  const float d[3] = {emf->dx, emf->dy, emf->dz};
  const float src[3] = {acq->src_x1[0], acq->src_x2[0], acq->src_x3[0]};
  std::vector<float> rec((size_t)acq->nrec * 3);
  for (int i = 0; i < acq->nrec; i++) {
    rec[3 * i] = acq->rec_x1[i];
    rec[3 * i + 1] = acq->rec_x2[i];
    rec[3 * i + 2] = acq->rec_x3[i];
  }
  if (emmi_build_gradient(emf->nx, emf->ny, emf->nz, o, d, 1, emf->nfreq, fwi->npar, fwi->idxpar,
                          fwi->preco, (const float*)&E1f[0][0][0][0],
                          (const float*)&E2f[0][0][0][0], (const float*)&E3f[0][0][0][0],
                          (const float*)&E1a[0][0][0][0], (const float*)&E2a[0][0][0][0],
                          (const float*)&E3a[0][0][0][0], &emf->rho11[0][0][0],
                          &emf->rho33[0][0][0], &emf->bathy[0][0], src, emf->dsmute, acq->nrec,
                          rec.data(), emf->drmute, &fwi->grad[0][0][0][0],
                          fwi->preco == 1 ? &fwi->phess[0][0][0][0] : nullptr) != EMMI_OK)
    die("build_gradient");
}

int emmi_gpu_last_status(int* cycles, double* rel) {
  if (cycles) *cycles = g.last_cycles;
  if (rel) *rel = g.last_rel;
  return g.last_status;
}

int emmi_gpu_set_param(const char* key, double value) {
  if (!key) return EMMI_EINVAL;
  g.params[key] = value;
  return EMMI_OK;
}

}  // extern "C"

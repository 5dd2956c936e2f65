// glasma_abi.cu -- the C ABI (include/glasma_gb300.h): handle, device memory, host copies
// and the orchestration of the kernels for each reference entry point.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "../../include/glasma_gb300.h"
#include "handle.h"

using glasma::cx;
using glasma::FieldPtrs;
using glasma::Geometry;


namespace {

thread_local std::string g_last_error;

int fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

}  // namespace

namespace glasma {
// records msg as glasma_last_error() of the calling thread (for entry points in other files)
int record_error(int status, const std::string& msg) { return fail(status, msg); }

// The plaquette method's contribution buffer (every slot a step reads is written earlier in it).
bool ensure_contrib(glasma_lattice* h) {
  if (h->contrib) return true;
  if (cudaMalloc(&h->contrib, (size_t)h->g.S * 48 * h->real_bytes) != cudaSuccess) {
    cudaGetLastError();
    h->contrib = nullptr;
    return false;
  }
  return true;
}
}  // namespace glasma

namespace {

int cuda_fail(cudaError_t e, const char* where) {
  return fail(GLASMA_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define GLASMA_CUDA(call, where)                 \
  do {                                            \
    cudaError_t _e = (call);                      \
    if (_e != cudaSuccess) return cuda_fail(_e, where); \
  } while (0)

#define GLASMA_CHECK_HANDLE(h)                                                  \
  do {                                                                          \
    if (!(h)) return fail(GLASMA_ERR_INVALID_ARGUMENT, "null lattice handle");  \
    cudaError_t _d = cudaSetDevice((h)->device);                                \
    if (_d != cudaSuccess) return cuda_fail(_d, "cudaSetDevice");               \
  } while (0)

// Components per site on the device side, and doubles per site in the host layout.
int field_components(int field) {  // number of SoA component arrays (complex ones count once)
  switch (field) {
    case GLASMA_FIELD_U:
    case GLASMA_FIELD_UOLD:
    case GLASMA_FIELD_UG: return 27;
    case GLASMA_FIELD_G: return 9;
    case GLASMA_FIELD_E:
    case GLASMA_FIELD_EG: return 24;
    default: return 8;
  }
}
bool field_is_complex(int field) {
  return field == GLASMA_FIELD_U || field == GLASMA_FIELD_UOLD || field == GLASMA_FIELD_UG || field == GLASMA_FIELD_G;
}
int host_doubles_per_site(int field) { return field_components(field) * (field_is_complex(field) ? 2 : 1); }

size_t field_bytes(const glasma_lattice* h, int field) {
  return (size_t)h->g.S * (size_t)host_doubles_per_site(field) * h->real_bytes;
}

template <typename T>
FieldPtrs<T> ptrs(glasma_lattice* h) {
  FieldPtrs<T> p;
  p.U = static_cast<cx<T>*>(h->f[GLASMA_FIELD_U]);
  p.UOld = static_cast<cx<T>*>(h->f[GLASMA_FIELD_UOLD]);
  p.E = static_cast<T*>(h->f[GLASMA_FIELD_E]);
  p.Jp = static_cast<T*>(h->f[GLASMA_FIELD_JP]);
  p.Jm = static_cast<T*>(h->f[GLASMA_FIELD_JM]);
  p.JpStat = static_cast<T*>(h->f[GLASMA_FIELD_JPSTAT]);
  p.JmStat = static_cast<T*>(h->f[GLASMA_FIELD_JMSTAT]);
  return p;
}

// Buffers of the one-pass step's second set: the fields it writes (U, the four currents).
constexpr int kSwapFields[5] = {GLASMA_FIELD_U, GLASMA_FIELD_JP, GLASMA_FIELD_JM, GLASMA_FIELD_JPSTAT,
                                GLASMA_FIELD_JMSTAT};

// FieldPtrs of the second set: E and UOld are shared with the first.
template <typename T>
FieldPtrs<T> alt_ptrs(glasma_lattice* h) {
  FieldPtrs<T> p = ptrs<T>(h);
  p.U = static_cast<cx<T>*>(h->alt[GLASMA_FIELD_U]);
  p.Jp = static_cast<T*>(h->alt[GLASMA_FIELD_JP]);
  p.Jm = static_cast<T*>(h->alt[GLASMA_FIELD_JM]);
  p.JpStat = static_cast<T*>(h->alt[GLASMA_FIELD_JPSTAT]);
  p.JmStat = static_cast<T*>(h->alt[GLASMA_FIELD_JMSTAT]);
  return p;
}

// Allocates the second set (contents need no initialisation: every step writes all of it, ghost
// slices included).  False, with nothing left allocated, when device memory is short.
bool ensure_alt(glasma_lattice* h) {
  for (int f : kSwapFields) {
    if (h->alt[f]) continue;
    void* p = nullptr;
    if (cudaMalloc(&p, field_bytes(h, f)) != cudaSuccess) {
      cudaGetLastError();
      for (int k : kSwapFields) {
        if (h->alt[k]) cudaFree(h->alt[k]);
        h->alt[k] = nullptr;
      }
      return false;
    }
    h->alt[f] = p;
  }
  return true;
}

using glasma::ensure_contrib;

void swap_buffers(glasma_lattice* h) {
  for (int f : kSwapFields) std::swap(h->f[f], h->alt[f]);
  h->swaps++;
}

// identity links / zero fields, ghost slices included
template <typename T>
__global__ void init_identity_kernel(cx<T>* U, long long S, int nmat) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = S * 9 * nmat;
  if (i >= n) return;
  const long long comp = i / S;
  const int k = (int)(comp % 9);
  cx<T> v;
  v.re = (k == 0 || k == 4 || k == 8) ? T(1) : T(0);
  v.im = T(0);
  U[i] = v;
}

int ensure_field(glasma_lattice* h, int field) {
  if (h->f[field]) return GLASMA_OK;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, field_bytes(h, field));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(GLASMA_ERR_OUT_OF_MEMORY, std::string("cudaMalloc field: ") + cudaGetErrorString(e));
  }
  h->f[field] = p;
  if (field_is_complex(field)) {
    const int nmat = field_components(field) / 9;
    const long long n = h->g.S * 9 * nmat;
    const unsigned grid = (unsigned)((n + 255) / 256);
    if (h->precision == GLASMA_FP64)
      init_identity_kernel<double><<<grid, 256, 0, h->stream>>>(static_cast<cx<double>*>(p), h->g.S, nmat);
    else
      init_identity_kernel<float><<<grid, 256, 0, h->stream>>>(static_cast<cx<float>*>(p), h->g.S, nmat);
    GLASMA_CUDA(cudaGetLastError(), "init identity");
  } else {
    GLASMA_CUDA(cudaMemsetAsync(p, 0, field_bytes(h, field), h->stream), "cudaMemsetAsync");
  }
  return GLASMA_OK;
}

int ensure_staging(glasma_lattice* h, size_t bytes) {
  if (h->staging_bytes >= bytes) return GLASMA_OK;
  if (h->staging) {
    cudaStreamSynchronize(h->stream);
    cudaFree(h->staging);
    h->staging = nullptr;
    h->staging_bytes = 0;
  }
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(GLASMA_ERR_OUT_OF_MEMORY, std::string("cudaMalloc staging: ") + cudaGetErrorString(e));
  }
  h->staging = static_cast<double*>(p);
  h->staging_bytes = bytes;
  return GLASMA_OK;
}

int ensure_scratch(glasma_lattice* h) {
  size_t need = (size_t)glasma::observable_scratch_doubles(h->g) + (size_t)h->g.nz * 16 + 64;
  if (need < glasma::gaugefix_scratch_doubles()) need = glasma::gaugefix_scratch_doubles();
  if (h->scratch_doubles >= need) return GLASMA_OK;
  if (h->scratch) {
    cudaStreamSynchronize(h->stream);
    cudaFree(h->scratch);
    h->scratch = nullptr;
  }
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, need * sizeof(double));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(GLASMA_ERR_OUT_OF_MEMORY, std::string("cudaMalloc scratch: ") + cudaGetErrorString(e));
  }
  h->scratch = static_cast<double*>(p);
  h->scratch_doubles = need;
  return GLASMA_OK;
}

bool valid_field(int field) { return field >= GLASMA_FIELD_U && field <= GLASMA_FIELD_EG; }

int sync_field_ghosts(glasma_lattice* h, int field) {
  cudaError_t e;
  const int comps = field_components(field);
  if (h->precision == GLASMA_FP64) {
    if (field_is_complex(field))
      e = glasma::launch_sync_ghosts<cx<double>>(h->g, static_cast<cx<double>*>(h->f[field]), comps, h->stream);
    else
      e = glasma::launch_sync_ghosts<double>(h->g, static_cast<double*>(h->f[field]), comps, h->stream);
  } else {
    if (field_is_complex(field))
      e = glasma::launch_sync_ghosts<cx<float>>(h->g, static_cast<cx<float>*>(h->f[field]), comps, h->stream);
    else
      e = glasma::launch_sync_ghosts<float>(h->g, static_cast<float*>(h->f[field]), comps, h->stream);
  }
  if (e != cudaSuccess) return cuda_fail(e, "ghost sync");
  return GLASMA_OK;
}

// Results come back through a small page-locked, mapped buffer that a kernel writes: a device-to-host
// cudaMemcpy (into the caller's pageable memory) queued behind the copy engines' uploads of
// glasma_upload_begin and waited for all of them, so a step's result read serialised the next step's
// input copies with the step.
constexpr size_t kResultDoubles = 8192;
__global__ void result_copy_kernel(const double* __restrict__ src, double* __restrict__ dst, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

int copy_results_to_host(glasma_lattice* h, const double* dev, double* host, size_t n) {
  if (!h->result_host) {
    void* p = nullptr;
    GLASMA_CUDA(cudaHostAlloc(&p, kResultDoubles * sizeof(double), cudaHostAllocMapped), "result buffer");
    void* d = nullptr;
    cudaError_t e = cudaHostGetDevicePointer(&d, p, 0);
    if (e != cudaSuccess) {
      cudaFreeHost(p);
      return cuda_fail(e, "result buffer address");
    }
    h->result_host = static_cast<double*>(p);
    h->result_dev = static_cast<double*>(d);
  }
  for (size_t done = 0; done < n; done += kResultDoubles) {
    const size_t m = n - done < kResultDoubles ? n - done : kResultDoubles;
    result_copy_kernel<<<1, 256, 0, h->stream>>>(dev + done, h->result_dev, (int)m);
    GLASMA_CUDA(cudaGetLastError(), "result copy");
    GLASMA_CUDA(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
    std::memcpy(host + done, h->result_host, m * sizeof(double));
  }
  return GLASMA_OK;
}

// 12-real links: the step kernels left row 2 of every link stale; write it from rows 0 and 1 so that
// every other kernel and the downloads see full links between calls.
template <typename T>
int complete_links(glasma_lattice* h) {
  if (h->link_rows != 2) return GLASMA_OK;
  cudaError_t e = glasma::launch_complete_links<T>(h->g, static_cast<cx<T>*>(h->f[GLASMA_FIELD_U]), h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "complete links");
  return GLASMA_OK;
}

// When `ev` is non-null it holds 3 events per step (before K1, between K1 and K2, after K2),
// recorded on the handle's stream.
template <typename T>
int step_impl(glasma_lattice* h, double dt, int nsteps, unsigned flags, cudaEvent_t* ev = nullptr) {
  FieldPtrs<T> p = ptrs<T>(h);
  // UpdateElectricFields starts with U->SynchronizeGhostCells() (S/DYNAMICS/SUNcDynamics.cpp:151);
  // the fused kernels keep every ghost slice in sync after that.
  cudaError_t e = glasma::launch_sync_ghosts<cx<T>>(h->g, p.U, 27, h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "ghost sync U");
  if (h->step_method == GLASMA_STEP_ONE_PASS && ensure_alt(h)) {
    h->last_method = GLASMA_STEP_ONE_PASS;
    for (int n = 0; n < nsteps; n++) {
      if (ev) cudaEventRecord(ev[3 * n], h->stream);
      const bool save = (flags & GLASMA_STEP_SAVE_UOLD) && (n == nsteps - 1);
      e = glasma::launch_fused_step<T>(h->g, ptrs<T>(h), alt_ptrs<T>(h), dt, save, h->tile_x, false, h->stream,
                                       h->link_rows);
      if (e != cudaSuccess) return cuda_fail(e, "fused step");
      if (ev) {
        cudaEventRecord(ev[3 * n + 1], h->stream);
        cudaEventRecord(ev[3 * n + 2], h->stream);
      }
      swap_buffers(h);
      h->steps_done++;
      if (h->reunit_every > 0 && h->steps_done % h->reunit_every == 0) {
        e = glasma::launch_reunitarize<T>(h->g, static_cast<cx<T>*>(h->f[GLASMA_FIELD_U]), h->stream, h->link_rows);
        if (e != cudaSuccess) return cuda_fail(e, "reunitarize");
      }
    }
    return complete_links<T>(h);
  }
  if (h->step_method == GLASMA_STEP_MARCH && ensure_alt(h)) {
    h->last_method = GLASMA_STEP_MARCH;
    for (int n = 0; n < nsteps; n++) {
      if (ev) cudaEventRecord(ev[3 * n], h->stream);
      const bool save = (flags & GLASMA_STEP_SAVE_UOLD) && (n == nsteps - 1);
      e = glasma::launch_march_step<T>(h->g, ptrs<T>(h), alt_ptrs<T>(h), dt, save, h->march_lz, h->stream,
                                       h->link_rows);
      if (e != cudaSuccess) return cuda_fail(e, "march step");
      if (ev) {
        cudaEventRecord(ev[3 * n + 1], h->stream);
        cudaEventRecord(ev[3 * n + 2], h->stream);
      }
      swap_buffers(h);
      h->steps_done++;
      if (h->reunit_every > 0 && h->steps_done % h->reunit_every == 0) {
        e = glasma::launch_reunitarize<T>(h->g, static_cast<cx<T>*>(h->f[GLASMA_FIELD_U]), h->stream, h->link_rows);
        if (e != cudaSuccess) return cuda_fail(e, "reunitarize");
      }
    }
    return complete_links<T>(h);
  }
  if (h->step_method == GLASMA_STEP_PLAQUETTE && ensure_contrib(h)) {
    h->last_method = GLASMA_STEP_PLAQUETTE;
    for (int n = 0; n < nsteps; n++) {
      if (ev) cudaEventRecord(ev[3 * n], h->stream);
      const bool save = (flags & GLASMA_STEP_SAVE_UOLD) && (n == nsteps - 1);
      e = glasma::launch_plaquette_step<T>(h->g, p, static_cast<T*>(h->contrib), dt, save, h->stream,
                                           ev ? ev[3 * n + 1] : nullptr, h->link_rows,
                                           h->fp64_arith == GLASMA_FP64_DOUBLE_FLOAT);
      if (e != cudaSuccess) return cuda_fail(e, "plaquette step");
      if (ev) cudaEventRecord(ev[3 * n + 2], h->stream);
      h->steps_done++;
      if (h->reunit_every > 0 && h->steps_done % h->reunit_every == 0) {
        e = glasma::launch_reunitarize<T>(h->g, p.U, h->stream, h->link_rows);
        if (e != cudaSuccess) return cuda_fail(e, "reunitarize");
      }
    }
    return complete_links<T>(h);
  }
  h->last_method = GLASMA_STEP_TWO_PASS;
  for (int n = 0; n < nsteps; n++) {
    if (ev) cudaEventRecord(ev[3 * n], h->stream);
    e = glasma::launch_efield_jstat<T>(h->g, p, dt, h->tile_x, h->stream, h->link_rows);
    if (e != cudaSuccess) return cuda_fail(e, "efield_jstat");
    if (ev) cudaEventRecord(ev[3 * n + 1], h->stream);
    const bool save = (flags & GLASMA_STEP_SAVE_UOLD) && (n == nsteps - 1);
    e = glasma::launch_links_j<T>(h->g, p, dt, save, true, true, h->stream, h->link_rows);
    if (e != cudaSuccess) return cuda_fail(e, "links_j");
    if (ev) cudaEventRecord(ev[3 * n + 2], h->stream);
    h->steps_done++;
    if (h->reunit_every > 0 && h->steps_done % h->reunit_every == 0) {
      e = glasma::launch_reunitarize<T>(h->g, p.U, h->stream, h->link_rows);
      if (e != cudaSuccess) return cuda_fail(e, "reunitarize");
    }
  }
  return complete_links<T>(h);
}

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" {

const char* glasma_last_error(void) { return g_last_error.c_str(); }

const char* glasma_status_string(int status) {
  switch (status) {
    case GLASMA_OK: return "ok";
    case GLASMA_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GLASMA_ERR_BAD_SHAPE: return "bad lattice shape";
    case GLASMA_ERR_OUT_OF_MEMORY: return "out of device memory";
    case GLASMA_ERR_CUDA: return "CUDA error";
    case GLASMA_ERR_NUMERICAL: return "numerical guard fired";
    case GLASMA_ERR_TIMEOUT: return "device wait timed out";
    case GLASMA_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

int glasma_create(int nx, int ny, int nz, double ax, double ay, double az, int precision, int reunitarize_every,
                  glasma_lattice** out) {
  if (!out) return fail(GLASMA_ERR_INVALID_ARGUMENT, "out is null");
  *out = nullptr;
  if (nx < 2 || ny < 2 || nz < 2) return fail(GLASMA_ERR_BAD_SHAPE, "each extent must be >= 2");
  if ((long long)nx * ny * (nz + 2) > (1LL << 40)) return fail(GLASMA_ERR_BAD_SHAPE, "lattice too large");
  if (!(ax > 0) || !(ay > 0) || !(az > 0)) return fail(GLASMA_ERR_BAD_SHAPE, "spacings must be positive");
  if (precision != GLASMA_FP64 && precision != GLASMA_FP32) return fail(GLASMA_ERR_INVALID_ARGUMENT, "unknown precision");
  if (reunitarize_every < 0) return fail(GLASMA_ERR_INVALID_ARGUMENT, "reunitarize_every < 0");
  glasma_lattice* h = new glasma_lattice;
  std::memset(h, 0, sizeof(*h));
  h->g.nx = nx;
  h->g.ny = ny;
  h->g.nz = nz;
  h->g.plane = (long long)nx * ny;
  h->g.S = h->g.plane * (nz + 2);
  h->g.vol = h->g.plane * nz;
  h->g.a[0] = ax;
  h->g.a[1] = ay;
  h->g.a[2] = az;
  h->precision = precision;
  h->reunit_every = precision == GLASMA_FP32 ? reunitarize_every : 0;
  h->a_scale = 1.0;
  h->real_bytes = precision == GLASMA_FP64 ? 8 : 4;
  h->tile_x = glasma::default_tile_x(nx);
  // the plaquette method: ~25 % fewer matrix products in the force (FP64 step 75.5 -> 68.2 ms on GB300
  // at 128x128x512); falls back to two-pass when its buffer cannot be allocated
  h->step_method = GLASMA_STEP_PLAQUETTE;
  h->march_lz = 0;
  h->link_rows = 3;
  h->fp64_arith = GLASMA_FP64_NATIVE;
  h->last_method = GLASMA_STEP_TWO_PASS;
  cudaError_t e = cudaGetDevice(&h->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete h;
    return cuda_fail(e, "create");
  }
  h->stream = h->own_stream;
  for (int f = GLASMA_FIELD_U; f <= GLASMA_FIELD_JMSTAT; f++) {
    int st = ensure_field(h, f);
    if (st != GLASMA_OK) {
      glasma_destroy(h);
      return st;
    }
  }
  e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    glasma_destroy(h);
    return cuda_fail(e, "create sync");
  }
  *out = h;
  return GLASMA_OK;
}

int glasma_destroy(glasma_lattice* h) {
  if (!h) return GLASMA_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (int i = 0; i < 10; i++) {
    if (h->f[i]) cudaFree(h->f[i]);
    if (h->alt[i]) cudaFree(h->alt[i]);
  }
  if (h->contrib) cudaFree(h->contrib);
  if (h->staging) cudaFree(h->staging);
  if (h->scratch) cudaFree(h->scratch);
  if (h->result_host) cudaFreeHost(h->result_host);
  if (h->xfer_stream) cudaStreamSynchronize(h->xfer_stream);
  for (int b = 0; b < 2; b++) {
    for (int i = 0; i < 10; i++)
      if (h->stage_f[b][i]) cudaFree(h->stage_f[b][i]);
    if (h->stage_free[b]) cudaEventDestroy(h->stage_free[b]);
  }
  if (h->xfer_done) cudaEventDestroy(h->xfer_done);
  if (h->xfer_stream) cudaStreamDestroy(h->xfer_stream);
  glasma::gaugefix_destroy(h->gf);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
  return GLASMA_OK;
}

int glasma_set_stream(glasma_lattice* h, void* stream) {
  GLASMA_CHECK_HANDLE(h);
  GLASMA_CUDA(cudaStreamSynchronize(h->stream), "sync old stream");
  h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
  return GLASMA_OK;
}

int glasma_set_scale(glasma_lattice* h, double a_scale) {
  if (!h) return fail(GLASMA_ERR_INVALID_ARGUMENT, "null lattice handle");
  if (!(a_scale > 0)) return fail(GLASMA_ERR_INVALID_ARGUMENT, "a_scale must be positive");
  h->a_scale = a_scale;
  return GLASMA_OK;
}

int glasma_get_shape(const glasma_lattice* h, int* nx, int* ny, int* nz, int* precision) {
  if (!h) return fail(GLASMA_ERR_INVALID_ARGUMENT, "null lattice handle");
  if (nx) *nx = h->g.nx;
  if (ny) *ny = h->g.ny;
  if (nz) *nz = h->g.nz;
  if (precision) *precision = h->precision;
  return GLASMA_OK;
}

long long glasma_field_doubles(const glasma_lattice* h, int field) {
  if (!h || !valid_field(field)) return -1;
  return h->g.S * host_doubles_per_site(field);
}

// Device address of page-locked (pinned or registered) host memory, else null.  Such memory is
// read and written in place by the layout kernels over the host link (NVLink-C2C on Grace
// systems), fusing the copy with the AoS <-> SoA conversion; pageable memory goes through the
// staging buffer with cudaMemcpyAsync.
static void* mapped_host(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

static int upload_common(glasma_lattice* h, int field, const double* src, cudaMemcpyKind kind) {
  GLASMA_CHECK_HANDLE(h);
  if (!valid_field(field)) return fail(GLASMA_ERR_INVALID_ARGUMENT, "unknown field");
  if (!src) return fail(GLASMA_ERR_INVALID_ARGUMENT, "null source");
  int st = ensure_field(h, field);
  if (st) return st;
  const int P = host_doubles_per_site(field);
  const size_t bytes = (size_t)h->g.S * P * sizeof(double);
  if (kind == cudaMemcpyHostToDevice) {
    if (const double* dsrc = static_cast<const double*>(mapped_host(src))) {
      cudaError_t e = h->precision == GLASMA_FP64
                          ? glasma::launch_aos_to_soa<double>(dsrc, static_cast<double*>(h->f[field]), h->g.S, P, h->stream)
                          : glasma::launch_aos_to_soa<float>(dsrc, static_cast<float*>(h->f[field]), h->g.S, P, h->stream);
      return e == cudaSuccess ? GLASMA_OK : cuda_fail(e, "aos_to_soa from host");
    }
  }
  st = ensure_staging(h, bytes);
  if (st) return st;
  GLASMA_CUDA(cudaMemcpyAsync(h->staging, src, bytes, kind, h->stream), "upload copy");
  cudaError_t e = h->precision == GLASMA_FP64
                      ? glasma::launch_aos_to_soa<double>(h->staging, static_cast<double*>(h->f[field]), h->g.S, P, h->stream)
                      : glasma::launch_aos_to_soa<float>(h->staging, static_cast<float*>(h->f[field]), h->g.S, P, h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "aos_to_soa");
  return GLASMA_OK;
}

static int download_common(glasma_lattice* h, int field, double* dst, cudaMemcpyKind kind) {
  GLASMA_CHECK_HANDLE(h);
  if (!valid_field(field)) return fail(GLASMA_ERR_INVALID_ARGUMENT, "unknown field");
  if (!dst) return fail(GLASMA_ERR_INVALID_ARGUMENT, "null destination");
  int st = ensure_field(h, field);
  if (st) return st;
  const int P = host_doubles_per_site(field);
  const size_t bytes = (size_t)h->g.S * P * sizeof(double);
  if (kind == cudaMemcpyDeviceToHost) {
    if (double* ddst = static_cast<double*>(mapped_host(dst))) {
      cudaError_t e = h->precision == GLASMA_FP64
                          ? glasma::launch_soa_to_aos<double>(static_cast<const double*>(h->f[field]), ddst, h->g.S, P, h->stream)
                          : glasma::launch_soa_to_aos<float>(static_cast<const float*>(h->f[field]), ddst, h->g.S, P, h->stream);
      if (e != cudaSuccess) return cuda_fail(e, "soa_to_aos to host");
      GLASMA_CUDA(cudaStreamSynchronize(h->stream), "download sync");
      return GLASMA_OK;
    }
  }
  st = ensure_staging(h, bytes);
  if (st) return st;
  cudaError_t e = h->precision == GLASMA_FP64
                      ? glasma::launch_soa_to_aos<double>(static_cast<const double*>(h->f[field]), h->staging, h->g.S, P, h->stream)
                      : glasma::launch_soa_to_aos<float>(static_cast<const float*>(h->f[field]), h->staging, h->g.S, P, h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "soa_to_aos");
  GLASMA_CUDA(cudaMemcpyAsync(dst, h->staging, bytes, kind, h->stream), "download copy");
  GLASMA_CUDA(cudaStreamSynchronize(h->stream), "download sync");
  return GLASMA_OK;
}

int glasma_upload_begin(glasma_lattice* h, int field, const double* host) {
  GLASMA_CHECK_HANDLE(h);
  if (!valid_field(field)) return fail(GLASMA_ERR_INVALID_ARGUMENT, "unknown field");
  if (!host) return fail(GLASMA_ERR_INVALID_ARGUMENT, "null source");
  int st = ensure_field(h, field);
  if (st) return st;
  if (!h->xfer_stream) {
    GLASMA_CUDA(cudaStreamCreateWithFlags(&h->xfer_stream, cudaStreamNonBlocking), "transfer stream");
    GLASMA_CUDA(cudaEventCreateWithFlags(&h->xfer_done, cudaEventDisableTiming), "transfer event");
    for (int b = 0; b < 2; b++)
      GLASMA_CUDA(cudaEventCreateWithFlags(&h->stage_free[b], cudaEventDisableTiming), "staging event");
  }
  const int b = h->stage_slot;
  const size_t bytes = (size_t)h->g.S * host_doubles_per_site(field) * sizeof(double);
  if (!h->stage_f[b][field]) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(GLASMA_ERR_OUT_OF_MEMORY, std::string("cudaMalloc upload staging: ") + cudaGetErrorString(e));
    }
    h->stage_f[b][field] = static_cast<double*>(p);
  }
  // The conversion that last read this set (two finishes ago) must be done before it is overwritten
  // (an event never recorded is complete).  With one set the wait would be on the finish just before,
  // whose conversion is usually still queued: measured on GB300, copies that wait on such an event
  // did not start until the next call on the transfer stream, so a begin/step/sync/finish loop ran
  // the copies after the step instead of under it (116.6 ms against 66.0 per 128x128x512 FP64 step).
  GLASMA_CUDA(cudaStreamWaitEvent(h->xfer_stream, h->stage_free[b], 0), "wait for staging");
  GLASMA_CUDA(cudaMemcpyAsync(h->stage_f[b][field], host, bytes, cudaMemcpyHostToDevice, h->xfer_stream),
              "upload copy");
  h->pending |= 1u << field;
  return GLASMA_OK;
}

int glasma_upload_finish(glasma_lattice* h) {
  GLASMA_CHECK_HANDLE(h);
  if (!h->pending) return GLASMA_OK;
  GLASMA_CUDA(cudaEventRecord(h->xfer_done, h->xfer_stream), "record transfers");
  GLASMA_CUDA(cudaStreamWaitEvent(h->stream, h->xfer_done, 0), "wait for transfers");
  const int b = h->stage_slot;
  for (int f = 0; f < 10; f++) {
    if (!(h->pending & (1u << f))) continue;
    const int P = host_doubles_per_site(f);
    double* src = h->stage_f[b][f];
    cudaError_t e = h->precision == GLASMA_FP64
                        ? glasma::launch_aos_to_soa<double>(src, static_cast<double*>(h->f[f]), h->g.S, P, h->stream)
                        : glasma::launch_aos_to_soa<float>(src, static_cast<float*>(h->f[f]), h->g.S, P, h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "aos_to_soa of staged upload");
  }
  GLASMA_CUDA(cudaEventRecord(h->stage_free[b], h->stream), "record staging read");
  h->stage_slot = b ^ 1;
  h->pending = 0;
  return GLASMA_OK;
}

int glasma_upload(glasma_lattice* h, int field, const double* host) {
  return upload_common(h, field, host, cudaMemcpyHostToDevice);
}
int glasma_download(glasma_lattice* h, int field, double* host) {
  return download_common(h, field, host, cudaMemcpyDeviceToHost);
}
int glasma_upload_device(glasma_lattice* h, int field, const double* dev) {
  return upload_common(h, field, dev, cudaMemcpyDeviceToDevice);
}
int glasma_download_device(glasma_lattice* h, int field, double* dev) {
  return download_common(h, field, dev, cudaMemcpyDeviceToDevice);
}

int glasma_step(glasma_lattice* h, double dt, int nsteps, unsigned flags) {
  GLASMA_CHECK_HANDLE(h);
  if (nsteps < 0) return fail(GLASMA_ERR_INVALID_ARGUMENT, "nsteps < 0");
  if (flags & ~GLASMA_STEP_SAVE_UOLD) return fail(GLASMA_ERR_INVALID_ARGUMENT, "unknown step flag");
  if (nsteps == 0) return GLASMA_OK;
  return h->precision == GLASMA_FP64 ? step_impl<double>(h, dt, nsteps, flags) : step_impl<float>(h, dt, nsteps, flags);
}

int glasma_set_step_method(glasma_lattice* h, int method) {
  GLASMA_CHECK_HANDLE(h);
  if (method != GLASMA_STEP_ONE_PASS && method != GLASMA_STEP_TWO_PASS && method != GLASMA_STEP_PLAQUETTE &&
      method != GLASMA_STEP_MARCH)
    return fail(GLASMA_ERR_INVALID_ARGUMENT, "unknown step method");
  h->step_method = method;
  if (method != GLASMA_STEP_ONE_PASS && method != GLASMA_STEP_MARCH) {  // give the second buffer set back
    GLASMA_CUDA(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
    for (int f : kSwapFields) {
      if (h->alt[f]) cudaFree(h->alt[f]);
      h->alt[f] = nullptr;
    }
  }
  if (method != GLASMA_STEP_PLAQUETTE && h->contrib) {  // and the contribution buffer
    GLASMA_CUDA(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
    cudaFree(h->contrib);
    h->contrib = nullptr;
  }
  return GLASMA_OK;
}

int glasma_set_march_chunk(glasma_lattice* h, int slices) {
  GLASMA_CHECK_HANDLE(h);
  if (slices < 0) return fail(GLASMA_ERR_INVALID_ARGUMENT, "slices < 0");
  h->march_lz = slices;
  return GLASMA_OK;
}

int glasma_set_fp64_arithmetic(glasma_lattice* h, int mode) {
  GLASMA_CHECK_HANDLE(h);
  if (mode != GLASMA_FP64_NATIVE && mode != GLASMA_FP64_DOUBLE_FLOAT)
    return fail(GLASMA_ERR_INVALID_ARGUMENT, "unknown FP64 arithmetic mode");
  h->fp64_arith = mode;
  return GLASMA_OK;
}

int glasma_get_fp64_arithmetic(glasma_lattice* h, int* mode) {
  GLASMA_CHECK_HANDLE(h);
  if (!mode) return fail(GLASMA_ERR_INVALID_ARGUMENT, "mode is null");
  *mode = h->fp64_arith;
  return GLASMA_OK;
}

int glasma_set_link_storage(glasma_lattice* h, int reals_per_link) {
  GLASMA_CHECK_HANDLE(h);
  if (reals_per_link != 18 && reals_per_link != 12)
    return fail(GLASMA_ERR_INVALID_ARGUMENT, "reals_per_link must be 18 or 12");
  if (reals_per_link == 12 && h->precision != GLASMA_FP32)
    return fail(GLASMA_ERR_UNSUPPORTED, "12-real links are built for FP32 handles only");
  h->link_rows = reals_per_link == 12 ? 2 : 3;
  return GLASMA_OK;
}

int glasma_get_link_storage(glasma_lattice* h, int* reals_per_link) {
  GLASMA_CHECK_HANDLE(h);
  if (!reals_per_link) return fail(GLASMA_ERR_INVALID_ARGUMENT, "reals_per_link is null");
  *reals_per_link = h->link_rows == 2 ? 12 : 18;
  return GLASMA_OK;
}

int glasma_get_step_method(glasma_lattice* h, int* method) {
  GLASMA_CHECK_HANDLE(h);
  if (!method) return fail(GLASMA_ERR_INVALID_ARGUMENT, "method is null");
  *method = h->last_method;
  return GLASMA_OK;
}

int glasma_step_profiled(glasma_lattice* h, double dt, int nsteps, unsigned flags, double* kernel_ms) {
  GLASMA_CHECK_HANDLE(h);
  if (nsteps <= 0 || !kernel_ms) return fail(GLASMA_ERR_INVALID_ARGUMENT, "nsteps <= 0 or null kernel_ms");
  if (flags & ~GLASMA_STEP_SAVE_UOLD) return fail(GLASMA_ERR_INVALID_ARGUMENT, "unknown step flag");
  std::vector<cudaEvent_t> ev((size_t)nsteps * 3);
  for (auto& x : ev) GLASMA_CUDA(cudaEventCreate(&x), "cudaEventCreate");
  int st = h->precision == GLASMA_FP64 ? step_impl<double>(h, dt, nsteps, flags, ev.data())
                                       : step_impl<float>(h, dt, nsteps, flags, ev.data());
  if (st == GLASMA_OK) {
    cudaError_t e = cudaEventSynchronize(ev.back());
    if (e != cudaSuccess) st = cuda_fail(e, "cudaEventSynchronize");
  }
  kernel_ms[0] = kernel_ms[1] = 0.0;
  if (st == GLASMA_OK) {
    for (int n = 0; n < nsteps; n++) {
      float a = 0.f, b = 0.f;
      cudaEventElapsedTime(&a, ev[3 * n], ev[3 * n + 1]);
      cudaEventElapsedTime(&b, ev[3 * n + 1], ev[3 * n + 2]);
      kernel_ms[0] += a;
      kernel_ms[1] += b;
    }
  }
  for (auto& x : ev) cudaEventDestroy(x);
  return st;
}

#define GLASMA_DISPATCH(h, call_double, call_float) \
  ((h)->precision == GLASMA_FP64 ? (call_double) : (call_float))

int glasma_update_efield(glasma_lattice* h, double dt) {
  GLASMA_CHECK_HANDLE(h);
  int st = sync_field_ghosts(h, GLASMA_FIELD_U);
  if (st) return st;
  cudaError_t e = GLASMA_DISPATCH(h, glasma::launch_efield_only<double>(h->g, ptrs<double>(h), dt, h->tile_x, h->stream),
                                  glasma::launch_efield_only<float>(h->g, ptrs<float>(h), dt, h->tile_x, h->stream));
  return e == cudaSuccess ? GLASMA_OK : cuda_fail(e, "update_efield");
}

int glasma_update_jstat(glasma_lattice* h, double dt) {
  GLASMA_CHECK_HANDLE(h);
  cudaError_t e = GLASMA_DISPATCH(h, glasma::launch_jstat_only<double>(h->g, ptrs<double>(h), dt, h->tile_x, h->stream),
                                  glasma::launch_jstat_only<float>(h->g, ptrs<float>(h), dt, h->tile_x, h->stream));
  return e == cudaSuccess ? GLASMA_OK : cuda_fail(e, "update_jstat");
}

int glasma_update_links(glasma_lattice* h, double dt_arg) {
  GLASMA_CHECK_HANDLE(h);
  cudaError_t e = GLASMA_DISPATCH(h, glasma::launch_links_only<double>(h->g, ptrs<double>(h), dt_arg, h->stream),
                                  glasma::launch_links_only<float>(h->g, ptrs<float>(h), dt_arg, h->stream));
  return e == cudaSuccess ? GLASMA_OK : cuda_fail(e, "update_links");
}

int glasma_save_old_link(glasma_lattice* h) {
  GLASMA_CHECK_HANDLE(h);
  int st = sync_field_ghosts(h, GLASMA_FIELD_U);
  if (st) return st;
  cudaError_t e = GLASMA_DISPATCH(
      h,
      glasma::launch_copy_links<double>(h->g, static_cast<const cx<double>*>(h->f[GLASMA_FIELD_U]),
                                        static_cast<cx<double>*>(h->f[GLASMA_FIELD_UOLD]), h->stream),
      glasma::launch_copy_links<float>(h->g, static_cast<const cx<float>*>(h->f[GLASMA_FIELD_U]),
                                       static_cast<cx<float>*>(h->f[GLASMA_FIELD_UOLD]), h->stream));
  return e == cudaSuccess ? GLASMA_OK : cuda_fail(e, "save_old_link");
}

int glasma_update_j(glasma_lattice* h, double dt) {
  GLASMA_CHECK_HANDLE(h);
  cudaError_t e = GLASMA_DISPATCH(h, glasma::launch_j_only<double>(h->g, ptrs<double>(h), dt, h->stream),
                                  glasma::launch_j_only<float>(h->g, ptrs<float>(h), dt, h->stream));
  return e == cudaSuccess ? GLASMA_OK : cuda_fail(e, "update_j");
}

int glasma_bulk(glasma_lattice* h, double out[16]) {
  GLASMA_CHECK_HANDLE(h);
  if (!out) return fail(GLASMA_ERR_INVALID_ARGUMENT, "out is null");
  int st = ensure_scratch(h);
  if (st) return st;
  double* res = h->scratch + h->scratch_doubles - 32;
  cudaError_t e = GLASMA_DISPATCH(h, glasma::launch_bulk<double>(h->g, ptrs<double>(h), h->scratch, res, h->stream),
                                  glasma::launch_bulk<float>(h->g, ptrs<float>(h), h->scratch, res, h->stream));
  if (e != cudaSuccess) return cuda_fail(e, "bulk");
  double r[7];
  st = copy_results_to_host(h, res, r, 7);
  if (st) return st;
  // Observables::Bulk constants and accessors (S/OBSERVABLES/BulkObservables.cpp:22-62)
  const double a3 = h->g.a[0] * h->g.a[1] * h->g.a[2];
  double cB[3], cE[3], cS[3];
  for (int mu = 0; mu < 3; mu++) {
    const double q = h->g.a[mu] * h->a_scale * h->a_scale / a3;
    cB[mu] = q * q;
    cE[mu] = q * q;
    cS[mu] = h->g.a[mu] * h->a_scale / (a3 * a3);
  }
  const double ES[3] = {r[3], r[4], r[5]}, BS[3] = {r[0], r[1], r[2]}, ED[3] = {0.0, 0.0, r[6]};
  for (int i = 0; i < 3; i++) {
    out[i] = ES[i];
    out[3 + i] = BS[i];
    out[6 + i] = ED[i];
  }
  const double e0 = cE[0] * ES[0], e1 = cE[1] * ES[1], e2 = cE[2] * ES[2];
  const double b0 = cB[0] * BS[0], b1 = cB[1] * BS[1], b2 = cB[2] * BS[2];
  out[9] = 0.5 * (e0 + e1 + e2 + b0 + b1 + b2);
  out[10] = 0.5 * ((e1 + e2 + b1 + b2) - (e0 + b0));
  out[11] = 0.5 * ((e0 + e2 + b0 + b2) - (e1 + b1));
  out[12] = 0.5 * ((e0 + e1 + b0 + b1) - (e2 + b2));
  out[13] = 0.5 * (e0 + e1 + e2);
  out[14] = 0.5 * (b0 + b1 + b2);
  out[15] = cS[0] * ED[0] + cS[1] * ED[1] + cS[2] * ED[2];
  return GLASMA_OK;
}

int glasma_gauss(glasma_lattice* h, int sync_first, double* max_violation, double* avg_violation, double* zprofile) {
  GLASMA_CHECK_HANDLE(h);
  if (!max_violation || !avg_violation) return fail(GLASMA_ERR_INVALID_ARGUMENT, "null output");
  int st = ensure_scratch(h);
  if (st) return st;
  if (sync_first) {
    const int fs[4] = {GLASMA_FIELD_JPSTAT, GLASMA_FIELD_JMSTAT, GLASMA_FIELD_U, GLASMA_FIELD_E};
    for (int f : fs)
      if ((st = sync_field_ghosts(h, f))) return st;
  }
  double* res = h->scratch + h->scratch_doubles - 32;
  double* prof = zprofile ? h->scratch + h->scratch_doubles - 64 - (size_t)h->g.nz : nullptr;
  cudaError_t e = GLASMA_DISPATCH(
      h, glasma::launch_gauss<double>(h->g, ptrs<double>(h), h->a_scale, h->scratch, res, prof, h->stream),
      glasma::launch_gauss<float>(h->g, ptrs<float>(h), h->a_scale, h->scratch, res, prof, h->stream));
  if (e != cudaSuccess) return cuda_fail(e, "gauss");
  double r[2];
  if ((st = copy_results_to_host(h, res, r, 2))) return st;
  if (zprofile && (st = copy_results_to_host(h, prof, zprofile, (size_t)h->g.nz))) return st;
  *max_violation = r[1];
  *avg_violation = std::sqrt(r[0] / (8.0 * (double)h->g.vol));
  return GLASMA_OK;
}

int glasma_unitarity(glasma_lattice* h, double* max_violation, double* avg_violation) {
  GLASMA_CHECK_HANDLE(h);
  if (!max_violation || !avg_violation) return fail(GLASMA_ERR_INVALID_ARGUMENT, "null output");
  int st = ensure_scratch(h);
  if (st) return st;
  double* res = h->scratch + h->scratch_doubles - 32;
  cudaError_t e = GLASMA_DISPATCH(
      h,
      glasma::launch_unitarity<double>(h->g, static_cast<const cx<double>*>(h->f[GLASMA_FIELD_U]), h->scratch, res, h->stream),
      glasma::launch_unitarity<float>(h->g, static_cast<const cx<float>*>(h->f[GLASMA_FIELD_U]), h->scratch, res, h->stream));
  if (e != cudaSuccess) return cuda_fail(e, "unitarity");
  double r[2];
  if ((st = copy_results_to_host(h, res, r, 2))) return st;
  *max_violation = r[1];
  *avg_violation = std::sqrt(r[0] / (3.0 * (double)h->g.vol));
  return GLASMA_OK;
}

int glasma_emt_map(glasma_lattice* h, double* out) {
  GLASMA_CHECK_HANDLE(h);
  if (!out) return fail(GLASMA_ERR_INVALID_ARGUMENT, "out is null");
  int st = ensure_scratch(h);
  if (st) return st;
  // CreateMap syncs the ghosts of UOld and U inside its site loop (S/OBSERVABLES/EnergyMomentumTensor.cpp:132-133)
  if ((st = sync_field_ghosts(h, GLASMA_FIELD_UOLD))) return st;
  if ((st = sync_field_ghosts(h, GLASMA_FIELD_U))) return st;
  const long long nres = (long long)h->g.nz * 10;
  double* res = h->scratch + h->scratch_doubles - 64 - (size_t)h->g.nz * 11;
  cudaError_t e = GLASMA_DISPATCH(
      h, glasma::launch_emt_map<double>(h->g, ptrs<double>(h), h->a_scale, h->scratch, res, h->stream),
      glasma::launch_emt_map<float>(h->g, ptrs<float>(h), h->a_scale, h->scratch, res, h->stream));
  if (e != cudaSuccess) return cuda_fail(e, "emt_map");
  return copy_results_to_host(h, res, out, (size_t)nres);
}

int glasma_pressure_anisotropy(glasma_lattice* h, int z_begin, int z_end, double* ratio, double* p_l, double* p_t) {
  GLASMA_CHECK_HANDLE(h);
  if (z_begin < 0 || z_end > h->g.nz || z_begin >= z_end) return fail(GLASMA_ERR_INVALID_ARGUMENT, "bad slice range");
  std::vector<double> map((size_t)h->g.nz * 10);
  int st = glasma_emt_map(h, map.data());
  if (st) return st;
  double pl = 0.0, pt = 0.0;
  for (int z = z_begin; z < z_end; z++) {
    pl += map[(size_t)z * 10 + 3];
    pt += 0.5 * (map[(size_t)z * 10 + 1] + map[(size_t)z * 10 + 2]);
  }
  pl /= (z_end - z_begin);
  pt /= (z_end - z_begin);
  if (p_l) *p_l = pl;
  if (p_t) *p_t = pt;
  if (ratio) *ratio = pl / pt;
  return GLASMA_OK;
}

int glasma_reunitarize(glasma_lattice* h) {
  GLASMA_CHECK_HANDLE(h);
  cudaError_t e = GLASMA_DISPATCH(
      h, glasma::launch_reunitarize<double>(h->g, static_cast<cx<double>*>(h->f[GLASMA_FIELD_U]), h->stream),
      glasma::launch_reunitarize<float>(h->g, static_cast<cx<float>*>(h->f[GLASMA_FIELD_U]), h->stream));
  return e == cudaSuccess ? GLASMA_OK : cuda_fail(e, "reunitarize");
}

int glasma_gauge_reset(glasma_lattice* h) {
  GLASMA_CHECK_HANDLE(h);
  if (h->f[GLASMA_FIELD_G]) {
    cudaFree(h->f[GLASMA_FIELD_G]);
    h->f[GLASMA_FIELD_G] = nullptr;
  }
  return ensure_field(h, GLASMA_FIELD_G);
}

int glasma_coulomb_fix(glasma_lattice* h, double alpha, int max_iters, double tol, unsigned flags, double* log,
                       int* iterations) {
  GLASMA_CHECK_HANDLE(h);
  if (max_iters < 0) return fail(GLASMA_ERR_INVALID_ARGUMENT, "max_iters < 0");
  if (flags & ~(GLASMA_GF_PROJECT_ZERO_MODE | GLASMA_GF_FFT_FP32 | GLASMA_GF_OPEN_Z | GLASMA_GF_MIXED))
    return fail(GLASMA_ERR_INVALID_ARGUMENT, "unknown gauge-fixing flag");
  int st;
  for (int f : {GLASMA_FIELD_G, GLASMA_FIELD_UG, GLASMA_FIELD_EG})
    if ((st = ensure_field(h, f))) return st;
  if ((st = ensure_scratch(h))) return st;
  glasma::GaugeFixArgs a;
  a.g = h->g;
  a.precision = h->precision;
  a.a_scale = h->a_scale;
  a.stream = h->stream;
  a.U = h->f[GLASMA_FIELD_U];
  a.E = h->f[GLASMA_FIELD_E];
  a.G = h->f[GLASMA_FIELD_G];
  a.UG = h->f[GLASMA_FIELD_UG];
  a.EG = h->f[GLASMA_FIELD_EG];
  a.scratch = h->scratch;
  a.scratch_doubles = h->scratch_doubles;
  std::string err;
  int n = 0;
  st = glasma::gaugefix_run(&h->gf, a, alpha, max_iters, tol, flags, log, &n, &err);
  if (iterations) *iterations = n;
  if (st != GLASMA_OK) return fail(st, err);
  return GLASMA_OK;
}

int glasma_coulomb_fix_algorithm(glasma_lattice* h, int algorithm, double param, unsigned long long seed, int max_iters,
                                 double tol, unsigned flags, double* log, int* iterations) {
  GLASMA_CHECK_HANDLE(h);
  if (algorithm == GLASMA_GF_FOURIER) return glasma_coulomb_fix(h, param, max_iters, tol, flags, log, iterations);
  if (algorithm != GLASMA_GF_LOS_ALAMOS && algorithm != GLASMA_GF_JACOBI)
    return fail(GLASMA_ERR_INVALID_ARGUMENT, "unknown gauge-fixing algorithm");
  if (max_iters < 0) return fail(GLASMA_ERR_INVALID_ARGUMENT, "max_iters < 0");
  if (flags) return fail(GLASMA_ERR_INVALID_ARGUMENT, "gauge-fixing flags apply to the Fourier update only");
  int st;
  for (int f : {GLASMA_FIELD_G, GLASMA_FIELD_UG, GLASMA_FIELD_EG})
    if ((st = ensure_field(h, f))) return st;
  if ((st = ensure_scratch(h))) return st;
  glasma::GaugeFixArgs a = {};
  a.g = h->g;
  a.precision = h->precision;
  a.a_scale = h->a_scale;
  a.stream = h->stream;
  a.U = h->f[GLASMA_FIELD_U];
  a.E = h->f[GLASMA_FIELD_E];
  a.G = h->f[GLASMA_FIELD_G];
  a.UG = h->f[GLASMA_FIELD_UG];
  a.EG = h->f[GLASMA_FIELD_EG];
  a.scratch = h->scratch;
  a.scratch_doubles = h->scratch_doubles;
  std::string err;
  int n = 0;
  st = glasma::gaugefix_run_local(a, algorithm, param, seed, max_iters, tol, log, &n, &err);
  if (iterations) *iterations = n;
  if (st != GLASMA_OK) return fail(st, err);
  return GLASMA_OK;
}

int glasma_transform_charge(glasma_lattice* h, int field, double* out) {
  GLASMA_CHECK_HANDLE(h);
  if (field < GLASMA_FIELD_JP || field > GLASMA_FIELD_JMSTAT)
    return fail(GLASMA_ERR_INVALID_ARGUMENT, "field must be one of GLASMA_FIELD_JP .. GLASMA_FIELD_JMSTAT");
  if (!out) return fail(GLASMA_ERR_INVALID_ARGUMENT, "null destination");
  int st;
  if ((st = ensure_field(h, GLASMA_FIELD_G))) return st;
  const size_t bytes = (size_t)h->g.S * 8 * sizeof(double);
  if ((st = ensure_staging(h, bytes))) return st;
  glasma::GaugeFixArgs a = {};
  a.g = h->g;
  a.precision = h->precision;
  a.stream = h->stream;
  a.G = h->f[GLASMA_FIELD_G];
  cudaError_t e = glasma::launch_transform_charge(a, h->f[field], h->staging);
  if (e != cudaSuccess) return cuda_fail(e, "transform charge");
  GLASMA_CUDA(cudaMemcpyAsync(out, h->staging, bytes, cudaMemcpyDefault, h->stream), "transform charge copy");
  GLASMA_CUDA(cudaStreamSynchronize(h->stream), "transform charge sync");
  return GLASMA_OK;
}

int glasma_fft3d(glasma_lattice* h, const double* in, double* out, int inverse) {
  GLASMA_CHECK_HANDLE(h);
  if (!in || !out) return fail(GLASMA_ERR_INVALID_ARGUMENT, "null buffer");
  int st = ensure_scratch(h);
  if (st) return st;
  glasma::GaugeFixArgs a = {};
  a.g = h->g;
  a.precision = h->precision;
  a.a_scale = h->a_scale;
  a.stream = h->stream;
  a.scratch = h->scratch;
  a.scratch_doubles = h->scratch_doubles;
  std::string err;
  st = glasma::gaugefix_fft_test(&h->gf, a, reinterpret_cast<const double2*>(in), reinterpret_cast<double2*>(out),
                                 inverse ? 1 : 0, &err);
  return st == GLASMA_OK ? GLASMA_OK : fail(st, err);
}

int glasma_fft3d_f32(glasma_lattice* h, const float* in, float* out, int inverse) {
  GLASMA_CHECK_HANDLE(h);
  if (!in || !out) return fail(GLASMA_ERR_INVALID_ARGUMENT, "null buffer");
  int st = ensure_scratch(h);
  if (st) return st;
  glasma::GaugeFixArgs a = {};
  a.g = h->g;
  a.precision = h->precision;
  a.a_scale = h->a_scale;
  a.stream = h->stream;
  a.scratch = h->scratch;
  a.scratch_doubles = h->scratch_doubles;
  std::string err;
  st = glasma::gaugefix_fft_test_f32(&h->gf, a, reinterpret_cast<const float2*>(in), reinterpret_cast<float2*>(out),
                                     inverse ? 1 : 0, &err);
  return st == GLASMA_OK ? GLASMA_OK : fail(st, err);
}

int glasma_autotune(glasma_lattice* h, double dt, int* tile_x) {
  GLASMA_CHECK_HANDLE(h);
  if (h->step_method == GLASMA_STEP_PLAQUETTE) {  // its kernels are pointwise: no tile to choose
    if (tile_x) *tile_x = h->tile_x;
    return GLASMA_OK;
  }
  return glasma_autotune_staple(h, dt, tile_x);
}

int glasma_autotune_staple(glasma_lattice* h, double dt, int* tile_x) {
  GLASMA_CHECK_HANDLE(h);
  const int candidates[5] = {128, 64, 32, 16, 8};
  cudaEvent_t e0, e1;
  GLASMA_CUDA(cudaEventCreate(&e0), "cudaEventCreate");
  GLASMA_CUDA(cudaEventCreate(&e1), "cudaEventCreate");
  const bool one_pass = h->step_method == GLASMA_STEP_ONE_PASS && ensure_alt(h);
  float best = 1e30f;
  int best_tx = h->tile_x;
  for (int tx : candidates) {
    if (tx > 2 * h->g.nx && tx != glasma::default_tile_x(h->g.nx)) continue;  // mostly idle threads
    float total = 0.f;
    for (int rep = 0; rep < 4; rep++) {
      cudaEventRecord(e0, h->stream);
      cudaError_t e =
          one_pass ? GLASMA_DISPATCH(h, glasma::launch_fused_step<double>(h->g, ptrs<double>(h), alt_ptrs<double>(h), dt,
                                                                          false, tx, true, h->stream),
                                     glasma::launch_fused_step<float>(h->g, ptrs<float>(h), alt_ptrs<float>(h), dt, false,
                                                                      tx, true, h->stream, h->link_rows))
                   : GLASMA_DISPATCH(h, glasma::launch_efield_dry<double>(h->g, ptrs<double>(h), dt, tx, h->stream),
                                     glasma::launch_efield_dry<float>(h->g, ptrs<float>(h), dt, tx, h->stream,
                                                                      h->link_rows));
      cudaEventRecord(e1, h->stream);
      if (e != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return cuda_fail(e, "autotune");
      }
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) total += ms;  // first run warms caches
    }
    if (total < best) {
      best = total;
      best_tx = tx;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  h->tile_x = best_tx;
  if (tile_x) *tile_x = best_tx;
  return GLASMA_OK;
}

int glasma_set_tile(glasma_lattice* h, int tile_x) {
  if (!h) return fail(GLASMA_ERR_INVALID_ARGUMENT, "null lattice handle");
  if (tile_x < 1 || tile_x > 128 || 128 % tile_x) return fail(GLASMA_ERR_INVALID_ARGUMENT, "tile_x must divide 128");
  h->tile_x = tile_x;
  return GLASMA_OK;
}

int glasma_synchronize(glasma_lattice* h) {
  GLASMA_CHECK_HANDLE(h);
  GLASMA_CUDA(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
  GLASMA_CUDA(cudaGetLastError(), "pending error");
  return GLASMA_OK;
}

}  // extern "C"

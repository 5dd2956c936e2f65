// noalloc.cu -- Gauss-law violation without any device allocation (glasma_gauss_noalloc).
//
// Some callers cannot call cudaMalloc: code that runs while another framework is capturing a
// CUDA graph on the stream, code whose device memory is owned by a pool or arena that forbids
// outside allocations, and real-time loops where an allocation (and the implicit
// synchronisation it can cause) is not allowed.  They already hold the fields in device memory
// and want the measurement without the library creating a lattice handle.
//
// This entry point reads the caller's device buffers and writes to the caller's device output.
// Its block partials live in one file-scope __device__ array of fixed size, so nothing is
// allocated.  Host code cannot use that array's name as a device address; the address is
// looked up once per device with cudaGetSymbolAddress (the first call on each device does
// this, so make that first call before any stream capture begins) and then passed to the
// kernels.  The address is cached for the life of the process: a cudaDeviceReset (or anything
// else that destroys the device's primary context) invalidates it, and later calls on that device
// would then use a stale address, so do not call this entry point after such a reset.  Every call on a device shares the one array: calls whose kernels overlap on the
// GPU (different streams without ordering) race on it and must be serialised by the caller.
// The array keeps the last call's contents; nothing in it has to start at zero, because every
// partial that a call reads was written earlier in the same call.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/glasma_gb300.h"
#include "lattice.cuh"

namespace glasma {
namespace {

// Per-slice Gauss reduction: 32 blocks x 2 values per z slice, then 2 values per slice,
// plus a little room for the two results -> Nz <= kNoAllocMaxNz.
constexpr long long kNoAllocScratchDoubles = 65536;  // 512 KiB per device
constexpr int kNoAllocMaxNz = (int)((kNoAllocScratchDoubles - 64) / (32 * 2 + 2));

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_ptr[kMaxDevices] = {};

// result = {sum G^2, max |G|} -> {max |G|, sqrt(sum G^2 / (8 V))}
__global__ void finish_noalloc_kernel(const double* sums, double inv8v, double* result) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const double s = sums[0], m = sums[1];
    result[0] = m;
    result[1] = sqrt(s * inv8v);
  }
}

}  // namespace
}  // namespace glasma

namespace glasma {
int record_error(int status, const std::string& msg);  // glasma_abi.cu: sets glasma_last_error()
}

namespace {
int noalloc_fail(int status, const std::string& m) { return glasma::record_error(status, "glasma_gauss_noalloc: " + m); }
}  // namespace

extern "C" int glasma_gauss_noalloc(const double* U, const double* E, const double* JpStat, const double* JmStat,
                                    int nx, int ny, int nz, double ax, double ay, double az, double a_scale,
                                    double* result, double* zprofile, void* stream) {
  using namespace glasma;
  if (nx < 2 || ny < 2 || nz < 2) return noalloc_fail(GLASMA_ERR_BAD_SHAPE, "each extent must be >= 2");
  if ((long long)nx * ny * (nz + 2) > (1LL << 40))  // the limit glasma_create applies
    return noalloc_fail(GLASMA_ERR_BAD_SHAPE, "lattice too large");
  if (nz > kNoAllocMaxNz)
    return noalloc_fail(GLASMA_ERR_BAD_SHAPE, "Nz = " + std::to_string(nz) + " exceeds the maximum " +
                                                  std::to_string(kNoAllocMaxNz) +
                                                  " that the fixed 512 KiB device scratch can reduce");
  if (!(ax > 0) || !(ay > 0) || !(az > 0) || !(a_scale > 0))
    return noalloc_fail(GLASMA_ERR_BAD_SHAPE, "spacings and a_scale must be positive");
  if (!U || !E || !JpStat || !JmStat || !result) return noalloc_fail(GLASMA_ERR_INVALID_ARGUMENT, "null pointer");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(GLASMA_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(GLASMA_ERR_UNSUPPORTED, "device index out of range");
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) return noalloc_fail(GLASMA_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  Geometry g;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.plane = (long long)nx * ny;
  g.S = g.plane * (nz + 2);
  g.vol = g.plane * nz;
  g.a[0] = ax;
  g.a[1] = ay;
  g.a[2] = az;
  FieldPtrs<double> f = {};
  f.U = reinterpret_cast<cx<double>*>(const_cast<double*>(U));
  f.E = const_cast<double*>(E);
  f.JpStat = const_cast<double*>(JpStat);
  f.JmStat = const_cast<double*>(JmStat);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* sums = scratch + kNoAllocScratchDoubles - 8;
  e = launch_gauss<double>(g, f, a_scale, scratch, sums, zprofile, st);
  if (e != cudaSuccess) return noalloc_fail(GLASMA_ERR_CUDA, cudaGetErrorString(e));
  finish_noalloc_kernel<<<1, 32, 0, st>>>(sums, 1.0 / (8.0 * (double)g.vol), result);
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(GLASMA_ERR_CUDA, cudaGetErrorString(e));
  return GLASMA_OK;
}

// synthetic.cu -- seeded synthetic fields generated on the device (benchmarks and demos).
//
// Every value comes from a counter-based generator (SplitMix64 of seed and a global element
// counter, Box-Muller pairs), so the same seed gives the same fields for any launch shape:
// links exp(i link_amp t^a r^a), E = e_amp r, currents = j_amp r, r ~ N(0,1) per component.
// Ghost slices are then synced (open z boundary).
#include <cuda_runtime.h>

#include "../../include/glasma_gb300.h"
#include "handle.h"
#include "lattice.cuh"

namespace glasma {
namespace {

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
// two N(0,1) numbers from counter c of stream `seed`
__device__ __forceinline__ void gauss2(unsigned long long seed, unsigned long long c, double& g0, double& g1) {
  const unsigned long long r = splitmix64(seed ^ splitmix64(c));
  const unsigned long long r2 = splitmix64(r);
  const double u1 = ((r >> 11) + 1.0) * (1.0 / 9007199254740993.0);  // (0, 1]
  const double u2 = (r2 >> 11) * (1.0 / 9007199254740992.0);         // [0, 1)
  const double rad = sqrt(-2.0 * log(u1));
  double s, co;
  sincospi(2.0 * u2, &s, &co);
  g0 = rad * co;
  g1 = rad * s;
}

template <typename T>
__global__ void fill_kernel(Geometry g, cx<T>* U, T* E, T* Jp, T* Jm, T* JpS, T* JmS, unsigned long long seed,
                            double link_amp, double e_amp, double j_amp) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.vol) return;
  const long long s = i + g.plane;
  const unsigned long long base = (unsigned long long)i * 64ull;  // 64 counters per site
  for (int mu = 0; mu < 3; mu++) {
    Alg<double> al;
    for (int a = 0; a < 8; a += 2) gauss2(seed, base + mu * 4 + a / 2, al.a[a], al.a[a + 1]);
    Mat<double> X;
    expi(link_amp, al, X);
    for (int k = 0; k < 9; k++) U[(long long)(mu * 9 + k) * g.S + s] = mk<T>((T)X.e[k].re, (T)X.e[k].im);
    for (int a = 0; a < 8; a += 2) {
      double g0, g1;
      gauss2(seed, base + 12 + mu * 4 + a / 2, g0, g1);
      E[(long long)(mu * 8 + a) * g.S + s] = (T)(e_amp * g0);
      E[(long long)(mu * 8 + a + 1) * g.S + s] = (T)(e_amp * g1);
    }
  }
  T* J[4] = {Jp, Jm, JpS, JmS};
  for (int c = 0; c < 4; c++)
    for (int a = 0; a < 8; a += 2) {
      double g0, g1;
      gauss2(seed, base + 24 + c * 4 + a / 2, g0, g1);
      J[c][(long long)a * g.S + s] = (T)(j_amp * g0);
      J[c][(long long)(a + 1) * g.S + s] = (T)(j_amp * g1);
    }
}

}  // namespace
}  // namespace glasma

extern "C" int glasma_fill_synthetic(glasma_lattice* h, unsigned long long seed, double link_amp, double e_amp,
                                     double j_amp) {
  using namespace glasma;
  if (!h) return GLASMA_ERR_INVALID_ARGUMENT;
  if (cudaSetDevice(h->device) != cudaSuccess) return GLASMA_ERR_CUDA;
  const unsigned grid = (unsigned)((h->g.vol + 127) / 128);
  if (h->precision == GLASMA_FP64)
    fill_kernel<double><<<grid, 128, 0, h->stream>>>(
        h->g, static_cast<cx<double>*>(h->f[GLASMA_FIELD_U]), static_cast<double*>(h->f[GLASMA_FIELD_E]),
        static_cast<double*>(h->f[GLASMA_FIELD_JP]), static_cast<double*>(h->f[GLASMA_FIELD_JM]),
        static_cast<double*>(h->f[GLASMA_FIELD_JPSTAT]), static_cast<double*>(h->f[GLASMA_FIELD_JMSTAT]), seed, link_amp,
        e_amp, j_amp);
  else
    fill_kernel<float><<<grid, 128, 0, h->stream>>>(
        h->g, static_cast<cx<float>*>(h->f[GLASMA_FIELD_U]), static_cast<float*>(h->f[GLASMA_FIELD_E]),
        static_cast<float*>(h->f[GLASMA_FIELD_JP]), static_cast<float*>(h->f[GLASMA_FIELD_JM]),
        static_cast<float*>(h->f[GLASMA_FIELD_JPSTAT]), static_cast<float*>(h->f[GLASMA_FIELD_JMSTAT]), seed, link_amp,
        e_amp, j_amp);
  if (cudaGetLastError() != cudaSuccess) return GLASMA_ERR_CUDA;
  const int fields[6] = {GLASMA_FIELD_U, GLASMA_FIELD_E, GLASMA_FIELD_JP, GLASMA_FIELD_JM, GLASMA_FIELD_JPSTAT,
                         GLASMA_FIELD_JMSTAT};
  const int comps[6] = {27, 24, 8, 8, 8, 8};
  for (int i = 0; i < 6; i++) {
    cudaError_t e;
    if (fields[i] == GLASMA_FIELD_U)
      e = h->precision == GLASMA_FP64 ? launch_sync_ghosts<cx<double>>(h->g, static_cast<cx<double>*>(h->f[fields[i]]), 27, h->stream)
                                      : launch_sync_ghosts<cx<float>>(h->g, static_cast<cx<float>*>(h->f[fields[i]]), 27, h->stream);
    else
      e = h->precision == GLASMA_FP64 ? launch_sync_ghosts<double>(h->g, static_cast<double*>(h->f[fields[i]]), comps[i], h->stream)
                                      : launch_sync_ghosts<float>(h->g, static_cast<float*>(h->f[fields[i]]), comps[i], h->stream);
    if (e != cudaSuccess) return GLASMA_ERR_CUDA;
  }
  return GLASMA_OK;
}

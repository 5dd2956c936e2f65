// layout.cu -- transposes between the reference's host layout (array of structures,
// FP64, ghost slices included; S/LATTICE/GaugeLinks.cpp:38-41, ElectricFields.cpp:31-35,
// ChargeDensity.cpp:24-33) and the device layout (one array per component).
//
// A block moves a tile of 32 sites x P values through shared memory, so the AoS side is
// read/written as one contiguous run of 32*P doubles and every SoA component is read/written
// as 32 consecutive elements.
#include "lattice.cuh"

namespace glasma {

namespace {

constexpr int kTileSites = 32;
constexpr int kLayoutThreads = 256;
constexpr int kMaxPerSite = 54;  // 27 complex link elements

// per_site P doubles per site.  complex_pairs: the SoA side stores P/2 complex components.
template <typename T, bool kComplex>
__global__ void __launch_bounds__(kLayoutThreads) aos_to_soa_kernel(const double* __restrict__ aos, T* __restrict__ soa,
                                                                     long long S, int P) {
  __shared__ double tile[kTileSites * kMaxPerSite];
  const long long s0 = (long long)blockIdx.x * kTileSites;
  const int nsite = (int)((S - s0) < kTileSites ? (S - s0) : kTileSites);
  const int n = nsite * P;
  for (int i = threadIdx.x; i < n; i += blockDim.x) tile[i] = aos[s0 * P + i];
  __syncthreads();
  const int total = kTileSites * P;
  for (int i = threadIdx.x; i < total; i += blockDim.x) {
    if (kComplex) {
      const int part = i & 1, ls = (i >> 1) % kTileSites, k = (i >> 1) / kTileSites;
      if (ls < nsite) soa[((long long)k * S + s0 + ls) * 2 + part] = (T)tile[ls * P + 2 * k + part];
    } else {
      const int ls = i % kTileSites, q = i / kTileSites;
      if (ls < nsite) soa[(long long)q * S + s0 + ls] = (T)tile[ls * P + q];
    }
  }
}

template <typename T, bool kComplex>
__global__ void __launch_bounds__(kLayoutThreads) soa_to_aos_kernel(const T* __restrict__ soa, double* __restrict__ aos,
                                                                     long long S, int P) {
  __shared__ double tile[kTileSites * kMaxPerSite];
  const long long s0 = (long long)blockIdx.x * kTileSites;
  const int nsite = (int)((S - s0) < kTileSites ? (S - s0) : kTileSites);
  const int total = kTileSites * P;
  for (int i = threadIdx.x; i < total; i += blockDim.x) {
    if (kComplex) {
      const int part = i & 1, ls = (i >> 1) % kTileSites, k = (i >> 1) / kTileSites;
      if (ls < nsite) tile[ls * P + 2 * k + part] = (double)soa[((long long)k * S + s0 + ls) * 2 + part];
    } else {
      const int ls = i % kTileSites, q = i / kTileSites;
      if (ls < nsite) tile[ls * P + q] = (double)soa[(long long)q * S + s0 + ls];
    }
  }
  __syncthreads();
  const int n = nsite * P;
  for (int i = threadIdx.x; i < n; i += blockDim.x) aos[s0 * P + i] = tile[i];
}

}  // namespace

// per_site: doubles per site on the AoS side (54 links, 18 gauge transformation, 24 E, 8 J).
// Link-type fields (54, 18) are complex on the SoA side.
template <typename T>
cudaError_t launch_aos_to_soa(const double* aos, T* soa, long long S, int per_site, cudaStream_t stream) {
  if (per_site > kMaxPerSite) return cudaErrorInvalidValue;
  const unsigned grid = (unsigned)((S + kTileSites - 1) / kTileSites);
  if (per_site == 54 || per_site == 18)
    aos_to_soa_kernel<T, true><<<grid, kLayoutThreads, 0, stream>>>(aos, soa, S, per_site);
  else
    aos_to_soa_kernel<T, false><<<grid, kLayoutThreads, 0, stream>>>(aos, soa, S, per_site);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_soa_to_aos(const T* soa, double* aos, long long S, int per_site, cudaStream_t stream) {
  if (per_site > kMaxPerSite) return cudaErrorInvalidValue;
  const unsigned grid = (unsigned)((S + kTileSites - 1) / kTileSites);
  if (per_site == 54 || per_site == 18)
    soa_to_aos_kernel<T, true><<<grid, kLayoutThreads, 0, stream>>>(soa, aos, S, per_site);
  else
    soa_to_aos_kernel<T, false><<<grid, kLayoutThreads, 0, stream>>>(soa, aos, S, per_site);
  return cudaGetLastError();
}

template cudaError_t launch_aos_to_soa<double>(const double*, double*, long long, int, cudaStream_t);
template cudaError_t launch_aos_to_soa<float>(const double*, float*, long long, int, cudaStream_t);
template cudaError_t launch_soa_to_aos<double>(const double*, double*, long long, int, cudaStream_t);
template cudaError_t launch_soa_to_aos<float>(const float*, double*, long long, int, cudaStream_t);

}  // namespace glasma

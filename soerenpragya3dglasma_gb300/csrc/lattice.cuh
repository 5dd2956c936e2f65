// lattice.cuh -- device data layout of one lattice and the internal launch API.
//
// HBM layout (structure of arrays, one array per matrix element / colour):
//   site   s = x + Nx*(y + Ny*(z+1)), x,y periodic, z in [-1, Nz]; the slices
//          z=-1 and z=Nz are the reference's open-boundary ghost slices
//          (S/SUNcIndexing.cpp:82, S/LATTICE/GaugeLinks.cpp:27-36, 59-66)
//   links  U[(mu*9 + k)*S + s]  complex (k = i + 3*j, the reference's element order)
//   E      E[(mu*8 + a)*S + s]
//   J      J[a*S + s]           (Jp, Jm, JpStat, JmStat)
//   G      G[k*S + s]           complex
// S = Nx*Ny*(Nz+2).  Consecutive x are consecutive addresses, so a warp that
// walks x reads 32 consecutive elements of every component array.
#pragma once

#include <cstddef>
#include <cstdint>

#include "ddf.cuh"
#include "su3.cuh"

namespace glasma {

struct Geometry {
  int nx, ny, nz;
  long long plane;  // nx*ny
  long long S;      // plane*(nz+2), sites including ghost slices
  long long vol;    // plane*nz, interior sites
  double a[3];
};

template <typename T>
struct FieldPtrs {
  cx<T>* U;
  cx<T>* UOld;
  T* E;
  T* Jp;
  T* Jm;
  T* JpStat;
  T* JmStat;
};

__device__ __forceinline__ long long site_index(const Geometry& g, int x, int y, int z) {
  return (long long)x + (long long)g.nx * ((long long)y + (long long)g.ny * (long long)(z + 1));
}

// Component offsets are computed in the index type I: 32-bit when 27*S < 2^31 (every lattice up to
// 256x256x1200), 64-bit otherwise; fewer registers and integer instructions in the 32-bit case.
template <typename T, typename I>
__device__ __forceinline__ void load_link(const cx<T>* __restrict__ U, I S, int mu, I s, Mat<T>& m) {
  const cx<T>* p = U + ((I)(mu * 9) * S + s);
#pragma unroll
  for (int k = 0; k < 9; k++) m.e[k] = p[(I)k * S];
}
template <typename T, typename I>
__device__ __forceinline__ void store_link(cx<T>* __restrict__ U, I S, int mu, I s, const Mat<T>& m) {
  cx<T>* p = U + ((I)(mu * 9) * S + s);
#pragma unroll
  for (int k = 0; k < 9; k++) p[(I)k * S] = m.e[k];
}
// 12-real links: the leapfrog kernels of a handle in two-row storage read and write rows 0 and 1 of
// each link only (k = 0,1,3,4,6,7: 12 reals of 18) and form row 2 in registers as the unitary
// complement with unit determinant, row2 = conj(row0 x row1): for U in SU(3) the rows are orthonormal
// and det U = row2 . (row0 x row1) = 1 fix it.  R = rows stored (3 = full, 2 = two-row).
template <typename T>
__device__ __forceinline__ void complete_row2(Mat<T>& m) {
  // m(0,j) = e[3j], m(1,j) = e[3j+1], m(2,j) = e[3j+2]
  auto cross = [](const cx<T>& a, const cx<T>& b, const cx<T>& c, const cx<T>& d) {
    // conj(a b - c d)
    cx<T> r;
    r.re = fma(a.re, b.re, fma(-a.im, b.im, fma(-c.re, d.re, c.im * d.im)));
    r.im = -fma(a.re, b.im, fma(a.im, b.re, fma(-c.re, d.im, -(c.im * d.re))));
    return r;
  };
  m.e[2] = cross(m.e[3], m.e[7], m.e[6], m.e[4]);
  m.e[5] = cross(m.e[6], m.e[1], m.e[0], m.e[7]);
  m.e[8] = cross(m.e[0], m.e[4], m.e[3], m.e[1]);
}
template <int R, typename T, typename I>
__device__ __forceinline__ void load_link_r(const cx<T>* __restrict__ U, I S, int mu, I s, Mat<T>& m) {
  if constexpr (R == 3) {
    load_link(U, S, mu, s, m);
  } else {
    const cx<T>* p = U + ((I)(mu * 9) * S + s);
#pragma unroll
    for (int j = 0; j < 3; j++) {
      m.e[3 * j] = p[(I)(3 * j) * S];
      m.e[3 * j + 1] = p[(I)(3 * j + 1) * S];
    }
    complete_row2(m);
  }
}
template <int R, typename T, typename I>
__device__ __forceinline__ void store_link_r(cx<T>* __restrict__ U, I S, int mu, I s, const Mat<T>& m) {
  if constexpr (R == 3) {
    store_link(U, S, mu, s, m);
  } else {
    cx<T>* p = U + ((I)(mu * 9) * S + s);
#pragma unroll
    for (int j = 0; j < 3; j++) {
      p[(I)(3 * j) * S] = m.e[3 * j];
      p[(I)(3 * j + 1) * S] = m.e[3 * j + 1];
    }
  }
}
// Loads and stores that convert between the storage type T and a compute type TC (identity when equal;
// double <-> ddf for the FP64 step computed in double-float arithmetic, ddf.cuh).
template <int R, typename TC, typename T, typename I>
__device__ __forceinline__ void load_link_c(const cx<T>* __restrict__ U, I S, int mu, I s, Mat<TC>& m) {
  if constexpr (std::is_same<T, TC>::value) {
    load_link_r<R>(U, S, mu, s, m);
  } else if constexpr (std::is_same<T, double>::value && std::is_same<TC, ddf>::value && R == 3) {
    ddf_load_link9(U + ((I)(mu * 9) * S + s), (long long)S, m);
  } else {
    Mat<T> t;
    load_link_r<R>(U, S, mu, s, t);
#pragma unroll
    for (int k = 0; k < 9; k++) m.e[k] = mk<TC>(to_compute<TC>(t.e[k].re), to_compute<TC>(t.e[k].im));
  }
}
template <typename T, typename I>
__device__ __forceinline__ void load_alg(const T* __restrict__ F, I S, int base, I s, Alg<T>& v);
template <typename T, typename I>
__device__ __forceinline__ void store_alg(T* __restrict__ F, I S, int base, I s, const Alg<T>& v);
template <typename TC, typename T, typename I>
__device__ __forceinline__ void load_alg_c(const T* __restrict__ F, I S, int base, I s, Alg<TC>& v) {
  if constexpr (std::is_same<T, TC>::value) {
    load_alg(F, S, base, s, v);
  } else {
    Alg<T> t;
    load_alg(F, S, base, s, t);
#pragma unroll
    for (int a = 0; a < 8; a++) v.a[a] = to_compute<TC>(t.a[a]);
  }
}
template <typename TC, typename T, typename I>
__device__ __forceinline__ void store_alg_c(T* __restrict__ F, I S, int base, I s, const Alg<TC>& v) {
  if constexpr (std::is_same<T, TC>::value) {
    store_alg(F, S, base, s, v);
  } else {
    Alg<T> t;
#pragma unroll
    for (int a = 0; a < 8; a++) t.a[a] = from_compute<T>(v.a[a]);
    store_alg(F, S, base, s, t);
  }
}
template <typename T, typename I>
__device__ __forceinline__ void load_alg(const T* __restrict__ F, I S, int base, I s, Alg<T>& v) {
  const T* p = F + ((I)base * S + s);
#pragma unroll
  for (int a = 0; a < 8; a++) v.a[a] = p[(I)a * S];
}
template <typename T, typename I>
__device__ __forceinline__ void store_alg(T* __restrict__ F, I S, int base, I s, const Alg<T>& v) {
  T* p = F + ((I)base * S + s);
#pragma unroll
  for (int a = 0; a < 8; a++) p[(I)a * S] = v.a[a];
}

inline bool use_32bit_index(const Geometry& g) { return g.S * 27 < (1LL << 31) - 1; }

// ---- launch API shared between translation units (host side) ------------------
// All launches go to `stream`.  Return cudaGetLastError() of the launch.
// tile_x: sites along x per K1 block tile (kThreads/tile_x along y); chosen by the autotuner.
template <typename T>
cudaError_t launch_efield_jstat(const Geometry& g, FieldPtrs<T> f, double dt, int tile_x, cudaStream_t stream,
                                int link_rows = 3);
// K1 computing everything and storing nothing: timing runs of the autotuner.
template <typename T>
cudaError_t launch_efield_dry(const Geometry& g, FieldPtrs<T> f, double dt, int tile_x, cudaStream_t stream,
                              int link_rows = 3);
template <typename T>
cudaError_t launch_links_j(const Geometry& g, FieldPtrs<T> f, double dt, bool save_uold, bool do_j, bool do_second_half,
                           cudaStream_t stream, int link_rows = 3);
// The whole step in one launch: reads U, J, JStat of time t from `in`, writes those of t+dt to `out`
// (distinct buffers), E in place in in.E, UOld (when save_uold) in in.UOld.  Bit-identical to
// launch_efield_jstat followed by launch_links_j.  dry: compute, store nothing (autotuner).
template <typename T>
cudaError_t launch_fused_step(const Geometry& g, FieldPtrs<T> in, FieldPtrs<T> out, double dt, bool save_uold,
                              int tile_x, bool dry, cudaStream_t stream, int link_rows = 3);
template <typename T>
cudaError_t launch_sync_ghosts(const Geometry& g, T* base, int components, cudaStream_t stream);
template <typename T>
cudaError_t launch_reunitarize(const Geometry& g, cx<T>* U, cudaStream_t stream, int link_rows = 3);
// link_rows (3 = full links, 2 = 12-real two-row storage, FP32 only) selects the link accessors of the
// leapfrog and reunitarisation kernels above; complete_links writes row 2 of every link from rows 0
// and 1, which returns a two-row array to full matrices for every other kernel.
template <typename T>
cudaError_t launch_complete_links(const Geometry& g, cx<T>* U, cudaStream_t stream);
// One step by the plaquette method: the force kernel over the plaquette owners, then the link kernel
// gathering their contributions into E.  `contrib` holds 48 S reals; `between` (optional) is recorded
// between the two launches.
// double_float (FP64 fields only): the force kernel computes in double-float arithmetic (ddf.cuh).
template <typename T>
cudaError_t launch_plaquette_step(const Geometry& g, FieldPtrs<T> f, T* contrib, double dt, bool save_uold,
                                  cudaStream_t stream, cudaEvent_t between, int link_rows = 3,
                                  bool double_float = false);

// One step by the plaquette method in one launch (march.cuh): blocks own (x, y) tiles and march along
// z; reads U, J, JStat of time t from `in`, writes those of t+dt to `out` (distinct buffers), E in
// place in in.E, UOld (when save_uold) in in.UOld.  Equal to launch_plaquette_step up to rounding.  lz: z
// slices per block (0 = chosen from the lattice).
template <typename T>
cudaError_t launch_march_step(const Geometry& g, FieldPtrs<T> in, FieldPtrs<T> out, double dt, bool save_uold, int lz,
                              cudaStream_t stream, int link_rows = 3);

// Sub-step kernels with the reference's exact sub-step boundaries.
template <typename T>
cudaError_t launch_efield_only(const Geometry& g, FieldPtrs<T> f, double dt, int tile_x, cudaStream_t stream);
template <typename T>
cudaError_t launch_jstat_only(const Geometry& g, FieldPtrs<T> f, double dt, int tile_x, cudaStream_t stream);
template <typename T>
cudaError_t launch_j_only(const Geometry& g, FieldPtrs<T> f, double dt, cudaStream_t stream);
template <typename T>
cudaError_t launch_links_only(const Geometry& g, FieldPtrs<T> f, double dt, cudaStream_t stream);
template <typename T>
cudaError_t launch_copy_links(const Geometry& g, const cx<T>* src, cx<T>* dst, cudaStream_t stream);

// AoS (reference host layout, double) <-> SoA (device, T).  `aos` is device memory.
template <typename T>
cudaError_t launch_aos_to_soa(const double* aos, T* soa, long long S, int per_site, cudaStream_t stream);
template <typename T>
cudaError_t launch_soa_to_aos(const T* soa, double* aos, long long S, int per_site, cudaStream_t stream);

// Observables.  `partials` is device scratch of at least observable_scratch_doubles(g) doubles.
long long observable_scratch_doubles(const Geometry& g);
template <typename T>
cudaError_t launch_bulk(const Geometry& g, FieldPtrs<T> f, double* partials, double* result7, cudaStream_t stream);
template <typename T>
cudaError_t launch_gauss(const Geometry& g, FieldPtrs<T> f, double a_scale, double* partials, double* result2,
                         double* zprofile, cudaStream_t stream);
template <typename T>
cudaError_t launch_unitarity(const Geometry& g, const cx<T>* U, double* partials, double* result2, cudaStream_t stream);
template <typename T>
cudaError_t launch_emt_map(const Geometry& g, FieldPtrs<T> f, double a_scale, double* partials, double* result,
                           cudaStream_t stream);

}  // namespace glasma

// leapfrog.cu -- one real-time leapfrog step of classical SU(3) Yang-Mills with
// colour currents, as Dynamics::SUNc::Update (S/DYNAMICS/SUNcDynamics.cpp:353-378)
// defines it, in two fused launches per step:
//
//   K1 efield_jstat  (stencil)   UpdateElectricFields (:134-203) + UpdateJStat (:205-236)
//                                Both read the links of time t only, so they share a launch.
//   K2 links_j       (pointwise) UpdateGaugeLinks(dt/2) (:62-106), SaveOldLink (:108-128, optional),
//                                UpdateJ (:238-269), UpdateGaugeLinks(dt/2) again.
//                                UpdateJ reads U_z at t+dt/2 of the same site and JpStat/JmStat
//                                (finished by K1), so the whole tail of the step is pointwise;
//                                exp(i cU E) is formed once per link and applied twice.
//
// The electric force uses the staple form
//   E_mu^a += gamma c_mu ReTr(i t^a U_mu(x) sum_nu c_nu [S_{+nu} + S_{-nu}]),
//   S_{+nu} = U_nu(x+mu) U_mu^d(x+nu) U_nu^d(x),  S_{-nu} = U_nu^d(x+mu-nu) U_mu^d(x-nu) U_nu(x-nu),
// which is the reference's nine-plaquette expression (S/CALC/Plaquettes.cpp:83-97 with
// SUNcDynamics.cpp:181-183) regrouped by linearity of ReTr(i t^a .) and the identity
// ReTr(i t^a W^dagger) = -ReTr(i t^a W).  Ghost slices are written by the threads that own
// slice 0 and slice Nz-1, which is the reference's SynchronizeGhostCells after each sub-step.
#include "leapfrog_sites.cuh"
#include "march.cuh"

namespace glasma {

namespace {

// R: rows of each link the kernel reads and writes (3 full, 2 for 12-real links).
// The parameter structs are __grid_constant__: the site bodies take them by reference, and without
// the annotation the compiler copies them to each thread's stack (FP32 K1: 208 B of stack, 304 B of
// spill stores; with it 88 and 104 B, and none at all with 12-real links), read from the constant
// bank in place instead.
template <typename T, typename I, int R>
__global__ void __launch_bounds__(kThreads, Occupancy<T>::kMinBlocks)
    efield_jstat_kernel(const __grid_constant__ Geometry g, const __grid_constant__ FieldPtrs<T> f,
                        const __grid_constant__ EParams<T> p, const __grid_constant__ TileMap tm) {
  __shared__ cx<T> sh[StapleShare<T>::kSlots * 9 * kThreads + 1];
  int x, y, z;
  if (!tm.site(blockIdx.x, threadIdx.x, g.nx, g.ny, x, y, z)) return;
  efield_site<T, I, R>(g, f, p, x, y, z, StapleShare<T>::kSlots ? sh : nullptr);
}

template <typename T, typename I, int R>
__global__ void __launch_bounds__(kThreads, Occupancy<T>::kLinksMinBlocks)
    links_j_kernel(const __grid_constant__ Geometry g, const __grid_constant__ FieldPtrs<T> f,
                   const __grid_constant__ LParams<T> p) {
  const I idx = (I)blockIdx.x * (I)blockDim.x + (I)threadIdx.x;
  if (idx >= (I)g.vol) return;
  links_site<T, I, R>(g, f, p, idx);
}

template <typename T, typename I, int R>
__global__ void __launch_bounds__(kThreads, Occupancy<T>::kFusedMinBlocks)
    fused_step_kernel(const __grid_constant__ Geometry g, const __grid_constant__ FieldPtrs<T> in,
                      const __grid_constant__ FieldPtrs<T> out, const __grid_constant__ EParams<T> pe,
                      const __grid_constant__ LParams<T> pl, const __grid_constant__ TileMap tm) {
  __shared__ cx<T> sh[StapleShare<T>::kSlots * 9 * kThreads + 1];
  int x, y, z;
  if (!tm.site(blockIdx.x, threadIdx.x, g.nx, g.ny, x, y, z)) return;
  fused_site<T, I, R>(g, in, out, pe, pl, x, y, z, StapleShare<T>::kSlots ? sh : nullptr);
}

// The plaquette method (leapfrog_sites.cuh): K1' over the plaquette owners of slices -1 .. Nz-1,
// K2' gathering the contributions into E before the link update.
template <typename T, typename I, int R, typename TC>
__global__ void __launch_bounds__(kThreads, PlaqOccupancy<T, TC>::kMinBlocks)
    plaquette_kernel(const __grid_constant__ Geometry g, const __grid_constant__ FieldPtrs<T> f, T* __restrict__ C,
                     const __grid_constant__ EParams<T> p) {
  const I idx = (I)blockIdx.x * (I)blockDim.x + (I)threadIdx.x;
  if (idx >= (I)(g.plane * (g.nz + 1))) return;
  plaquette_site<T, I, R, TC>(g, f, C, p, idx);
}

template <typename T, typename I, int R>
__global__ void __launch_bounds__(kThreads, Occupancy<T>::kLinksMinBlocks)
    links_gather_kernel(const __grid_constant__ Geometry g, const __grid_constant__ FieldPtrs<T> f,
                        const T* __restrict__ C, const __grid_constant__ LParams<T> p) {
  const I idx = (I)blockIdx.x * (I)blockDim.x + (I)threadIdx.x;
  if (idx >= (I)g.vol) return;
  links_site<T, I, R, true>(g, f, p, idx, C);
}

template <typename T, typename I>
__global__ void __launch_bounds__(kThreads) j_only_kernel(Geometry g, FieldPtrs<T> f, T cj) {
  const I idx = (I)blockIdx.x * (I)blockDim.x + (I)threadIdx.x;
  if (idx >= (I)g.vol) return;
  const I S = (I)g.S, plane = (I)g.plane;
  const I s = idx + plane;
  const int z = (int)(idx / plane);
  const I sg = (z == 0) ? s - plane : (z == g.nz - 1 ? s + plane : (I)-1);
  Mat<T> uz;
  load_link(f.U, S, 2, s, uz);
  Alg<T> up, um, st, j;
  load_alg(f.JpStat, S, 0, s + plane, st);
  load_alg(f.JmStat, S, 0, s + plane, j);
  rotate_currents<T, true>(uz, st, j, up, um);
  load_alg(f.JpStat, S, 0, s, st);
  load_alg(f.Jp, S, 0, s, j);
#pragma unroll
  for (int a = 0; a < 8; a++) j.a[a] += -cj * (up.a[a] - st.a[a]);
  store_alg(f.Jp, S, 0, s, j);
  if (sg >= 0) store_alg(f.Jp, S, 0, sg, j);
  up = um;
  load_alg(f.JmStat, S, 0, s, st);
  load_alg(f.Jm, S, 0, s, j);
#pragma unroll
  for (int a = 0; a < 8; a++) j.a[a] += cj * (up.a[a] - st.a[a]);
  store_alg(f.Jm, S, 0, s, j);
  if (sg >= 0) store_alg(f.Jm, S, 0, sg, j);
}

// Ghost-slice copy for `components` component arrays of element type E.
template <typename E>
__global__ void sync_ghosts_kernel(E* base, long long S, long long plane, int nz, int components) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long per = plane * components;
  if (i >= per) return;
  const long long c = i / plane, r = i - c * plane;
  E* p = base + c * S;
  p[r] = p[plane + r];                                   // z=-1  <- z=0
  p[(long long)(nz + 1) * plane + r] = p[(long long)nz * plane + r];  // z=Nz <- z=Nz-1
}

template <typename T, int R>
__global__ void reunitarize_kernel(Geometry g, cx<T>* U) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.S * 3) return;
  const int mu = (int)(i / g.S);
  const long long s = i - (long long)mu * g.S;
  Mat<T> u;
  load_link_r<R, T, long long>(U, g.S, mu, s, u);
  reunitarize(u);
  store_link_r<R, T, long long>(U, g.S, mu, s, u);
}

// Row 2 of every link (ghost slices included) from rows 0 and 1: two-row storage back to full links.
template <typename T>
__global__ void complete_links_kernel(Geometry g, cx<T>* U) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.S * 3) return;
  const int mu = (int)(i / g.S);
  const long long s = i - (long long)mu * g.S;
  Mat<T> u;
  load_link_r<2, T, long long>(U, g.S, mu, s, u);
  cx<T>* p = U + (long long)(mu * 9) * g.S + s;
#pragma unroll
  for (int j = 0; j < 3; j++) p[(long long)(3 * j + 2) * g.S] = u.e[3 * j + 2];
}

template <typename E>
__global__ void copy_kernel(const E* __restrict__ src, E* __restrict__ dst, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i];
}

inline unsigned grid_for(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// Stencil kernels without shared memory (the FP32 ones) ask for the whole unified L1/shared array as
// L1, since their neighbour links are re-read from L1.  The FP64 ones keep per-thread staple slots in
// shared memory and leave the split to the driver (a zero carve-out would cost them resident
// blocks).  Once per kernel and process.
template <typename T, typename K>
void prefer_l1(K kernel) {
  static bool done = false;
  if (!done) {
    if (StapleShare<T>::kSlots == 0) {
      cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
      cudaGetLastError();
    }
    done = true;
  }
}

// Two-row (12-real) link storage is built for FP32 only: the FP64 kernels are bound by the FP64 pipe,
// and the row reconstruction would add FP64 work to save bytes that do not bound them.
template <typename T>
bool two_row(int link_rows) {
  return sizeof(T) == 4 && link_rows == 2;
}

template <typename T, int R>
void launch_efield_rows(const Geometry& g, FieldPtrs<T> f, const EParams<T>& p, const TileMap& tm, unsigned grid,
                        cudaStream_t stream) {
  if (use_32bit_index(g)) {
    prefer_l1<T>(efield_jstat_kernel<T, int, R>);
    efield_jstat_kernel<T, int, R><<<grid, kThreads, 0, stream>>>(g, f, p, tm);
  } else {
    prefer_l1<T>(efield_jstat_kernel<T, long long, R>);
    efield_jstat_kernel<T, long long, R><<<grid, kThreads, 0, stream>>>(g, f, p, tm);
  }
}

template <typename T>
cudaError_t launch_efield_kernel(const Geometry& g, FieldPtrs<T> f, const EParams<T>& p, int tile_x,
                                 cudaStream_t stream, int link_rows = 3) {
  if (tile_x <= 0 || tile_x > kThreads || kThreads % tile_x) tile_x = kThreads;
  const TileMap tm = TileMap::make(g.nx, g.ny, tile_x, kThreads);
  const unsigned grid = (unsigned)tm.tiles(g.nz);
  if constexpr (sizeof(T) == 4) {
    if (two_row<T>(link_rows)) {
      launch_efield_rows<T, 2>(g, f, p, tm, grid, stream);
      return cudaGetLastError();
    }
  }
  launch_efield_rows<T, 3>(g, f, p, tm, grid, stream);
  return cudaGetLastError();
}

template <typename T>
EParams<T> make_eparams(const Geometry& g, double dt, int do_e, int do_jstat, int dry) {
  EParams<T> p;
  const double a3 = g.a[0] * g.a[1] * g.a[2];
  const double gamma = -2.0 * dt * a3;
  for (int mu = 0; mu < 3; mu++) {
    const double ce = 1.0 / (g.a[mu] * g.a[mu]);
    p.gc[mu] = (T)(gamma * ce);
    p.cnu[mu] = (T)ce;
  }
  p.jz = (T)(-(dt / g.a[2]) * 0.70710678118654752440084436210484903928483593768847);
  p.cj = (T)(dt / g.a[2]);
  p.do_e = do_e;
  p.do_jstat = do_jstat;
  p.dry = dry;
  return p;
}

}  // namespace

template <typename T>
cudaError_t launch_efield_jstat(const Geometry& g, FieldPtrs<T> f, double dt, int tile_x, cudaStream_t stream,
                                int link_rows) {
  return launch_efield_kernel<T>(g, f, make_eparams<T>(g, dt, 1, 1, 0), tile_x, stream, link_rows);
}

template <typename T>
cudaError_t launch_efield_dry(const Geometry& g, FieldPtrs<T> f, double dt, int tile_x, cudaStream_t stream,
                              int link_rows) {
  return launch_efield_kernel<T>(g, f, make_eparams<T>(g, dt, 1, 1, 1), tile_x, stream, link_rows);
}

template <typename T>
cudaError_t launch_efield_only(const Geometry& g, FieldPtrs<T> f, double dt, int tile_x, cudaStream_t stream) {
  return launch_efield_kernel<T>(g, f, make_eparams<T>(g, dt, 1, 0, 0), tile_x, stream);
}

template <typename T>
cudaError_t launch_jstat_only(const Geometry& g, FieldPtrs<T> f, double dt, int tile_x, cudaStream_t stream) {
  return launch_efield_kernel<T>(g, f, make_eparams<T>(g, dt, 0, 1, 0), tile_x, stream);
}

template <typename T>
LParams<T> make_lparams(const Geometry& g, double dt, bool save_uold, bool do_j, bool do_second) {
  LParams<T> p;
  const double a3 = g.a[0] * g.a[1] * g.a[2];
  for (int mu = 0; mu < 3; mu++) p.cU[mu] = (T)(-(0.5 * dt) * g.a[mu] * g.a[mu] / a3);
  p.cj = (T)(dt / g.a[2]);
  p.save_uold = save_uold ? 1 : 0;
  p.do_j = do_j ? 1 : 0;
  p.do_second = do_second ? 1 : 0;
  return p;
}

template <typename T, int R>
void launch_fused_rows(const Geometry& g, FieldPtrs<T> in, FieldPtrs<T> out, const EParams<T>& pe,
                       const LParams<T>& pl, const TileMap& tm, unsigned grid, cudaStream_t stream) {
  if (use_32bit_index(g)) {
    prefer_l1<T>(fused_step_kernel<T, int, R>);
    fused_step_kernel<T, int, R><<<grid, kThreads, 0, stream>>>(g, in, out, pe, pl, tm);
  } else {
    prefer_l1<T>(fused_step_kernel<T, long long, R>);
    fused_step_kernel<T, long long, R><<<grid, kThreads, 0, stream>>>(g, in, out, pe, pl, tm);
  }
}

template <typename T>
cudaError_t launch_fused_step(const Geometry& g, FieldPtrs<T> in, FieldPtrs<T> out, double dt, bool save_uold,
                              int tile_x, bool dry, cudaStream_t stream, int link_rows) {
  if (tile_x <= 0 || tile_x > kThreads || kThreads % tile_x) tile_x = kThreads;
  const TileMap tm = TileMap::make(g.nx, g.ny, tile_x, kThreads);
  const unsigned grid = (unsigned)tm.tiles(g.nz);
  const EParams<T> pe = make_eparams<T>(g, dt, 1, 1, dry ? 1 : 0);
  const LParams<T> pl = make_lparams<T>(g, dt, save_uold, true, true);
  if constexpr (sizeof(T) == 4) {
    if (two_row<T>(link_rows)) {
      launch_fused_rows<T, 2>(g, in, out, pe, pl, tm, grid, stream);
      return cudaGetLastError();
    }
  }
  launch_fused_rows<T, 3>(g, in, out, pe, pl, tm, grid, stream);
  return cudaGetLastError();
}

#ifndef GLASMA_MARCH_TX
#define GLASMA_MARCH_TX 32
#endif
constexpr int kMarchTileX = GLASMA_MARCH_TX;  // tile of kMarchTileX x (128 / kMarchTileX) sites

template <typename T, typename I, int R>
void launch_march_kernel(const Geometry& g, FieldPtrs<T> in, FieldPtrs<T> out, const MarchParams<T>& mp, unsigned grid,
                         cudaStream_t stream) {
  const int smem = (int)(kMarchSmemReals * sizeof(T));
  cudaFuncSetAttribute(march_step_kernel<T, I, R, kMarchTileX>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  march_step_kernel<T, I, R, kMarchTileX><<<grid, kMarchThreads, smem, stream>>>(g, in, out, mp);
}

template <typename T, int R>
void launch_march_rows(const Geometry& g, FieldPtrs<T> in, FieldPtrs<T> out, const MarchParams<T>& mp, unsigned grid,
                       cudaStream_t stream) {
  if (use_32bit_index(g))
    launch_march_kernel<T, int, R>(g, in, out, mp, grid, stream);
  else
    launch_march_kernel<T, long long, R>(g, in, out, mp, grid, stream);
}

// Slices per block of the z-marching step: enough (tile, chunk) blocks to fill every SM several times
// over, and chunks long enough that the warm-up slice below each chunk stays a small share.
int march_chunk(const Geometry& g, long long tiles) {
  const long long want = 152LL * 8;  // blocks
  long long chunks = (want + tiles - 1) / tiles;
  if (chunks > g.nz) chunks = g.nz;
  if (chunks < 1) chunks = 1;
  int lz = (int)((g.nz + chunks - 1) / chunks);
  const int min_lz = g.nz < 8 ? g.nz : 8;
  return lz < min_lz ? min_lz : lz;
}

template <typename T>
cudaError_t launch_march_step(const Geometry& g, FieldPtrs<T> in, FieldPtrs<T> out, double dt, bool save_uold, int lz,
                              cudaStream_t stream, int link_rows) {
  MarchParams<T> mp;
  mp.pe = make_eparams<T>(g, dt, 1, 1, 0);
  mp.pl = make_lparams<T>(g, dt, save_uold, true, true);
  constexpr int ty = kMarchThreads / kMarchTileX;
  mp.ntx = (g.nx + kMarchTileX - 1) / kMarchTileX;
  mp.nty = (g.ny + ty - 1) / ty;
  const long long tiles = (long long)mp.ntx * mp.nty;
  mp.lz = lz > 0 ? (lz < g.nz ? lz : g.nz) : march_chunk(g, tiles);
  const long long chunks = (g.nz + mp.lz - 1) / mp.lz;
  const unsigned grid = (unsigned)(tiles * chunks);
  if constexpr (sizeof(T) == 4) {
    if (two_row<T>(link_rows)) {
      launch_march_rows<T, 2>(g, in, out, mp, grid, stream);
      return cudaGetLastError();
    }
  }
  launch_march_rows<T, 3>(g, in, out, mp, grid, stream);
  return cudaGetLastError();
}

template <typename T, int R>
void launch_links_rows(const Geometry& g, FieldPtrs<T> f, const LParams<T>& p, cudaStream_t stream) {
  if (use_32bit_index(g))
    links_j_kernel<T, int, R><<<grid_for(g.vol, kThreads), kThreads, 0, stream>>>(g, f, p);
  else
    links_j_kernel<T, long long, R><<<grid_for(g.vol, kThreads), kThreads, 0, stream>>>(g, f, p);
}

template <typename T, typename I, int R>
void launch_plaquette_rows(const Geometry& g, FieldPtrs<T> f, T* C, const EParams<T>& pe, const LParams<T>& pl,
                           cudaStream_t stream, cudaEvent_t between, bool double_float) {
  const unsigned grid = grid_for(g.plane * (g.nz + 1), kThreads);
  if constexpr (sizeof(T) == 8) {
    if (double_float)
      plaquette_kernel<T, I, R, ddf><<<grid, kThreads, 0, stream>>>(g, f, C, pe);
    else
      plaquette_kernel<T, I, R, T><<<grid, kThreads, 0, stream>>>(g, f, C, pe);
  } else {
    plaquette_kernel<T, I, R, T><<<grid, kThreads, 0, stream>>>(g, f, C, pe);
  }
  if (between) cudaEventRecord(between, stream);
  links_gather_kernel<T, I, R><<<grid_for(g.vol, kThreads), kThreads, 0, stream>>>(g, f, C, pl);
}

template <typename T>
cudaError_t launch_plaquette_step(const Geometry& g, FieldPtrs<T> f, T* contrib, double dt, bool save_uold,
                                  cudaStream_t stream, cudaEvent_t between, int link_rows, bool double_float) {
  const EParams<T> pe = make_eparams<T>(g, dt, 1, 1, 0);
  const LParams<T> pl = make_lparams<T>(g, dt, save_uold, true, true);
  // the contribution buffer has 48 S entries: 32-bit offsets only while that fits
  const bool i32 = g.S * 48 < (1LL << 31) - 1;
  if constexpr (sizeof(T) == 4) {
    if (two_row<T>(link_rows)) {
      i32 ? launch_plaquette_rows<T, int, 2>(g, f, contrib, pe, pl, stream, between, false)
          : launch_plaquette_rows<T, long long, 2>(g, f, contrib, pe, pl, stream, between, false);
      return cudaGetLastError();
    }
  }
  i32 ? launch_plaquette_rows<T, int, 3>(g, f, contrib, pe, pl, stream, between, double_float)
      : launch_plaquette_rows<T, long long, 3>(g, f, contrib, pe, pl, stream, between, double_float);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_links_j(const Geometry& g, FieldPtrs<T> f, double dt, bool save_uold, bool do_j, bool do_second,
                           cudaStream_t stream, int link_rows) {
  const LParams<T> p = make_lparams<T>(g, dt, save_uold, do_j, do_second);
  if constexpr (sizeof(T) == 4) {
    if (two_row<T>(link_rows)) {
      launch_links_rows<T, 2>(g, f, p, stream);
      return cudaGetLastError();
    }
  }
  launch_links_rows<T, 3>(g, f, p, stream);
  return cudaGetLastError();
}

// UpdateGaugeLinks(dt) alone: U <- exp(i (-dt a_mu^2/a^3) t.E_mu) U.
template <typename T>
cudaError_t launch_links_only(const Geometry& g, FieldPtrs<T> f, double dt, cudaStream_t stream) {
  return launch_links_j<T>(g, f, 2.0 * dt, false, false, false, stream);
}

template <typename T>
cudaError_t launch_j_only(const Geometry& g, FieldPtrs<T> f, double dt, cudaStream_t stream) {
  if (use_32bit_index(g))
    j_only_kernel<T, int><<<grid_for(g.vol, kThreads), kThreads, 0, stream>>>(g, f, (T)(dt / g.a[2]));
  else
    j_only_kernel<T, long long><<<grid_for(g.vol, kThreads), kThreads, 0, stream>>>(g, f, (T)(dt / g.a[2]));
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_sync_ghosts(const Geometry& g, T* base, int components, cudaStream_t stream) {
  const long long n = g.plane * components;
  sync_ghosts_kernel<T><<<grid_for(n, 256), 256, 0, stream>>>(base, g.S, g.plane, g.nz, components);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_reunitarize(const Geometry& g, cx<T>* U, cudaStream_t stream, int link_rows) {
  if constexpr (sizeof(T) == 4) {
    if (two_row<T>(link_rows)) {
      reunitarize_kernel<T, 2><<<grid_for(g.S * 3, kThreads), kThreads, 0, stream>>>(g, U);
      return cudaGetLastError();
    }
  }
  reunitarize_kernel<T, 3><<<grid_for(g.S * 3, kThreads), kThreads, 0, stream>>>(g, U);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_complete_links(const Geometry& g, cx<T>* U, cudaStream_t stream) {
  complete_links_kernel<T><<<grid_for(g.S * 3, 256), 256, 0, stream>>>(g, U);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_copy_links(const Geometry& g, const cx<T>* src, cx<T>* dst, cudaStream_t stream) {
  const long long n = g.S * 27;
  copy_kernel<cx<T>><<<grid_for(n, 256), 256, 0, stream>>>(src, dst, n);
  return cudaGetLastError();
}

#define GLASMA_INSTANTIATE(T)                                                                                   \
  template cudaError_t launch_fused_step<T>(const Geometry&, FieldPtrs<T>, FieldPtrs<T>, double, bool, int, bool, \
                                            cudaStream_t, int);                                                 \
  template cudaError_t launch_efield_jstat<T>(const Geometry&, FieldPtrs<T>, double, int, cudaStream_t, int);  \
  template cudaError_t launch_efield_dry<T>(const Geometry&, FieldPtrs<T>, double, int, cudaStream_t, int);    \
  template cudaError_t launch_efield_only<T>(const Geometry&, FieldPtrs<T>, double, int, cudaStream_t);        \
  template cudaError_t launch_jstat_only<T>(const Geometry&, FieldPtrs<T>, double, int, cudaStream_t);         \
  template cudaError_t launch_links_j<T>(const Geometry&, FieldPtrs<T>, double, bool, bool, bool, cudaStream_t,  \
                                         int);                                                                  \
  template cudaError_t launch_links_only<T>(const Geometry&, FieldPtrs<T>, double, cudaStream_t);              \
  template cudaError_t launch_j_only<T>(const Geometry&, FieldPtrs<T>, double, cudaStream_t);                  \
  template cudaError_t launch_reunitarize<T>(const Geometry&, cx<T>*, cudaStream_t, int);                      \
  template cudaError_t launch_complete_links<T>(const Geometry&, cx<T>*, cudaStream_t);                        \
  template cudaError_t launch_march_step<T>(const Geometry&, FieldPtrs<T>, FieldPtrs<T>, double, bool, int,      \
                                            cudaStream_t, int);                                                 \
  template cudaError_t launch_plaquette_step<T>(const Geometry&, FieldPtrs<T>, T*, double, bool, cudaStream_t,  \
                                                cudaEvent_t, int, bool);                                        \
  template cudaError_t launch_copy_links<T>(const Geometry&, const cx<T>*, cx<T>*, cudaStream_t);              \
  template cudaError_t launch_sync_ghosts<T>(const Geometry&, T*, int, cudaStream_t);                          \
  template cudaError_t launch_sync_ghosts<cx<T>>(const Geometry&, cx<T>*, int, cudaStream_t);

GLASMA_INSTANTIATE(double)
GLASMA_INSTANTIATE(float)

}  // namespace glasma

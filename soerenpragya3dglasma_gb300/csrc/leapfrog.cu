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
#include "lattice.cuh"

namespace glasma {

namespace {

constexpr int kThreads = 128;

// Blocks per SM the register allocation must leave room for (the register cap is 64K / (128 * n)),
// chosen by measurement on GB300; overridable at build time for tuning sweeps.
#ifndef GLASMA_FP64_MIN_BLOCKS
#define GLASMA_FP64_MIN_BLOCKS 2
#endif
#ifndef GLASMA_FP32_MIN_BLOCKS
#define GLASMA_FP32_MIN_BLOCKS 3
#endif
template <typename T>
struct Occupancy;
template <>
struct Occupancy<double> {
  static constexpr int kMinBlocks = GLASMA_FP64_MIN_BLOCKS;
};
template <>
struct Occupancy<float> {
  static constexpr int kMinBlocks = GLASMA_FP32_MIN_BLOCKS;
};

template <typename I>
__device__ __forceinline__ I nb(const Geometry& g, int x, int y, int z, int dx, int dy, int dz) {
  int xx = x + dx, yy = y + dy;
  xx = xx < 0 ? xx + g.nx : (xx >= g.nx ? xx - g.nx : xx);
  yy = yy < 0 ? yy + g.ny : (yy >= g.ny ? yy - g.ny : yy);
  return (I)xx + (I)g.nx * ((I)yy + (I)g.ny * (I)(z + dz + 1));
}

template <typename I>
__device__ __forceinline__ void decode(const Geometry& g, I idx, int& x, int& y, int& z) {
  const I r = idx / (I)g.nx;
  x = (int)(idx - r * (I)g.nx);
  z = (int)(r / (I)g.ny);
  y = (int)(r - (I)z * (I)g.ny);
}

// Staples of link mu at x in the (mu,nu) plane, weighted by c, added to acc.
template <typename T, typename I>
__device__ __forceinline__ void add_staples(const cx<T>* __restrict__ U, I S, int mu, int nu, I s, I s_pmu, I s_pnu,
                                            I s_pmu_mnu, I s_mnu, T c, Mat<T>& acc) {
  Mat<T> a, b, t;
  load_link(U, S, nu, s_pmu, a);
  load_link(U, S, mu, s_pnu, b);
  mul_nd(a, b, t);
  load_link(U, S, nu, s, a);
  add_mul_nd(t, a, c, acc);
  load_link(U, S, nu, s_pmu_mnu, a);
  load_link(U, S, mu, s_mnu, b);
  mul_dd(a, b, t);
  load_link(U, S, nu, s_mnu, a);
  add_mul_nn(t, a, c, acc);
}

template <typename T>
struct EParams {
  T gc[3];    // gamma * cE[mu],   gamma = -2 dt a^3, cE = 1/a_mu^2
  T cnu[3];   // cE[nu]
  T jz;       // -(dt/a_z)/sqrt(2)
  T cj;       // dt/a_z
  int do_e, do_jstat;
};

template <typename T, typename I>
__global__ void __launch_bounds__(kThreads, Occupancy<T>::kMinBlocks)
    efield_jstat_kernel(Geometry g, FieldPtrs<T> f, EParams<T> p) {
  const I idx = (I)blockIdx.x * (I)blockDim.x + (I)threadIdx.x;
  if (idx >= (I)g.vol) return;
  int x, y, z;
  decode<I>(g, idx, x, y, z);
  const I S = (I)g.S, plane = (I)g.plane;
  const I s = idx + plane;
  const bool lo = (z == 0), hi = (z == g.nz - 1);
  const I sg = lo ? s - plane : (hi ? s + plane : (I)-1);
  if (p.do_e) {
    const I sxp = nb<I>(g, x, y, z, 1, 0, 0), sxm = nb<I>(g, x, y, z, -1, 0, 0);
    const I syp = nb<I>(g, x, y, z, 0, 1, 0), sym = nb<I>(g, x, y, z, 0, -1, 0);
    const I szp = s + plane, szm = s - plane;
#pragma unroll 1
    for (int mu = 0; mu < 3; mu++) {
      Mat<T> acc;
      set_zero(acc);
      if (mu == 0) {
        add_staples(f.U, S, 0, 1, s, sxp, syp, nb<I>(g, x, y, z, 1, -1, 0), sym, p.cnu[1], acc);
        add_staples(f.U, S, 0, 2, s, sxp, szp, nb<I>(g, x, y, z, 1, 0, -1), szm, p.cnu[2], acc);
      } else if (mu == 1) {
        add_staples(f.U, S, 1, 0, s, syp, sxp, nb<I>(g, x, y, z, -1, 1, 0), sxm, p.cnu[0], acc);
        add_staples(f.U, S, 1, 2, s, syp, szp, nb<I>(g, x, y, z, 0, 1, -1), szm, p.cnu[2], acc);
      } else {
        add_staples(f.U, S, 2, 0, s, szp, sxp, nb<I>(g, x, y, z, -1, 0, 1), sxm, p.cnu[0], acc);
        add_staples(f.U, S, 2, 1, s, szp, syp, nb<I>(g, x, y, z, 0, -1, 1), sym, p.cnu[1], acc);
      }
      Mat<T> u, P;
      load_link(f.U, S, mu, s, u);
      mul_nn(u, acc, P);
      Alg<T> force, e;
      retr_itg(P, p.gc[mu], force);
      load_alg(f.E, S, mu * 8, s, e);
#pragma unroll
      for (int a = 0; a < 8; a++) e.a[a] += force.a[a];
      if (mu == 2) {
        Alg<T> jp, jm;
        load_alg(f.Jp, S, 0, s, jp);
        load_alg(f.Jm, S, 0, s, jm);
#pragma unroll
        for (int a = 0; a < 8; a++) e.a[a] += p.jz * (jp.a[a] - jm.a[a]);
      }
      store_alg(f.E, S, mu * 8, s, e);
      if (sg >= 0) store_alg(f.E, S, mu * 8, sg, e);
    }
  }
  if (p.do_jstat) {
    const I szm = s - plane;
    Mat<T> uzm;
    load_link(f.U, S, 2, szm, uzm);
    Alg<T> down, jc, st;
    load_alg(f.Jp, S, 0, szm, jc);
    inv_adj_mul(uzm, jc, down);
    load_alg(f.Jp, S, 0, s, jc);
    load_alg(f.JpStat, S, 0, s, st);
#pragma unroll
    for (int a = 0; a < 8; a++) st.a[a] += -p.cj * (jc.a[a] - down.a[a]);
    store_alg(f.JpStat, S, 0, s, st);
    if (sg >= 0) store_alg(f.JpStat, S, 0, sg, st);
    load_alg(f.Jm, S, 0, szm, jc);
    inv_adj_mul(uzm, jc, down);
    load_alg(f.Jm, S, 0, s, jc);
    load_alg(f.JmStat, S, 0, s, st);
#pragma unroll
    for (int a = 0; a < 8; a++) st.a[a] += p.cj * (jc.a[a] - down.a[a]);
    store_alg(f.JmStat, S, 0, s, st);
    if (sg >= 0) store_alg(f.JmStat, S, 0, sg, st);
  }
}

template <typename T>
struct LParams {
  T cU[3];  // -(h) a_mu^2 / a^3 for the half step h
  T cj;     // dt/a_z
  int save_uold, do_j, do_second;
};

template <typename T, typename I>
__global__ void __launch_bounds__(kThreads, Occupancy<T>::kMinBlocks)
    links_j_kernel(Geometry g, FieldPtrs<T> f, LParams<T> p) {
  const I idx = (I)blockIdx.x * (I)blockDim.x + (I)threadIdx.x;
  if (idx >= (I)g.vol) return;
  const I S = (I)g.S, plane = (I)g.plane;
  const I s = idx + plane;
  const int z = (int)(idx / plane);
  const bool lo = (z == 0), hi = (z == g.nz - 1);
  const I sg = lo ? s - plane : (hi ? s + plane : (I)-1);
#pragma unroll 1
  for (int mu = 0; mu < 3; mu++) {
    Alg<T> e;
    load_alg(f.E, S, mu * 8, s, e);
    Mat<T> X, u, uh;
    expi(p.cU[mu], e, X);
    load_link(f.U, S, mu, s, u);
    mul_nn(X, u, uh);
    if (p.save_uold) {
      store_link(f.UOld, S, mu, s, uh);
      if (sg >= 0) store_link(f.UOld, S, mu, sg, uh);
    }
    if (mu == 2 && p.do_j) {
      Alg<T> up, st, j;
      const I szp = s + plane;
      load_alg(f.JpStat, S, 0, szp, st);
      adj_mul(uh, st, up);
      load_alg(f.JpStat, S, 0, s, st);
      load_alg(f.Jp, S, 0, s, j);
#pragma unroll
      for (int a = 0; a < 8; a++) j.a[a] += -p.cj * (up.a[a] - st.a[a]);
      store_alg(f.Jp, S, 0, s, j);
      if (sg >= 0) store_alg(f.Jp, S, 0, sg, j);
      load_alg(f.JmStat, S, 0, szp, st);
      adj_mul(uh, st, up);
      load_alg(f.JmStat, S, 0, s, st);
      load_alg(f.Jm, S, 0, s, j);
#pragma unroll
      for (int a = 0; a < 8; a++) j.a[a] += p.cj * (up.a[a] - st.a[a]);
      store_alg(f.Jm, S, 0, s, j);
      if (sg >= 0) store_alg(f.Jm, S, 0, sg, j);
    }
    if (p.do_second) {
      mul_nn(X, uh, u);
    } else {
      u = uh;
    }
    store_link(f.U, S, mu, s, u);
    if (sg >= 0) store_link(f.U, S, mu, sg, u);
  }
}

// UpdateJ alone (S/DYNAMICS/SUNcDynamics.cpp:238-269) with the links as they stand.
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
  Alg<T> up, st, j;
  load_alg(f.JpStat, S, 0, s + plane, st);
  adj_mul(uz, st, up);
  load_alg(f.JpStat, S, 0, s, st);
  load_alg(f.Jp, S, 0, s, j);
#pragma unroll
  for (int a = 0; a < 8; a++) j.a[a] += -cj * (up.a[a] - st.a[a]);
  store_alg(f.Jp, S, 0, s, j);
  if (sg >= 0) store_alg(f.Jp, S, 0, sg, j);
  load_alg(f.JmStat, S, 0, s + plane, st);
  adj_mul(uz, st, up);
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

template <typename T>
__global__ void reunitarize_kernel(Geometry g, cx<T>* U) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.S * 3) return;
  const int mu = (int)(i / g.S);
  const long long s = i - (long long)mu * g.S;
  Mat<T> u;
  load_link<T, long long>(U, g.S, mu, s, u);
  reunitarize(u);
  store_link<T, long long>(U, g.S, mu, s, u);
}

template <typename E>
__global__ void copy_kernel(const E* __restrict__ src, E* __restrict__ dst, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i];
}

inline unsigned grid_for(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

template <typename T>
cudaError_t launch_efield_kernel(const Geometry& g, FieldPtrs<T> f, const EParams<T>& p, cudaStream_t stream) {
  if (use_32bit_index(g))
    efield_jstat_kernel<T, int><<<grid_for(g.vol, kThreads), kThreads, 0, stream>>>(g, f, p);
  else
    efield_jstat_kernel<T, long long><<<grid_for(g.vol, kThreads), kThreads, 0, stream>>>(g, f, p);
  return cudaGetLastError();
}

}  // namespace

template <typename T>
cudaError_t launch_efield_jstat(const Geometry& g, FieldPtrs<T> f, double dt, cudaStream_t stream) {
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
  p.do_e = 1;
  p.do_jstat = 1;
  return launch_efield_kernel<T>(g, f, p, stream);
}

template <typename T>
cudaError_t launch_efield_only(const Geometry& g, FieldPtrs<T> f, double dt, cudaStream_t stream) {
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
  p.do_e = 1;
  p.do_jstat = 0;
  return launch_efield_kernel<T>(g, f, p, stream);
}

template <typename T>
cudaError_t launch_jstat_only(const Geometry& g, FieldPtrs<T> f, double dt, cudaStream_t stream) {
  EParams<T> p = {};
  p.cj = (T)(dt / g.a[2]);
  p.do_e = 0;
  p.do_jstat = 1;
  return launch_efield_kernel<T>(g, f, p, stream);
}

template <typename T>
cudaError_t launch_links_j(const Geometry& g, FieldPtrs<T> f, double dt, bool save_uold, bool do_j, bool do_second,
                           cudaStream_t stream) {
  LParams<T> p;
  const double a3 = g.a[0] * g.a[1] * g.a[2];
  for (int mu = 0; mu < 3; mu++) p.cU[mu] = (T)(-(0.5 * dt) * g.a[mu] * g.a[mu] / a3);
  p.cj = (T)(dt / g.a[2]);
  p.save_uold = save_uold ? 1 : 0;
  p.do_j = do_j ? 1 : 0;
  p.do_second = do_second ? 1 : 0;
  if (use_32bit_index(g))
    links_j_kernel<T, int><<<grid_for(g.vol, kThreads), kThreads, 0, stream>>>(g, f, p);
  else
    links_j_kernel<T, long long><<<grid_for(g.vol, kThreads), kThreads, 0, stream>>>(g, f, p);
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
cudaError_t launch_reunitarize(const Geometry& g, cx<T>* U, cudaStream_t stream) {
  reunitarize_kernel<T><<<grid_for(g.S * 3, kThreads), kThreads, 0, stream>>>(g, U);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_copy_links(const Geometry& g, const cx<T>* src, cx<T>* dst, cudaStream_t stream) {
  const long long n = g.S * 27;
  copy_kernel<cx<T>><<<grid_for(n, 256), 256, 0, stream>>>(src, dst, n);
  return cudaGetLastError();
}

#define GLASMA_INSTANTIATE(T)                                                                                   \
  template cudaError_t launch_efield_jstat<T>(const Geometry&, FieldPtrs<T>, double, cudaStream_t);            \
  template cudaError_t launch_efield_only<T>(const Geometry&, FieldPtrs<T>, double, cudaStream_t);             \
  template cudaError_t launch_jstat_only<T>(const Geometry&, FieldPtrs<T>, double, cudaStream_t);              \
  template cudaError_t launch_links_j<T>(const Geometry&, FieldPtrs<T>, double, bool, bool, bool, cudaStream_t); \
  template cudaError_t launch_links_only<T>(const Geometry&, FieldPtrs<T>, double, cudaStream_t);              \
  template cudaError_t launch_j_only<T>(const Geometry&, FieldPtrs<T>, double, cudaStream_t);                  \
  template cudaError_t launch_reunitarize<T>(const Geometry&, cx<T>*, cudaStream_t);                           \
  template cudaError_t launch_copy_links<T>(const Geometry&, const cx<T>*, cx<T>*, cudaStream_t);              \
  template cudaError_t launch_sync_ghosts<T>(const Geometry&, T*, int, cudaStream_t);                          \
  template cudaError_t launch_sync_ghosts<cx<T>>(const Geometry&, cx<T>*, int, cudaStream_t);

GLASMA_INSTANTIATE(double)
GLASMA_INSTANTIATE(float)

}  // namespace glasma

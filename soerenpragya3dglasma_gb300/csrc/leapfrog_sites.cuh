// leapfrog_sites.cuh -- per-site bodies of the two leapfrog kernels, shared by the single-lattice
// launches (leapfrog.cu) and the batched multi-event launches (batch.cu).
#pragma once

#include "lattice.cuh"

namespace glasma {


constexpr int kThreads = 128;

// Blocks per SM the register allocation must leave room for (the register cap is 64K / (128 * n)),
// chosen by measurement on GB300; overridable at build time for tuning sweeps.
// (GB300 sweep, 128x128x512: FP32 K1 fastest at 5 blocks/SM, K2 at 8; FP64 is FP64-ALU bound.)
#ifndef GLASMA_FP64_MIN_BLOCKS
#define GLASMA_FP64_MIN_BLOCKS 2
#endif
#ifndef GLASMA_FP32_MIN_BLOCKS
#define GLASMA_FP32_MIN_BLOCKS 5
#endif
#ifndef GLASMA_FP32_LINKS_MIN_BLOCKS
#define GLASMA_FP32_LINKS_MIN_BLOCKS 8
#endif
#ifndef GLASMA_FP32_FUSED_MIN_BLOCKS
#define GLASMA_FP32_FUSED_MIN_BLOCKS 4
#endif
template <typename T>
struct Occupancy;
template <>
struct Occupancy<double> {
  static constexpr int kMinBlocks = GLASMA_FP64_MIN_BLOCKS;       // electric-field kernel
  static constexpr int kLinksMinBlocks = GLASMA_FP64_MIN_BLOCKS;  // link/J kernel
  static constexpr int kFusedMinBlocks = GLASMA_FP64_MIN_BLOCKS;  // one-pass step kernel
};
template <>
struct Occupancy<float> {
  static constexpr int kMinBlocks = GLASMA_FP32_MIN_BLOCKS;
  static constexpr int kLinksMinBlocks = GLASMA_FP32_LINKS_MIN_BLOCKS;
  static constexpr int kFusedMinBlocks = GLASMA_FP32_FUSED_MIN_BLOCKS;
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

// v[mu] for a runtime mu without indexing the kernel-parameter array (which would copy it to the stack)
template <typename T>
__device__ __forceinline__ T pick3(const T (&v)[3], int mu) {
  return mu == 0 ? v[0] : (mu == 1 ? v[1] : v[2]);
}

// acc += c (a - b), componentwise: the update form of UpdateJStat and UpdateJ.  Every path (K1, K2,
// the fused step) uses this one expression, so they round identically.
template <typename T>
__device__ __forceinline__ void axpy_diff(Alg<T>& acc, T c, const Alg<T>& a, const Alg<T>& b) {
#pragma unroll
  for (int k = 0; k < 8; k++) acc.a[k] += c * (a.a[k] - b.a[k]);
}

// FP64 staple sharing: for mu < nu the first product of link mu's upper staple in plane nu,
// A = U_nu(x+mu) U_mu^d(x+nu), is the dagger of the first product of link nu's upper staple in plane
// mu, so it is formed once and parked in the thread's own shared-memory slot until link nu needs it
// (3 of the 27 staple matmuls saved; two slots suffice since the links are processed in order).
// On for FP32 too (measured 5 % faster K1 on GB300; GLASMA_FP32_STAPLE_SHARE=0 turns it off there).  Slot k, element e of thread t: sh[(k*9+e)*kThreads+t].
#ifndef GLASMA_FP32_STAPLE_SHARE
#define GLASMA_FP32_STAPLE_SHARE 1
#endif
template <typename T>
struct StapleShare {
  static constexpr int kSlots = (sizeof(T) == 8 || GLASMA_FP32_STAPLE_SHARE) ? 2 : 0;
};
enum StapleMode { kStapleCompute = 0, kStapleStore = 1, kStapleReuse = 2 };

// Staples of link mu at x in the (mu,nu) plane, weighted by c, added to acc.  R: rows of each link
// stored (3 full, 2 for 12-real links, see load_link_r).
template <typename T, typename I, int R = 3>
__device__ __forceinline__ void add_staples(const cx<T>* __restrict__ U, I S, int mu, int nu, I s, I s_pmu, I s_pnu,
                                            I s_pmu_mnu, I s_mnu, T c, Mat<T>& acc, cx<T>* sh = nullptr,
                                            int mode = kStapleCompute, int slot = 0) {
  Mat<T> a, b, t;
  if (sh && mode == kStapleReuse) {
    const cx<T>* q = sh + (slot * 9) * kThreads + threadIdx.x;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const cx<T> v = q[(j + 3 * i) * kThreads];
        t.e[i + 3 * j] = mk<T>(v.re, -v.im);
      }
  } else {
    load_link_r<R>(U, S, nu, s_pmu, a);
    load_link_r<R>(U, S, mu, s_pnu, b);
    mul_nd(a, b, t);
    if (sh && mode == kStapleStore) {
      cx<T>* q = sh + (slot * 9) * kThreads + threadIdx.x;
#pragma unroll
      for (int k = 0; k < 9; k++) q[k * kThreads] = t.e[k];
    }
  }
  load_link_r<R>(U, S, nu, s, a);
  add_mul_nd(t, a, c, acc);
  load_link_r<R>(U, S, nu, s_pmu_mnu, a);
  load_link_r<R>(U, S, mu, s_mnu, b);
  mul_dd(a, b, t);
  load_link_r<R>(U, S, nu, s_mnu, a);
  add_mul_nn(t, a, c, acc);
}

template <typename T>
struct EParams {
  T gc[3];    // gamma * cE[mu],   gamma = -2 dt a^3, cE = 1/a_mu^2
  T cnu[3];   // cE[nu]
  T jz;       // -(dt/a_z)/sqrt(2)
  T cj;       // dt/a_z
  int do_e, do_jstat;
  int dry;    // compute, store nothing (autotuner timing runs)
};

// The electric-field and JStat update of one site (K1's per-site body).
template <typename T, typename I, int R = 3>
__device__ __forceinline__ void efield_site(const Geometry& g, const FieldPtrs<T>& f, const EParams<T>& p, int x, int y,
                                            int z, cx<T>* sh = nullptr) {
  const I S = (I)g.S, plane = (I)g.plane;
  const I s = (I)x + (I)g.nx * ((I)y + (I)g.ny * (I)(z + 1));
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
        add_staples<T, I, R>(f.U, S, 0, 1, s, sxp, syp, nb<I>(g, x, y, z, 1, -1, 0), sym, p.cnu[1], acc, sh, kStapleStore, 0);
        add_staples<T, I, R>(f.U, S, 0, 2, s, sxp, szp, nb<I>(g, x, y, z, 1, 0, -1), szm, p.cnu[2], acc, sh, kStapleStore, 1);
      } else if (mu == 1) {
        add_staples<T, I, R>(f.U, S, 1, 0, s, syp, sxp, nb<I>(g, x, y, z, -1, 1, 0), sxm, p.cnu[0], acc, sh, kStapleReuse, 0);
        add_staples<T, I, R>(f.U, S, 1, 2, s, syp, szp, nb<I>(g, x, y, z, 0, 1, -1), szm, p.cnu[2], acc, sh, kStapleStore, 0);
      } else {
        add_staples<T, I, R>(f.U, S, 2, 0, s, szp, sxp, nb<I>(g, x, y, z, -1, 0, 1), sxm, p.cnu[0], acc, sh, kStapleReuse, 1);
        add_staples<T, I, R>(f.U, S, 2, 1, s, szp, syp, nb<I>(g, x, y, z, 0, -1, 1), sym, p.cnu[1], acc, sh, kStapleReuse, 0);
      }
      Mat<T> u, P;
      load_link_r<R>(f.U, S, mu, s, u);
      mul_nn_traceless(u, acc, P);
      Alg<T> force, e;
      retr_itg(P, pick3(p.gc, mu), force);
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
      if (!p.dry) {
        store_alg(f.E, S, mu * 8, s, e);
        if (sg >= 0) store_alg(f.E, S, mu * 8, sg, e);
      }
    }
  }
  if (p.do_jstat) {
    const I szm = s - plane;
    Mat<T> uzm;
    load_link_r<R>(f.U, S, 2, szm, uzm);
    Alg<T> down, jc, st;
    load_alg(f.Jp, S, 0, szm, jc);
    inv_adj_mul(uzm, jc, down);
    load_alg(f.Jp, S, 0, s, jc);
    load_alg(f.JpStat, S, 0, s, st);
    axpy_diff(st, -p.cj, jc, down);
    if (!p.dry) {
      store_alg(f.JpStat, S, 0, s, st);
      if (sg >= 0) store_alg(f.JpStat, S, 0, sg, st);
    }
    load_alg(f.Jm, S, 0, szm, jc);
    inv_adj_mul(uzm, jc, down);
    load_alg(f.Jm, S, 0, s, jc);
    load_alg(f.JmStat, S, 0, s, st);
    axpy_diff(st, p.cj, jc, down);
    if (!p.dry) {
      store_alg(f.JmStat, S, 0, s, st);
      if (sg >= 0) store_alg(f.JmStat, S, 0, sg, st);
    }
  }
}

// Thread-to-site map of K1: a block of kThreads threads covers a tile of tile_x x (kThreads/tile_x)
// sites of one z slice, so most y-neighbours a block reads are its own sites (L1 hits).
struct TileMap {
  int tile_x, tile_y, ntx, nty;
  __host__ __device__ static TileMap make(int nx, int ny, int tile_x, int threads) {
    TileMap t;
    t.tile_x = tile_x;
    t.tile_y = threads / tile_x;
    t.ntx = (nx + t.tile_x - 1) / t.tile_x;
    t.nty = (ny + t.tile_y - 1) / t.tile_y;
    return t;
  }
  __host__ __device__ long long tiles(int nz) const { return (long long)ntx * nty * nz; }
  // tile index -> site of thread `t` (false when the thread falls outside the lattice)
  __device__ bool site(long long tile, int t, int nx, int ny, int& x, int& y, int& z) const {
    const long long per_z = (long long)ntx * nty;
    z = (int)(tile / per_z);
    const int r = (int)(tile - (long long)z * per_z);
    const int by = r / ntx, bx = r - by * ntx;
    x = bx * tile_x + t % tile_x;
    y = by * tile_y + t / tile_x;
    return x < nx && y < ny;
  }
};

template <typename T>
struct LParams {
  T cU[3];  // -(h) a_mu^2 / a^3 for the half step h
  T cj;     // dt/a_z
  int save_uold, do_j, do_second;
};

// K2's per-site body: links to t+dt (two applications of one exp), UOld, J transport.
template <typename T, typename I, int R = 3>
__device__ __forceinline__ void links_site(const Geometry& g, const FieldPtrs<T>& f, const LParams<T>& p, I idx) {
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
    load_link_r<R>(f.U, S, mu, s, u);
    // Without a use for U(t+dt/2) (UOld, the z-link J transport), the two half steps are one:
    // exp(i c t.E)^2 = exp(2i c t.E), one matmul less (equal up to rounding).
    if (p.do_second && !p.save_uold && !(mu == 2 && p.do_j)) {
      link_exp(T(2) * pick3(p.cU, mu), e, X);
      link_apply(X, u, uh);
      store_link_r<R>(f.U, S, mu, s, uh);
      if (sg >= 0) store_link_r<R>(f.U, S, mu, sg, uh);
      continue;
    }
    link_exp(pick3(p.cU, mu), e, X);
    link_apply(X, u, uh);
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
      axpy_diff(j, -p.cj, up, st);
      store_alg(f.Jp, S, 0, s, j);
      if (sg >= 0) store_alg(f.Jp, S, 0, sg, j);
      load_alg(f.JmStat, S, 0, szp, st);
      adj_mul(uh, st, up);
      load_alg(f.JmStat, S, 0, s, st);
      load_alg(f.Jm, S, 0, s, j);
      axpy_diff(j, p.cj, up, st);
      store_alg(f.Jm, S, 0, s, j);
      if (sg >= 0) store_alg(f.Jm, S, 0, sg, j);
    }
    if (p.do_second) {
      link_apply(X, uh, u);
    } else {
      u = uh;
    }
    store_link_r<R>(f.U, S, mu, s, u);
    if (sg >= 0) store_link_r<R>(f.U, S, mu, sg, u);
  }
}

// ---- the whole step in one pass -------------------------------------------------------------------
// fused_site reads the links, currents and static currents of time t from `in` and writes those of
// t+dt to `out` (a second set of buffers; E is updated in place, it is read only at its own site).
// Because nothing it reads is written in the same launch, the sites are independent and the step is
// one launch.  The static currents of t+dt at x+z, which UpdateJ at x needs, are recomputed here from
// the inputs with K1's own expression, so the result is bit-identical to K1 followed by K2.
//   E_mu(x)      += force(U(t)) [+ J term]                          UpdateElectricFields
//   JStat(x)     += -/+ cj (J(x) - U_z^d(x-z) J(x-z) U_z(x-z))      UpdateJStat (also at x+z)
//   Uh            = exp(i cU E_mu(x)) U_mu(x)                        UpdateGaugeLinks(dt/2)
//   J(x)         += -/+ cj (Uh_z J Stat(x+z) Uh_z^d - JStat(x))     UpdateJ
//   U_mu(x; t+dt) = exp(i cU E_mu(x)) Uh                             UpdateGaugeLinks(dt/2)
template <typename T, typename I, int R = 3>
__device__ __forceinline__ void fused_currents(const FieldPtrs<T>& in, const FieldPtrs<T>& out, I S, I plane, I s,
                                               I sg, bool hi, const Mat<T>& uz, const Mat<T>& uhz, T cj, bool dry) {
  const I szm = s - plane, szp = s + plane;
  Alg<T> jc, down, sp, sm;
  {
    Mat<T> w;
    load_link_r<R>(in.U, S, 2, szm, w);
    load_alg(in.Jp, S, 0, szm, jc);
    inv_adj_mul(w, jc, down);
    load_alg(in.Jp, S, 0, s, jc);
    load_alg(in.JpStat, S, 0, s, sp);
    axpy_diff(sp, -cj, jc, down);
    load_alg(in.Jm, S, 0, szm, jc);
    inv_adj_mul(w, jc, down);
    load_alg(in.Jm, S, 0, s, jc);
    load_alg(in.JmStat, S, 0, s, sm);
    axpy_diff(sm, cj, jc, down);
  }
  if (!dry) {
    store_alg(out.JpStat, S, 0, s, sp);
    store_alg(out.JmStat, S, 0, s, sm);
    if (sg >= 0) {
      store_alg(out.JpStat, S, 0, sg, sp);
      store_alg(out.JmStat, S, 0, sg, sm);
    }
  }
  // static currents of t+dt one slice up (the ghost copy of this site's at the top slice)
  Alg<T> up, um;
  if (hi) {
    up = sp;
    um = sm;
  } else {
    load_alg(in.Jp, S, 0, s, jc);
    inv_adj_mul(uz, jc, down);
    load_alg(in.Jp, S, 0, szp, jc);
    load_alg(in.JpStat, S, 0, szp, up);
    axpy_diff(up, -cj, jc, down);
    load_alg(in.Jm, S, 0, s, jc);
    inv_adj_mul(uz, jc, down);
    load_alg(in.Jm, S, 0, szp, jc);
    load_alg(in.JmStat, S, 0, szp, um);
    axpy_diff(um, cj, jc, down);
  }
  Alg<T> t, j;
  adj_mul(uhz, up, t);
  load_alg(in.Jp, S, 0, s, j);
  axpy_diff(j, -cj, t, sp);
  if (!dry) {
    store_alg(out.Jp, S, 0, s, j);
    if (sg >= 0) store_alg(out.Jp, S, 0, sg, j);
  }
  adj_mul(uhz, um, t);
  load_alg(in.Jm, S, 0, s, j);
  axpy_diff(j, cj, t, sm);
  if (!dry) {
    store_alg(out.Jm, S, 0, s, j);
    if (sg >= 0) store_alg(out.Jm, S, 0, sg, j);
  }
}

template <typename T, typename I, int R = 3>
__device__ __forceinline__ void fused_site(const Geometry& g, const FieldPtrs<T>& in, const FieldPtrs<T>& out,
                                           const EParams<T>& pe, const LParams<T>& pl, int x, int y, int z,
                                           cx<T>* sh = nullptr) {
  const I S = (I)g.S, plane = (I)g.plane;
  const I s = (I)x + (I)g.nx * ((I)y + (I)g.ny * (I)(z + 1));
  const bool lo = (z == 0), hi = (z == g.nz - 1);
  const I sg = lo ? s - plane : (hi ? s + plane : (I)-1);
  const bool dry = pe.dry != 0;
  const I sxp = nb<I>(g, x, y, z, 1, 0, 0), sxm = nb<I>(g, x, y, z, -1, 0, 0);
  const I syp = nb<I>(g, x, y, z, 0, 1, 0), sym = nb<I>(g, x, y, z, 0, -1, 0);
  const I szp = s + plane, szm = s - plane;
#pragma unroll 1
  for (int mu = 0; mu < 3; mu++) {
    Mat<T> acc;
    set_zero(acc);
    if (mu == 0) {
      add_staples<T, I, R>(in.U, S, 0, 1, s, sxp, syp, nb<I>(g, x, y, z, 1, -1, 0), sym, pe.cnu[1], acc, sh, kStapleStore, 0);
      add_staples<T, I, R>(in.U, S, 0, 2, s, sxp, szp, nb<I>(g, x, y, z, 1, 0, -1), szm, pe.cnu[2], acc, sh, kStapleStore, 1);
    } else if (mu == 1) {
      add_staples<T, I, R>(in.U, S, 1, 0, s, syp, sxp, nb<I>(g, x, y, z, -1, 1, 0), sxm, pe.cnu[0], acc, sh, kStapleReuse, 0);
      add_staples<T, I, R>(in.U, S, 1, 2, s, syp, szp, nb<I>(g, x, y, z, 0, 1, -1), szm, pe.cnu[2], acc, sh, kStapleStore, 0);
    } else {
      add_staples<T, I, R>(in.U, S, 2, 0, s, szp, sxp, nb<I>(g, x, y, z, -1, 0, 1), sxm, pe.cnu[0], acc, sh, kStapleReuse, 1);
      add_staples<T, I, R>(in.U, S, 2, 1, s, szp, syp, nb<I>(g, x, y, z, 0, -1, 1), sym, pe.cnu[1], acc, sh, kStapleReuse, 0);
    }
    Mat<T> u, w;
    load_link_r<R>(in.U, S, mu, s, u);
    mul_nn_traceless(u, acc, w);
    Alg<T> force, e;
    retr_itg(w, pick3(pe.gc, mu), force);
    load_alg(in.E, S, mu * 8, s, e);
#pragma unroll
    for (int a = 0; a < 8; a++) e.a[a] += force.a[a];
    if (mu == 2) {
      Alg<T> jp, jm;
      load_alg(in.Jp, S, 0, s, jp);
      load_alg(in.Jm, S, 0, s, jm);
#pragma unroll
      for (int a = 0; a < 8; a++) e.a[a] += pe.jz * (jp.a[a] - jm.a[a]);
    }
    if (!dry) {
      store_alg(in.E, S, mu * 8, s, e);
      if (sg >= 0) store_alg(in.E, S, mu * 8, sg, e);
    }
    Mat<T> X, uh;
    if (!pl.save_uold && mu != 2) {  // one exp at twice the angle, as in links_site
      link_exp(T(2) * pick3(pl.cU, mu), e, X);
      link_apply(X, u, w);
      if (!dry) {
        store_link_r<R>(out.U, S, mu, s, w);
        if (sg >= 0) store_link_r<R>(out.U, S, mu, sg, w);
      }
      continue;
    }
    link_exp(pick3(pl.cU, mu), e, X);
    link_apply(X, u, uh);
    if (pl.save_uold && !dry) {
      store_link(in.UOld, S, mu, s, uh);
      if (sg >= 0) store_link(in.UOld, S, mu, sg, uh);
    }
    link_apply(X, uh, w);
    if (!dry) {
      store_link_r<R>(out.U, S, mu, s, w);
      if (sg >= 0) store_link_r<R>(out.U, S, mu, sg, w);
    }
    if (mu == 2) fused_currents<T, I, R>(in, out, S, plane, s, sg, hi, u, uh, pl.cj, dry);
  }
}

}  // namespace glasma

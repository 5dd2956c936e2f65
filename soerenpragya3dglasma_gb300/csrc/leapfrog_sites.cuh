// leapfrog_sites.cuh -- per-site bodies of the two leapfrog kernels, shared by the single-lattice
// launches (leapfrog.cu) and the batched multi-event launches (batch.cu).
#pragma once

#include "lattice.cuh"

namespace glasma {


constexpr int kThreads = 128;

// Pairs of adjoint actions by one matrix go through inv_adj_mul2 / adj_mul2 (one product pair instead
// of two); the double-float force kernel keeps its out-of-line single actions (ddf.cuh).
template <typename TC>
constexpr bool kPairRotations = !std::is_same<TC, ddf>::value;
// The pairs of the current transport (Jp and Jm rotated by one link) only in FP64, where the FP64 pipe
// bounds the kernels: at the FP32 link kernels' 64-register cap the paired form spills.
template <typename T>
constexpr bool kPairCurrents = std::is_same<T, double>::value;

// out_p = V (t.ep) V^d, out_m = V (t.em) V^d (adj = true) or the V^d . V forms, paired where kPairCurrents
template <typename T, bool adj>
__device__ __forceinline__ void rotate_currents(const Mat<T>& V, const Alg<T>& ep, const Alg<T>& em, Alg<T>& out_p,
                                                Alg<T>& out_m) {
  if constexpr (kPairCurrents<T>) {
    if constexpr (adj)
      adj_mul2(V, ep, em, out_p, out_m);
    else
      inv_adj_mul2(V, ep, em, out_p, out_m);
  } else {
    if constexpr (adj) {
      adj_mul(V, ep, out_p);
      adj_mul(V, em, out_m);
    } else {
      inv_adj_mul(V, ep, out_p);
      inv_adj_mul(V, em, out_m);
    }
  }
}

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
#ifndef GLASMA_FP32_PLAQ_MIN_BLOCKS
#define GLASMA_FP32_PLAQ_MIN_BLOCKS 4
#endif
#ifndef GLASMA_DDF_PLAQ_MIN_BLOCKS
#define GLASMA_DDF_PLAQ_MIN_BLOCKS 3
#endif
template <typename T>
struct Occupancy;
template <>
struct Occupancy<double> {
  static constexpr int kMinBlocks = GLASMA_FP64_MIN_BLOCKS;       // electric-field kernel
  static constexpr int kLinksMinBlocks = GLASMA_FP64_MIN_BLOCKS;  // link/J kernel
  static constexpr int kFusedMinBlocks = GLASMA_FP64_MIN_BLOCKS;  // one-pass step kernel
  static constexpr int kPlaqMinBlocks = GLASMA_FP64_MIN_BLOCKS;   // plaquette-method force kernel
};
template <>
struct Occupancy<float> {
  static constexpr int kMinBlocks = GLASMA_FP32_MIN_BLOCKS;
  static constexpr int kLinksMinBlocks = GLASMA_FP32_LINKS_MIN_BLOCKS;
  static constexpr int kFusedMinBlocks = GLASMA_FP32_FUSED_MIN_BLOCKS;
  static constexpr int kPlaqMinBlocks = GLASMA_FP32_PLAQ_MIN_BLOCKS;
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
    Alg<T> down, downm, jc, st;
    load_alg(f.Jp, S, 0, szm, jc);
    load_alg(f.Jm, S, 0, szm, st);
    rotate_currents<T, false>(uzm, jc, st, down, downm);
    load_alg(f.Jp, S, 0, s, jc);
    load_alg(f.JpStat, S, 0, s, st);
    axpy_diff(st, -p.cj, jc, down);
    if (!p.dry) {
      store_alg(f.JpStat, S, 0, s, st);
      if (sg >= 0) store_alg(f.JpStat, S, 0, sg, st);
    }
    down = downm;
    load_alg(f.Jm, S, 0, s, jc);
    load_alg(f.JmStat, S, 0, s, st);
    axpy_diff(st, p.cj, jc, down);
    if (!p.dry) {
      store_alg(f.JmStat, S, 0, s, st);
      if (sg >= 0) store_alg(f.JmStat, S, 0, sg, st);
    }
  }
}

// ---- the plaquette method --------------------------------------------------------------------------
// The force of UpdateElectricFields is a sum over plaquettes: the plaquette P = a b c^d d^d at y in the
// plane (p, q), p < q (a = U_p(y), b = U_q(y+p), c = U_p(y+q), d = U_q(y)), with al = ReTr(i t P),
// enters four links, as the upper or lower staple of each (c_mu = cE[mu], gc_mu = gamma c_mu):
//   link p at y     +gc_p c_q al                      (U_p(y) S_{+q} = P)
//   link q at y     -gc_q c_p al                      (U_q(y) S_{+p} = P^d)
//   link p at y+q   -gc_p c_q InvAdj(d, al)           (U_p(y+q) S_{-q} = d^d P^d d)
//   link q at y+p   +gc_q c_p InvAdj(a, al)           (U_q(y+p) S_{-p} = a^d P a)
// using ReTr(i t X^d) = -ReTr(i t X) and ReTr(i t^a V^d X V) = InvAdj(V, ReTr(i t X))_a, the SU(3)
// InverseAdjointMultiplication.  The same terms as the staple form (K1), regrouped: three plaquettes
// (three products each) and six adjoint rotations per site instead of twelve staples (two products
// each, three shared) and three final products: ~18 instead of ~24 matrix products per site.
// K1' (plaquette_site) runs one thread per plaquette owner y, slices -1 .. Nz-1 (the ghost slice owns
// the plaquettes whose lower-staple terms reach slice 0): it adds the first two terms and the current
// source to E at y and stores the last two, already weighted, in a contribution buffer at y.  K2'
// (links_site with kGather) adds the two contributions each link receives, from y = x-q and x-p, to
// E before it exponentiates it.  Contribution slots C[(slot*8 + a)*S + y]:
enum ContribSlot {
  kC01p = 0,  // plane (0,1), to link 1 at y+x
  kC01q = 1,  // plane (0,1), to link 0 at y+y
  kC02p = 2,  // plane (0,2), to link 2 at y+x
  kC02q = 3,  // plane (0,2), to link 0 at y+z
  kC12p = 4,  // plane (1,2), to link 2 at y+y
  kC12q = 5,  // plane (1,2), to link 1 at y+z
  kCSlots = 6
};

template <typename T>
__device__ __forceinline__ void scale_alg(T w, Alg<T>& v) {
#pragma unroll
  for (int k = 0; k < 8; k++) v.a[k] *= w;
}

// al = ReTr(i t^a a b c^d d^d)
template <typename T>
__device__ __forceinline__ void plaquette_alg(const Mat<T>& a, const Mat<T>& b, const Mat<T>& c, const Mat<T>& d,
                                              Alg<T>& al) {
  Mat<T> ab, dc, P;
  mul_nn(a, b, ab);
  mul_nn(d, c, dc);
  mul_nd_traceless(ab, dc, P);
  retr_itg(P, T(1), al);
}

// K1' per owner site: idx = owner site s (slice -1 starts at s = 0); covers (Nz+1) slices.  TC is the
// arithmetic type: T itself, or ddf for FP64 fields (double-float arithmetic on the FP32 pipe, the
// fields converted on load and store).
template <typename T, typename I, int R, typename TC = T>
__device__ __forceinline__ void plaquette_site(const Geometry& g, const FieldPtrs<T>& f, T* __restrict__ C,
                                               const EParams<T>& p, I idx) {
  const I S = (I)g.S, plane = (I)g.plane;
  const I s = idx;
  const int zz = (int)(idx / plane);
  const int z = zz - 1;
  const int r = (int)(idx - (I)zz * plane);
  const int y = r / g.nx, x = r - y * g.nx;
  const bool interior = z >= 0;
  const bool below_top = z < g.nz - 1;  // y+z is an interior site
  const I sxp = nb<I>(g, x, y, z, 1, 0, 0), syp = nb<I>(g, x, y, z, 0, 1, 0), szp = s + plane;
  // wp = gc_p c_q, wq = gc_q c_p (formed in the storage type, then converted)
  const TC w01p = to_compute<TC>(p.gc[0] * p.cnu[1]), w01q = to_compute<TC>(p.gc[1] * p.cnu[0]);
  const TC w02p = to_compute<TC>(p.gc[0] * p.cnu[2]), w02q = to_compute<TC>(p.gc[2] * p.cnu[0]);
  const TC w12p = to_compute<TC>(p.gc[1] * p.cnu[2]), w12q = to_compute<TC>(p.gc[2] * p.cnu[1]);
  Alg<TC> F0, F1, F2, al, out;
  Mat<TC> u0, u1, u2, b, c;
  load_link_c<R>(f.U, S, 0, s, u0);
  load_link_c<R>(f.U, S, 1, s, u1);
  load_link_c<R>(f.U, S, 2, s, u2);
  if constexpr (kPairRotations<TC>) {
    // the three plaquettes first, then the six rotations in pairs by the same link:
    // u1 (al01 -> link 0 at y+y, al12 -> link 2 at y+y), u0 (al01 -> link 1 at y+x, al02 -> link 2 at
    // y+x), u2 (al02 -> link 0 at y+z, al12 -> link 1 at y+z)
    Alg<TC> al01, al12, out2;
    if (interior) {
      // plane (0,1): a = U_0(y), b = U_1(y+x), c = U_0(y+y), d = U_1(y)
      load_link_c<R>(f.U, S, 1, sxp, b);
      load_link_c<R>(f.U, S, 0, syp, c);
      plaquette_alg(u0, b, c, u1, al01);
#pragma unroll
      for (int k = 0; k < 8; k++) {
        F0.a[k] = w01p * al01.a[k];
        F1.a[k] = -w01q * al01.a[k];
      }
    }
    // plane (0,2): a = U_0(y), b = U_2(y+x), c = U_0(y+z), d = U_2(y)
    load_link_c<R>(f.U, S, 2, sxp, b);
    load_link_c<R>(f.U, S, 0, szp, c);
    plaquette_alg(u0, b, c, u2, al);
    // plane (1,2): a = U_1(y), b = U_2(y+y), c = U_1(y+z), d = U_2(y)
    load_link_c<R>(f.U, S, 2, syp, b);
    load_link_c<R>(f.U, S, 1, szp, c);
    plaquette_alg(u1, b, c, u2, al12);
    if (below_top) {
      inv_adj_mul2(u2, al, al12, out, out2);
      scale_alg(-w02p, out);  // to link 0 at y+z
      scale_alg(-w12p, out2);  // to link 1 at y+z
      if (!p.dry) {
        store_alg_c(C, S, kC02q * 8, s, out);
        store_alg_c(C, S, kC12q * 8, s, out2);
      }
    }
    if (!interior) return;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      F0.a[k] += w02p * al.a[k];
      F2.a[k] = -w02q * al.a[k];
      F1.a[k] += w12p * al12.a[k];
      F2.a[k] -= w12q * al12.a[k];
    }
    inv_adj_mul2(u1, al01, al12, out, out2);
    scale_alg(-w01p, out);  // to link 0 at y+y
    scale_alg(w12q, out2);  // to link 2 at y+y
    if (!p.dry) {
      store_alg_c(C, S, kC01q * 8, s, out);
      store_alg_c(C, S, kC12p * 8, s, out2);
    }
    inv_adj_mul2(u0, al01, al, out, out2);
    scale_alg(w01q, out);  // to link 1 at y+x
    scale_alg(w02q, out2);  // to link 2 at y+x
    if (!p.dry) {
      store_alg_c(C, S, kC01p * 8, s, out);
      store_alg_c(C, S, kC02p * 8, s, out2);
    }
  } else {
    if (interior) {
      // plane (0,1): a = U_0(y), b = U_1(y+x), c = U_0(y+y), d = U_1(y)
      load_link_c<R>(f.U, S, 1, sxp, b);
      load_link_c<R>(f.U, S, 0, syp, c);
      plaquette_alg(u0, b, c, u1, al);
#pragma unroll
      for (int k = 0; k < 8; k++) {
        F0.a[k] = w01p * al.a[k];
        F1.a[k] = -w01q * al.a[k];
      }
      inv_adj_mul(u1, al, out);  // to link 0 at y+y
      scale_alg(-w01p, out);
      if (!p.dry) store_alg_c(C, S, kC01q * 8, s, out);
      inv_adj_mul(u0, al, out);  // to link 1 at y+x
      scale_alg(w01q, out);
      if (!p.dry) store_alg_c(C, S, kC01p * 8, s, out);
    }
    // plane (0,2): a = U_0(y), b = U_2(y+x), c = U_0(y+z), d = U_2(y)
    load_link_c<R>(f.U, S, 2, sxp, b);
    load_link_c<R>(f.U, S, 0, szp, c);
    plaquette_alg(u0, b, c, u2, al);
    if (below_top) {
      inv_adj_mul(u2, al, out);  // to link 0 at y+z
      scale_alg(-w02p, out);
      if (!p.dry) store_alg_c(C, S, kC02q * 8, s, out);
    }
    if (interior) {
#pragma unroll
      for (int k = 0; k < 8; k++) {
        F0.a[k] += w02p * al.a[k];
        F2.a[k] = -w02q * al.a[k];
      }
      inv_adj_mul(u0, al, out);  // to link 2 at y+x
      scale_alg(w02q, out);
      if (!p.dry) store_alg_c(C, S, kC02p * 8, s, out);
    }
    // plane (1,2): a = U_1(y), b = U_2(y+y), c = U_1(y+z), d = U_2(y)
    load_link_c<R>(f.U, S, 2, syp, b);
    load_link_c<R>(f.U, S, 1, szp, c);
    plaquette_alg(u1, b, c, u2, al);
    if (below_top) {
      inv_adj_mul(u2, al, out);  // to link 1 at y+z
      scale_alg(-w12p, out);
      if (!p.dry) store_alg_c(C, S, kC12q * 8, s, out);
    }
    if (!interior) return;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      F1.a[k] += w12p * al.a[k];
      F2.a[k] -= w12q * al.a[k];
    }
    inv_adj_mul(u1, al, out);  // to link 2 at y+y
    scale_alg(w12q, out);
    if (!p.dry) store_alg_c(C, S, kC12p * 8, s, out);
  }
  // E += the forces of the plaquettes owned here (+ the current source on E_z); K2' adds the rest
  Alg<TC> e;
  load_alg_c(f.E, S, 0, s, e);
#pragma unroll
  for (int k = 0; k < 8; k++) e.a[k] += F0.a[k];
  if (!p.dry) store_alg_c(f.E, S, 0, s, e);
  load_alg_c(f.E, S, 8, s, e);
#pragma unroll
  for (int k = 0; k < 8; k++) e.a[k] += F1.a[k];
  if (!p.dry) store_alg_c(f.E, S, 8, s, e);
  {
    Alg<TC> jp, jm;
    const TC jz = to_compute<TC>(p.jz);
    load_alg_c(f.E, S, 16, s, e);
    load_alg_c(f.Jp, S, 0, s, jp);
    load_alg_c(f.Jm, S, 0, s, jm);
#pragma unroll
    for (int k = 0; k < 8; k++) e.a[k] += F2.a[k] + jz * (jp.a[k] - jm.a[k]);
    if (!p.dry) store_alg_c(f.E, S, 16, s, e);
  }
  // UpdateJStat, as K1
  const bool lo = (z == 0), hi = (z == g.nz - 1);
  const I sg = lo ? s - plane : (hi ? s + plane : (I)-1);
  const I szm = s - plane;
  const TC cj = to_compute<TC>(p.cj);
  Mat<TC> uzm;
  load_link_c<R>(f.U, S, 2, szm, uzm);
  Alg<TC> down, downm, jc, st;
  load_alg_c(f.Jp, S, 0, szm, jc);
  if constexpr (kPairRotations<TC>) {
    load_alg_c(f.Jm, S, 0, szm, st);
    rotate_currents<TC, false>(uzm, jc, st, down, downm);
  } else {
    inv_adj_mul(uzm, jc, down);
  }
  load_alg_c(f.Jp, S, 0, s, jc);
  load_alg_c(f.JpStat, S, 0, s, st);
  axpy_diff(st, -cj, jc, down);
  if (!p.dry) {
    store_alg_c(f.JpStat, S, 0, s, st);
    if (sg >= 0) store_alg_c(f.JpStat, S, 0, sg, st);
  }
  if constexpr (kPairRotations<TC>) {
    down = downm;
  } else {
    load_alg_c(f.Jm, S, 0, szm, jc);
    inv_adj_mul(uzm, jc, down);
  }
  load_alg_c(f.Jm, S, 0, s, jc);
  load_alg_c(f.JmStat, S, 0, s, st);
  axpy_diff(st, cj, jc, down);
  if (!p.dry) {
    store_alg_c(f.JmStat, S, 0, s, st);
    if (sg >= 0) store_alg_c(f.JmStat, S, 0, sg, st);
  }
}

// Blocks per SM of the force kernel: by storage type, and for FP64 fields computed in double-float.
template <typename T, typename TC>
struct PlaqOccupancy {
  static constexpr int kMinBlocks = Occupancy<T>::kPlaqMinBlocks;
};
template <>
struct PlaqOccupancy<double, ddf> {
  static constexpr int kMinBlocks = GLASMA_DDF_PLAQ_MIN_BLOCKS;
};

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

// K2's per-site body: links to t+dt (two applications of one exp), UOld, J transport.  kGather (the
// plaquette method): first E_mu += the two contributions link mu receives from the plaquette owners
// x-nu (see plaquette_site), stored with its ghost copy.
template <typename T, typename I, int R = 3, bool kGather = false>
__device__ __forceinline__ void links_site(const Geometry& g, const FieldPtrs<T>& f, const LParams<T>& p, I idx,
                                           const T* __restrict__ C = nullptr) {
  const I S = (I)g.S, plane = (I)g.plane;
  const I s = idx + plane;
  const int z = (int)(idx / plane);
  const bool lo = (z == 0), hi = (z == g.nz - 1);
  const I sg = lo ? s - plane : (hi ? s + plane : (I)-1);
  I sxm = 0, sym = 0;
  if constexpr (kGather) {
    const int r = (int)(idx - (I)z * plane);
    const int y = r / g.nx, x = r - y * g.nx;
    sxm = nb<I>(g, x, y, z, -1, 0, 0);
    sym = nb<I>(g, x, y, z, 0, -1, 0);
  }
#pragma unroll 1
  for (int mu = 0; mu < 3; mu++) {
    Alg<T> e;
    load_alg(f.E, S, mu * 8, s, e);
    if constexpr (kGather) {
      // link 0: from (0,1) at x-y and (0,2) at x-z; link 1: (0,1) at x-x, (1,2) at x-z;
      // link 2: (0,2) at x-x, (1,2) at x-y
      const I s1 = mu == 0 ? sym : sxm;
      const I s2 = mu == 2 ? sym : s - plane;
      const int c1 = mu == 0 ? kC01q : (mu == 1 ? kC01p : kC02p);
      const int c2 = mu == 0 ? kC02q : (mu == 1 ? kC12q : kC12p);
      Alg<T> a1, a2;
      load_alg(C, S, c1 * 8, s1, a1);
      load_alg(C, S, c2 * 8, s2, a2);
#pragma unroll
      for (int k = 0; k < 8; k++) e.a[k] += a1.a[k] + a2.a[k];
      store_alg(f.E, S, mu * 8, s, e);
      if (sg >= 0) store_alg(f.E, S, mu * 8, sg, e);
    }
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
      Alg<T> up, um, st, j;
      const I szp = s + plane;
      load_alg(f.JpStat, S, 0, szp, st);
      if constexpr (kPairCurrents<T>) {
        load_alg(f.JmStat, S, 0, szp, j);
        rotate_currents<T, true>(uh, st, j, up, um);
      } else {
        adj_mul(uh, st, up);
      }
      load_alg(f.JpStat, S, 0, s, st);
      load_alg(f.Jp, S, 0, s, j);
      axpy_diff(j, -p.cj, up, st);
      store_alg(f.Jp, S, 0, s, j);
      if (sg >= 0) store_alg(f.Jp, S, 0, sg, j);
      if constexpr (kPairCurrents<T>) {
        up = um;
      } else {
        load_alg(f.JmStat, S, 0, szp, st);
        adj_mul(uh, st, up);
      }
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
  Alg<T> jc, down, downm, sp, sm;
  {
    Mat<T> w;
    load_link_r<R>(in.U, S, 2, szm, w);
    load_alg(in.Jp, S, 0, szm, jc);
    load_alg(in.Jm, S, 0, szm, sm);
    rotate_currents<T, false>(w, jc, sm, down, downm);
    load_alg(in.Jp, S, 0, s, jc);
    load_alg(in.JpStat, S, 0, s, sp);
    axpy_diff(sp, -cj, jc, down);
    load_alg(in.Jm, S, 0, s, jc);
    load_alg(in.JmStat, S, 0, s, sm);
    axpy_diff(sm, cj, jc, downm);
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
    load_alg(in.Jm, S, 0, s, um);
    rotate_currents<T, false>(uz, jc, um, down, downm);
    load_alg(in.Jp, S, 0, szp, jc);
    load_alg(in.JpStat, S, 0, szp, up);
    axpy_diff(up, -cj, jc, down);
    load_alg(in.Jm, S, 0, szp, jc);
    load_alg(in.JmStat, S, 0, szp, um);
    axpy_diff(um, cj, jc, downm);
  }
  Alg<T> t, tm, j;
  rotate_currents<T, true>(uhz, up, um, t, tm);
  load_alg(in.Jp, S, 0, s, j);
  axpy_diff(j, -cj, t, sp);
  if (!dry) {
    store_alg(out.Jp, S, 0, s, j);
    if (sg >= 0) store_alg(out.Jp, S, 0, sg, j);
  }
  t = tm;
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

// march.cuh -- the whole leapfrog step in one launch by the plaquette method, each block marching
// along z through a column of the lattice.
//
// The plaquette method (leapfrog_sites.cuh: plaquette_site, links_site<kGather>) computes each
// plaquette once, at its owner site y, and hands the two rotated force terms that belong to other
// links (U_p(y+q), U_q(y+p)) to the link kernel through a contribution buffer in HBM: 48 reals per
// site written and read back, and E, U and the currents read by both kernels.  Here one block owns a
// TX x (128/TX) tile of (x, y) sites and walks a chunk of z slices; per slice
//   A  every thread forms the three plaquettes it owns (planes (0,1), (0,2), (1,2)) and their direct
//      force terms; the rotated terms for its in-tile neighbours x+1 and y+1 go to shared memory, the
//      two for the links one slice up (U_0(y+z), U_1(y+z)) stay in the thread's registers for the
//      next slice;
//   B  the plaquettes owned by the column x0-1 and the row y0-1 just outside the tile, whose rotated
//      terms reach the tile's first column / row, are formed again by some of the threads (the
//      neighbouring tiles form them too: recomputation instead of an exchange between blocks);
//   C  each thread finishes E_mu at its site (old E + direct terms + the two rotated terms, in the
//      order the two-kernel method adds them), then runs the link/J tail of links_site: the two half
//      steps of the links, SaveOldLink, UpdateJ with the static currents of t+dt at z and z+1 (the
//      latter formed here, carried to the next slice).
// Every plaquette, rotation and sum is the two-kernel method's own expression with the same inputs
// in the same order, so the fields equal that method's up to rounding (the compiler contracts a few
// products into fused multiply-adds differently in the two kernels: 1e-15 in FP64).  The links, currents and static currents of t are
// read from one buffer set and those of t+dt written to a second (`out`), as in the one-pass step:
// neighbouring blocks still read the links of t while this one writes; E is updated in place (read
// and written only by its own site).  Per site and step each per-site array is read and written once
// (880 B in FP32), against ~1800 B for the two kernels.
#pragma once

#include "leapfrog_sites.cuh"

namespace glasma {

constexpr int kMarchThreads = 128;  // threads per block: a tile of TX x (128 / TX) sites

#ifndef GLASMA_FP32_MARCH_MIN_BLOCKS
#define GLASMA_FP32_MARCH_MIN_BLOCKS 3
#endif
template <typename T>
struct MarchOccupancy {
  static constexpr int kMinBlocks = sizeof(T) == 8 ? GLASMA_FP64_MIN_BLOCKS : GLASMA_FP32_MARCH_MIN_BLOCKS;
};

template <typename T>
struct MarchParams {
  EParams<T> pe;
  LParams<T> pl;
  int ntx, nty, lz;  // tiles along x and y, z slices per block
};

// in-plane rotated terms, stored at the consuming site of the tile: slot s, colour a, consumer c at
// csm[(s * 8 + a) * kMarchThreads + c]
enum MarchSlot {
  kM01p = 0,  // plane (0,1) owned at x-1: to link 1
  kM01q = 1,  // plane (0,1) owned at y-1: to link 0
  kM02p = 2,  // plane (0,2) owned at x-1: to link 2
  kM12p = 3,  // plane (1,2) owned at y-1: to link 2
};

template <typename T>
__device__ __forceinline__ void march_put(T* csm, int slot, int c, const Alg<T>& v) {
#pragma unroll
  for (int a = 0; a < 8; a++) csm[(slot * 8 + a) * kMarchThreads + c] = v.a[a];
}
template <typename T>
__device__ __forceinline__ void march_get(const T* csm, int slot, int c, Alg<T>& v) {
#pragma unroll
  for (int a = 0; a < 8; a++) v.a[a] = csm[(slot * 8 + a) * kMarchThreads + c];
}

// UpdateJStat at slice site sz from the state of t (as plaquette_site forms it): uzm = U_z one slice down.
template <typename T, typename I>
__device__ __forceinline__ void march_jstat(const FieldPtrs<T>& in, I S, I plane, I sz, const Mat<T>& uzm, T cj,
                                            Alg<T>& stp, Alg<T>& stm) {
  Alg<T> down, downm, jc;
  load_alg(in.Jp, S, 0, sz - plane, jc);
  load_alg(in.Jm, S, 0, sz - plane, stm);
  rotate_currents<T, false>(uzm, jc, stm, down, downm);
  load_alg(in.Jp, S, 0, sz, jc);
  load_alg(in.JpStat, S, 0, sz, stp);
  axpy_diff(stp, -cj, jc, down);
  load_alg(in.Jm, S, 0, sz, jc);
  load_alg(in.JmStat, S, 0, sz, stm);
  axpy_diff(stm, cj, jc, downm);
}

// The plaquette in plane (p, q) owned at site so: a = U_p(so), b = U_q(so+p), c = U_p(so+q), d = U_q(so).
template <typename T, typename I, int R>
__device__ __forceinline__ void march_plaquette(const cx<T>* __restrict__ U, I S, int p, int q, I so, I sp, I sq,
                                                Alg<T>& al) {
  Mat<T> a, b, c, d;
  load_link_r<R>(U, S, p, so, a);
  load_link_r<R>(U, S, q, sp, b);
  load_link_r<R>(U, S, p, sq, c);
  load_link_r<R>(U, S, q, so, d);
  plaquette_alg(a, b, c, d, al);
}

// Dynamic shared memory of the marching kernel, in reals: the in-plane terms by consumer (4 x 8), this
// thread's plaquettes (planes (0,1), (0,2), (1,2) and its halo plaquette: 4 x 8) and the z-terms by
// slice parity (2 x 16), per thread.
constexpr int kMarchSmemReals = (32 + 32 + 32) * kMarchThreads;

// The body is written for a small instruction footprint: one code path for every plaquette (own and
// halo, in a loop), one for every rotation (a loop over pairs; the halo's single rotation is a pair
// with a zero second vector), one for the next slice's static currents (the warm-up slice below the
// chunk runs the same loop iteration), one exponential and one link application per link.  The first
// version, with every case written out, stalled on instruction fetch (ncu: "no instruction" the
// largest stall) at 1.7x the two-kernel method's time.
template <typename T, typename I, int R, int kMarchTX>
__global__ void __launch_bounds__(kMarchThreads, MarchOccupancy<T>::kMinBlocks)
    march_step_kernel(const __grid_constant__ Geometry g, const __grid_constant__ FieldPtrs<T> in,
                      const __grid_constant__ FieldPtrs<T> out, const __grid_constant__ MarchParams<T> mp) {
  extern __shared__ __align__(16) unsigned char march_smem[];
  T* csm = reinterpret_cast<T*>(march_smem);  // [slot][a][consumer]
  T* asm_ = csm + 32 * kMarchThreads;          // [plaquette slot][a][thread]
  T* zsm = asm_ + 32 * kMarchThreads;          // [parity][16][thread]
  const I S = (I)g.S, plane = (I)g.plane;
  constexpr int kMarchTY = kMarchThreads / kMarchTX;
  static_assert(kMarchTY * kMarchTX == kMarchThreads && 2 * (kMarchTX + kMarchTY) <= kMarchThreads,
                "one halo plaquette per thread: the tile must leave enough threads");
  const int tid = threadIdx.x;
  const int lx = tid % kMarchTX, ly = tid / kMarchTX;
  int b = blockIdx.x;
  const int tx = b % mp.ntx;
  b /= mp.ntx;
  const int ty = b % mp.nty;
  const int chunk = b / mp.nty;
  const int x0 = tx * kMarchTX, y0 = ty * kMarchTY;
  const int x = x0 + lx, y = y0 + ly;
  const bool own = x < g.nx && y < g.ny;
  const int za = chunk * mp.lz;
  const int zb = za + mp.lz < g.nz ? za + mp.lz : g.nz;
  const EParams<T>& pe = mp.pe;
  const LParams<T>& pl = mp.pl;
  const T w01p = pe.gc[0] * pe.cnu[1], w01q = pe.gc[1] * pe.cnu[0];
  const T w02p = pe.gc[0] * pe.cnu[2], w02q = pe.gc[2] * pe.cnu[0];
  const T w12p = pe.gc[1] * pe.cnu[2], w12q = pe.gc[2] * pe.cnu[1];
  auto put = [&](T* base, int slot, int idx, const Alg<T>& v) {
#pragma unroll
    for (int a = 0; a < 8; a++) base[(slot * 8 + a) * kMarchThreads + idx] = v.a[a];
  };
  auto get = [&](const T* base, int slot, int idx, Alg<T>& v) {
#pragma unroll
    for (int a = 0; a < 8; a++) v.a[a] = base[(slot * 8 + a) * kMarchThreads + idx];
  };
  // one halo plaquette of this thread (the owners just outside the tile: the row y0-1 and the column
  // x0-1), grouped so that a warp mostly runs one kind:
  //   [0, TX)            row owner (x0+t, y0-1), plane (0,1) -> link 0 at (x0+t, y0), rotated by d = U_1
  //   [TX, TX+TY)        column owner (x0-1, y0+t), plane (0,1) -> link 1 at (x0, y0+t), by a = U_0
  //   [TX+TY, 2TX+TY)    row owner, plane (1,2) -> link 2 at (x0+t, y0), by a = U_1
  //   [2TX+TY, 2TX+2TY)  column owner, plane (0,2) -> link 2 at (x0, y0+t), by a = U_0
  int hplane = -1, hx = 0, hy = 0, hc = 0, hrot = 0, hslot = 0;
  T hw = T(0);
  {
    int t = tid, kind = -1;
    if (t < kMarchTX) {
      kind = 0;
    } else if ((t -= kMarchTX) < kMarchTY) {
      kind = 1;
    } else if ((t -= kMarchTY) < kMarchTX) {
      kind = 2;
    } else if ((t -= kMarchTX) < kMarchTY) {
      kind = 3;
    }
    const bool row = kind == 0 || kind == 2;
    if (kind >= 0 && (row ? x0 + t < g.nx : y0 + t < g.ny)) {
      hx = row ? x0 + t : (x0 == 0 ? g.nx - 1 : x0 - 1);
      hy = row ? (y0 == 0 ? g.ny - 1 : y0 - 1) : y0 + t;
      hc = row ? t : t * kMarchTX;
      hplane = kind <= 1 ? 0 : (kind == 2 ? 2 : 1);
      hrot = kind == 0 ? 1 : (kind == 2 ? 1 : 0);  // the direction of the rotating link at the owner
      hslot = kind == 0 ? kM01q : (kind == 1 ? kM01p : (kind == 2 ? kM12p : kM02p));
      hw = kind == 0 ? -w01p : (kind == 1 ? w01q : (kind == 2 ? w12q : w02q));
    }
  }
  const bool put_x = lx + 1 < kMarchTX && x + 1 < g.nx;  // the x-neighbour is a site of this tile
  const bool put_y = ly + 1 < kMarchTY && y + 1 < g.ny;  // the y-neighbour is a site of this tile

  Alg<T> stp = {}, stm = {};  // the static currents of t+dt at this slice
#pragma unroll 1
  for (int z = za - 1; z < zb; z++) {
    // z = za - 1: the slice below the chunk (the ghost slice for the first chunk): only its z-terms for
    // the chunk's first slice and the static currents of t+dt there
    const bool warm = z < za;
    const bool below_top = z < g.nz - 1;
    const I s = own ? (I)site_index(g, x, y, z) : (I)0;
    // ---- A: the plaquettes: this site's (planes (0,1), (0,2), (1,2); (0,2), (1,2) below the chunk)
    // and this thread's halo plaquette, into the thread's slots
    {
      const int p0 = warm ? 1 : 0;
      const int nown = own ? 3 - p0 : 0;
      const int ntask = nown + ((!warm && hplane >= 0) ? 1 : 0);
#pragma unroll 1
      for (int t = 0; t < ntask; t++) {
        const bool mine = t < nown;
        const int xx = mine ? x : hx, yy = mine ? y : hy, pln = mine ? p0 + t : hplane;
        const int p = pln == 2 ? 1 : 0, q = pln == 0 ? 1 : 2;
        const I so = (I)site_index(g, xx, yy, z);
        const I sp = nb<I>(g, xx, yy, z, p == 0 ? 1 : 0, p == 1 ? 1 : 0, 0);
        const I sq = q == 2 ? so + plane : nb<I>(g, xx, yy, z, 0, 1, 0);
        Alg<T> al;
        march_plaquette<T, I, R>(in.U, S, p, q, so, sp, sq, al);
        put(asm_, mine ? pln : 3, tid, al);
      }
    }
    // ---- the rotated terms, in pairs by one link: U_2 (planes (0,2), (1,2): to links 0 and 1 one slice
    // up), U_1 ((0,1), (1,2): to links 0 and 2 at y+y), U_0 ((0,1), (0,2): to links 1 and 2 at y+x), and
    // the halo plaquette's single term
    {
      const unsigned mask = (own && below_top ? 1u : 0u) | (own && !warm && put_y ? 2u : 0u) |
                            (own && !warm && put_x ? 4u : 0u) | (!warm && hplane >= 0 ? 8u : 0u);
#pragma unroll 1
      for (int r = 0; r < 4; r++) {
        if (!(mask & (1u << r))) continue;
        int dir, s1, s2 = -1;
        I vs = s;
        T c1, c2 = T(0);
        if (r == 0) {
          dir = 2, s1 = 1, s2 = 2, c1 = -w02p, c2 = -w12p;
        } else if (r == 1) {
          dir = 1, s1 = 0, s2 = 2, c1 = -w01p, c2 = w12q;
        } else if (r == 2) {
          dir = 0, s1 = 0, s2 = 1, c1 = w01q, c2 = w02q;
        } else {
          dir = hrot, s1 = 3, c1 = hw;
          vs = (I)site_index(g, hx, hy, z);
        }
        Mat<T> V;
        Alg<T> e1, e2, o1, o2;
        load_link_r<R>(in.U, S, dir, vs, V);
        get(asm_, s1, tid, e1);
        if (s2 >= 0) {
          get(asm_, s2, tid, e2);
        } else {
#pragma unroll
          for (int a = 0; a < 8; a++) e2.a[a] = T(0);
        }
        inv_adj_mul2(V, e1, e2, o1, o2);
        scale_alg(c1, o1);
        scale_alg(c2, o2);
        if (r == 0) {
#pragma unroll
          for (int a = 0; a < 8; a++) {
            zsm[((z & 1) * 16 + a) * kMarchThreads + tid] = o1.a[a];
            zsm[((z & 1) * 16 + 8 + a) * kMarchThreads + tid] = o2.a[a];
          }
        } else if (r == 1) {
          put(csm, kM01q, tid + kMarchTX, o1);
          put(csm, kM12p, tid + kMarchTX, o2);
        } else if (r == 2) {
          put(csm, kM01p, tid + 1, o1);
          put(csm, kM02p, tid + 1, o2);
        } else {
          put(csm, hslot, hc, o1);
        }
      }
    }
    // the static currents of t+dt one slice up (its ghost copy at the top slice), from U_z(z) of t
    Alg<T> sp1, sm1;
    if (own) {
      if (below_top) {
        Mat<T> uz;
        load_link_r<R>(in.U, S, 2, s, uz);
        march_jstat(in, S, plane, s + plane, uz, pe.cj, sp1, sm1);
      } else {
        sp1 = stp;
        sm1 = stm;
      }
    }
    if (warm) {
      stp = sp1;
      stm = sm1;
      continue;
    }
    __syncthreads();
    // ---- C: E, the links and the currents of this site
    if (own) {
      const bool lo = (z == 0), hi = (z == g.nz - 1);
      const I sg = lo ? s - plane : (hi ? s + plane : (I)-1);
      store_alg(out.JpStat, S, 0, s, stp);
      store_alg(out.JmStat, S, 0, s, stm);
      if (sg >= 0) {
        store_alg(out.JpStat, S, 0, sg, stp);
        store_alg(out.JmStat, S, 0, sg, stm);
      }
#pragma unroll 1
      for (int mu = 0; mu < 3; mu++) {
        // E_mu + the direct terms (as plaquette_site sums them) + the two rotated terms (as links_site
        // adds them)
        Alg<T> e, a1, a2, alA, alB;
        load_alg(in.E, S, mu * 8, s, e);
        const int sa = mu == 2 ? 1 : 0, sb = mu == 0 ? 1 : 2;  // the two plaquettes that contain link mu here
        const T wa = mu == 0 ? w01p : (mu == 1 ? -w01q : -w02q);
        const T wb = mu == 0 ? w02p : (mu == 1 ? w12p : -w12q);
        get(asm_, sa, tid, alA);
        get(asm_, sb, tid, alB);
        if (mu == 2) {
          Alg<T> jp, jm;
          load_alg(in.Jp, S, 0, s, jp);
          load_alg(in.Jm, S, 0, s, jm);
#pragma unroll
          for (int k = 0; k < 8; k++) {
            T f = wa * alA.a[k];
            f -= w12q * alB.a[k];
            e.a[k] += f + pe.jz * (jp.a[k] - jm.a[k]);
          }
        } else {
#pragma unroll
          for (int k = 0; k < 8; k++) {
            T f = wa * alA.a[k];
            f += wb * alB.a[k];
            e.a[k] += f;
          }
        }
        if (mu == 2) {
          get(csm, kM02p, tid, a1);
          get(csm, kM12p, tid, a2);
        } else {
          get(csm, mu == 0 ? kM01q : kM01p, tid, a1);
#pragma unroll
          for (int a = 0; a < 8; a++) a2.a[a] = zsm[(((z - 1) & 1) * 16 + (mu == 0 ? 0 : 8) + a) * kMarchThreads + tid];
        }
#pragma unroll
        for (int k = 0; k < 8; k++) e.a[k] += a1.a[k] + a2.a[k];
        store_alg(in.E, S, mu * 8, s, e);
        if (sg >= 0) store_alg(in.E, S, mu * 8, sg, e);
        // the links: one exponential at twice the angle where U(t+dt/2) has no use, else two half steps
        // with SaveOldLink and UpdateJ between them
        const bool doubled = pl.do_second && !pl.save_uold && !(mu == 2 && pl.do_j);
        Mat<T> X, u, w;
        load_link_r<R>(in.U, S, mu, s, u);
        link_exp(doubled ? T(2) * pick3(pl.cU, mu) : pick3(pl.cU, mu), e, X);
        const int napply = (doubled || !pl.do_second) ? 1 : 2;
#pragma unroll 1
        for (int ap = 0; ap < napply; ap++) {
          link_apply(X, u, w);
          u = w;
          if (ap == 0 && !doubled) {
            if (pl.save_uold) {
              store_link(in.UOld, S, mu, s, u);
              if (sg >= 0) store_link(in.UOld, S, mu, sg, u);
            }
            if (mu == 2 && pl.do_j) {
              Alg<T> up, um, j;
              rotate_currents<T, true>(u, sp1, sm1, up, um);
              load_alg(in.Jp, S, 0, s, j);
              axpy_diff(j, -pl.cj, up, stp);
              store_alg(out.Jp, S, 0, s, j);
              if (sg >= 0) store_alg(out.Jp, S, 0, sg, j);
              load_alg(in.Jm, S, 0, s, j);
              axpy_diff(j, pl.cj, um, stm);
              store_alg(out.Jm, S, 0, s, j);
              if (sg >= 0) store_alg(out.Jm, S, 0, sg, j);
            }
          }
        }
        store_link_r<R>(out.U, S, mu, s, u);
        if (sg >= 0) store_link_r<R>(out.U, S, mu, sg, u);
      }
      stp = sp1;
      stm = sm1;
    }
    __syncthreads();
  }
}

}  // namespace glasma

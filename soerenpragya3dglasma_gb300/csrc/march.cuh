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

template <typename T, typename I, int R, int kMarchTX>
__global__ void __launch_bounds__(kMarchThreads, MarchOccupancy<T>::kMinBlocks)
    march_step_kernel(const __grid_constant__ Geometry g, const __grid_constant__ FieldPtrs<T> in,
                      const __grid_constant__ FieldPtrs<T> out, const __grid_constant__ MarchParams<T> mp) {
  __shared__ T csm[4 * 8 * kMarchThreads];
  // FP32: the z-terms carried to the next slice wait in shared memory (each thread its own entries,
  // two buffers by slice parity) instead of 16 registers; FP64 keeps them in registers
  constexpr bool kZsm = sizeof(T) == 4;
  __shared__ T zsm[kZsm ? 2 * 16 * kMarchThreads : 1];
  auto zput = [&](int z, const Alg<T>& v0, const Alg<T>& v1) {
#pragma unroll
    for (int a = 0; a < 8; a++) {
      zsm[((z & 1) * 16 + a) * kMarchThreads + threadIdx.x] = v0.a[a];
      zsm[((z & 1) * 16 + 8 + a) * kMarchThreads + threadIdx.x] = v1.a[a];
    }
  };
  auto zget = [&](int z, Alg<T>& v0, Alg<T>& v1) {
#pragma unroll
    for (int a = 0; a < 8; a++) {
      v0.a[a] = zsm[((z & 1) * 16 + a) * kMarchThreads + threadIdx.x];
      v1.a[a] = zsm[((z & 1) * 16 + 8 + a) * kMarchThreads + threadIdx.x];
    }
  };
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
  // one halo plaquette of this thread in phase B (the owners just outside the tile: the row y0-1 and
  // the column x0-1), grouped so that a warp mostly runs one kind:
  //   [0, TX)            row owner (x0+t, y0-1), plane (0,1) -> link 0 at (x0+t, y0)
  //   [TX, TX+TY)        column owner (x0-1, y0+t), plane (0,1) -> link 1 at (x0, y0+t)
  //   [TX+TY, 2TX+TY)    row owner, plane (1,2) -> link 2 at (x0+t, y0)
  //   [2TX+TY, 2TX+2TY)  column owner, plane (0,2) -> link 2 at (x0, y0+t)
  int htask = -1, hx = 0, hy = 0, hc = 0;
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
    if (kind == 0 || kind == 2) {
      if (x0 + t < g.nx) {
        htask = kind;
        hx = x0 + t;
        hy = y0 == 0 ? g.ny - 1 : y0 - 1;
        hc = t;
      }
    } else if (kind == 1 || kind == 3) {
      if (y0 + t < g.ny) {
        htask = kind;
        hx = x0 == 0 ? g.nx - 1 : x0 - 1;
        hy = y0 + t;
        hc = t * kMarchTX;
      }
    }
  }
  const bool put_x = lx + 1 < kMarchTX && x + 1 < g.nx;  // the x-neighbour is a site of this tile
  const bool put_y = ly + 1 < kMarchTY && y + 1 < g.ny;  // the y-neighbour is a site of this tile

  // warm-up: the z-terms of the plaquettes owned one slice below the chunk (the ghost slice -1 for the
  // first chunk), and the static currents of t+dt at the chunk's first slice
  Alg<T> zc0, zc1, stp, stm;
  if (own) {
    const int zw = za - 1;
    const I s = (I)site_index(g, x, y, zw);
    const I sxp = nb<I>(g, x, y, zw, 1, 0, 0), syp = nb<I>(g, x, y, zw, 0, 1, 0), szp = s + plane;
    Mat<T> u0, u1, u2, bb, cc;
    Alg<T> al;
    load_link_r<R>(in.U, S, 0, s, u0);
    load_link_r<R>(in.U, S, 1, s, u1);
    load_link_r<R>(in.U, S, 2, s, u2);
    Alg<T> al12;
    load_link_r<R>(in.U, S, 2, sxp, bb);
    load_link_r<R>(in.U, S, 0, szp, cc);
    plaquette_alg(u0, bb, cc, u2, al);
    load_link_r<R>(in.U, S, 2, syp, bb);
    load_link_r<R>(in.U, S, 1, szp, cc);
    plaquette_alg(u1, bb, cc, u2, al12);
    inv_adj_mul2(u2, al, al12, zc0, zc1);
    scale_alg(-w02p, zc0);
    scale_alg(-w12p, zc1);
    march_jstat(in, S, plane, s + plane, u2, pe.cj, stp, stm);
    if constexpr (kZsm) zput(zw, zc0, zc1);
  }

#pragma unroll 1
  for (int z = za; z < zb; z++) {
    const bool below_top = z < g.nz - 1;
    Alg<T> F0, F1, F2, zn0 = {}, zn1 = {};
    I s = 0;
    // ---- A: the plaquettes owned at this site
    if (own) {
      s = (I)site_index(g, x, y, z);
      const I sxp = nb<I>(g, x, y, z, 1, 0, 0), syp = nb<I>(g, x, y, z, 0, 1, 0), szp = s + plane;
      Mat<T> u0, u1, u2, bb, cc;
      Alg<T> al, o;
      load_link_r<R>(in.U, S, 0, s, u0);
      load_link_r<R>(in.U, S, 1, s, u1);
      load_link_r<R>(in.U, S, 2, s, u2);
      // the three plaquettes, then the rotations in pairs by the same link (as plaquette_site)
      Alg<T> al01, al12, o2;
      // plane (0,1): a = U_0(y), b = U_1(y+x), c = U_0(y+y), d = U_1(y)
      load_link_r<R>(in.U, S, 1, sxp, bb);
      load_link_r<R>(in.U, S, 0, syp, cc);
      plaquette_alg(u0, bb, cc, u1, al01);
#pragma unroll
      for (int k = 0; k < 8; k++) {
        F0.a[k] = w01p * al01.a[k];
        F1.a[k] = -w01q * al01.a[k];
      }
      // plane (0,2): a = U_0(y), b = U_2(y+x), c = U_0(y+z), d = U_2(y)
      load_link_r<R>(in.U, S, 2, sxp, bb);
      load_link_r<R>(in.U, S, 0, szp, cc);
      plaquette_alg(u0, bb, cc, u2, al);
      // plane (1,2): a = U_1(y), b = U_2(y+y), c = U_1(y+z), d = U_2(y)
      load_link_r<R>(in.U, S, 2, syp, bb);
      load_link_r<R>(in.U, S, 1, szp, cc);
      plaquette_alg(u1, bb, cc, u2, al12);
#pragma unroll
      for (int k = 0; k < 8; k++) {
        F0.a[k] += w02p * al.a[k];
        F2.a[k] = -w02q * al.a[k];
        F1.a[k] += w12p * al12.a[k];
        F2.a[k] -= w12q * al12.a[k];
      }
      if (below_top) {  // to links 0 and 1 at y+z: the next slice of this thread
        inv_adj_mul2(u2, al, al12, zn0, zn1);
        scale_alg(-w02p, zn0);
        scale_alg(-w12p, zn1);
      }
      if (put_y) {  // to links 0 and 2 at y+y
        inv_adj_mul2(u1, al01, al12, o, o2);
        scale_alg(-w01p, o);
        scale_alg(w12q, o2);
        march_put(csm, kM01q, tid + kMarchTX, o);
        march_put(csm, kM12p, tid + kMarchTX, o2);
      }
      if (put_x) {  // to links 1 and 2 at y+x
        inv_adj_mul2(u0, al01, al, o, o2);
        scale_alg(w01q, o);
        scale_alg(w02q, o2);
        march_put(csm, kM01p, tid + 1, o);
        march_put(csm, kM02p, tid + 1, o2);
      }
      if constexpr (kZsm) {
        if (below_top) zput(z, zn0, zn1);
      }
    }
    // ---- B: the plaquettes owned just outside the tile whose rotated terms reach its first column / row
    if (htask >= 0) {
      const I hs = (I)site_index(g, hx, hy, z);
      const I hxp = nb<I>(g, hx, hy, z, 1, 0, 0), hyp = nb<I>(g, hx, hy, z, 0, 1, 0), hzp = hs + plane;
      Mat<T> a, bb, cc, d;
      Alg<T> al, o;
      if (htask <= 1) {  // plane (0,1): a = U_0(y), b = U_1(y+x), c = U_0(y+y), d = U_1(y)
        load_link_r<R>(in.U, S, 0, hs, a);
        load_link_r<R>(in.U, S, 1, hxp, bb);
        load_link_r<R>(in.U, S, 0, hyp, cc);
        load_link_r<R>(in.U, S, 1, hs, d);
        plaquette_alg(a, bb, cc, d, al);
        if (htask == 0) {  // to link 0 at y+y
          inv_adj_mul(d, al, o);
          scale_alg(-w01p, o);
          march_put(csm, kM01q, hc, o);
        } else {  // to link 1 at y+x
          inv_adj_mul(a, al, o);
          scale_alg(w01q, o);
          march_put(csm, kM01p, hc, o);
        }
      } else if (htask == 2) {  // plane (1,2): a = U_1(y), b = U_2(y+y), c = U_1(y+z), d = U_2(y)
        load_link_r<R>(in.U, S, 1, hs, a);
        load_link_r<R>(in.U, S, 2, hyp, bb);
        load_link_r<R>(in.U, S, 1, hzp, cc);
        load_link_r<R>(in.U, S, 2, hs, d);
        plaquette_alg(a, bb, cc, d, al);
        inv_adj_mul(a, al, o);  // to link 2 at y+y
        scale_alg(w12q, o);
        march_put(csm, kM12p, hc, o);
      } else {  // plane (0,2): a = U_0(y), b = U_2(y+x), c = U_0(y+z), d = U_2(y)
        load_link_r<R>(in.U, S, 0, hs, a);
        load_link_r<R>(in.U, S, 2, hxp, bb);
        load_link_r<R>(in.U, S, 0, hzp, cc);
        load_link_r<R>(in.U, S, 2, hs, d);
        plaquette_alg(a, bb, cc, d, al);
        inv_adj_mul(a, al, o);  // to link 2 at y+x
        scale_alg(w02q, o);
        march_put(csm, kM02p, hc, o);
      }
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
        Alg<T> e, a1, a2;
        load_alg(in.E, S, mu * 8, s, e);
        if (mu == 0) {
#pragma unroll
          for (int k = 0; k < 8; k++) e.a[k] += F0.a[k];
          march_get(csm, kM01q, tid, a1);
          if constexpr (kZsm) {
            Alg<T> unused;
            zget(z - 1, a2, unused);
          } else {
            a2 = zc0;
          }
        } else if (mu == 1) {
#pragma unroll
          for (int k = 0; k < 8; k++) e.a[k] += F1.a[k];
          march_get(csm, kM01p, tid, a1);
          if constexpr (kZsm) {
            Alg<T> unused;
            zget(z - 1, unused, a2);
          } else {
            a2 = zc1;
          }
        } else {
          Alg<T> jp, jm;
          load_alg(in.Jp, S, 0, s, jp);
          load_alg(in.Jm, S, 0, s, jm);
#pragma unroll
          for (int k = 0; k < 8; k++) e.a[k] += F2.a[k] + pe.jz * (jp.a[k] - jm.a[k]);
          march_get(csm, kM02p, tid, a1);
          march_get(csm, kM12p, tid, a2);
        }
#pragma unroll
        for (int k = 0; k < 8; k++) e.a[k] += a1.a[k] + a2.a[k];
        store_alg(in.E, S, mu * 8, s, e);
        if (sg >= 0) store_alg(in.E, S, mu * 8, sg, e);
        Mat<T> X, u, uh;
        load_link_r<R>(in.U, S, mu, s, u);
        if (mu == 2) {
          // static currents of t+dt one slice up, from U_z(z) of t (its ghost copy at the top slice);
          // carried to the next slice as its own
          Alg<T> sp1, sm1;
          if (hi) {
            sp1 = stp;
            sm1 = stm;
          } else {
            march_jstat(in, S, plane, s + plane, u, pe.cj, sp1, sm1);
          }
          if (pl.do_j) {
            // UpdateJ needs U_z at t+dt/2 (formed below); keep both static currents until then
            link_exp(pick3(pl.cU, mu), e, X);
            link_apply(X, u, uh);
            if (pl.save_uold) {
              store_link(in.UOld, S, mu, s, uh);
              if (sg >= 0) store_link(in.UOld, S, mu, sg, uh);
            }
            Alg<T> up, um, j;
            rotate_currents<T, true>(uh, sp1, sm1, up, um);
            load_alg(in.Jp, S, 0, s, j);
            axpy_diff(j, -pl.cj, up, stp);
            store_alg(out.Jp, S, 0, s, j);
            if (sg >= 0) store_alg(out.Jp, S, 0, sg, j);
            up = um;
            load_alg(in.Jm, S, 0, s, j);
            axpy_diff(j, pl.cj, up, stm);
            store_alg(out.Jm, S, 0, s, j);
            if (sg >= 0) store_alg(out.Jm, S, 0, sg, j);
            stp = sp1;
            stm = sm1;
            if (pl.do_second) {
              link_apply(X, uh, u);
            } else {
              u = uh;
            }
            store_link_r<R>(out.U, S, mu, s, u);
            if (sg >= 0) store_link_r<R>(out.U, S, mu, sg, u);
            continue;
          }
          stp = sp1;
          stm = sm1;
        }
        if (pl.do_second && !pl.save_uold && !(mu == 2 && pl.do_j)) {
          link_exp(T(2) * pick3(pl.cU, mu), e, X);
          link_apply(X, u, uh);
          store_link_r<R>(out.U, S, mu, s, uh);
          if (sg >= 0) store_link_r<R>(out.U, S, mu, sg, uh);
          continue;
        }
        link_exp(pick3(pl.cU, mu), e, X);
        link_apply(X, u, uh);
        if (pl.save_uold) {
          store_link(in.UOld, S, mu, s, uh);
          if (sg >= 0) store_link(in.UOld, S, mu, sg, uh);
        }
        if (pl.do_second) {
          link_apply(X, uh, u);
        } else {
          u = uh;
        }
        store_link_r<R>(out.U, S, mu, s, u);
        if (sg >= 0) store_link_r<R>(out.U, S, mu, sg, u);
      }
    }
    if constexpr (!kZsm) {
      zc0 = zn0;
      zc1 = zn1;
    }
    __syncthreads();
  }
}

}  // namespace glasma

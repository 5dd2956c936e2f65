// efield_tile.cuh -- K1 (electric field + JStat) with a block's links staged in shared memory.
//
// A block of kThreads threads owns a TX x TY tile of one z slice.  Before any arithmetic it copies
// into shared memory exactly the links its staples read (cp.async, every copy in flight at once):
//
//   link   plane z                  plane z-1              plane z+1
//   U_x    x in [-1,TX-1], y [-1,TY]  the tile             x in [-1,TX-1], y in the tile
//   U_y    x in [-1,TX], y [-1,TY-1]  the tile             x in the tile, y in [-1,TY-1]
//   U_z    x in [-1,TX], y [-1,TY]    x [0,TX], y [0,TY]   -
//
// (coordinates relative to the tile origin; 1285 links, 92.5 KB in FP32 for 32 x 4).  The staple
// arithmetic then reads its links from shared memory in the same order, with the same operations, as
// efield_site reads them from global memory, so the result is bit-identical to the untiled kernel
// (and to the batched launch, which keeps the untiled body).  What changes is the memory access: every
// link is fetched once per block as part of a coalesced burst instead of ~30 dependent L1/L2 loads per
// site, which is what left the untiled FP32 kernel latency-bound at a third of HBM bandwidth.
#pragma once

#include "leapfrog_sites.cuh"

namespace glasma {

struct LinkBox {
  int xlo, xhi, ylo, yhi;
};

// The box of link direction mu in plane p (0: z, 1: z-1, 2: z+1), relative to the tile origin.
template <int TX, int TY>
__host__ __device__ constexpr LinkBox link_box(int mu, int p) {
  return mu == 0 ? (p == 0 ? LinkBox{-1, TX - 1, -1, TY} : p == 1 ? LinkBox{0, TX - 1, 0, TY - 1}
                                                                   : LinkBox{-1, TX - 1, 0, TY - 1})
       : mu == 1 ? (p == 0 ? LinkBox{-1, TX, -1, TY - 1} : p == 1 ? LinkBox{0, TX - 1, 0, TY - 1}
                                                                   : LinkBox{0, TX - 1, -1, TY - 1})
                 : (p == 0 ? LinkBox{-1, TX, -1, TY} : p == 1 ? LinkBox{0, TX, 0, TY} : LinkBox{0, -1, 0, -1});
}
__host__ __device__ constexpr int box_width(LinkBox b) { return b.xhi - b.xlo + 1; }
__host__ __device__ constexpr int box_sites(LinkBox b) {
  return b.xhi < b.xlo ? 0 : (b.xhi - b.xlo + 1) * (b.yhi - b.ylo + 1);
}
// sites of all three planes of direction mu, and the first site of plane p among them
template <int TX, int TY>
__host__ __device__ constexpr int dir_sites(int mu) {
  return box_sites(link_box<TX, TY>(mu, 0)) + box_sites(link_box<TX, TY>(mu, 1)) + box_sites(link_box<TX, TY>(mu, 2));
}
template <int TX, int TY>
__host__ __device__ constexpr int plane_first(int mu, int p) {
  return p == 0 ? 0 : (p == 1 ? box_sites(link_box<TX, TY>(mu, 0)) : box_sites(link_box<TX, TY>(mu, 0)) +
                                                                        box_sites(link_box<TX, TY>(mu, 1)));
}
// shared-memory element offset of direction mu (element k of local site i at offset + k * dir_sites + i)
template <int TX, int TY>
__host__ __device__ constexpr int dir_offset(int mu) {
  return mu == 0 ? 0 : (mu == 1 ? 9 * dir_sites<TX, TY>(0) : 9 * (dir_sites<TX, TY>(0) + dir_sites<TX, TY>(1)));
}
template <int TX, int TY>
__host__ __device__ constexpr int tile_link_elems() {
  return 9 * (dir_sites<TX, TY>(0) + dir_sites<TX, TY>(1) + dir_sites<TX, TY>(2));
}

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// The links of one thread's site, read from the block's staged tile.
template <typename T, int TX, int TY>
struct TileLinks {
  const cx<T>* sm;
  int tx, ty;
  // link mu at offset (dx, dy, dz) from the site; every argument is a constant after inlining except
  // for the final U_mu(x) load, whose mu is the loop variable
  __device__ __forceinline__ void load(int mu, int dx, int dy, int dz, Mat<T>& m) const {
    const int p = dz == 0 ? 0 : (dz < 0 ? 1 : 2);
    const LinkBox b = link_box<TX, TY>(mu, p);
    const int n = dir_sites<TX, TY>(mu);
    const cx<T>* q = sm + dir_offset<TX, TY>(mu) + plane_first<TX, TY>(mu, p) +
                     (ty + dy - b.ylo) * box_width(b) + (tx + dx - b.xlo);
#pragma unroll
    for (int k = 0; k < 9; k++) m.e[k] = q[k * n];
  }
};

// add_staples with the links from the tile: link MU at the site, staples in the (MU, NU) plane.
template <typename T, int TX, int TY, int MU, int NU>
__device__ __forceinline__ void add_staples_tile(const TileLinks<T, TX, TY>& L, T c, Mat<T>& acc, cx<T>* sh, int mode,
                                                 int slot) {
  constexpr int mx = MU == 0, my = MU == 1, mz = MU == 2;
  constexpr int nx = NU == 0, ny = NU == 1, nz = NU == 2;
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
    L.load(NU, mx, my, mz, a);  // U_nu(x + mu)
    L.load(MU, nx, ny, nz, b);  // U_mu(x + nu)
    mul_nd(a, b, t);
    if (sh && mode == kStapleStore) {
      cx<T>* q = sh + (slot * 9) * kThreads + threadIdx.x;
#pragma unroll
      for (int k = 0; k < 9; k++) q[k * kThreads] = t.e[k];
    }
  }
  L.load(NU, 0, 0, 0, a);  // U_nu(x)
  add_mul_nd(t, a, c, acc);
  L.load(NU, mx - nx, my - ny, mz - nz, a);  // U_nu(x + mu - nu)
  L.load(MU, -nx, -ny, -nz, b);              // U_mu(x - nu)
  mul_dd(a, b, t);
  L.load(NU, -nx, -ny, -nz, a);  // U_nu(x - nu)
  add_mul_nn(t, a, c, acc);
}

// K1 with staged links.  Tiles: blockIdx.x = (z * nty + by) * ntx + bx.  Needs nx >= TX + 2 and
// ny >= TY + 2 (one periodic wrap covers every halo coordinate).  Dynamic shared memory:
// (tile_link_elems + StapleShare slots) elements of cx<T>.
template <typename T, int TX, int TY>
__global__ void __launch_bounds__(kThreads, 2) efield_tile_kernel(Geometry g, FieldPtrs<T> f, EParams<T> p) {
  static_assert(TX * TY == kThreads, "one thread per tile site");
  extern __shared__ __align__(16) unsigned char tile_smem[];
  cx<T>* sm = reinterpret_cast<cx<T>*>(tile_smem);
  cx<T>* sh = sm + tile_link_elems<TX, TY>();
  const int ntx = (g.nx + TX - 1) / TX, nty = (g.ny + TY - 1) / TY;
  const int z = blockIdx.x / (ntx * nty);
  const int r = blockIdx.x - z * (ntx * nty);
  const int x0 = (r % ntx) * TX, y0 = (r / ntx) * TY;
  const long long S = g.S, plane = g.plane;
  // ---- stage the links (coalesced along x; all copies in flight before the one wait)
  if (p.do_e || p.do_jstat) {
#pragma unroll
    for (int mu = 0; mu < 3; mu++) {
#pragma unroll
      for (int pl = 0; pl < 3; pl++) {
        const LinkBox b = link_box<TX, TY>(mu, pl);
        const int w = box_width(b), n = box_sites(b);
        if (n == 0) continue;
        const int dz = pl == 0 ? 0 : (pl == 1 ? -1 : 1);
        const long long zoff = plane * (long long)(z + dz + 1);
        cx<T>* dst = sm + dir_offset<TX, TY>(mu) + plane_first<TX, TY>(mu, pl);
        const int nd = dir_sites<TX, TY>(mu);
        for (int i = threadIdx.x; i < 9 * n; i += kThreads) {
          const int k = i / n, j = i - k * n;
          const int ly = j / w, lx = j - ly * w;
          int gx = x0 + b.xlo + lx, gy = y0 + b.ylo + ly;
          gx = gx < 0 ? gx + g.nx : (gx >= g.nx ? gx - g.nx : gx);
          gy = gy < 0 ? gy + g.ny : (gy >= g.ny ? gy - g.ny : gy);
          cp_async8(dst + k * nd + j, f.U + (long long)(mu * 9 + k) * S + zoff + gx + (long long)g.nx * gy);
        }
      }
    }
    cp_async_wait_all();
  }
  __syncthreads();
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  const int x = x0 + tx, y = y0 + ty;
  if (x >= g.nx || y >= g.ny) return;
  const TileLinks<T, TX, TY> L{sm, tx, ty};
  cx<T>* shs = StapleShare<T>::kSlots ? sh : nullptr;
  const long long s = (long long)x + (long long)g.nx * ((long long)y + (long long)g.ny * (long long)(z + 1));
  const bool lo = (z == 0), hi = (z == g.nz - 1);
  const long long sg = lo ? s - plane : (hi ? s + plane : -1LL);
  if (p.do_e) {
#pragma unroll 1
    for (int mu = 0; mu < 3; mu++) {
      Mat<T> acc;
      set_zero(acc);
      if (mu == 0) {
        add_staples_tile<T, TX, TY, 0, 1>(L, p.cnu[1], acc, shs, kStapleStore, 0);
        add_staples_tile<T, TX, TY, 0, 2>(L, p.cnu[2], acc, shs, kStapleStore, 1);
      } else if (mu == 1) {
        add_staples_tile<T, TX, TY, 1, 0>(L, p.cnu[0], acc, shs, kStapleReuse, 0);
        add_staples_tile<T, TX, TY, 1, 2>(L, p.cnu[2], acc, shs, kStapleStore, 0);
      } else {
        add_staples_tile<T, TX, TY, 2, 0>(L, p.cnu[0], acc, shs, kStapleReuse, 1);
        add_staples_tile<T, TX, TY, 2, 1>(L, p.cnu[1], acc, shs, kStapleReuse, 0);
      }
      Mat<T> u, P;
      if (mu == 0)
        L.load(0, 0, 0, 0, u);
      else if (mu == 1)
        L.load(1, 0, 0, 0, u);
      else
        L.load(2, 0, 0, 0, u);
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
    const long long szm = s - plane;
    Mat<T> uzm;
    L.load(2, 0, 0, -1, uzm);
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

}  // namespace glasma

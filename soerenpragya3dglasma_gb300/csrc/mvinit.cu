// mvinit.cu -- initial conditions on the GPU: McLerran-Venugopalan colliding nuclei as in
// Simulation::Run (S/Simulation.cpp:337-374), or one left-moving nucleus as in
// S/LeftNucleusSimulation.cpp, built from injected charge fluctuations; and the TMD / Glauber
// state of SimulationmitPC::Run (second half of this file).
//
// Reference steps (S/COLLIDINGOBJECTS/CollidingObjects.cpp, S/INITIALCONDITIONS/SUNCCURRENTS/RevSingleNucleus.cpp):
//   rho(x,z)  = sqrt(ax ay) T(z) zeta(x),  T(z) = exp(-(z-c)^2 / 2 sigma^2) / sqrt(2 pi sigma^2)   (:30-47)
//   rho~      = 2D-smoothed rho, kernel exp(-p^2/2 Lambda^2) p^2/(p^2+m^2)                         (:58-83)
//   Phi       = Poisson(rho~), 1/p^2, zero mode removed                                               (:131-176)
//   V(z)      = prod over slices of exp(-+ i Phi(z')/sqrt2) (ordered from the far edge)                (:179-226)
//   SingleSheet: UOld = V^d V(x+i), U_z = 1; rho evolved by dt in z-Fourier space; V' from it;
//   U = V'^d V'(x+i); E_i = ILog(U UOld^d) / coff; JStat from the Gauss law; J by z-FFT filter      (RevSingleNucleus.cpp:7-210)
// The same zeta is used on every slice and T(z) is a scalar, so every slice's Poisson solution is
// T(z) Phi0 with Phi0 = Poisson(Smooth(sqrt(ax ay) zeta)); all factors of the path-ordered product
// then commute and V(z) = exp(i c(z) t.Phi0) with c(z) the signed cumulative sum of T.  The same
// holds for the evolved profile T'(z).  So the 2D transforms run once per nucleus (device FFT), the
// profile sums run on the host (Nz numbers), and the per-site work (links, ILog, Gauss law, the z
// FFT of the currents) runs in kernels.
// The SU(3) MatrixILog is absent from the reference (only SU(2)/U(1) forms exist,
// S/SUNc/SU2/AlgebraOperations.cpp:90-107); here it solves exp(i c t.L) = W by the anti-Hermitian part
// followed by twelve refinements L <- L + P[(R - R^d)/2i], R = exp(-i c t.L) W.
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <string>
#include <vector>

#include "../../include/glasma_gb300.h"
#include "handle.h"
#include "lattice.cuh"

namespace glasma {
namespace {

typedef cx<double> C;
typedef Mat<double> M3;
typedef Alg<double> A8;
using L = long long;

// zeta (host layout a + 8 (x + Nx y)) -> X[a][y][x] complex, scaled
__global__ void load_zeta_kernel(const double* zeta, int nx, int ny, double scale, double2* X) {
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  const L plane = (L)nx * ny;
  if (i >= 8 * plane) return;
  const int a = (int)(i / plane);
  const L r = i - (L)a * plane;
  X[i] = make_double2(scale * zeta[a + 8 * r], 0.0);
}

// multiply the n values of consecutive Nx x Ny planes by f(p^2)/(Nx Ny): mode 0 smoothing, mode 1
// Poisson (zero mode -> 0); keeping the real part afterwards is done by the caller
__global__ void filter2d_kernel(double2* X, L n, int nx, int ny, double ax, double ay, double lambda, double meff,
                                int mode) {
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  const L plane = (L)nx * ny;
  if (i >= n) return;
  const L r = i % plane;
  const int px = (int)(r % nx), py = (int)(r / nx);
  const double p2 = (2.0 - 2.0 * cospi(2.0 * px / (double)nx)) / (ax * ax) +
                    (2.0 - 2.0 * cospi(2.0 * py / (double)ny)) / (ay * ay);
  const double norm = 1.0 / (double)plane;
  double f;
  if (mode == 0)
    f = norm * exp(-p2 / (2.0 * lambda * lambda)) * p2 / (p2 + meff * meff);
  else
    f = (px == 0 && py == 0) ? 0.0 : norm / p2;
  double2 v = X[i];
  X[i] = make_double2(v.x * f, v.y * f);
}
__global__ void real_part_kernel(double2* X, L n) {
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) X[i].y = 0.0;
}

__device__ __forceinline__ void phi_at(const double2* phi, int nx, int ny, int x, int y, A8& v) {
  x = x >= nx ? x - nx : x;
  y = y >= ny ? y - ny : y;
  const L plane = (L)nx * ny, r = x + (L)nx * y;
#pragma unroll
  for (int a = 0; a < 8; a++) v.a[a] = phi[a * plane + r].x;
}

// exp(-i c t.L) W, then (R - R^d)/2i projected, for the ILog refinement
__device__ void matrix_ilog(double c, const M3& W, A8& out) {
  M3 H;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const C a = W.e[i + 3 * j], b = W.e[j + 3 * i];
      // (a - conj(b)) / 2i
      H.e[i + 3 * j] = mk<double>(0.5 * (a.im + b.im), -0.5 * (a.re - b.re));
    }
  A8 Lg;
  alg_from_herm(H, Lg);
  for (int it = 0; it < 12; it++) {
    M3 R0, R;
    expi(-1.0, Lg, R0);
    mul_nn(R0, W, R);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const C a = R.e[i + 3 * j], b = R.e[j + 3 * i];
        H.e[i + 3 * j] = mk<double>(0.5 * (a.im + b.im), -0.5 * (a.re - b.re));
      }
    A8 d;
    alg_from_herm(H, d);
#pragma unroll
    for (int a = 0; a < 8; a++) Lg.a[a] += d.a[a];
  }
#pragma unroll
  for (int a = 0; a < 8; a++) out.a[a] = Lg.a[a] / c;
}

// Links at t (UOld) and t+dt (U) and E for the slices of one nucleus.
template <typename T>
__global__ void sheet_links_kernel(Geometry g, const double2* phi, const double* cz, const double* cz_ev, int zlo,
                                   int zhi, double coff0, double coff1, cx<T>* U, cx<T>* UOld, T* E) {
  const L plane = g.plane;
  const L n = plane * (zhi - zlo + 1);
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int z = zlo + (int)(i / plane);
  const L r = i % plane;
  const int x = (int)(r % g.nx), y = (int)(r / g.nx);
  const L s = r + plane * (z + 1);
  A8 p0, px, py;
  phi_at(phi, g.nx, g.ny, x, y, p0);
  phi_at(phi, g.nx, g.ny, x + 1, y, px);
  phi_at(phi, g.nx, g.ny, x, y + 1, py);
  M3 V0, Vx, Vy, u_old[2], u_new[2];
  for (int pass = 0; pass < 2; pass++) {
    const double c = pass == 0 ? cz[z] : cz_ev[z];
    expi(c, p0, V0);
    expi(c, px, Vx);
    expi(c, py, Vy);
    M3* dst = pass == 0 ? u_old : u_new;
    mul_dn(V0, Vx, dst[0]);
    mul_dn(V0, Vy, dst[1]);
  }
  const double coff[2] = {coff0, coff1};
  M3 id;
  set_zero(id);
  id.e[0].re = id.e[4].re = id.e[8].re = 1.0;
  for (int mu = 0; mu < 2; mu++) {
    M3 W;
    mul_nd(u_new[mu], u_old[mu], W);
    A8 e;
    matrix_ilog(coff[mu], W, e);
    for (int k = 0; k < 9; k++) {
      UOld[(L)(mu * 9 + k) * g.S + s] = mk<T>((T)u_old[mu].e[k].re, (T)u_old[mu].e[k].im);
      U[(L)(mu * 9 + k) * g.S + s] = mk<T>((T)u_new[mu].e[k].re, (T)u_new[mu].e[k].im);
    }
    for (int a = 0; a < 8; a++) E[(L)(mu * 8 + a) * g.S + s] = (T)e.a[a];
  }
  for (int k = 0; k < 9; k++) {
    UOld[(L)(18 + k) * g.S + s] = mk<T>((T)id.e[k].re, 0);
    U[(L)(18 + k) * g.S + s] = mk<T>((T)id.e[k].re, 0);
  }
  for (int a = 0; a < 8; a++) E[(L)(16 + a) * g.S + s] = (T)0;
}

// JStat from the Gauss law inside [zlo,zhi], zero elsewhere, into X[a][site] (complex, imaginary 0)
template <typename T>
__global__ void sheet_jstat_kernel(Geometry g, const cx<T>* U, const T* E, int zlo, int zhi, double2* X) {
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.vol) return;
  const L plane = g.plane;
  const int z = (int)(i / plane);
  const L r = i - (L)z * plane;
  const int x = (int)(r % g.nx), y = (int)(r / g.nx);
  A8 tot;
#pragma unroll
  for (int a = 0; a < 8; a++) tot.a[a] = 0.0;
  if (z >= zlo && z <= zhi) {
    const L s = i + plane;
    const int xm = x == 0 ? g.nx - 1 : x - 1, ym = y == 0 ? g.ny - 1 : y - 1;
    const L nb[2] = {xm + (L)g.nx * y + plane * (z + 1), x + (L)g.nx * ym + plane * (z + 1)};
    for (int mu = 0; mu < 2; mu++) {
      M3 v;
      A8 e, em, down;
      for (int k = 0; k < 9; k++) {
        const cx<T> q = U[(L)(mu * 9 + k) * g.S + nb[mu]];
        v.e[k] = mk<double>((double)q.re, (double)q.im);
      }
      for (int a = 0; a < 8; a++) {
        e.a[a] = (double)E[(L)(mu * 8 + a) * g.S + s];
        em.a[a] = (double)E[(L)(mu * 8 + a) * g.S + nb[mu]];
      }
      inv_adj_mul(v, em, down);
      for (int a = 0; a < 8; a++) tot.a[a] += e.a[a] - down.a[a];
    }
  }
  for (int a = 0; a < 8; a++) X[a * g.vol + i] = make_double2(1.4142135623730950488016887242096980785697 * tot.a[a], 0.0);
}

// z-Fourier filter turning JStat into J (RevSingleNucleus.cpp:146-192); filt[p] precomputed on the host
__global__ void zfilter_kernel(double2* X, L vol, L plane, int nz, const double2* filt) {
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 8 * vol) return;
  const int pz = (int)((i % vol) / plane);
  const double2 f = filt[pz], v = X[i];
  X[i] = make_double2(v.x * f.x - v.y * f.y, v.x * f.y + v.y * f.x);
}

template <typename T>
__global__ void store_real_kernel(const double2* X, T* J, L vol, L plane, L S) {
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 8 * vol) return;
  const int a = (int)(i / vol);
  const L site = i - (L)a * vol;
  J[(L)a * S + plane + site] = (T)X[i].x;
}
template <typename T>
__global__ void identity_links_kernel(cx<T>* U, L S) {
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 27 * S) return;
  const int k = (int)((i / S) % 9);
  U[i] = mk<T>((k == 0 || k == 4 || k == 8) ? T(1) : T(0), T(0));
}

inline unsigned g1(L n) { return (unsigned)((n + 255) / 256); }

// ---------------------------------------------------------------- TMD / Glauber initial state
// noise in the reference's draw order (a + 8 (x + Nx (y + Ny z))) -> X[a][z][y][x], scaled
__global__ void noise_planes_kernel(const double* noise, L vol, double scale, double2* X) {
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 8 * vol) return;
  const int a = (int)(i / vol);
  const L site = i - (L)a * vol;
  X[i] = make_double2(scale * noise[a + 8 * site], 0.0);
}

// ChargeFluctuation's momentum-space weight (S/TMDNUCLEUS/CorrelationFunction.cpp:12-19, 55-80):
// X(p) <- X(p) sqrt(GammaK(x, pT^2)) / V for x = pLong / (sqrt(s)/sqrt2) <= 1, else 0, with
// pLong = |2 sin(pi pz/Nz)| / (sqrt2 a_z[fm]), Qs = Qs0A x^-0.1 (1 - x) / sqrt(ax ay) and
// GammaK = 4 pi Nc/(Nc^2-1) pT^4/Qs^2 exp(-pT^2/Qs^2).  At pz = 0, x = 0 and Qs is infinite: the weight is 0.
__global__ void cf_filter_kernel(double2* X, int nx, int ny, int nz, double ax, double ay, double az_fm,
                                 double com_energy, double qs0a) {
  const L vol = (L)nx * ny * nz;
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= vol) return;
  const L plane = (L)nx * ny;
  const int pz = (int)(i / plane);
  const L r = i - (L)pz * plane;
  const int px = (int)(r % nx), py = (int)(r / nx);
  const double inv_sqrt2 = 0.70710678118654752440084436210484903928483593768847;
  const double pl = inv_sqrt2 * sqrt((2.0 - 2.0 * cos(2.0 * M_PI * pz / (double)nz)) / (az_fm * az_fm));
  const double pt2 = (2.0 - 2.0 * cos(2.0 * M_PI * px / (double)nx)) / (ax * ax) +
                     (2.0 - 2.0 * cos(2.0 * M_PI * py / (double)ny)) / (ay * ay);
  const double x = pl / (com_energy * inv_sqrt2);
  double f = 0.0;
  if (x <= 1.0) {
    const double qs = qs0a * pow(x, -0.1) * (1.0 - x) / sqrt(ax * ay);
    const double gk = 4.0 * M_PI * 3.0 / 8.0 * pt2 * pt2 / (qs * qs) * exp(-pt2 / (qs * qs));
    f = sqrt(gk) / (double)vol;
  }
#pragma unroll
  for (int a = 0; a < 8; a++) {
    const double2 v = X[(L)a * vol + i];
    X[(L)a * vol + i] = make_double2(v.x * f, v.y * f);
  }
}

// rho(x,y,z,a) = a^3 sqrt(a_z[fm] T(x,y,z) / a_z) CF(x,y,z,a) (TMDbased.cpp:25-51) with the nuclear
// profile T = sum_n gamma exp(-((x-x_n)^2 + (y-y_n)^2 + (gamma z - z_n)^2) / 2 BG) / sqrt(2 pi BG)
// (GBWSampling.cpp:104-110) factorised into per-nucleon tables ex[n][x], ey[n][y], ez[n][z] (ez carries
// gamma / sqrt(2 pi BG)).  CF is the real part of X; X becomes (rho, 0).
__global__ void tmd_rho_kernel(double2* X, int nx, int ny, int nz, int A, const double* __restrict__ ex,
                               const double* __restrict__ ey, const double* __restrict__ ez, double pref) {
  const L vol = (L)nx * ny * nz;
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= vol) return;
  const L plane = (L)nx * ny;
  const int z = (int)(i / plane);
  const L r = i - (L)z * plane;
  const int x = (int)(r % nx), y = (int)(r / nx);
  double T = 0.0;
  for (int n = 0; n < A; n++) T += ex[(L)n * nx + x] * ey[(L)n * ny + y] * ez[(L)n * nz + z];
  const double f = pref * sqrt(T);
#pragma unroll
  for (int a = 0; a < 8; a++) X[(L)a * vol + i] = make_double2(f * X[(L)a * vol + i].x, 0.0);
}

// One forward 2D transform feeds both outputs of a slice: the filtered density (X, weight
// p^2/(p^2+m^2)/(Nx Ny), TMDbased.cpp:53-80) and the Poisson field of that filtered density (Y, weight
// 1/(p^2+m^2)/(Nx Ny), zero mode 0; the reference transforms the filtered density again and divides by
// p^2, TMDbased.cpp:125-174, which is the same up to rounding).
__global__ void split_filter_kernel(double2* X, double2* Y, L n, int nx, int ny, double ax, double ay, double meff) {
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const L plane = (L)nx * ny;
  const L r = i % plane;
  const int px = (int)(r % nx), py = (int)(r / nx);
  const double p2 = (2.0 - 2.0 * cos(2.0 * M_PI * px / (double)nx)) / (ax * ax) +
                    (2.0 - 2.0 * cos(2.0 * M_PI * py / (double)ny)) / (ay * ay);
  const double norm = 1.0 / (double)plane;
  const double2 v = X[i];
  const double fx = norm * p2 / (p2 + meff * meff);
  const double fy = (px == 0 && py == 0) ? 0.0 : norm / (p2 + meff * meff);
  X[i] = make_double2(v.x * fx, v.y * fx);
  Y[i] = make_double2(v.x * fy, v.y * fy);
}

// Path-ordered Wilson lines (SetNewWilsonLines, TMDbased.cpp:176-221 / CollidingObjects.cpp:180-226):
// per transverse site W <- exp(i c t.Phi(z)) W over the slices in order ('R' from z = 0 up with
// c = +1/sqrt2, 'L' from the top slice down with c = -1/sqrt2), V(z) = W; Phi = real part of P[a][site],
// V[k][site] complex, k = i + 3j.  A walk over all slices per transverse site leaves the GPU nearly idle
// (one thread per site), so the product is a chunked scan: the ordered slices are cut into chunks of
// kPathChunk; per (site, chunk) the exponentials are
// stored in V and their ordered product in `prod` (phase 1); per site a prefix over the chunks turns
// `prod` into each chunk's incoming product (phase 2); per (site, chunk) the incoming product is carried
// through the stored exponentials into V (phase 3).  prod[q][chunk][col], nch chunks.
constexpr int kPathChunk = 32;
__global__ void path_chunk_kernel(const double2* P, int nx, int ny, int nz, int up, double c, double2* V,
                                  double2* prod) {
  const L plane = (L)nx * ny, vol = plane * nz;
  const int nch = (nz + kPathChunk - 1) / kPathChunk;
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= plane * nch) return;
  const int ch = (int)(i / plane);
  const L col = i - (L)ch * plane;
  M3 W;
  set_zero(W);
  W.e[0].re = W.e[4].re = W.e[8].re = 1.0;
  const int k1 = min(nz, (ch + 1) * kPathChunk);
  for (int k = ch * kPathChunk; k < k1; k++) {
    const int z = up ? k : nz - 1 - k;
    const L site = col + plane * z;
    A8 phi;
#pragma unroll
    for (int a = 0; a < 8; a++) phi.a[a] = P[(L)a * vol + site].x;
    M3 X, Wn;
    expi(c, phi, X);
#pragma unroll
    for (int q = 0; q < 9; q++) V[(L)q * vol + site] = make_double2(X.e[q].re, X.e[q].im);
    mul_nn(X, W, Wn);
    W = Wn;
  }
#pragma unroll
  for (int q = 0; q < 9; q++) prod[((L)q * nch + ch) * plane + col] = make_double2(W.e[q].re, W.e[q].im);
}
__global__ void path_prefix_kernel(double2* prod, L plane, int nch) {
  const L col = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= plane) return;
  M3 In;
  set_zero(In);
  In.e[0].re = In.e[4].re = In.e[8].re = 1.0;
  for (int ch = 0; ch < nch; ch++) {
    M3 Pc, Wn;
#pragma unroll
    for (int q = 0; q < 9; q++) {
      double2* p = prod + ((L)q * nch + ch) * plane + col;
      Pc.e[q] = mk<double>(p->x, p->y);
      *p = make_double2(In.e[q].re, In.e[q].im);
    }
    mul_nn(Pc, In, Wn);
    In = Wn;
  }
}
__global__ void path_apply_kernel(int nx, int ny, int nz, int up, const double2* prod, double2* V) {
  const L plane = (L)nx * ny, vol = plane * nz;
  const int nch = (nz + kPathChunk - 1) / kPathChunk;
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= plane * nch) return;
  const int ch = (int)(i / plane);
  const L col = i - (L)ch * plane;
  M3 W;
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const double2 v = prod[((L)q * nch + ch) * plane + col];
    W.e[q] = mk<double>(v.x, v.y);
  }
  const int k1 = min(nz, (ch + 1) * kPathChunk);
  for (int k = ch * kPathChunk; k < k1; k++) {
    const int z = up ? k : nz - 1 - k;
    const L site = col + plane * z;
    M3 X, Wn;
#pragma unroll
    for (int q = 0; q < 9; q++) {
      const double2 v = V[(L)q * vol + site];
      X.e[q] = mk<double>(v.x, v.y);
    }
    mul_nn(X, W, Wn);
    W = Wn;
#pragma unroll
    for (int q = 0; q < 9; q++) V[(L)q * vol + site] = make_double2(W.e[q].re, W.e[q].im);
  }
}

__device__ __forceinline__ void load_v(const double2* V, L vol, L site, M3& m) {
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const double2 v = V[(L)q * vol + site];
    m.e[q] = mk<double>(v.x, v.y);
  }
}
// SingleSheet's links and E from the Wilson lines before (V) and after (Vp) the density's dt shift
// (RevSingleNucleus.cpp:12-110): UOld_i = V^d(x) V(x+i), U_i = Vp^d(x) Vp(x+i), U_z = UOld_z = 1,
// E_i = ILog(U_i UOld_i^d) / coff_i, E_z = 0, on the slices [zlo, zhi].
template <typename T>
__global__ void sheet_links_v_kernel(Geometry g, const double2* V, const double2* Vp, int zlo, int zhi, double coff0,
                                     double coff1, cx<T>* U, cx<T>* UOld, T* E) {
  const L plane = g.plane, vol = g.vol;
  const L n = plane * (zhi - zlo + 1);
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int z = zlo + (int)(i / plane);
  const L r = i % plane;
  const int x = (int)(r % g.nx), y = (int)(r / g.nx);
  const L site = r + plane * z, s = site + plane;
  const L sx = (x + 1 == g.nx ? 0 : x + 1) + (L)g.nx * y + plane * z;
  const L sy = x + (L)g.nx * (y + 1 == g.ny ? 0 : y + 1) + plane * z;
  M3 u_old[2], u_new[2];
  for (int pass = 0; pass < 2; pass++) {
    const double2* W = pass == 0 ? V : Vp;
    M3 V0, Vx, Vy;
    load_v(W, vol, site, V0);
    load_v(W, vol, sx, Vx);
    load_v(W, vol, sy, Vy);
    M3* dst = pass == 0 ? u_old : u_new;
    mul_dn(V0, Vx, dst[0]);
    mul_dn(V0, Vy, dst[1]);
  }
  const double coff[2] = {coff0, coff1};
  for (int mu = 0; mu < 2; mu++) {
    M3 W;
    mul_nd(u_new[mu], u_old[mu], W);
    A8 e;
    matrix_ilog(coff[mu], W, e);
    for (int k = 0; k < 9; k++) {
      UOld[(L)(mu * 9 + k) * g.S + s] = mk<T>((T)u_old[mu].e[k].re, (T)u_old[mu].e[k].im);
      U[(L)(mu * 9 + k) * g.S + s] = mk<T>((T)u_new[mu].e[k].re, (T)u_new[mu].e[k].im);
    }
    for (int a = 0; a < 8; a++) E[(L)(mu * 8 + a) * g.S + s] = (T)e.a[a];
  }
  for (int k = 0; k < 9; k++) {
    const T d = (k == 0 || k == 4 || k == 8) ? T(1) : T(0);
    UOld[(L)(18 + k) * g.S + s] = mk<T>(d, T(0));
    U[(L)(18 + k) * g.S + s] = mk<T>(d, T(0));
  }
  for (int a = 0; a < 8; a++) E[(L)(16 + a) * g.S + s] = (T)0;
}

// real parts of X[a][site] -> out[a + 8 s] in the reference's ChargeDensity layout, ghost slices copied
// from the edge slices (ChargeDensity::SynchronizeGhostCells, open boundaries)
__global__ void pack_density_kernel(const double2* X, int nz, L plane, double* out) {
  const L S = plane * (nz + 2), vol = plane * nz;
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 8 * S) return;
  const int a = (int)(i % 8);
  const L s = i / 8;
  L zs = s / plane - 1;
  zs = zs < 0 ? 0 : (zs >= nz ? nz - 1 : zs);
  out[i] = X[(L)a * vol + (s % plane) + plane * zs].x;
}

struct Nucleus {
  char D;          // 'L' or 'R'
  int zlo, zhi;    // slices the sheet covers
  const double* zeta;
  double qs;
  int center;
};

}  // namespace
}  // namespace glasma

namespace {
thread_local std::string g_mv_error;
int mvfail(int st, const std::string& m) {
  g_mv_error = m;
  return st;
}
struct Dev {
  void* p = nullptr;
  ~Dev() {
    if (p) cudaFree(p);
  }
  bool alloc(size_t b) { return cudaMalloc(&p, b) == cudaSuccess; }
};
}  // namespace

// JStat of one nucleus from the Gauss law on its slices, and J = JStat filtered in z-Fourier space
// (S/INITIALCONDITIONS/SUNCCURRENTS/RevSingleNucleus.cpp:112-192).  Z: 8 vol complex work array;
// twz: z twiddles; filt: nz complex.
template <typename T>
static int sheet_currents(glasma_lattice* h, char D, int zlo, int zhi, double dt, double2* Z, double2* twz,
                          double2* filt) {
  using namespace glasma;
  const Geometry& g = h->g;
  cudaStream_t st = h->stream;
  const int nz = g.nz;
  const L plane = g.plane;
  const int fstat = D == 'L' ? GLASMA_FIELD_JPSTAT : GLASMA_FIELD_JMSTAT;
  const int fj = D == 'L' ? GLASMA_FIELD_JP : GLASMA_FIELD_JM;
  sheet_jstat_kernel<T><<<g1(g.vol), 256, 0, st>>>(g, static_cast<const cx<T>*>(h->f[GLASMA_FIELD_U]),
                                                   static_cast<const T*>(h->f[GLASMA_FIELD_E]), zlo, zhi, Z);
  store_real_kernel<T><<<g1(8 * g.vol), 256, 0, st>>>(Z, static_cast<T*>(h->f[fstat]), g.vol, plane, g.S);
  std::vector<double2> fh(nz);
  for (int p = 0; p < nz; p++) {
    const double om = std::sqrt((2.0 - 2.0 * std::cos(2.0 * M_PI * p / nz)) / (g.a[2] * g.a[2]));
    const std::complex<double> zd = (D == 'R' ? 1.0 : -1.0) * (1.0 - std::polar(1.0, -2.0 * M_PI * (double)p / nz)) / g.a[2];
    const std::complex<double> npos = std::polar(1.0, (D == 'R' ? 1.0 : -1.0) * om * dt) - 1.0;
    const std::complex<double> nneg = std::polar(1.0, (D == 'R' ? -1.0 : 1.0) * om * dt) - 1.0;
    std::complex<double> f;
    if (p == 0)
      f = 1.0;
    else if (2 * p < nz)
      f = npos / (dt * zd);
    else if (2 * p == nz)
      f = 0.0;
    else
      f = nneg / (dt * zd);
    f /= (double)nz;
    fh[p] = make_double2(f.real(), f.imag());
  }
  // from pageable memory: the table has been taken when the call returns
  cudaError_t e = cudaMemcpyAsync(filt, fh.data(), sizeof(double2) * nz, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = fft_lines(Z, nz, plane, 8 * g.vol, 0, twz, st);
  zfilter_kernel<<<g1(8 * g.vol), 256, 0, st>>>(Z, g.vol, plane, nz, filt);
  if (e == cudaSuccess) e = fft_lines(Z, nz, plane, 8 * g.vol, 1, twz, st);
  store_real_kernel<T><<<g1(8 * g.vol), 256, 0, st>>>(Z, static_cast<T*>(h->f[fj]), g.vol, plane, g.S);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return mvfail(GLASMA_ERR_CUDA, std::string("sheet currents: ") + cudaGetErrorString(e));
  return GLASMA_OK;
}

template <typename T>
static int mv_impl(glasma_lattice* h, const std::vector<glasma::Nucleus>& nuclei, double sigma, double lambda,
                   double meff, double dt) {
  using namespace glasma;
  const Geometry& g = h->g;
  cudaStream_t st = h->stream;
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const L plane = g.plane;
  Dev X2, phi, zbuf, twx, twy, twz, czd, czed, filt;
  if (!X2.alloc(sizeof(double2) * 8 * plane) || !phi.alloc(sizeof(double2) * 8 * plane) ||
      !zbuf.alloc(sizeof(double2) * 8 * g.vol) || !czd.alloc(sizeof(double) * nz) || !czed.alloc(sizeof(double) * nz) ||
      !filt.alloc(sizeof(double2) * nz))
    return mvfail(GLASMA_ERR_OUT_OF_MEMORY, "MV buffers");
  twx.p = make_twiddles(nx, st);
  twy.p = make_twiddles(ny, st);
  twz.p = make_twiddles(nz, st);
  if (!twx.p || !twy.p || !twz.p) return mvfail(GLASMA_ERR_OUT_OF_MEMORY, "twiddles");
  Dev zeta_dev;
  if (!zeta_dev.alloc(sizeof(double) * 8 * plane)) return mvfail(GLASMA_ERR_OUT_OF_MEMORY, "zeta");
  double2* X = static_cast<double2*>(X2.p);
  auto fft2 = [&](double2* buf, int inverse) {
    cudaError_t e = fft_lines(buf, nx, 1, 8 * plane, inverse, static_cast<double2*>(twx.p), st);
    if (e == cudaSuccess) e = fft_lines(buf, ny, nx, 8 * plane, inverse, static_cast<double2*>(twy.p), st);
    return e;
  };
  // every field starts from Lattice::Init's state: identity links, zero E and currents
  for (int f : {GLASMA_FIELD_U, GLASMA_FIELD_UOLD})
    identity_links_kernel<T><<<g1(27 * g.S), 256, 0, st>>>(static_cast<cx<T>*>(h->f[f]), g.S);
  for (int f : {GLASMA_FIELD_E, GLASMA_FIELD_JP, GLASMA_FIELD_JM, GLASMA_FIELD_JPSTAT, GLASMA_FIELD_JMSTAT})
    cudaMemsetAsync(h->f[f], 0, (size_t)g.S * (f == GLASMA_FIELD_E ? 24 : 8) * h->real_bytes, st);
  const double a3 = g.a[0] * g.a[1] * g.a[2];
  const double inv_sqrt2 = 0.70710678118654752440084436210484903928483593768847;
  for (const Nucleus& nu : nuclei) {
    // ---- Phi0 = Poisson(Smooth(sqrt(ax ay) qs zeta))
    cudaMemcpyAsync(zeta_dev.p, nu.zeta, sizeof(double) * 8 * plane, cudaMemcpyHostToDevice, st);
    load_zeta_kernel<<<g1(8 * plane), 256, 0, st>>>(static_cast<const double*>(zeta_dev.p), nx, ny,
                                                    std::sqrt(g.a[0] * g.a[1]) * nu.qs, X);
    cudaError_t e = fft2(X, 0);
    filter2d_kernel<<<g1(8 * plane), 256, 0, st>>>(X, 8 * plane, nx, ny, g.a[0], g.a[1], lambda, meff, 0);
    if (e == cudaSuccess) e = fft2(X, 1);
    real_part_kernel<<<g1(8 * plane), 256, 0, st>>>(X, 8 * plane);
    if (e == cudaSuccess) e = fft2(X, 0);
    filter2d_kernel<<<g1(8 * plane), 256, 0, st>>>(X, 8 * plane, nx, ny, g.a[0], g.a[1], lambda, meff, 1);
    if (e == cudaSuccess) e = fft2(X, 1);
    real_part_kernel<<<g1(8 * plane), 256, 0, st>>>(X, 8 * plane);
    if (e != cudaSuccess) return mvfail(GLASMA_ERR_CUDA, std::string("MV 2D FFT: ") + cudaGetErrorString(e));
    cudaMemcpyAsync(phi.p, X, sizeof(double2) * 8 * plane, cudaMemcpyDeviceToDevice, st);
    // ---- profiles on the host: T(z), evolved T'(z), cumulative Wilson-line coefficients
    std::vector<double> prof(nz), Tev(nz), cz(nz), czev(nz);
    for (int z = 0; z < nz; z++)
      prof[z] = std::exp(-0.5 * ((z - nu.center) / sigma) * ((z - nu.center) / sigma)) / std::sqrt(2 * M_PI * sigma * sigma);
    {
      // EvolveRhoViaFourier (S/DYNAMICS/SUNcDynamics.cpp:275-350) applied to the profile
      std::vector<std::complex<double>> P(nz);
      for (int p = 0; p < nz; p++) {
        std::complex<double> acc = 0.0;
        for (int z = 0; z < nz; z++) acc += prof[z] * std::polar(1.0, -2.0 * M_PI * (double)((long)p * z % nz) / nz);
        const double om = std::sqrt((2.0 - 2.0 * std::cos(2.0 * M_PI * p / nz)) / (g.a[2] * g.a[2]));
        const bool low = p < nz / 2;
        const double sgn = (nu.D == 'L') ? (low ? -1.0 : 1.0) : (low ? 1.0 : -1.0);
        P[p] = acc / (double)nz * std::polar(1.0, sgn * om * dt);
      }
      for (int z = 0; z < nz; z++) {
        std::complex<double> acc = 0.0;
        for (int p = 0; p < nz; p++) acc += P[p] * std::polar(1.0, 2.0 * M_PI * (double)((long)p * z % nz) / nz);
        Tev[z] = acc.real();
      }
    }
    // 'L' accumulates from the top slice down with exp(-i Phi/sqrt2), 'R' from slice 0 up with exp(+i Phi/sqrt2)
    if (nu.D == 'L') {
      double a1 = 0.0, a2 = 0.0;
      for (int z = nz - 1; z >= 0; z--) {
        a1 += prof[z];
        a2 += Tev[z];
        cz[z] = -inv_sqrt2 * a1;
        czev[z] = -inv_sqrt2 * a2;
      }
    } else {
      double a1 = 0.0, a2 = 0.0;
      for (int z = 0; z < nz; z++) {
        a1 += prof[z];
        a2 += Tev[z];
        cz[z] = inv_sqrt2 * a1;
        czev[z] = inv_sqrt2 * a2;
      }
    }
    cudaMemcpyAsync(czd.p, cz.data(), sizeof(double) * nz, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(czed.p, czev.data(), sizeof(double) * nz, cudaMemcpyHostToDevice, st);
    // ---- links and E on the sheet's slices
    const double coff0 = -dt * g.a[0] * g.a[0] / a3, coff1 = -dt * g.a[1] * g.a[1] / a3;
    const L nsheet = plane * (nu.zhi - nu.zlo + 1);
    sheet_links_kernel<T><<<g1(nsheet), 256, 0, st>>>(
        g, static_cast<const double2*>(phi.p), static_cast<const double*>(czd.p), static_cast<const double*>(czed.p),
        nu.zlo, nu.zhi, coff0, coff1, static_cast<cx<T>*>(h->f[GLASMA_FIELD_U]),
        static_cast<cx<T>*>(h->f[GLASMA_FIELD_UOLD]), static_cast<T*>(h->f[GLASMA_FIELD_E]));
    if ((e = cudaGetLastError()) != cudaSuccess) return mvfail(GLASMA_ERR_CUDA, "sheet links");
    // ---- JStat and J = z-filtered JStat
    int cst = sheet_currents<T>(h, nu.D, nu.zlo, nu.zhi, dt, static_cast<double2*>(zbuf.p),
                                static_cast<double2*>(twz.p), static_cast<double2*>(filt.p));
    if (cst != GLASMA_OK) return cst;
  }
  // Simulation::Run syncs every field afterwards (S/Simulation.cpp:365-374)
  const int fields[7] = {GLASMA_FIELD_U, GLASMA_FIELD_UOLD, GLASMA_FIELD_E, GLASMA_FIELD_JP, GLASMA_FIELD_JM,
                         GLASMA_FIELD_JPSTAT, GLASMA_FIELD_JMSTAT};
  for (int f : fields) {
    cudaError_t e;
    if (f == GLASMA_FIELD_U || f == GLASMA_FIELD_UOLD)
      e = launch_sync_ghosts<cx<T>>(g, static_cast<cx<T>*>(h->f[f]), 27, st);
    else
      e = launch_sync_ghosts<T>(g, static_cast<T*>(h->f[f]), f == GLASMA_FIELD_E ? 24 : 8, st);
    if (e != cudaSuccess) return mvfail(GLASMA_ERR_CUDA, "ghost sync");
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return mvfail(GLASMA_ERR_CUDA, "MV sync");
  return GLASMA_OK;
}

extern "C" int glasma_mv_init(glasma_lattice* h, int single_left, const double* zeta_left, const double* zeta_right,
                              double qs_left, double qs_right, int center_left, int center_right, double sigma,
                              double lambda, double meff, double dt) {
  using namespace glasma;
  if (!h || !zeta_left || (!single_left && !zeta_right)) return mvfail(GLASMA_ERR_INVALID_ARGUMENT, "null argument");
  if (!(sigma > 0) || !(lambda > 0) || !(meff >= 0) || !(dt > 0)) return mvfail(GLASMA_ERR_INVALID_ARGUMENT, "bad parameters");
  if (cudaSetDevice(h->device) != cudaSuccess) return mvfail(GLASMA_ERR_CUDA, "cudaSetDevice");
  std::vector<Nucleus> nuclei;
  const int nz = h->g.nz;
  if (single_left) {
    nuclei.push_back({'L', 0, nz - 1, zeta_left, qs_left, center_left});
  } else {
    nuclei.push_back({'L', 0, (nz - 2) / 2, zeta_left, qs_left, center_left});
    nuclei.push_back({'R', nz / 2, nz - 1, zeta_right, qs_right, center_right});
  }
  return h->precision == GLASMA_FP64 ? mv_impl<double>(h, nuclei, sigma, lambda, meff, dt)
                                     : mv_impl<float>(h, nuclei, sigma, lambda, meff, dt);
}

extern "C" const char* glasma_mv_last_error(void) { return g_mv_error.c_str(); }

// ---------------------------------------------------------------- TMD / Glauber initial state
// SimulationmitPC::Run (S/SimulationmitPC.cpp:315-367).  Per nucleus:
//   CF     = ChargeFluctuation: 3D transform of the injected noise / sqrt(a^3), weight sqrt(GammaK)/V,
//            inverse transform, real part (S/TMDNUCLEUS/CorrelationFunction.cpp:23-97)
//   rho    = a^3 sqrt(a_z[fm] T / a_z) CF with the Glauber nucleus' profile T (TMDbased.cpp:25-51)
//   rho_f  = 2D filter p^2/(p^2+m^2) of every slice; Phi = Poisson(rho_f) (TMDbased.cpp:53-174)
//   V      = path-ordered exp(-+ i Phi/sqrt2) over the slices (TMDbased.cpp:176-221, 243-291)
//   then SingleSheet (RevSingleNucleus.cpp:7-210): UOld from V, rho_f shifted by dt in z-Fourier
//   space (EvolveRhoViaFourier, S/DYNAMICS/SUNcDynamics.cpp:275-350), V' from its per-slice Poisson
//   field (CollidingObjects::SetWilsonLinesForFirstStep), U from V', E = ILog(U UOld^d)/coff, JStat
//   from the Gauss law, J from JStat by the z filter.
// Unlike the MV state the density differs from slice to slice, so every slice gets its own Poisson
// field: the 2D transforms run batched over all 8 Nz planes at once, and the path ordering is a
// chunked scan over the slices.
namespace {
const double kTmdBG = 4.0 * 0.197 * 0.197;  // nucleon width^2 in fm^2 (GBWSampling.cpp:4)

// Woods-Saxon radius and surface thickness in fm (S/TMDNUCLEUS/NuclearData.cpp:3-87)
bool woods_saxon(int A, double* R, double* s) {
  switch (A) {
    case 16: *R = 2.608; *s = 0.5130; return true;
    case 54: *R = 5.420; *s = 0.57; return true;
    case 197: *R = 6.38; *s = 0.535; return true;
    case 208: *R = 6.62; *s = 0.546; return true;
    default: return false;
  }
}
}  // namespace

template <typename T>
static int tmd_impl(glasma_lattice* h, const double* const noise[2], const double* const nucleons[2],
                    const glasma_tmd_params& p, double* const rho_out[2]) {
  using namespace glasma;
  const Geometry& g = h->g;
  cudaStream_t st = h->stream;
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const L plane = g.plane, vol = g.vol;
  const int A = p.atomic_number;
  Dev stage, X2, Y2, V2, Vp2, twx, twy, twz, filt, tabs;
  if (!stage.alloc(sizeof(double) * 8 * g.S) || !X2.alloc(sizeof(double2) * 8 * vol) ||
      !Y2.alloc(sizeof(double2) * 8 * vol) || !V2.alloc(sizeof(double2) * 9 * vol) ||
      !Vp2.alloc(sizeof(double2) * 9 * vol) || !filt.alloc(sizeof(double2) * nz) ||
      !tabs.alloc(sizeof(double) * (size_t)A * (nx + ny + nz)))
    return mvfail(GLASMA_ERR_OUT_OF_MEMORY, "TMD buffers");
  twx.p = make_twiddles(nx, st);
  twy.p = make_twiddles(ny, st);
  twz.p = make_twiddles(nz, st);
  if (!twx.p || !twy.p || !twz.p) return mvfail(GLASMA_ERR_OUT_OF_MEMORY, "twiddles");
  double2* X = static_cast<double2*>(X2.p);
  double2* Y = static_cast<double2*>(Y2.p);
  double2* V = static_cast<double2*>(V2.p);
  double2* Vp = static_cast<double2*>(Vp2.p);
  const double2* tw[3] = {static_cast<double2*>(twx.p), static_cast<double2*>(twy.p), static_cast<double2*>(twz.p)};
  auto fft2 = [&](double2* buf, int inverse) {
    cudaError_t e = fft_lines(buf, nx, 1, 8 * vol, inverse, tw[0], st);
    if (e == cudaSuccess) e = fft_lines(buf, ny, nx, 8 * vol, inverse, tw[1], st);
    return e;
  };
  auto fftz = [&](double2* buf, int inverse) { return fft_lines(buf, nz, plane, 8 * vol, inverse, tw[2], st); };
  // path-ordered Wilson lines: the chunked scan (small per-chunk products keep every SM busy)
  const int nch = (nz + kPathChunk - 1) / kPathChunk;
  Dev chunk;
  if (!chunk.alloc(sizeof(double2) * 9 * (size_t)nch * plane)) return mvfail(GLASMA_ERR_OUT_OF_MEMORY, "path chunks");
  auto path_scan = [&](const double2* Pin, int up, double c, double2* Vout) {
    double2* pr = static_cast<double2*>(chunk.p);
    const L n = plane * nch;
    path_chunk_kernel<<<g1(n), 256, 0, st>>>(Pin, nx, ny, nz, up, c, Vout, pr);
    path_prefix_kernel<<<(unsigned)((plane + 63) / 64), 64, 0, st>>>(pr, plane, nch);
    path_apply_kernel<<<g1(n), 256, 0, st>>>(nx, ny, nz, up, pr, Vout);
  };
  // every field starts from Lattice::Init's state: identity links, zero E and currents
  for (int f : {GLASMA_FIELD_U, GLASMA_FIELD_UOLD})
    identity_links_kernel<T><<<g1(27 * g.S), 256, 0, st>>>(static_cast<cx<T>*>(h->f[f]), g.S);
  for (int f : {GLASMA_FIELD_E, GLASMA_FIELD_JP, GLASMA_FIELD_JM, GLASMA_FIELD_JPSTAT, GLASMA_FIELD_JMSTAT})
    cudaMemsetAsync(h->f[f], 0, (size_t)g.S * (f == GLASMA_FIELD_E ? 24 : 8) * h->real_bytes, st);
  const double a3 = g.a[0] * g.a[1] * g.a[2];
  const double gamma = p.com_energy * 0.197 / 2.0;
  const double inv_sqrt2 = 0.70710678118654752440084436210484903928483593768847;
  std::vector<double> tab((size_t)A * (nx + ny + nz));
  for (int k = 0; k < 2; k++) {
    const char D = k == 0 ? 'L' : 'R';
    const int zlo = D == 'L' ? 0 : nz / 2, zhi = D == 'L' ? (nz - 2) / 2 : nz - 1;
    const int center = D == 'L' ? p.center_left : p.center_right;
    cudaError_t e;
    // ---- CF
    if ((e = cudaMemcpyAsync(stage.p, noise[k], sizeof(double) * 8 * vol, cudaMemcpyHostToDevice, st)) != cudaSuccess)
      return mvfail(GLASMA_ERR_CUDA, std::string("noise upload: ") + cudaGetErrorString(e));
    noise_planes_kernel<<<g1(8 * vol), 256, 0, st>>>(static_cast<const double*>(stage.p), vol, 1.0 / std::sqrt(a3), X);
    e = fft2(X, 0);
    if (e == cudaSuccess) e = fftz(X, 0);
    cf_filter_kernel<<<g1(vol), 256, 0, st>>>(X, nx, ny, nz, g.a[0], g.a[1], p.az_fm, p.com_energy, p.qs0a);
    if (e == cudaSuccess) e = fft2(X, 1);
    if (e == cudaSuccess) e = fftz(X, 1);
    if (e != cudaSuccess) return mvfail(GLASMA_ERR_CUDA, std::string("TMD 3D FFT: ") + cudaGetErrorString(e));
    // ---- rho from the nucleus profile (per-nucleon 1D factors of the Gaussian)
    const double* xn = nucleons[k];
    double* ex = tab.data();
    double* ey = ex + (size_t)A * nx;
    double* ez = ey + (size_t)A * ny;
    for (int n = 0; n < A; n++) {
      for (int x = 0; x < nx; x++) {
        const double d = (x - nx / 2) * p.ax_fm - xn[3 * n];
        ex[(size_t)n * nx + x] = std::exp(-0.5 * d * d / kTmdBG);
      }
      for (int y = 0; y < ny; y++) {
        const double d = (y - ny / 2) * p.ay_fm - xn[3 * n + 1];
        ey[(size_t)n * ny + y] = std::exp(-0.5 * d * d / kTmdBG);
      }
      for (int z = 0; z < nz; z++) {
        const double d = gamma * ((z - center) * p.az_fm) - xn[3 * n + 2];
        ez[(size_t)n * nz + z] = gamma * std::exp(-0.5 * d * d / kTmdBG) / std::sqrt(2.0 * M_PI * kTmdBG);
      }
    }
    // pageable source: the table has been taken when the call returns
    if ((e = cudaMemcpyAsync(tabs.p, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, st)) !=
        cudaSuccess)
      return mvfail(GLASMA_ERR_CUDA, std::string("profile upload: ") + cudaGetErrorString(e));
    const double* tb = static_cast<const double*>(tabs.p);
    tmd_rho_kernel<<<g1(vol), 256, 0, st>>>(X, nx, ny, nz, A, tb, tb + (size_t)A * nx, tb + (size_t)A * (nx + ny),
                                            a3 * std::sqrt(p.az_fm / g.a[2]));
    // ---- filtered density (X) and its Poisson field (Y), every slice in one batch
    e = fft2(X, 0);
    split_filter_kernel<<<g1(8 * vol), 256, 0, st>>>(X, Y, 8 * vol, nx, ny, g.a[0], g.a[1], p.meff);
    if (e == cudaSuccess) e = fft2(X, 1);
    if (e == cudaSuccess) e = fft2(Y, 1);
    real_part_kernel<<<g1(8 * vol), 256, 0, st>>>(X, 8 * vol);
    if (e != cudaSuccess) return mvfail(GLASMA_ERR_CUDA, std::string("TMD 2D FFT: ") + cudaGetErrorString(e));
    if (rho_out[k]) {
      pack_density_kernel<<<g1(8 * g.S), 256, 0, st>>>(X, nz, plane, static_cast<double*>(stage.p));
      if ((e = cudaMemcpyAsync(rho_out[k], stage.p, sizeof(double) * 8 * g.S, cudaMemcpyDeviceToHost, st)) !=
          cudaSuccess)
        return mvfail(GLASMA_ERR_CUDA, std::string("density download: ") + cudaGetErrorString(e));
    }
    const int up = D == 'R' ? 1 : 0;
    const double c = D == 'R' ? inv_sqrt2 : -inv_sqrt2;
    path_scan(Y, up, c, V);
    // ---- SingleSheet: the density shifted by dt, its per-slice Poisson field, V'
    {
      std::vector<double2> ph(nz);
      for (int q = 0; q < nz; q++) {
        const double om = std::sqrt((2.0 - 2.0 * std::cos(2.0 * M_PI * (double)q / (double)nz)) / (g.a[2] * g.a[2]));
        const bool low = q < nz / 2;
        const double sgn = D == 'L' ? (low ? -1.0 : 1.0) : (low ? 1.0 : -1.0);
        const std::complex<double> f = std::polar(1.0, sgn * om * p.dt) / (double)nz;
        ph[q] = make_double2(f.real(), f.imag());
      }
      if ((e = cudaMemcpyAsync(filt.p, ph.data(), sizeof(double2) * nz, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return mvfail(GLASMA_ERR_CUDA, std::string("phase upload: ") + cudaGetErrorString(e));
    }
    e = fftz(X, 0);
    zfilter_kernel<<<g1(8 * vol), 256, 0, st>>>(X, vol, plane, nz, static_cast<const double2*>(filt.p));
    if (e == cudaSuccess) e = fftz(X, 1);
    real_part_kernel<<<g1(8 * vol), 256, 0, st>>>(X, 8 * vol);
    if (e == cudaSuccess) e = fft2(X, 0);
    filter2d_kernel<<<g1(8 * vol), 256, 0, st>>>(X, 8 * vol, nx, ny, g.a[0], g.a[1], 1.0, 0.0, 1);
    if (e == cudaSuccess) e = fft2(X, 1);
    if (e != cudaSuccess) return mvfail(GLASMA_ERR_CUDA, std::string("TMD first step: ") + cudaGetErrorString(e));
    path_scan(X, up, c, Vp);
    const double coff0 = -p.dt * g.a[0] * g.a[0] / a3, coff1 = -p.dt * g.a[1] * g.a[1] / a3;
    sheet_links_v_kernel<T><<<g1(plane * (zhi - zlo + 1)), 256, 0, st>>>(
        g, V, Vp, zlo, zhi, coff0, coff1, static_cast<cx<T>*>(h->f[GLASMA_FIELD_U]),
        static_cast<cx<T>*>(h->f[GLASMA_FIELD_UOLD]), static_cast<T*>(h->f[GLASMA_FIELD_E]));
    if ((e = cudaGetLastError()) != cudaSuccess)
      return mvfail(GLASMA_ERR_CUDA, std::string("TMD links: ") + cudaGetErrorString(e));
    const int cst = sheet_currents<T>(h, D, zlo, zhi, p.dt, Y, static_cast<double2*>(twz.p),
                                      static_cast<double2*>(filt.p));
    if (cst != GLASMA_OK) return cst;
    // the staging buffer and the host tables are reused by the next nucleus
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return mvfail(GLASMA_ERR_CUDA, "TMD sync");
  }
  // SimulationmitPC::Run syncs every field afterwards (S/SimulationmitPC.cpp:354-362)
  const int fields[7] = {GLASMA_FIELD_U, GLASMA_FIELD_UOLD, GLASMA_FIELD_E, GLASMA_FIELD_JP, GLASMA_FIELD_JM,
                         GLASMA_FIELD_JPSTAT, GLASMA_FIELD_JMSTAT};
  for (int f : fields) {
    cudaError_t e;
    if (f == GLASMA_FIELD_U || f == GLASMA_FIELD_UOLD)
      e = launch_sync_ghosts<cx<T>>(g, static_cast<cx<T>*>(h->f[f]), 27, st);
    else
      e = launch_sync_ghosts<T>(g, static_cast<T*>(h->f[f]), f == GLASMA_FIELD_E ? 24 : 8, st);
    if (e != cudaSuccess) return mvfail(GLASMA_ERR_CUDA, "ghost sync");
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return mvfail(GLASMA_ERR_CUDA, "TMD sync");
  return GLASMA_OK;
}

extern "C" void glasma_tmd_default_params(glasma_tmd_params* p, double dt) {
  if (!p) return;
  p->atomic_number = 197;
  p->qs0a = 0.33;
  p->meff = p->qs0a;
  p->ax_fm = p->qs0a * 0.197 / 0.5;
  p->ay_fm = p->ax_fm;
  p->az_fm = p->ax_fm * 1.0 / (p->qs0a * 512);
  p->com_energy = 500 / 0.197;
  p->center_left = 785;
  p->center_right = 1261;
  p->dt = dt;
}

extern "C" int glasma_glauber_sample(int A, const double* uniforms, long n_uniforms, double* positions, long* used) {
  double R, s;
  if (used) *used = 0;
  if (!uniforms || !positions || !woods_saxon(A, &R, &s))
    return mvfail(GLASMA_ERR_INVALID_ARGUMENT, "no Woods-Saxon parameters for this A (16, 54, 197, 208)");
  long k = 0;
  // GlauberSamplePosition (S/TMDNUCLEUS/GBWSampling.cpp:20-40): a point of the cube [-4R, 4R)^3, kept with
  // probability (1 + e^{-R/s}) / (1 + e^{(r-R)/s})
  for (int n = 0; n < A; n++) {
    for (;;) {
      if (k + 4 > n_uniforms) {
        if (used) *used = k;
        return mvfail(GLASMA_ERR_INVALID_ARGUMENT, "uniform stream exhausted");
      }
      double* x = positions + 3 * n;
      x[0] = 8.0 * R * (uniforms[k] - 0.5);
      x[1] = 8.0 * R * (uniforms[k + 1] - 0.5);
      x[2] = 8.0 * R * (uniforms[k + 2] - 0.5);
      const double r = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
      const double prob = (1.0 + std::exp(-R / s)) / (1.0 + std::exp((r - R) / s));
      const bool accept = uniforms[k + 3] < prob;
      k += 4;
      if (accept) break;
    }
  }
  // centre of mass to the origin (:62-74), accumulated in the reference's order
  double bar[3] = {0.0, 0.0, 0.0};
  for (int n = 0; n < A; n++)
    for (int d = 0; d < 3; d++) bar[d] += positions[3 * n + d] / double(A);
  for (int n = 0; n < A; n++)
    for (int d = 0; d < 3; d++) positions[3 * n + d] -= bar[d];
  if (used) *used = k;
  return GLASMA_OK;
}

extern "C" int glasma_tmd_init(glasma_lattice* h, const double* noise_left, const double* noise_right,
                               const double* nucleons_left, const double* nucleons_right,
                               const glasma_tmd_params* params, double* rho_left, double* rho_right) {
  using namespace glasma;
  if (!h || !noise_left || !noise_right || !nucleons_left || !nucleons_right || !params)
    return mvfail(GLASMA_ERR_INVALID_ARGUMENT, "null argument");
  const glasma_tmd_params& p = *params;
  double R, s;
  if (!woods_saxon(p.atomic_number, &R, &s))
    return mvfail(GLASMA_ERR_INVALID_ARGUMENT, "no Woods-Saxon parameters for this A (16, 54, 197, 208)");
  if (!(p.qs0a > 0) || !(p.meff > 0) || !(p.ax_fm > 0) || !(p.ay_fm > 0) || !(p.az_fm > 0) || !(p.com_energy > 0) ||
      !(p.dt > 0))
    return mvfail(GLASMA_ERR_INVALID_ARGUMENT, "bad parameters");
  if (cudaSetDevice(h->device) != cudaSuccess) return mvfail(GLASMA_ERR_CUDA, "cudaSetDevice");
  const double* noise[2] = {noise_left, noise_right};
  const double* nuc[2] = {nucleons_left, nucleons_right};
  double* rho[2] = {rho_left, rho_right};
  return h->precision == GLASMA_FP64 ? tmd_impl<double>(h, noise, nuc, p, rho) : tmd_impl<float>(h, noise, nuc, p, rho);
}

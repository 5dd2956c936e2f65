// mvinit.cu -- McLerran-Venugopalan initial conditions on the GPU: colliding nuclei as in
// Simulation::Run (S/Simulation.cpp:337-374), or one left-moving nucleus as in
// S/LeftNucleusSimulation.cpp, built from injected charge fluctuations.
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

// multiply by f(p^2)/(Nx Ny): mode 0 smoothing, mode 1 Poisson (zero mode -> 0); keep the real part
// afterwards is done by the caller
__global__ void filter2d_kernel(double2* X, int nx, int ny, double ax, double ay, double lambda, double meff, int mode) {
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  const L plane = (L)nx * ny;
  if (i >= 8 * plane) return;
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
    filter2d_kernel<<<g1(8 * plane), 256, 0, st>>>(X, nx, ny, g.a[0], g.a[1], lambda, meff, 0);
    if (e == cudaSuccess) e = fft2(X, 1);
    real_part_kernel<<<g1(8 * plane), 256, 0, st>>>(X, 8 * plane);
    if (e == cudaSuccess) e = fft2(X, 0);
    filter2d_kernel<<<g1(8 * plane), 256, 0, st>>>(X, nx, ny, g.a[0], g.a[1], lambda, meff, 1);
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
    const int fstat = nu.D == 'L' ? GLASMA_FIELD_JPSTAT : GLASMA_FIELD_JMSTAT;
    const int fj = nu.D == 'L' ? GLASMA_FIELD_JP : GLASMA_FIELD_JM;
    double2* Z = static_cast<double2*>(zbuf.p);
    sheet_jstat_kernel<T><<<g1(g.vol), 256, 0, st>>>(g, static_cast<const cx<T>*>(h->f[GLASMA_FIELD_U]),
                                                     static_cast<const T*>(h->f[GLASMA_FIELD_E]), nu.zlo, nu.zhi, Z);
    store_real_kernel<T><<<g1(8 * g.vol), 256, 0, st>>>(Z, static_cast<T*>(h->f[fstat]), g.vol, plane, g.S);
    std::vector<double2> fh(nz);
    for (int p = 0; p < nz; p++) {
      const double om = std::sqrt((2.0 - 2.0 * std::cos(2.0 * M_PI * p / nz)) / (g.a[2] * g.a[2]));
      const std::complex<double> zd = (nu.D == 'R' ? 1.0 : -1.0) *
                                      (1.0 - std::polar(1.0, -2.0 * M_PI * (double)p / nz)) / g.a[2];
      const std::complex<double> npos = std::polar(1.0, (nu.D == 'R' ? 1.0 : -1.0) * om * dt) - 1.0;
      const std::complex<double> nneg = std::polar(1.0, (nu.D == 'R' ? -1.0 : 1.0) * om * dt) - 1.0;
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
    cudaMemcpyAsync(filt.p, fh.data(), sizeof(double2) * nz, cudaMemcpyHostToDevice, st);
    e = fft_lines(Z, nz, plane, 8 * g.vol, 0, static_cast<double2*>(twz.p), st);
    zfilter_kernel<<<g1(8 * g.vol), 256, 0, st>>>(Z, g.vol, plane, nz, static_cast<const double2*>(filt.p));
    if (e == cudaSuccess) e = fft_lines(Z, nz, plane, 8 * g.vol, 1, static_cast<double2*>(twz.p), st);
    store_real_kernel<T><<<g1(8 * g.vol), 256, 0, st>>>(Z, static_cast<T*>(h->f[fj]), g.vol, plane, g.S);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return mvfail(GLASMA_ERR_CUDA, std::string("MV currents: ") + cudaGetErrorString(e));
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

// gaugefix.cu -- Fourier-accelerated Coulomb gauge fixing with a hand-written batched 3D FFT.
//
// Follows CoulombGaugeFixing::SetCoulombGauge (S/GAUGETRANSFORMATION/CoulombGaugeFixing.cpp:32-88)
// and FourierAccelerationAlgorithm::UpdateGaugeTransformation
// (S/GAUGETRANSFORMATION/ALGORITHMS/FourierAcceleration.cpp:15-142), per iteration:
//   deviation   w(x) = sum_mu c_mu (UG_mu(x) + UG_mu^d(x-mu)), Delta^a = ReTr(i t^a w)
//               (S/GAUGETRANSFORMATION/CoulombGaugeDeviation.cpp:23-41); z term only if Nz > 1
//   FFT         8 colours, unnormalised, forward sign -1 (FFTW semantics of S/FFT/FFT3D.cpp:126-138)
//   accelerate  Delta(p) <- Delta(p) / (p^2 V) for p^2 > 0; the p = 0 mode is left as it is
//               (optionally projected out: GLASMA_GF_PROJECT_ZERO_MODE)
// With open z boundaries the reference's deviation counts the top slice's forward z link (into the
// ghost slice) at one end only.  Its contribution cannot be gauged away (the ghost G follows the top
// slice, so the link is only conjugated), sum_x Delta(x) is then not zero, and the unnormalised
// p = 0 mode turns it into a global rotation V times too large: the iteration leaves SU(3) (the
// compiled reference exits on its unitarity guard within a few tens of iterations on an evolved MV
// collision).  GLASMA_GF_OPEN_Z leaves that link out of the deviation, which makes Delta the gradient
// of sum Re tr UG over the links inside the lattice; sum_x Delta(x) is then zero up to rounding and
// the iteration converges (documented variant; the reference's iteration stays the default).
//   inverse FFT
//   update      wt = exp(-i alpha t.Re Delta), guard ||wt wt^d - 1|| <= 1e-13, G <- wt^d G
//   transform   UG_mu(x) = G(x) U_mu(x) G^d(x+mu), reading the ghost G(x,y,Nz) before the ghost
//               sync, as GaugeTransformLinks does (S/GAUGETRANSFORMATION/GaugeTransformation.cpp:111-124)
// The ghost slices of UG are never written (the reference's gauge-fixed container keeps the
// identity it was created with), so the backward z link at z = 0 is the identity.
//
// The Los Alamos and Jacobi updates that the reference compiles beside the Fourier one
// (S/GAUGETRANSFORMATION/ALGORITHMS/LosAlamos.cpp, Jacobi.cpp) run through the same loop with a
// local update in place of the FFT steps: local_update_kernel, one launch per checkerboard pass.
//
// All arithmetic is FP64 (G / UG / EG are stored in the handle's precision), except that with
// GLASMA_GF_FFT_FP32 the two transforms of the acceleration step run in FP32: they only
// precondition the step, so the iteration still converges to the same gauge, measured in FP64.
//
// FFT: the gradient Delta^a is real, so colours (2q, 2q+1) travel as one complex plane
// X[q] = Delta^{2q} + i Delta^{2q+1}: four complex 3D transforms per direction instead of the
// reference's eight (the real factor, even in p, keeps the two colours apart on the way back).
// A 3D transform is three passes of batched 1D transforms along x, y and z over X[q][z][y][x].
// A block stages a tile of lines in shared memory (consecutive lines for the x pass; for the y
// and z passes a tile of consecutive x, so every global access is a contiguous run), transforms it
// there and writes it back in place: radix-2 decimation in time for power-of-two lengths, a
// mixed-radix Stockham transform (radices 4, 2, 3, 5, other primes directly) otherwise.  On GB300 the FP64 transform is bound by the FP64 pipe, not by HBM.
#include <map>
#include <vector>

#include "../../include/glasma_gb300.h"
#include "gaugefix.h"
#include "reduce.cuh"

namespace glasma {

namespace {

constexpr int kGfThreads = red::kThreads;
constexpr int kGfBlocks = 1216;
constexpr int kFftThreads = 256;
constexpr int kFftMaxTile = 4096;  // complex doubles staged per block (64 KB)
constexpr size_t kFftMaxSmem = 227 * 1024;  // shared memory a block may opt into
// Build knob: power-of-two lengths through the mixed-radix Stockham kernel (radix 4) instead of the
// radix-2 kernel.
#ifndef GLASMA_FFT_POW2_STOCKHAM
#define GLASMA_FFT_POW2_STOCKHAM 0
#endif

inline unsigned blocks_for(long long n, int threads, int cap) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  return (unsigned)(b < cap ? b : cap);
}

template <typename T>
__device__ __forceinline__ void ld_d(const cx<T>* __restrict__ U, long long S, long long comp0, long long s, Mat<double>& m) {
  const cx<T>* p = U + comp0 * S + s;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const cx<T> v = p[(long long)k * S];
    m.e[k] = mk<double>((double)v.re, (double)v.im);
  }
}
template <typename T>
__device__ __forceinline__ void st_d(cx<T>* __restrict__ U, long long S, long long comp0, long long s, const Mat<double>& m) {
  cx<T>* p = U + comp0 * S + s;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    cx<T> v;
    v.re = (T)m.e[k].re;
    v.im = (T)m.e[k].im;
    p[(long long)k * S] = v;
  }
}

__device__ __forceinline__ double2 cmk(double r, double i) { return make_double2(r, i); }
__device__ __forceinline__ float2 cmk(float r, float i) { return make_float2(r, i); }

__device__ __forceinline__ long long nbr(const Geometry& g, int x, int y, int z, int dx, int dy, int dz) {
  int xx = x + dx, yy = y + dy;
  xx = xx < 0 ? xx + g.nx : (xx >= g.nx ? xx - g.nx : xx);
  yy = yy < 0 ? yy + g.ny : (yy >= g.ny ? yy - g.ny : yy);
  return site_index(g, xx, yy, z + dz);
}

// (x, y, z) of index idx = x + nx (y + ny z), in 32-bit arithmetic when every index fits: a 64-bit
// integer division here kept the FP32 acceleration kernel's FP64 pipe 30 % busy on GB300 (ncu), and the
// FP64 kernels are bound by that pipe
__device__ __forceinline__ void gf_decode(long long idx, int nx, int ny, long long total, int& x, int& y, int& z) {
  if (total < (1LL << 31)) {
    const unsigned u = (unsigned)idx, r = u / (unsigned)nx;
    x = (int)(u - r * (unsigned)nx);
    z = (int)(r / (unsigned)ny);
    y = (int)(r - (unsigned)z * (unsigned)ny);
  } else {
    const long long r = idx / nx;
    x = (int)(idx - r * nx);
    z = (int)(r / ny);
    y = (int)(r - (long long)z * ny);
  }
}

// w(x) = sum_mu c_mu (UG_mu(x) + UG_mu^d(x - mu)) at interior site s = (x, y, z); c2 = 0 when Nz = 1
// (GET_LOCAL_GAUGE_VIOLATION, S/GAUGETRANSFORMATION/CoulombGaugeDeviation.cpp:23-41).
// open_top (GLASMA_GF_OPEN_Z): the forward z link of the top slice, which points into the ghost slice,
// is left out, so that every link in w is counted at both of its ends (the backward z link of slice 0
// is the identity ghost, which adds nothing to Delta) and Delta is the gradient of one functional.
template <typename T>
__device__ __forceinline__ void site_w(const Geometry& g, const cx<T>* UG, int x, int y, int z, long long s, double c0,
                                       double c1, double c2, Mat<double>& w, int open_top = 0) {
  const double c[3] = {c0, c1, c2};
  const long long back[3] = {nbr(g, x, y, z, -1, 0, 0), nbr(g, x, y, z, 0, -1, 0), s - g.plane};
  const double fwd2 = (open_top && z == g.nz - 1) ? 0.0 : 1.0;
  set_zero(w);
  for (int mu = 0; mu < 3; mu++) {
    if (c[mu] == 0.0) continue;
    const double cf = mu == 2 ? fwd2 : 1.0;
    Mat<double> u, d;
    ld_d(UG, g.S, mu * 9, s, u);
    ld_d(UG, g.S, mu * 9, back[mu], d);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const int k = i + 3 * j, kt = j + 3 * i;
        w.e[k].re += c[mu] * (cf * u.e[k].re + d.e[kt].re);
        w.e[k].im += c[mu] * (cf * u.e[k].im - d.e[kt].im);
      }
  }
}

// ---- deviation: X[q] = Delta^{2q} + i Delta^{2q+1}, q < 4 (Delta is real: two colours share one
// complex transform, and since the acceleration multiplies by a real factor even in p, the inverse
// transform returns them in the real and imaginary parts); partials {max|Delta|, sum Delta^2,
// min ReTr w, sum ReTr w}
template <typename T, typename C>
__global__ void __launch_bounds__(kGfThreads) deviation_kernel(Geometry g, const cx<T>* UG, double c0, double c1,
                                                               double c2, C* X, double* partials, int open_top) {
  double v[4] = {0.0, 0.0, 1.0e300, 0.0};
  const int op[4] = {1, 0, 2, 0};
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < g.vol;
       idx += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    gf_decode(idx, g.nx, g.ny, g.vol, x, y, z);
    const long long s = idx + g.plane;
    Mat<double> w;
    site_w(g, UG, x, y, z, s, c0, c1, c2, w, open_top);
    Alg<double> dev;
    retr_itg(w, 1.0, dev);
#pragma unroll
    for (int a = 0; a < 8; a++) {
      v[0] = fmax(v[0], fabs(dev.a[a]));
      v[1] += dev.a[a] * dev.a[a];
    }
#pragma unroll
    for (int q = 0; q < 4; q++)
      X[(long long)q * g.vol + idx] = cmk((decltype(C::x))dev.a[2 * q], (decltype(C::x))dev.a[2 * q + 1]);
    const double lf = w.e[0].re + w.e[4].re + w.e[8].re;
    v[2] = fmin(v[2], lf);
    v[3] += lf;
  }
  red::block_reduce_store<4>(v, op, partials + (long long)blockIdx.x * 4);
}

// ---- momentum-space acceleration of the 4 colour-pair planes
// lattice momenta per axis, (2 - 2 cos(2 pi k / n)) / a^2 for k < n: tab[0 .. nx), then ny, then nz
__global__ void p2_table_kernel(int nx, int ny, int nz, double ax, double ay, double az, double* tab) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nx)
    tab[i] = (2.0 - 2.0 * cospi(2.0 * i / (double)nx)) / (ax * ax);
  else if (i < nx + ny)
    tab[i] = (2.0 - 2.0 * cospi(2.0 * (i - nx) / (double)ny)) / (ay * ay);
  else if (i < nx + ny + nz)
    tab[i] = (2.0 - 2.0 * cospi(2.0 * (i - nx - ny) / (double)nz)) / (az * az);
}
// p^2 from the per-axis table: the same three terms summed in the same order as evaluating them here,
// without three FP64 cosines per element on GB300's FP64 pipe
__global__ void narrow_table_kernel(const double* __restrict__ tab, float* __restrict__ tab32, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) tab32[i] = (float)tab[i];
}
// FP32 planes (FP32 transforms, the FP32 sweeps): the factor in FP32 from an FP32 table, so that no
// element costs an FP64 division and FP64 products on GB300's FP64 pipe
__global__ void accelerate32_kernel(int nx, int ny, int nz, float vf, const float* __restrict__ tab, float2* X,
                                    int project_zero) {
  const long long V = (long long)nx * ny * nz;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 4 * V) return;
  int px, py, pz;
  gf_decode(i, nx, ny * nz, 4 * V, px, py, pz);  // (x, y + ny z, plane): the plane index is not needed
  pz = py / ny;
  py -= pz * ny;
  const float p2 = tab[px] + tab[nx + py] + tab[nx + ny + pz];
  if (p2 > 0.f) {
    const float f = 1.f / (vf * p2);
    float2 v = X[i];
    v.x *= f;
    v.y *= f;
    X[i] = v;
  } else if (project_zero) {
    X[i] = make_float2(0.f, 0.f);
  }
}
template <typename C>
__global__ void accelerate_kernel(int nx, int ny, int nz, double vd, const double* __restrict__ tab, C* X,
                                  int project_zero) {
  const long long V = (long long)nx * ny * nz;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 4 * V) return;
  int px, py, pz;
  gf_decode(i, nx, ny * nz, 4 * V, px, py, pz);  // (x, y + ny z, plane)
  pz = py / ny;
  py -= pz * ny;
  const double p2 = tab[px] + tab[nx + py] + tab[nx + ny + pz];
  if (p2 > 0.0) {
    const double f = 1.0 / (vd * p2);
    C v = X[i];
    v.x *= f;
    v.y *= f;
    X[i] = v;
  } else if (project_zero) {
    X[i] = cmk((decltype(C::x))0, (decltype(C::x))0);
  }
}

// ---- update of G; partials {max step, sum step^2, guard count}
template <typename T, typename C>
__global__ void __launch_bounds__(kGfThreads) update_kernel(Geometry g, const C* X, cx<T>* G, double alpha,
                                                            double* partials) {
  double v[3] = {0.0, 0.0, 0.0};
  const int op[3] = {1, 0, 0};
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < g.vol;
       idx += (long long)gridDim.x * blockDim.x) {
    Alg<double> upd;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const C v = X[(long long)q * g.vol + idx];
      upd.a[2 * q] = (double)v.x;
      upd.a[2 * q + 1] = (double)v.y;
    }
    Mat<double> wt, gm, gn;
    expi(-alpha, upd, wt);
    // the reference's guard (CoulombGaugeDeviation.cpp:57-68); written so that a NaN also trips it
    if (!(unitarity_norm(wt) <= 1e-13)) v[2] += 1.0;
    const double sr = 3.0 - wt.e[0].re - wt.e[4].re - wt.e[8].re, si = -(wt.e[0].im + wt.e[4].im + wt.e[8].im);
    const double step = sqrt(sr * sr + si * si);
    v[0] = fmax(v[0], step);
    v[1] += step * step;
    const long long s = idx + g.plane;
    ld_d(G, g.S, 0, s, gm);
    mul_dn(wt, gm, gn);
    st_d(G, g.S, 0, s, gn);
  }
  red::block_reduce_store<3>(v, op, partials + (long long)blockIdx.x * 3);
}

// ---- mixed-precision sweeps (GLASMA_GF_MIXED, FP64 handles): the Fourier-accelerated iteration on
// FP32 copies of U and G with FP32 arithmetic (GB300 runs FP32 at 64x its FP64 rate) until the FP32
// deviation reaches its rounding floor; the monitors' sums and extrema stay FP64.  Then G is widened,
// projected back onto SU(3) in FP64, and the FP64 iteration makes the final sweeps.
__device__ __forceinline__ void ld_f(const cx<float>* __restrict__ U, long long S, long long comp0, long long s,
                                     Mat<float>& m) {
  const cx<float>* p = U + comp0 * S + s;
#pragma unroll
  for (int k = 0; k < 9; k++) m.e[k] = p[(long long)k * S];
}
__device__ __forceinline__ void st_f(cx<float>* __restrict__ U, long long S, long long comp0, long long s,
                                     const Mat<float>& m) {
  cx<float>* p = U + comp0 * S + s;
#pragma unroll
  for (int k = 0; k < 9; k++) p[(long long)k * S] = m.e[k];
}

__global__ void narrow_kernel(const cx<double>* __restrict__ src, cx<float>* __restrict__ dst, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const cx<double> v = src[i];
  dst[i] = mk<float>((float)v.re, (float)v.im);
}

// UG_mu(x) = G(x) U_mu(x) G^d(x+mu) in FP32, interior sites
__global__ void __launch_bounds__(128) transform_links32_kernel(Geometry g, const cx<float>* U, const cx<float>* G,
                                                                cx<float>* UG) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.vol) return;
  int x, y, z;
  gf_decode(idx, g.nx, g.ny, g.vol, x, y, z);
  const long long s = idx + g.plane;
  const long long fwd[3] = {nbr(g, x, y, z, 1, 0, 0), nbr(g, x, y, z, 0, 1, 0), s + g.plane};
  Mat<float> gx, u, gy, t, o;
  ld_f(G, g.S, 0, s, gx);
  for (int mu = 0; mu < 3; mu++) {
    ld_f(U, g.S, mu * 9, s, u);
    ld_f(G, g.S, 0, fwd[mu], gy);
    mul_nn(gx, u, t);
    mul_nd(t, gy, o);
    st_f(UG, g.S, mu * 9, s, o);
  }
}

// deviation_kernel in FP32 (site_w's sum, the projection and X); partials in FP64
__global__ void __launch_bounds__(kGfThreads) deviation32_kernel(Geometry g, const cx<float>* UG, float c0, float c1,
                                                                 float c2, float2* X, double* partials, int open_top) {
  // each thread's sites summed in FP32 (a few dozen terms), the block and grid sums in FP64: FP64
  // arithmetic and conversions run on GB300's slow FP64 pipe, which this kernel then leaves alone
  double v[4];
  float tmax = 0.f, tsq = 0.f, tmin = 3.0e38f, tlf = 0.f;
  const int op[4] = {1, 0, 2, 0};
  const float c[3] = {c0, c1, c2};
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < g.vol;
       idx += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    gf_decode(idx, g.nx, g.ny, g.vol, x, y, z);
    const long long s = idx + g.plane;
    const long long back[3] = {nbr(g, x, y, z, -1, 0, 0), nbr(g, x, y, z, 0, -1, 0), s - g.plane};
    const float fwd2 = (open_top && z == g.nz - 1) ? 0.f : 1.f;
    Mat<float> w;
    set_zero(w);
    for (int mu = 0; mu < 3; mu++) {
      if (c[mu] == 0.f) continue;
      const float cf = mu == 2 ? fwd2 : 1.f;
      Mat<float> u, d;
      ld_f(UG, g.S, mu * 9, s, u);
      ld_f(UG, g.S, mu * 9, back[mu], d);
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
          const int k = i + 3 * j, kt = j + 3 * i;
          w.e[k].re += c[mu] * (cf * u.e[k].re + d.e[kt].re);
          w.e[k].im += c[mu] * (cf * u.e[k].im - d.e[kt].im);
        }
    }
    Alg<float> dev;
    retr_itg(w, 1.f, dev);
#pragma unroll
    for (int a = 0; a < 8; a++) {
      tmax = fmaxf(tmax, fabsf(dev.a[a]));
      tsq = fmaf(dev.a[a], dev.a[a], tsq);
    }
#pragma unroll
    for (int q = 0; q < 4; q++) X[(long long)q * g.vol + idx] = make_float2(dev.a[2 * q], dev.a[2 * q + 1]);
    const float lf = w.e[0].re + w.e[4].re + w.e[8].re;
    tmin = fminf(tmin, lf);
    tlf += lf;
  }
  v[0] = tmax;
  v[1] = tsq;
  v[2] = tmin;
  v[3] = tlf;
  red::block_reduce_store<4>(v, op, partials + (long long)blockIdx.x * 4);
}

// update_kernel in FP32.  The unitarity guard cannot hold FP64's 1e-13 here (an FP32 exponential is
// unitary to ~1e-7): it trips at `guard`, which still catches the runaway the reference's guard exists for.
__global__ void __launch_bounds__(kGfThreads) update32_kernel(Geometry g, const float2* X, cx<float>* G, float alpha,
                                                              double* partials, float guard) {
  // per-thread sums in FP32, block and grid sums in FP64 (as deviation32_kernel)
  double v[3];
  float tmax = 0.f, tsq = 0.f, tbad = 0.f;
  const int op[3] = {1, 0, 0};
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < g.vol;
       idx += (long long)gridDim.x * blockDim.x) {
    Alg<float> upd;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const float2 x = X[(long long)q * g.vol + idx];
      upd.a[2 * q] = x.x;
      upd.a[2 * q + 1] = x.y;
    }
    Mat<float> wt, gm, gn;
    expi(-alpha, upd, wt);
    if (!(unitarity_norm(wt) <= guard)) tbad += 1.f;
    const float sr = 3.f - wt.e[0].re - wt.e[4].re - wt.e[8].re, si = -(wt.e[0].im + wt.e[4].im + wt.e[8].im);
    const float step2 = sr * sr + si * si;
    tmax = fmaxf(tmax, sqrtf(step2));
    tsq += step2;
    const long long s = idx + g.plane;
    ld_f(G, g.S, 0, s, gm);
    mul_dn(wt, gm, gn);
    st_f(G, g.S, 0, s, gn);
  }
  v[0] = tmax;
  v[1] = tsq;
  v[2] = tbad;
  red::block_reduce_store<3>(v, op, partials + (long long)blockIdx.x * 3);
}

// G = the SU(3) projection (FP64 Newton, reunitarize_newton) of the widened FP32 G, every site
__global__ void widen_gauge_kernel(const cx<float>* __restrict__ G32, cx<double>* __restrict__ G, long long S) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  Mat<double> m;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const cx<float> v = G32[(long long)k * S + s];
    m.e[k] = mk<double>((double)v.re, (double)v.im);
  }
  reunitarize_newton(m);
#pragma unroll
  for (int k = 0; k < 9; k++) G[(long long)k * S + s] = m.e[k];
}

// ---- local updates: Los Alamos (LosAlamos.cpp:13-95) and Jacobi (Jacobi.cpp:13-80)
// The over-relaxation draw of one site of one checkerboard pass: splitmix64's finaliser (Steele, Lea &
// Flood, OOPSLA 2014) over (seed, 2 * iteration + pass, site), uniform in [0, 1).  Counter-based, so
// the draw does not depend on the order in which threads visit the sites.
__device__ __forceinline__ unsigned long long gf_mix(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double gf_uniform(unsigned long long seed, int iteration, int pass, long long site) {
  const unsigned long long k = gf_mix(seed ^ gf_mix((unsigned long long)(2LL * iteration + pass)));
  return (double)(gf_mix(k ^ (unsigned long long)site) >> 11) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ cx<double> cmul(const cx<double>& a, const cx<double>& b) {
  return mk<double>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
// One Cabibbo-Marinari step in the SU(2) subgroup of rows/columns (p, q)
// (S/SUNc/SU3/util/CabbiboMarinariProjection.cpp:4-62, step :73-92): the subgroup element
//   A_pp = (V_pp^* + V_qq)/n, A_pq = (V_qp^* - V_pq)/n, A_qp = (V_pq^* - V_qp)/n, A_qq = (V_qq^* + V_pp)/n
// multiplies Gc and V from the left; only their rows p and q change.
template <int p, int q>
__device__ __forceinline__ void cm_subgroup(Mat<double>& Gc, Mat<double>& V) {
  const cx<double> vpp = V.e[p + 3 * p], vqq = V.e[q + 3 * q], vpq = V.e[p + 3 * q], vqp = V.e[q + 3 * p];
  const cx<double> s = mk<double>(vpp.re + vqq.re, vqq.im - vpp.im);
  const cx<double> t = mk<double>(vqp.re - vpq.re, -vqp.im - vpq.im);
  const double inv = 1.0 / sqrt(s.re * s.re + s.im * s.im + (t.re * t.re + t.im * t.im));
  const cx<double> App = mk<double>(inv * s.re, inv * s.im), Apq = mk<double>(inv * t.re, inv * t.im);
  const cx<double> Aqp = mk<double>(inv * (vpq.re - vqp.re), inv * (-vpq.im - vqp.im));
  const cx<double> Aqq = mk<double>(inv * (vqq.re + vpp.re), inv * (vpp.im - vqq.im));
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const cx<double> gp = Gc.e[p + 3 * j], gq = Gc.e[q + 3 * j];
    const cx<double> a = cmul(App, gp), b = cmul(Apq, gq), c = cmul(Aqp, gp), d = cmul(Aqq, gq);
    Gc.e[p + 3 * j] = mk<double>(a.re + b.re, a.im + b.im);
    Gc.e[q + 3 * j] = mk<double>(c.re + d.re, c.im + d.im);
    const cx<double> vp = V.e[p + 3 * j], vq = V.e[q + 3 * j];
    const cx<double> e = cmul(App, vp), f = cmul(Apq, vq), h = cmul(Aqp, vp), k = cmul(Aqq, vq);
    V.e[p + 3 * j] = mk<double>(e.re + f.re, e.im + f.im);
    V.e[q + 3 * j] = mk<double>(h.re + k.re, h.im + k.im);
  }
}
// SUNcGroup::Extended::MaxTraceProjection (S/SUNc/SU3/GroupOperations.cpp:358-378): seven sweeps over
// the subgroups (0,1), (0,2), (1,2); returns Gc^d, Gc the accumulated product (it maximises Re tr(Gc w)).
__device__ __forceinline__ void max_trace_projection(const Mat<double>& w, Mat<double>& out) {
  Mat<double> Gc, V = w;
#pragma unroll
  for (int k = 0; k < 9; k++) Gc.e[k] = mk<double>(k % 4 == 0 ? 1.0 : 0.0, 0.0);
#pragma unroll 1
  for (int n = 0; n < 7; n++) {
    cm_subgroup<0, 1>(Gc, V);
    cm_subgroup<0, 2>(Gc, V);
    cm_subgroup<1, 2>(Gc, V);
  }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) out.e[i + 3 * j] = mk<double>(Gc.e[j + 3 * i].re, -Gc.e[j + 3 * i].im);
}

// One pass of a local update over the sites of one checkerboard parity (pass 0 / 1, Los Alamos) or over
// every site (pass -1, Jacobi).  A parity pass enumerates half-rows: slot k of row (y, z) is
// x = ((pass + y + z) & 1) + 2k, so a warp's lanes all hold sites of the pass.  Each site reads only
// the transformed links UG and writes only its own G, so the sites of a pass are independent.
// partials {max|Delta|, sum Delta^2, min ReTr w, sum ReTr w, max step, sum step^2, guard count}
template <typename T>
__global__ void __launch_bounds__(kGfThreads) local_update_kernel(Geometry g, const cx<T>* UG, cx<T>* G, double c0,
                                                                  double c1, double c2, int los_alamos, int pass,
                                                                  double param, unsigned long long seed, int iteration,
                                                                  double* partials) {
  double v[7] = {0.0, 0.0, 1.0e300, 0.0, 0.0, 0.0, 0.0};
  const int op[7] = {1, 0, 2, 0, 1, 0, 0};
  const int hx = pass < 0 ? g.nx : (g.nx + 1) >> 1;
  const long long n = (long long)hx * g.ny * g.nz;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    int k, y, z;
    gf_decode(idx, hx, g.ny, n, k, y, z);
    const int x = pass < 0 ? k : (((pass + y + z) & 1) + 2 * k);
    if (x >= g.nx) continue;
    const long long s = site_index(g, x, y, z);
    Mat<double> w, wt, gm, gn;
    site_w(g, UG, x, y, z, s, c0, c1, c2, w);
    Alg<double> dev;
    retr_itg(w, 1.0, dev);
#pragma unroll
    for (int a = 0; a < 8; a++) {
      v[0] = fmax(v[0], fabs(dev.a[a]));
      v[1] += dev.a[a] * dev.a[a];
    }
    const double lf = w.e[0].re + w.e[4].re + w.e[8].re;
    v[2] = fmin(v[2], lf);
    v[3] += lf;
    if (los_alamos)
      max_trace_projection(w, wt);
    else
      expi(-param, dev, wt);
    // the reference's guard (CoulombGaugeDeviation.cpp:57-68); written so that a NaN also trips it
    if (!(unitarity_norm(wt) <= 1e-13)) v[6] += 1.0;
    const double sr = 3.0 - wt.e[0].re - wt.e[4].re - wt.e[8].re, si = -(wt.e[0].im + wt.e[4].im + wt.e[8].im);
    const double step = sqrt(sr * sr + si * si);
    v[4] = fmax(v[4], step);
    v[5] += step * step;
    ld_d(G, g.S, 0, s, gm);
    if (los_alamos && !(gf_uniform(seed, iteration, pass, s - g.plane) > param)) {
      Mat<double> t;
      mul_dd(wt, wt, t);  // over-relaxation, DDU (S/SUNc/AdvancedOperations.cpp:119-131)
      mul_nn(t, gm, gn);
    } else {
      mul_dn(wt, gm, gn);  // DU (S/SUNc/SU3/GroupOperations.cpp:166-180)
    }
    st_d(G, g.S, 0, s, gn);
  }
  red::block_reduce_store<7>(v, op, partials + (long long)blockIdx.x * 7);
}

// ---- UG_mu(x) = G(x) U_mu(x) G^d(x+mu), interior sites
template <typename T>
__global__ void __launch_bounds__(128) transform_links_kernel(Geometry g, const cx<T>* U, const cx<T>* G, cx<T>* UG) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.vol) return;
  int x, y, z;
  gf_decode(idx, g.nx, g.ny, g.vol, x, y, z);
  const long long s = idx + g.plane;
  const long long fwd[3] = {nbr(g, x, y, z, 1, 0, 0), nbr(g, x, y, z, 0, 1, 0), s + g.plane};
  Mat<double> gx, u, gy, t, o;
  ld_d(G, g.S, 0, s, gx);
  for (int mu = 0; mu < 3; mu++) {
    ld_d(U, g.S, mu * 9, s, u);
    ld_d(G, g.S, 0, fwd[mu], gy);
    mul_nn(gx, u, t);
    mul_nd(t, gy, o);
    st_d(UG, g.S, mu * 9, s, o);
  }
}

// ---- EG_mu(x) = G(x) E_mu(x) G^d(x)
template <typename T>
__global__ void __launch_bounds__(128) transform_efield_kernel(Geometry g, const T* E, const cx<T>* G, T* EG) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.vol) return;
  const long long s = idx + g.plane;
  Mat<double> gx;
  ld_d(G, g.S, 0, s, gx);
  for (int mu = 0; mu < 3; mu++) {
    Alg<double> e, o;
#pragma unroll
    for (int a = 0; a < 8; a++) e.a[a] = (double)E[(long long)(mu * 8 + a) * g.S + s];
    adj_mul(gx, e, o);
#pragma unroll
    for (int a = 0; a < 8; a++) EG[(long long)(mu * 8 + a) * g.S + s] = (T)o.a[a];
  }
}

// ---- jG(x) = G(x) j(x) G^d(x): PERFORM_COLOR_CHARGE_TRANSFORMATION (S/CALC/GaugeTransformation.cpp:28-31),
// the per-component action of PERFORM_COLOR_CURRENT_TRANSFORMATION (:20-25).  One thread per site of
// the host layout; a ghost site takes the transformed value of the edge slice it mirrors.
template <typename T>
__global__ void __launch_bounds__(128) transform_charge_kernel(Geometry g, const T* J, const cx<T>* G, double* out) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= g.S) return;
  const long long top = g.plane * (g.nz + 1);
  const long long si = s < g.plane ? s + g.plane : (s >= top ? s - g.plane : s);
  Mat<double> gx;
  ld_d(G, g.S, 0, si, gx);
  Alg<double> j, o;
#pragma unroll
  for (int a = 0; a < 8; a++) j.a[a] = (double)J[(long long)a * g.S + si];
  adj_mul(gx, j, o);
#pragma unroll
  for (int a = 0; a < 8; a++) out[s * 8 + a] = o.a[a];
}

// ---- FFT
__global__ void twiddle_kernel(double2* tw, int n, int count) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  double s, c;
  sincospi(-2.0 * (double)k / (double)n, &s, &c);
  tw[k] = make_double2(c, s);
}
__global__ void twiddle_narrow_kernel(const double2* tw, float2* out, int count) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < count) out[k] = make_float2((float)tw[k].x, (float)tw[k].y);
}

// Radix-2 decimation in time over a tile of 2^log_tl lines of length 2^logn staged in shared
// memory, with the twiddles (rows padded to n+1 values against bank conflicts).  Element k of
// line t of tile `tile`:
//   st == 1 : X[base + t*n + k],  base = tile * 2^log_tl * n            (consecutive lines)
//   st  > 1 : X[base + t + k*st], base = o*st*n + i0, (o, i0) from tile (consecutive inner index)
// so every global access is a contiguous run.  Shifts only: n and the tile height are powers of 2.
template <typename C>
__global__ void __launch_bounds__(kFftThreads) fft_pow2_kernel(C* X, int logn, long long st, int log_tl,
                                                               long long tiles_per_row, const C* __restrict__ tw,
                                                               int inverse) {
  extern __shared__ __align__(16) unsigned char fft_smem[];
  const int n = 1 << logn, half_n = n >> 1, tl = 1 << log_tl, pitch = n + 1;
  C* tws = reinterpret_cast<C*>(fft_smem);
  C* sm = tws + half_n;
  for (int k = threadIdx.x; k < half_n; k += blockDim.x) {
    C w = tw[k];
    if (inverse) w.y = -w.y;
    tws[k] = w;
  }
  const long long tile = blockIdx.x;
  long long base, lstride, kstride;
  if (st == 1) {
    base = (tile << log_tl) << logn;
    lstride = n;
    kstride = 1;
  } else {
    const long long o = tile / tiles_per_row;
    base = o * st * n + ((tile - o * tiles_per_row) << log_tl);
    lstride = 1;
    kstride = st;
  }
  const int total = tl << logn;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int t, k;
    if (st == 1) {
      t = idx >> logn;
      k = idx & (n - 1);
    } else {
      t = idx & (tl - 1);
      k = idx >> log_tl;
    }
    const int rk = (int)(__brev((unsigned)k) >> (32 - logn));
    sm[t * pitch + rk] = X[base + t * lstride + k * kstride];
  }
  __syncthreads();
  const int nbfly = tl << (logn - 1);
  // stage 1: every twiddle is 1
  for (int j = threadIdx.x; j < nbfly; j += blockDim.x) {
    const int t = j >> (logn - 1), b = j & (half_n - 1);
    const int i0 = t * pitch + 2 * b, i1 = i0 + 1;
    const C a = sm[i0], c = sm[i1];
    sm[i0] = cmk(a.x + c.x, a.y + c.y);
    sm[i1] = cmk(a.x - c.x, a.y - c.y);
  }
  __syncthreads();
  for (int s = 2; s <= logn; s++) {
    const int hs = s - 1;
    for (int j = threadIdx.x; j < nbfly; j += blockDim.x) {
      const int t = j >> (logn - 1), b = j & (half_n - 1);
      const int grp = b >> hs, pos = b & ((1 << hs) - 1);
      const int i0 = t * pitch + (grp << s) + pos, i1 = i0 + (1 << hs);
      const C w = tws[pos << (logn - s)];
      const C a = sm[i0], c = sm[i1];
      const auto tr = w.x * c.x - w.y * c.y, ti = w.x * c.y + w.y * c.x;
      sm[i0] = cmk(a.x + tr, a.y + ti);
      sm[i1] = cmk(a.x - tr, a.y - ti);
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int t, k;
    if (st == 1) {
      t = idx >> logn;
      k = idx & (n - 1);
    } else {
      t = idx & (tl - 1);
      k = idx >> log_tl;
    }
    X[base + t * lstride + k * kstride] = sm[t * pitch + k];
  }
}

// Element (line l, k) of a batch of 1D transforms of length n, stride st (mixed-radix path):
//   st == 1 : l*n + k
//   st  > 1 : o*st*n + i + k*st  with l = (o, i), i in [0, st)
__device__ __forceinline__ long long fft_addr(long long tile, int t, int k, int n, long long st, int tile_lines) {
  if (st == 1) return (tile * tile_lines + t) * (long long)n + k;
  const long long tiles_per_block = st / tile_lines;
  const long long o = tile / tiles_per_block;
  const long long i = (tile - o * tiles_per_block) * tile_lines + t;
  return o * st * n + i + (long long)k * st;
}

// The radices of a mixed-radix transform of length n = radix[0] * radix[1] * ...: fours first, then
// two, three, five, then the remaining prime factors (each done as a direct DFT of its length).
struct FftPlan {
  int nstages;
  int radix[24];
};

template <typename C>
__device__ __forceinline__ C cmul_c(const C& a, const C& w) {
  return cmk(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x);
}
// -i z (forward) or +i z (inverse) as sgn * (z.y, -z.x) with sgn = +1 / -1
template <typename C, typename R>
__device__ __forceinline__ C rot_i(const C& z, R sgn) {
  return cmk(sgn * z.y, -sgn * z.x);
}

// Mixed-radix Stockham transform (self-sorting, no bit reversal) of a tile of lines of length n in
// shared memory, ping-ponging between two buffers; one stage per radix R of the plan.  Stage with
// Ns = product of the earlier radices, butterfly j < n/R of a line:
//   v_r = in[j + r n/R] * w^(r (j mod Ns) n/(Ns R)),  r < R            (w = exp(-+2 pi i / n))
//   out[(j / Ns) Ns R + (j mod Ns) + q Ns] = sum_r v_r exp(-+2 pi i r q / R),  q < R
// (the Stockham formulation of, e.g., Govindaraju et al., SC 2008), with hand-written butterflies
// for R = 2, 3, 4, 5 and the direct sum for other primes.  tw[k] = exp(-2 pi i k / n), k < n.
template <typename C>
__global__ void __launch_bounds__(kFftThreads) fft_mixed_kernel(C* X, int n, long long st, int tile_lines,
                                                                const C* __restrict__ tw,
                                                                const __grid_constant__ FftPlan plan, int inverse) {
  using R = decltype(C::x);
  extern __shared__ __align__(16) unsigned char fft_smem[];
  C* a = reinterpret_cast<C*>(fft_smem);
  C* b = a + tile_lines * n;
  const long long tile = blockIdx.x;
  const int total = tile_lines * n;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int t = st == 1 ? idx / n : idx % tile_lines;
    const int k = st == 1 ? idx - t * n : idx / tile_lines;
    a[t * n + k] = X[fft_addr(tile, t, k, n, st, tile_lines)];
  }
  __syncthreads();
  const R sgn = inverse ? R(-1) : R(1);  // the sign of -i in the butterflies
  int Ns = 1;
  for (int s = 0; s < plan.nstages; s++) {
    const int rad = plan.radix[s];
    const int nb = n / rad;
    const int tstep = n / (Ns * rad);
    for (int idx = threadIdx.x; idx < tile_lines * nb; idx += blockDim.x) {
      const int t = idx / nb, j = idx - t * nb;
      const int jm = j % Ns;
      const C* src = a + t * n + j;
      C* dst = b + t * n + (j - jm) * rad + jm;
      auto twd = [&](int r) {  // w^(r jm tstep), conjugated for the inverse
        C w = tw[(int)(((long long)r * jm * tstep) % n)];
        if (inverse) w.y = -w.y;
        return w;
      };
      if (rad == 2) {
        const C v0 = src[0], v1 = cmul_c(src[nb], twd(1));
        dst[0] = cmk(v0.x + v1.x, v0.y + v1.y);
        dst[Ns] = cmk(v0.x - v1.x, v0.y - v1.y);
      } else if (rad == 4) {
        const C v0 = src[0], v1 = cmul_c(src[nb], twd(1)), v2 = cmul_c(src[2 * nb], twd(2)),
                v3 = cmul_c(src[3 * nb], twd(3));
        const C s02 = cmk(v0.x + v2.x, v0.y + v2.y), d02 = cmk(v0.x - v2.x, v0.y - v2.y);
        const C s13 = cmk(v1.x + v3.x, v1.y + v3.y), d13 = rot_i(cmk(v1.x - v3.x, v1.y - v3.y), sgn);
        dst[0] = cmk(s02.x + s13.x, s02.y + s13.y);
        dst[Ns] = cmk(d02.x + d13.x, d02.y + d13.y);
        dst[2 * Ns] = cmk(s02.x - s13.x, s02.y - s13.y);
        dst[3 * Ns] = cmk(d02.x - d13.x, d02.y - d13.y);
      } else if (rad == 3) {
        const R h = R(0.86602540378443864676);  // sin(2 pi / 3)
        const C v0 = src[0], v1 = cmul_c(src[nb], twd(1)), v2 = cmul_c(src[2 * nb], twd(2));
        const C s = cmk(v1.x + v2.x, v1.y + v2.y);
        const C m = cmk(v0.x - R(0.5) * s.x, v0.y - R(0.5) * s.y);
        const C d = rot_i(cmk(h * (v1.x - v2.x), h * (v1.y - v2.y)), sgn);
        dst[0] = cmk(v0.x + s.x, v0.y + s.y);
        dst[Ns] = cmk(m.x + d.x, m.y + d.y);
        dst[2 * Ns] = cmk(m.x - d.x, m.y - d.y);
      } else if (rad == 5) {
        const R c1 = R(0.30901699437494742410), c2 = R(-0.80901699437494742410);  // cos(2 pi/5), cos(4 pi/5)
        const R s1 = R(0.95105651629515357212), s2 = R(0.58778525229247312917);   // sin(2 pi/5), sin(4 pi/5)
        const C v0 = src[0], v1 = cmul_c(src[nb], twd(1)), v2 = cmul_c(src[2 * nb], twd(2)),
                v3 = cmul_c(src[3 * nb], twd(3)), v4 = cmul_c(src[4 * nb], twd(4));
        const C p1 = cmk(v1.x + v4.x, v1.y + v4.y), m1 = cmk(v1.x - v4.x, v1.y - v4.y);
        const C p2 = cmk(v2.x + v3.x, v2.y + v3.y), m2 = cmk(v2.x - v3.x, v2.y - v3.y);
        const C a1 = cmk(v0.x + c1 * p1.x + c2 * p2.x, v0.y + c1 * p1.y + c2 * p2.y);
        const C a2 = cmk(v0.x + c2 * p1.x + c1 * p2.x, v0.y + c2 * p1.y + c1 * p2.y);
        const C b1 = rot_i(cmk(s1 * m1.x + s2 * m2.x, s1 * m1.y + s2 * m2.y), sgn);
        const C b2 = rot_i(cmk(s2 * m1.x - s1 * m2.x, s2 * m1.y - s1 * m2.y), sgn);
        dst[0] = cmk(v0.x + p1.x + p2.x, v0.y + p1.y + p2.y);
        dst[Ns] = cmk(a1.x + b1.x, a1.y + b1.y);
        dst[4 * Ns] = cmk(a1.x - b1.x, a1.y - b1.y);
        dst[2 * Ns] = cmk(a2.x + b2.x, a2.y + b2.y);
        dst[3 * Ns] = cmk(a2.x - b2.x, a2.y - b2.y);
      } else {
        // any other prime: the direct sum, with the stage twiddle folded into the DFT's:
        // out_q = sum_r in_r w^(r (jm + q Ns) tstep)
        for (int q = 0; q < rad; q++) {
          R re = 0, im = 0;
          const long long e = (long long)(jm + q * Ns) * tstep;
          for (int r = 0; r < rad; r++) {
            C w = tw[(int)((r * e) % n)];
            if (inverse) w.y = -w.y;
            const C v = src[r * nb];
            re += v.x * w.x - v.y * w.y;
            im += v.x * w.y + v.y * w.x;
          }
          dst[q * Ns] = cmk(re, im);
        }
      }
    }
    __syncthreads();
    C* tmp = a;
    a = b;
    b = tmp;
    Ns *= rad;
  }
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int t = st == 1 ? idx / n : idx % tile_lines;
    const int k = st == 1 ? idx - t * n : idx / tile_lines;
    X[fft_addr(tile, t, k, n, st, tile_lines)] = a[t * n + k];
  }
}

FftPlan make_plan(int n) {
  FftPlan p{};
  int m = n;
  auto push = [&](int r) { p.radix[p.nstages++] = r; m /= r; };
  while (m % 4 == 0) push(4);
  while (m % 2 == 0) push(2);
  while (m % 3 == 0) push(3);
  while (m % 5 == 0) push(5);
  for (int f = 7; m > 1;) {
    if ((long long)f * f > m) {
      push(m);
      break;
    }
    if (m % f == 0)
      push(f);
    else
      f += 2;
  }
  return p;
}

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
int ilog2(int n) {
  int l = 0;
  while ((1 << l) < n) l++;
  return l;
}
// the radix-2 kernel reads exp(-2 pi i k/n) for k < n/2, the mixed-radix kernel for k < n
int twiddle_count(int n) { return (is_pow2(n) && !GLASMA_FFT_POW2_STOCKHAM) ? (n / 2 > 0 ? n / 2 : 1) : n; }

// Lines per block: up to kFftMaxTile complex values staged (half that for the mixed-radix kernel, which
// keeps two buffers: at 2 x 64 KB a block of the z pass left one block per SM and the FP64 pipe 55 %
// busy, ncu), at most 16, a power of two dividing the batch.
int tile_lines_for(int n, long long st, long long nlines_total, int max_tile = kFftMaxTile) {
  int cap = max_tile / n;
  if (cap < 1) cap = 1;
  if (cap > 16) cap = 16;
  if (st == 1) {
    int t = 1;
    while (t * 2 <= cap && nlines_total % (t * 2) == 0) t *= 2;
    return t;
  }
  int t = 1;
  while (t * 2 <= cap && st % (t * 2) == 0) t *= 2;
  return t;
}

template <typename C>
cudaError_t fft_lines_t(C* X, int n, long long st, long long total, int inverse, const C* tw, cudaStream_t stream) {
  const long long nlines = total / n;
  const bool mixed = !(is_pow2(n) && !GLASMA_FFT_POW2_STOCKHAM);
  const int tl = tile_lines_for(n, st, nlines, mixed ? kFftMaxTile / 2 : kFftMaxTile);
  const long long tiles = nlines / tl;
  if (n == 1) return cudaSuccess;
  if (is_pow2(n) && !GLASMA_FFT_POW2_STOCKHAM) {
    const size_t smem = ((size_t)(n / 2) + (size_t)tl * (n + 1)) * sizeof(C);
    cudaFuncSetAttribute(fft_pow2_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    fft_pow2_kernel<C><<<(unsigned)tiles, kFftThreads, smem, stream>>>(X, ilog2(n), st, ilog2(tl), st > 1 ? st / tl : 0,
                                                                       tw, inverse);
  } else {
    const size_t smem = 2 * (size_t)tl * n * sizeof(C);
    if (smem > kFftMaxSmem) return cudaErrorInvalidValue;  // lines longer than the shared-memory tile
    cudaFuncSetAttribute(fft_mixed_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(smem > 48 * 1024 ? smem : 48 * 1024));
    fft_mixed_kernel<C><<<(unsigned)tiles, kFftThreads, smem, stream>>>(X, n, st, tl, tw, make_plan(n), inverse);
  }
  return cudaGetLastError();
}

}  // namespace

double2* make_twiddles(int n, cudaStream_t stream) {
  const int count = twiddle_count(n);
  double2* tw = nullptr;
  if (cudaMalloc(&tw, sizeof(double2) * count) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  twiddle_kernel<<<(count + 255) / 256, 256, 0, stream>>>(tw, n, count);
  return tw;
}

cudaError_t fft_lines(double2* X, int n, long long st, long long total, int inverse, const double2* tw,
                      cudaStream_t stream) {
  return fft_lines_t<double2>(X, n, st, total, inverse, tw, stream);
}

struct GaugeFixState {
  Geometry g;
  int precision = -1;
  void* X = nullptr;  // 8 V complex doubles: the gauge update uses 4 colour-pair planes of it
  double* p2tab = nullptr;  // per-axis lattice momenta squared (p2_table_kernel), nx + ny + nz
  float* p2tab32 = nullptr;  // the same rounded to FP32, for the FP32 planes
  double p2a[3] = {0, 0, 0};  // the spacings the table was made for
  std::map<int, double2*> twiddles;
  std::map<int, float2*> twiddles32;
  std::vector<double> host_results;
};

namespace {

// 3D transform (unnormalised) of `planes` planes X[p][z][y][x]: three passes of batched 1D transforms
template <typename C>
cudaError_t fft3d_t(const GaugeFixState* s, C* X, int planes, int inverse, const std::map<int, C*>& tws,
                    cudaStream_t stream) {
  const Geometry& g = s->g;
  const long long total = (long long)planes * g.vol;
  cudaError_t e = fft_lines_t<C>(X, g.nx, 1, total, inverse, tws.at(g.nx), stream);
  if (e == cudaSuccess) e = fft_lines_t<C>(X, g.ny, g.nx, total, inverse, tws.at(g.ny), stream);
  if (e == cudaSuccess) e = fft_lines_t<C>(X, g.nz, g.plane, total, inverse, tws.at(g.nz), stream);
  return e;
}

// FP32 twiddles, narrowed from the FP64 ones on first use
cudaError_t ensure_twiddles32(GaugeFixState* s, cudaStream_t stream) {
  for (auto& kv : s->twiddles) {
    if (s->twiddles32.count(kv.first)) continue;
    const int count = twiddle_count(kv.first);
    float2* tw = nullptr;
    cudaError_t e = cudaMalloc(&tw, sizeof(float2) * count);
    if (e != cudaSuccess) return e;
    twiddle_narrow_kernel<<<(count + 255) / 256, 256, 0, stream>>>(kv.second, tw, count);
    s->twiddles32[kv.first] = tw;
  }
  return cudaGetLastError();
}

// the acceleration step's per-axis momentum table, for this lattice's spacings
cudaError_t ensure_p2tab(GaugeFixState* s, const Geometry& g, cudaStream_t stream) {
  const int n = g.nx + g.ny + g.nz;
  if (!s->p2tab) {
    cudaError_t e = cudaMalloc(&s->p2tab, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&s->p2tab32, sizeof(float) * n);
    if (e != cudaSuccess) {
      cudaGetLastError();
      cudaFree(s->p2tab);
      s->p2tab = nullptr;
      s->p2tab32 = nullptr;
      return e;
    }
    s->p2a[0] = s->p2a[1] = s->p2a[2] = 0.0;
  }
  if (s->p2a[0] != g.a[0] || s->p2a[1] != g.a[1] || s->p2a[2] != g.a[2]) {
    p2_table_kernel<<<(n + 127) / 128, 128, 0, stream>>>(g.nx, g.ny, g.nz, g.a[0], g.a[1], g.a[2], s->p2tab);
    narrow_table_kernel<<<(n + 127) / 128, 128, 0, stream>>>(s->p2tab, s->p2tab32, n);
    for (int k = 0; k < 3; k++) s->p2a[k] = g.a[k];
  }
  return cudaGetLastError();
}

int prepare(GaugeFixState** ps, const GaugeFixArgs& a, std::string* err) {
  GaugeFixState* s = *ps;
  if (s && (s->g.nx != a.g.nx || s->g.ny != a.g.ny || s->g.nz != a.g.nz)) {
    gaugefix_destroy(s);
    s = nullptr;
  }
  if (!s) {
    s = new GaugeFixState;
    s->g = a.g;
    s->precision = a.precision;
    *ps = s;
    cudaError_t e = cudaMalloc(&s->X, sizeof(double2) * 8 * a.g.vol);
    if (e != cudaSuccess) {
      cudaGetLastError();
      *err = std::string("cudaMalloc FFT array: ") + cudaGetErrorString(e);
      return GLASMA_ERR_OUT_OF_MEMORY;
    }
    const int ns[3] = {a.g.nx, a.g.ny, a.g.nz};
    for (int n : ns) {
      if (s->twiddles.count(n)) continue;
      const int count = twiddle_count(n);
      double2* tw = nullptr;
      e = cudaMalloc(&tw, sizeof(double2) * count);
      if (e != cudaSuccess) {
        cudaGetLastError();
        *err = "cudaMalloc twiddles";
        return GLASMA_ERR_OUT_OF_MEMORY;
      }
      twiddle_kernel<<<(count + 255) / 256, 256, 0, a.stream>>>(tw, n, count);
      s->twiddles[n] = tw;
    }
  }
  return GLASMA_OK;
}

// CopyFields (S/GAUGETRANSFORMATION/GaugeTransformation.cpp:93-97): interior slices only
template <typename T>
cudaError_t copy_fields(const GaugeFixArgs& a) {
  const Geometry& g = a.g;
  const cx<T>* U = static_cast<const cx<T>*>(a.U);
  const T* E = static_cast<const T*>(a.E);
  cx<T>* UG = static_cast<cx<T>*>(a.UG);
  T* EG = static_cast<T*>(a.EG);
  cudaError_t e = cudaSuccess;
  for (int c = 0; c < 27 && e == cudaSuccess; c++)
    e = cudaMemcpyAsync(UG + (long long)c * g.S + g.plane, U + (long long)c * g.S + g.plane, sizeof(cx<T>) * g.vol,
                        cudaMemcpyDeviceToDevice, a.stream);
  for (int c = 0; c < 24 && e == cudaSuccess; c++)
    e = cudaMemcpyAsync(EG + (long long)c * g.S + g.plane, E + (long long)c * g.S + g.plane, sizeof(T) * g.vol,
                        cudaMemcpyDeviceToDevice, a.stream);
  return e;
}
// GaugeTransformLinks: UG from U and G, then the ghost slices of G
template <typename T>
cudaError_t transform_links_all(const GaugeFixArgs& a) {
  const unsigned tb = (unsigned)((a.g.vol + 127) / 128);
  transform_links_kernel<T><<<tb, 128, 0, a.stream>>>(a.g, static_cast<const cx<T>*>(a.U),
                                                      static_cast<const cx<T>*>(a.G), static_cast<cx<T>*>(a.UG));
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = launch_sync_ghosts<cx<T>>(a.g, static_cast<cx<T>*>(a.G), 9, a.stream);
  return e;
}
// After the last iteration (CoulombGaugeFixing.cpp:84-86): GaugeTransformLinks, GaugeTransformElectricFields
template <typename T>
cudaError_t finish_fields(const GaugeFixArgs& a) {
  cudaError_t e = transform_links_all<T>(a);
  if (e != cudaSuccess) return e;
  const unsigned tb = (unsigned)((a.g.vol + 127) / 128);
  transform_efield_kernel<T><<<tb, 128, 0, a.stream>>>(a.g, static_cast<const T*>(a.E),
                                                       static_cast<const cx<T>*>(a.G), static_cast<T*>(a.EG));
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = launch_sync_ghosts<cx<T>>(a.g, static_cast<cx<T>*>(a.G), 9, a.stream)) != cudaSuccess) return e;
  return cudaStreamSynchronize(a.stream);
}

// n_start > 0: the final FP64 sweeps after the FP32 ones of run_mixed (the fields already copied, log
// rows and the iteration count continued)
template <typename T>
int run_impl(GaugeFixState* s, const GaugeFixArgs& a, double alpha, int max_iters, double tol, unsigned flags,
             double* log, int* iterations, std::string* err, int n_start = 0) {
  const Geometry& g = a.g;
  cudaStream_t st = a.stream;
  cx<T>* G = static_cast<cx<T>*>(a.G);
  const cx<T>* UG = static_cast<const cx<T>*>(a.UG);
  auto cuda_err = [&](cudaError_t e, const char* where) {
    *err = std::string(where) + ": " + cudaGetErrorString(e);
    return GLASMA_ERR_CUDA;
  };
  cudaError_t e;
  if (n_start == 0 && (e = copy_fields<T>(a)) != cudaSuccess) return cuda_err(e, "copy fields");
  auto transform_links = [&]() { return transform_links_all<T>(a); };
  if ((e = transform_links()) != cudaSuccess) return cuda_err(e, "transform links");

  const double cw[3] = {(a.a_scale / g.a[0]) * (a.a_scale / g.a[0]), (a.a_scale / g.a[1]) * (a.a_scale / g.a[1]),
                        g.nz > 1 ? (a.a_scale / g.a[2]) * (a.a_scale / g.a[2]) : 0.0};
  const unsigned nb = blocks_for(g.vol, kGfThreads, kGfBlocks);
  double* part_dev = a.scratch;                 // nb * 4
  double* part_upd = a.scratch + (size_t)nb * 4;  // nb * 3
  double* res = a.scratch + (size_t)nb * 7;     // 8 results
  double h[8];
  double gmax = 1.0;
  int n = n_start;
  int status = GLASMA_OK;
  const double minf0 = 2.0 * 3 * (1.0 / (g.a[0] * g.a[0]) + 1.0 / (g.a[1] * g.a[1]) + 1.0 / (g.a[2] * g.a[2]));
  const bool fft32 = (flags & GLASMA_GF_FFT_FP32) != 0;
  if (fft32 && (e = ensure_twiddles32(s, st)) != cudaSuccess) return cuda_err(e, "FP32 twiddles");
  if ((e = ensure_p2tab(s, g, st)) != cudaSuccess) return cuda_err(e, "momentum table");
  double2* X64 = static_cast<double2*>(s->X);
  float2* X32 = static_cast<float2*>(s->X);
  const long long tot = 4 * g.vol;
  const int project = (flags & GLASMA_GF_PROJECT_ZERO_MODE) ? 1 : 0;
  const int open_top = (flags & GLASMA_GF_OPEN_Z) ? 1 : 0;
  while (n < max_iters && gmax > tol) {
    if (fft32)
      deviation_kernel<T, float2><<<nb, kGfThreads, 0, st>>>(g, UG, cw[0], cw[1], cw[2], X32, part_dev, open_top);
    else
      deviation_kernel<T, double2><<<nb, kGfThreads, 0, st>>>(g, UG, cw[0], cw[1], cw[2], X64, part_dev, open_top);
    red::finish_kernel<4><<<1, red::kThreads, 0, st>>>(part_dev, (int)nb, 1 | (0 << 2) | (2 << 4) | (0 << 6), res);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err(e, "deviation");
    e = fft32 ? fft3d_t<float2>(s, X32, 4, 0, s->twiddles32, st) : fft3d_t<double2>(s, X64, 4, 0, s->twiddles, st);
    if (e != cudaSuccess) return cuda_err(e, "fft forward");
    if (fft32)
      accelerate32_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(g.nx, g.ny, g.nz, (float)g.vol, s->p2tab32, X32,
                                                                         project);
    else
      accelerate_kernel<double2><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(g.nx, g.ny, g.nz, (double)g.vol, s->p2tab,
                                                                          X64, project);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err(e, "accelerate");
    e = fft32 ? fft3d_t<float2>(s, X32, 4, 1, s->twiddles32, st) : fft3d_t<double2>(s, X64, 4, 1, s->twiddles, st);
    if (e != cudaSuccess) return cuda_err(e, "fft backward");
    if (fft32)
      update_kernel<T, float2><<<nb, kGfThreads, 0, st>>>(g, X32, G, alpha, part_upd);
    else
      update_kernel<T, double2><<<nb, kGfThreads, 0, st>>>(g, X64, G, alpha, part_upd);
    red::finish_kernel<3><<<1, red::kThreads, 0, st>>>(part_upd, (int)nb, 1 | (0 << 2) | (0 << 4), res + 4);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err(e, "update");
    if ((e = transform_links()) != cudaSuccess) return cuda_err(e, "transform links");
    if ((e = cudaMemcpyAsync(h, res, sizeof(double) * 7, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
      return cuda_err(e, "monitor copy");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_err(e, "monitor sync");
    const double V = (double)g.vol;
    gmax = h[0];
    if (log) {
      double* o = log + 7 * (size_t)n;
      o[0] = n;
      o[1] = h[0];
      o[2] = sqrt(h[1] / (8.0 * V));
      o[3] = h[4];
      o[4] = sqrt(h[5] / (8.0 * V));
      o[5] = h[2] < minf0 ? h[2] : minf0;
      o[6] = h[3] / V;
    }
    n++;
    if (h[6] > 0.0) {
      *err = "gauge update left SU(3) by more than 1e-13 (the reference exits here)";
      status = GLASMA_ERR_NUMERICAL;
      break;
    }
  }
  *iterations = n;
  if (status != GLASMA_OK) return status;
  if ((e = finish_fields<T>(a)) != cudaSuccess) return cuda_err(e, "final transform");
  return GLASMA_OK;
}

// GLASMA_GF_MIXED on FP64 handles: the sweeps on FP32 copies of U and G until the FP32 maximum
// deviation reaches kMixedSwitch or stops falling (its rounding floor), then G widened and projected
// onto SU(3) in FP64 and the FP64 sweeps to the stopping rule (run_impl, continuing the count and log).
constexpr double kMixedSwitch = 1e-5;  // max |Delta| at which the FP32 sweeps hand over
constexpr int kMixedStall = 20;        // or after this many FP32 sweeps without a 5 % better maximum
constexpr float kMixedGuard = 1e-5f;   // unitarity guard of the FP32 update

struct Fp32Copies {
  cx<float>* U = nullptr;
  cx<float>* G = nullptr;
  cx<float>* UG = nullptr;
  cudaStream_t stream = nullptr;
  ~Fp32Copies() {
    if (stream) cudaStreamSynchronize(stream);
    cudaFree(U);
    cudaFree(G);
    cudaFree(UG);
  }
};

int run_mixed(GaugeFixState* s, const GaugeFixArgs& a, double alpha, int max_iters, double tol, unsigned flags,
              double* log, int* iterations, std::string* err) {
  const Geometry& g = a.g;
  cudaStream_t st = a.stream;
  auto cuda_err = [&](cudaError_t e, const char* where) {
    *err = std::string(where) + ": " + cudaGetErrorString(e);
    return GLASMA_ERR_CUDA;
  };
  Fp32Copies c;
  c.stream = st;
  cudaError_t e = cudaMalloc(&c.U, sizeof(cx<float>) * 27 * g.S);
  if (e == cudaSuccess) e = cudaMalloc(&c.G, sizeof(cx<float>) * 9 * g.S);
  if (e == cudaSuccess) e = cudaMalloc(&c.UG, sizeof(cx<float>) * 27 * g.S);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *err = std::string("cudaMalloc FP32 gauge-fixing copies: ") + cudaGetErrorString(e);
    return GLASMA_ERR_OUT_OF_MEMORY;
  }
  if ((e = copy_fields<double>(a)) != cudaSuccess) return cuda_err(e, "copy fields");
  narrow_kernel<<<(unsigned)((27 * g.S + 255) / 256), 256, 0, st>>>(static_cast<const cx<double>*>(a.U), c.U, 27 * g.S);
  narrow_kernel<<<(unsigned)((9 * g.S + 255) / 256), 256, 0, st>>>(static_cast<const cx<double>*>(a.G), c.G, 9 * g.S);
  const unsigned tb = (unsigned)((g.vol + 127) / 128);
  auto transform32 = [&]() {
    transform_links32_kernel<<<tb, 128, 0, st>>>(g, c.U, c.G, c.UG);
    cudaError_t x = cudaGetLastError();
    if (x == cudaSuccess) x = launch_sync_ghosts<cx<float>>(g, c.G, 9, st);
    return x;
  };
  if ((e = transform32()) != cudaSuccess) return cuda_err(e, "FP32 transform links");
  if ((e = ensure_twiddles32(s, st)) != cudaSuccess) return cuda_err(e, "FP32 twiddles");
  if ((e = ensure_p2tab(s, g, st)) != cudaSuccess) return cuda_err(e, "momentum table");
  const float cw[3] = {(float)((a.a_scale / g.a[0]) * (a.a_scale / g.a[0])),
                       (float)((a.a_scale / g.a[1]) * (a.a_scale / g.a[1])),
                       g.nz > 1 ? (float)((a.a_scale / g.a[2]) * (a.a_scale / g.a[2])) : 0.f};
  const unsigned nb = blocks_for(g.vol, kGfThreads, kGfBlocks);
  double* part_dev = a.scratch;
  double* part_upd = a.scratch + (size_t)nb * 4;
  double* res = a.scratch + (size_t)nb * 7;
  const double minf0 = 2.0 * 3 * (1.0 / (g.a[0] * g.a[0]) + 1.0 / (g.a[1] * g.a[1]) + 1.0 / (g.a[2] * g.a[2]));
  float2* X32 = static_cast<float2*>(s->X);
  const long long tot = 4 * g.vol;
  const int project = (flags & GLASMA_GF_PROJECT_ZERO_MODE) ? 1 : 0;
  const int open_top = (flags & GLASMA_GF_OPEN_Z) ? 1 : 0;
  double h[8];
  double gmax = 1.0, best = 1e300;
  int n = 0, since_best = 0;
  while (n < max_iters && gmax > tol) {
    deviation32_kernel<<<nb, kGfThreads, 0, st>>>(g, c.UG, cw[0], cw[1], cw[2], X32, part_dev, open_top);
    red::finish_kernel<4><<<1, red::kThreads, 0, st>>>(part_dev, (int)nb, 1 | (0 << 2) | (2 << 4) | (0 << 6), res);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err(e, "FP32 deviation");
    if ((e = fft3d_t<float2>(s, X32, 4, 0, s->twiddles32, st)) != cudaSuccess) return cuda_err(e, "fft forward");
    accelerate32_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(g.nx, g.ny, g.nz, (float)g.vol, s->p2tab32, X32,
                                                                         project);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err(e, "accelerate");
    if ((e = fft3d_t<float2>(s, X32, 4, 1, s->twiddles32, st)) != cudaSuccess) return cuda_err(e, "fft backward");
    update32_kernel<<<nb, kGfThreads, 0, st>>>(g, X32, c.G, (float)alpha, part_upd, kMixedGuard);
    red::finish_kernel<3><<<1, red::kThreads, 0, st>>>(part_upd, (int)nb, 1 | (0 << 2) | (0 << 4), res + 4);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err(e, "FP32 update");
    if ((e = transform32()) != cudaSuccess) return cuda_err(e, "FP32 transform links");
    if ((e = cudaMemcpyAsync(h, res, sizeof(double) * 7, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
      return cuda_err(e, "monitor copy");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_err(e, "monitor sync");
    const double V = (double)g.vol;
    gmax = h[0];
    if (log) {
      double* o = log + 7 * (size_t)n;
      o[0] = n;
      o[1] = h[0];
      o[2] = sqrt(h[1] / (8.0 * V));
      o[3] = h[4];
      o[4] = sqrt(h[5] / (8.0 * V));
      o[5] = h[2] < minf0 ? h[2] : minf0;
      o[6] = h[3] / V;
    }
    n++;
    if (h[6] > 0.0) {
      *iterations = n;
      *err = "FP32 gauge update left SU(3) by more than 1e-5";
      return GLASMA_ERR_NUMERICAL;
    }
    if (gmax < 0.95 * best) {
      best = gmax;
      since_best = 0;
    } else if (++since_best >= kMixedStall) {
      break;
    }
    if (gmax <= kMixedSwitch) break;
  }
  // hand over: G from the FP32 sweeps, widened and projected, then the FP64 sweeps
  widen_gauge_kernel<<<(unsigned)((g.S + 255) / 256), 256, 0, st>>>(c.G, static_cast<cx<double>*>(a.G), g.S);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err(e, "widen gauge");
  *iterations = n;
  if (gmax <= tol && n > 0) {
    if ((e = finish_fields<double>(a)) != cudaSuccess) return cuda_err(e, "final transform");
    return GLASMA_OK;
  }
  return run_impl<double>(s, a, alpha, max_iters, tol, flags, log, iterations, err, n);
}

// SetCoulombGauge with the Los Alamos (los_alamos != 0) or the Jacobi update: per iteration one pass
// over every site (Jacobi) or the even and then the odd sites (Los Alamos), the links re-transformed
// after each pass; the monitors of both passes of an iteration are reduced together (the reference
// resets them before the even pass only, LosAlamos.cpp:16-23).
template <typename T>
int run_local_impl(const GaugeFixArgs& a, int los_alamos, double param, unsigned long long seed, int max_iters,
                   double tol, double* log, int* iterations, std::string* err) {
  const Geometry& g = a.g;
  cudaStream_t st = a.stream;
  cx<T>* G = static_cast<cx<T>*>(a.G);
  cx<T>* UG = static_cast<cx<T>*>(a.UG);
  auto cuda_err = [&](cudaError_t e, const char* where) {
    *err = std::string(where) + ": " + cudaGetErrorString(e);
    return GLASMA_ERR_CUDA;
  };
  cudaError_t e;
  if ((e = copy_fields<T>(a)) != cudaSuccess) return cuda_err(e, "copy fields");
  if ((e = transform_links_all<T>(a)) != cudaSuccess) return cuda_err(e, "transform links");
  const double cw[3] = {(a.a_scale / g.a[0]) * (a.a_scale / g.a[0]), (a.a_scale / g.a[1]) * (a.a_scale / g.a[1]),
                        g.nz > 1 ? (a.a_scale / g.a[2]) * (a.a_scale / g.a[2]) : 0.0};
  const int passes = los_alamos ? 2 : 1;
  const long long slots = (long long)(los_alamos ? (g.nx + 1) / 2 : g.nx) * g.ny * g.nz;
  const unsigned nb = blocks_for(slots, kGfThreads, kGfBlocks);
  double* part = a.scratch;                        // passes * nb * 7
  double* res = a.scratch + (size_t)kGfBlocks * 14;  // 7 results
  const double minf0 = 2.0 * 3 * (1.0 / (g.a[0] * g.a[0]) + 1.0 / (g.a[1] * g.a[1]) + 1.0 / (g.a[2] * g.a[2]));
  double h[7];
  double gmax = 1.0;
  int n = 0, status = GLASMA_OK;
  while (n < max_iters && gmax > tol) {
    for (int pass = 0; pass < passes; pass++) {
      local_update_kernel<T><<<nb, kGfThreads, 0, st>>>(g, UG, G, cw[0], cw[1], cw[2], los_alamos,
                                                        los_alamos ? pass : -1, param, seed, n,
                                                        part + (size_t)pass * nb * 7);
      if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err(e, "local update");
      if ((e = transform_links_all<T>(a)) != cudaSuccess) return cuda_err(e, "transform links");
    }
    red::finish_kernel<7><<<1, red::kThreads, 0, st>>>(
        part, (int)(nb * passes), 1 | (0 << 2) | (2 << 4) | (0 << 6) | (1 << 8) | (0 << 10) | (0 << 12), res);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err(e, "monitor reduction");
    if ((e = cudaMemcpyAsync(h, res, sizeof(double) * 7, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
      return cuda_err(e, "monitor copy");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_err(e, "monitor sync");
    const double V = (double)g.vol;
    gmax = h[0];
    if (log) {
      double* o = log + 7 * (size_t)n;
      o[0] = n;
      o[1] = h[0];
      o[2] = sqrt(h[1] / (8.0 * V));
      o[3] = h[4];
      o[4] = sqrt(h[5] / (8.0 * V));
      o[5] = h[2] < minf0 ? h[2] : minf0;
      o[6] = h[3] / V;
    }
    n++;
    if (h[6] > 0.0) {
      *err = "gauge update left SU(3) by more than 1e-13 (the reference exits here)";
      status = GLASMA_ERR_NUMERICAL;
      break;
    }
  }
  *iterations = n;
  if (status != GLASMA_OK) return status;
  if ((e = finish_fields<T>(a)) != cudaSuccess) return cuda_err(e, "final transform");
  return GLASMA_OK;
}

}  // namespace

int gaugefix_run(GaugeFixState** state, const GaugeFixArgs& a, double alpha, int max_iters, double tol, unsigned flags,
                 double* log, int* iterations, std::string* err) {
  *iterations = 0;
  int st = prepare(state, a, err);
  if (st != GLASMA_OK) return st;
  if (a.scratch_doubles < (size_t)kGfBlocks * 7 + 16) {
    *err = "scratch too small";
    return GLASMA_ERR_INVALID_ARGUMENT;
  }
  if (flags & GLASMA_GF_MIXED) {
    if (a.precision != GLASMA_FP64) {
      *err = "GLASMA_GF_MIXED applies to FP64 handles (FP32 handles store FP32 fields already)";
      return GLASMA_ERR_UNSUPPORTED;
    }
    return run_mixed(*state, a, alpha, max_iters, tol, flags, log, iterations, err);
  }
  return a.precision == GLASMA_FP64 ? run_impl<double>(*state, a, alpha, max_iters, tol, flags, log, iterations, err)
                                    : run_impl<float>(*state, a, alpha, max_iters, tol, flags, log, iterations, err);
}

int gaugefix_run_local(const GaugeFixArgs& a, int algorithm, double param, unsigned long long seed, int max_iters,
                       double tol, double* log, int* iterations, std::string* err) {
  *iterations = 0;
  if (a.scratch_doubles < gaugefix_scratch_doubles()) {
    *err = "scratch too small";
    return GLASMA_ERR_INVALID_ARGUMENT;
  }
  const int los_alamos = algorithm == GLASMA_GF_LOS_ALAMOS ? 1 : 0;
  return a.precision == GLASMA_FP64
             ? run_local_impl<double>(a, los_alamos, param, seed, max_iters, tol, log, iterations, err)
             : run_local_impl<float>(a, los_alamos, param, seed, max_iters, tol, log, iterations, err);
}

size_t gaugefix_scratch_doubles() { return (size_t)kGfBlocks * 14 + 16; }

cudaError_t launch_transform_charge(const GaugeFixArgs& a, const void* J, double* out) {
  const unsigned blocks = (unsigned)((a.g.S + 127) / 128);
  if (a.precision == GLASMA_FP64)
    transform_charge_kernel<double><<<blocks, 128, 0, a.stream>>>(a.g, static_cast<const double*>(J),
                                                                  static_cast<const cx<double>*>(a.G), out);
  else
    transform_charge_kernel<float><<<blocks, 128, 0, a.stream>>>(a.g, static_cast<const float*>(J),
                                                                 static_cast<const cx<float>*>(a.G), out);
  return cudaGetLastError();
}

void gaugefix_destroy(GaugeFixState* s) {
  if (!s) return;
  if (s->X) cudaFree(s->X);
  if (s->p2tab) cudaFree(s->p2tab);
  if (s->p2tab32) cudaFree(s->p2tab32);
  for (auto& kv : s->twiddles) cudaFree(kv.second);
  for (auto& kv : s->twiddles32) cudaFree(kv.second);
  delete s;
}

// Exposed for the FFT test entry point: forward or backward 3D transform of 8 colour planes.
int gaugefix_fft_test(GaugeFixState** state, const GaugeFixArgs& a, const double2* in, double2* out, int inverse,
                      std::string* err) {
  int st = prepare(state, a, err);
  if (st != GLASMA_OK) return st;
  const size_t bytes = sizeof(double2) * 8 * a.g.vol;
  cudaError_t e = cudaMemcpyAsync((*state)->X, in, bytes, cudaMemcpyDefault, a.stream);
  if (e == cudaSuccess)
    e = fft3d_t<double2>(*state, static_cast<double2*>((*state)->X), 8, inverse, (*state)->twiddles, a.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, (*state)->X, bytes, cudaMemcpyDefault, a.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(a.stream);
  if (e != cudaSuccess) {
    *err = cudaGetErrorString(e);
    return GLASMA_ERR_CUDA;
  }
  return GLASMA_OK;
}

int gaugefix_fft_test_f32(GaugeFixState** state, const GaugeFixArgs& a, const float2* in, float2* out, int inverse,
                          std::string* err) {
  int st = prepare(state, a, err);
  if (st != GLASMA_OK) return st;
  const size_t bytes = sizeof(float2) * 8 * a.g.vol;
  cudaError_t e = ensure_twiddles32(*state, a.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync((*state)->X, in, bytes, cudaMemcpyDefault, a.stream);
  if (e == cudaSuccess)
    e = fft3d_t<float2>(*state, static_cast<float2*>((*state)->X), 8, inverse, (*state)->twiddles32, a.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, (*state)->X, bytes, cudaMemcpyDefault, a.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(a.stream);
  if (e != cudaSuccess) {
    *err = cudaGetErrorString(e);
    return GLASMA_ERR_CUDA;
  }
  return GLASMA_OK;
}

}  // namespace glasma

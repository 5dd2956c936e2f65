// observables.cu -- volume and per-slice reductions of the measurement path.
//
//   bulk       Observables::Bulk::Update (S/OBSERVABLES/BulkObservables.cpp:65-183):
//              sum_x 4 ReTr(1 - P_jk) per plane, sum_x E_mu^2, sum_x E_z (Jp-Jm)/sqrt2
//   gauss      GaussLaw::UpdateViolation (S/OBSERVABLES/GaussLawViolation.cpp:16-124) with
//              COMPUTE_GAUSS_VIOLATION (S/CALC/GaussViolation.cpp:13-23): max |G^a|, sum G^2 and
//              the per-z profile sum_{x,y,a} G^2 / (Nx Ny)
//   unitarity  Unitarity::UpdateViolation (S/OBSERVABLES/UnitarityViolation.cpp:13-51)
//   emt map    EnergyMomentumTensor::CreateMap (S/OBSERVABLES/EnergyMomentumTensor.cpp:92-170) with
//              COMPUTE_AVG_FIELD_STRENGTH (S/CALC/AvgFieldStrength.cpp:68-112)
//
// Every reduction is two-pass and deterministic: a fixed grid writes FP64 block partials
// (warp shuffles, then shared memory), a one-block pass sums them in a fixed order.
// Site arithmetic runs in FP64, except the magnetic term of the bulk energy on FP32 lattices,
// which uses the identity
//   3 - ReTr(a b c^d d^d) = 1/2 ||A - B||^2 - 1/2 (n(a) + n(b) + n(c) + n(d)),
//   A = a b, B = d c, n(u) = ||u||_F^2 - 3  (zero for unitary u),
// exact with n(A) + n(B) in place of the four link terms and equal to it to first order in the links'
// departure from unitarity (~1e-7 for FP32-rounded links, so the difference is ~1e-14); the link
// terms are preferred because the products' own FP32 rounding never enters them:
// A, B and ||A - B||^2 are formed in FP32, whose rounding then costs about 1e-7 ||A - B|| per
// plaquette instead of 1e-7 (no cancellation against 3, so weak fields keep their digits), and the
// norm terms are summed in FP64 per link (each link's n counted for the plaquettes it belongs to).
#include <type_traits>

#include "lattice.cuh"

namespace glasma {

namespace {

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 1216;  // 8 x 152 SMs
constexpr int kZChunks = 32;      // blocks per z slice for per-slice reductions

template <typename T>
__device__ __forceinline__ void load_link_d(const cx<T>* __restrict__ U, long long S, int mu, long long s, Mat<double>& m) {
  const cx<T>* p = U + (long long)(mu * 9) * S + s;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const cx<T> v = p[(long long)k * S];
    m.e[k] = mk<double>((double)v.re, (double)v.im);
  }
}
template <typename T>
__device__ __forceinline__ void load_alg_d(const T* __restrict__ F, long long S, long long base, long long s, Alg<double>& v) {
  const T* p = F + base * S + s;
#pragma unroll
  for (int a = 0; a < 8; a++) v.a[a] = (double)p[(long long)a * S];
}

__device__ __forceinline__ long long nbs(const Geometry& g, int x, int y, int z, int dx, int dy, int dz) {
  int xx = x + dx, yy = y + dy;
  xx = xx < 0 ? xx + g.nx : (xx >= g.nx ? xx - g.nx : xx);
  yy = yy < 0 ? yy + g.ny : (yy >= g.ny ? yy - g.ny : yy);
  return site_index(g, xx, yy, z + dz);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// Block-reduce K values (the first KMAX of which are maxima when is_max[k]); thread 0 writes out[k].
template <int K>
__device__ __forceinline__ void block_reduce_store(double (&v)[K], const bool (&is_max)[K], double* out) {
  __shared__ double sh[K][kRedThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    const double r = is_max[k] ? warp_max(v[k]) : warp_sum(v[k]);
    if (lane == 0) sh[k][warp] = r;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      double r = (lane < (int)(blockDim.x / 32)) ? sh[k][lane] : 0.0;  // all reduced values are >= 0 or sums
      r = is_max[k] ? warp_max(r) : warp_sum(r);
      if (lane == 0) out[k] = r;
    }
  }
}

// Sum (or max) partials[b*K + k] over b in a fixed order; one block.
template <int K>
__global__ void finish_kernel(const double* __restrict__ partials, int nblocks, unsigned max_mask, double* out) {
  double v[K];
  bool is_max[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    v[k] = 0.0;
    is_max[k] = (max_mask >> k) & 1u;
  }
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < K; k++) {
      const double x = partials[(long long)b * K + k];
      v[k] = is_max[k] ? fmax(v[k], x) : v[k] + x;
    }
  block_reduce_store<K>(v, is_max, out);
}

// Per-slice finish: out[z*K + k] = sum_c partials[(z*kZChunks + c)*K + k] (max for masked k).
template <int K>
__global__ void finish_slices_kernel(const double* __restrict__ partials, int nz, unsigned max_mask, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nz * K) return;
  const int z = i / K, k = i - z * K;
  const bool is_max = (max_mask >> k) & 1u;
  double v = 0.0;
  for (int c = 0; c < kZChunks; c++) {
    const double x = partials[((long long)z * kZChunks + c) * K + k];
    v = is_max ? fmax(v, x) : v + x;
  }
  out[i] = v;
}

// Index decodes in 32-bit arithmetic whenever the indices fit: GB300 runs the 64-bit integer
// division sequence partly on its FP64 pipe (measured on the gauge fixer's FP32 kernels), the pipe
// the FP64 observables are bound by.
__device__ __forceinline__ void decode_vol(const Geometry& g, long long idx, int& x, int& y, int& z) {
  if (g.vol < (1LL << 31)) {
    const unsigned u = (unsigned)idx, r = u / (unsigned)g.nx;
    x = (int)(u - r * (unsigned)g.nx);
    z = (int)(r / (unsigned)g.ny);
    y = (int)(r - (unsigned)z * (unsigned)g.ny);
    return;
  }
  const long long r = idx / g.nx;
  x = (int)(idx - r * g.nx);
  z = (int)(r / g.ny);
  y = (int)(r - (long long)z * g.ny);
}
// (x, y) of r = x + nx y within a transverse plane
__device__ __forceinline__ void decode_plane(const Geometry& g, long long r, int& x, int& y) {
  if (g.plane < (1LL << 31)) {
    const unsigned u = (unsigned)r;
    y = (int)(u / (unsigned)g.nx);
    x = (int)(u - (unsigned)y * (unsigned)g.nx);
    return;
  }
  y = (int)(r / g.nx);
  x = (int)(r - (long long)y * g.nx);
}

// Re tr(a b c^d d^d) = Re sum_ij (a b)_ij conj((d c)_ij): two products and a dot product instead of
// the three products of the full plaquette (the bulk energy needs only its trace)
__device__ __forceinline__ double retr_plaq(const Mat<double>& a, const Mat<double>& b, const Mat<double>& c,
                                           const Mat<double>& d) {
  Mat<double> A, B;
  mul_nn(a, b, A);
  mul_nn(d, c, B);
  double t = 0.0;
#pragma unroll
  for (int k = 0; k < 9; k++) t = fma(A.e[k].re, B.e[k].re, fma(A.e[k].im, B.e[k].im, t));
  return t;
}

// ||A - B||^2 of the plaquette a b (d c)^d in the (j,k) plane, A = U_j(x) U_k(x+j), B = U_k(x) U_j(x+k), FP32
__device__ __forceinline__ float plaq_sqdiff_f(const cx<float>* __restrict__ U, long long S, int j, int k,
                                               long long s, long long sj, long long sk) {
  Mat<float> a, b, A, B;
  load_link<float, long long>(U, S, j, s, a);
  load_link<float, long long>(U, S, k, sj, b);
  mul_nn(a, b, A);
  load_link<float, long long>(U, S, k, s, a);
  load_link<float, long long>(U, S, j, sk, b);
  mul_nn(a, b, B);
  float d2 = 0.f;
#pragma unroll
  for (int e = 0; e < 9; e++) {
    const float dr = A.e[e].re - B.e[e].re, di = A.e[e].im - B.e[e].im;
    d2 = fmaf(dr, dr, fmaf(di, di, d2));
  }
  return d2;
}

// n(u) = ||u||_F^2 - 3 in FP64 (every float x float product is exact in FP64)
__device__ __forceinline__ double link_norm_dev(const cx<float>* __restrict__ U, long long S, int mu, long long s) {
  const cx<float>* p = U + (long long)(mu * 9) * S + s;
  double n = -3.0;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const cx<float> v = p[(long long)k * S];
    n = fma((double)v.re, (double)v.re, fma((double)v.im, (double)v.im, n));
  }
  return n;
}

template <typename T>
__global__ void __launch_bounds__(kRedThreads) bulk_kernel(Geometry g, FieldPtrs<T> f, double* partials) {
  double v[7] = {0, 0, 0, 0, 0, 0, 0};
  const bool is_max[7] = {false, false, false, false, false, false, false};
  const long long S = g.S;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < g.vol;
       idx += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    decode_vol(g, idx, x, y, z);
    const long long s = idx + g.plane;
    const long long sxp = nbs(g, x, y, z, 1, 0, 0), syp = nbs(g, x, y, z, 0, 1, 0), szp = s + g.plane;
    if constexpr (std::is_same<T, float>::value) {
      // 4 (3 - ReTr P) = 2 ||A - B||^2 - 2 (n(a) + n(b) + n(c) + n(d)).  Summed over the lattice, a
      // plane with two periodic directions counts each of its links twice; in the planes with z
      // (open), the transverse link counts once at slice 0 and once more on the top ghost slice.
      const double nx = link_norm_dev(f.U, S, 0, s), ny = link_norm_dev(f.U, S, 1, s), nz = link_norm_dev(f.U, S, 2, s);
      const double wz = (z == 0) ? 1.0 : 2.0;
      double gx = 0.0, gy = 0.0;
      if (z == g.nz - 1) {
        gx = link_norm_dev(f.U, S, 0, szp);
        gy = link_norm_dev(f.U, S, 1, szp);
      }
      v[2] += 2.0 * (double)plaq_sqdiff_f(f.U, S, 0, 1, s, sxp, syp) - 2.0 * (2.0 * nx + 2.0 * ny);
      v[0] += 2.0 * (double)plaq_sqdiff_f(f.U, S, 1, 2, s, syp, szp) - 2.0 * (2.0 * nz + wz * ny + gy);
      v[1] += 2.0 * (double)plaq_sqdiff_f(f.U, S, 2, 0, s, szp, sxp) - 2.0 * (2.0 * nz + wz * nx + gx);
    } else {
      Mat<double> a, b, c, d;
      // Uxy = U_x(x) U_y(x+x) U_x^d(x+y) U_y^d(x)
      load_link_d(f.U, S, 0, s, a);
      load_link_d(f.U, S, 1, sxp, b);
      load_link_d(f.U, S, 0, syp, c);
      load_link_d(f.U, S, 1, s, d);
      v[2] += 4.0 * (3.0 - retr_plaq(a, b, c, d));
      // Uyz = U_y(x) U_z(x+y) U_y^d(x+z) U_z^d(x)
      load_link_d(f.U, S, 1, s, a);
      load_link_d(f.U, S, 2, syp, b);
      load_link_d(f.U, S, 1, szp, c);
      load_link_d(f.U, S, 2, s, d);
      v[0] += 4.0 * (3.0 - retr_plaq(a, b, c, d));
      // Uzx = U_z(x) U_x(x+z) U_z^d(x+x) U_x^d(x)
      load_link_d(f.U, S, 2, s, a);
      load_link_d(f.U, S, 0, szp, b);
      load_link_d(f.U, S, 2, sxp, c);
      load_link_d(f.U, S, 0, s, d);
      v[1] += 4.0 * (3.0 - retr_plaq(a, b, c, d));
    }
    for (int mu = 0; mu < 3; mu++) {
      Alg<double> e;
      load_alg_d(f.E, S, mu * 8, s, e);
      double q = 0.0;
#pragma unroll
      for (int k = 0; k < 8; k++) q += e.a[k] * e.a[k];
      v[3 + mu] += q;
      if (mu == 2) {
        Alg<double> jp, jm;
        load_alg_d(f.Jp, S, 0, s, jp);
        load_alg_d(f.Jm, S, 0, s, jm);
        double w = 0.0;
#pragma unroll
        for (int k = 0; k < 8; k++) w += e.a[k] * (jp.a[k] - jm.a[k]) * 0.70710678118654752440084436210484903928483593768847;
        v[6] += w;
      }
    }
  }
  block_reduce_store<7>(v, is_max, partials + (long long)blockIdx.x * 7);
}

// Gauss law, per slice: grid (kZChunks, nz).  Partials per (z, chunk): {sum G^2, max |G|}.
template <typename T>
__global__ void __launch_bounds__(kRedThreads) gauss_kernel(Geometry g, FieldPtrs<T> f, double norm, double* partials) {
  double v[2] = {0.0, 0.0};
  const bool is_max[2] = {false, true};
  const int z = blockIdx.y;
  const long long S = g.S;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < g.plane; r += (long long)gridDim.x * blockDim.x) {
    int x, y;
    decode_plane(g, r, x, y);
    const long long s = site_index(g, x, y, z);
    Mat<double> u;
    Alg<double> e, down, tot;
#pragma unroll
    for (int a = 0; a < 8; a++) tot.a[a] = 0.0;
    const long long nbr[3] = {nbs(g, x, y, z, -1, 0, 0), nbs(g, x, y, z, 0, -1, 0), s - g.plane};
    for (int mu = 0; mu < 3; mu++) {
      load_link_d(f.U, S, mu, nbr[mu], u);
      load_alg_d(f.E, S, mu * 8, nbr[mu], e);
      inv_adj_mul(u, e, down);
      load_alg_d(f.E, S, mu * 8, s, e);
#pragma unroll
      for (int a = 0; a < 8; a++) tot.a[a] += (e.a[a] - down.a[a]);
    }
    Alg<double> jp, jm;
    load_alg_d(f.JpStat, S, 0, s, jp);
    load_alg_d(f.JmStat, S, 0, s, jm);
#pragma unroll
    for (int a = 0; a < 8; a++) {
      const double G = norm * (tot.a[a] - (jp.a[a] + jm.a[a]) * 0.70710678118654752440084436210484903928483593768847);
      v[0] += G * G;
      v[1] = fmax(v[1], fabs(G));
    }
  }
  block_reduce_store<2>(v, is_max, partials + ((long long)z * kZChunks + blockIdx.x) * 2);
}

template <typename T>
__global__ void __launch_bounds__(kRedThreads) unitarity_kernel(Geometry g, const cx<T>* U, double* partials) {
  double v[2] = {0.0, 0.0};
  const bool is_max[2] = {false, true};
  const long long n = g.vol * 3;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int mu = i < g.vol ? 0 : (i < 2 * g.vol ? 1 : 2);
    const long long s = i - (long long)mu * g.vol + g.plane;
    Mat<double> u;
    load_link_d(U, g.S, mu, s, u);
    const double nrm = unitarity_norm(u);
    v[0] += nrm * nrm;
    v[1] = fmax(v[1], nrm);
  }
  block_reduce_store<2>(v, is_max, partials + (long long)blockIdx.x * 2);
}

__device__ __forceinline__ double dot8(const Alg<double>& p, const Alg<double>& q) {
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += p.a[k] * q.a[k];
  return s;
}

// Clover average of the four plaquettes in plane (mu,nu) around x, as COMPUTE_AVG_MAGNETIC_FIELD_STRENGTH
// builds it from the elementary, neighbouring and extended plaquettes (S/CALC/Plaquettes.cpp:83-103).
template <typename T>
__device__ void clover(const Geometry& g, const cx<T>* U, int x, int y, int z, int mu, int nu, Mat<double>& avg) {
  const long long S = g.S;
  int dmu[3] = {0, 0, 0}, dnu[3] = {0, 0, 0};
  dmu[mu] = 1;
  dnu[nu] = 1;
  auto at = [&](int amu, int anu) { return nbs(g, x, y, z, amu * dmu[0] + anu * dnu[0], amu * dmu[1] + anu * dnu[1], amu * dmu[2] + anu * dnu[2]); };
  Mat<double> a, b, c, d, t1, t2, P;
  set_zero(avg);
  // elementary U_{mu nu}(x) = U_mu(x) U_nu(x+mu) U_mu^d(x+nu) U_nu^d(x)            (UUDD)
  load_link_d(U, S, mu, at(0, 0), a);
  load_link_d(U, S, nu, at(1, 0), b);
  load_link_d(U, S, mu, at(0, 1), c);
  load_link_d(U, S, nu, at(0, 0), d);
  mul_nn(a, b, t1);
  mul_dd(c, d, t2);
  mul_nn(t1, t2, P);
  for (int k = 0; k < 9; k++) { avg.e[k].re += P.e[k].re; avg.e[k].im += P.e[k].im; }
  // U_{-mu nu}(x) = U_nu(x) U_mu^d(x+nu-mu) U_nu^d(x-mu) U_mu(x-mu)                    (UDDU)
  load_link_d(U, S, nu, at(0, 0), a);
  load_link_d(U, S, mu, at(-1, 1), b);
  load_link_d(U, S, nu, at(-1, 0), c);
  load_link_d(U, S, mu, at(-1, 0), d);
  mul_nd(a, b, t1);
  mul_dn(c, d, t2);
  mul_nn(t1, t2, P);
  for (int k = 0; k < 9; k++) { avg.e[k].re += P.e[k].re; avg.e[k].im += P.e[k].im; }
  // U_{mu -nu}(x) = U_nu^d(x-nu) U_mu(x-nu) U_nu(x-nu+mu) U_mu^d(x)                    (DUUD)
  load_link_d(U, S, nu, at(0, -1), a);
  load_link_d(U, S, mu, at(0, -1), b);
  load_link_d(U, S, nu, at(1, -1), c);
  load_link_d(U, S, mu, at(0, 0), d);
  mul_dn(a, b, t1);
  mul_nd(c, d, t2);
  mul_nn(t1, t2, P);
  for (int k = 0; k < 9; k++) { avg.e[k].re += P.e[k].re; avg.e[k].im += P.e[k].im; }
  // U_{-mu -nu}(x) = U_mu^d(x-mu) U_nu^d(x-mu-nu) U_mu(x-mu-nu) U_nu(x-nu)             (DDUU)
  load_link_d(U, S, mu, at(-1, 0), a);
  load_link_d(U, S, nu, at(-1, -1), b);
  load_link_d(U, S, mu, at(-1, -1), c);
  load_link_d(U, S, nu, at(0, -1), d);
  mul_dd(a, b, t1);
  mul_nn(c, d, t2);
  mul_nn(t1, t2, P);
  for (int k = 0; k < 9; k++) { avg.e[k].re += P.e[k].re; avg.e[k].im += P.e[k].im; }
  for (int k = 0; k < 9; k++) { avg.e[k].re *= 0.25; avg.e[k].im *= 0.25; }
}

// Energy-momentum tensor map, grid (kZChunks, nz); partials per (z, chunk): 10 sums.
template <typename T>
__global__ void __launch_bounds__(kRedThreads) emt_kernel(Geometry g, FieldPtrs<T> f, double aScale, double* partials) {
  double v[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  const bool is_max[10] = {false, false, false, false, false, false, false, false, false, false};
  const int z = blockIdx.y;
  const long long S = g.S;
  const double a3 = g.a[0] * g.a[1] * g.a[2];
  double q[3];
  for (int mu = 0; mu < 3; mu++) q[mu] = g.a[mu] * aScale * aScale / a3;
  const double inv = 1.0 / ((double)g.nx * g.ny);
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < g.plane; r += (long long)gridDim.x * blockDim.x) {
    int x, y;
    decode_plane(g, r, x, y);
    const long long s = site_index(g, x, y, z);
    // magnetic: clover averages of UOld in the planes yz (B0), zx (B1), xy (B2)
    Alg<double> B[3];
    double Bs[3];
    {
      Mat<double> avg;
      const int planes[3][2] = {{1, 2}, {2, 0}, {0, 1}};
      for (int i = 0; i < 3; i++) {
        clover(g, f.UOld, x, y, z, planes[i][0], planes[i][1], avg);
        retr_itg(avg, 2.0, B[i]);
        Bs[i] = 4.0 * (3.0 - avg.e[0].re - avg.e[4].re - avg.e[8].re);
      }
    }
    // electric: average with the parallel-transported backward neighbour, using U
    Alg<double> Ev[3];
    double Es[3];
    {
      const long long nbr[3] = {nbs(g, x, y, z, -1, 0, 0), nbs(g, x, y, z, 0, -1, 0), s - g.plane};
      for (int mu = 0; mu < 3; mu++) {
        Mat<double> u;
        Alg<double> em, e, down;
        load_link_d(f.U, S, mu, nbr[mu], u);
        load_alg_d(f.E, S, mu * 8, nbr[mu], em);
        inv_adj_mul(u, em, down);
        load_alg_d(f.E, S, mu * 8, s, e);
        double sq = 0.0;
#pragma unroll
        for (int a = 0; a < 8; a++) {
          Ev[mu].a[a] = 0.5 * (e.a[a] + down.a[a]);
          sq += 0.5 * (e.a[a] * e.a[a] + em.a[a] * em.a[a]);
        }
        Es[mu] = sq;
      }
    }
    const double e0 = q[0] * q[0] * Es[0], e1 = q[1] * q[1] * Es[1], e2 = q[2] * q[2] * Es[2];
    const double b0 = q[0] * q[0] * Bs[0], b1 = q[1] * q[1] * Bs[1], b2 = q[2] * q[2] * Bs[2];
    v[0] += (0.5 * (e0 + e1 + e2 + b0 + b1 + b2)) * inv;
    v[1] += (0.5 * ((e1 + e2 + b1 + b2) - (e0 + b0))) * inv;
    v[2] += (0.5 * ((e0 + e2 + b0 + b2) - (e1 + b1))) * inv;
    v[3] += (0.5 * ((e0 + e1 + b0 + b1) - (e2 + b2))) * inv;
    v[4] += (q[1] * q[2] * dot8(Ev[1], B[2]) - q[2] * q[1] * dot8(Ev[2], B[1])) * inv;
    v[5] += (q[2] * q[0] * dot8(Ev[2], B[0]) - q[0] * q[2] * dot8(Ev[0], B[2])) * inv;
    v[6] += (q[0] * q[1] * dot8(Ev[0], B[1]) - q[1] * q[0] * dot8(Ev[1], B[0])) * inv;
    v[7] += (q[0] * q[1] * dot8(Ev[0], Ev[1]) + q[0] * q[1] * dot8(B[0], B[1])) * inv;
    v[8] += (q[1] * q[2] * dot8(Ev[1], Ev[2]) + q[1] * q[2] * dot8(B[1], B[2])) * inv;
    v[9] += (q[2] * q[0] * dot8(Ev[2], Ev[0]) + q[2] * q[0] * dot8(B[2], B[0])) * inv;
  }
  block_reduce_store<10>(v, is_max, partials + ((long long)z * kZChunks + blockIdx.x) * 10);
}

// zprofile[z] = slices[2z] / (Nx Ny)
__global__ void profile_scale_kernel(const double* sl, int nz, double inv, double* out) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  if (z < nz) out[z] = sl[2 * z] * inv;
}

}  // namespace

long long observable_scratch_doubles(const Geometry& g) {
  long long a = (long long)kRedBlocks * 8;
  long long b = (long long)g.nz * kZChunks * 10 + (long long)g.nz * 10;
  return (a > b ? a : b) + 64;
}

static unsigned red_blocks(long long n) {
  long long b = (n + kRedThreads - 1) / kRedThreads;
  return (unsigned)(b < kRedBlocks ? (b < 1 ? 1 : b) : kRedBlocks);
}

template <typename T>
cudaError_t launch_bulk(const Geometry& g, FieldPtrs<T> f, double* partials, double* result7, cudaStream_t stream) {
  const unsigned nb = red_blocks(g.vol);
  bulk_kernel<T><<<nb, kRedThreads, 0, stream>>>(g, f, partials);
  finish_kernel<7><<<1, kRedThreads, 0, stream>>>(partials, (int)nb, 0u, result7);
  return cudaGetLastError();
}

// result2 = {sum G^2, max|G|}; zprofile (device, may be null) = per-slice sum G^2 / (Nx Ny)
template <typename T>
cudaError_t launch_gauss(const Geometry& g, FieldPtrs<T> f, double a_scale, double* partials, double* result2,
                         double* zprofile, cudaStream_t stream) {
  const double norm = a_scale * a_scale * a_scale / (g.a[0] * g.a[1] * g.a[2]);
  dim3 grid(kZChunks, g.nz);
  gauss_kernel<T><<<grid, kRedThreads, 0, stream>>>(g, f, norm, partials);
  double* slices = partials + (long long)g.nz * kZChunks * 2;
  finish_slices_kernel<2><<<(g.nz * 2 + 255) / 256, 256, 0, stream>>>(partials, g.nz, 2u, slices);
  finish_kernel<2><<<1, kRedThreads, 0, stream>>>(slices, g.nz, 2u, result2);
  if (zprofile) {
    profile_scale_kernel<<<(g.nz + 255) / 256, 256, 0, stream>>>(slices, g.nz, 1.0 / ((double)g.nx * g.ny), zprofile);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_unitarity(const Geometry& g, const cx<T>* U, double* partials, double* result2, cudaStream_t stream) {
  const unsigned nb = red_blocks(g.vol * 3);
  unitarity_kernel<T><<<nb, kRedThreads, 0, stream>>>(g, U, partials);
  finish_kernel<2><<<1, kRedThreads, 0, stream>>>(partials, (int)nb, 2u, result2);
  return cudaGetLastError();
}

// result (device) = Nz x 10
template <typename T>
cudaError_t launch_emt_map(const Geometry& g, FieldPtrs<T> f, double a_scale, double* partials, double* result,
                           cudaStream_t stream) {
  dim3 grid(kZChunks, g.nz);
  emt_kernel<T><<<grid, kRedThreads, 0, stream>>>(g, f, a_scale, partials);
  finish_slices_kernel<10><<<(g.nz * 10 + 255) / 256, 256, 0, stream>>>(partials, g.nz, 0u, result);
  return cudaGetLastError();
}

#define GLASMA_OBS_INSTANTIATE(T)                                                                               \
  template cudaError_t launch_bulk<T>(const Geometry&, FieldPtrs<T>, double*, double*, cudaStream_t);          \
  template cudaError_t launch_gauss<T>(const Geometry&, FieldPtrs<T>, double, double*, double*, double*,       \
                                       cudaStream_t);                                                           \
  template cudaError_t launch_unitarity<T>(const Geometry&, const cx<T>*, double*, double*, cudaStream_t);     \
  template cudaError_t launch_emt_map<T>(const Geometry&, FieldPtrs<T>, double, double*, double*, cudaStream_t);

GLASMA_OBS_INSTANTIATE(double)
GLASMA_OBS_INSTANTIATE(float)

}  // namespace glasma

// glasma_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the reference's SU(3) glasma hot path, used as the parity
// checker for the CUDA library and as the timed CPU baseline ("port").  It is
// never linked into, loaded by or called from the product library.
//
// Everything here works on the reference's own host layout (AoS, one ghost
// slice below z=0 and one above z=Nz-1):
//   site index   s(x,y,z) = x + Nx*(y + Ny*(z+1)), x,y periodic, z in [-1,Nz]
//                (S/SUNcIndexing.cpp:82, S/LATTICE/GaugeLinks.cpp:27-36)
//   links        U[9*(mu+3*s) + i+3*j]   complex double, column-major i+3j
//                (S/LATTICE/GaugeLinks.cpp:38-41, S/SUNc/SU3/GroupOperations.cpp:13-15)
//   E field      E[a+8*(mu+3*s)]         (S/LATTICE/ElectricFields.cpp:31-35)
//   currents     J[a+8*s]                (S/LATTICE/ChargeDensity.cpp:24-33)
//   gauge trafo  G[9*s + i+3*j]          (S/LATTICE/GaugeTransformations.cpp:25-38)
// Paths below are relative to the reference's SourceCode directory (S/).
//
// The one deliberate algorithmic substitution: exp(i c t^a alpha^a) is computed
// with the Cayley-Hamilton closed form of Morningstar & Peardon (PRD 69 (2004)
// 054501) instead of the reference's Hermitian eigen-decomposition
// (S/SUNc/SU3/AlgebraOperations.cpp:48-89).  Both are exact up to rounding; the
// harness in oracle/ref pins the difference against the compiled reference.
//
// The SU(3) adjoint actions and the matrix logarithm are absent from the
// reference for SU(3) (only the SU(2) forms exist, S/SUNc/SU2/AlgebraOperations.cpp:90-124);
// they are restated here from their definitions:
//   AdjointMultiplication(V,e)        = 2 tr(t^a V (t.e) V^dagger)
//   InverseAdjointMultiplication(V,e) = 2 tr(t^a V^dagger (t.e) V)

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>
#include <omp.h>

typedef std::complex<double> cplx;

namespace {

const double kSqrt3 = 1.7320508075688772935274463415058723669428;
const double kSqrt2 = 1.4142135623730950488016887242096980785697;

struct Lat {
  int N[3];
  double a[3];
  double aScale;
  long plane() const { return (long)N[0] * N[1]; }
  long volume() const { return plane() * N[2]; }
  long total() const { return plane() * (N[2] + 2); }
  long s(int x, int y, int z) const {
    int xm = (x % N[0] + N[0]) % N[0];
    int ym = (y % N[1] + N[1]) % N[1];
    return xm + (long)N[0] * (ym + (long)N[1] * (z + 1));
  }
  double aCube() const { return a[0] * a[1] * a[2]; }
};

inline cplx* L(cplx* U, const Lat& l, int x, int y, int z, int mu) { return U + 9 * (mu + 3 * l.s(x, y, z)); }
inline const cplx* L(const cplx* U, const Lat& l, int x, int y, int z, int mu) { return U + 9 * (mu + 3 * l.s(x, y, z)); }
inline double* EF(double* E, const Lat& l, int x, int y, int z, int mu) { return E + 8 * (mu + 3 * l.s(x, y, z)); }
inline const double* EF(const double* E, const Lat& l, int x, int y, int z, int mu) { return E + 8 * (mu + 3 * l.s(x, y, z)); }
inline double* JF(double* J, const Lat& l, int x, int y, int z) { return J + 8 * l.s(x, y, z); }
inline const double* JF(const double* J, const Lat& l, int x, int y, int z) { return J + 8 * l.s(x, y, z); }
inline cplx* GF(cplx* G, const Lat& l, int x, int y, int z) { return G + 9 * l.s(x, y, z); }

// ---------------------------------------------------------------- SU(3) algebra
inline int mi(int i, int j) { return i + 3 * j; }

// C = A B   (S/SUNc/SU3/GroupOperations.cpp:133-147, "UU")
void mul_nn(const cplx* A, const cplx* B, cplx* C) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      cplx acc = 0.0;
      for (int k = 0; k < 3; k++) acc += A[mi(i, k)] * B[mi(k, j)];
      C[mi(i, j)] = acc;
    }
}
// C = A B^dagger ("UD", :150-164)
void mul_nd(const cplx* A, const cplx* B, cplx* C) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      cplx acc = 0.0;
      for (int k = 0; k < 3; k++) acc += A[mi(i, k)] * std::conj(B[mi(j, k)]);
      C[mi(i, j)] = acc;
    }
}
// C = A^dagger B ("DU", :166-180)
void mul_dn(const cplx* A, const cplx* B, cplx* C) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      cplx acc = 0.0;
      for (int k = 0; k < 3; k++) acc += std::conj(A[mi(k, i)]) * B[mi(k, j)];
      C[mi(i, j)] = acc;
    }
}
// C = A^dagger B^dagger ("DD", :182-196)
void mul_dd(const cplx* A, const cplx* B, cplx* C) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      cplx acc = 0.0;
      for (int k = 0; k < 3; k++) acc += std::conj(A[mi(k, i)]) * std::conj(B[mi(j, k)]);
      C[mi(i, j)] = acc;
    }
}
// V1 V2 V3^d V4^d, grouped as (V1 V2)(V3^d V4^d)   (S/SUNc/AdvancedOperations.cpp:175-186)
void uudd(const cplx* a, const cplx* b, const cplx* c, const cplx* d, cplx* out) {
  cplx t1[9], t2[9];
  mul_nn(a, b, t1);
  mul_dd(c, d, t2);
  mul_nn(t1, t2, out);
}
// V1 V2^d V3^d V4, grouped as (V1 V2^d)(V3^d V4)   (:203-214)
void uddu(const cplx* a, const cplx* b, const cplx* c, const cplx* d, cplx* out) {
  cplx t1[9], t2[9];
  mul_nd(a, b, t1);
  mul_dn(c, d, t2);
  mul_nn(t1, t2, out);
}
// V1^d V2 V3 V4^d, grouped as (V1^d V2)(V3 V4^d)   (:217-228)
void duud(const cplx* a, const cplx* b, const cplx* c, const cplx* d, cplx* out) {
  cplx t1[9], t2[9];
  mul_dn(a, b, t1);
  mul_nd(c, d, t2);
  mul_nn(t1, t2, out);
}
// V1^d V2^d V3 V4, grouped as (V1^d V2^d)(V3 V4)   (:189-200)
void dduu(const cplx* a, const cplx* b, const cplx* c, const cplx* d, cplx* out) {
  cplx t1[9], t2[9];
  mul_dd(a, b, t1);
  mul_nn(c, d, t2);
  mul_nn(t1, t2, out);
}
// V1 V2 V3^d  (:77-88)
void uud(const cplx* a, const cplx* b, const cplx* c, cplx* out) {
  cplx t1[9];
  mul_nn(a, b, t1);
  mul_nd(t1, c, out);
}

// out_a = Re tr(i t^a V), t^a = lambda^a/2 (Gell-Mann)   (S/SUNc/SU3/GroupOperations.cpp:93-103)
void retr_itg(const cplx* V, double* out, double c = 1.0) {
  const double h = -0.5 * c;
  out[0] = h * (V[mi(0, 1)].imag() + V[mi(1, 0)].imag());
  out[1] = h * (V[mi(0, 1)].real() - V[mi(1, 0)].real());
  out[2] = h * (V[mi(0, 0)].imag() - V[mi(1, 1)].imag());
  out[3] = h * (V[mi(0, 2)].imag() + V[mi(2, 0)].imag());
  out[4] = h * (V[mi(0, 2)].real() - V[mi(2, 0)].real());
  out[5] = h * (V[mi(1, 2)].imag() + V[mi(2, 1)].imag());
  out[6] = h * (V[mi(1, 2)].real() - V[mi(2, 1)].real());
  out[7] = h * (V[mi(0, 0)].imag() + V[mi(1, 1)].imag() - 2.0 * V[mi(2, 2)].imag()) / kSqrt3;
}
double retr(const cplx* V) { return V[0].real() + V[4].real() + V[8].real(); }
// Re tr(1 - V)  (:71-73)
double retr_1m(const cplx* V) { return 3.0 - V[0].real() - V[4].real() - V[8].real(); }

// M = t^a alpha^a, Hermitian traceless   (S/SUNc/SU3/AlgebraOperations.cpp:31-45)
void alg_to_herm(const double* al, cplx* M) {
  M[mi(0, 0)] = 0.5 * (al[2] + al[7] / kSqrt3);
  M[mi(1, 1)] = -0.5 * (al[2] - al[7] / kSqrt3);
  M[mi(2, 2)] = -al[7] / kSqrt3;
  M[mi(1, 0)] = 0.5 * cplx(al[0], al[1]);
  M[mi(2, 0)] = 0.5 * cplx(al[3], al[4]);
  M[mi(2, 1)] = 0.5 * cplx(al[5], al[6]);
  M[mi(0, 1)] = std::conj(M[mi(1, 0)]);
  M[mi(0, 2)] = std::conj(M[mi(2, 0)]);
  M[mi(1, 2)] = std::conj(M[mi(2, 1)]);
}
// out_a = 2 tr(t^a W) for Hermitian W (inverse of alg_to_herm)
void herm_to_alg(const cplx* W, double* out) {
  out[0] = 2.0 * W[mi(0, 1)].real();
  out[1] = -2.0 * W[mi(0, 1)].imag();
  out[2] = W[mi(0, 0)].real() - W[mi(1, 1)].real();
  out[3] = 2.0 * W[mi(0, 2)].real();
  out[4] = -2.0 * W[mi(0, 2)].imag();
  out[5] = 2.0 * W[mi(1, 2)].real();
  out[6] = -2.0 * W[mi(1, 2)].imag();
  out[7] = (W[mi(0, 0)].real() + W[mi(1, 1)].real() - 2.0 * W[mi(2, 2)].real()) / kSqrt3;
}
// V (t.e) V^dagger   -- SU(3) AdjointMultiplication (absent in the reference; the
// SU(2) form S/SUNc/SU2/AlgebraOperations.cpp:110-116 fixes the convention)
void adj_mul(const cplx* V, const double* e, double* out) {
  cplx M[9], T[9], W[9];
  alg_to_herm(e, M);
  mul_nn(V, M, T);
  mul_nd(T, V, W);
  herm_to_alg(W, out);
}
// V^dagger (t.e) V   -- SU(3) InverseAdjointMultiplication (SU(2) form :118-124)
void inv_adj_mul(const cplx* V, const double* e, double* out) {
  cplx M[9], T[9], W[9];
  alg_to_herm(e, M);
  mul_dn(V, M, T);
  mul_nn(T, V, W);
  herm_to_alg(W, out);
}

// exp(i c t^a alpha^a) by the Cayley-Hamilton closed form (Morningstar & Peardon 2004).
// Same contract as MatrixIExp (S/SUNc/SU3/AlgebraOperations.cpp:48-89).
void expi(double c, const double* al, cplx* out) {
  cplx Q[9], Q2[9];
  double sc[8];
  for (int a = 0; a < 8; a++) sc[a] = c * al[a];
  alg_to_herm(sc, Q);
  mul_nn(Q, Q, Q2);
  const double c1 = 0.5 * (Q2[0].real() + Q2[4].real() + Q2[8].real());
  // det Q (real for Hermitian Q)
  const cplx det = Q[mi(0, 0)] * (Q[mi(1, 1)] * Q[mi(2, 2)] - Q[mi(1, 2)] * Q[mi(2, 1)]) -
                   Q[mi(0, 1)] * (Q[mi(1, 0)] * Q[mi(2, 2)] - Q[mi(1, 2)] * Q[mi(2, 0)]) +
                   Q[mi(0, 2)] * (Q[mi(1, 0)] * Q[mi(2, 1)] - Q[mi(1, 1)] * Q[mi(2, 0)]);
  double c0 = det.real();
  cplx f0, f1, f2;
  if (c1 < 1e-6) {
    // Taylor series through (iQ)^6, reduced with Q^3 = c1 Q + c0.
    f0 = cplx(1.0 - c0 * c0 / 720.0, -c0 / 6.0 + c1 * c0 / 120.0);
    f1 = cplx(c0 / 24.0 - c0 * c1 / 360.0, 1.0 - c1 / 6.0 + c1 * c1 / 120.0);
    f2 = cplx(-0.5 + c1 / 24.0 - c1 * c1 / 720.0, c0 / 120.0);
  } else {
    const bool neg = c0 < 0.0;
    if (neg) c0 = -c0;
    const double c0max = 2.0 * std::pow(c1 / 3.0, 1.5);
    double r = c0 / c0max;
    if (r > 1.0) r = 1.0;
    const double theta = std::acos(r);
    const double u = std::sqrt(c1 / 3.0) * std::cos(theta / 3.0);
    const double w = std::sqrt(c1) * std::sin(theta / 3.0);
    const double w2 = w * w, u2 = u * u;
    double xi0;
    if (std::fabs(w) < 0.05)
      xi0 = 1.0 - w2 / 6.0 * (1.0 - w2 / 20.0 * (1.0 - w2 / 42.0 * (1.0 - w2 / 72.0)));
    else
      xi0 = std::sin(w) / w;
    const double cw = std::cos(w);
    const cplx e2iu(std::cos(2.0 * u), std::sin(2.0 * u));
    const cplx emiu(std::cos(u), -std::sin(u));
    const cplx h0 = (u2 - w2) * e2iu + emiu * cplx(8.0 * u2 * cw, 2.0 * u * (3.0 * u2 + w2) * xi0);
    const cplx h1 = 2.0 * u * e2iu - emiu * cplx(2.0 * u * cw, -(3.0 * u2 - w2) * xi0);
    const cplx h2 = e2iu - emiu * cplx(cw, 3.0 * u * xi0);
    const double den = 1.0 / (9.0 * u2 - w2);
    f0 = h0 * den;
    f1 = h1 * den;
    f2 = h2 * den;
    if (neg) {
      f0 = std::conj(f0);
      f1 = -std::conj(f1);
      f2 = std::conj(f2);
    }
  }
  for (int k = 0; k < 9; k++) out[k] = f1 * Q[k] + f2 * Q2[k];
  out[0] += f0;
  out[4] += f0;
  out[8] += f0;
}

// || V V^dagger - 1 ||_F  (S/SUNc/SU3/GroupOperations.cpp:337-349)
double unitarity_norm(const cplx* V) {
  cplx C[9];
  mul_nd(V, V, C);
  double n = 0.0;
  for (int k = 0; k < 9; k++) {
    cplx d = C[k] - ((k % 4 == 0) ? 1.0 : 0.0);
    n += std::norm(d);
  }
  return std::sqrt(n);
}

// ------------------------------------------------------------- ghost slices
// Open z boundary: slice -1 <- slice 0, slice Nz <- slice Nz-1
// (S/LATTICE/GaugeLinks.cpp:59-66, ElectricFields.cpp:51-57, ChargeDensity.cpp:24-30,
//  GaugeTransformations.cpp:40-46)
template <typename T>
void sync_ghosts(T* F, const Lat& l, long per_site) {
  const long n = l.plane() * per_site;
  std::memcpy(F + l.s(0, 0, -1) * per_site, F + l.s(0, 0, 0) * per_site, n * sizeof(T));
  std::memcpy(F + l.s(0, 0, l.N[2]) * per_site, F + l.s(0, 0, l.N[2] - 1) * per_site, n * sizeof(T));
}
void sync_U(cplx* U, const Lat& l) { sync_ghosts(U, l, 27); }
void sync_E(double* E, const Lat& l) { sync_ghosts(E, l, 24); }
void sync_J(double* J, const Lat& l) { sync_ghosts(J, l, 8); }
void sync_G(cplx* G, const Lat& l) { sync_ghosts(G, l, 9); }

// ------------------------------------------------------------- leapfrog
// Dynamics::SUNc::UpdateElectricFields  (S/DYNAMICS/SUNcDynamics.cpp:134-203)
// with the plaquette macros of S/CALC/Plaquettes.cpp:83-128.
void update_efield(const Lat& l, cplx* U, double* E, const double* Jp, const double* Jm, double dt) {
  const double gamma = -2.0 * dt * l.aCube();
  double cE[3];
  for (int mu = 0; mu < 3; mu++) cE[mu] = 1.0 / (l.a[mu] * l.a[mu]);
  sync_U(U, l);
  const int Nx = l.N[0], Ny = l.N[1], Nz = l.N[2];
#pragma omp parallel for schedule(static)
  for (int z = 0; z < Nz; z++)
    for (int y = 0; y < Ny; y++)
      for (int x = 0; x < Nx; x++) {
        cplx Uxy[9], Uyz[9], Uzx[9], UMxy[9], UMyz[9], UMzx[9], UxMy[9], UyMz[9], UzMx[9];
        uudd(L(U, l, x, y, z, 0), L(U, l, x + 1, y, z, 1), L(U, l, x, y + 1, z, 0), L(U, l, x, y, z, 1), Uxy);
        uudd(L(U, l, x, y, z, 1), L(U, l, x, y + 1, z, 2), L(U, l, x, y, z + 1, 1), L(U, l, x, y, z, 2), Uyz);
        uudd(L(U, l, x, y, z, 2), L(U, l, x, y, z + 1, 0), L(U, l, x + 1, y, z, 2), L(U, l, x, y, z, 0), Uzx);
        uddu(L(U, l, x, y, z, 1), L(U, l, x - 1, y + 1, z, 0), L(U, l, x - 1, y, z, 1), L(U, l, x - 1, y, z, 0), UMxy);
        uddu(L(U, l, x, y, z, 2), L(U, l, x, y - 1, z + 1, 1), L(U, l, x, y - 1, z, 2), L(U, l, x, y - 1, z, 1), UMyz);
        uddu(L(U, l, x, y, z, 0), L(U, l, x + 1, y, z - 1, 2), L(U, l, x, y, z - 1, 0), L(U, l, x, y, z - 1, 2), UMzx);
        duud(L(U, l, x, y - 1, z, 1), L(U, l, x, y - 1, z, 0), L(U, l, x + 1, y - 1, z, 1), L(U, l, x, y, z, 0), UxMy);
        duud(L(U, l, x, y, z - 1, 2), L(U, l, x, y, z - 1, 1), L(U, l, x, y + 1, z - 1, 2), L(U, l, x, y, z, 1), UyMz);
        duud(L(U, l, x - 1, y, z, 0), L(U, l, x - 1, y, z, 2), L(U, l, x - 1, y, z + 1, 0), L(U, l, x, y, z, 2), UzMx);
        double Txy[8], Tyz[8], Tzx[8], TMxy[8], TMyz[8], TMzx[8], TxMy[8], TyMz[8], TzMx[8];
        retr_itg(Uxy, Txy); retr_itg(Uyz, Tyz); retr_itg(Uzx, Tzx);
        retr_itg(UMxy, TMxy); retr_itg(UMyz, TMyz); retr_itg(UMzx, TMzx);
        retr_itg(UxMy, TxMy); retr_itg(UyMz, TyMz); retr_itg(UzMx, TzMx);
        double* Ex = EF(E, l, x, y, z, 0);
        double* Ey = EF(E, l, x, y, z, 1);
        double* Ez = EF(E, l, x, y, z, 2);
        for (int a = 0; a < 8; a++) {
          Ex[a] += gamma * cE[0] * (cE[1] * (Txy[a] - TxMy[a]) - cE[2] * (Tzx[a] - TMzx[a]));
          Ey[a] += gamma * cE[1] * (cE[2] * (Tyz[a] - TyMz[a]) - cE[0] * (Txy[a] - TMxy[a]));
          Ez[a] += gamma * cE[2] * (cE[0] * (Tzx[a] - TzMx[a]) - cE[1] * (Tyz[a] - TMyz[a]));
        }
        const double* jp = JF(Jp, l, x, y, z);
        const double* jm = JF(Jm, l, x, y, z);
        for (int a = 0; a < 8; a++) Ez[a] += -(dt / l.a[2]) * ((jp[a] - jm[a]) / kSqrt2);
      }
  sync_E(E, l);
}

// Dynamics::SUNc::UpdateJStat  (S/DYNAMICS/SUNcDynamics.cpp:205-236)
void update_jstat(const Lat& l, const cplx* U, double* JpStat, double* JmStat, const double* Jp, const double* Jm, double dt) {
  const int Nx = l.N[0], Ny = l.N[1], Nz = l.N[2];
  const double c = dt / l.a[2];
#pragma omp parallel for schedule(static)
  for (int z = 0; z < Nz; z++)
    for (int y = 0; y < Ny; y++)
      for (int x = 0; x < Nx; x++) {
        double pd[8], md[8];
        inv_adj_mul(L(U, l, x, y, z - 1, 2), JF(Jp, l, x, y, z - 1), pd);
        inv_adj_mul(L(U, l, x, y, z - 1, 2), JF(Jm, l, x, y, z - 1), md);
        double* ps = JF(JpStat, l, x, y, z);
        double* ms = JF(JmStat, l, x, y, z);
        const double* jp = JF(Jp, l, x, y, z);
        const double* jm = JF(Jm, l, x, y, z);
        for (int a = 0; a < 8; a++) {
          ps[a] += -c * (jp[a] - pd[a]);
          ms[a] += c * (jm[a] - md[a]);
        }
      }
  sync_J(JmStat, l);
  sync_J(JpStat, l);
}

// Dynamics::SUNc::UpdateJ  (S/DYNAMICS/SUNcDynamics.cpp:238-269)
void update_j(const Lat& l, const cplx* U, double* Jp, double* Jm, const double* JpStat, const double* JmStat, double dt) {
  const int Nx = l.N[0], Ny = l.N[1], Nz = l.N[2];
  const double c = dt / l.a[2];
#pragma omp parallel for schedule(static)
  for (int z = 0; z < Nz; z++)
    for (int y = 0; y < Ny; y++)
      for (int x = 0; x < Nx; x++) {
        double pu[8], mu_[8];
        adj_mul(L(U, l, x, y, z, 2), JF(JpStat, l, x, y, z + 1), pu);
        adj_mul(L(U, l, x, y, z, 2), JF(JmStat, l, x, y, z + 1), mu_);
        double* jp = JF(Jp, l, x, y, z);
        double* jm = JF(Jm, l, x, y, z);
        const double* ps = JF(JpStat, l, x, y, z);
        const double* ms = JF(JmStat, l, x, y, z);
        for (int a = 0; a < 8; a++) {
          jp[a] += -c * (pu[a] - ps[a]);
          jm[a] += c * (mu_[a] - ms[a]);
        }
      }
  sync_J(Jm, l);
  sync_J(Jp, l);
}

// Dynamics::SUNc::UpdateGaugeLinks  (S/DYNAMICS/SUNcDynamics.cpp:62-106)
void update_links(const Lat& l, cplx* U, const double* E, double dt) {
  double cU[3];
  for (int mu = 0; mu < 3; mu++) cU[mu] = -dt * l.a[mu] * l.a[mu] / l.aCube();
  const int Nx = l.N[0], Ny = l.N[1], Nz = l.N[2];
#pragma omp parallel for schedule(static)
  for (int z = 0; z < Nz; z++)
    for (int y = 0; y < Ny; y++)
      for (int x = 0; x < Nx; x++)
        for (int mu = 0; mu < 3; mu++) {
          cplx X[9], old[9];
          expi(cU[mu], EF(E, l, x, y, z, mu), X);
          cplx* u = L(U, l, x, y, z, mu);
          std::memcpy(old, u, sizeof(old));
          mul_nn(X, old, u);
        }
  sync_U(U, l);
}

// Dynamics::SUNc::SaveOldLink  (S/DYNAMICS/SUNcDynamics.cpp:108-128)
void save_old_link(const Lat& l, cplx* U, cplx* UOld) {
  sync_U(U, l);
  std::memcpy(UOld + 27 * l.s(0, 0, 0), U + 27 * l.s(0, 0, 0), sizeof(cplx) * 27 * l.volume());
  sync_U(UOld, l);
}

// Dynamics::SUNc::Update  (S/DYNAMICS/SUNcDynamics.cpp:353-378)
void leapfrog_step(const Lat& l, double dt, cplx* U, cplx* UOld, double* E, double* Jp, double* Jm, double* JpStat, double* JmStat) {
  update_efield(l, U, E, Jp, Jm, dt);
  update_jstat(l, U, JpStat, JmStat, Jp, Jm, dt);
  update_links(l, U, E, 0.5 * dt);
  if (UOld) save_old_link(l, U, UOld);
  update_j(l, U, Jp, Jm, JpStat, JmStat, dt);
  update_links(l, U, E, 0.5 * dt);
}

// ------------------------------------------------------------- FFT (oracle-only)
// Unnormalised complex DFT, sign -1 forward / +1 backward, the convention of
// FFTW's fftw_plan_many_dft as used by S/FFT/FFT3D.cpp:126-138.  Radix-2 for
// powers of two, direct DFT otherwise.
void fft1d_inplace(cplx* a, int n, int sign, std::vector<cplx>& scratch) {
  if (n <= 1) return;
  if ((n & (n - 1)) == 0) {
    for (int i = 1, j = 0; i < n; i++) {
      int bit = n >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) std::swap(a[i], a[j]);
    }
    for (int len = 2; len <= n; len <<= 1) {
      const double ang = sign * 2.0 * M_PI / len;
      for (int i = 0; i < n; i += len)
        for (int k = 0; k < len / 2; k++) {
          const cplx w(std::cos(ang * k), std::sin(ang * k));
          const cplx u = a[i + k], v = a[i + k + len / 2] * w;
          a[i + k] = u + v;
          a[i + k + len / 2] = u - v;
        }
    }
  } else {
    scratch.assign(n, cplx(0.0));
    for (int k = 0; k < n; k++) {
      cplx acc = 0.0;
      for (int j = 0; j < n; j++) {
        const long m = ((long)j * k) % n;
        const double ang = sign * 2.0 * M_PI * (double)m / n;
        acc += a[j] * cplx(std::cos(ang), std::sin(ang));
      }
      scratch[k] = acc;
    }
    for (int k = 0; k < n; k++) a[k] = scratch[k];
  }
}

// 3D transform of nc interleaved components: X[a + nc*(x + Nx*(y + Ny*z))]
// (index convention of S/FFT/FFT3D.cpp:41-47).
void fft3d(cplx* X, const int N[3], int nc, int sign) {
  const long Nx = N[0], Ny = N[1], Nz = N[2];
  // along x
#pragma omp parallel
  {
    std::vector<cplx> line, scratch;
#pragma omp for collapse(2)
    for (long z = 0; z < Nz; z++)
      for (long y = 0; y < Ny; y++)
        for (int a = 0; a < nc; a++) {
          line.resize(Nx);
          for (long x = 0; x < Nx; x++) line[x] = X[a + nc * (x + Nx * (y + Ny * z))];
          fft1d_inplace(line.data(), (int)Nx, sign, scratch);
          for (long x = 0; x < Nx; x++) X[a + nc * (x + Nx * (y + Ny * z))] = line[x];
        }
#pragma omp for collapse(2)
    for (long z = 0; z < Nz; z++)
      for (long x = 0; x < Nx; x++)
        for (int a = 0; a < nc; a++) {
          line.resize(Ny);
          for (long y = 0; y < Ny; y++) line[y] = X[a + nc * (x + Nx * (y + Ny * z))];
          fft1d_inplace(line.data(), (int)Ny, sign, scratch);
          for (long y = 0; y < Ny; y++) X[a + nc * (x + Nx * (y + Ny * z))] = line[y];
        }
#pragma omp for collapse(2)
    for (long y = 0; y < Ny; y++)
      for (long x = 0; x < Nx; x++)
        for (int a = 0; a < nc; a++) {
          line.resize(Nz);
          for (long z = 0; z < Nz; z++) line[z] = X[a + nc * (x + Nx * (y + Ny * z))];
          fft1d_inplace(line.data(), (int)Nz, sign, scratch);
          for (long z = 0; z < Nz; z++) X[a + nc * (x + Nx * (y + Ny * z))] = line[z];
        }
  }
}

// ------------------------------------------------------------- gauge transforms
// GaugeTransformation::Operations::GaugeTransformLinks  (S/GAUGETRANSFORMATION/GaugeTransformation.cpp:111-124)
// with PERFORM_GAUGE_LINK_TRANSFORMATION (S/CALC/GaugeTransformation.cpp:5-9):
// UG_mu(x) = G(x) U_mu(x) G^dagger(x+mu).  G(x,y,Nz) is the ghost as it stands; G is synced afterwards.
void gauge_transform_links(const Lat& l, const cplx* U, cplx* UG, cplx* G) {
  const int Nx = l.N[0], Ny = l.N[1], Nz = l.N[2];
#pragma omp parallel for schedule(static)
  for (int z = 0; z < Nz; z++)
    for (int y = 0; y < Ny; y++)
      for (int x = 0; x < Nx; x++) {
        uud(GF(G, l, x, y, z), L(U, l, x, y, z, 0), GF(G, l, x + 1, y, z), L(UG, l, x, y, z, 0));
        uud(GF(G, l, x, y, z), L(U, l, x, y, z, 1), GF(G, l, x, y + 1, z), L(UG, l, x, y, z, 1));
        uud(GF(G, l, x, y, z), L(U, l, x, y, z, 2), GF(G, l, x, y, z + 1), L(UG, l, x, y, z, 2));
      }
  sync_G(G, l);
}
// GaugeTransformElectricFields (S/GAUGETRANSFORMATION/GaugeTransformation.cpp:139-152; S/CALC/GaugeTransformation.cpp:12-17)
void gauge_transform_efield(const Lat& l, const double* E, double* EG, cplx* G) {
  const int Nx = l.N[0], Ny = l.N[1], Nz = l.N[2];
#pragma omp parallel for schedule(static)
  for (int z = 0; z < Nz; z++)
    for (int y = 0; y < Ny; y++)
      for (int x = 0; x < Nx; x++)
        for (int mu = 0; mu < 3; mu++) adj_mul(GF(G, l, x, y, z), EF(E, l, x, y, z, mu), EF(EG, l, x, y, z, mu));
  sync_G(G, l);
}

// PERFORM_COLOR_CHARGE_TRANSFORMATION (S/CALC/GaugeTransformation.cpp:28-31; the current form :20-25
// applies the same action to each spatial component): jG(x) = AdjointMultiplication(G(x), j(x)) on
// the interior slices, the ghost slices copied from the edge slices as SynchronizeGhostCells does.
void gauge_transform_charge(const Lat& l, const cplx* G, const double* J, double* JG) {
  const int Nx = l.N[0], Ny = l.N[1], Nz = l.N[2];
#pragma omp parallel for schedule(static)
  for (int z = 0; z < Nz; z++)
    for (int y = 0; y < Ny; y++)
      for (int x = 0; x < Nx; x++) adj_mul(G + 9 * l.s(x, y, z), JF(J, l, x, y, z), JF(JG, l, x, y, z));
  for (int y = 0; y < Ny; y++)
    for (int x = 0; x < Nx; x++)
      for (int a = 0; a < 8; a++) {
        JF(JG, l, x, y, -1)[a] = JF(JG, l, x, y, 0)[a];
        JF(JG, l, x, y, Nz)[a] = JF(JG, l, x, y, Nz - 1)[a];
      }
}

// ------------------------------------------------------------- Coulomb gauge deviation at one site
// GET_LOCAL_GAUGE_VIOLATION (S/GAUGETRANSFORMATION/CoulombGaugeDeviation.cpp:23-41):
// w(x) = sum_mu c_mu (UG_mu(x) + UG_mu^dagger(x - mu)), the z term only if Nz > 1; Delta^a = ReTr(i t^a w).
// open_top != 0 (the open-z functional, a documented variant): the forward z link of the top slice,
// which points into the ghost slice, is left out, so Delta is the gradient of
// F = sum over links with both ends in [0, Nz-1] of Re tr UG.
void gauge_deviation(const Lat& l, const cplx* UG, int x, int y, int z, const double* cw, cplx* w, double* dev,
                     int open_top = 0) {
  const double zterm = l.N[2] > 1 ? 1.0 : 0.0;
  const double ztop = (open_top && z == l.N[2] - 1) ? 0.0 : 1.0;
  const cplx* u0 = L(UG, l, x, y, z, 0);
  const cplx* u1 = L(UG, l, x, y, z, 1);
  const cplx* u2 = L(UG, l, x, y, z, 2);
  const cplx* d0 = L(UG, l, x - 1, y, z, 0);
  const cplx* d1 = L(UG, l, x, y - 1, z, 1);
  const cplx* d2 = L(UG, l, x, y, z - 1, 2);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      const int k = mi(i, j), kt = mi(j, i);
      w[k] = cw[0] * (u0[k] + std::conj(d0[kt])) + cw[1] * (u1[k] + std::conj(d1[kt])) +
             zterm * cw[2] * (ztop * u2[k] + std::conj(d2[kt]));
    }
  retr_itg(w, dev);
}

// ------------------------------------------------------------- local gauge-fixing updates
// The draw that decides over-relaxation at one site of one checkerboard pass (the reference calls
// RandomNumberGenerator::rng() there, S/GAUGETRANSFORMATION/ALGORITHMS/LosAlamos.cpp:51): a
// counter-based hash of (seed, 2 * iteration + pass, site), so that any implementation draws the
// same number for the same site whatever order it visits the sites in.  The mixing function is the
// splitmix64 finaliser (Steele, Lea & Flood, OOPSLA 2014); the result is uniform in [0, 1).
inline uint64_t gf_mix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double gf_uniform(uint64_t seed, long iteration, int pass, long site) {
  const uint64_t k = gf_mix(seed ^ gf_mix((uint64_t)(2 * iteration + pass)));
  return (double)(gf_mix(k ^ (uint64_t)site) >> 11) * (1.0 / 9007199254740992.0);
}

// One Cabibbo-Marinari step in the SU(2) subgroup of rows/columns (p, q)
// (S/SUNc/SU3/util/CabbiboMarinariProjection.cpp:4-62, CABBIBO_MARINARI_STEP :73-92):
//   A_pp = (V_pp^* + V_qq)/n, A_pq = (V_qp^* - V_pq)/n, A_qp = (V_pq^* - V_qp)/n, A_qq = (V_qq^* + V_pp)/n,
//   n = sqrt(|V_pp^* + V_qq|^2 + |V_qp^* - V_pq|^2), the identity elsewhere; Gc <- A Gc, V <- A V.
// Only rows p and q of Gc and V change.
void cm_subgroup(int p, int q, cplx* Gc, cplx* V) {
  const cplx s = std::conj(V[mi(p, p)]) + V[mi(q, q)];
  const cplx t = std::conj(V[mi(q, p)]) - V[mi(p, q)];
  const double inv = 1.0 / std::sqrt(std::norm(s) + std::norm(t));
  const cplx App = inv * s, Apq = inv * t;
  const cplx Aqp = inv * (std::conj(V[mi(p, q)]) - V[mi(q, p)]), Aqq = inv * (std::conj(V[mi(q, q)]) + V[mi(p, p)]);
  for (cplx* M : {Gc, V})
    for (int j = 0; j < 3; j++) {
      const cplx rp = M[mi(p, j)], rq = M[mi(q, j)];
      M[mi(p, j)] = App * rp + Apq * rq;
      M[mi(q, j)] = Aqp * rp + Aqq * rq;
    }
}
// SUNcGroup::Extended::MaxTraceProjection (S/SUNc/SU3/GroupOperations.cpp:358-378): seven sweeps over
// the subgroups (0,1), (0,2), (1,2) accumulate Gc, which maximises Re tr(Gc w); the result is Gc^dagger.
void max_trace_projection(const cplx* w, cplx* out) {
  cplx Gc[9] = {1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0};
  cplx V[9];
  std::memcpy(V, w, sizeof(V));
  for (int n = 0; n < 7; n++) {
    cm_subgroup(0, 1, Gc, V);
    cm_subgroup(0, 2, Gc, V);
    cm_subgroup(1, 2, Gc, V);
  }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) out[mi(i, j)] = std::conj(Gc[mi(j, i)]);
}

}  // namespace

// =============================================================== C entry points
extern "C" {

static const double kUnitSpacing[3] = {1.0, 1.0, 1.0};

static Lat make_lat(const int* N, const double* a, double aScale) {
  Lat l;
  for (int i = 0; i < 3; i++) {
    l.N[i] = N[i];
    l.a[i] = a[i];
  }
  l.aScale = aScale;
  return l;
}

void oracle_set_threads(int n) { omp_set_num_threads(n); }
int oracle_get_threads() { return omp_get_max_threads(); }

void oracle_expi(double c, const double* alpha, double* out18) { expi(c, alpha, reinterpret_cast<cplx*>(out18)); }
void oracle_adj_mul(const double* V18, const double* e, double* out) { adj_mul(reinterpret_cast<const cplx*>(V18), e, out); }
void oracle_inv_adj_mul(const double* V18, const double* e, double* out) { inv_adj_mul(reinterpret_cast<const cplx*>(V18), e, out); }

void oracle_transform_charge(const int* N, const double* Gin, const double* J, double* JG) {
  Lat l = make_lat(N, kUnitSpacing, 1);
  gauge_transform_charge(l, reinterpret_cast<const cplx*>(Gin), J, JG);
}

void oracle_sync_links(const int* N, double* U) {
  Lat l = make_lat(N, kUnitSpacing, 1);
  sync_U(reinterpret_cast<cplx*>(U), l);
}

// nsteps full Dynamics::SUNc::Update steps; UOld may be null (no SaveOldLink).
void oracle_update(const int* N, const double* a, double dt, int nsteps, double* U, double* UOld, double* E, double* Jp,
                   double* Jm, double* JpStat, double* JmStat) {
  Lat l = make_lat(N, a, 1.0);
  for (int n = 0; n < nsteps; n++)
    leapfrog_step(l, dt, reinterpret_cast<cplx*>(U), reinterpret_cast<cplx*>(UOld), E, Jp, Jm, JpStat, JmStat);
}

void oracle_update_efield(const int* N, const double* a, double dt, double* U, double* E, const double* Jp, const double* Jm) {
  Lat l = make_lat(N, a, 1.0);
  update_efield(l, reinterpret_cast<cplx*>(U), E, Jp, Jm, dt);
}
void oracle_update_links(const int* N, const double* a, double dt, double* U, const double* E) {
  Lat l = make_lat(N, a, 1.0);
  update_links(l, reinterpret_cast<cplx*>(U), E, dt);
}

// Observables::Bulk::Update (S/OBSERVABLES/BulkObservables.cpp:22-183).
// out[0..2] ESqr, out[3..5] BSqr, out[6..8] EDotJ, out[9..15] T00,TXX,TYY,TZZ,ELECTRIC,MAGNETIC,SOURCE
void oracle_bulk(const int* N, const double* a, double aScale, const double* Uin, const double* E, const double* Jp,
                 const double* Jm, double* out) {
  Lat l = make_lat(N, a, aScale);
  const cplx* U = reinterpret_cast<const cplx*>(Uin);
  double cB[3], cE[3], cS[3];
  for (int mu = 0; mu < 3; mu++) {
    const double q = l.a[mu] * aScale * aScale / l.aCube();
    cB[mu] = q * q;
    cE[mu] = q * q;
    cS[mu] = l.a[mu] * aScale / (l.aCube() * l.aCube());
  }
  const int Nx = l.N[0], Ny = l.N[1], Nz = l.N[2];
  double B0 = 0, B1 = 0, B2 = 0, E0 = 0, E1 = 0, E2 = 0, S2 = 0;
#pragma omp parallel for reduction(+ : B0, B1, B2, E0, E1, E2, S2) schedule(static)
  for (int z = 0; z < Nz; z++)
    for (int y = 0; y < Ny; y++)
      for (int x = 0; x < Nx; x++) {
        cplx Uxy[9], Uyz[9], Uzx[9];
        uudd(L(U, l, x, y, z, 0), L(U, l, x + 1, y, z, 1), L(U, l, x, y + 1, z, 0), L(U, l, x, y, z, 1), Uxy);
        uudd(L(U, l, x, y, z, 1), L(U, l, x, y + 1, z, 2), L(U, l, x, y, z + 1, 1), L(U, l, x, y, z, 2), Uyz);
        uudd(L(U, l, x, y, z, 2), L(U, l, x, y, z + 1, 0), L(U, l, x + 1, y, z, 2), L(U, l, x, y, z, 0), Uzx);
        B0 += 4.0 * retr_1m(Uyz);
        B1 += 4.0 * retr_1m(Uzx);
        B2 += 4.0 * retr_1m(Uxy);
        for (int aa = 0; aa < 8; aa++) {
          E0 += EF(E, l, x, y, z, 0)[aa] * EF(E, l, x, y, z, 0)[aa];
          E1 += EF(E, l, x, y, z, 1)[aa] * EF(E, l, x, y, z, 1)[aa];
          E2 += EF(E, l, x, y, z, 2)[aa] * EF(E, l, x, y, z, 2)[aa];
          S2 += EF(E, l, x, y, z, 2)[aa] * (JF(Jp, l, x, y, z)[aa] - JF(Jm, l, x, y, z)[aa]) / kSqrt2;
        }
      }
  const double ES[3] = {E0, E1, E2}, BS[3] = {B0, B1, B2}, ED[3] = {0.0, 0.0, S2};
  for (int i = 0; i < 3; i++) {
    out[i] = ES[i];
    out[3 + i] = BS[i];
    out[6 + i] = ED[i];
  }
  const double e0 = cE[0] * ES[0], e1 = cE[1] * ES[1], e2 = cE[2] * ES[2];
  const double b0 = cB[0] * BS[0], b1 = cB[1] * BS[1], b2 = cB[2] * BS[2];
  out[9] = 0.5 * (e0 + e1 + e2 + b0 + b1 + b2);
  out[10] = 0.5 * ((e1 + e2 + b1 + b2) - (e0 + b0));
  out[11] = 0.5 * ((e0 + e2 + b0 + b2) - (e1 + b1));
  out[12] = 0.5 * ((e0 + e1 + b0 + b1) - (e2 + b2));
  out[13] = 0.5 * (e0 + e1 + e2);
  out[14] = 0.5 * (b0 + b1 + b2);
  out[15] = cS[0] * ED[0] + cS[1] * ED[1] + cS[2] * ED[2];
}

// Observables::GaussLaw::UpdateViolation, global form (S/OBSERVABLES/GaussLawViolation.cpp:75-124)
// and per-z profile form (:16-72), both with COMPUTE_GAUSS_VIOLATION (S/CALC/GaussViolation.cpp:13-23).
// Syncs JpStat, JmStat, U, E ghosts first as the per-z form does (:33-37); the global form
// reads the ghosts as they stand, so sync_first=0 reproduces it exactly.
void oracle_gauss(const int* N, const double* a, double aScale, double* Uin, double* E, double* JpStat, double* JmStat,
                  int sync_first, double* max_out, double* avg_out, double* zprofile) {
  Lat l = make_lat(N, a, aScale);
  cplx* U = reinterpret_cast<cplx*>(Uin);
  if (sync_first) {
    sync_J(JpStat, l);
    sync_J(JmStat, l);
    sync_U(U, l);
    sync_E(E, l);
  }
  const double norm = aScale * aScale * aScale / (l.a[0] * l.a[1] * l.a[2]);
  const int Nx = l.N[0], Ny = l.N[1], Nz = l.N[2];
  double mx = 0.0, sq = 0.0;
#pragma omp parallel for reduction(+ : sq) reduction(max : mx) schedule(static)
  for (int z = 0; z < Nz; z++) {
    double prof = 0.0;
    for (int y = 0; y < Ny; y++)
      for (int x = 0; x < Nx; x++) {
        double ex[8], ey[8], ez[8];
        inv_adj_mul(L(U, l, x - 1, y, z, 0), EF(E, l, x - 1, y, z, 0), ex);
        inv_adj_mul(L(U, l, x, y - 1, z, 1), EF(E, l, x, y - 1, z, 1), ey);
        inv_adj_mul(L(U, l, x, y, z - 1, 2), EF(E, l, x, y, z - 1, 2), ez);
        double v = 0.0;
        for (int aa = 0; aa < 8; aa++) {
          const double g = norm * ((EF(E, l, x, y, z, 0)[aa] - ex[aa]) + (EF(E, l, x, y, z, 1)[aa] - ey[aa]) +
                                   (EF(E, l, x, y, z, 2)[aa] - ez[aa]) -
                                   (JF(JpStat, l, x, y, z)[aa] + JF(JmStat, l, x, y, z)[aa]) / kSqrt2);
          mx = std::max(mx, std::fabs(g));
          sq += g * g;
          v += g * g;
        }
        prof += v;
      }
    if (zprofile) zprofile[z] = prof / ((double)Nx * Ny);
  }
  *max_out = mx;
  *avg_out = std::sqrt(sq / (8.0 * l.volume()));
}

// Observables::Unitarity::UpdateViolation (S/OBSERVABLES/UnitarityViolation.cpp:13-51)
void oracle_unitarity(const int* N, const double* Uin, double* max_out, double* avg_out) {
  Lat l = make_lat(N, kUnitSpacing, 1);
  const cplx* U = reinterpret_cast<const cplx*>(Uin);
  double mx = 0.0, sq = 0.0;
  const int Nx = l.N[0], Ny = l.N[1], Nz = l.N[2];
#pragma omp parallel for reduction(+ : sq) reduction(max : mx) schedule(static)
  for (int z = 0; z < Nz; z++)
    for (int y = 0; y < Ny; y++)
      for (int x = 0; x < Nx; x++)
        for (int mu = 0; mu < 3; mu++) {
          const double v = unitarity_norm(L(U, l, x, y, z, mu));
          mx = std::max(mx, v);
          sq += v * v;
        }
  *max_out = mx;
  *avg_out = std::sqrt(sq / (3.0 * l.volume()));
}

// Observables::EnergyMomentumTensor::CreateMap (S/OBSERVABLES/EnergyMomentumTensor.cpp:92-170) with
// COMPUTE_AVG_FIELD_STRENGTH (S/CALC/AvgFieldStrength.cpp:68-112): clover-averaged B from UOld,
// transported E average using U.  out[z*10 + k], k = T00,TXX,TYY,TZZ,T0X,T0Y,T0Z,TXY,TYZ,TZX.
// Syncs the U and UOld ghosts first, as the reference does inside its site loop (:132-133).
void oracle_emt_map(const int* N, const double* a, double aScale, double* Uin, double* UOldin, const double* E, double* out) {
  Lat l = make_lat(N, a, aScale);
  cplx* U = reinterpret_cast<cplx*>(Uin);
  cplx* UO = reinterpret_cast<cplx*>(UOldin);
  sync_U(UO, l);
  sync_U(U, l);
  double qB[3], qE[3];
  for (int mu = 0; mu < 3; mu++) {
    qB[mu] = l.a[mu] * aScale * aScale / l.aCube();
    qE[mu] = qB[mu];
  }
  const int Nx = l.N[0], Ny = l.N[1], Nz = l.N[2];
  const double inv = 1.0 / ((double)Nx * Ny);
  for (int z = 0; z < Nz; z++) {
    double T00 = 0, TXX = 0, TYY = 0, TZZ = 0, T0X = 0, T0Y = 0, T0Z = 0, TXY = 0, TYZ = 0, TZX = 0;
#pragma omp parallel for reduction(+ : T00, TXX, TYY, TZZ, T0X, T0Y, T0Z, TXY, TYZ, TZX) schedule(static)
    for (int y = 0; y < Ny; y++)
      for (int x = 0; x < Nx; x++) {
        cplx P[12][9];
        // elementary (0..2), neighbouring (3..8), extended (9..11); as in S/CALC/Plaquettes.cpp:83-103
        uudd(L(UO, l, x, y, z, 0), L(UO, l, x + 1, y, z, 1), L(UO, l, x, y + 1, z, 0), L(UO, l, x, y, z, 1), P[0]);  // Uxy
        uudd(L(UO, l, x, y, z, 1), L(UO, l, x, y + 1, z, 2), L(UO, l, x, y, z + 1, 1), L(UO, l, x, y, z, 2), P[1]);  // Uyz
        uudd(L(UO, l, x, y, z, 2), L(UO, l, x, y, z + 1, 0), L(UO, l, x + 1, y, z, 2), L(UO, l, x, y, z, 0), P[2]);  // Uzx
        uddu(L(UO, l, x, y, z, 1), L(UO, l, x - 1, y + 1, z, 0), L(UO, l, x - 1, y, z, 1), L(UO, l, x - 1, y, z, 0), P[3]);  // UMxy
        uddu(L(UO, l, x, y, z, 2), L(UO, l, x, y - 1, z + 1, 1), L(UO, l, x, y - 1, z, 2), L(UO, l, x, y - 1, z, 1), P[4]);  // UMyz
        uddu(L(UO, l, x, y, z, 0), L(UO, l, x + 1, y, z - 1, 2), L(UO, l, x, y, z - 1, 0), L(UO, l, x, y, z - 1, 2), P[5]);  // UMzx
        duud(L(UO, l, x, y - 1, z, 1), L(UO, l, x, y - 1, z, 0), L(UO, l, x + 1, y - 1, z, 1), L(UO, l, x, y, z, 0), P[6]);  // UxMy
        duud(L(UO, l, x, y, z - 1, 2), L(UO, l, x, y, z - 1, 1), L(UO, l, x, y + 1, z - 1, 2), L(UO, l, x, y, z, 1), P[7]);  // UyMz
        duud(L(UO, l, x - 1, y, z, 0), L(UO, l, x - 1, y, z, 2), L(UO, l, x - 1, y, z + 1, 0), L(UO, l, x, y, z, 2), P[8]);  // UzMx
        dduu(L(UO, l, x - 1, y, z, 0), L(UO, l, x - 1, y - 1, z, 1), L(UO, l, x - 1, y - 1, z, 0), L(UO, l, x, y - 1, z, 1), P[9]);   // UMxMy
        dduu(L(UO, l, x, y - 1, z, 1), L(UO, l, x, y - 1, z - 1, 2), L(UO, l, x, y - 1, z - 1, 1), L(UO, l, x, y, z - 1, 2), P[10]);  // UMyMz
        dduu(L(UO, l, x, y, z - 1, 2), L(UO, l, x - 1, y, z - 1, 0), L(UO, l, x - 1, y, z - 1, 2), L(UO, l, x - 1, y, z, 0), P[11]);  // UMzMx
        cplx zx[9], xy[9], yz[9];
        for (int k = 0; k < 9; k++) {
          zx[k] = 0.25 * (P[2][k] + P[5][k] + P[8][k] + P[11][k]);
          xy[k] = 0.25 * (P[0][k] + P[3][k] + P[6][k] + P[9][k]);
          yz[k] = 0.25 * (P[1][k] + P[4][k] + P[7][k] + P[10][k]);
        }
        double B0[8], B1[8], B2[8];
        retr_itg(yz, B0, 2.0);
        retr_itg(zx, B1, 2.0);
        retr_itg(xy, B2, 2.0);
        const double B0s = 4.0 * retr_1m(yz), B1s = 4.0 * retr_1m(zx), B2s = 4.0 * retr_1m(xy);
        double e0d[8], e1d[8], e2d[8];
        inv_adj_mul(L(U, l, x - 1, y, z, 0), EF(E, l, x - 1, y, z, 0), e0d);
        inv_adj_mul(L(U, l, x, y - 1, z, 1), EF(E, l, x, y - 1, z, 1), e1d);
        inv_adj_mul(L(U, l, x, y, z - 1, 2), EF(E, l, x, y, z - 1, 2), e2d);
        double E0[8], E1[8], E2[8], E0s = 0, E1s = 0, E2s = 0;
        for (int aa = 0; aa < 8; aa++) {
          E0[aa] = 0.5 * (EF(E, l, x, y, z, 0)[aa] + e0d[aa]);
          E1[aa] = 0.5 * (EF(E, l, x, y, z, 1)[aa] + e1d[aa]);
          E2[aa] = 0.5 * (EF(E, l, x, y, z, 2)[aa] + e2d[aa]);
        }
        for (int aa = 0; aa < 8; aa++) {
          const double a0 = EF(E, l, x, y, z, 0)[aa], a0m = EF(E, l, x - 1, y, z, 0)[aa];
          const double a1 = EF(E, l, x, y, z, 1)[aa], a1m = EF(E, l, x, y - 1, z, 1)[aa];
          const double a2 = EF(E, l, x, y, z, 2)[aa], a2m = EF(E, l, x, y, z - 1, 2)[aa];
          E0s += 0.5 * (a0 * a0 + a0m * a0m);
          E1s += 0.5 * (a1 * a1 + a1m * a1m);
          E2s += 0.5 * (a2 * a2 + a2m * a2m);
        }
        auto dot = [](const double* p, const double* q) {
          double s = 0;
          for (int k = 0; k < 8; k++) s += p[k] * q[k];
          return s;
        };
        const double e0 = qE[0] * qE[0] * E0s, e1 = qE[1] * qE[1] * E1s, e2 = qE[2] * qE[2] * E2s;
        const double b0 = qB[0] * qB[0] * B0s, b1 = qB[1] * qB[1] * B1s, b2 = qB[2] * qB[2] * B2s;
        T00 += (0.5 * (e0 + e1 + e2 + b0 + b1 + b2)) * inv;
        TXX += (0.5 * ((e1 + e2 + b1 + b2) - (e0 + b0))) * inv;
        TYY += (0.5 * ((e0 + e2 + b0 + b2) - (e1 + b1))) * inv;
        TZZ += (0.5 * ((e0 + e1 + b0 + b1) - (e2 + b2))) * inv;
        T0X += (qE[1] * qB[2] * dot(E1, B2) - qE[2] * qB[1] * dot(E2, B1)) * inv;
        T0Y += (qE[2] * qB[0] * dot(E2, B0) - qE[0] * qB[2] * dot(E0, B2)) * inv;
        T0Z += (qE[0] * qB[1] * dot(E0, B1) - qE[1] * qB[0] * dot(E1, B0)) * inv;
        TXY += (qE[0] * qE[1] * dot(E0, E1) + qB[0] * qB[1] * dot(B0, B1)) * inv;
        TYZ += (qE[1] * qE[2] * dot(E1, E2) + qB[1] * qB[2] * dot(B1, B2)) * inv;
        TZX += (qE[2] * qE[0] * dot(E2, E0) + qB[2] * qB[0] * dot(B2, B0)) * inv;
      }
    double* o = out + 10 * z;
    o[0] = T00; o[1] = TXX; o[2] = TYY; o[3] = TZZ; o[4] = T0X;
    o[5] = T0Y; o[6] = T0Z; o[7] = TXY; o[8] = TYZ; o[9] = TZX;
  }
}

// CoulombGaugeFixing::SetCoulombGauge (S/GAUGETRANSFORMATION/CoulombGaugeFixing.cpp:32-88) with the
// Fourier-accelerated update (S/GAUGETRANSFORMATION/ALGORITHMS/FourierAcceleration.cpp:15-142) and
// the deviation / monitor macros (S/GAUGETRANSFORMATION/CoulombGaugeDeviation.cpp:23-73).
// G (with ghosts) carries the gauge transformation between calls.  UG and EG receive the gauge-fixed
// fields; their ghost slices are never written (the reference's GaugeFixedVariables keep the identity /
// zero ghosts they were created with).  log_out[n*7 + k] = n, maxdev, avgdev, maxstep, avgstep,
// minfunctional, sumfunctional/V.  Returns 0, or 5 when the unitarity guard fires (the reference exits).
// flags: 0 for the reference's iteration; 0x1 drops the p = 0 mode of the update (the reference leaves it
// unnormalised, FourierAcceleration.cpp:69-77); 0x4 the open-z functional (gauge_deviation's open_top).
int oracle_coulomb_fix(const int* N, const double* a, double aScale, const double* Uin, const double* E, double* Gin,
                       double* UGin, double* EG, double alpha, int total_steps, double tol, double* log_out, int* n_out,
                       unsigned flags) {
  const int project_zero = (flags & 0x1u) ? 1 : 0, open_top = (flags & 0x4u) ? 1 : 0;
  Lat l = make_lat(N, a, aScale);
  const cplx* U = reinterpret_cast<const cplx*>(Uin);
  cplx* G = reinterpret_cast<cplx*>(Gin);
  cplx* UG = reinterpret_cast<cplx*>(UGin);
  const long V = l.volume();
  // CopyFields (GaugeTransformation.cpp:93-97): interior only
  std::memcpy(UG + 27 * l.s(0, 0, 0), U + 27 * l.s(0, 0, 0), sizeof(cplx) * 27 * V);
  std::memcpy(EG + 24 * l.s(0, 0, 0), E + 24 * l.s(0, 0, 0), sizeof(double) * 24 * V);
  gauge_transform_links(l, U, UG, G);
  const int Nx = l.N[0], Ny = l.N[1], Nz = l.N[2];
  std::vector<cplx> X((size_t)8 * V);
  double cw[3];
  for (int mu = 0; mu < 3; mu++) cw[mu] = (aScale / l.a[mu]) * (aScale / l.a[mu]);
  double gmaxdev = 1.0;
  int n = 0;
  int status = 0;
  while (n < total_steps && gmaxdev > tol) {
    double maxdev = 0.0, sqdev = 0.0, sumf = 0.0;
    double minf = 2.0 * 3 * (1.0 / (l.a[0] * l.a[0]) + 1.0 / (l.a[1] * l.a[1]) + 1.0 / (l.a[2] * l.a[2]));
#pragma omp parallel for reduction(+ : sqdev, sumf) reduction(max : maxdev) reduction(min : minf) schedule(static)
    for (int z = 0; z < Nz; z++)
      for (int y = 0; y < Ny; y++)
        for (int x = 0; x < Nx; x++) {
          cplx w[9];
          double dev[8];
          gauge_deviation(l, UG, x, y, z, cw, w, dev, open_top);
          const long site = x + (long)Nx * (y + (long)Ny * z);
          for (int aa = 0; aa < 8; aa++) {
            maxdev = std::max(maxdev, std::fabs(dev[aa]));
            sqdev += dev[aa] * dev[aa];
            X[aa + 8 * site] = dev[aa];
          }
          const double lf = retr(w);
          minf = std::min(minf, lf);
          sumf += lf;
        }
    fft3d(X.data(), l.N, 8, -1);
    const double nf = 1.0 / ((double)Nx * Ny * Nz);
#pragma omp parallel for schedule(static)
    for (int pz = 0; pz < Nz; pz++)
      for (int py = 0; py < Ny; py++)
        for (int px = 0; px < Nx; px++) {
          const double p2 = (2.0 - 2.0 * std::cos(2.0 * M_PI * px / (double)Nx)) / (l.a[0] * l.a[0]) +
                            (2.0 - 2.0 * std::cos(2.0 * M_PI * py / (double)Ny)) / (l.a[1] * l.a[1]) +
                            (2.0 - 2.0 * std::cos(2.0 * M_PI * pz / (double)Nz)) / (l.a[2] * l.a[2]);
          const long site = px + (long)Nx * (py + (long)Ny * pz);
          if (p2 > 0.0) {
            for (int aa = 0; aa < 8; aa++) X[aa + 8 * site] = nf * X[aa + 8 * site] / p2;
          } else if (project_zero) {
            for (int aa = 0; aa < 8; aa++) X[aa + 8 * site] = 0.0;
          }
        }
    fft3d(X.data(), l.N, 8, +1);
    double maxstep = 0.0, sqstep = 0.0;
    int bad = 0;
#pragma omp parallel for reduction(+ : sqstep, bad) reduction(max : maxstep) schedule(static)
    for (int z = 0; z < Nz; z++)
      for (int y = 0; y < Ny; y++)
        for (int x = 0; x < Nx; x++) {
          const long site = x + (long)Nx * (y + (long)Ny * z);
          double upd[8];
          for (int aa = 0; aa < 8; aa++) upd[aa] = X[aa + 8 * site].real();
          cplx wt[9], gn[9];
          expi(-alpha, upd, wt);
          if (unitarity_norm(wt) > 1e-13) bad += 1;
          const double st = std::abs(cplx(3.0) - wt[0] - wt[4] - wt[8]);
          maxstep = std::max(maxstep, st);
          sqstep += st * st;
          mul_dn(wt, GF(G, l, x, y, z), gn);
          std::memcpy(GF(G, l, x, y, z), gn, sizeof(gn));
        }
    gauge_transform_links(l, U, UG, G);
    gmaxdev = maxdev;
    if (log_out) {
      double* o = log_out + 7 * n;
      o[0] = n;
      o[1] = maxdev;
      o[2] = std::sqrt(sqdev / (8.0 * V));
      o[3] = maxstep;
      o[4] = std::sqrt(sqstep / (8.0 * V));
      o[5] = minf;
      o[6] = sumf / V;
    }
    n++;
    if (bad) {
      status = 5;
      break;
    }
  }
  if (status == 0) {
    gauge_transform_links(l, U, UG, G);
    gauge_transform_efield(l, E, EG, G);
  }
  *n_out = n;
  return status;
}

double oracle_gf_uniform(unsigned long long seed, long iteration, int pass, long site) {
  return gf_uniform(seed, iteration, pass, site);
}

// SetCoulombGauge (S/GAUGETRANSFORMATION/CoulombGaugeFixing.cpp:32-88) with one of the two local updates
// the reference compiles next to the Fourier-accelerated one:
//   algorithm 1  LosAlamosAlgorithm (S/GAUGETRANSFORMATION/ALGORITHMS/LosAlamos.cpp:13-95): the even
//                sites ((x+y+z) % 2 == 0), the links re-transformed, the odd sites, the links
//                re-transformed.  At each site wTilde = MaxTraceProjection(w), G <- wTilde^d G, or
//                G <- wTilde^d wTilde^d G (over-relaxation) unless the site's draw exceeds param (the
//                reference's OverRelaxationProbability).  The monitors are reset before the even pass
//                and accumulate over both.
//   algorithm 2  JacobiAlgorithm (S/GAUGETRANSFORMATION/ALGORITHMS/Jacobi.cpp:13-80): every site at
//                once, wTilde = exp(-i param t.Delta) (param: the reference's alphaStepSize), G <- wTilde^d G.
// Both read only the links transformed before the pass and write only G at the site itself, so the
// sites of a pass are independent.  Monitors, guard and log rows as in oracle_coulomb_fix; seed and the
// iteration index of this call select the over-relaxation draws (gf_uniform).
int oracle_coulomb_fix_local(const int* N, const double* a, double aScale, const double* Uin, const double* E,
                             double* Gin, double* UGin, double* EG, int algorithm, double param,
                             unsigned long long seed, int total_steps, double tol, double* log_out, int* n_out) {
  *n_out = 0;
  if (algorithm != 1 && algorithm != 2) return 1;
  Lat l = make_lat(N, a, aScale);
  const cplx* U = reinterpret_cast<const cplx*>(Uin);
  cplx* G = reinterpret_cast<cplx*>(Gin);
  cplx* UG = reinterpret_cast<cplx*>(UGin);
  const long V = l.volume();
  std::memcpy(UG + 27 * l.s(0, 0, 0), U + 27 * l.s(0, 0, 0), sizeof(cplx) * 27 * V);
  std::memcpy(EG + 24 * l.s(0, 0, 0), E + 24 * l.s(0, 0, 0), sizeof(double) * 24 * V);
  gauge_transform_links(l, U, UG, G);
  const int Nx = l.N[0], Ny = l.N[1], Nz = l.N[2];
  double cw[3];
  for (int mu = 0; mu < 3; mu++) cw[mu] = (aScale / l.a[mu]) * (aScale / l.a[mu]);
  const double minf0 = 2.0 * 3 * (1.0 / (l.a[0] * l.a[0]) + 1.0 / (l.a[1] * l.a[1]) + 1.0 / (l.a[2] * l.a[2]));
  const int passes = algorithm == 1 ? 2 : 1;
  double gmaxdev = 1.0;
  int n = 0, status = 0;
  while (n < total_steps && gmaxdev > tol) {
    double maxdev = 0.0, sqdev = 0.0, sumf = 0.0, minf = minf0, maxstep = 0.0, sqstep = 0.0;
    int bad = 0;
    for (int pass = 0; pass < passes; pass++) {
#pragma omp parallel for reduction(+ : sqdev, sumf, sqstep, bad) reduction(max : maxdev, maxstep) \
    reduction(min : minf) schedule(static)
      for (int z = 0; z < Nz; z++)
        for (int y = 0; y < Ny; y++)
          for (int x = 0; x < Nx; x++) {
            if (algorithm == 1 && (x + y + z) % 2 != pass) continue;
            cplx w[9], wt[9], gn[9];
            double dev[8];
            gauge_deviation(l, UG, x, y, z, cw, w, dev);
            for (int aa = 0; aa < 8; aa++) {
              maxdev = std::max(maxdev, std::fabs(dev[aa]));
              sqdev += dev[aa] * dev[aa];
            }
            const double lf = retr(w);
            minf = std::min(minf, lf);
            sumf += lf;
            if (algorithm == 1)
              max_trace_projection(w, wt);
            else
              expi(-param, dev, wt);
            if (unitarity_norm(wt) > 1e-13) bad += 1;
            const double st = std::abs(cplx(3.0) - wt[0] - wt[4] - wt[8]);
            maxstep = std::max(maxstep, st);
            sqstep += st * st;
            cplx* g = GF(G, l, x, y, z);
            const long site = x + (long)Nx * (y + (long)Ny * z);
            if (algorithm == 1 && !(gf_uniform(seed, n, pass, site) > param)) {
              cplx t[9];
              mul_dd(wt, wt, t);  // DDU (S/SUNc/AdvancedOperations.cpp:119-131)
              mul_nn(t, g, gn);
            } else {
              mul_dn(wt, g, gn);  // DU (S/SUNc/SU3/GroupOperations.cpp:166-180)
            }
            std::memcpy(g, gn, sizeof(gn));
          }
      gauge_transform_links(l, U, UG, G);
    }
    gmaxdev = maxdev;
    if (log_out) {
      double* o = log_out + 7 * n;
      o[0] = n;
      o[1] = maxdev;
      o[2] = std::sqrt(sqdev / (8.0 * V));
      o[3] = maxstep;
      o[4] = std::sqrt(sqstep / (8.0 * V));
      o[5] = minf;
      o[6] = sumf / V;
    }
    n++;
    if (bad) {
      status = 5;
      break;
    }
  }
  if (status == 0) {
    gauge_transform_links(l, U, UG, G);
    gauge_transform_efield(l, E, EG, G);
  }
  *n_out = n;
  return status;
}

}  // extern "C"

// adjoint.cu -- adjoint (reverse-mode) leapfrog: gradients of a late-time observable with respect
// to the initial electric field and the initial colour currents.  FP64.
//
// No reference counterpart.  Method:
//   forward   nsteps of the ordinary leapfrog, storing the state every `checkpoint_every` steps;
//   objective L = N(q)/D(q), q = (e0,e1,e2,b0,b1,b2) slice sums over z in [z0,z1):
//             e_mu = cE_mu sum_x E_mu^2, b_i = cB_i sum_x 4 ReTr(1 - P_jk) (the bulk observables'
//             constants, S/OBSERVABLES/BulkObservables.cpp:22-97), N, D linear forms (D = 1 when its
//             coefficients are all zero).  P_L/P_T: N = (1,1,-1,1,1,-1), D = (0,0,1,0,0,1).
//   backward  for t = nsteps-1 .. 0: reconstruct the state at t from the state at t+1 by
//             time-reversed integration (the step is an exact composition of shears: the forward
//             kernels run with -dt, the links are rotated back by X^dagger), or reload the checkpoint
//             at t; then pull the cotangents back through the step's sub-steps in reverse order.
// Cotangent convention: for a complex matrix W, Lambda_W is the matrix with dL = Re tr(Lambda_W^dagger dW).
//   W' = A W           -> Lambda_W = A^dagger Lambda_W', Lambda_A = Lambda_W' W^dagger
//   f = ReTr(M W1..W4) -> link k: Lambda = (B A)^dagger if W_k = U, B A if W_k = U^dagger,
//                         A = M W1..W_{k-1}, B = W_{k+1}..W4
//   X = exp(iQ)        -> closed-form derivative of the Cayley-Hamilton coefficients (expi_vjp below)
//   Adj(V,e)           -> Lambda_V = 4 (t.mu) V (t.e), transpose in e = InvAdj(V, .)
//   InvAdj(V,e)        -> Lambda_V = 4 (t.e) V (t.mu), transpose in e = Adj(V, .)
// Ghost slices are copies of the boundary slices, so cotangents that land on a ghost are added to
// the slice it copies.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "../../include/glasma_gb300.h"
#include "handle.h"
#include "leapfrog_sites.cuh"

namespace glasma {
namespace {

using L = long long;
typedef cx<double> C;
typedef Mat<double> M3;
typedef Alg<double> A8;

constexpr int kAT = 128;

__device__ __forceinline__ void site_xyz(const Geometry& g, L idx, int& x, int& y, int& z) {
  const L r = idx / g.nx;
  x = (int)(idx - r * g.nx);
  z = (int)(r / g.ny);
  y = (int)(r - (L)z * g.ny);
}
__device__ __forceinline__ L nbl(const Geometry& g, int x, int y, int z, int dx, int dy, int dz) {
  int xx = x + dx, yy = y + dy;
  xx = xx < 0 ? xx + g.nx : (xx >= g.nx ? xx - g.nx : xx);
  yy = yy < 0 ? yy + g.ny : (yy >= g.ny ? yy - g.ny : yy);
  return (L)xx + (L)g.nx * ((L)yy + (L)g.ny * (L)(z + dz + 1));
}
__device__ __forceinline__ void ld(const C* U, L S, int mu, L s, M3& m) { load_link<double, L>(U, S, mu, s, m); }
__device__ __forceinline__ void st(C* U, L S, int mu, L s, const M3& m) { store_link<double, L>(U, S, mu, s, m); }
__device__ __forceinline__ void dagger(const M3& a, M3& o) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) o.e[i + 3 * j] = mk<double>(a.e[j + 3 * i].re, -a.e[j + 3 * i].im);
}
__device__ __forceinline__ void set_id(M3& m) {
  set_zero(m);
  m.e[0].re = m.e[4].re = m.e[8].re = 1.0;
}
__device__ __forceinline__ void axpy(double s, const M3& a, M3& acc) {
#pragma unroll
  for (int k = 0; k < 9; k++) {
    acc.e[k].re = fma(s, a.e[k].re, acc.e[k].re);
    acc.e[k].im = fma(s, a.e[k].im, acc.e[k].im);
  }
}
__device__ __forceinline__ void atomic_add_link(C* LU, L S, int mu, L s, const M3& m) {
  C* p = LU + (L)(mu * 9) * S + s;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    double* q = reinterpret_cast<double*>(p + (L)k * S);
    atomicAdd(q, m.e[k].re);
    atomicAdd(q + 1, m.e[k].im);
  }
}
// i (t.l) scaled: the matrix M with ReTr(M W) = sum_a l^a ReTr(i t^a W)
__device__ __forceinline__ void i_herm(const A8& l, double scale, M3& m) {
  A8 s;
#pragma unroll
  for (int a = 0; a < 8; a++) s.a[a] = scale * l.a[a];
  M3 h;
  herm_from_alg(s, h);
#pragma unroll
  for (int k = 0; k < 9; k++) m.e[k] = mk<double>(-h.e[k].im, h.e[k].re);
}

// ---- exact vector-Jacobian product of X = exp(iQ), Q = c t.e
// exp(iQ) = f0 + f1 Q + f2 Q^2 with f_j(c0, c1), c0 = det Q, c1 = tr Q^2 / 2 (the Cayley-Hamilton form
// of expi).  dX = sum_j df_j Q^j + f1 dQ + f2 (dQ Q + Q dQ), df_j = b1_j dc1 + b2_j dc0,
// dc1 = tr(Q dQ), dc0 = tr(Q^2 dQ), so for dL = ReTr(Lx^d dX):
//   dL = ReTr(G dQ),  G = beta1 Q + beta2 Q^2 + f1 Lx^d + f2 (Q Lx^d + Lx^d Q),
//   beta_k = Re sum_j b_kj tr(Lx^d Q^j),
// and dL/de^a = c ReTr(G t^a).  The derivatives b are taken in the variables (u, v = w^2) of the
// closed form (eigenvalues 2u, -u +- w), where every factor is an entire function of v, then mapped
// to (c0, c1) by the inverse Jacobian of c1 = 3u^2 + v, c0 = 2u^3 - 2uv (determinant
// 2 (9u^2 - w^2) >= 16 u^2 once c0 is folded to |c0|); below c1 = 1e-6 the Taylor series of f_j is
// differentiated instead.  Checked against the exact Frechet derivative (block exponential) to 4e-13.
__device__ __forceinline__ C cm(double r, double i) { return mk<double>(r, i); }
__device__ __forceinline__ C cmul(C a, C b) { return cm(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
__device__ __forceinline__ C cadd(C a, C b) { return cm(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ C csub(C a, C b) { return cm(a.re - b.re, a.im - b.im); }
__device__ __forceinline__ C cscale(double s, C a) { return cm(s * a.re, s * a.im); }

__device__ void exp_coeff_derivs(double c0, double c1, C (&f)[3], C (&b2)[3], C (&b1)[3]) {
  if (c1 < 1e-6) {
    f[0] = cm(1.0 - c0 * c0 / 720.0, -c0 / 6.0 + c1 * c0 / 120.0);
    f[1] = cm(c0 / 24.0 - c0 * c1 / 360.0, 1.0 - c1 / 6.0 + c1 * c1 / 120.0);
    f[2] = cm(-0.5 + c1 / 24.0 - c1 * c1 / 720.0, c0 / 120.0);
    b2[0] = cm(-c0 / 360.0, -1.0 / 6.0 + c1 / 120.0);
    b2[1] = cm(1.0 / 24.0 - c1 / 360.0, 0.0);
    b2[2] = cm(0.0, 1.0 / 120.0);
    b1[0] = cm(0.0, c0 / 120.0);
    b1[1] = cm(-c0 / 360.0, -1.0 / 6.0 + c1 / 60.0);
    b1[2] = cm(1.0 / 24.0 - c1 / 360.0, 0.0);
    return;
  }
  const bool neg = c0 < 0.0;
  const double ac0 = neg ? -c0 : c0;
  const double s3 = sqrt(c1 / 3.0);
  double r = ac0 / (2.0 * s3 * s3 * s3);
  r = r > 1.0 ? 1.0 : r;
  double st, ct;
  sincos(acos(r) / 3.0, &st, &ct);
  const double u = s3 * ct, w = sqrt(c1) * st, v = w * w, uu = u * u;
  double sw, cw;
  sincos(w, &sw, &cw);
  double x0, x1;  // sin w / w and (cos w - sin w / w) / w^2
  if (w < 0.05) {
    x0 = 1.0 - v / 6.0 * (1.0 - v / 20.0 * (1.0 - v / 42.0 * (1.0 - v / 72.0)));
    x1 = -1.0 / 3.0 + v / 30.0 - v * v / 840.0 + v * v * v / 45360.0;
  } else {
    x0 = sw / w;
    x1 = (cw - x0) / v;
  }
  double s2u, c2u, su, cu;
  sincos(2.0 * u, &s2u, &c2u);
  sincos(u, &su, &cu);
  const C e2 = cm(c2u, s2u), em = cm(cu, -su), I = cm(0.0, 1.0);
  const C A0 = cm(8.0 * uu * cw, 2.0 * u * (3.0 * uu + v) * x0);
  const C A1 = cm(2.0 * u * cw, -(3.0 * uu - v) * x0);
  const C A2 = cm(cw, 3.0 * u * x0);
  C h[3], hu[3], hv[3];
  h[0] = cadd(cscale(uu - v, e2), cmul(em, A0));
  h[1] = csub(cscale(2.0 * u, e2), cmul(em, A1));
  h[2] = csub(e2, cmul(em, A2));
  const C iem = cmul(I, em);  // i e^{-iu}: d e^{-iu}/du = -i e^{-iu}
  hu[0] = cadd(cadd(cmul(cm(2.0 * u, 2.0 * (uu - v)), e2), cscale(-1.0, cmul(iem, A0))),
               cmul(em, cm(16.0 * u * cw, 2.0 * (9.0 * uu + v) * x0)));
  hu[1] = csub(cmul(cm(2.0, 4.0 * u), e2), csub(cmul(em, cm(2.0 * cw, -6.0 * u * x0)), cmul(iem, A1)));
  hu[2] = csub(cmul(cm(0.0, 2.0), e2), csub(cmul(em, cm(0.0, 3.0 * x0)), cmul(iem, A2)));
  hv[0] = cadd(cscale(-1.0, e2), cmul(em, cm(-4.0 * uu * x0, 2.0 * u * x0 + u * (3.0 * uu + v) * x1)));
  hv[1] = cscale(-1.0, cmul(em, cm(-u * x0, x0 - 0.5 * (3.0 * uu - v) * x1)));
  hv[2] = cscale(-1.0, cmul(em, cm(-0.5 * x0, 1.5 * u * x1)));
  const double d = 9.0 * uu - v, id = 1.0 / d;
  const double iD = 1.0 / (18.0 * uu - 2.0 * v);
  const double du0 = iD, du1 = 2.0 * u * iD, dv0 = -6.0 * u * iD, dv1 = (6.0 * uu - 2.0 * v) * iD;
#pragma unroll
  for (int j = 0; j < 3; j++) {
    f[j] = cscale(id, h[j]);
    const C fu = cscale(id, csub(hu[j], cscale(18.0 * u, f[j])));
    const C fv = cscale(id, cadd(hv[j], f[j]));
    b2[j] = cadd(cscale(du0, fu), cscale(dv0, fv));
    b1[j] = cadd(cscale(du1, fu), cscale(dv1, fv));
  }
  if (neg) {  // f_j(-c0) = (-1)^j conj f_j(c0); d/dc0 picks up one more sign
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const double sg = (j == 1) ? -1.0 : 1.0;
      f[j] = cm(sg * f[j].re, -sg * f[j].im);
      b1[j] = cm(sg * b1[j].re, -sg * b1[j].im);
      b2[j] = cm(-sg * b2[j].re, sg * b2[j].im);
    }
  }
}

// dl^a = dL/de^a for X = exp(i c t.e) given Lx (dL = ReTr(Lx^d dX))
__device__ void expi_vjp(double c, const A8& e, const M3& lx, A8& dl) {
  A8 sc;
#pragma unroll
  for (int a = 0; a < 8; a++) sc.a[a] = c * e.a[a];
  M3 Q, Q2;
  herm_from_alg(sc, Q);
  mul_nn(Q, Q, Q2);
  const double c1 = 0.5 * (Q2.e[0].re + Q2.e[4].re + Q2.e[8].re);
  double c0 = 0.0;  // tr(Q^2 Q) / 3, real
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const C a = Q2.e[i + 3 * j], b = Q.e[j + 3 * i];
      c0 += a.re * b.re - a.im * b.im;
    }
  c0 *= 1.0 / 3.0;
  C f[3], b2[3], b1[3];
  exp_coeff_derivs(c0, c1, f, b2, b1);
  // tau_j = tr(Lx^d Q^j) = sum_k conj(Lx_k) Q^j_k
  C tau[3] = {cm(0, 0), cm(0, 0), cm(0, 0)};
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const C l = cm(lx.e[k].re, -lx.e[k].im);
    if (k % 4 == 0) tau[0] = cadd(tau[0], l);
    tau[1] = cadd(tau[1], cmul(l, Q.e[k]));
    tau[2] = cadd(tau[2], cmul(l, Q2.e[k]));
  }
  double beta1 = 0.0, beta2 = 0.0;
#pragma unroll
  for (int j = 0; j < 3; j++) {
    beta1 += cmul(b1[j], tau[j]).re;
    beta2 += cmul(b2[j], tau[j]).re;
  }
  M3 L, QL, LQ;
  dagger(lx, L);
  mul_nn(Q, L, QL);
  mul_nn(L, Q, LQ);
  M3 M;  // M = -i G
#pragma unroll
  for (int k = 0; k < 9; k++) {
    C g = cadd(cscale(beta1, Q.e[k]), cscale(beta2, Q2.e[k]));
    g = cadd(g, cmul(f[1], L.e[k]));
    g = cadd(g, cmul(f[2], cadd(QL.e[k], LQ.e[k])));
    M.e[k] = cm(g.im, -g.re);
  }
  retr_itg(M, c, dl);
}

// Cotangents of the four links of f = ReTr(M W1 W2 W3 W4); dag[k] tells whether W_k = U^dagger.
// Adds each link's cotangent atomically at (mu[k], site[k]).
__device__ void path_vjp(C* LU, L S, const M3& Mx, const M3 (&W)[4], const bool (&dag)[4], const int (&mu)[4],
                         const L (&site)[4]) {
  M3 P[4];  // P[k] = M W1..W_k  (P[0] = M)
  P[0] = Mx;
  for (int k = 1; k < 4; k++) mul_nn(P[k - 1], W[k - 1], P[k]);
  M3 Sx[4];  // Sx[k] = W_{k+1}..W_4  (Sx[3] = 1)
  set_id(Sx[3]);
  Sx[2] = W[3];
  mul_nn(W[2], W[3], Sx[1]);
  mul_nn(W[1], Sx[1], Sx[0]);
  for (int k = 0; k < 4; k++) {
    M3 BA, out;
    mul_nn(Sx[k], P[k], BA);
    if (dag[k])
      out = BA;
    else
      dagger(BA, out);
    atomic_add_link(LU, S, mu[k], site[k], out);
  }
}

// ---------------------------------------------------------------- reverse reconstruction
// z link: U_{t+1} = X X U_t, store X = exp(i cU E_{t+1}) and Uh = X^d U_{t+1}, leave U = Uh (for the J
// inversion); x, y links: U_{t+1} = X2 U_t, store X2 = exp(2i cU E_{t+1}), leave U = U_t.
__global__ void __launch_bounds__(kAT) rev_links_kernel(Geometry g, C* U, const double* E, C* X, C* Uh, double c0,
                                                          double c1, double c2) {
  const L idx = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.vol) return;
  const L s = idx + g.plane;
  const double cU[3] = {c0, c1, c2};
  for (int mu = 0; mu < 3; mu++) {
    A8 e;
    load_alg<double, L>(E, g.S, mu * 8, s, e);
    M3 x, u, uh;
    // the x and y links advance in one step U_{t+1} = exp(2i cU t.E) U_t (as the forward step
    // computes them): X holds that exponential and U_t follows at once; the z link keeps its half step
    expi(mu == 2 ? cU[mu] : 2.0 * cU[mu], e, x);
    ld(U, g.S, mu, s, u);
    mul_dn(x, u, uh);
    st(X, g.S, mu, s, x);
    if (mu == 2) st(Uh, g.S, mu, s, uh);
    st(U, g.S, mu, s, uh);
  }
}
// U_z <- X^d U_z  (from the half step to U_t)
__global__ void __launch_bounds__(kAT) rev_links2_kernel(Geometry g, C* U, const C* X) {
  const L idx = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.vol) return;
  const L s = idx + g.plane;
  M3 x, u, o;
  ld(X, g.S, 2, s, x);
  ld(U, g.S, 2, s, u);
  mul_dn(x, u, o);
  st(U, g.S, 2, s, o);
}

// ---------------------------------------------------------------- adjoint sub-steps
struct AdjPtrs {
  C* LU;
  double* LE;
  double* LJp;
  double* LJm;
  double* LJpS;
  double* LJmS;
};

// Fold cotangents that landed on ghost slices into the boundary slices they copy; clear the ghosts.
// `stride` = doubles per component array, `plane` = doubles per z slice of one component.
__global__ void fold_ghosts_kernel(double* base, L stride, L plane, int nz, int comps) {
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= plane * comps) return;
  const L c = i / plane, r = i - c * plane;
  double* p = base + c * stride;
  p[plane + r] += p[r];
  p[r] = 0.0;
  p[(L)nz * plane + r] += p[(L)(nz + 1) * plane + r];
  p[(L)(nz + 1) * plane + r] = 0.0;
}

// Link-update tail of the step, in reverse: U1 = X Uh, J transport with Uh (A4), Uh = X U (A3).
// Inputs: X, Uh, U (= U_t), JpS1/JmS1 (state at t+1), cotangents at t+1.  Per site; the J
// transport's cross-slice term is gathered from the slice below (and the top ghost folded in).
__global__ void __launch_bounds__(kAT) adj_links_kernel(Geometry g, AdjPtrs a, const C* X, const C* Uh, const C* U,
                                                          const double* E, const double* JpS1, const double* JmS1,
                                                          double c0, double c1, double c2, double cj) {
  const L idx = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.vol) return;
  int x, y, z;
  site_xyz(g, idx, x, y, z);
  const L S = g.S, s = idx + g.plane;
  const double cU[3] = {c0, c1, c2};
  // J transport cotangents (A4).  Jp1 = Jp - cj (Adj(Uh_z, JpS1(z+1)) - JpS1), Jm1 = Jm + cj (...)
  {
    A8 lp, lm, ps, ms, tmp;
    load_alg<double, L>(a.LJp, S, 0, s, lp);
    load_alg<double, L>(a.LJm, S, 0, s, lm);
    load_alg<double, L>(a.LJpS, S, 0, s, ps);
    load_alg<double, L>(a.LJmS, S, 0, s, ms);
#pragma unroll
    for (int k = 0; k < 8; k++) {
      ps.a[k] += cj * lp.a[k];
      ms.a[k] -= cj * lm.a[k];
    }
    // from the site below: lambda_JpS1(z) += -cj InvAdj(Uh_z(z-1), lambda_Jp1(z-1))
    if (z > 0) {
      const L sb = s - g.plane;
      M3 vb;
      ld(Uh, S, 2, sb, vb);
      A8 lpb, lmb;
      load_alg<double, L>(a.LJp, S, 0, sb, lpb);
      load_alg<double, L>(a.LJm, S, 0, sb, lmb);
      inv_adj_mul(vb, lpb, tmp);
#pragma unroll
      for (int k = 0; k < 8; k++) ps.a[k] -= cj * tmp.a[k];
      inv_adj_mul(vb, lmb, tmp);
#pragma unroll
      for (int k = 0; k < 8; k++) ms.a[k] += cj * tmp.a[k];
    }
    // the top slice read JpS1 at the ghost z = Nz, a copy of its own slice
    if (z == g.nz - 1) {
      M3 v;
      ld(Uh, S, 2, s, v);
      inv_adj_mul(v, lp, tmp);
#pragma unroll
      for (int k = 0; k < 8; k++) ps.a[k] -= cj * tmp.a[k];
      inv_adj_mul(v, lm, tmp);
#pragma unroll
      for (int k = 0; k < 8; k++) ms.a[k] += cj * tmp.a[k];
    }
    store_alg<double, L>(a.LJpS, S, 0, s, ps);
    store_alg<double, L>(a.LJmS, S, 0, s, ms);
  }
  for (int mu = 0; mu < 3; mu++) {
    M3 xx, uh, u, lu, luh, lx, t1;
    ld(X, S, mu, s, xx);
    ld(U, S, mu, s, u);
    ld(a.LU, S, mu, s, lu);
    if (mu != 2) {  // U_{t+1} = X2 U_t with X2 = exp(2i cU t.E)
      A8 e, le, dl;
      mul_dn(xx, lu, luh);
      st(a.LU, S, mu, s, luh);
      mul_nd(lu, u, lx);
      load_alg<double, L>(E, S, mu * 8, s, e);
      expi_vjp(2.0 * cU[mu], e, lx, dl);
      load_alg<double, L>(a.LE, S, mu * 8, s, le);
#pragma unroll
      for (int k = 0; k < 8; k++) le.a[k] += dl.a[k];
      store_alg<double, L>(a.LE, S, mu * 8, s, le);
      continue;
    }
    ld(Uh, S, mu, s, uh);
    // A5: U1 = X Uh
    mul_dn(xx, lu, luh);
    mul_nd(lu, uh, lx);
    if (mu == 2) {
      // A4: d/dUh of -cj Adj(Uh, JpS1(z+1)) contracted with lambda_Jp1, and +cj ... for Jm
      A8 lp, lm, sp, sm;
      load_alg<double, L>(a.LJp, S, 0, s, lp);
      load_alg<double, L>(a.LJm, S, 0, s, lm);
      load_alg<double, L>(JpS1, S, 0, s + g.plane, sp);
      load_alg<double, L>(JmS1, S, 0, s + g.plane, sm);
      M3 Mh, Nh, tmp, tmp2;
      herm_from_alg(lp, Mh);
      herm_from_alg(sp, Nh);
      mul_nn(Mh, uh, tmp);
      mul_nn(tmp, Nh, tmp2);
      axpy(-4.0 * cj, tmp2, luh);
      herm_from_alg(lm, Mh);
      herm_from_alg(sm, Nh);
      mul_nn(Mh, uh, tmp);
      mul_nn(tmp, Nh, tmp2);
      axpy(4.0 * cj, tmp2, luh);
    }
    // A3: Uh = X U
    M3 lu_new;
    mul_dn(xx, luh, lu_new);
    mul_nd(luh, u, t1);
#pragma unroll
    for (int k = 0; k < 9; k++) {
      lx.e[k].re += t1.e[k].re;
      lx.e[k].im += t1.e[k].im;
    }
    st(a.LU, S, mu, s, lu_new);
    // X = exp(i cU t.E): lambda_E += dL/dE through the exact exp VJP
    A8 e, le, dl;
    load_alg<double, L>(E, S, mu * 8, s, e);
    expi_vjp(cU[mu], e, lx, dl);
    load_alg<double, L>(a.LE, S, mu * 8, s, le);
#pragma unroll
    for (int k = 0; k < 8; k++) le.a[k] += dl.a[k];
    store_alg<double, L>(a.LE, S, mu * 8, s, le);
  }
}

// JStat sub-step in reverse (A2).  JpS1 = JpS - cj (Jp - InvAdj(U_z(z-1), Jp(z-1))), JmS1 = JmS + cj (...).
// Gathers: site z owns lambda_Jp(z) and Lambda_U_z(z); the terms from slice z+1 are read here, and the
// bottom ghost (U_z(-1), Jp(-1) copies of slice 0) is folded into slice 0.
__global__ void __launch_bounds__(kAT) adj_jstat_kernel(Geometry g, AdjPtrs a, const C* U, const double* Jp,
                                                          const double* Jm, double cj) {
  const L idx = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.vol) return;
  int x, y, z;
  site_xyz(g, idx, x, y, z);
  const L S = g.S, s = idx + g.plane;
  A8 lp, lm, sp, sm, tmp;
  load_alg<double, L>(a.LJp, S, 0, s, lp);
  load_alg<double, L>(a.LJm, S, 0, s, lm);
  load_alg<double, L>(a.LJpS, S, 0, s, sp);
  load_alg<double, L>(a.LJmS, S, 0, s, sm);
#pragma unroll
  for (int k = 0; k < 8; k++) {
    lp.a[k] -= cj * sp.a[k];
    lm.a[k] += cj * sm.a[k];
  }
  M3 luz;
  ld(a.LU, S, 2, s, luz);
  // contributions of the JStat update at site (z+1), which reads U_z(z) and Jp(z)
  auto from_above = [&](L s_above_lambda, L s_link, L s_j) {
    A8 spa, sma, jp, jm, t2;
    load_alg<double, L>(a.LJpS, S, 0, s_above_lambda, spa);
    load_alg<double, L>(a.LJmS, S, 0, s_above_lambda, sma);
    load_alg<double, L>(Jp, S, 0, s_j, jp);
    load_alg<double, L>(Jm, S, 0, s_j, jm);
    M3 v;
    ld(U, S, 2, s_link, v);
    adj_mul(v, spa, t2);
#pragma unroll
    for (int k = 0; k < 8; k++) lp.a[k] += cj * t2.a[k];
    adj_mul(v, sma, t2);
#pragma unroll
    for (int k = 0; k < 8; k++) lm.a[k] -= cj * t2.a[k];
    // Lambda_V = 4 (t.e) V (t.mu) for InvAdj(V, e) contracted with mu
    M3 Nh, Mh, t3, t4;
    herm_from_alg(jp, Nh);
    herm_from_alg(spa, Mh);
    mul_nn(Nh, v, t3);
    mul_nn(t3, Mh, t4);
    axpy(4.0 * cj, t4, luz);
    herm_from_alg(jm, Nh);
    herm_from_alg(sma, Mh);
    mul_nn(Nh, v, t3);
    mul_nn(t3, Mh, t4);
    axpy(-4.0 * cj, t4, luz);
  };
  if (z < g.nz - 1) from_above(s + g.plane, s, s);
  if (z == 0) from_above(s, s - g.plane, s - g.plane);  // ghost link and ghost currents below slice 0
  st(a.LU, S, 2, s, luz);
  store_alg<double, L>(a.LJp, S, 0, s, lp);
  store_alg<double, L>(a.LJm, S, 0, s, lm);
}

// Electric-field sub-step in reverse (A1): E1 = E + F(U) + jz (Jp - Jm).  lambda_E unchanged;
// lambda_Jp/Jm get the jz term; Lambda_U gets the force's link cotangents (scattered atomically).
// Electric-field sub-step in reverse, one plaquette at a time.  For the plaquette at x in plane
// (p, q), p < q, with links a = U_p(x), b = U_q(x+p), c = U_p(x+q), d = U_q(x), P = a b c^d d^d, the
// force terms that contain it are the four staples
//   ReTr(M1 P) + ReTr(M2 c b^d a^d d) + ReTr(M3 d c b^d a^d) + ReTr(M4 b c^d d^d a),
// M1 = i t.lambda_p(x) gc_p cn_q, M2 = i t.lambda_p(x+q) gc_p cn_q, M3 = i t.lambda_q(x) gc_q cn_p,
// M4 = i t.lambda_q(x+p) gc_q cn_p (anti-Hermitian).  On SU(3) (a^d a = d^d d = 1) they sum to
// ReTr(N P), N = M1 - M3 + a M4 a^d - d M2 d^d, whose link cotangents are those of the path
// N a b c^d d^d plus the explicit a- and d-dependence of N.  These agree with the four separate
// staple cotangents along every SU(3) tangent direction (the only directions the E and current
// gradients see) at 22 instead of 36 matmuls and a quarter of the atomics.  Open z: a plaquette at
// the top slice has no M2 term (its link at x+z is a ghost), and the threads of slice 0 also take
// the M2 term of the plaquette at the bottom ghost slice (the backward staple of U_p(x, z=0)).
__device__ __forceinline__ void atomic_add_alg(double* F, L S, int base, L s, double w, const A8& v) {
  double* q = F + (L)base * S + s;
#pragma unroll
  for (int k = 0; k < 8; k++) atomicAdd(q + (L)k * S, w * v.a[k]);
}

// Also undoes this plaquette's share of the electric-field update on E (E_{t+1} -> E_t): the force
// on a is wp ReTr(i t P), on d wq ReTr(i t P^d) = -wq ReTr(i t P), on c wp ReTr(i t d^d P^d d), on b
// wq ReTr(i t a^d P a); rev_mask bit k selects the links (a, b, c, d) whose force is removed.
// V M V^d for anti-Hermitian M: the result is anti-Hermitian, so only its upper triangle and
// imaginary diagonal are formed and the rest filled by -conjugation.
__device__ __forceinline__ void conj_antiherm(const M3& V, const M3& M, M3& out) {
  M3 VM;
  mul_nn(V, M, VM);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      C acc = mk<double>(0, 0);
      if (i == j) {
#pragma unroll
        for (int k = 0; k < 3; k++) {  // Im sum_k VM_ik conj(V_ik)
          acc.im = fma(-VM.e[i + 3 * k].re, V.e[i + 3 * k].im, acc.im);
          acc.im = fma(VM.e[i + 3 * k].im, V.e[i + 3 * k].re, acc.im);
        }
      } else {
#pragma unroll
        for (int k = 0; k < 3; k++) cfma_nc(acc, VM.e[i + 3 * k], V.e[j + 3 * k]);
        out.e[j + 3 * i] = mk<double>(-acc.re, acc.im);
      }
      out.e[i + 3 * j] = acc;
    }
}

// Also undoes this plaquette's share of the electric-field update on E (E_{t+1} -> E_t): the force
// on a is wp ReTr(i t P), on d -wq ReTr(i t P), on c wp ReTr(i t d^d P^d d), on b wq ReTr(i t a^d P a);
// rev_mask bit k selects the links (a, b, c, d) whose force is removed.
// With D = P - P^d and the M's anti-Hermitian, the explicit a- and d-dependence of N contributes
// D a M4 to a's cotangent and -D d M2 to d's, and the b and c forces are (1/2) ReTr(i t a^d D a) and
// -(1/2) ReTr(i t d^d D d) (ReTr(i t X) only sees the anti-Hermitian part of X).
__device__ void plaquette_vjp(C* LU, double* E, L S, int p, int q, L sa, L sb, L sc, L sd, const M3& a,
                              const M3& b, const M3& c, const M3& d, const M3& M1, const M3& M2, const M3& Mm3,
                              const M3& M4, double wp, double wq, unsigned rev_mask) {
  M3 cd, P, t, N, Dm;
  mul_dd(c, d, cd);  // c^d d^d
  mul_nn(a, b, t);
  mul_nn(t, cd, P);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      Dm.e[i + 3 * j] = mk<double>(P.e[i + 3 * j].re - P.e[j + 3 * i].re, P.e[i + 3 * j].im + P.e[j + 3 * i].im);
  conj_antiherm(a, M4, N);
  {
    M3 v;
    conj_antiherm(d, M2, v);
#pragma unroll
    for (int k = 0; k < 9; k++)
      N.e[k] = mk<double>(N.e[k].re - v.e[k].re + M1.e[k].re - Mm3.e[k].re,
                          N.e[k].im - v.e[k].im + M1.e[k].im - Mm3.e[k].im);
  }
  M3 La, Lb, Lc, Ld, bcd, Na, Nab, w;
  mul_nn(b, cd, bcd);
  mul_nn(bcd, N, w);
  dagger(w, La);
  mul_nn(N, a, Na);
  mul_nn(cd, Na, w);
  dagger(w, Lb);
  mul_nn(Na, b, Nab);
  mul_dn(d, Nab, Lc);
  mul_nd(Nab, c, Ld);
  {
    M3 Dx, v;
    mul_nn(Dm, a, Dx);  // D a
    mul_nn(Dx, M4, v);
    axpy(1.0, v, La);
    if (rev_mask & 2u) {  // force on b
      A8 fb;
      mul_dn(a, Dx, v);
      retr_itg(v, 0.5, fb);
      atomic_add_alg(E, S, q * 8, sb, -wq, fb);
    }
    mul_nn(Dm, d, Dx);  // D d
    mul_nn(Dx, M2, v);
    axpy(-1.0, v, Ld);
    if (rev_mask & 4u) {  // force on c
      A8 fc;
      mul_dn(d, Dx, v);
      retr_itg(v, -0.5, fc);
      atomic_add_alg(E, S, p * 8, sc, -wp, fc);
    }
  }
  if (rev_mask & 9u) {  // forces on a and d
    A8 fa;
    retr_itg(P, 1.0, fa);
    if (rev_mask & 1u) atomic_add_alg(E, S, p * 8, sa, -wp, fa);
    if (rev_mask & 8u) atomic_add_alg(E, S, q * 8, sd, wq, fa);
  }
  atomic_add_link(LU, S, p, sa, La);
  atomic_add_link(LU, S, q, sb, Lb);
  atomic_add_link(LU, S, p, sc, Lc);
  atomic_add_link(LU, S, q, sd, Ld);
}

__global__ void __launch_bounds__(kAT) adj_efield_kernel(Geometry g, AdjPtrs a, const C* U, double* E, const double* Jp,
                                                           const double* Jm, double gc0, double gc1, double gc2,
                                                           double cn0, double cn1, double cn2, double jz) {
  const L idx = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.vol) return;
  int x, y, z;
  site_xyz(g, idx, x, y, z);
  const L S = g.S, s = idx + g.plane;
  const double gc[3] = {gc0, gc1, gc2}, cn[3] = {cn0, cn1, cn2};
  {
    A8 lez, lp, lm;
    load_alg<double, L>(a.LE, S, 16, s, lez);
    load_alg<double, L>(a.LJp, S, 0, s, lp);
    load_alg<double, L>(a.LJm, S, 0, s, lm);
#pragma unroll
    for (int k = 0; k < 8; k++) {
      lp.a[k] += jz * lez.a[k];
      lm.a[k] -= jz * lez.a[k];
    }
    store_alg<double, L>(a.LJp, S, 0, s, lp);
    store_alg<double, L>(a.LJm, S, 0, s, lm);
    // E_z(t) = E_z(t+1) - jz (Jp - Jm)(t); the plaquette forces are removed below
    A8 jp, jm, dj;
    load_alg<double, L>(Jp, S, 0, s, jp);
    load_alg<double, L>(Jm, S, 0, s, jm);
#pragma unroll
    for (int k = 0; k < 8; k++) dj.a[k] = jp.a[k] - jm.a[k];
    atomic_add_alg(E, S, 16, s, -jz, dj);
  }
  const int planes[3][2] = {{0, 1}, {0, 2}, {1, 2}};
#pragma unroll 1
  for (int pl = 0; pl < 3; pl++) {
    const int p = planes[pl][0], q = planes[pl][1];
    int dp[3] = {0, 0, 0}, dq[3] = {0, 0, 0};
    dp[p] = 1;
    dq[q] = 1;
    const L sp = nbl(g, x, y, z, dp[0], dp[1], dp[2]), sq = nbl(g, x, y, z, dq[0], dq[1], dq[2]);
    const double wp = gc[p] * cn[q], wq = gc[q] * cn[p];
    M3 A, B, Cc, Dd, M1, M2, Mm3, M4;
    A8 l;
    ld(U, S, p, s, A);
    ld(U, S, q, sp, B);
    ld(U, S, p, sq, Cc);
    ld(U, S, q, s, Dd);
    load_alg<double, L>(a.LE, S, p * 8, s, l);
    i_herm(l, wp, M1);
    load_alg<double, L>(a.LE, S, q * 8, s, l);
    i_herm(l, wq, Mm3);
    load_alg<double, L>(a.LE, S, q * 8, sp, l);
    i_herm(l, wq, M4);
    const bool top = (q == 2 && z == g.nz - 1);
    if (top) {
      set_zero(M2);  // U_p(x+z) is a ghost link: no staple of its own
    } else {
      load_alg<double, L>(a.LE, S, p * 8, sq, l);
      i_herm(l, wp, M2);
    }
    plaquette_vjp(a.LU, E, S, p, q, s, sp, sq, s, A, B, Cc, Dd, M1, M2, Mm3, M4, wp, wq, top ? 11u : 15u);
    if (q == 2 && z == 0) {
      // plaquette at the bottom ghost slice: only the backward staple of U_p(x) (= its c link)
      const L gs = s - g.plane, gsp = nbl(g, x, y, -1, dp[0], dp[1], 0);
      ld(U, S, p, gs, A);
      ld(U, S, q, gsp, B);
      ld(U, S, p, s, Cc);
      ld(U, S, q, gs, Dd);
      load_alg<double, L>(a.LE, S, p * 8, s, l);
      i_herm(l, wp, M2);
      set_zero(M1);
      set_zero(Mm3);
      set_zero(M4);
      plaquette_vjp(a.LU, E, S, p, q, gs, gsp, s, gs, A, B, Cc, Dd, M1, M2, Mm3, M4, wp, wq, 4u);
    }
  }
}

// ---------------------------------------------------------------- objective
// q = (e0,e1,e2,b0,b1,b2) over z in [z0,z1): block partials (6 values per block)
__global__ void __launch_bounds__(256) objective_kernel(Geometry g, const C* U, const double* E, int z0, int z1,
                                                          double* partials) {
  double v[6] = {0, 0, 0, 0, 0, 0};
  const L plane = g.plane, n = plane * (z1 - z0);
  for (L i = (L)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (L)gridDim.x * blockDim.x) {
    const L idx = i + plane * z0;
    int x, y, z;
    site_xyz(g, idx, x, y, z);
    const L s = idx + plane;
    for (int mu = 0; mu < 3; mu++) {
      A8 e;
      load_alg<double, L>(E, g.S, mu * 8, s, e);
      double q = 0.0;
#pragma unroll
      for (int k = 0; k < 8; k++) q += e.a[k] * e.a[k];
      v[mu] += q;
    }
    // b_i: plaquette in the plane (j,k), i = yz:0, zx:1, xy:2
    const int pj[3] = {1, 2, 0}, pk[3] = {2, 0, 1};
    for (int i2 = 0; i2 < 3; i2++) {
      const int j = pj[i2], k = pk[i2];
      int dj[3] = {0, 0, 0}, dk[3] = {0, 0, 0};
      dj[j] = 1;
      dk[k] = 1;
      M3 a, b, c, d, t1, t2, P;
      ld(U, g.S, j, s, a);
      ld(U, g.S, k, nbl(g, x, y, z, dj[0], dj[1], dj[2]), b);
      ld(U, g.S, j, nbl(g, x, y, z, dk[0], dk[1], dk[2]), c);
      ld(U, g.S, k, s, d);
      mul_nn(a, b, t1);
      mul_dd(c, d, t2);
      mul_nn(t1, t2, P);
      v[3 + i2] += 4.0 * (3.0 - P.e[0].re - P.e[4].re - P.e[8].re);
    }
  }
  __shared__ double sh[6][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < 6; k++) {
    double r = v[k];
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    if (lane == 0) sh[k][warp] = r;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double r = 0.0;
    for (int w = 0; w < (int)(blockDim.x / 32); w++) r += sh[threadIdx.x][w];
    partials[(L)blockIdx.x * 6 + threadIdx.x] = r;
  }
}

// Objective VJP at the final state: lambda_E = 2 w_e cE E, Lambda_U from -4 w_b cB ReTr P.
__global__ void __launch_bounds__(kAT) objective_vjp_kernel(Geometry g, AdjPtrs a, const C* U, const double* E, int z0,
                                                              int z1, double we0, double we1, double we2, double wb0,
                                                              double wb1, double wb2) {
  const L n = g.plane * (z1 - z0);
  const L i = (L)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const L idx = i + g.plane * z0;
  int x, y, z;
  site_xyz(g, idx, x, y, z);
  const L S = g.S, s = idx + g.plane;
  const double we[3] = {we0, we1, we2}, wb[3] = {wb0, wb1, wb2};
  for (int mu = 0; mu < 3; mu++) {
    A8 e, le;
    load_alg<double, L>(E, S, mu * 8, s, e);
    load_alg<double, L>(a.LE, S, mu * 8, s, le);
#pragma unroll
    for (int k = 0; k < 8; k++) le.a[k] += 2.0 * we[mu] * e.a[k];
    store_alg<double, L>(a.LE, S, mu * 8, s, le);
  }
  const int pj[3] = {1, 2, 0}, pk[3] = {2, 0, 1};
  for (int i2 = 0; i2 < 3; i2++) {
    if (wb[i2] == 0.0) continue;
    const int j = pj[i2], k = pk[i2];
    int dj[3] = {0, 0, 0}, dk[3] = {0, 0, 0};
    dj[j] = 1;
    dk[k] = 1;
    const L sites[4] = {s, nbl(g, x, y, z, dj[0], dj[1], dj[2]), nbl(g, x, y, z, dk[0], dk[1], dk[2]), s};
    const int mus[4] = {j, k, j, k};
    const bool dag[4] = {false, false, true, true};
    M3 W[4], t, Mx;
    ld(U, S, j, sites[0], W[0]);
    ld(U, S, k, sites[1], W[1]);
    ld(U, S, j, sites[2], t);
    dagger(t, W[2]);
    ld(U, S, k, sites[3], t);
    dagger(t, W[3]);
    set_id(Mx);
#pragma unroll
    for (int q = 0; q < 9; q++) Mx.e[q].re *= -4.0 * wb[i2];
    path_vjp(a.LU, S, Mx, W, dag, mus, sites);
  }
}

inline unsigned gridv(L n) { return (unsigned)((n + kAT - 1) / kAT); }

}  // namespace
}  // namespace glasma

namespace {

thread_local std::string g_adj_error;
int afail(int st, const std::string& m) {
  g_adj_error = m;
  return st;
}

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  bool alloc(size_t bytes) { return cudaMalloc(&p, bytes) == cudaSuccess; }
};

// q = (e0,e1,e2,b0,b1,b2) with the bulk constants, on the handle's current state
int objective_q(glasma_lattice* h, int z0, int z1, double* q, double* scratch) {
  using namespace glasma;
  const int nb = 608;
  objective_kernel<<<nb, 256, 0, h->stream>>>(h->g, static_cast<const C*>(h->f[GLASMA_FIELD_U]),
                                               static_cast<const double*>(h->f[GLASMA_FIELD_E]), z0, z1, scratch);
  if (cudaGetLastError() != cudaSuccess) return afail(GLASMA_ERR_CUDA, "objective kernel");
  std::vector<double> part((size_t)nb * 6);
  if (cudaMemcpyAsync(part.data(), scratch, sizeof(double) * nb * 6, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
      cudaStreamSynchronize(h->stream) != cudaSuccess)
    return afail(GLASMA_ERR_CUDA, "objective copy");
  for (int k = 0; k < 6; k++) {
    q[k] = 0.0;
    for (int b = 0; b < nb; b++) q[k] += part[(size_t)b * 6 + k];
  }
  // constants of Observables::Bulk::SetConstants (S/OBSERVABLES/BulkObservables.cpp:22-31)
  const double a3 = h->g.a[0] * h->g.a[1] * h->g.a[2];
  for (int mu = 0; mu < 3; mu++) {
    const double c = (h->g.a[mu] * h->a_scale * h->a_scale / a3) * (h->g.a[mu] * h->a_scale * h->a_scale / a3);
    q[mu] *= c;
    q[3 + mu] *= c;
  }
  return GLASMA_OK;
}

double ratio(const double* num, const double* den, const double* q, double* Nout, double* Dout) {
  double N = 0.0, D = 0.0;
  bool has_den = false;
  for (int k = 0; k < 6; k++) {
    N += num[k] * q[k];
    D += den[k] * q[k];
    if (den[k] != 0.0) has_den = true;
  }
  if (!has_den) D = 1.0;
  *Nout = N;
  *Dout = D;
  return N / D;
}

}  // namespace

extern "C" {

int glasma_objective(glasma_lattice* h, int z_begin, int z_end, const double* num, const double* den, double* value) {
  if (!h || !num || !den || !value) return afail(GLASMA_ERR_INVALID_ARGUMENT, "null argument");
  if (h->precision != GLASMA_FP64) return afail(GLASMA_ERR_UNSUPPORTED, "the objective is computed on FP64 lattices");
  if (z_begin < 0 || z_end > h->g.nz || z_begin >= z_end) return afail(GLASMA_ERR_INVALID_ARGUMENT, "bad slice range");
  cudaSetDevice(h->device);
  DevBuf scratch;
  if (!scratch.alloc(sizeof(double) * 608 * 6)) return afail(GLASMA_ERR_OUT_OF_MEMORY, "scratch");
  double q[6], N, D;
  int st = objective_q(h, z_begin, z_end, q, static_cast<double*>(scratch.p));
  if (st) return st;
  *value = ratio(num, den, q, &N, &D);
  return GLASMA_OK;
}

int glasma_adjoint(glasma_lattice* h, double dt, int nsteps, int checkpoint_every, int z_begin, int z_end,
                   const double* num, const double* den, double* objective, double* grad_E, double* grad_Jp,
                   double* grad_Jm, double* grad_JpStat, double* grad_JmStat) {
  using namespace glasma;
  if (!h || !num || !den) return afail(GLASMA_ERR_INVALID_ARGUMENT, "null argument");
  if (h->precision != GLASMA_FP64) return afail(GLASMA_ERR_UNSUPPORTED, "the adjoint runs on FP64 lattices");
  if (nsteps < 1 || checkpoint_every < 1) return afail(GLASMA_ERR_INVALID_ARGUMENT, "nsteps, checkpoint_every >= 1");
  if (z_begin < 0 || z_end > h->g.nz || z_begin >= z_end) return afail(GLASMA_ERR_INVALID_ARGUMENT, "bad slice range");
  if (cudaSetDevice(h->device) != cudaSuccess) return afail(GLASMA_ERR_CUDA, "cudaSetDevice");
  const Geometry& g = h->g;
  cudaStream_t stm = h->stream;
  const int state_fields[6] = {GLASMA_FIELD_U, GLASMA_FIELD_E, GLASMA_FIELD_JP, GLASMA_FIELD_JM, GLASMA_FIELD_JPSTAT,
                               GLASMA_FIELD_JMSTAT};
  const size_t bytes_f[6] = {sizeof(C) * 27 * g.S, sizeof(double) * 24 * g.S, sizeof(double) * 8 * g.S,
                             sizeof(double) * 8 * g.S, sizeof(double) * 8 * g.S, sizeof(double) * 8 * g.S};
  size_t state_bytes = 0;
  for (size_t b : bytes_f) state_bytes += b;
  const int nck = nsteps / checkpoint_every + 1;
  DevBuf ck, X, Uh, LU, LE, LJ, JS1, scratch;
  if (!ck.alloc(state_bytes * nck) || !X.alloc(sizeof(C) * 27 * g.S) || !Uh.alloc(sizeof(C) * 27 * g.S) ||
      !LU.alloc(sizeof(C) * 27 * g.S) || !LE.alloc(sizeof(double) * 24 * g.S) || !LJ.alloc(sizeof(double) * 32 * g.S) ||
      !JS1.alloc(sizeof(double) * 16 * g.S) || !scratch.alloc(sizeof(double) * 608 * 6))
    return afail(GLASMA_ERR_OUT_OF_MEMORY, "adjoint buffers (checkpoints: " + std::to_string(nck) + " states)");
  auto save_state = [&](int k) {
    char* base = static_cast<char*>(ck.p) + state_bytes * k;
    for (int i = 0; i < 6; i++) {
      cudaMemcpyAsync(base, h->f[state_fields[i]], bytes_f[i], cudaMemcpyDeviceToDevice, stm);
      base += bytes_f[i];
    }
  };
  auto load_state = [&](int k) {
    const char* base = static_cast<const char*>(ck.p) + state_bytes * k;
    for (int i = 0; i < 6; i++) {
      cudaMemcpyAsync(h->f[state_fields[i]], base, bytes_f[i], cudaMemcpyDeviceToDevice, stm);
      base += bytes_f[i];
    }
  };
  // ---- forward with checkpoints
  save_state(0);
  for (int t = 0; t < nsteps; t++) {
    int st = glasma_step(h, dt, 1, 0);
    if (st) return st;
    if ((t + 1) % checkpoint_every == 0 && (t + 1) / checkpoint_every < nck) save_state((t + 1) / checkpoint_every);
  }
  // ---- objective and its cotangents at the final state
  double q[6], N, D;
  int st = objective_q(h, z_begin, z_end, q, static_cast<double*>(scratch.p));
  if (st) return st;
  const double Lval = ratio(num, den, q, &N, &D);
  if (objective) *objective = Lval;
  bool has_den = false;
  for (int k = 0; k < 6; k++) has_den = has_den || den[k] != 0.0;
  double w[6];
  for (int k = 0; k < 6; k++) w[k] = has_den ? (num[k] * D - N * den[k]) / (D * D) : num[k];
  const double a3 = g.a[0] * g.a[1] * g.a[2];
  double cq[3];
  for (int mu = 0; mu < 3; mu++) {
    const double c = g.a[mu] * h->a_scale * h->a_scale / a3;
    cq[mu] = c * c;
  }
  AdjPtrs ap;
  ap.LU = static_cast<C*>(LU.p);
  ap.LE = static_cast<double*>(LE.p);
  ap.LJp = static_cast<double*>(LJ.p);
  ap.LJm = ap.LJp + 8 * g.S;
  ap.LJpS = ap.LJp + 16 * g.S;
  ap.LJmS = ap.LJp + 24 * g.S;
  cudaMemsetAsync(LU.p, 0, sizeof(C) * 27 * g.S, stm);
  cudaMemsetAsync(LE.p, 0, sizeof(double) * 24 * g.S, stm);
  cudaMemsetAsync(LJ.p, 0, sizeof(double) * 32 * g.S, stm);
  C* U = static_cast<C*>(h->f[GLASMA_FIELD_U]);
  double* E = static_cast<double*>(h->f[GLASMA_FIELD_E]);
  double* Jp = static_cast<double*>(h->f[GLASMA_FIELD_JP]);
  double* Jm = static_cast<double*>(h->f[GLASMA_FIELD_JM]);
  double* JpS = static_cast<double*>(h->f[GLASMA_FIELD_JPSTAT]);
  double* JmS = static_cast<double*>(h->f[GLASMA_FIELD_JMSTAT]);
  objective_vjp_kernel<<<gridv(g.plane * (z_end - z_begin)), kAT, 0, stm>>>(
      g, ap, U, E, z_begin, z_end, w[0] * cq[0], w[1] * cq[1], w[2] * cq[2], w[3] * cq[0], w[4] * cq[1],
      w[5] * cq[2]);
  if (cudaGetLastError() != cudaSuccess) return afail(GLASMA_ERR_CUDA, "objective vjp");
  FieldPtrs<double> fp;
  fp.U = U;
  fp.UOld = static_cast<C*>(h->f[GLASMA_FIELD_UOLD]);
  fp.E = E;
  fp.Jp = Jp;
  fp.Jm = Jm;
  fp.JpStat = JpS;
  fp.JmStat = JmS;
  double cU[3];
  for (int mu = 0; mu < 3; mu++) cU[mu] = -(0.5 * dt) * g.a[mu] * g.a[mu] / a3;
  const double cj = dt / g.a[2];
  const double gamma = -2.0 * dt * a3;
  const double jz = -(dt / g.a[2]) * 0.70710678118654752440084436210484903928483593768847;
  auto fold = [&](double* base, int comps) {  // real component arrays
    const L n = g.plane * comps;
    fold_ghosts_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stm>>>(base, g.S, g.plane, g.nz, comps);
  };
  auto fold_links = [&](C* base) {  // 27 complex component arrays of S complex values each
    const L n = 2 * g.plane * 27;
    fold_ghosts_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stm>>>(reinterpret_cast<double*>(base), 2 * g.S,
                                                                     2 * g.plane, g.nz, 27);
  };
  // ---- backward
  for (int t = nsteps - 1; t >= 0; t--) {
    // cotangents scattered onto ghost slices by the previous (later) adjoint step
    fold_links(ap.LU);
    fold(ap.LJp, 8);
    fold(ap.LJm, 8);
    // state at t+1 -> intermediates and U_t
    rev_links_kernel<<<gridv(g.vol), kAT, 0, stm>>>(g, U, E, static_cast<C*>(X.p), static_cast<C*>(Uh.p), cU[0], cU[1],
                                                   cU[2]);  // U = Uh
    launch_sync_ghosts<C>(g, U, 27, stm);
    cudaMemcpyAsync(JS1.p, JpS, sizeof(double) * 8 * g.S, cudaMemcpyDeviceToDevice, stm);
    cudaMemcpyAsync(static_cast<double*>(JS1.p) + 8 * g.S, JmS, sizeof(double) * 8 * g.S, cudaMemcpyDeviceToDevice, stm);
    // Jp_t, Jm_t: the J sub-step with -dt (U currently holds Uh)
    launch_j_only<double>(g, fp, -dt, stm);
    rev_links2_kernel<<<gridv(g.vol), kAT, 0, stm>>>(g, U, static_cast<const C*>(X.p));  // U = U_t
    launch_sync_ghosts<C>(g, U, 27, stm);
    // adjoint of the link/J tail (needs X, Uh, U_t, E_{t+1}, JStat_{t+1})
    adj_links_kernel<<<gridv(g.vol), kAT, 0, stm>>>(g, ap, static_cast<const C*>(X.p), static_cast<const C*>(Uh.p), U, E,
                                                   static_cast<const double*>(JS1.p),
                                                   static_cast<const double*>(JS1.p) + 8 * g.S, cU[0], cU[1], cU[2], cj);
    // adjoint of JStat (needs U_t, Jp_t, Jm_t)
    adj_jstat_kernel<<<gridv(g.vol), kAT, 0, stm>>>(g, ap, U, Jp, Jm, cj);
    // JStat_t: the JStat sub-step with -dt
    launch_jstat_only<double>(g, fp, -dt, h->tile_x, stm);
    // adjoint of the electric-field update (needs U_t), and E_t from E_{t+1}: the same plaquettes
    // give the force that the sub-step added, which is removed again (then the E ghosts re-synced)
    adj_efield_kernel<<<gridv(g.vol), kAT, 0, stm>>>(g, ap, U, E, Jp, Jm, gamma / (g.a[0] * g.a[0]),
                                                    gamma / (g.a[1] * g.a[1]), gamma / (g.a[2] * g.a[2]),
                                                    1.0 / (g.a[0] * g.a[0]), 1.0 / (g.a[1] * g.a[1]),
                                                    1.0 / (g.a[2] * g.a[2]), jz);
    launch_sync_ghosts<double>(g, E, 24, stm);
    // re-anchor on a stored checkpoint
    if (t % checkpoint_every == 0) load_state(t / checkpoint_every);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return afail(GLASMA_ERR_CUDA, std::string("adjoint step: ") + cudaGetErrorString(e));
  }
  fold_links(ap.LU);
  fold(ap.LJp, 8);
  fold(ap.LJm, 8);
  fold(ap.LJpS, 8);
  fold(ap.LJmS, 8);
  fold(ap.LE, 24);
  // ---- gradients out, in the reference's host layout (ghost entries zero)
  double* outs[5] = {grad_E, grad_Jp, grad_Jm, grad_JpStat, grad_JmStat};
  double* srcs[5] = {ap.LE, ap.LJp, ap.LJm, ap.LJpS, ap.LJmS};
  const int per[5] = {24, 8, 8, 8, 8};
  DevBuf stage;
  if (!stage.alloc(sizeof(double) * 24 * g.S)) return afail(GLASMA_ERR_OUT_OF_MEMORY, "stage");
  for (int i = 0; i < 5; i++) {
    if (!outs[i]) continue;
    launch_soa_to_aos<double>(srcs[i], static_cast<double*>(stage.p), g.S, per[i], stm);
    if (cudaMemcpyAsync(outs[i], stage.p, sizeof(double) * per[i] * g.S, cudaMemcpyDeviceToHost, stm) != cudaSuccess)
      return afail(GLASMA_ERR_CUDA, "gradient copy");
  }
  if (cudaStreamSynchronize(stm) != cudaSuccess) return afail(GLASMA_ERR_CUDA, "adjoint sync");
  return GLASMA_OK;
}

const char* glasma_adjoint_last_error(void) { return g_adj_error.c_str(); }

}  // extern "C"

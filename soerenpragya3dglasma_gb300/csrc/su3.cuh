// su3.cuh -- SU(3) group and algebra arithmetic for the device kernels.
//
// Conventions follow the reference (S/ = the reference's SourceCode directory):
//   * matrix element (i,j) is stored at index i+3*j (S/SUNc/SU3/GroupOperations.cpp:13-15);
//   * generators t^a = lambda^a/2 with the standard Gell-Mann matrices, and
//     t^a alpha^a as in S/SUNc/SU3/AlgebraOperations.cpp:31-45;
//   * ReTrIGen(V)_a = Re tr(i t^a V) (S/SUNc/SU3/GroupOperations.cpp:93-103);
//   * adjoint actions V (t.e) V^dagger and V^dagger (t.e) V, the SU(3) forms of
//     the reference's AdjointMultiplication / InverseAdjointMultiplication
//     (only the SU(2) forms exist in the reference, S/SUNc/SU2/AlgebraOperations.cpp:110-124).
// exp(i c t^a alpha^a) uses the Cayley-Hamilton closed form of Morningstar and
// Peardon, Phys. Rev. D 69 (2004) 054501, in place of the reference's
// eigen-decomposition (S/SUNc/SU3/AlgebraOperations.cpp:48-89).
#pragma once

#include <cuda_runtime.h>

namespace glasma {

template <typename T>
struct alignas(2 * sizeof(T)) cx {
  T re, im;
};

template <typename T>
__device__ __forceinline__ cx<T> mk(T r, T i) {
  cx<T> c;
  c.re = r;
  c.im = i;
  return c;
}

template <typename T>
struct Mat {
  cx<T> e[9];  // e[i + 3*j]
};

template <typename T>
struct Alg {
  T a[8];
};

template <typename T>
struct Consts;
template <>
struct Consts<double> {
  static __device__ __forceinline__ double inv_sqrt3() { return 0.57735026918962576450914878050195745564760175127013; }
  static __device__ __forceinline__ double inv_sqrt2() { return 0.70710678118654752440084436210484903928483593768847; }
};
template <>
struct Consts<float> {
  static __device__ __forceinline__ float inv_sqrt3() { return 0.577350269189625764509f; }
  static __device__ __forceinline__ float inv_sqrt2() { return 0.707106781186547524401f; }
};

// acc += a*b (complex)
template <typename T>
__device__ __forceinline__ void cfma(cx<T>& acc, const cx<T>& a, const cx<T>& b) {
  acc.re = fma(a.re, b.re, acc.re);
  acc.re = fma(-a.im, b.im, acc.re);
  acc.im = fma(a.re, b.im, acc.im);
  acc.im = fma(a.im, b.re, acc.im);
}
// acc += a*conj(b)
template <typename T>
__device__ __forceinline__ void cfma_nc(cx<T>& acc, const cx<T>& a, const cx<T>& b) {
  acc.re = fma(a.re, b.re, acc.re);
  acc.re = fma(a.im, b.im, acc.re);
  acc.im = fma(-a.re, b.im, acc.im);
  acc.im = fma(a.im, b.re, acc.im);
}
// acc += conj(a)*b
template <typename T>
__device__ __forceinline__ void cfma_cn(cx<T>& acc, const cx<T>& a, const cx<T>& b) {
  acc.re = fma(a.re, b.re, acc.re);
  acc.re = fma(a.im, b.im, acc.re);
  acc.im = fma(a.re, b.im, acc.im);
  acc.im = fma(-a.im, b.re, acc.im);
}
// acc += conj(a)*conj(b)
template <typename T>
__device__ __forceinline__ void cfma_cc(cx<T>& acc, const cx<T>& a, const cx<T>& b) {
  acc.re = fma(a.re, b.re, acc.re);
  acc.re = fma(-a.im, b.im, acc.re);
  acc.im = fma(-a.re, b.im, acc.im);
  acc.im = fma(-a.im, b.re, acc.im);
}

// C = A B
template <typename T>
__device__ __forceinline__ void mul_nn(const Mat<T>& A, const Mat<T>& B, Mat<T>& C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      cx<T> acc = mk<T>(T(0), T(0));
#pragma unroll
      for (int k = 0; k < 3; k++) cfma(acc, A.e[i + 3 * k], B.e[k + 3 * j]);
      C.e[i + 3 * j] = acc;
    }
}
// C = A B^dagger
template <typename T>
__device__ __forceinline__ void mul_nd(const Mat<T>& A, const Mat<T>& B, Mat<T>& C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      cx<T> acc = mk<T>(T(0), T(0));
#pragma unroll
      for (int k = 0; k < 3; k++) cfma_nc(acc, A.e[i + 3 * k], B.e[j + 3 * k]);
      C.e[i + 3 * j] = acc;
    }
}
// C = A^dagger B
template <typename T>
__device__ __forceinline__ void mul_dn(const Mat<T>& A, const Mat<T>& B, Mat<T>& C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      cx<T> acc = mk<T>(T(0), T(0));
#pragma unroll
      for (int k = 0; k < 3; k++) cfma_cn(acc, A.e[k + 3 * i], B.e[k + 3 * j]);
      C.e[i + 3 * j] = acc;
    }
}
// C = A^dagger B^dagger
template <typename T>
__device__ __forceinline__ void mul_dd(const Mat<T>& A, const Mat<T>& B, Mat<T>& C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      cx<T> acc = mk<T>(T(0), T(0));
#pragma unroll
      for (int k = 0; k < 3; k++) cfma_cc(acc, A.e[k + 3 * i], B.e[j + 3 * k]);
      C.e[i + 3 * j] = acc;
    }
}
// C += s * A B^dagger
template <typename T>
__device__ __forceinline__ void add_mul_nd(const Mat<T>& A, const Mat<T>& B, T s, Mat<T>& C) {
  Mat<T> t;
  mul_nd(A, B, t);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    C.e[k].re = fma(s, t.e[k].re, C.e[k].re);
    C.e[k].im = fma(s, t.e[k].im, C.e[k].im);
  }
}
// C += s * A B
template <typename T>
__device__ __forceinline__ void add_mul_nn(const Mat<T>& A, const Mat<T>& B, T s, Mat<T>& C) {
  Mat<T> t;
  mul_nn(A, B, t);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    C.e[k].re = fma(s, t.e[k].re, C.e[k].re);
    C.e[k].im = fma(s, t.e[k].im, C.e[k].im);
  }
}

template <typename T>
__device__ __forceinline__ void set_zero(Mat<T>& A) {
#pragma unroll
  for (int k = 0; k < 9; k++) A.e[k] = mk<T>(T(0), T(0));
}

// out_a = c * Re tr(i t^a V)
template <typename T>
__device__ __forceinline__ void retr_itg(const Mat<T>& V, T c, Alg<T>& out) {
  const T h = T(-0.5) * c;
  out.a[0] = h * (V.e[3].im + V.e[1].im);
  out.a[1] = h * (V.e[3].re - V.e[1].re);
  out.a[2] = h * (V.e[0].im - V.e[4].im);
  out.a[3] = h * (V.e[6].im + V.e[2].im);
  out.a[4] = h * (V.e[6].re - V.e[2].re);
  out.a[5] = h * (V.e[7].im + V.e[5].im);
  out.a[6] = h * (V.e[7].re - V.e[5].re);
  out.a[7] = h * (V.e[0].im + V.e[4].im - T(2) * V.e[8].im) * Consts<T>::inv_sqrt3();
}

// M = t^a al^a (Hermitian, traceless)
template <typename T>
__device__ __forceinline__ void herm_from_alg(const Alg<T>& al, Mat<T>& M) {
  const T s8 = al.a[7] * Consts<T>::inv_sqrt3();
  M.e[0] = mk<T>(T(0.5) * (al.a[2] + s8), T(0));
  M.e[4] = mk<T>(T(-0.5) * (al.a[2] - s8), T(0));
  M.e[8] = mk<T>(-s8, T(0));
  M.e[1] = mk<T>(T(0.5) * al.a[0], T(0.5) * al.a[1]);   // (1,0)
  M.e[2] = mk<T>(T(0.5) * al.a[3], T(0.5) * al.a[4]);   // (2,0)
  M.e[5] = mk<T>(T(0.5) * al.a[5], T(0.5) * al.a[6]);   // (2,1)
  M.e[3] = mk<T>(M.e[1].re, -M.e[1].im);                // (0,1)
  M.e[6] = mk<T>(M.e[2].re, -M.e[2].im);                // (0,2)
  M.e[7] = mk<T>(M.e[5].re, -M.e[5].im);                // (1,2)
}

// out_a = 2 tr(t^a W) for Hermitian W (only the upper triangle and the real diagonal are read)
template <typename T>
__device__ __forceinline__ void alg_from_herm(const Mat<T>& W, Alg<T>& out) {
  out.a[0] = T(2) * W.e[3].re;
  out.a[1] = T(-2) * W.e[3].im;
  out.a[2] = W.e[0].re - W.e[4].re;
  out.a[3] = T(2) * W.e[6].re;
  out.a[4] = T(-2) * W.e[6].im;
  out.a[5] = T(2) * W.e[7].re;
  out.a[6] = T(-2) * W.e[7].im;
  out.a[7] = (W.e[0].re + W.e[4].re - T(2) * W.e[8].re) * Consts<T>::inv_sqrt3();
}

// The entries of a Hermitian product that alg_from_herm reads: the upper triangle (0,1), (0,2),
// (1,2) and the real diagonal.  Same arithmetic, per entry, as mul_nd / mul_nn.
template <typename T>
__device__ __forceinline__ void mul_nd_herm(const Mat<T>& A, const Mat<T>& B, Mat<T>& C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      cx<T> acc = mk<T>(T(0), T(0));
      if (i == j) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          acc.re = fma(A.e[i + 3 * k].re, B.e[j + 3 * k].re, acc.re);
          acc.re = fma(A.e[i + 3 * k].im, B.e[j + 3 * k].im, acc.re);
        }
      } else {
#pragma unroll
        for (int k = 0; k < 3; k++) cfma_nc(acc, A.e[i + 3 * k], B.e[j + 3 * k]);
      }
      C.e[i + 3 * j] = acc;
    }
}
template <typename T>
__device__ __forceinline__ void mul_nn_herm(const Mat<T>& A, const Mat<T>& B, Mat<T>& C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      cx<T> acc = mk<T>(T(0), T(0));
      if (i == j) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          acc.re = fma(A.e[i + 3 * k].re, B.e[k + 3 * j].re, acc.re);
          acc.re = fma(-A.e[i + 3 * k].im, B.e[k + 3 * j].im, acc.re);
        }
      } else {
#pragma unroll
        for (int k = 0; k < 3; k++) cfma(acc, A.e[i + 3 * k], B.e[k + 3 * j]);
      }
      C.e[i + 3 * j] = acc;
    }
}

// out = V (t.e) V^dagger  (AdjointMultiplication)
template <typename T>
__device__ __forceinline__ void adj_mul(const Mat<T>& V, const Alg<T>& e, Alg<T>& out) {
  Mat<T> M, W, R;
  herm_from_alg(e, M);
  mul_nn(V, M, W);
  mul_nd_herm(W, V, R);
  alg_from_herm(R, out);
}
// out = V^dagger (t.e) V  (InverseAdjointMultiplication)
template <typename T>
__device__ __forceinline__ void inv_adj_mul(const Mat<T>& V, const Alg<T>& e, Alg<T>& out) {
  Mat<T> M, W, R;
  herm_from_alg(e, M);
  mul_dn(V, M, W);
  mul_nn_herm(W, V, R);
  alg_from_herm(R, out);
}

// Two adjoint actions by one matrix from one pair of complex products: with M = t.e1 + i t.e2, the
// product C = V M V^d (or V^d M V) is A + iB, where A and B are the two (Hermitian) actions, so A and B
// are C's Hermitian and anti-Hermitian parts: A_ij = (C_ij + C_ji^*)/2, B_ij = (C_ij - C_ji^*)/(2i).
// Two full products (~216 FMA) instead of two Hermitian-result pairs (~288 FMA); equal to the single
// forms up to rounding.  out1 / out2 as alg_from_herm of A / B.
template <typename T>
__device__ __forceinline__ void split_herm_pair(const Mat<T>& C, Alg<T>& out1, Alg<T>& out2) {
  // C_ij at e[i + 3j]: 01 -> 3, 10 -> 1, 02 -> 6, 20 -> 2, 12 -> 7, 21 -> 5
  out1.a[0] = C.e[3].re + C.e[1].re;
  out1.a[1] = C.e[1].im - C.e[3].im;
  out1.a[2] = C.e[0].re - C.e[4].re;
  out1.a[3] = C.e[6].re + C.e[2].re;
  out1.a[4] = C.e[2].im - C.e[6].im;
  out1.a[5] = C.e[7].re + C.e[5].re;
  out1.a[6] = C.e[5].im - C.e[7].im;
  out1.a[7] = (C.e[0].re + C.e[4].re - T(2) * C.e[8].re) * Consts<T>::inv_sqrt3();
  out2.a[0] = C.e[3].im + C.e[1].im;
  out2.a[1] = C.e[3].re - C.e[1].re;
  out2.a[2] = C.e[0].im - C.e[4].im;
  out2.a[3] = C.e[6].im + C.e[2].im;
  out2.a[4] = C.e[6].re - C.e[2].re;
  out2.a[5] = C.e[7].im + C.e[5].im;
  out2.a[6] = C.e[7].re - C.e[5].re;
  out2.a[7] = (C.e[0].im + C.e[4].im - T(2) * C.e[8].im) * Consts<T>::inv_sqrt3();
}
template <typename T>
__device__ __forceinline__ void herm_pair(const Alg<T>& e1, const Alg<T>& e2, Mat<T>& M) {
  Mat<T> M1, M2;
  herm_from_alg(e1, M1);
  herm_from_alg(e2, M2);
#pragma unroll
  for (int k = 0; k < 9; k++) M.e[k] = mk<T>(M1.e[k].re - M2.e[k].im, M1.e[k].im + M2.e[k].re);
}
// C = A B (kDag: A B^dagger) for a product known to be traceless (a similarity transform of a
// traceless matrix): entry (2,2) as -(C00 + C11) instead of its own three products.
template <typename T, bool kDag>
__device__ __forceinline__ void mul_traceless_result(const Mat<T>& A, const Mat<T>& B, Mat<T>& C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      if (i == 2 && j == 2) continue;
      cx<T> acc = mk<T>(T(0), T(0));
#pragma unroll
      for (int k = 0; k < 3; k++) {
        if constexpr (kDag)
          cfma_nc(acc, A.e[i + 3 * k], B.e[j + 3 * k]);
        else
          cfma(acc, A.e[i + 3 * k], B.e[k + 3 * j]);
      }
      C.e[i + 3 * j] = acc;
    }
  C.e[8] = mk<T>(-(C.e[0].re + C.e[4].re), -(C.e[0].im + C.e[4].im));
}
// out1 = V (t.e1) V^dagger, out2 = V (t.e2) V^dagger
template <typename T>
__device__ __forceinline__ void adj_mul2(const Mat<T>& V, const Alg<T>& e1, const Alg<T>& e2, Alg<T>& out1,
                                         Alg<T>& out2) {
  Mat<T> M, W, C;
  herm_pair(e1, e2, M);
  mul_nn(V, M, W);
  mul_traceless_result<T, true>(W, V, C);
  split_herm_pair(C, out1, out2);
}
// out1 = V^dagger (t.e1) V, out2 = V^dagger (t.e2) V
template <typename T>
__device__ __forceinline__ void inv_adj_mul2(const Mat<T>& V, const Alg<T>& e1, const Alg<T>& e2, Alg<T>& out1,
                                             Alg<T>& out2) {
  Mat<T> M, W, C;
  herm_pair(e1, e2, M);
  mul_dn(V, M, W);
  mul_traceless_result<T, false>(W, V, C);
  split_herm_pair(C, out1, out2);
}

// The entries of C = A B that retr_itg reads: every off-diagonal entry and the imaginary diagonal.
// Same arithmetic, per entry, as mul_nn.
template <typename T>
__device__ __forceinline__ void mul_nn_traceless(const Mat<T>& A, const Mat<T>& B, Mat<T>& C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      cx<T> acc = mk<T>(T(0), T(0));
      if (i == j) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          acc.im = fma(A.e[i + 3 * k].re, B.e[k + 3 * j].im, acc.im);
          acc.im = fma(A.e[i + 3 * k].im, B.e[k + 3 * j].re, acc.im);
        }
      } else {
#pragma unroll
        for (int k = 0; k < 3; k++) cfma(acc, A.e[i + 3 * k], B.e[k + 3 * j]);
      }
      C.e[i + 3 * j] = acc;
    }
}

// The entries of C = A B^dagger that retr_itg reads (as mul_nn_traceless, for mul_nd).
template <typename T>
__device__ __forceinline__ void mul_nd_traceless(const Mat<T>& A, const Mat<T>& B, Mat<T>& C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      cx<T> acc = mk<T>(T(0), T(0));
      if (i == j) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          acc.im = fma(-A.e[i + 3 * k].re, B.e[j + 3 * k].im, acc.im);
          acc.im = fma(A.e[i + 3 * k].im, B.e[j + 3 * k].re, acc.im);
        }
      } else {
#pragma unroll
        for (int k = 0; k < 3; k++) cfma_nc(acc, A.e[i + 3 * k], B.e[j + 3 * k]);
      }
      C.e[i + 3 * j] = acc;
    }
}

// The entries of C = A^dagger B that retr_itg reads (as mul_nn_traceless, for mul_dn).
template <typename T>
__device__ __forceinline__ void mul_dn_traceless(const Mat<T>& A, const Mat<T>& B, Mat<T>& C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      cx<T> acc = mk<T>(T(0), T(0));
      if (i == j) {
#pragma unroll
        for (int k = 0; k < 3; k++) {  // Im conj(A_ki) B_ki
          acc.im = fma(A.e[k + 3 * i].re, B.e[k + 3 * j].im, acc.im);
          acc.im = fma(-A.e[k + 3 * i].im, B.e[k + 3 * j].re, acc.im);
        }
      } else {
#pragma unroll
        for (int k = 0; k < 3; k++) cfma_cn(acc, A.e[k + 3 * i], B.e[k + 3 * j]);
      }
      C.e[i + 3 * j] = acc;
    }
}

// C = A^dagger B when the product is anti-Hermitian (A^dagger D A with D anti-Hermitian and B = D A):
// the upper triangle and the imaginary diagonal are formed, the lower triangle as -conj of the upper.
template <typename T>
__device__ __forceinline__ void mul_dn_antiherm(const Mat<T>& A, const Mat<T>& B, Mat<T>& C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      cx<T> acc = mk<T>(T(0), T(0));
      if (i == j) {
#pragma unroll
        for (int k = 0; k < 3; k++) {  // Im conj(A_ki) B_ki
          acc.im = fma(A.e[k + 3 * i].re, B.e[k + 3 * j].im, acc.im);
          acc.im = fma(-A.e[k + 3 * i].im, B.e[k + 3 * j].re, acc.im);
        }
      } else {
#pragma unroll
        for (int k = 0; k < 3; k++) cfma_cn(acc, A.e[k + 3 * i], B.e[k + 3 * j]);
        C.e[j + 3 * i] = mk<T>(-acc.re, acc.im);
      }
      C.e[i + 3 * j] = acc;
    }
}

template <typename T>
struct Trig;
template <>
struct Trig<double> {
  static __device__ __forceinline__ void sincos_(double x, double* s, double* c) { sincos(x, s, c); }
  static __device__ __forceinline__ double acos_(double x) { return acos(x); }
  static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
  static __device__ __forceinline__ double taylor_c1() { return 1e-6; }
};
template <>
struct Trig<float> {
  static __device__ __forceinline__ void sincos_(float x, float* s, float* c) { sincosf(x, s, c); }
  static __device__ __forceinline__ float acos_(float x) { return acosf(x); }
  static __device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
  static __device__ __forceinline__ float taylor_c1() { return 1e-3f; }
};

// X = exp(i c t^a al^a), Cayley-Hamilton form exp(iQ) = f0 + f1 Q + f2 Q^2.  kMinusOne: X - 1
// instead, with f0 - 1 formed directly (expi_m1 below).
template <typename T, bool kMinusOne = false>
__device__ __forceinline__ void expi_impl(T c, const Alg<T>& al, Mat<T>& X) {
  Alg<T> sc;
#pragma unroll
  for (int a = 0; a < 8; a++) sc.a[a] = c * al.a[a];
  Mat<T> Q, Q2;
  herm_from_alg(sc, Q);
  // Q^2 is Hermitian: its upper triangle and real diagonal, the rest by conjugation
  mul_nn_herm(Q, Q, Q2);
  Q2.e[1] = mk<T>(Q2.e[3].re, -Q2.e[3].im);
  Q2.e[2] = mk<T>(Q2.e[6].re, -Q2.e[6].im);
  Q2.e[5] = mk<T>(Q2.e[7].re, -Q2.e[7].im);
  Q2.e[0].im = Q2.e[4].im = Q2.e[8].im = T(0);
  const T c1 = T(0.5) * (Q2.e[0].re + Q2.e[4].re + Q2.e[8].re);
  // det Q = Q00 (Q11 Q22 - |Q12|^2) - ... ; real for Hermitian Q.  Expanded in the
  // Gell-Mann components for brevity: det Q = tr(Q^3)/3.
  T c0 = (Q2.e[0].re * Q.e[0].re + Q2.e[4].re * Q.e[4].re + Q2.e[8].re * Q.e[8].re);
  // tr(Q2 Q) = sum_ij Q2_ij Q_ji; add off-diagonal terms (both triangles)
  c0 += T(2) * (Q2.e[3].re * Q.e[1].re - Q2.e[3].im * Q.e[1].im);  // (0,1)*(1,0) + (1,0)*(0,1)
  c0 += T(2) * (Q2.e[6].re * Q.e[2].re - Q2.e[6].im * Q.e[2].im);  // (0,2)*(2,0) + (2,0)*(0,2)
  c0 += T(2) * (Q2.e[7].re * Q.e[5].re - Q2.e[7].im * Q.e[5].im);  // (1,2)*(2,1) + (2,1)*(1,2)
  c0 *= T(1) / T(3);
  cx<T> f0, f1, f2;
  if (sizeof(T) == 8 && !kMinusOne && c1 >= Trig<T>::taylor_c1() && c1 < T(0.5)) {
    // FP64 without transcendental functions (they cost ~60 % of this exponential on GB300's FP64 pipe):
    // exp(iQ) = sum_n i^n Q^n / n!, and by Cayley-Hamilton (Q^3 = c1 Q + c0) Q^n / n! = a_n + b_n Q + d_n
    // Q^2 with a_{n+1} = c0 d_n / (n+1), b_{n+1} = (a_n + c1 d_n) / (n+1), d_{n+1} = b_n / (n+1).  The
    // eigenvalues of Q are at most l = sqrt(4 c1 / 3) in size, so after N terms the first omitted one is
    // below l^(N+1) / (N+1)!: with 17 terms for c1 < 0.5 below 0.82^18 / 18! ~ 4e-18, with 11 for
    // c1 < 0.02 below 0.17^12 / 12! ~ 8e-19, with 8 for c1 < 1e-3 below 0.037^9 / 9! ~ 3e-19, with 7 for
    // c1 < 1e-4 below 0.012^8 / 8! ~ 8e-21 (the leapfrog's links mostly fall in the last two tiers);
    // beyond c1 = 0.5 the closed form below.
    const int nterms = c1 < T(1e-4) ? 7 : (c1 < T(1e-3) ? 8 : (c1 < T(0.02) ? 11 : 17));
    T a = T(1), b = T(0), d = T(0);
    T f0r = T(1), f0i = T(0), f1r = T(0), f1i = T(0), f2r = T(0), f2i = T(0);
#pragma unroll
    for (int n = 1; n <= 17; n++) {
      if (n > nterms) break;
      const T inv = T(1) / T(n);
      const T an = c0 * d * inv, bn = fma(c1, d, a) * inv, dn = b * inv;
      a = an;
      b = bn;
      d = dn;
      if ((n & 3) == 1) {  // i^n = i
        f0i += a;
        f1i += b;
        f2i += d;
      } else if ((n & 3) == 2) {  // -1
        f0r -= a;
        f1r -= b;
        f2r -= d;
      } else if ((n & 3) == 3) {  // -i
        f0i -= a;
        f1i -= b;
        f2i -= d;
      } else {  // +1
        f0r += a;
        f1r += b;
        f2r += d;
      }
    }
    f0 = mk<T>(f0r, f0i);
    f1 = mk<T>(f1r, f1i);
    f2 = mk<T>(f2r, f2i);
  } else if (c1 < Trig<T>::taylor_c1()) {
    // the Taylor coefficients as products with folded reciprocals: a division by a constant whose
    // reciprocal is inexact compiles to a full division, which GB300 runs on its FP64 pipe (ten per
    // exponential here, on most links of weak fields)
    constexpr T r6 = T(1) / T(6), r24 = T(1) / T(24), r120 = T(1) / T(120), r360 = T(1) / T(360),
                r720 = T(1) / T(720);
    f0 = mk<T>(kMinusOne ? -(c0 * c0 * r720) : T(1) - c0 * c0 * r720, -c0 * r6 + c1 * c0 * r120);
    f1 = mk<T>(c0 * r24 - c0 * c1 * r360, T(1) - c1 * r6 + c1 * c1 * r120);
    f2 = mk<T>(T(-0.5) + c1 * r24 - c1 * c1 * r720, c0 * r120);
  } else {
    const bool neg = c0 < T(0);
    const T ac0 = neg ? -c0 : c0;
    const T s3 = Trig<T>::sqrt_(c1 * (T(1) / T(3)));
    const T c0max = T(2) * s3 * s3 * s3;
    T r = ac0 / c0max;
    r = r > T(1) ? T(1) : r;
    const T theta = Trig<T>::acos_(r);
    T st, ct;
    Trig<T>::sincos_(theta * (T(1) / T(3)), &st, &ct);
    const T u = s3 * ct;
    const T w = Trig<T>::sqrt_(c1) * st;
    const T u2 = u * u, w2 = w * w;
    T sw, cw;
    Trig<T>::sincos_(w, &sw, &cw);
    T xi0;
    if (w < T(0.05)) {
      xi0 = T(1) - w2 * (T(1) / T(6)) *
                       (T(1) - w2 * (T(1) / T(20)) * (T(1) - w2 * (T(1) / T(42)) * (T(1) - w2 * (T(1) / T(72)))));
    } else {
      xi0 = sw / w;
    }
    T su, cu;
    Trig<T>::sincos_(u, &su, &cu);
    const T c2u = cu * cu - su * su, s2u = T(2) * su * cu;  // e^{2iu} = (e^{iu})^2
    // e^{-iu} = (cu, -su)
    // h0 = (u^2-w^2) e^{2iu} + e^{-iu} (8u^2 cos w + 2iu(3u^2+w^2) xi0)
    const T a0r = T(8) * u2 * cw, a0i = T(2) * u * (T(3) * u2 + w2) * xi0;
    const T h0r = (u2 - w2) * c2u + (cu * a0r + su * a0i);
    const T h0i = (u2 - w2) * s2u + (cu * a0i - su * a0r);
    // h1 = 2u e^{2iu} - e^{-iu} (2u cos w - i(3u^2-w^2) xi0)
    const T a1r = T(2) * u * cw, a1i = -(T(3) * u2 - w2) * xi0;
    const T h1r = T(2) * u * c2u - (cu * a1r + su * a1i);
    const T h1i = T(2) * u * s2u - (cu * a1i - su * a1r);
    // h2 = e^{2iu} - e^{-iu} (cos w + 3iu xi0)
    const T a2r = cw, a2i = T(3) * u * xi0;
    const T h2r = c2u - (cu * a2r + su * a2i);
    const T h2i = s2u - (cu * a2i - su * a2r);
    const T den = T(1) / (T(9) * u2 - w2);
    f0 = mk<T>(h0r * den, h0i * den);
    f1 = mk<T>(h1r * den, h1i * den);
    f2 = mk<T>(h2r * den, h2i * den);
    if (neg) {
      f0.im = -f0.im;
      f1.re = -f1.re;
      f2.im = -f2.im;
    }
    if (kMinusOne) f0.re -= T(1);
  }
#pragma unroll
  for (int k = 0; k < 9; k++) {
    cx<T> v = mk<T>(T(0), T(0));
    cfma(v, f1, Q.e[k]);
    cfma(v, f2, Q2.e[k]);
    X.e[k] = v;
  }
  X.e[0].re += f0.re;
  X.e[0].im += f0.im;
  X.e[4].re += f0.re;
  X.e[4].im += f0.im;
  X.e[8].re += f0.re;
  X.e[8].im += f0.im;
}
template <typename T>
__device__ __forceinline__ void expi(T c, const Alg<T>& al, Mat<T>& X) {
  expi_impl<T, false>(c, al, X);
}
// exp(i c t.al) - 1.  Near the identity the diagonal of exp(iQ) is 1 - (Q^2)_ii/2 + ..., and in FP32 a
// deviation below ~3e-8 vanishes when it is added to 1, every step the same way: the links' norms then
// grow by ~tr Q^2 per step (measured: unitarity defect 2.9e-5 after 400 steps of an MV collision).
// Formed as X - 1 the small terms keep their relative precision; the link update U + (X - 1) U rounds
// once, at a point that moves from step to step, so they survive on average.
template <typename T>
__device__ __forceinline__ void expi_m1(T c, const Alg<T>& al, Mat<T>& Xm1) {
  expi_impl<T, true>(c, al, Xm1);
}
// a + b rounded stochastically: to the FP32 neighbour of the exact sum with probability equal to the
// fraction of the gap, so the rounding is unbiased.  The exact residual comes from TwoSum; the random
// number is a hash of the operands' bits (they change from step to step, so it needs no counter and
// gives the same bits in every launch path).
__device__ __forceinline__ float add_stochastic(float a, float b, unsigned salt) {
  const float s = a + b, bb = s - a;
  const float r = (a - (s - bb)) + (b - bb);
  if (r == 0.f) return s;
  const float t = nextafterf(s, r > 0.f ? 3.0e38f : -3.0e38f);
  const float p = fabsf(r / (t - s));
  unsigned h = (__float_as_uint(a) * 0x9E3779B1u) ^ (__float_as_uint(b) * 0x85EBCA77u) ^ salt;
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  h *= 0x297A2D39u;
  h ^= h >> 15;
  return (float)(h >> 8) * (1.f / 16777216.f) < p ? t : s;
}
// out = (1 + Xm1) u.  In FP32 the real parts of the diagonal are added with stochastic rounding: near
// the identity they receive only the second-order -(Q^2)_ii/2 per step (the first-order i Q u is
// imaginary there), which round-to-nearest would drop in the same direction every step, growing the
// links' norms between reunitarisations.
template <typename T>
__device__ __forceinline__ void mul_near_identity(const Mat<T>& Xm1, const Mat<T>& u, Mat<T>& out) {
  mul_nn(Xm1, u, out);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    if (sizeof(T) == 4 && (k == 0 || k == 4 || k == 8))
      out.e[k].re = (T)add_stochastic((float)u.e[k].re, (float)out.e[k].re, (unsigned)k);
    else
      out.e[k].re += u.e[k].re;
    out.e[k].im += u.e[k].im;
  }
}
// The link update's exponential and its application: FP32 keeps X - 1 (expi_m1), FP64 forms X.
template <typename T>
__device__ __forceinline__ void link_exp(T c, const Alg<T>& al, Mat<T>& X) {
  if (sizeof(T) == 4)
    expi_m1(c, al, X);
  else
    expi(c, al, X);
}
template <typename T>
__device__ __forceinline__ void link_apply(const Mat<T>& X, const Mat<T>& u, Mat<T>& out) {
  if (sizeof(T) == 4)
    mul_near_identity(X, u, out);
  else
    mul_nn(X, u, out);
}

// ||V V^dagger - 1||_F  (S/SUNc/SU3/GroupOperations.cpp:337-349)
template <typename T>
__device__ __forceinline__ T unitarity_norm(const Mat<T>& V) {
  Mat<T> C;
  mul_nd(V, V, C);
  T n = 0;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const T d = C.e[k].re - ((k % 4 == 0) ? T(1) : T(0));
    n += d * d + C.e[k].im * C.e[k].im;
  }
  return sqrt(n);
}

// Project onto SU(3) without rotating it: two Newton steps U <- (U + U^{-dagger})/2 towards the
// unitary polar factor (the unitary matrix closest in Frobenius norm), then the phase of the
// determinant is divided out, det^(-1/3).  FP64 arithmetic for either storage type.  (A Gram-Schmidt
// projection would turn the accumulated non-unitary part into a small rotation of the link, which
// shows up as a systematic shift of the plaquette energy.)
template <typename T>
__device__ __forceinline__ void reunitarize_newton(Mat<T>& V) {
  Mat<double> U;
#pragma unroll
  for (int k = 0; k < 9; k++) U.e[k] = mk<double>((double)V.e[k].re, (double)V.e[k].im);
#pragma unroll 1
  for (int it = 0; it < 2; it++) {
    Mat<double> C;  // signed cofactors C(i,j)
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
        cx<double> c = mk<double>(0, 0);
        cfma(c, U.e[i1 + 3 * j1], U.e[i2 + 3 * j2]);
        const cx<double> m = mk<double>(-U.e[i1 + 3 * j2].re, -U.e[i1 + 3 * j2].im);
        cfma(c, m, U.e[i2 + 3 * j1]);
        C.e[i + 3 * j] = c;
      }
    cx<double> det = mk<double>(0, 0);
#pragma unroll
    for (int j = 0; j < 3; j++) cfma(det, U.e[3 * j], C.e[3 * j]);
    // U^{-dagger}(i,j) = conj(C(i,j)) / conj(det) = conj(C(i,j)) * det / |det|^2
    const double n2 = det.re * det.re + det.im * det.im;
    const cx<double> f = mk<double>(det.re / n2, det.im / n2);
#pragma unroll
    for (int k = 0; k < 9; k++) {
      cx<double> w = mk<double>(0, 0);
      cfma(w, mk<double>(C.e[k].re, -C.e[k].im), f);
      U.e[k].re = 0.5 * (U.e[k].re + w.re);
      U.e[k].im = 0.5 * (U.e[k].im + w.im);
    }
  }
  // remove the determinant's phase
  cx<double> det = mk<double>(0, 0);
  {
    const cx<double> c0 = [&] {
      cx<double> c = mk<double>(0, 0);
      cfma(c, U.e[4], U.e[8]);
      cfma(c, mk<double>(-U.e[7].re, -U.e[7].im), U.e[5]);
      return c;
    }();
    const cx<double> c1 = [&] {
      cx<double> c = mk<double>(0, 0);
      cfma(c, U.e[5], U.e[6]);
      cfma(c, mk<double>(-U.e[8].re, -U.e[8].im), U.e[3]);
      return c;
    }();
    const cx<double> c2 = [&] {
      cx<double> c = mk<double>(0, 0);
      cfma(c, U.e[3], U.e[7]);
      cfma(c, mk<double>(-U.e[6].re, -U.e[6].im), U.e[4]);
      return c;
    }();
    cfma(det, U.e[0], c0);
    cfma(det, U.e[1], c1);
    cfma(det, U.e[2], c2);
  }
  double sp, cp;
  sincos(-atan2(det.im, det.re) / 3.0, &sp, &cp);
  const cx<double> ph = mk<double>(cp, sp);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    cx<double> w = mk<double>(0, 0);
    cfma(w, U.e[k], ph);
    V.e[k] = mk<T>((T)w.re, (T)w.im);
  }
}

// Same projection for FP32 links, kept unbiased.  A link within ~1e-6 of SU(3) is U = W (1 + e) with
// W the projection and e Hermitian and small; U W-ward is U (1 - e) to first order, and e = (U^d U - 1)/2.
// Everything small is formed as a small number: the diagonal of U^d U - 1 exactly (error-free FMA
// products, then the exact subtraction of 1), its off-diagonal in FP32 (no cancellation against 1
// there), the determinant's phase theta from an FP32 determinant, and the link is corrected as
// U + U M, M = -e - i theta/3, with one rounding.  Forming 1.5 - H/2 and U (1.5 - H/2) in FP32 instead
// (plain Newton-Schulz) rounds the ~1e-8 corrections at 1 and was measured to shrink the links' norms
// by 2e-8 on average, raising a weak-field plaquette energy by 1.8e-3.  Links that drifted far from
// SU(3) (||U^d U - 1|| > 1e-4) take the FP64 Newton path.
__device__ __forceinline__ float two_prod_sq_err(float a) { return fmaf(a, a, -a * a); }
__device__ __forceinline__ void reunitarize_f32(Mat<float>& U) {
  // e = (U^d U - 1)/2: the diagonal from exact squares, summed with their error terms
  float d[3];
#pragma unroll
  for (int j = 0; j < 3; j++) {
    float hi = 0.f, lo = 0.f;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const cx<float> u = U.e[k + 3 * j];
      const float pr = u.re * u.re, pi = u.im * u.im;
      lo += two_prod_sq_err(u.re) + two_prod_sq_err(u.im);
      // TwoSum of hi + pr and of that + pi
      float s = hi + pr, bb = s - hi;
      lo += (hi - (s - bb)) + (pr - bb);
      hi = s;
      s = hi + pi;
      bb = s - hi;
      lo += (hi - (s - bb)) + (pi - bb);
      hi = s;
    }
    d[j] = (hi - 1.f) + lo;  // hi - 1 is exact for hi in [0.5, 2]
  }
  cx<float> h01 = mk<float>(0, 0), h02 = mk<float>(0, 0), h12 = mk<float>(0, 0);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    cfma_cn(h01, U.e[k], U.e[k + 3]);
    cfma_cn(h02, U.e[k], U.e[k + 6]);
    cfma_cn(h12, U.e[k + 3], U.e[k + 6]);
  }
  const float dev = d[0] * d[0] + d[1] * d[1] + d[2] * d[2] +
                    2.f * (h01.re * h01.re + h01.im * h01.im + h02.re * h02.re + h02.im * h02.im +
                           h12.re * h12.re + h12.im * h12.im);
  // ||U^d U - 1||^2 <= 1e-8: the first-order correction leaves |e|^2 < 3e-9, below FP32 rounding
  if (!(dev <= 1e-8f)) {
    reunitarize_newton(U);
    return;
  }
  // the determinant's phase (~1e-7 for a link this close to SU(3)); its FP32 rounding is random in sign,
  // so the correction it drives is unbiased
  float theta;
  {
    cx<float> c0 = mk<float>(0, 0), c1 = mk<float>(0, 0), c2 = mk<float>(0, 0), det = mk<float>(0, 0);
    cfma(c0, U.e[4], U.e[8]);
    cfma(c0, mk<float>(-U.e[7].re, -U.e[7].im), U.e[5]);
    cfma(c1, U.e[5], U.e[6]);
    cfma(c1, mk<float>(-U.e[8].re, -U.e[8].im), U.e[3]);
    cfma(c2, U.e[3], U.e[7]);
    cfma(c2, mk<float>(-U.e[6].re, -U.e[6].im), U.e[4]);
    cfma(det, U.e[0], c0);
    cfma(det, U.e[1], c1);
    cfma(det, U.e[2], c2);
    theta = atan2f(det.im, det.re);
  }
  // M = -e - i theta/3 (e Hermitian: e_ij = h_ij / 2 off the diagonal, d_j / 2 on it)
  Mat<float> M, C;
  const float t3 = theta * (1.f / 3.f);
  M.e[0] = mk<float>(-0.5f * d[0], -t3);
  M.e[4] = mk<float>(-0.5f * d[1], -t3);
  M.e[8] = mk<float>(-0.5f * d[2], -t3);
  M.e[3] = mk<float>(-0.5f * h01.re, -0.5f * h01.im);  // (0,1)
  M.e[6] = mk<float>(-0.5f * h02.re, -0.5f * h02.im);  // (0,2)
  M.e[7] = mk<float>(-0.5f * h12.re, -0.5f * h12.im);  // (1,2)
  M.e[1] = mk<float>(M.e[3].re, -M.e[3].im);
  M.e[2] = mk<float>(M.e[6].re, -M.e[6].im);
  M.e[5] = mk<float>(M.e[7].re, -M.e[7].im);
  mul_nn(U, M, C);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    U.e[k].re += C.e[k].re;
    U.e[k].im += C.e[k].im;
  }
}

template <typename T>
__device__ __forceinline__ void reunitarize(Mat<T>& V) {
  if constexpr (sizeof(T) == 4)
    reunitarize_f32(V);
  else
    reunitarize_newton(V);
}

}  // namespace glasma

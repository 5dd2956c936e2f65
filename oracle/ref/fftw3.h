// fftw3.h -- TEST INFRASTRUCTURE ONLY.
//
// A minimal stand-in for the subset of FFTW 3's interface that the reference
// calls (S/FFT/FFT1D.cpp, S/FFT/FFT2D.cpp, S/FFT/FFT3D.cpp): fftw_plan_many_dft
// with unit embedding, fftw_execute, fftw_destroy_plan, fftw_alloc_complex,
// fftw_free and the threading calls.  FFTW (third-party, not vendored; the
// reference's job scripts load fftw/3.3.10) is absent from this machine, so the
// reference harness links this header instead.  It implements FFTW's documented
// transform: unnormalised multi-dimensional DFT, exponent sign -1 for
// FFTW_FORWARD and +1 for FFTW_BACKWARD, row-major dims (last fastest), element
// (i0..i_{r-1}) of transform k at  base[k*dist + stride*linear(i)].
// Written for this project; it is not FFTW code.
#ifndef GLASMA_ORACLE_FFTW3_SHIM_H
#define GLASMA_ORACLE_FFTW3_SHIM_H

#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>

typedef double fftw_complex[2];

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

struct glasma_fftw_plan_s {
  int rank;
  std::vector<int> n;
  int howmany;
  fftw_complex* in;
  fftw_complex* out;
  int istride, idist, ostride, odist;
  int sign;
};
typedef glasma_fftw_plan_s* fftw_plan;

inline fftw_complex* fftw_alloc_complex(size_t count) {
  return static_cast<fftw_complex*>(std::calloc(count ? count : 1, sizeof(fftw_complex)));
}
inline void fftw_free(void* p) { std::free(p); }
inline int fftw_init_threads(void) { return 1; }
inline void fftw_plan_with_nthreads(int) {}
inline void fftw_cleanup_threads(void) {}

inline fftw_plan fftw_plan_many_dft(int rank, const int* n, int howmany, fftw_complex* in, const int* /*inembed*/,
                                    int istride, int idist, fftw_complex* out, const int* /*onembed*/, int ostride,
                                    int odist, int sign, unsigned /*flags*/) {
  fftw_plan p = new glasma_fftw_plan_s;
  p->rank = rank;
  p->n.assign(n, n + rank);
  p->howmany = howmany;
  p->in = in;
  p->out = out;
  p->istride = istride;
  p->idist = idist;
  p->ostride = ostride;
  p->odist = odist;
  p->sign = sign;
  return p;
}

inline void glasma_fftw_dft1(std::complex<double>* a, int len, long step, int sign, std::vector<std::complex<double>>& buf) {
  buf.resize(len);
  for (int k = 0; k < len; k++) {
    std::complex<double> acc = 0.0;
    for (int j = 0; j < len; j++) {
      const long m = ((long)j * k) % len;
      const double ang = sign * 2.0 * M_PI * (double)m / len;
      acc += a[j * step] * std::complex<double>(std::cos(ang), std::sin(ang));
    }
    buf[k] = acc;
  }
  for (int k = 0; k < len; k++) a[k * step] = buf[k];
}

inline void glasma_fftw_pow2(std::complex<double>* a, int len, long step, int sign, std::vector<std::complex<double>>& buf) {
  buf.resize(len);
  for (int i = 0; i < len; i++) buf[i] = a[i * step];
  for (int i = 1, j = 0; i < len; i++) {
    int bit = len >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(buf[i], buf[j]);
  }
  for (int m = 2; m <= len; m <<= 1) {
    const double ang = sign * 2.0 * M_PI / m;
    for (int i = 0; i < len; i += m)
      for (int k = 0; k < m / 2; k++) {
        const std::complex<double> w(std::cos(ang * k), std::sin(ang * k));
        const std::complex<double> u = buf[i + k], v = buf[i + k + m / 2] * w;
        buf[i + k] = u + v;
        buf[i + k + m / 2] = u - v;
      }
  }
  for (int i = 0; i < len; i++) a[i * step] = buf[i];
}

inline void fftw_execute(const fftw_plan p) {
  long total = 1;
  for (int d = 0; d < p->rank; d++) total *= p->n[d];
  std::vector<std::complex<double>> work(total), buf;
  for (int k = 0; k < p->howmany; k++) {
    for (long i = 0; i < total; i++) {
      const fftw_complex& v = p->in[(long)k * p->idist + (long)p->istride * i];
      work[i] = std::complex<double>(v[0], v[1]);
    }
    long inner = total;
    for (int d = 0; d < p->rank; d++) {
      const int len = p->n[d];
      inner /= len;  // stride of axis d in the row-major linear index
      const long outer = total / ((long)len * inner);
      for (long o = 0; o < outer; o++)
        for (long in = 0; in < inner; in++) {
          std::complex<double>* line = work.data() + o * (long)len * inner + in;
          if ((len & (len - 1)) == 0)
            glasma_fftw_pow2(line, len, inner, p->sign, buf);
          else
            glasma_fftw_dft1(line, len, inner, p->sign, buf);
        }
    }
    for (long i = 0; i < total; i++) {
      fftw_complex& v = p->out[(long)k * p->odist + (long)p->ostride * i];
      v[0] = work[i].real();
      v[1] = work[i].imag();
    }
  }
}

inline void fftw_destroy_plan(fftw_plan p) { delete p; }

#endif

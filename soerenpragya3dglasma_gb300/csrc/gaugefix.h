// gaugefix.h -- internal interface of the Coulomb gauge fixer (gaugefix.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "lattice.cuh"

namespace glasma {

struct GaugeFixState;  // FFT plan, work arrays; owned by the lattice handle

struct GaugeFixArgs {
  Geometry g;
  int precision;
  double a_scale;
  cudaStream_t stream;
  void* U;
  void* E;
  void* G;
  void* UG;
  void* EG;
  double* scratch;
  size_t scratch_doubles;
};

int gaugefix_run(GaugeFixState** state, const GaugeFixArgs& a, double alpha, int max_iters, double tol, unsigned flags,
                 double* log, int* iterations, std::string* err);
// Los Alamos (GLASMA_GF_LOS_ALAMOS, param = over-relaxation probability) or Jacobi (GLASMA_GF_JACOBI,
// param = step size) Coulomb gauge fixing; needs no FFT state.
int gaugefix_run_local(const GaugeFixArgs& a, int algorithm, double param, unsigned long long seed, int max_iters,
                       double tol, double* log, int* iterations, std::string* err);
// scratch doubles the gauge fixers need (reduction partials and results)
size_t gaugefix_scratch_doubles();
void gaugefix_destroy(GaugeFixState* state);

// jG(x) = G(x) j(x) G^dagger(x) of one colour-charge field (device SoA j[a][S], precision of the handle)
// into `out`, FP64 in the host layout [S][8]; the ghost slices take the edge slices' values.
cudaError_t launch_transform_charge(const GaugeFixArgs& a, const void* J, double* out);

// Batched 1D transforms of length n in place over `total` complex values: element k of line l is
// at l*n + k (st == 1) or at o*st*n + i + k*st (st > 1, l = (o, i)); unnormalised, sign -1 forward,
// +1 inverse.  tw = make_twiddles(n) (cudaFree it when done).
cudaError_t fft_lines(double2* X, int n, long long st, long long total, int inverse, const double2* tw,
                      cudaStream_t stream);
double2* make_twiddles(int n, cudaStream_t stream);
// 3D transform (unnormalised, sign -1 forward / +1 inverse) of 8 colour planes X[a][z][y][x];
// `in` / `out` may be host or device memory.
int gaugefix_fft_test(GaugeFixState** state, const GaugeFixArgs& a, const double2* in, double2* out, int inverse,
                      std::string* err);
int gaugefix_fft_test_f32(GaugeFixState** state, const GaugeFixArgs& a, const float2* in, float2* out, int inverse,
                          std::string* err);

}  // namespace glasma

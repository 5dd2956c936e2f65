// adjoint.cu -- adjoint (reverse-mode) leapfrog: gradients of a late-time observable with respect
// to the initial electric field and the initial colour currents, in the lattice's precision (FP64 or FP32).
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

namespace glasma {
namespace adj64 {
#define ADJ_REAL double
#include "adjoint_kernels.inc"
#undef ADJ_REAL
}  // namespace adj64
namespace adj32 {
#define ADJ_REAL float
#include "adjoint_kernels.inc"
#undef ADJ_REAL
}  // namespace adj32
}  // namespace glasma

extern "C" {

int glasma_objective(glasma_lattice* h, int z_begin, int z_end, const double* num, const double* den, double* value) {
  if (!h || !num || !den || !value) return afail(GLASMA_ERR_INVALID_ARGUMENT, "null argument");
  if (z_begin < 0 || z_end > h->g.nz || z_begin >= z_end) return afail(GLASMA_ERR_INVALID_ARGUMENT, "bad slice range");
  cudaSetDevice(h->device);
  DevBuf scratch;
  if (!scratch.alloc(sizeof(double) * 608 * 6)) return afail(GLASMA_ERR_OUT_OF_MEMORY, "scratch");
  double q[6], N, D;
  int st = h->precision == GLASMA_FP64 ? glasma::adj64::objective_q(h, z_begin, z_end, q, static_cast<double*>(scratch.p))
                                       : glasma::adj32::objective_q(h, z_begin, z_end, q, static_cast<double*>(scratch.p));
  if (st) return st;
  *value = ratio(num, den, q, &N, &D);
  return GLASMA_OK;
}

int glasma_adjoint(glasma_lattice* h, double dt, int nsteps, int checkpoint_every, int z_begin, int z_end,
                   const double* num, const double* den, double* objective, double* grad_E, double* grad_Jp,
                   double* grad_Jm, double* grad_JpStat, double* grad_JmStat) {
  if (!h || !num || !den) return afail(GLASMA_ERR_INVALID_ARGUMENT, "null argument");
  if (nsteps < 1 || checkpoint_every < 1) return afail(GLASMA_ERR_INVALID_ARGUMENT, "nsteps, checkpoint_every >= 1");
  if (z_begin < 0 || z_end > h->g.nz || z_begin >= z_end) return afail(GLASMA_ERR_INVALID_ARGUMENT, "bad slice range");
  if (cudaSetDevice(h->device) != cudaSuccess) return afail(GLASMA_ERR_CUDA, "cudaSetDevice");
  return h->precision == GLASMA_FP64
             ? glasma::adj64::run_adjoint(h, dt, nsteps, checkpoint_every, z_begin, z_end, num, den, objective, grad_E,
                                          grad_Jp, grad_Jm, grad_JpStat, grad_JmStat)
             : glasma::adj32::run_adjoint(h, dt, nsteps, checkpoint_every, z_begin, z_end, num, den, objective, grad_E,
                                          grad_Jp, grad_Jm, grad_JpStat, grad_JmStat);
}

const char* glasma_adjoint_last_error(void) { return g_adj_error.c_str(); }

}  // extern "C"

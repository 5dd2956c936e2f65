// handle.h -- the lattice handle behind the C ABI (internal to the library).
#pragma once

#include <cuda_runtime.h>

#include "gaugefix.h"
#include "lattice.cuh"

struct glasma_lattice {
  glasma::Geometry g;
  int precision;
  int reunit_every;
  long long steps_done;
  double a_scale;
  int device;
  cudaStream_t own_stream;
  cudaStream_t stream;
  size_t real_bytes;  // 8 or 4
  void* f[10];        // device SoA fields, indexed by glasma_field (G, UG, EG allocated lazily)
  double* staging;    // device AoS staging buffer for host copies
  size_t staging_bytes;
  double* scratch;    // reduction partials and results
  double* result_host;  // page-locked, mapped: observables' results written here by a kernel (first use)
  double* result_dev;   // its device address
  size_t scratch_doubles;
  glasma::GaugeFixState* gf;
  int tile_x;         // K1 tile width along x (autotuned)
  void* alt[10];      // second buffer set of the one-pass step (U, JP, JM, JPSTAT, JMSTAT; lazily)
  int step_method;    // GLASMA_STEP_ONE_PASS / _TWO_PASS / _PLAQUETTE / _MARCH
  int march_lz;       // z slices per block of the marching step (0: chosen from the lattice)
  int last_method;    // method the last glasma_step used
  int link_rows;      // rows of each link the step kernels read and write: 3, or 2 (12-real links, FP32)
  void* contrib;      // plaquette method: 6 x 8 weighted force contributions per site (lazily)
  int fp64_arith;     // GLASMA_FP64_NATIVE or GLASMA_FP64_DOUBLE_FLOAT (the plaquette force kernel)
  unsigned long long swaps;  // buffer swaps so far (batched launches rebuild their tables on change)
  // asynchronous uploads (glasma_upload_begin / glasma_upload_finish)
  cudaStream_t xfer_stream;  // copies host -> staging, overlapping the handle's kernels (first use)
  cudaEvent_t xfer_done;     // recorded on xfer_stream at finish: every begun copy has landed
  cudaEvent_t stage_free[2];  // recorded on the handle's stream at finish: that set's staging has been read
  double* stage_f[2][10];     // two sets of per-field staging areas (reference host layout), alternating
  int stage_slot;             // the set the next begin copies into (flips at each finish)
  unsigned pending;          // fields begun and not yet finished (bit per glasma_field)
};

// The autotuner of the staple kernels whatever the handle's step method (batches stepping with the
// two-pass method use the staple kernels).
extern "C" int glasma_autotune_staple(glasma_lattice* h, double dt, int* tile_x);

namespace glasma {
// Default K1 tile width: the widest power of two dividing the block that does not exceed Nx.
// allocates the plaquette method's contribution buffer of h (false when that fails)
bool ensure_contrib(glasma_lattice* h);

inline int default_tile_x(int nx) {
  int t = 128;
  while (t > 1 && t > nx) t >>= 1;
  return t;
}
}  // namespace glasma

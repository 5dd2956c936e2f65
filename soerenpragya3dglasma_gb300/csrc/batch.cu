// batch.cu -- many independent lattices ("events") of uneven sizes advanced together.
//
// Each event is an ordinary lattice handle (its own fields, ghost slices, tile shape).  A step of
// the whole batch is two launches: the electric-field/JStat kernel walks the list of all events'
// K1 tiles, the link/J kernel the list of all events' 128-site chunks (one block per tile, or a
// persistent grid that strides through the list); a block finds its event by binary search over the
// per-event tile offsets.  The per-site arithmetic is the
// single-lattice kernels' (leapfrog_sites.cuh), so a batched step is bit-identical to stepping
// every event on its own.  Blocks of steps are captured once into a CUDA graph and replayed.
// No reference counterpart: the reference farms independent seeds out as separate jobs
// (W/Script.sh), one lattice per process.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/glasma_gb300.h"
#include "handle.h"
#include "leapfrog_sites.cuh"

namespace glasma {
namespace {

template <typename T>
struct EventDesc {
  Geometry g;
  FieldPtrs<T> f;
  EParams<T> ep;
  LParams<T> lp;
  TileMap tm;
  long long k1_begin;  // first K1 tile of this event in the batch's tile list
  long long k2_begin;  // first 128-site chunk of this event
};

// R: rows of each link read and written (3 full, 2 for 12-real links).
template <typename T, typename I, int R>
__global__ void __launch_bounds__(kThreads, Occupancy<T>::kMinBlocks)
    efield_batch_kernel(const EventDesc<T>* __restrict__ ev, const unsigned short* __restrict__ tile_ev, long long total) {
  __shared__ cx<T> sh[StapleShare<T>::kSlots * 9 * kThreads + 1];
  for (long long t = blockIdx.x; t < total; t += gridDim.x) {
    const int e = tile_ev[t];
    // Local copies: the site body stores through these pointers, so references into the table
    // would have to be re-read from global memory after every store.
    const Geometry g = ev[e].g;
    const FieldPtrs<T> f = ev[e].f;
    const EParams<T> ep = ev[e].ep;
    const TileMap tm = ev[e].tm;
    int x, y, z;
    if (tm.site(t - ev[e].k1_begin, threadIdx.x, g.nx, g.ny, x, y, z)) efield_site<T, I, R>(g, f, ep, x, y, z, StapleShare<T>::kSlots ? sh : nullptr);
  }
}

template <typename T, typename I, int R>
__global__ void __launch_bounds__(kThreads, Occupancy<T>::kLinksMinBlocks)
    links_batch_kernel(const EventDesc<T>* __restrict__ ev, const unsigned short* __restrict__ tile_ev, long long total) {
  for (long long t = blockIdx.x; t < total; t += gridDim.x) {
    const int e = tile_ev[t];
    const Geometry g = ev[e].g;
    const FieldPtrs<T> f = ev[e].f;
    const LParams<T> lp = ev[e].lp;
    const long long idx = (t - ev[e].k2_begin) * kThreads + threadIdx.x;
    if (idx < g.vol) links_site<T, I, R>(g, f, lp, (I)idx);
  }
}

}  // namespace
}  // namespace glasma

struct glasma_batch {
  std::vector<glasma_lattice*> ev;
  int precision = 0;
  int reunit_every = 0;
  long long steps_done = 0;
  cudaStream_t own_stream = nullptr, stream = nullptr;
  void* d_desc = nullptr;
  unsigned short* d_tile_ev = nullptr;  // event of every K1 tile, then of every K2 chunk
  long long tile_ev_cap = 0;
  double desc_dt = NAN;
  long long k1_total = 0, k2_total = 0;
  bool idx32 = true;
  int grid1 = 0, grid2 = 0;
  int launch_mode = GLASMA_BATCH_TILE_GRID;
  int link_rows = 3;  // 2: 12-real links (FP32), as glasma_set_link_storage
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  double graph_dt = NAN;
  std::vector<unsigned long long> swaps;  // each event's buffer-swap count when the table was built
};

namespace {

thread_local std::string g_batch_error;
int bfail(int st, const std::string& m) {
  g_batch_error = m;
  return st;
}
int bcuda(cudaError_t e, const char* where) { return bfail(GLASMA_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e)); }

template <typename T>
glasma::FieldPtrs<T> handle_ptrs(glasma_lattice* h) {
  glasma::FieldPtrs<T> p;
  p.U = static_cast<glasma::cx<T>*>(h->f[GLASMA_FIELD_U]);
  p.UOld = static_cast<glasma::cx<T>*>(h->f[GLASMA_FIELD_UOLD]);
  p.E = static_cast<T*>(h->f[GLASMA_FIELD_E]);
  p.Jp = static_cast<T*>(h->f[GLASMA_FIELD_JP]);
  p.Jm = static_cast<T*>(h->f[GLASMA_FIELD_JM]);
  p.JpStat = static_cast<T*>(h->f[GLASMA_FIELD_JPSTAT]);
  p.JmStat = static_cast<T*>(h->f[GLASMA_FIELD_JMSTAT]);
  return p;
}

template <typename T, int R>
void batch_occupancy(const glasma_batch* b, int& per1, int& per2) {
  using namespace glasma;
  if (b->idx32) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, efield_batch_kernel<T, int, R>, kThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, links_batch_kernel<T, int, R>, kThreads, 0);
  } else {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, efield_batch_kernel<T, long long, R>, kThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, links_batch_kernel<T, long long, R>, kThreads, 0);
  }
}

// (Re)build the device event table for time step dt.
template <typename T>
int build_descriptors(glasma_batch* b, double dt) {
  using namespace glasma;
  std::vector<EventDesc<T>> d(b->ev.size());
  long long k1 = 0, k2 = 0;
  b->idx32 = true;
  for (size_t i = 0; i < b->ev.size(); i++) {
    glasma_lattice* h = b->ev[i];
    EventDesc<T>& e = d[i];
    e.g = h->g;
    e.f = handle_ptrs<T>(h);
    // same constants as the single-lattice launches (leapfrog.cu)
    const double a3 = h->g.a[0] * h->g.a[1] * h->g.a[2];
    const double gamma = -2.0 * dt * a3;
    for (int mu = 0; mu < 3; mu++) {
      const double ce = 1.0 / (h->g.a[mu] * h->g.a[mu]);
      e.ep.gc[mu] = (T)(gamma * ce);
      e.ep.cnu[mu] = (T)ce;
      e.lp.cU[mu] = (T)(-(0.5 * dt) * h->g.a[mu] * h->g.a[mu] / a3);
    }
    e.ep.jz = (T)(-(dt / h->g.a[2]) * 0.70710678118654752440084436210484903928483593768847);
    e.ep.cj = (T)(dt / h->g.a[2]);
    e.ep.do_e = 1;
    e.ep.do_jstat = 1;
    e.ep.dry = 0;
    e.lp.cj = (T)(dt / h->g.a[2]);
    e.lp.save_uold = 0;
    e.lp.do_j = 1;
    e.lp.do_second = 1;
    e.tm = TileMap::make(h->g.nx, h->g.ny, h->tile_x, kThreads);
    e.k1_begin = k1;
    e.k2_begin = k2;
    k1 += e.tm.tiles(h->g.nz);
    k2 += (h->g.vol + kThreads - 1) / kThreads;
    if (!use_32bit_index(h->g)) b->idx32 = false;
  }
  b->k1_total = k1;
  b->k2_total = k2;
  b->swaps.clear();
  for (glasma_lattice* h : b->ev) b->swaps.push_back(h->swaps);
  const size_t bytes = sizeof(EventDesc<T>) * d.size();
  if (!b->d_desc) {
    cudaError_t e = cudaMalloc(&b->d_desc, bytes);
    if (e != cudaSuccess) return bfail(GLASMA_ERR_OUT_OF_MEMORY, "cudaMalloc event table");
  }
  // tile -> event table: one load per block instead of a search through the event table
  std::vector<unsigned short> tev((size_t)(k1 + k2));
  for (size_t i = 0; i < d.size(); i++) {
    const long long k1_end = i + 1 < d.size() ? d[i + 1].k1_begin : k1;
    const long long k2_end = i + 1 < d.size() ? d[i + 1].k2_begin : k2;
    for (long long t = d[i].k1_begin; t < k1_end; t++) tev[(size_t)t] = (unsigned short)i;
    for (long long t = d[i].k2_begin; t < k2_end; t++) tev[(size_t)(k1 + t)] = (unsigned short)i;
  }
  if (b->tile_ev_cap < k1 + k2) {
    if (b->d_tile_ev) {
      cudaStreamSynchronize(b->stream);
      cudaFree(b->d_tile_ev);
      b->d_tile_ev = nullptr;
    }
    if (cudaMalloc(&b->d_tile_ev, sizeof(unsigned short) * (size_t)(k1 + k2)) != cudaSuccess) {
      cudaGetLastError();
      b->tile_ev_cap = 0;
      return bfail(GLASMA_ERR_OUT_OF_MEMORY, "cudaMalloc tile table");
    }
    b->tile_ev_cap = k1 + k2;
  }
  cudaError_t e = cudaMemcpyAsync(b->d_tile_ev, tev.data(), sizeof(unsigned short) * tev.size(),
                                  cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_desc, d.data(), bytes, cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bcuda(e, "event table upload");
  // persistent grids: as many blocks as fit on the device at once
  int dev = 0, sms = 0, per1 = 0, per2 = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  bool two_row = false;
  if constexpr (sizeof(T) == 4) two_row = b->link_rows == 2;
  if (two_row)
    batch_occupancy<T, 2>(b, per1, per2);
  else
    batch_occupancy<T, 3>(b, per1, per2);
  if (b->launch_mode == GLASMA_BATCH_TILE_GRID && k1 < (1LL << 31) && k2 < (1LL << 31)) {
    b->grid1 = (int)k1;
    b->grid2 = (int)k2;
  } else {
    b->grid1 = (int)std::min<long long>(k1, (long long)sms * std::max(per1, 1));
    b->grid2 = (int)std::min<long long>(k2, (long long)sms * std::max(per2, 1));
  }
  b->desc_dt = dt;
  return GLASMA_OK;
}

template <typename T, int R>
void launch_batch_rows(glasma_batch* b) {
  using namespace glasma;
  const EventDesc<T>* ev = static_cast<const EventDesc<T>*>(b->d_desc);
  if (b->idx32) {
    efield_batch_kernel<T, int, R><<<b->grid1, kThreads, 0, b->stream>>>(ev, b->d_tile_ev, b->k1_total);
    links_batch_kernel<T, int, R><<<b->grid2, kThreads, 0, b->stream>>>(ev, b->d_tile_ev + b->k1_total, b->k2_total);
  } else {
    efield_batch_kernel<T, long long, R><<<b->grid1, kThreads, 0, b->stream>>>(ev, b->d_tile_ev, b->k1_total);
    links_batch_kernel<T, long long, R><<<b->grid2, kThreads, 0, b->stream>>>(ev, b->d_tile_ev + b->k1_total,
                                                                              b->k2_total);
  }
}

template <typename T>
cudaError_t launch_batch_step(glasma_batch* b) {
  if constexpr (sizeof(T) == 4) {
    if (b->link_rows == 2) {
      launch_batch_rows<T, 2>(b);
      return cudaGetLastError();
    }
  }
  launch_batch_rows<T, 3>(b);
  return cudaGetLastError();
}

cudaError_t reunitarize_all(glasma_batch* b) {
  for (glasma_lattice* h : b->ev) {
    cudaError_t e = b->precision == GLASMA_FP64
                        ? glasma::launch_reunitarize<double>(h->g, static_cast<glasma::cx<double>*>(h->f[GLASMA_FIELD_U]), b->stream)
                        : glasma::launch_reunitarize<float>(h->g, static_cast<glasma::cx<float>*>(h->f[GLASMA_FIELD_U]), b->stream,
                                                            b->link_rows);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// 12-real links: row 2 of every event's links from rows 0 and 1 (full links between calls).
cudaError_t complete_all(glasma_batch* b) {
  if (b->link_rows != 2) return cudaSuccess;
  for (glasma_lattice* h : b->ev) {
    cudaError_t e =
        glasma::launch_complete_links<float>(h->g, static_cast<glasma::cx<float>*>(h->f[GLASMA_FIELD_U]), b->stream);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// One step of every event; reunitarisation on the batch's step counter.
cudaError_t one_step(glasma_batch* b) {
  cudaError_t e = b->precision == GLASMA_FP64 ? launch_batch_step<double>(b) : launch_batch_step<float>(b);
  if (e != cudaSuccess) return e;
  b->steps_done++;
  if (b->reunit_every > 0 && b->steps_done % b->reunit_every == 0) e = reunitarize_all(b);
  return e;
}

}  // namespace

extern "C" {

int glasma_batch_create(int n_events, const int* extents, const double* spacings, int precision, int reunitarize_every,
                        glasma_batch** out) {
  if (!out || !extents || !spacings || n_events < 1) return bfail(GLASMA_ERR_INVALID_ARGUMENT, "bad arguments");
  if (n_events > 65535) return bfail(GLASMA_ERR_INVALID_ARGUMENT, "at most 65535 events per batch");
  *out = nullptr;
  glasma_batch* b = new glasma_batch;
  b->precision = precision;
  b->reunit_every = precision == GLASMA_FP32 ? reunitarize_every : 0;
  cudaError_t e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete b;
    return bcuda(e, "stream");
  }
  b->stream = b->own_stream;
  for (int i = 0; i < n_events; i++) {
    glasma_lattice* h = nullptr;
    int st = glasma_create(extents[3 * i], extents[3 * i + 1], extents[3 * i + 2], spacings[3 * i], spacings[3 * i + 1],
                           spacings[3 * i + 2], precision, 0, &h);
    if (st != GLASMA_OK) {
      g_batch_error = std::string("event ") + std::to_string(i) + ": " + glasma_last_error();
      for (glasma_lattice* x : b->ev) glasma_destroy(x);
      cudaStreamDestroy(b->own_stream);
      delete b;
      return st;
    }
    glasma_set_stream(h, b->stream);
    b->ev.push_back(h);
  }
  *out = b;
  return GLASMA_OK;
}

int glasma_batch_destroy(glasma_batch* b) {
  if (!b) return GLASMA_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (glasma_lattice* h : b->ev) glasma_destroy(h);
  if (b->d_desc) cudaFree(b->d_desc);
  if (b->d_tile_ev) cudaFree(b->d_tile_ev);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
  return GLASMA_OK;
}

int glasma_batch_set_stream(glasma_batch* b, void* stream) {
  if (!b) return bfail(GLASMA_ERR_INVALID_ARGUMENT, "null batch");
  cudaStreamSynchronize(b->stream);
  b->stream = stream ? static_cast<cudaStream_t>(stream) : b->own_stream;
  for (glasma_lattice* h : b->ev) glasma_set_stream(h, b->stream);
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return GLASMA_OK;
}

int glasma_batch_event(glasma_batch* b, int event, glasma_lattice** out) {
  if (!b || !out || event < 0 || event >= (int)b->ev.size()) return bfail(GLASMA_ERR_INVALID_ARGUMENT, "bad event");
  *out = b->ev[event];
  return GLASMA_OK;
}

int glasma_batch_autotune(glasma_batch* b, double dt, int* tiles) {
  if (!b) return bfail(GLASMA_ERR_INVALID_ARGUMENT, "null batch");
  std::map<std::tuple<int, int, int>, int> chosen;  // one tuning run per distinct lattice shape
  for (size_t i = 0; i < b->ev.size(); i++) {
    glasma_lattice* h = b->ev[i];
    const auto key = std::make_tuple(h->g.nx, h->g.ny, h->g.nz);
    auto it = chosen.find(key);
    int tx = 0;
    if (it == chosen.end()) {
      int st = glasma_autotune(h, dt, &tx);
      if (st != GLASMA_OK) return st;
      chosen[key] = tx;
    } else {
      tx = it->second;
      glasma_set_tile(h, tx);
    }
    if (tiles) tiles[i] = tx;
  }
  b->desc_dt = NAN;  // tile shapes changed: rebuild the event table and the graph
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return GLASMA_OK;
}

int glasma_batch_step(glasma_batch* b, double dt, int nsteps, int use_graph) {
  if (!b || nsteps < 0) return bfail(GLASMA_ERR_INVALID_ARGUMENT, "bad arguments");
  if (nsteps == 0) return GLASMA_OK;
  int st;
  bool stale = b->swaps.size() != b->ev.size();  // an event stepped on its own swapped its buffers
  for (size_t i = 0; !stale && i < b->ev.size(); i++) stale = b->swaps[i] != b->ev[i]->swaps;
  if (!(b->desc_dt == dt) || stale) {
    st = b->precision == GLASMA_FP64 ? build_descriptors<double>(b, dt) : build_descriptors<float>(b, dt);
    if (st != GLASMA_OK) return st;
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
  }
  // UpdateElectricFields syncs the U ghosts first (S/DYNAMICS/SUNcDynamics.cpp:151)
  for (glasma_lattice* h : b->ev) {
    cudaError_t e = b->precision == GLASMA_FP64
                        ? glasma::launch_sync_ghosts<glasma::cx<double>>(h->g, static_cast<glasma::cx<double>*>(h->f[GLASMA_FIELD_U]), 27, b->stream)
                        : glasma::launch_sync_ghosts<glasma::cx<float>>(h->g, static_cast<glasma::cx<float>*>(h->f[GLASMA_FIELD_U]), 27, b->stream);
    if (e != cudaSuccess) return bcuda(e, "ghost sync");
  }
  const int block = b->reunit_every > 0 ? b->reunit_every : 16;
  int done = 0;
  cudaError_t e = cudaSuccess;
  // single steps until the step counter is aligned to a graph block
  while (done < nsteps && (!use_graph || b->steps_done % block != 0 || nsteps - done < block)) {
    if ((e = one_step(b)) != cudaSuccess) return bcuda(e, "batch step");
    done++;
  }
  if (nsteps - done >= block && !b->graph) {
    cudaGraph_t g;
    if ((e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return bcuda(e, "capture");
    const long long saved = b->steps_done;
    for (int i = 0; i < block && e == cudaSuccess; i++) e = one_step(b);
    b->steps_done = saved;
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess) return bcuda(e, "captured step");
    if (e2 != cudaSuccess) return bcuda(e2, "end capture");
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bcuda(e, "graph instantiate");
    b->graph_steps = block;
  }
  while (nsteps - done >= block && b->graph) {
    if ((e = cudaGraphLaunch(b->graph, b->stream)) != cudaSuccess) return bcuda(e, "graph launch");
    b->steps_done += block;
    done += block;
  }
  while (done < nsteps) {
    if ((e = one_step(b)) != cudaSuccess) return bcuda(e, "batch step");
    done++;
  }
  if ((e = complete_all(b)) != cudaSuccess) return bcuda(e, "complete links");
  return GLASMA_OK;
}

int glasma_batch_set_link_storage(glasma_batch* b, int reals_per_link) {
  if (!b) return bfail(GLASMA_ERR_INVALID_ARGUMENT, "null batch");
  if (reals_per_link != 18 && reals_per_link != 12)
    return bfail(GLASMA_ERR_INVALID_ARGUMENT, "reals_per_link must be 18 or 12");
  if (reals_per_link == 12 && b->precision != GLASMA_FP32)
    return bfail(GLASMA_ERR_UNSUPPORTED, "12-real links are built for FP32 batches only");
  const int rows = reals_per_link == 12 ? 2 : 3;
  if (rows != b->link_rows) {
    b->link_rows = rows;
    b->desc_dt = NAN;  // persistent grids are sized for the kernels of this storage
    if (b->graph) {
      cudaStreamSynchronize(b->stream);
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
  }
  for (glasma_lattice* h : b->ev) glasma_set_link_storage(h, reals_per_link);  // events stepped alone
  return GLASMA_OK;
}

int glasma_batch_set_launch(glasma_batch* b, int mode) {
  if (!b || (mode != GLASMA_BATCH_PERSISTENT && mode != GLASMA_BATCH_TILE_GRID))
    return bfail(GLASMA_ERR_INVALID_ARGUMENT, "bad batch or launch mode");
  if (mode != b->launch_mode) {
    b->launch_mode = mode;
    b->desc_dt = NAN;  // grids are sized when the event table is built
    if (b->graph) {
      cudaStreamSynchronize(b->stream);
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
  }
  return GLASMA_OK;
}

int glasma_batch_energy(glasma_batch* b, double* t00) {
  if (!b || !t00) return bfail(GLASMA_ERR_INVALID_ARGUMENT, "bad arguments");
  for (size_t i = 0; i < b->ev.size(); i++) {
    double out[16];
    int st = glasma_bulk(b->ev[i], out);
    if (st != GLASMA_OK) return st;
    t00[i] = out[9];
  }
  return GLASMA_OK;
}

int glasma_batch_synchronize(glasma_batch* b) {
  if (!b) return bfail(GLASMA_ERR_INVALID_ARGUMENT, "null batch");
  cudaError_t e = cudaStreamSynchronize(b->stream);
  return e == cudaSuccess ? GLASMA_OK : bcuda(e, "sync");
}

const char* glasma_batch_last_error(void) { return g_batch_error.c_str(); }

}  // extern "C"

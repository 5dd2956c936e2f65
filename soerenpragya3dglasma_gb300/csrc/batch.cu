// batch.cu -- many independent lattices ("events") of uneven sizes advanced together.
//
// Each event is an ordinary lattice handle (its own fields, ghost slices, tile shape).  A step of
// the whole batch is two launches per group of up to kTableEvents events (one group for the
// 64-event workload).  With the staple kernels (two-pass method) the electric-field/JStat kernel
// walks the list of the group's K1 tiles, the link/J kernel the list of its 128-site chunks; with
// the plaquette method the force kernel walks 128-site chunks of every event's plaquette owners
// (slices -1 .. Nz-1) and writes the event's contribution buffer, and the gathering link kernel
// walks the 128-site chunks of the sites.  One block takes one tile or chunk, or a persistent grid
// strides through the list; a block finds its event in a tile -> event table.  The group's event
// descriptors are a __grid_constant__ kernel parameter, read in place from the constant bank.  The
// per-site arithmetic is the
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
  T* C;                // plaquette method: the event's contribution buffer (48 S reals)
  long long k1_begin;  // first K1 tile (plaquette method: owner chunk) of this event in the batch's list
  long long k2_begin;  // first 128-site chunk of this event
};

// Event descriptors of one launch group, passed by value: 96 x 280 B (FP64) stays inside the 32 KB
// kernel-parameter limit.  As __grid_constant__ the table is read in place from the constant bank;
// the earlier global-memory table, copied into registers per tile, cost the link kernel 452 B of
// spill stores per thread (116 B in the single-lattice kernel).
constexpr int kTableEvents = 96;
template <typename T>
struct EventTable {
  EventDesc<T> ev[kTableEvents];
  int ev0;         // batch index of ev[0]
  long long t0;    // the group's tiles (K1) or chunks (K2) are [t0, t1) of the batch's list
  long long t1;
};
static_assert(sizeof(EventTable<double>) <= 32764, "event table exceeds the kernel-parameter limit");

// R: rows of each link read and written (3 full, 2 for 12-real links).  kStride: the persistent grid
// strides through the tile list; without it each block takes one tile (the tile grid), and the
// kernel carries no loop state across the site body (FP32 link kernel: 100 B of spill stores
// instead of 360, none with 12-real links).
template <typename T, typename I, int R, bool kStride>
__global__ void __launch_bounds__(kThreads, Occupancy<T>::kMinBlocks)
    efield_batch_kernel(const __grid_constant__ EventTable<T> tab, const unsigned short* __restrict__ tile_ev) {
  __shared__ cx<T> sh[StapleShare<T>::kSlots * 9 * kThreads + 1];
  for (long long t = tab.t0 + blockIdx.x; t < tab.t1; t += gridDim.x) {
    const EventDesc<T>& d = tab.ev[tile_ev[t] - tab.ev0];
    int x, y, z;
    if (d.tm.site(t - d.k1_begin, threadIdx.x, d.g.nx, d.g.ny, x, y, z))
      efield_site<T, I, R>(d.g, d.f, d.ep, x, y, z, StapleShare<T>::kSlots ? sh : nullptr);
    if (!kStride) break;
  }
}

template <typename T, typename I, int R, bool kStride>
__global__ void __launch_bounds__(kThreads, Occupancy<T>::kLinksMinBlocks)
    links_batch_kernel(const __grid_constant__ EventTable<T> tab, const unsigned short* __restrict__ tile_ev) {
  for (long long t = tab.t0 + blockIdx.x; t < tab.t1; t += gridDim.x) {
    const EventDesc<T>& d = tab.ev[tile_ev[t] - tab.ev0];
    const long long idx = (t - d.k2_begin) * kThreads + threadIdx.x;
    if (idx < d.g.vol) links_site<T, I, R>(d.g, d.f, d.lp, (I)idx);
    if (!kStride) break;
  }
}

// The plaquette method over the batch: the single-lattice kernels' site functions on every event's
// owner chunks (force) and site chunks (gather + link update).
template <typename T, typename I, int R, bool kStride>
__global__ void __launch_bounds__(kThreads, PlaqOccupancy<T, T>::kMinBlocks)
    plaquette_batch_kernel(const __grid_constant__ EventTable<T> tab, const unsigned short* __restrict__ tile_ev) {
  for (long long t = tab.t0 + blockIdx.x; t < tab.t1; t += gridDim.x) {
    const EventDesc<T>& d = tab.ev[tile_ev[t] - tab.ev0];
    const long long idx = (t - d.k1_begin) * kThreads + threadIdx.x;
    if (idx < d.g.plane * (d.g.nz + 1)) plaquette_site<T, I, R, T>(d.g, d.f, d.C, d.ep, (I)idx);
    if (!kStride) break;
  }
}

template <typename T, typename I, int R, bool kStride>
__global__ void __launch_bounds__(kThreads, Occupancy<T>::kLinksMinBlocks)
    links_gather_batch_kernel(const __grid_constant__ EventTable<T> tab, const unsigned short* __restrict__ tile_ev) {
  for (long long t = tab.t0 + blockIdx.x; t < tab.t1; t += gridDim.x) {
    const EventDesc<T>& d = tab.ev[tile_ev[t] - tab.ev0];
    const long long idx = (t - d.k2_begin) * kThreads + threadIdx.x;
    if (idx < d.g.vol) links_site<T, I, R, true>(d.g, d.f, d.lp, (I)idx, d.C);
    if (!kStride) break;
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
  // launch groups of up to kTableEvents events: the K1 and K2 parameter tables and grid sizes
  std::vector<glasma::EventTable<float>> tab1_f, tab2_f;
  std::vector<glasma::EventTable<double>> tab1_d, tab2_d;
  std::vector<int> grid1, grid2;
  unsigned short* d_tile_ev = nullptr;  // event of every K1 tile, then of every K2 chunk
  long long tile_ev_cap = 0;
  double desc_dt = NAN;
  long long k1_total = 0, k2_total = 0;
  bool idx32 = true;
  bool strided = false;  // some group's grid is smaller than its tile list (strided kernels needed)
  int launch_mode = GLASMA_BATCH_TILE_GRID;
  int link_rows = 3;  // 2: 12-real links (FP32), as glasma_set_link_storage
  int method = GLASMA_STEP_PLAQUETTE;  // or GLASMA_STEP_TWO_PASS (glasma_batch_set_step_method)
  int method_used = GLASMA_STEP_PLAQUETTE;  // two-pass when the contribution buffers could not be allocated
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

template <typename T>
std::vector<glasma::EventTable<T>>& tables1(glasma_batch* b);
template <>
std::vector<glasma::EventTable<float>>& tables1<float>(glasma_batch* b) { return b->tab1_f; }
template <>
std::vector<glasma::EventTable<double>>& tables1<double>(glasma_batch* b) { return b->tab1_d; }
template <typename T>
std::vector<glasma::EventTable<T>>& tables2(glasma_batch* b);
template <>
std::vector<glasma::EventTable<float>>& tables2<float>(glasma_batch* b) { return b->tab2_f; }
template <>
std::vector<glasma::EventTable<double>>& tables2<double>(glasma_batch* b) { return b->tab2_d; }

template <typename T, int R>
void batch_occupancy(const glasma_batch* b, int& per1, int& per2) {
  using namespace glasma;
  if (b->method_used == GLASMA_STEP_PLAQUETTE) {
    if (b->idx32) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, plaquette_batch_kernel<T, int, R, true>, kThreads, 0);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, links_gather_batch_kernel<T, int, R, true>, kThreads, 0);
    } else {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, plaquette_batch_kernel<T, long long, R, true>, kThreads, 0);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, links_gather_batch_kernel<T, long long, R, true>, kThreads,
                                                    0);
    }
    return;
  }
  if (b->idx32) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, efield_batch_kernel<T, int, R, true>, kThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, links_batch_kernel<T, int, R, true>, kThreads, 0);
  } else {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, efield_batch_kernel<T, long long, R, true>, kThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, links_batch_kernel<T, long long, R, true>, kThreads, 0);
  }
}

// (Re)build the device event table for time step dt.
template <typename T>
int build_descriptors(glasma_batch* b, double dt) {
  using namespace glasma;
  std::vector<EventDesc<T>> d(b->ev.size());
  long long k1 = 0, k2 = 0;
  b->idx32 = true;
  // the plaquette method needs every event's contribution buffer; without them the batch steps with
  // the staple kernels (as a single lattice does)
  bool plaq = b->method == GLASMA_STEP_PLAQUETTE;
  for (size_t i = 0; plaq && i < b->ev.size(); i++) plaq = ensure_contrib(b->ev[i]);
  b->method_used = plaq ? GLASMA_STEP_PLAQUETTE : GLASMA_STEP_TWO_PASS;
  for (size_t i = 0; i < b->ev.size(); i++) {
    glasma_lattice* h = b->ev[i];
    EventDesc<T>& e = d[i];
    e.g = h->g;
    e.f = handle_ptrs<T>(h);
    e.C = plaq ? static_cast<T*>(h->contrib) : nullptr;
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
    k1 += plaq ? (h->g.plane * (h->g.nz + 1) + kThreads - 1) / kThreads : e.tm.tiles(h->g.nz);
    k2 += (h->g.vol + kThreads - 1) / kThreads;
    if (!use_32bit_index(h->g)) b->idx32 = false;
    // the contribution buffer has 48 S entries: 32-bit offsets only while that fits
    if (plaq && h->g.S * 48 >= (1LL << 31) - 1) b->idx32 = false;
  }
  b->k1_total = k1;
  b->k2_total = k2;
  b->swaps.clear();
  for (glasma_lattice* h : b->ev) b->swaps.push_back(h->swaps);
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
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bcuda(e, "event table upload");
  // persistent grids: as many blocks as fit on the device at once
  int dev = 0, sms = 0, per1 = 0, per2 = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if constexpr (sizeof(T) == 4) {
    if (b->link_rows == 2)
      batch_occupancy<T, 2>(b, per1, per2);
    else
      batch_occupancy<T, 3>(b, per1, per2);
  } else {
    batch_occupancy<T, 3>(b, per1, per2);
  }
  // launch groups of up to kTableEvents consecutive events, each with its own parameter tables
  std::vector<EventTable<T>>& tab1 = tables1<T>(b);
  std::vector<EventTable<T>>& tab2 = tables2<T>(b);
  tab1.clear();
  tab2.clear();
  b->grid1.clear();
  b->grid2.clear();
  const bool tile_grid = b->launch_mode == GLASMA_BATCH_TILE_GRID;
  b->strided = false;
  for (size_t e0 = 0; e0 < d.size(); e0 += kTableEvents) {
    const size_t e1 = std::min(d.size(), e0 + (size_t)kTableEvents);
    EventTable<T> t{};
    for (size_t i = e0; i < e1; i++) t.ev[i - e0] = d[i];
    t.ev0 = (int)e0;
    t.t0 = d[e0].k1_begin;
    t.t1 = e1 < d.size() ? d[e1].k1_begin : k1;
    tab1.push_back(t);
    const long long n1 = t.t1 - t.t0;
    t.t0 = d[e0].k2_begin;
    t.t1 = e1 < d.size() ? d[e1].k2_begin : k2;
    tab2.push_back(t);
    const long long n2 = t.t1 - t.t0;
    if (tile_grid && n1 < (1LL << 31) && n2 < (1LL << 31)) {
      b->grid1.push_back((int)n1);
      b->grid2.push_back((int)n2);
    } else {
      b->grid1.push_back((int)std::min<long long>(n1, (long long)sms * std::max(per1, 1)));
      b->grid2.push_back((int)std::min<long long>(n2, (long long)sms * std::max(per2, 1)));
      if (tile_grid) b->strided = true;
    }
  }
  b->desc_dt = dt;
  return GLASMA_OK;
}

template <typename T, typename I, int R, bool kStride>
void launch_batch_group(glasma_batch* b, size_t grp) {
  using namespace glasma;
  if (b->method_used == GLASMA_STEP_PLAQUETTE) {
    plaquette_batch_kernel<T, I, R, kStride><<<b->grid1[grp], kThreads, 0, b->stream>>>(tables1<T>(b)[grp],
                                                                                        b->d_tile_ev);
    links_gather_batch_kernel<T, I, R, kStride><<<b->grid2[grp], kThreads, 0, b->stream>>>(
        tables2<T>(b)[grp], b->d_tile_ev + b->k1_total);
    return;
  }
  efield_batch_kernel<T, I, R, kStride><<<b->grid1[grp], kThreads, 0, b->stream>>>(tables1<T>(b)[grp], b->d_tile_ev);
  links_batch_kernel<T, I, R, kStride><<<b->grid2[grp], kThreads, 0, b->stream>>>(tables2<T>(b)[grp],
                                                                                  b->d_tile_ev + b->k1_total);
}

template <typename T, int R>
void launch_batch_rows(glasma_batch* b) {
  // the tile grid gives every tile its own block, unless a list outgrew a grid dimension
  const bool stride = b->launch_mode != GLASMA_BATCH_TILE_GRID || b->strided;
  for (size_t grp = 0; grp < b->grid1.size(); grp++) {
    if (b->idx32)
      stride ? launch_batch_group<T, int, R, true>(b, grp) : launch_batch_group<T, int, R, false>(b, grp);
    else
      stride ? launch_batch_group<T, long long, R, true>(b, grp) : launch_batch_group<T, long long, R, false>(b, grp);
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
      int st = glasma_autotune_staple(h, dt, &tx);
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

int glasma_batch_set_step_method(glasma_batch* b, int method) {
  if (!b) return bfail(GLASMA_ERR_INVALID_ARGUMENT, "null batch");
  if (method != GLASMA_STEP_TWO_PASS && method != GLASMA_STEP_PLAQUETTE)
    return bfail(GLASMA_ERR_UNSUPPORTED, "batches step with the two-pass or the plaquette method");
  if (method != b->method) {
    b->method = method;
    b->desc_dt = NAN;  // the force kernel's list and the persistent grids depend on the method
    if (b->graph) {
      cudaStreamSynchronize(b->stream);
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
  }
  return GLASMA_OK;
}

int glasma_batch_get_step_method(glasma_batch* b, int* method) {
  if (!b || !method) return bfail(GLASMA_ERR_INVALID_ARGUMENT, "bad arguments");
  *method = std::isnan(b->desc_dt) ? b->method : b->method_used;
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

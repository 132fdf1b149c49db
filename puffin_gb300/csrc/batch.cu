// Batched runs: many independent instances -- each a pf_handle with its own
// macroparticles, field mesh, undulator and step size -- advanced together.
//
// Every instance follows the schedule of pf_run (UndSection's loop,
// puffin/lib/undulator.f90:33-358) exactly: the same step blocks between
// diffraction calls, the same periodic z2 wraps on its cumulative step count,
// the same window retries.  What changes is how the work reaches the GPU:
// one launch per RK4 stage covers the macroparticles of every instance, one
// per stage covers their window nodes, and one wrap launch per step covers
// all instances due for a wrap.  Each launch walks a list of tiles
// (instance, range) with a grid sized by the autotuner (one block per tile,
// or a persistent grid of the blocks resident at once).  A block of steps is
// captured once as a CUDA graph and replayed; the per-(instance, step, stage)
// coefficients come from a device table indexed by the batch's step counter.
// Small instances, which alone fill a fraction of the SMs and are bound by
// launch latency, share the device with the large ones.
//
// After a block, one status word per instance is read.  An instance whose
// block failed (a macroparticle left its window) is restored from the state
// saved before the block and replays it step by step with the reference's
// retries (pf_run's path); the others go on.
//
// The autotuner (pf_batch_tune) picks, by timing on the instances' own
// state (restored afterwards): per instance, the deposit mode -- direct
// atomics, or the shared-memory tile with its range length -- and for the
// batch, the macroparticles per direct tile, the FP64 stage block size, the
// node tile length and whether the launches use a persistent grid.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "pf_internal.h"

namespace {

struct Shape {
  int stage_threads = 256;     // FP64 stage block size (the mixed stage uses 512)
  int64_t stage_tile = 1024;   // macroparticles per direct tile
  int64_t node_tile = 4096;    // window nodes per node tile
  int stage_grid = 0;          // 0: one block per tile; -1: persistent grid
  int node_grid = 0;
};

constexpr int64_t WRAP_TILE = 16384;

// per-instance deposit mode chosen by the tuner: 0 direct atomics, else the
// macroparticles per shared-tile range; cached by instance shape
typedef std::tuple<int, int, int, int64_t, int64_t> ModeKey;  // precision, nix, niy, npl, np
std::map<ModeKey, int64_t> g_mode_cache;
std::mutex g_mode_mutex;  // batches may be tuned from several host threads

bool cached_mode(const ModeKey &key, int64_t *mode) {
  std::lock_guard<std::mutex> lock(g_mode_mutex);
  auto it = g_mode_cache.find(key);
  if (it == g_mode_cache.end()) return false;
  *mode = it->second;
  return true;
}

void cache_mode(const ModeKey &key, int64_t mode) {
  std::lock_guard<std::mutex> lock(g_mode_mutex);
  g_mode_cache[key] = mode;
}

}  // namespace

struct pf_batch {
  std::vector<pf_handle *> inst;
  int n = 0;
  int dev = 0;
  bool mixed = false;
  cudaStream_t stream = nullptr;
  std::string err;
  int64_t launches = 0;

  Shape shape;
  std::vector<int64_t> mode;   // per instance: 0 direct, else shared-tile range length
  std::vector<char> active;
  bool tuned = false;
  bool use_graphs = true;

  // sizes of the argument records
  size_t sa = 0, na = 0, ce = 0;  // stage args, node args, coefficient entry (4 stages)

  unsigned *d_status = nullptr, *h_status = nullptr;
  int *step_ctr = nullptr;
  char *d_args = nullptr;
  size_t args_cap = 0;
  char *h_args = nullptr;       // pinned staging
  std::vector<char> args_prev;  // what the device holds
  int args_len = -1;            // block length the coefficient pointers were laid out for

  BatchTile *d_tiles = nullptr;
  size_t tiles_cap = 0;
  std::vector<BatchTile> tiles;
  int off_direct = 0, n_direct = 0, off_dense = 0, n_dense = 0, off_nodes = 0, n_nodes = 0,
      off_wrap = 0, n_wrap = 0;
  size_t dense_smem = 0;
  bool tiles_dirty = true;
  std::vector<int64_t> tile_sig;  // per instance (np, nwin, nix*65536+niy) the tiles were cut for

  void *coef_dev = nullptr, *coef_host = nullptr;
  size_t coef_cap = 0;

  cudaGraphExec_t gexec = nullptr;
  int g_len = 0;
  int64_t g_nlaunch = 0;
  std::vector<int64_t> g_sig;

  cudaEvent_t ev0 = nullptr, ev1 = nullptr;

  // the per-instance work between blocks (diffraction, wrap) runs on a pool
  // of streams, forked from and joined back into the batch's stream: each
  // instance's small FFT launches fill a fraction of the SMs
  std::vector<cudaStream_t> pool;
  cudaEvent_t ev_fork = nullptr;
  std::vector<cudaEvent_t> ev_join;
};

namespace {

#define PB_CUDA(call)                                                    \
  do {                                                                   \
    cudaError_t e_ = (call);                                             \
    if (e_ != cudaSuccess) {                                             \
      b->err = std::string(#call) + ": " + cudaGetErrorString(e_);       \
      return PF_CUDA_ERR;                                                \
    }                                                                    \
  } while (0)

// The instances launch on the batch's stream while the batch drives them.
struct StreamSwap {
  pf_batch *b;
  std::vector<cudaStream_t> saved;
  explicit StreamSwap(pf_batch *bb) : b(bb) {
    for (pf_handle *h : b->inst) {
      saved.push_back(h->stream);
      h->stream = b->stream;
    }
  }
  ~StreamSwap() {
    cudaStreamSynchronize(b->stream);  // nothing of the batch stays queued
    for (int i = 0; i < b->n; ++i) b->inst[i]->stream = saved[i];
  }
};

int64_t max_dense_tile(const pf_batch *b) { return b->mixed ? (int64_t)PF_MX_THREADS * PF_MX_PPT : PF_FT_PPB; }

size_t inst_tile_smem(const pf_batch *b, const pf_handle *h) {
  return b->mixed ? pf_mixed_tile_smem(h) : pf_stage_tile_smem(h);
}

std::vector<int64_t> inst_sig(const pf_handle *h) {
  return {h->np, h->nwin, (int64_t)h->nix * 65536 + h->niy};
}

// Cut the tile lists: round-robin over the instances (chunk 0 of every
// instance, then chunk 1, ...), which spreads the atomics of one launch over
// many instances' accumulators.
int build_tiles(pf_batch *b) {
  b->tiles.clear();
  b->tile_sig.clear();
  b->dense_smem = 0;
  auto cut = [&](std::vector<BatchTile> &out, auto len_of, auto take) {
    std::vector<int64_t> pos(b->n, 0);
    bool more = true;
    while (more) {
      more = false;
      for (int i = 0; i < b->n; ++i) {
        if (!b->active[i] || !take(i)) continue;
        const int64_t total = len_of(i);
        if (pos[i] >= total) continue;
        const int64_t chunk = take(i);
        const int64_t e = std::min(total, pos[i] + chunk);
        out.push_back(BatchTile{i, 0, pos[i], e});
        pos[i] = e;
        more = more || e < total;
      }
    }
  };
  // a window that grew past the shared-memory tile sends its instance back
  // to direct atomics
  for (int i = 0; i < b->n; ++i)
    if (b->mode[i] > 0 && inst_tile_smem(b, b->inst[i]) == 0) b->mode[i] = 0;
  std::vector<BatchTile> direct, dense, nodes, wrap;
  // direct: instances in mode 0, shape.stage_tile macroparticles per tile
  // (a multiple of the mixed block for the mixed stage)
  int64_t dt = b->shape.stage_tile;
  if (b->mixed) dt = std::max<int64_t>(PF_MX_THREADS, std::min<int64_t>(dt, max_dense_tile(b)) / PF_MX_THREADS * PF_MX_THREADS);
  cut(direct, [&](int i) { return b->inst[i]->np; },
      [&](int i) -> int64_t { return b->mode[i] == 0 ? dt : 0; });
  cut(dense, [&](int i) { return b->inst[i]->np; },
      [&](int i) -> int64_t { return b->mode[i] > 0 ? b->mode[i] : 0; });
  cut(nodes, [&](int i) { return b->inst[i]->nwin; },
      [&](int i) -> int64_t { return b->shape.node_tile; });
  cut(wrap, [&](int i) { return b->inst[i]->np; },
      [&](int i) -> int64_t { return b->inst[i]->p.mesh_type == PF_MESH_PERIODIC ? WRAP_TILE : 0; });
  for (int i = 0; i < b->n; ++i) {
    if (b->active[i] && b->mode[i] > 0)
      b->dense_smem = std::max(b->dense_smem, inst_tile_smem(b, b->inst[i]));
    const std::vector<int64_t> s = inst_sig(b->inst[i]);
    b->tile_sig.insert(b->tile_sig.end(), s.begin(), s.end());
  }
  b->off_direct = 0;
  b->n_direct = (int)direct.size();
  b->off_dense = b->n_direct;
  b->n_dense = (int)dense.size();
  b->off_nodes = b->off_dense + b->n_dense;
  b->n_nodes = (int)nodes.size();
  b->off_wrap = b->off_nodes + b->n_nodes;
  b->n_wrap = (int)wrap.size();
  for (auto *v : {&direct, &dense, &nodes, &wrap}) b->tiles.insert(b->tiles.end(), v->begin(), v->end());
  const size_t bytes = std::max<size_t>(1, b->tiles.size()) * sizeof(BatchTile);
  if (b->tiles_cap < bytes) {
    cudaFree(b->d_tiles);
    b->d_tiles = nullptr;
    b->tiles_cap = 0;
    PB_CUDA(cudaMalloc(&b->d_tiles, bytes));
    b->tiles_cap = bytes;
  }
  if (!b->tiles.empty())
    PB_CUDA(cudaMemcpyAsync(b->d_tiles, b->tiles.data(), b->tiles.size() * sizeof(BatchTile),
                            cudaMemcpyHostToDevice, b->stream));
  b->tiles_dirty = false;
  return PF_OK;
}

bool tiles_stale(const pf_batch *b) {
  if (b->tiles_dirty) return true;
  for (int i = 0; i < b->n; ++i) {
    const std::vector<int64_t> s = inst_sig(b->inst[i]);
    for (int k = 0; k < 3; ++k)
      if (b->tile_sig[3 * i + k] != s[k]) return true;
  }
  return false;
}

// device argument layout: stage [parity 2][stage 4][n], nodes [stage 4][n], wrap [n]
size_t stage_off(const pf_batch *b, int parity, int s, int i) {
  return ((size_t)(parity * 4 + s - 1) * b->n + i) * b->sa;
}
size_t node_off(const pf_batch *b, int s, int i) {
  return (size_t)8 * b->n * b->sa + ((size_t)(s - 1) * b->n + i) * b->na;
}
size_t wrap_off(const pf_batch *b, int i) {
  return (size_t)8 * b->n * b->sa + (size_t)4 * b->n * b->na + (size_t)i * sizeof(WrapArgs);
}
size_t args_bytes(const pf_batch *b) { return wrap_off(b, b->n); }

// Stage, node and wrap arguments of every instance for a block of len steps
// (coefficient table of instance i at coef_dev + i len ce); uploaded only
// where they changed.
int upload_args(pf_batch *b, int len, const double *hstep) {
  const size_t bytes = args_bytes(b);
  if (b->args_cap < bytes) {
    cudaFree(b->d_args);
    if (b->h_args) cudaFreeHost(b->h_args);
    b->d_args = b->h_args = nullptr;
    b->args_cap = 0;
    PB_CUDA(cudaMalloc(&b->d_args, bytes));
    PB_CUDA(cudaMallocHost(&b->h_args, bytes));
    b->args_cap = bytes;
    b->args_prev.clear();
  }
  char *H = b->h_args;
  memset(H, 0, bytes);
  for (int i = 0; i < b->n; ++i) {
    pf_handle *h = b->inst[i];
    const void *tab = (const char *)b->coef_dev + (size_t)i * len * b->ce;
    const double hs = hstep[i], hh = hs * 0.5;
    const double stage_c[4] = {0.0, hh, hh, hs};
    for (int p = 0; p < 2; ++p) {
      const int cur = h->cur ^ p;
      for (int s = 1; s <= 4; ++s) {
        char *dst = H + stage_off(b, p, s, i);
        if (b->mixed) {
          pf_mixed_fill_stage(h, s, cur, hs, b->mode[i] > 0 ? 1 : 0, tab, b->step_ctr,
                              b->d_status + i, dst);
        } else {
          StageArgs a;
          pf_fill_stage_args(h, a, hs / 6.0);
          pf_stage_pointers(h, a, s, cur);
          a.cstate = stage_c[s - 1];
          a.coef_tab = (const StageCoef *)tab;
          a.step_ctr = b->step_ctr;
          a.status = b->d_status + i;
          memcpy(dst, &a, sizeof(a));
        }
      }
    }
    for (int s = 1; s <= 4; ++s) {
      char *dst = H + node_off(b, s, i);
      if (b->mixed) {
        pf_mixed_fill_nodes(h, s, hs, b->d_status + i, dst);
      } else {
        NodeArgs nd;
        pf_fill_node_args(h, nd, hs);
        nd.coef = (s == 3) ? hs : hh;
        nd.status = b->d_status + i;
        memcpy(dst, &nd, sizeof(nd));
      }
    }
    WrapArgs w;
    memset(&w, 0, sizeof(w));
    w.z2[0] = h->y[0][2];
    w.z2[1] = h->y[1][2];
    w.csteps0 = h->csteps;
    w.lenz2 = h->p.dz2 * (double)(h->p.nz2 - 1);
    w.redist = h->p.redist_every > 0 ? h->p.redist_every : 60;
    w.cur0 = h->cur;
    w.periodic = (h->p.mesh_type == PF_MESH_PERIODIC);
    memcpy(H + wrap_off(b, i), &w, sizeof(w));
  }
  // upload the changed part: the stage/node records, then the wrap records
  const size_t sn = wrap_off(b, 0);
  if (b->args_prev.size() != bytes || memcmp(b->args_prev.data(), H, sn) != 0) {
    PB_CUDA(cudaMemcpyAsync(b->d_args, H, bytes, cudaMemcpyHostToDevice, b->stream));
  } else if (memcmp(b->args_prev.data() + sn, H + sn, bytes - sn) != 0) {
    PB_CUDA(cudaMemcpyAsync(b->d_args + sn, H + sn, bytes - sn, cudaMemcpyHostToDevice, b->stream));
  }
  b->args_prev.assign(H, H + bytes);
  b->args_len = len;
  return PF_OK;
}

// Coefficient tables of a block of len steps from each instance's szl (the
// taper state advances as the steps do); szl[i] ends at the block's last step.
int upload_coefs(pf_batch *b, int len, const double *hstep, double *szl) {
  const size_t bytes = (size_t)b->n * len * b->ce;
  if (b->coef_cap < bytes) {
    cudaFree(b->coef_dev);
    if (b->coef_host) cudaFreeHost(b->coef_host);
    b->coef_dev = b->coef_host = nullptr;
    b->coef_cap = 0;
    PB_CUDA(cudaMalloc(&b->coef_dev, bytes));
    PB_CUDA(cudaMallocHost(&b->coef_host, bytes));
    b->coef_cap = bytes;
    b->args_prev.clear();  // the records point into the table
    if (b->gexec) {
      cudaGraphExecDestroy(b->gexec);
      b->gexec = nullptr;
    }
  }
  for (int i = 0; i < b->n; ++i) {
    if (!b->active[i]) continue;
    pf_handle *h = b->inst[i];
    double z = szl[i];
    for (int k = 0; k < len; ++k) {
      char *dst = (char *)b->coef_host + ((size_t)i * len + k) * b->ce;
      if (b->mixed) pf_step_coefficients_f(h, z, hstep[i], dst);
      else pf_step_coefficients(h, z, hstep[i], (StageCoef *)dst);
      if (k < len - 1) z = z + hstep[i];
    }
    szl[i] = z;
  }
  PB_CUDA(cudaMemcpyAsync(b->coef_dev, b->coef_host, bytes, cudaMemcpyHostToDevice, b->stream));
  return PF_OK;
}

// Kernels of one step (k = 1..len) of a block.
int enqueue_step(pf_batch *b, int k, int len) {
  const int p = (k - 1) & 1;
  cudaError_t e = cudaSuccess;
  const BatchTile *T = b->d_tiles;
  for (int s = 1; s <= 4 && e == cudaSuccess; ++s) {
    const void *sargs = b->d_args + stage_off(b, p, s, 0);
    const void *nargs = b->d_args + node_off(b, s, 0);
    if (b->mixed) {
      if (b->n_direct) {
        e = pf_mixed_stage_batch(b->stream, s, sargs, T + b->off_direct, b->n_direct,
                                 b->shape.stage_grid, 0);
        b->launches++;
      }
      if (e == cudaSuccess && b->n_dense) {
        e = pf_mixed_stage_batch(b->stream, s, sargs, T + b->off_dense, b->n_dense,
                                 b->shape.stage_grid, b->dense_smem);
        b->launches++;
      }
      if (e == cudaSuccess && b->n_nodes) {
        e = pf_mixed_nodes_batch(b->stream, s, nargs, T + b->off_nodes, b->n_nodes,
                                 b->shape.node_grid, 256, s == 4 ? b->step_ctr : nullptr);
        b->launches++;
      }
    } else {
      if (b->n_direct) {
        e = pf_stage_batch(b->stream, s, false, (const StageArgs *)sargs, T + b->off_direct,
                           b->n_direct, b->shape.stage_grid, b->shape.stage_threads, 0);
        b->launches++;
      }
      if (e == cudaSuccess && b->n_dense) {
        e = pf_stage_batch(b->stream, s, true, (const StageArgs *)sargs, T + b->off_dense,
                           b->n_dense, b->shape.stage_grid, 256, b->dense_smem);
        b->launches++;
      }
      if (e == cudaSuccess && b->n_nodes) {
        e = pf_nodes_batch(b->stream, s, (const NodeArgs *)nargs, T + b->off_nodes, b->n_nodes,
                           b->shape.node_grid, 256, s == 4 ? b->step_ctr : nullptr);
        b->launches++;
      }
    }
  }
  if (e == cudaSuccess && k < len && b->n_wrap) {
    e = pf_wrap_batch(b->stream, (const WrapArgs *)(b->d_args + wrap_off(b, 0)), T + b->off_wrap,
                      b->n_wrap, -1, b->step_ctr);
    b->launches++;
  }
  if (e != cudaSuccess) {
    b->err = std::string("batched launch: ") + cudaGetErrorString(e);
    return PF_CUDA_ERR;
  }
  return PF_OK;
}

std::vector<int64_t> graph_sig(const pf_batch *b, int len) {
  return {len,
          b->n_direct,
          b->n_dense,
          b->n_nodes,
          b->n_wrap,
          (int64_t)b->dense_smem,
          b->shape.stage_threads,
          b->shape.stage_grid,
          b->shape.node_grid,
          (int64_t)(intptr_t)b->d_args,
          (int64_t)(intptr_t)b->d_tiles};
}

// Queue the len steps of a block: a captured graph when enabled (captured
// on first use and whenever the tiles, shapes or buffers change), else the
// launches themselves.
int enqueue_block(pf_batch *b, int len) {
  if (!b->use_graphs) {
    for (int k = 1; k <= len; ++k) {
      const int rc = enqueue_step(b, k, len);
      if (rc) return rc;
    }
    return PF_OK;
  }
  const std::vector<int64_t> sig = graph_sig(b, len);
  if (!b->gexec || b->g_sig != sig) {
    if (b->gexec) {
      cudaGraphExecDestroy(b->gexec);
      b->gexec = nullptr;
    }
    const int64_t l0 = b->launches;
    cudaGraph_t g = nullptr;
    PB_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    int rc = PF_OK;
    for (int k = 1; k <= len && rc == PF_OK; ++k) rc = enqueue_step(b, k, len);
    const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    b->g_nlaunch = b->launches - l0;
    b->launches = l0;
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ce != cudaSuccess) {
      b->err = std::string("batch capture: ") + cudaGetErrorString(ce);
      if (g) cudaGraphDestroy(g);
      return PF_CUDA_ERR;
    }
    const cudaError_t ie = cudaGraphInstantiate(&b->gexec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      b->gexec = nullptr;
      b->err = std::string("batch graph: ") + cudaGetErrorString(ie);
      return PF_CUDA_ERR;
    }
    b->g_sig = sig;
    b->g_len = len;
  }
  PB_CUDA(cudaGraphLaunch(b->gexec, b->stream));
  b->launches += b->g_nlaunch;
  return PF_OK;
}

constexpr int POOL = 8;

// Fork the pool from the batch stream; instance i then queues on pool[i % POOL].
int fork_pool(pf_batch *b) {
  PB_CUDA(cudaEventRecord(b->ev_fork, b->stream));
  for (cudaStream_t s : b->pool) PB_CUDA(cudaStreamWaitEvent(s, b->ev_fork, 0));
  return PF_OK;
}

int join_pool(pf_batch *b) {
  for (size_t k = 0; k < b->pool.size(); ++k) {
    PB_CUDA(cudaEventRecord(b->ev_join[k], b->pool[k]));
    PB_CUDA(cudaStreamWaitEvent(b->stream, b->ev_join[k], 0));
  }
  return PF_OK;
}

int check_instances(pf_batch *b) {
  for (int i = 0; i < b->n; ++i) {
    pf_handle *h = b->inst[i];
    if (!h->particles_set || h->nwin == 0) {
      b->err = "instance " + std::to_string(i) + ": particles not set";
      return PF_STATE;
    }
  }
  return PF_OK;
}

// Per-instance state a block (or a tuning trial) changes on the host.
struct HostState {
  double n2col, n2col0, undgrad;
  int64_t csteps;
  int cur;
};
HostState save_host(const pf_handle *h) { return {h->n2col, h->n2col0, h->undgrad, h->csteps, h->cur}; }
void restore_host(pf_handle *h, const HostState &s) {
  h->n2col = s.n2col;
  h->n2col0 = s.n2col0;
  h->undgrad = s.undgrad;
  h->csteps = s.csteps;
  h->cur = s.cur;
}

// Device time (ms) of one step of the batch's stage and node launches with
// the current tiles and shapes, from state already set up for a one-step
// block (median of repeats).
int time_step(pf_batch *b, int repeats, double *ms) {
  std::vector<float> t;
  for (int r = 0; r < repeats; ++r) {
    PB_CUDA(cudaMemsetAsync(b->step_ctr, 0, sizeof(int), b->stream));
    PB_CUDA(cudaEventRecord(b->ev0, b->stream));
    const int rc = enqueue_step(b, 1, 1);
    if (rc) return rc;
    PB_CUDA(cudaEventRecord(b->ev1, b->stream));
    PB_CUDA(cudaEventSynchronize(b->ev1));
    float v = 0.f;
    PB_CUDA(cudaEventElapsedTime(&v, b->ev0, b->ev1));
    t.push_back(v);
  }
  std::sort(t.begin(), t.end());
  *ms = t[t.size() / 2];
  return PF_OK;
}

}  // namespace

extern "C" {

int pf_batch_create(pf_handle *const *handles, int32_t n, pf_batch **out) {
  if (!handles || n < 1 || !out) return PF_BAD_ARG;
  *out = nullptr;
  const bool mixed = handles[0] && handles[0]->p.precision == PF_MIXED;
  for (int i = 0; i < n; ++i) {
    const pf_handle *h = handles[i];
    if (!h || h->dev != handles[0]->dev || (h->p.precision == PF_MIXED) != mixed || h->p.one_d)
      return PF_BAD_ARG;  // one device, one precision, 3D instances
    for (int j = 0; j < i; ++j)
      if (handles[j] == h) return PF_BAD_ARG;
  }
  pf_batch *b = new pf_batch();
  b->inst.assign(handles, handles + n);
  b->n = n;
  b->dev = handles[0]->dev;
  b->mixed = mixed;
  b->mode.assign(n, 0);
  b->active.assign(n, 1);
  b->sa = mixed ? pf_mixed_stage_args_bytes() : sizeof(StageArgs);
  b->na = mixed ? pf_mixed_node_args_bytes() : sizeof(NodeArgs);
  b->ce = mixed ? pf_step_coefficients_f_bytes() : 4 * sizeof(StageCoef);
  cudaSetDevice(b->dev);
  bool ok = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaMalloc(&b->d_status, sizeof(unsigned) * n) == cudaSuccess &&
            cudaMallocHost(&b->h_status, sizeof(unsigned) * n) == cudaSuccess &&
            cudaMalloc(&b->step_ctr, sizeof(int)) == cudaSuccess &&
            cudaEventCreate(&b->ev0) == cudaSuccess && cudaEventCreate(&b->ev1) == cudaSuccess;
  b->pool.assign(POOL, nullptr);
  b->ev_join.assign(POOL, nullptr);
  ok = ok && cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; k < POOL && ok; ++k)
    ok = cudaStreamCreateWithFlags(&b->pool[k], cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&b->ev_join[k], cudaEventDisableTiming) == cudaSuccess;
  // kernel attributes are set before any capture
  ok = ok && (mixed ? pf_mixed_stage_batch(b->stream, 1, nullptr, nullptr, 0, 0, 0)
                    : pf_stage_batch(b->stream, 1, false, nullptr, nullptr, 0, 0, 256, 0)) ==
                 cudaSuccess;
  if (!ok) {
    pf_batch_destroy(b);
    return PF_CUDA_ERR;
  }
  // default deposit modes: the dense rule of the single-instance path; the
  // batch keeps its instances' macroparticle order (no z2 ordering)
  for (int i = 0; i < n; ++i) {
    handles[i]->sort_z2 = false;
    const pf_handle *h = handles[i];
    const int64_t ntr = (int64_t)h->nix * h->niy;
    const bool dense = mixed ? pf_mixed_tile_smem(h) > 0
                             : (pf_stage_tile_smem(h) > 0 && h->np >= 8 * h->npl * ntr);
    b->mode[i] = dense ? max_dense_tile(b) : 0;
  }
  *out = b;
  return PF_OK;
}

int pf_batch_destroy(pf_batch *b) {
  if (!b) return PF_BAD_ARG;
  cudaSetDevice(b->dev);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  cudaFree(b->d_status);
  if (b->h_status) cudaFreeHost(b->h_status);
  cudaFree(b->step_ctr);
  cudaFree(b->d_args);
  if (b->h_args) cudaFreeHost(b->h_args);
  cudaFree(b->d_tiles);
  cudaFree(b->coef_dev);
  if (b->coef_host) cudaFreeHost(b->coef_host);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  for (cudaEvent_t e : b->ev_join)
    if (e) cudaEventDestroy(e);
  for (cudaStream_t s : b->pool)
    if (s) cudaStreamDestroy(s);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return PF_OK;
}

int pf_batch_run(pf_batch *b, int32_t nsteps, int32_t isteps4diff, int32_t qdiffraction,
                 const double *hstep, double *szl, int32_t *status) {
  if (!b || !hstep || !szl || nsteps < 0 || (qdiffraction && isteps4diff < 1)) return PF_BAD_ARG;
  cudaSetDevice(b->dev);
  int rc = check_instances(b);
  if (rc) return rc;
  StreamSwap swap(b);
  std::vector<RunSched> sc(b->n);
  std::vector<int32_t> rcs(b->n, PF_OK);
  std::fill(b->active.begin(), b->active.end(), 1);
  b->tiles_dirty = true;
  rc = fork_pool(b);
  if (rc) return rc;
  for (int i = 0; i < b->n; ++i) {
    pf_handle *h = b->inst[i];
    pf_sched_init(h, sc[i], nsteps, isteps4diff, qdiffraction, hstep[i], szl + i, nullptr);
    sc[i].sync = false;
    if (qdiffraction) {
      h->stream = b->pool[i % POOL];
      rc = pf_diffract_enqueue(h, sc[i].dzds);
      h->stream = b->stream;
      if (rc) {
        b->err = "instance " + std::to_string(i) + ": " + h->err;
        return rc;
      }
    }
  }
  rc = join_pool(b);
  if (rc) return rc;
  std::vector<HostState> hs(b->n);
  std::vector<double> szl0(b->n);
  int istep = 1;
  while (istep <= nsteps && std::count(b->active.begin(), b->active.end(), 1) > 0) {
    const int last = qdiffraction
                         ? std::min<int>(nsteps, ((istep - 1) / isteps4diff + 1) * isteps4diff)
                         : std::min<int>(nsteps, istep + 15);
    const int len = last - istep + 1;
    for (int i = 0; i < b->n; ++i) {
      if (!b->active[i]) continue;
      hs[i] = save_host(b->inst[i]);
      szl0[i] = szl[i];
      rc = pf_block_snapshot(b->inst[i], true);
      if (rc) return rc;
    }
    if (tiles_stale(b)) {
      rc = build_tiles(b);
      if (rc) return rc;
    }
    PB_CUDA(cudaMemsetAsync(b->d_status, 0, sizeof(unsigned) * b->n, b->stream));
    rc = upload_coefs(b, len, hstep, szl);
    if (rc) return rc;
    rc = upload_args(b, len, hstep);
    if (rc) return rc;
    PB_CUDA(cudaMemsetAsync(b->step_ctr, 0, sizeof(int), b->stream));
    rc = enqueue_block(b, len);
    if (rc) return rc;
    for (int i = 0; i < b->n; ++i) {
      if (!b->active[i]) continue;
      pf_handle *h = b->inst[i];
      h->cur ^= (len & 1);
      h->csteps += len - 1;
    }
    PB_CUDA(cudaMemcpyAsync(b->h_status, b->d_status, sizeof(unsigned) * b->n,
                            cudaMemcpyDeviceToHost, b->stream));
    PB_CUDA(cudaStreamSynchronize(b->stream));
    // the blocks that succeeded: their last step's position, diffraction and
    // wrap, instance by instance on the pool
    rc = fork_pool(b);
    if (rc) return rc;
    for (int i = 0; i < b->n; ++i) {
      if (!b->active[i] || b->h_status[i] != 0u) continue;
      pf_handle *h = b->inst[i];
      h->stream = b->pool[i % POOL];
      rc = pf_sched_after_step(h, sc[i], last);
      h->stream = b->stream;
      if (rc) {
        rcs[i] = rc;
        b->active[i] = 0;
        b->tiles_dirty = true;
        if (b->err.empty()) b->err = "instance " + std::to_string(i) + ": " + h->err;
      }
    }
    rc = join_pool(b);
    if (rc) return rc;
    for (int i = 0; i < b->n; ++i) {
      if (!b->active[i] || b->h_status[i] == 0u) continue;
      pf_handle *h = b->inst[i];
      // replay the block step by step from the saved state
      restore_host(h, hs[i]);
      szl[i] = szl0[i];
      rc = pf_block_snapshot(h, false);
      for (int k = istep; k <= last && rc == PF_OK; ++k) rc = pf_sched_eager_step(h, sc[i], k);
      if (rc) {
        rcs[i] = rc;
        b->active[i] = 0;
        b->tiles_dirty = true;
        if (b->err.empty()) b->err = "instance " + std::to_string(i) + ": " + h->err;
      }
    }
    istep = last + 1;
  }
  PB_CUDA(cudaStreamSynchronize(b->stream));
  int first = PF_OK;
  for (int i = 0; i < b->n; ++i) {
    if (status) status[i] = rcs[i];
    if (first == PF_OK) first = rcs[i];
  }
  return first;
}

int pf_batch_tune(pf_batch *b, const double *hstep, const double *szl, int32_t repeats) {
  if (!b || !hstep || !szl) return PF_BAD_ARG;
  if (repeats < 1) repeats = 3;
  cudaSetDevice(b->dev);
  int rc = check_instances(b);
  if (rc) return rc;
  StreamSwap swap(b);
  std::fill(b->active.begin(), b->active.end(), 1);
  std::vector<HostState> hs(b->n);
  for (int i = 0; i < b->n; ++i) {
    hs[i] = save_host(b->inst[i]);
    rc = pf_block_snapshot(b->inst[i], true);
    if (rc) return rc;
  }
  std::vector<double> z(szl, szl + b->n);
  rc = upload_coefs(b, 1, hstep, z.data());
  if (rc) return rc;
  for (int i = 0; i < b->n; ++i) restore_host(b->inst[i], hs[i]);
  rc = upload_args(b, 1, hstep);
  if (rc) return rc;
  PB_CUDA(cudaMemsetAsync(b->d_status, 0, sizeof(unsigned) * b->n, b->stream));

  const Shape shape0 = b->shape;
  const std::vector<int64_t> mode0 = b->mode;
  int out = PF_OK;
  double ms = 0.0;
  // 1. per instance: deposit mode, timed on the instance alone
  {
    std::vector<char> act0 = b->active;
    const std::vector<int64_t> cand =
        b->mixed ? std::vector<int64_t>{0, 1024, 2048, 3072, 4096}
                 : std::vector<int64_t>{0, 2048, 4096, 8192};
    for (int i = 0; i < b->n && out == PF_OK; ++i) {
      const pf_handle *h = b->inst[i];
      const ModeKey key{b->mixed ? 1 : 0, h->nix, h->niy, (int)h->npl, h->np};
      if (cached_mode(key, &b->mode[i])) continue;
      std::vector<int64_t> mine;
      for (int64_t m : cand)
        if (m == 0 || inst_tile_smem(b, h) > 0) mine.push_back(m);
      if (mine.size() == 1) {  // nothing to choose
        b->mode[i] = mine[0];
        continue;
      }
      std::fill(b->active.begin(), b->active.end(), 0);
      b->active[i] = 1;
      double best = 1e30;
      int64_t best_mode = b->mode[i];
      for (int64_t m : mine) {
        b->mode[i] = m;
        // the mixed stage keeps its tile flag in the arguments
        if (b->mixed && (out = upload_args(b, 1, hstep)) != PF_OK) break;
        if ((out = build_tiles(b)) != PF_OK) break;
        if ((out = time_step(b, repeats, &ms)) != PF_OK) break;
        if (ms < best) {
          best = ms;
          best_mode = m;
        }
      }
      b->mode[i] = best_mode;
      if (out == PF_OK) cache_mode(key, best_mode);
    }
    b->active = act0;
  }
  // 2. batch shapes, coordinate by coordinate on the whole batch
  auto trial = [&](Shape s, double *t) -> int {
    b->shape = s;
    int r = b->mixed ? upload_args(b, 1, hstep) : PF_OK;
    if (r == PF_OK) r = build_tiles(b);
    if (r == PF_OK) r = time_step(b, repeats, t);
    return r;
  };
  if (out == PF_OK) {
    double best = 1e30;
    Shape bs = b->shape;
    if ((out = trial(bs, &best)) == PF_OK) {
      std::vector<Shape> cands;
      const std::vector<int64_t> tiles_c = b->mixed ? std::vector<int64_t>{512, 1024, 2048}
                                                    : std::vector<int64_t>{256, 512, 1024, 2048, 4096};
      for (int64_t t : tiles_c) {
        Shape s = bs;
        s.stage_tile = t;
        double v;
        if ((out = trial(s, &v)) != PF_OK) break;
        if (v < best) best = v, bs = s;
      }
      if (out == PF_OK && !b->mixed) {
        for (int th : {128, 256}) {
          Shape s = bs;
          s.stage_threads = th;
          double v;
          if ((out = trial(s, &v)) != PF_OK) break;
          if (v < best) best = v, bs = s;
        }
      }
      for (int g : {0, -1}) {
        if (out != PF_OK) break;
        Shape s = bs;
        s.stage_grid = g;
        double v;
        if ((out = trial(s, &v)) != PF_OK) break;
        if (v < best) best = v, bs = s;
      }
      for (int64_t nt : {1024, 4096, 16384}) {
        if (out != PF_OK) break;
        for (int g : {0, -1}) {
          Shape s = bs;
          s.node_tile = nt;
          s.node_grid = g;
          double v;
          if ((out = trial(s, &v)) != PF_OK) break;
          if (v < best) best = v, bs = s;
        }
      }
      b->shape = bs;
    }
  }
  if (out != PF_OK) {
    b->shape = shape0;
    b->mode = mode0;
  }
  // restore the instances' state
  PB_CUDA(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < b->n; ++i) {
    restore_host(b->inst[i], hs[i]);
    rc = pf_block_snapshot(b->inst[i], false);
    if (rc) return rc;
  }
  PB_CUDA(cudaMemsetAsync(b->d_status, 0, sizeof(unsigned) * b->n, b->stream));
  PB_CUDA(cudaStreamSynchronize(b->stream));
  b->tiles_dirty = true;
  b->args_prev.clear();
  b->tuned = (out == PF_OK);
  return out;
}

int pf_batch_get_shape(const pf_batch *b, int64_t *shape5, int64_t *modes) {
  if (!b) return PF_BAD_ARG;
  if (shape5) {
    shape5[0] = b->shape.stage_threads;
    shape5[1] = b->shape.stage_tile;
    shape5[2] = b->shape.node_tile;
    shape5[3] = b->shape.stage_grid;
    shape5[4] = b->shape.node_grid;
  }
  if (modes)
    for (int i = 0; i < b->n; ++i) modes[i] = b->mode[i];
  return PF_OK;
}

int pf_batch_set_shape(pf_batch *b, const int64_t *shape5, const int64_t *modes) {
  if (!b) return PF_BAD_ARG;
  if (shape5) {
    if ((shape5[0] != 128 && shape5[0] != 256) || shape5[1] < 1 || shape5[2] < 1 ||
        shape5[3] < -1 || shape5[4] < -1)
      return PF_BAD_ARG;
    b->shape.stage_threads = (int)shape5[0];
    b->shape.stage_tile = shape5[1];
    b->shape.node_tile = shape5[2];
    b->shape.stage_grid = (int)shape5[3];
    b->shape.node_grid = (int)shape5[4];
  }
  if (modes) {
    for (int i = 0; i < b->n; ++i)
      if (modes[i] < 0 || modes[i] > max_dense_tile(b) ||
          (modes[i] > 0 && inst_tile_smem(b, b->inst[i]) == 0))
        return PF_BAD_ARG;
    for (int i = 0; i < b->n; ++i) b->mode[i] = modes[i];
  }
  b->tiles_dirty = true;
  b->args_prev.clear();
  return PF_OK;
}

int pf_batch_use_graphs(pf_batch *b, int32_t on) {
  if (!b) return PF_BAD_ARG;
  b->use_graphs = on != 0;
  return PF_OK;
}

int64_t pf_batch_launches(const pf_batch *b) { return b ? b->launches : -1; }

void *pf_batch_stream(const pf_batch *b) { return b ? (void *)b->stream : nullptr; }

const char *pf_batch_last_error(const pf_batch *b) { return b ? b->err.c_str() : "null batch"; }

}  // extern "C"

// Host runtime behind include/snow_mpm.h: contexts, scenes, uploads and
// downloads, the step sequence (captured in CUDA graphs), batches.
//
// The step follows ExplicitTimeUpdate::update
// (src/snow/simulation/timeUpdate/explicittimeupdate.cpp:36-63):
// rigid advance -> grid reset -> P2G -> grid update -> G2P -> particle advance.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <vector>

#include "snow_internal.h"

using namespace snow;

struct snow_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  size_t budget = 0;
  size_t used = 0;
  bool defer_sync = false;  // inside a run of allocations that waits for the stream once, at its end
  std::string err;
  bool profiling = false;
  bool graphs = true;  // replay each step as a captured CUDA graph
  // device memory of scenes and batches comes from this pool, which keeps
  // freed blocks for reuse (scenes of a serving loop come and go)
  cudaMemPool_t pool = nullptr;
  // statistics: slot 0 for snow_scene_stats, slots 1..SNOW_STATS_SLOTS for
  // the queued reads. The kernel's last block writes the totals into h_stats
  // (mapped pinned memory; d_hstats is its device address) and empties the
  // device slot, so a read is one launch and an event, no copies.
  StatsSlot* d_stats = nullptr;    // 1 + SNOW_STATS_SLOTS accumulators
  StatsAccum* h_stats = nullptr;   // mapped pinned, 1 + SNOW_STATS_SLOTS
  StatsAccum* d_hstats = nullptr;
  cudaEvent_t stat_ev[SNOW_STATS_SLOTS] = {};
  size_t stat_n[SNOW_STATS_SLOTS] = {};
  bool stat_pending[SNOW_STATS_SLOTS] = {};
  int* h_counters = nullptr;      // pinned, kCounterStride ints
  cudaEvent_t ev[8] = {};
  // side streams for independent per-scene work inside a batch step (the
  // re-binning of several scenes runs as parallel graph branches)
  static constexpr int kAux = 8;
  cudaStream_t aux[kAux] = {};
  cudaEvent_t fork_ev = nullptr;
  cudaEvent_t join_ev[kAux] = {};
  // the semi-implicit solve: its iteration counter and the stream its loop
  // body is captured from (all solves of a context run on `stream`, in order)
  int* d_iter = nullptr;
  cudaStream_t body_stream = nullptr;
  cudaStream_t gate_stream = nullptr;  // ... and the one the solve itself is captured from (inside its gate)
  // live children, destroyed with the context if the caller did not
  std::set<snow_scene*> scenes;
  std::set<snow_batch*> batches;
};

struct snow_scene {
  snow_ctx* ctx = nullptr;
  snow_params p{};
  int mode = SNOW_MODE_FAST;
  size_t cap = 0;
  size_t n = 0;
  bool uploaded = false;
  bool initialized = false;
  std::vector<snow_collider> coll_h;
  snow_collider* coll_d = nullptr;
  int ncoll = 0;
  std::vector<std::pair<void*, size_t>> allocs;
  size_t bytes = 0;
  long long G = 0;
  // reference mode
  RefArgs ra{};
  // fast mode
  SceneDev sd{};
  SceneDev* sd_dev = nullptr;
  BinScratch bin{};
  FastTuning tune{};
  int key_bits = 0;
  int* d_prefix = nullptr;  // [0,2) items, [2,4) active, [6,8) blocks
  int steps_since_sort = 1 << 30;
  // re-binning interval in use (1 .. tune.sort_interval): dropped to 1 when
  // particles leave their work items' tiles between binnings, doubled back
  // after a run of clean checks
  int bin_interval = 8;
  int clean_checks = 0;
  // the device counters as copied (without a wait) at the last binning point
  // and read at the next one
  int* h_cnt = nullptr;
  cudaEvent_t cnt_ev = nullptr;
  bool cnt_pending = false;
  long long fallbacks_seen = 0;
  int steps_at_snapshot = 0;  // steps between the last two snapshots
  int version = 0;
  bool volume_given = false;
  // FAST: acc holds the P2G sums of the current particle state (the next
  // step's grid update consumes them)
  bool p2g_ready = false;
  // graphs of one step, keyed by (dt, with binning)
  cudaGraphExec_t g_plain = nullptr, g_sort = nullptr;
  float g_dt = NAN;
  snow_phase_times times{};
  uint32_t wide_base = 0;  // FixState::wide at the last phase-times reset
  float last_dt = 1e-3f;
  // bounded copy waits of the FAST kernels (snow_scene_set_wait_limit)
  uint32_t wait_ns = kDefaultWaitNs;
  uint32_t tx_unsent = 0;
};

struct snow_batch {
  snow_ctx* ctx = nullptr;
  std::vector<snow_scene*> scenes;
  SceneDev* d_scenes = nullptr;
  int* d_prefix = nullptr;  // items (n+1), active (n+1), unused (n+1), blocks (n+1)
  std::vector<int> versions;
  long long total_blocks = 0;
  int step_count = 0;
  std::map<int, cudaGraphExec_t> graphs;  // 0: the step that re-bins every scene, 1: the others
  std::vector<float> g_dt;
  int g_threads = 0;
  size_t bytes = 0;
  std::vector<std::pair<void*, size_t>> allocs;
  // every scene's counters, written by a kernel into mapped pinned memory at
  // one checking point and read at the next
  int* h_cnt = nullptr;
  int* d_hcnt = nullptr;
  cudaEvent_t cnt_ev = nullptr;
  bool cnt_pending = false;
};

// ---------------------------------------------------------------------------
namespace {

snow_status fail(snow_ctx* c, snow_status st, const std::string& msg) {
  if (c) c->err = msg;
  return st;
}

snow_status cuda_fail(snow_ctx* c, cudaError_t e, const char* what) {
  cudaGetLastError();
  char buf[256];
  snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  return fail(c, SNOW_ECUDA, buf);
}

#define CK(x)                                            \
  do {                                                   \
    cudaError_t e_ = (x);                                \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #x); \
  } while (0)

// The device address of page-locked host memory (the caller pinned it: the
// GPU reads and writes it directly over the CPU-GPU link), or nullptr for
// pageable memory, which goes through a device staging buffer.
void* pinned_device_ptr(const void* host) {
  cudaPointerAttributes a{};
  if (!host || cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

snow_status dalloc(snow_ctx* ctx, std::vector<std::pair<void*, size_t>>& owner, size_t& owner_bytes, size_t bytes,
                   void** out) {
  *out = nullptr;
  if (bytes == 0) return SNOW_OK;
  bytes = (bytes + 255) & ~(size_t)255;
  if (ctx->budget && ctx->used + bytes > ctx->budget)
    return fail(ctx, SNOW_EBUDGET, "HBM budget exceeded");
  // stream-ordered, then waited for (here, or once at the end of a run of
  // allocations: AllocRun), so the memory is usable from any stream
  cudaError_t e = cudaMallocFromPoolAsync(out, bytes, ctx->pool, ctx->stream);
  if (e == cudaSuccess && !ctx->defer_sync) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return fail(ctx, SNOW_ENOMEM, std::string("cudaMallocFromPoolAsync: ") + cudaGetErrorString(e));
  }
  ctx->used += bytes;
  owner_bytes += bytes;
  owner.emplace_back(*out, bytes);
  return SNOW_OK;
}

// A run of allocations that waits for the stream once, when it ends (a
// scene's buffers are a few dozen allocations).
struct AllocRun {
  snow_ctx* ctx;
  bool outer;
  explicit AllocRun(snow_ctx* c) : ctx(c), outer(!c->defer_sync) { c->defer_sync = true; }
  ~AllocRun() {
    if (!outer) return;
    ctx->defer_sync = false;
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) cudaGetLastError();
  }
};

void dfree_all(snow_ctx* ctx, std::vector<std::pair<void*, size_t>>& owner, size_t& owner_bytes) {
  for (auto& a : owner) {
    cudaFreeAsync(a.first, ctx->stream);
    ctx->used -= a.second;
  }
  owner.clear();
  owner_bytes = 0;
}

void dfree_one(snow_ctx* ctx, snow_scene* s, void* p) {
  for (size_t i = 0; i < s->allocs.size(); i++)
    if (s->allocs[i].first == p) {
      cudaFreeAsync(p, ctx->stream);
      ctx->used -= s->allocs[i].second;
      s->bytes -= s->allocs[i].second;
      s->allocs.erase(s->allocs.begin() + (long)i);
      return;
    }
}

template <class T>
snow_status salloc(snow_scene* s, size_t count, T** out) {
  return dalloc(s->ctx, s->allocs, s->bytes, count * sizeof(T), reinterpret_cast<void**>(out));
}

int ceil_log2(unsigned long long v) {
  int b = 0;
  while ((1ull << b) < v) b++;
  return b;
}

void drop_graphs(snow_scene* s) {
  if (s->g_plain) cudaGraphExecDestroy(s->g_plain);
  if (s->g_sort) cudaGraphExecDestroy(s->g_sort);
  s->g_plain = s->g_sort = nullptr;
  s->g_dt = NAN;
}

bool valid_params(const snow_params* p) {
  if (!p) return false;
  for (int k = 0; k < 3; k++)
    if (p->grid_dim[k] <= 0 || p->grid_dim[k] > 4096) return false;
  if (!(p->grid_spacing > 0.0f)) return false;
  if ((double)p->grid_dim[0] * p->grid_dim[1] * p->grid_dim[2] > 2.0e9) return false;
  if (p->mode != SNOW_MODE_REFERENCE && p->mode != SNOW_MODE_FAST) return false;
  if (!(p->implicit_beta >= 0.0f && p->implicit_beta <= 1.0f)) return false;
  if (!(p->implicit_tolerance >= 0.0f) || !std::isfinite(p->implicit_tolerance)) return false;
  if (p->implicit_max_iters < 0 || p->implicit_max_iters > kCrMaxIters) return false;
  return true;
}

// The semi-implicit solve's settings with the library defaults filled in.
bool is_implicit(const snow_params& p) { return p.implicit_beta > 0.0f; }
int implicit_iters(const snow_params& p) { return p.implicit_max_iters > 0 ? p.implicit_max_iters : 50; }
float implicit_tol(const snow_params& p) { return p.implicit_tolerance > 0.0f ? p.implicit_tolerance : 1e-5f; }

void fill_sd_params(snow_scene* s) {
  SceneDev& d = s->sd;
  for (int k = 0; k < 3; k++) {
    d.gpos[k] = s->p.grid_pos[k];
    d.dim[k] = s->p.grid_dim[k];
    d.bdim[k] = (s->p.grid_dim[k] + 3) / 4;
    d.grav[k] = s->p.gravity[k];
  }
  d.h = s->p.grid_spacing;
  d.inv_h = 1.0f / s->p.grid_spacing;
  d.nblocks = d.bdim[0] * d.bdim[1] * d.bdim[2];
  d.young = s->p.young;
  // mu0 = E / (2 (1 + nu)), lambda0 = E nu / ((1 + nu)(1 - 2 nu)), in the
  // order and precision lame.include.glsl evaluates them per particle
  {
    const float E = s->p.young, nu = s->p.poisson;
    d.mu0 = E / (2.0f * (1.0f + nu));
    d.lambda0 = E * nu / ((1.0f + nu) * (1.0f - 2.0f * nu));
  }
  d.poisson = s->p.poisson;
  d.hardening = s->p.hardening;
  d.crit_lo = 1.0f - s->p.crit_compression;
  d.crit_hi = 1.0f + s->p.crit_stretch;
  d.alpha = s->p.alpha;
  d.ncoll = s->ncoll;
  d.coll = s->coll_d;
  d.imp_beta = s->p.implicit_beta;
  d.imp_tol = implicit_tol(s->p);
  d.imp_maxit = implicit_iters(s->p);
  d.wait_ns = s->wait_ns;
  d.tx_unsent = s->tx_unsent;
}

snow_status push_sd(snow_scene* s) {
  snow_ctx* ctx = s->ctx;
  CK(cudaMemcpyAsync(s->sd_dev, &s->sd, sizeof(SceneDev), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  s->version++;
  drop_graphs(s);
  return SNOW_OK;
}

// ---- fast-mode buffers ----------------------------------------------------
snow_status fast_alloc_particles(snow_scene* s, size_t cap) {
  AllocRun run(s->ctx);
  SceneDev& d = s->sd;
  snow_status st;
  if ((st = salloc(s, cap, &d.xm)) || (st = salloc(s, cap, &d.vv)) || (st = salloc(s, cap, &d.fa)) ||
      (st = salloc(s, cap, &d.fb)) || (st = salloc(s, cap, &d.fc)) || (st = salloc(s, cap, &d.pid)) ||
      (st = salloc(s, cap, &d.vq)))
    return st;
  BinScratch& b = s->bin;
  const size_t tiles = radix_tiles(cap);
  const size_t hist = 256 * tiles;
  const size_t partial = (hist + 4095) / 4096 + 1;
  if ((st = salloc(s, cap, &b.keys[0])) || (st = salloc(s, cap, &b.keys[1])) || (st = salloc(s, cap, &b.vals[0])) ||
      (st = salloc(s, cap, &b.vals[1])) || (st = salloc(s, hist, &b.hist)) || (st = salloc(s, partial, &b.scan_tmp)) ||
      (st = salloc(s, cap, &b.tmp4[0])) || (st = salloc(s, cap, &b.tmp4[1])) || (st = salloc(s, cap, &b.tmp4[2])) ||
      (st = salloc(s, cap, &b.tmp4[3])) || (st = salloc(s, cap, &b.tmp4[4])) || (st = salloc(s, cap, &b.tmp2)) ||
      (st = salloc(s, cap, &b.tmp_pid)))
    return st;
  b.n_cap = cap;
  d.bxm = b.tmp4[0];
  d.bvv = b.tmp4[1];
  d.bfa = b.tmp4[2];
  d.bfb = b.tmp4[3];
  d.bvq = b.tmp4[4];
  d.bfc = b.tmp2;
  d.item_cap = (int)(cap / kMinItemMax + std::min<size_t>(cap, (size_t)d.nblocks) + 1);
  if ((st = salloc(s, (size_t)d.item_cap, &d.items))) return st;
  return SNOW_OK;
}

snow_status fast_alloc_grid(snow_scene* s) {
  AllocRun run(s->ctx);
  SceneDev& d = s->sd;
  snow_status st;
  const size_t nb = (size_t)d.nblocks;
  if ((st = salloc(s, nb, &d.blk_slot)) || (st = salloc(s, nb, &d.blk_flag)) ||
      (st = salloc(s, nb * kAccBlockWords, &d.acc)) || (st = salloc(s, (size_t)1, &d.fix)) ||
      (st = salloc(s, nb, &s->bin.bstart)) ||
      (st = salloc(s, nb, &s->bin.bend)) || (st = salloc(s, nb, &s->bin.home)) ||
      (st = salloc(s, (size_t)kCounterStride, &d.counters)) || (st = salloc(s, (size_t)8, &s->d_prefix)) ||
      (st = salloc(s, (size_t)1, &s->sd_dev)))
    return st;
  if (is_implicit(s->p) && (st = salloc(s, (size_t)1, &d.crs))) return st;
  snow_ctx* ctx = s->ctx;
  if (d.crs) CK(cudaMemsetAsync(d.crs, 0, sizeof(CrScalars), ctx->stream));
  CK(cudaMemsetAsync(d.blk_flag, 0, nb * sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(d.blk_slot, 0xff, nb * sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(d.acc, 0, nb * kAccBlockWords * sizeof(unsigned long long), ctx->stream));
  {
    FixState f{};
    f.scale[0] = f.scale[1] = f.scale[2] = 1.0f;
    CK(cudaMemcpyAsync(d.fix, &f, sizeof f, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  CK(cudaMemsetAsync(d.counters, 0, kCounterStride * sizeof(int), ctx->stream));
  return SNOW_OK;
}

// The output pool (grid-update results of the active blocks).
snow_status fast_alloc_pool(snow_scene* s, int cap_blocks) {
  AllocRun run(s->ctx);
  SceneDev& d = s->sd;
  snow_ctx* ctx = s->ctx;
  if (d.gout) dfree_one(ctx, s, d.gout);
  if (d.active) dfree_one(ctx, s, d.active);
  if (d.crv) dfree_one(ctx, s, d.crv);
  if (d.cru) dfree_one(ctx, s, d.cru);
  d.gout = nullptr;
  d.active = nullptr;
  d.crv = nullptr;
  d.cru = nullptr;
  snow_status st;
  if ((st = salloc(s, (size_t)cap_blocks * kOutBlockFloats, &d.gout)) || (st = salloc(s, (size_t)cap_blocks, &d.active)))
    return st;
  if (d.crs && ((st = salloc(s, (size_t)cap_blocks * kBlockNodes * 3, &d.crv)) ||
                (st = salloc(s, (size_t)cap_blocks * kImpBlockFloats, &d.cru))))
    return st;
  d.pool_cap = cap_blocks;
  return SNOW_OK;
}

// Prefix arrays of a one-scene work space: [items 0,1][active 2,3][blocks 6,7];
// items and active are written on the device.
snow_status fast_single_prefix(snow_scene* s) {
  snow_ctx* ctx = s->ctx;
  int h[2] = {0, s->sd.nblocks};
  CK(cudaMemcpyAsync(s->d_prefix + 6, h, 2 * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return SNOW_OK;
}

int item_ctas(const FastTuning& t) { return num_sms() * t.ctas_per_sm; }
int grid_ctas() { return num_sms() * 8; }

// Binning: keys, radix sort, permutation, work items, item prefix.
// in_step: the step's fused kernel follows in the same stream and reads the
// particles from the binned copies (no copy back); else they are copied back
// for the per-kernel P2G that follows.
void fast_bin(snow_scene* s, cudaStream_t st, bool in_step) {
  fast_sort_keys(s->sd, s->sd_dev, s->bin, s->key_bits, st);
  fast_apply_bins(s->sd, s->sd_dev, s->bin, s->tune.items_max, !in_step, st);
  fast_prefix(s->sd_dev, 1, s->d_prefix + 0, s->d_prefix + 2, st);
}

// Active blocks of the pending P2G sums -> pool slots (and prefixes).
void fast_enqueue_compact(snow_scene* s, cudaStream_t st, bool counters_reset = false) {
  if (!counters_reset) fast_begin_step(s->sd_dev, 1, false, st);
  fast_compact(s->sd_dev, s->d_prefix + 6, 1, s->sd.nblocks, s->d_prefix + 0, s->d_prefix + 2, st);
}
void fast_enqueue_p2g(snow_scene* s, bool mass_only, cudaStream_t st) {
  fast_p2g(s->sd_dev, s->sd, s->d_prefix + 0, 1, item_ctas(s->tune), mass_only, st);
}
void fast_enqueue_grid(snow_scene* s, bool clear_only, cudaStream_t st) {
  fast_grid(s->sd_dev, s->d_prefix + 2, 1, grid_ctas(), clear_only, st);
}
// The semi-implicit solve after the grid update (explicit scenes: nothing).
void fast_enqueue_solve(snow_scene* s, cudaStream_t st) {
  if (s->sd.crs)
    fast_implicit_solve(s->sd_dev, s->d_prefix + 0, s->d_prefix + 2, 1, s->sd.imp_maxit, item_ctas(s->tune),
                        grid_ctas(), s->ctx->d_iter, s->ctx->body_stream, s->ctx->gate_stream, st);
}
// One step of a scene whose P2G sums of the current state are pending in
// acc: rigid advance, [binning], grid update, G2P + advance + next P2G.
void fast_enqueue_step(snow_scene* s, bool bin, cudaStream_t st) {
  fast_begin_step(s->sd_dev, 1, s->ncoll > 0, st);
  if (bin) fast_bin(s, st, true);
  fast_enqueue_compact(s, st, true);
  fast_enqueue_grid(s, false, st);
  fast_enqueue_solve(s, st);
  fast_g2p2g(s->sd_dev, s->d_prefix + 0, 1, item_ctas(s->tune), bin, st);
}

snow_status set_dt(snow_scene* s, float dt) {
  if (s->sd.dt != dt) {
    s->sd.dt = dt;
    return push_sd(s);
  }
  return SNOW_OK;
}

// Checks a copy of the device-side counters for the errors counted there.
// (The pool holds a slot for every grid block, so CNT_OVERFLOW stays 0; it is
// checked all the same.)
snow_status check_counters(snow_scene* s, const int* h) {
  snow_ctx* ctx = s->ctx;
  if (h[CNT_TIMEOUT] > 0) return fail(ctx, SNOW_ETIMEDOUT, "a bounded device wait ran out");
  if (h[CNT_OVERFLOW] > 0) return fail(ctx, SNOW_ECAPACITY, "grid block pool overflowed");
  if (h[CNT_NONFINITE] > 0) return fail(ctx, SNOW_ENUMERIC, "non-finite particle state");
  return SNOW_OK;
}

// At a binning point of snow_scene_step: checks the counters copied at the
// previous binning point (that copy has long landed, so there is no wait for
// the queued steps), adapts the re-binning interval to the share of
// particle-steps that left their work item's tile since then (above 1/256:
// re-bin every step; below 1/4096 eight times in a row: double the interval,
// up to the tuned one), and copies the counters again for the next point.
snow_status fast_check_async(snow_scene* s, int steps_since_last) {
  snow_ctx* ctx = s->ctx;
  if (s->cnt_pending) {
    CK(cudaEventSynchronize(s->cnt_ev));
    s->cnt_pending = false;
    const int* h = s->h_cnt;
    const long long fb = (long long)(unsigned)h[CNT_FALLBACK];
    const long long delta = fb - s->fallbacks_seen;
    s->fallbacks_seen = fb;
    const double work = (double)s->steps_at_snapshot * (double)std::max<size_t>(s->n, 1);
    if (s->steps_at_snapshot > 0 && delta > work / 256.0) {
      s->bin_interval = 1;
      s->clean_checks = 0;
    } else if (delta <= work / 4096.0 && ++s->clean_checks >= 8) {
      s->bin_interval = std::min(s->tune.sort_interval, 2 * s->bin_interval);
      s->clean_checks = 0;
    }
    snow_status r = check_counters(s, h);
    if (r) return r;
  }
  CK(cudaMemcpyAsync(s->h_cnt, s->sd.counters, kCounterStride * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaEventRecord(s->cnt_ev, ctx->stream));
  s->cnt_pending = true;
  s->steps_at_snapshot = steps_since_last;
  return SNOW_OK;
}

// Checks device-side error counters now (waits for the stream); grows the
// output pool when it runs full.
snow_status fast_check(snow_scene* s) {
  snow_ctx* ctx = s->ctx;
  CK(cudaMemcpyAsync(ctx->h_counters, s->sd.counters, kCounterStride * sizeof(int), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return check_counters(s, ctx->h_counters);
}

// ExplicitTimeUpdate::init (explicittimeupdate.cpp:29-33) -- grid mass and
// particle volumes -- followed by the P2G of the initial state, which the
// first step consumes.
snow_status fast_init(snow_scene* s) {
  snow_ctx* ctx = s->ctx;
  cudaStream_t st = ctx->stream;
  snow_status r;
  s->sd.n = (int)s->n;
  if (s->sd.crs) fast_implicit_setup();
  if ((r = fast_single_prefix(s))) return r;
  if ((r = push_sd(s))) return r;
  fast_bin(s, st, false);
  fast_enqueue_p2g(s, true, st);  // gMassCompute
  // The output pool has a slot for every grid block: however far the
  // particles spread, the compaction of a step finds a slot for each block
  // that received sums (the footprint bound always counted the pool at this
  // size). Only the active blocks' slots are written or read in a step.
  if (s->sd.pool_cap != s->sd.nblocks) {
    if ((r = fast_alloc_pool(s, s->sd.nblocks))) return r;
    if ((r = push_sd(s))) return r;
  }
  fast_enqueue_compact(s, st);
  if (!s->volume_given) fast_volume(s->sd_dev, (int)s->n, st);  // pVolumeCompute
  fast_enqueue_grid(s, true, st);                                // clear acc
  fast_enqueue_p2g(s, false, st);                                // P2G of step 1
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  s->steps_since_sort = 0;
  s->p2g_ready = true;
  return SNOW_OK;
}

RefArgs& ref_args(snow_scene* s) {
  RefArgs& a = s->ra;
  for (int k = 0; k < 3; k++) {
    a.gpos[k] = s->p.grid_pos[k];
    a.dim[k] = s->p.grid_dim[k];
    a.grav[k] = s->p.gravity[k];
  }
  a.h = s->p.grid_spacing;
  a.young = s->p.young;
  a.poisson = s->p.poisson;
  a.hardening = s->p.hardening;
  a.crit_c = s->p.crit_compression;
  a.crit_s = s->p.crit_stretch;
  a.alpha = s->p.alpha;
  a.ncoll = s->ncoll;
  a.coll = s->coll_d;
  a.n = (int)s->n;
  a.G = s->G;
  return a;
}

snow_status ref_alloc(snow_scene* s, size_t cap) {
  AllocRun run(s->ctx);
  RefArgs& a = s->ra;
  snow_status st;
  if ((st = salloc(s, cap, &a.pxm)) || (st = salloc(s, cap, &a.pv)) || (st = salloc(s, 4 * cap, &a.pfe)) ||
      (st = salloc(s, 4 * cap, &a.pfp)) || (st = salloc(s, cap, &a.pvn)) || (st = salloc(s, cap, &a.pd0)) ||
      (st = salloc(s, cap, &a.pd1)) || (st = salloc(s, cap, &a.pd2)))
    return st;
  if (!a.gv) {
    if ((st = salloc(s, (size_t)s->G, &a.gv)) || (st = salloc(s, (size_t)s->G, &a.gf)) ||
        (st = salloc(s, (size_t)s->G, &a.gvn)))
      return st;
  }
  return SNOW_OK;
}

snow_status ensure_capacity(snow_scene* s, size_t n) {
  if (n == 0) return fail(s->ctx, SNOW_EINVAL, "no particles");
  if (n > 0x7fffffffull) return fail(s->ctx, SNOW_EINVAL, "too many particles");
  if (s->cap == 0) {
    s->cap = n;
    return s->mode == SNOW_MODE_FAST ? fast_alloc_particles(s, n) : ref_alloc(s, n);
  }
  if (n > s->cap) return fail(s->ctx, SNOW_EINVAL, "more particles than the scene's capacity");
  return SNOW_OK;
}

double det_rowmajor(const float* f) {
  const double a = f[0], b = f[1], c = f[2], d = f[3], e = f[4], g = f[5], h = f[6], i = f[7], j = f[8];
  return a * (e * j - g * i) - b * (d * j - g * h) + c * (d * i - e * h);
}

snow_status fast_upload_soa(snow_scene* s, const std::vector<float4>& xm, const std::vector<float4>& vv,
                            const std::vector<float4>& fa, const std::vector<float4>& fb,
                            const std::vector<float2>& fc) {
  snow_ctx* ctx = s->ctx;
  const size_t n = xm.size();
  std::vector<uint32_t> pid(n);
  for (size_t i = 0; i < n; i++) pid[i] = (uint32_t)i;
  CK(cudaMemcpyAsync(s->sd.xm, xm.data(), n * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(s->sd.vv, vv.data(), n * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(s->sd.fa, fa.data(), n * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(s->sd.fb, fb.data(), n * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(s->sd.fc, fc.data(), n * sizeof(float2), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(s->sd.pid, pid.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream));
  const std::vector<float4> frame(n, make_float4(1.0f, 0.0f, 0.0f, 0.0f));  // no previous SVD: identity
  CK(cudaMemcpyAsync(s->sd.vq, frame.data(), n * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return SNOW_OK;
}

}  // namespace

// ===========================================================================
extern "C" {

void snow_params_default(snow_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  // src/snow/utils/defines.hpp:14-54
  p->grid_pos[0] = 0.5125f;
  p->grid_pos[1] = 0.5125f;
  p->grid_pos[2] = 1.5125f;
  p->grid_dim[0] = p->grid_dim[1] = p->grid_dim[2] = 201;
  p->grid_spacing = 0.05f;
  p->young = 6e6f;
  p->poisson = 0.2f;
  p->hardening = 30.0f;
  p->crit_compression = 1.0e-2f;
  p->crit_stretch = 1e-3f;
  p->alpha = 0.95f;  // g2pTransfer.glsl:2, particleAdvance.glsl:2
  p->gravity[0] = 0.0f;
  p->gravity[1] = -9.81f;  // gForceCompute.glsl:39
  p->gravity[2] = 0.0f;
  p->mode = SNOW_MODE_FAST;
  p->sort_interval = 0;
}

int snow_default_walls(const snow_params* p, snow_collider out[6]) {
  // explicit.cpp:9-67: positions formed in double, stored as float; normals
  // +x, +y, +z at offset 4 nodes, -x, -y, -z at dim - 4 nodes; friction 0.2.
  const int off = 4;
  for (int w = 0; w < 6; w++) {
    snow_collider& c = out[w];
    std::memset(&c, 0, sizeof c);
    const bool hi = w >= 3;
    for (int k = 0; k < 3; k++)
      c.pos[k] = (float)((double)p->grid_pos[k] + (double)(hi ? p->grid_dim[k] - off : off) * (double)p->grid_spacing);
    c.normal[w % 3] = hi ? -1.0f : 1.0f;
    c.type = 0;
    c.radius = 0.0f;
    c.friction = 0.2f;
  }
  return 6;
}

snow_status snow_ctx_create(int device, size_t hbm_budget_bytes, snow_ctx** out) {
  if (!out) return SNOW_EINVAL;
  *out = nullptr;
  snow_ctx* ctx = new snow_ctx();
  ctx->device = device;
  ctx->budget = hbm_budget_bytes;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    e = cudaMemPoolCreate(&ctx->pool, &props);
  }
  if (e == cudaSuccess) {
    // keep freed memory for reuse, up to the budget (all of it without one);
    // the pool returns what exceeds that at synchronisation points
    uint64_t keep = hbm_budget_bytes ? (uint64_t)hbm_budget_bytes : UINT64_MAX;
    e = cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_stats, sizeof(StatsSlot) * (1 + SNOW_STATS_SLOTS));
  if (e == cudaSuccess)
    e = cudaHostAlloc(&ctx->h_stats, sizeof(StatsAccum) * (1 + SNOW_STATS_SLOTS), cudaHostAllocMapped);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&ctx->d_hstats, ctx->h_stats, 0);
  if (e == cudaSuccess) e = cudaMemset(ctx->d_stats, 0, sizeof(StatsSlot) * (1 + SNOW_STATS_SLOTS));
  for (int i = 0; i < SNOW_STATS_SLOTS && e == cudaSuccess; i++)
    e = cudaEventCreateWithFlags(&ctx->stat_ev[i], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_counters, kCounterStride * sizeof(int));
  for (int i = 0; i < 8 && e == cudaSuccess; i++) e = cudaEventCreate(&ctx->ev[i]);
  for (int i = 0; i < snow_ctx::kAux && e == cudaSuccess; i++) {
    e = cudaStreamCreateWithFlags(&ctx->aux[i], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->join_ev[i], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_iter, sizeof(int));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->body_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->gate_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    cudaGetLastError();
    snow_ctx_destroy(ctx);
    return SNOW_ECUDA;
  }
  *out = ctx;
  return SNOW_OK;
}

void snow_ctx_destroy(snow_ctx* ctx) {
  if (!ctx) return;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  while (!ctx->batches.empty()) snow_batch_destroy(*ctx->batches.begin());
  while (!ctx->scenes.empty()) snow_scene_destroy(*ctx->scenes.begin());
  for (int i = 0; i < 8; i++)
    if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
  for (int i = 0; i < snow_ctx::kAux; i++) {
    if (ctx->aux[i]) {
      cudaStreamSynchronize(ctx->aux[i]);
      cudaStreamDestroy(ctx->aux[i]);
    }
    if (ctx->join_ev[i]) cudaEventDestroy(ctx->join_ev[i]);
  }
  if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
  if (ctx->body_stream) cudaStreamDestroy(ctx->body_stream);
  if (ctx->gate_stream) cudaStreamDestroy(ctx->gate_stream);
  if (ctx->d_iter) cudaFree(ctx->d_iter);
  for (int i = 0; i < SNOW_STATS_SLOTS; i++)
    if (ctx->stat_ev[i]) cudaEventDestroy(ctx->stat_ev[i]);
  if (ctx->d_stats) cudaFree(ctx->d_stats);
  if (ctx->h_stats) cudaFreeHost(ctx->h_stats);
  if (ctx->h_counters) cudaFreeHost(ctx->h_counters);
  if (ctx->stream) {
    cudaStreamSynchronize(ctx->stream);  // pending frees into the pool
    cudaStreamDestroy(ctx->stream);
  }
  if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
  delete ctx;
}

const char* snow_last_error(const snow_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }
size_t snow_ctx_bytes_in_use(const snow_ctx* ctx) { return ctx ? ctx->used : 0; }
snow_status snow_ctx_set_graphs(snow_ctx* ctx, int on) {
  if (!ctx) return SNOW_EINVAL;
  ctx->graphs = on != 0;
  return SNOW_OK;
}

snow_status snow_ctx_set_profiling(snow_ctx* ctx, int on) {
  if (!ctx) return SNOW_EINVAL;
  ctx->profiling = on != 0;
  return SNOW_OK;
}
void* snow_ctx_stream(const snow_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }
snow_status snow_ctx_synchronize(snow_ctx* ctx) {
  if (!ctx) return SNOW_EINVAL;
  CK(cudaStreamSynchronize(ctx->stream));
  return SNOW_OK;
}

size_t snow_scene_footprint(const snow_params* p, size_t n) {
  if (!valid_params(p)) return 0;
  const double G = (double)p->grid_dim[0] * p->grid_dim[1] * p->grid_dim[2];
  if (p->mode == SNOW_MODE_REFERENCE) return (size_t)(n * (16.0 * 6 + 128.0) + G * 48.0);
  const double nb = (double)((p->grid_dim[0] + 3) / 4) * ((p->grid_dim[1] + 3) / 4) * ((p->grid_dim[2] + 3) / 4);
  // An upper bound: particle streams (xm, vv, fa, fb, vq: 16 B, fc: 8 B, pid: 4 B)
  // + binning scratch (2 key + 2 value words, 5 x 16 B + 8 B + 4 B permutation
  // targets, radix histograms) + work items (16 B each) + per block the dense
  // fixed-point P2G sums (320 64-bit words), flags, slot and bin tables (5 ints) + the output
  // pool at its largest (every block: 384 floats + 1 int) + the upload's
  // staging copy of the caller's arrays (x, v, m, F_E, F_P: 100 B).
  const double tiles = (double)radix_tiles(n);
  const double items = (double)n / kMinItemMax + std::min((double)n, nb) + 1;
  // A semi-implicit scene adds per pool block its solver planes (64 nodes x
  // (3 float4 + 3 floats)) and one scalar record.
  const double solver = is_implicit(*p) ? nb * (64 * (48.0 + 12.0)) + sizeof(CrScalars) : 0.0;
  return (size_t)(n * (92.0 + 108.0 + 100.0) + tiles * 256 * 4.0 + 4096.0 + items * 16.0 + nb * (kAccBlockWords * 8.0 + 5 * 4.0) +
                  nb * (384 * 4.0 + 4.0) + solver + 1024.0);
}

snow_status snow_scene_create(snow_ctx* ctx, const snow_params* p, const snow_collider* colliders, int n_colliders,
                              size_t capacity, snow_scene** out) {
  if (!ctx || !out || !valid_params(p) || n_colliders < 0 || (n_colliders > 0 && !colliders))
    return fail(ctx, SNOW_EINVAL, "snow_scene_create: invalid argument");
  if (p->mode == SNOW_MODE_REFERENCE && is_implicit(*p))
    return fail(ctx, SNOW_EUNSUPPORTED, "the semi-implicit update has no shader counterpart: FAST mode only");
  *out = nullptr;
  CK(cudaSetDevice(ctx->device));
  snow_scene* s = new snow_scene();
  s->ctx = ctx;
  s->p = *p;
  s->mode = p->mode;
  s->G = (long long)p->grid_dim[0] * p->grid_dim[1] * p->grid_dim[2];
  s->coll_h.assign(colliders, colliders + n_colliders);
  s->ncoll = n_colliders;
  if (p->sort_interval > 0) s->tune.sort_interval = p->sort_interval;
  s->bin_interval = s->tune.sort_interval;
  snow_status st = SNOW_OK;
  if (n_colliders > 0) st = salloc(s, (size_t)n_colliders, &s->coll_d);
  if (!st && n_colliders > 0)
    if (cudaMemcpy(s->coll_d, colliders, sizeof(snow_collider) * n_colliders, cudaMemcpyHostToDevice) != cudaSuccess)
      st = cuda_fail(ctx, cudaGetLastError(), "collider upload");
  if (!st && s->mode == SNOW_MODE_FAST) {
    if (cudaMallocHost(&s->h_cnt, kCounterStride * sizeof(int)) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->cnt_ev, cudaEventDisableTiming) != cudaSuccess)
      st = cuda_fail(ctx, cudaGetLastError(), "counter snapshot");
  }
  if (!st && s->mode == SNOW_MODE_FAST) {
    fill_sd_params(s);
    s->sd.dt = 1e-3f;
    s->key_bits = ceil_log2((unsigned long long)s->sd.nblocks * 64ull);
    st = fast_alloc_grid(s);
  }
  if (!st && capacity > 0) st = ensure_capacity(s, capacity);
  ctx->scenes.insert(s);
  if (st) {
    snow_scene_destroy(s);
    return st;
  }
  *out = s;
  return SNOW_OK;
}

void snow_scene_destroy(snow_scene* s) {
  if (!s) return;
  snow_ctx* ctx = s->ctx;
  cudaStreamSynchronize(ctx->stream);
  // a batch that holds this scene can no longer step
  std::vector<snow_batch*> holders;
  for (snow_batch* b : ctx->batches)
    if (std::find(b->scenes.begin(), b->scenes.end(), s) != b->scenes.end()) holders.push_back(b);
  for (snow_batch* b : holders) snow_batch_destroy(b);
  drop_graphs(s);
  dfree_all(ctx, s->allocs, s->bytes);
  if (s->h_cnt) cudaFreeHost(s->h_cnt);
  if (s->cnt_ev) cudaEventDestroy(s->cnt_ev);
  ctx->scenes.erase(s);
  delete s;
}

size_t snow_scene_size(const snow_scene* s) { return s ? s->n : 0; }

snow_status snow_scene_upload(snow_scene* s, const float* x, const float* v, const float* m, const float* FE,
                              const float* FP, size_t n) {
  if (!s || !x || !v || !m) return fail(s ? s->ctx : nullptr, SNOW_EINVAL, "snow_scene_upload: null array");
  snow_ctx* ctx = s->ctx;
  snow_status st = ensure_capacity(s, n);
  if (st) return st;
  s->n = n;
  s->initialized = false;
  s->volume_given = false;
  if (s->mode == SNOW_MODE_REFERENCE) {
    // ParticleSystem::initSSBO: pxm = (x, m), pv = (v * 1e8, 0), FE / FP mat4
    std::vector<float4> pxm(n), pfe(4 * n), pfp(4 * n);
    std::vector<int4> pv(n), zero(n);
    for (size_t i = 0; i < n; i++) {
      pxm[i] = make_float4(x[3 * i], x[3 * i + 1], x[3 * i + 2], m[i]);
      pv[i] = make_int4((int)((double)v[3 * i] * 1e8), (int)((double)v[3 * i + 1] * 1e8),
                        (int)((double)v[3 * i + 2] * 1e8), 0);
      zero[i] = make_int4(0, 0, 0, 0);
      for (int c = 0; c < 4; c++) {
        float fe[4] = {0, 0, 0, 0}, fp[4] = {0, 0, 0, 0};
        for (int r = 0; r < 3 && c < 3; r++) {
          fe[r] = FE ? FE[9 * i + 3 * r + c] : (r == c ? 1.0f : 0.0f);
          fp[r] = FP ? FP[9 * i + 3 * r + c] : (r == c ? 1.0f : 0.0f);
        }
        pfe[4 * i + c] = make_float4(fe[0], fe[1], fe[2], fe[3]);
        pfp[4 * i + c] = make_float4(fp[0], fp[1], fp[2], fp[3]);
      }
    }
    RefArgs& a = ref_args(s);
    CK(cudaMemcpy(a.pxm, pxm.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(a.pv, pv.data(), n * sizeof(int4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(a.pfe, pfe.data(), 4 * n * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(a.pfp, pfp.data(), 4 * n * sizeof(float4), cudaMemcpyHostToDevice));
    for (int4* acc : {a.pvn, a.pd0, a.pd1, a.pd2}) CK(cudaMemcpy(acc, zero.data(), n * sizeof(int4), cudaMemcpyHostToDevice));
    s->uploaded = true;
    return SNOW_OK;
  }
  // the pack kernel reads the caller's arrays where they lie when they are
  // pinned; pageable ones are first copied as they are to a staging buffer
  s->sd.n = (int)n;
  if (n > 0) {
    const float* in[5] = {x, v, m, FE, FP};
    const size_t width[5] = {3, 3, 1, 9, 9};
    const float* dev[5] = {};
    size_t words = 0;
    for (int k = 0; k < 5; k++) {
      if (!in[k]) continue;
      dev[k] = static_cast<const float*>(pinned_device_ptr(in[k]));
      if (!dev[k]) words += width[k] * n;
    }
    std::vector<std::pair<void*, size_t>> tmp;
    size_t tmp_bytes = 0;
    float* stage = nullptr;
    st = dalloc(ctx, tmp, tmp_bytes, words * sizeof(float), (void**)&stage);
    if (st) return st;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 5 && e == cudaSuccess; k++) {
      if (!in[k] || dev[k]) continue;
      e = cudaMemcpyAsync(stage, in[k], width[k] * n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
      dev[k] = stage;
      stage += width[k] * n;
    }
    if (e == cudaSuccess) {
      fast_pack(dev[0], dev[1], dev[2], dev[3], dev[4], n, s->sd, ctx->stream);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);  // the caller may reuse its arrays
    dfree_all(ctx, tmp, tmp_bytes);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "snow_scene_upload");
  }
  s->uploaded = true;
  return SNOW_OK;
}

snow_status snow_scene_upload_std140(snow_scene* s, const float* pxm, const int32_t* pv, const float* pFE,
                                     const float* pFP, size_t n) {
  if (!s || !pxm || !pv || !pFE || !pFP) return fail(s ? s->ctx : nullptr, SNOW_EINVAL, "null buffer");
  snow_ctx* ctx = s->ctx;
  snow_status st = ensure_capacity(s, n);
  if (st) return st;
  s->n = n;
  s->initialized = false;
  s->volume_given = false;
  if (s->mode == SNOW_MODE_REFERENCE) {
    RefArgs& a = ref_args(s);
    CK(cudaMemcpy(a.pxm, pxm, n * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(a.pv, pv, n * sizeof(int4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(a.pfe, pFE, n * 16 * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(a.pfp, pFP, n * 16 * sizeof(float), cudaMemcpyHostToDevice));
    for (int4* acc : {a.pvn, a.pd0, a.pd1, a.pd2}) CK(cudaMemset(acc, 0, n * sizeof(int4)));
    s->uploaded = true;
    return SNOW_OK;
  }
  std::vector<float4> xm(n), vv(n), fa(n), fb(n);
  std::vector<float2> fc(n);
  for (size_t i = 0; i < n; i++) {
    xm[i] = make_float4(pxm[4 * i], pxm[4 * i + 1], pxm[4 * i + 2], pxm[4 * i + 3]);
    vv[i] = make_float4((float)pv[4 * i] * 1e-8f, (float)pv[4 * i + 1] * 1e-8f, (float)pv[4 * i + 2] * 1e-8f, 0.0f);
    const float* F = pFE + 16 * i;  // column-major mat4: m[c][r] at 4c + r
    float Fp[9];
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) Fp[3 * r + c] = pFP[16 * i + 4 * c + r];
    fa[i] = make_float4(F[0], F[1], F[2], F[4]);
    fb[i] = make_float4(F[5], F[6], F[8], F[9]);
    fc[i] = make_float2(F[10], (float)det_rowmajor(Fp));
  }
  s->sd.n = (int)n;
  st = fast_upload_soa(s, xm, vv, fa, fb, fc);
  if (st) return st;
  s->uploaded = true;
  return SNOW_OK;
}

snow_status snow_scene_set_volume(snow_scene* s, const float* volume, size_t n) {
  if (!s || !volume) return SNOW_EINVAL;
  snow_ctx* ctx = s->ctx;
  if (!s->uploaded || n != s->n) return fail(ctx, SNOW_ESTATE, "snow_scene_set_volume needs an upload of n particles");
  if (s->mode == SNOW_MODE_REFERENCE) {
    // density rho0 = m / V0, stored as int(rho0 * 1e6) in pv.w
    std::vector<float4> pxm(n);
    std::vector<int4> pv(n);
    RefArgs& a = ref_args(s);
    CK(cudaMemcpy(pxm.data(), a.pxm, n * sizeof(float4), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(pv.data(), a.pv, n * sizeof(int4), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; i++) pv[i].w = volume[i] > 0.0f ? (int)(pxm[i].w / volume[i] * 1e6f) : 0;
    CK(cudaMemcpy(a.pv, pv.data(), n * sizeof(int4), cudaMemcpyHostToDevice));
  } else {
    std::vector<float4> vv(n);
    std::vector<uint32_t> pid(n);
    CK(cudaMemcpy(vv.data(), s->sd.vv, n * sizeof(float4), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(pid.data(), s->sd.pid, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; i++) vv[i].w = volume[pid[i]];
    CK(cudaMemcpy(s->sd.vv, vv.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
  }
  s->volume_given = true;
  return SNOW_OK;
}

snow_status snow_scene_init(snow_scene* s) {
  if (!s) return SNOW_EINVAL;
  snow_ctx* ctx = s->ctx;
  if (!s->uploaded) return fail(ctx, SNOW_ESTATE, "snow_scene_init before upload");
  if (s->mode == SNOW_MODE_REFERENCE) {
    RefArgs& a = ref_args(s);
    ref_reset(a, ctx->stream);
    ref_p2g(a, true, ctx->stream);
    if (!s->volume_given) ref_volume(a, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));
  } else {
    snow_status st = fast_init(s);
    if (st) return st;
  }
  s->initialized = true;
  return SNOW_OK;
}

snow_status snow_dispatch(snow_scene* s, int kernel, double dt) {
  if (!s) return SNOW_EINVAL;
  snow_ctx* ctx = s->ctx;
  if (!(dt >= 0.0) || !std::isfinite(dt)) return fail(ctx, SNOW_EINVAL, "snow_dispatch: dt must be finite and >= 0");
  if (!s->uploaded) return fail(ctx, SNOW_ESTATE, "dispatch before upload");
  const float fdt = (float)dt;  // glUniform1f of the double dt
  cudaStream_t st = ctx->stream;
  if (s->mode == SNOW_MODE_REFERENCE) {
    RefArgs& a = ref_args(s);
    switch (kernel) {
      case SNOW_K_RIGID_ADVANCE: ref_rigid(s->coll_d, s->ncoll, fdt, st); break;
      case SNOW_K_G_RESET: ref_reset(a, st); break;
      case SNOW_K_P2G: ref_p2g(a, false, st); break;
      case SNOW_K_G_FORCE: ref_grid(a, fdt, st); break;
      case SNOW_K_G2P: ref_g2p(a, st); break;
      case SNOW_K_P_ADVANCE: ref_advance(a, fdt, st); break;
      case SNOW_K_G_MASS: ref_p2g(a, true, st); break;
      case SNOW_K_P_VOLUME: ref_volume(a, st); break;
      default: return fail(ctx, SNOW_EINVAL, "unknown kernel");
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    return SNOW_OK;
  }
  if (!s->initialized && kernel != SNOW_K_G_MASS && kernel != SNOW_K_P_VOLUME && kernel != SNOW_K_RIGID_ADVANCE)
    return fail(ctx, SNOW_ESTATE, "dispatch before init");
  snow_status r = set_dt(s, fdt);
  if (r) return r;
  switch (kernel) {
    case SNOW_K_RIGID_ADVANCE:
      if (s->ncoll > 0) fast_begin_step(s->sd_dev, 1, true, st);
      break;
    case SNOW_K_G_RESET:  // discard pending P2G sums
      if (s->p2g_ready) {
        fast_enqueue_compact(s, st);
        fast_enqueue_grid(s, true, st);
        s->p2g_ready = false;
      }
      break;
    case SNOW_K_P2G:
      if (s->p2g_ready) {
        fast_enqueue_compact(s, st);
        fast_enqueue_grid(s, true, st);
      }
      if (s->steps_since_sort >= s->bin_interval) {
        fast_bin(s, st, false);
        s->steps_since_sort = 0;
      }
      fast_enqueue_p2g(s, false, st);
      s->p2g_ready = true;
      break;
    case SNOW_K_G_FORCE:
      fast_enqueue_compact(s, st);
      fast_enqueue_grid(s, false, st);
      fast_enqueue_solve(s, st);
      s->p2g_ready = false;
      break;
    case SNOW_K_G2P:
      fast_g2p_advance(s->sd_dev, s->d_prefix + 0, 1, item_ctas(s->tune), st);
      s->steps_since_sort++;
      break;
    case SNOW_K_P_ADVANCE: break;
    case SNOW_K_G_MASS:
    case SNOW_K_P_VOLUME: return snow_scene_init(s);
    default: return fail(ctx, SNOW_EINVAL, "unknown kernel");
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  return SNOW_OK;
}

snow_status snow_scene_step(snow_scene* s, double dt, int n_steps) {
  if (!s || n_steps < 0) return SNOW_EINVAL;
  snow_ctx* ctx = s->ctx;
  if (!(dt >= 0.0) || !std::isfinite(dt)) return fail(ctx, SNOW_EINVAL, "snow_scene_step: dt must be finite and >= 0");
  if (!s->initialized) return fail(ctx, SNOW_ESTATE, "snow_scene_step before snow_scene_init");
  const float fdt = (float)dt;
  cudaStream_t st = ctx->stream;
  s->last_dt = fdt;
  if (s->mode == SNOW_MODE_REFERENCE) {
    RefArgs& a = ref_args(s);
    for (int i = 0; i < n_steps; i++) {
      ref_rigid(s->coll_d, s->ncoll, fdt, st);
      ref_reset(a, st);
      ref_p2g(a, false, st);
      ref_grid(a, fdt, st);
      ref_g2p(a, st);
      ref_advance(a, fdt, st);
    }
    CK(cudaGetLastError());
    return SNOW_OK;
  }
  snow_status r = set_dt(s, fdt);
  if (r) return r;
  if (!s->p2g_ready) {
    // after per-kernel dispatches: bin and scatter the current state first
    fast_bin(s, st, false);
    s->steps_since_sort = 0;
    fast_enqueue_p2g(s, false, st);
    s->p2g_ready = true;
  }
  for (int i = 0; i < n_steps; i++) {
    const bool bin = s->steps_since_sort >= s->bin_interval;
    if (bin) {
      // binning points are where the host looks at the device counters
      r = fast_check_async(s, std::min(s->steps_since_sort, 1 << 20));
      if (r) return r;
    }
    if (ctx->profiling) {
      cudaEvent_t* ev = ctx->ev;
      CK(cudaEventRecord(ev[0], st));
      fast_begin_step(s->sd_dev, 1, s->ncoll > 0, st);
      if (bin) fast_bin(s, st, true);
      CK(cudaEventRecord(ev[1], st));
      fast_enqueue_compact(s, st, true);
      fast_enqueue_grid(s, false, st);
      CK(cudaEventRecord(ev[2], st));
      fast_enqueue_solve(s, st);
      CK(cudaEventRecord(ev[3], st));
      fast_g2p2g(s->sd_dev, s->d_prefix + 0, 1, item_ctas(s->tune), bin, st);
      CK(cudaEventRecord(ev[4], st));
      CK(cudaEventSynchronize(ev[4]));
      float t[4];
      for (int k = 0; k < 4; k++) cudaEventElapsedTime(&t[k], ev[k], ev[k + 1]);
      s->times.sort_ms += t[0];
      s->times.grid_ms += t[1];
      s->times.other_ms += t[2];  // the semi-implicit solve
      s->times.g2p_ms += t[3];
      s->times.total_ms += t[0] + t[1] + t[2] + t[3];
      s->times.steps++;
    } else if (!ctx->graphs) {
      fast_enqueue_step(s, bin, st);
    } else {
      cudaGraphExec_t& g = bin ? s->g_sort : s->g_plain;
      if (!g || s->g_dt != fdt) {
        if (s->g_dt != fdt) drop_graphs(s);
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        fast_enqueue_step(s, bin, st);
        CK(cudaStreamEndCapture(st, &graph));
        CK(cudaGraphInstantiate(&g, graph, 0));
        cudaGraphDestroy(graph);
        s->g_dt = fdt;
      }
      CK(cudaGraphLaunch(g, st));
    }
    if (bin) {
      s->steps_since_sort = 0;
      s->times.binnings++;
    }
    s->steps_since_sort++;
  }
  CK(cudaGetLastError());
  return SNOW_OK;
}

snow_status snow_scene_download(snow_scene* s, float* x, float* v, float* FE, float* FP, float* Jp, float* volume) {
  if (!s) return SNOW_EINVAL;
  snow_ctx* ctx = s->ctx;
  const size_t n = s->n;
  CK(cudaStreamSynchronize(ctx->stream));
  if (s->mode == SNOW_MODE_REFERENCE) {
    std::vector<float4> pxm(n), pfe(4 * n), pfp(4 * n);
    std::vector<int4> pv(n);
    RefArgs& a = ref_args(s);
    CK(cudaMemcpy(pxm.data(), a.pxm, n * sizeof(float4), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(pv.data(), a.pv, n * sizeof(int4), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(pfe.data(), a.pfe, 4 * n * sizeof(float4), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(pfp.data(), a.pfp, 4 * n * sizeof(float4), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; i++) {
      const float* fe = &pfe[4 * i].x;
      const float* fp = &pfp[4 * i].x;
      float fpr[9];
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
          if (FE) FE[9 * i + 3 * r + c] = fe[4 * c + r];
          fpr[3 * r + c] = fp[4 * c + r];
          if (FP) FP[9 * i + 3 * r + c] = fpr[3 * r + c];
        }
      if (x) {
        x[3 * i] = pxm[i].x;
        x[3 * i + 1] = pxm[i].y;
        x[3 * i + 2] = pxm[i].z;
      }
      if (v) {
        v[3 * i] = (float)pv[i].x * 1e-8f;
        v[3 * i + 1] = (float)pv[i].y * 1e-8f;
        v[3 * i + 2] = (float)pv[i].z * 1e-8f;
      }
      if (Jp) Jp[i] = (float)det_rowmajor(fpr);
      if (volume) {
        const float rho = (float)pv[i].w * 1e-6f;
        volume[i] = rho > 0.0f ? pxm[i].w / rho : 0.0f;
      }
    }
    return SNOW_OK;
  }
  if (FP) return fail(ctx, SNOW_EUNSUPPORTED, "F_P is not kept in SNOW_MODE_FAST (J_p is)");
  if (n == 0) return SNOW_OK;
  // unpacked on the device into upload order in a staging buffer, then one
  // copy per requested array into the caller's memory (a DMA when it is
  // pinned; the unpack kernel writing pinned memory directly was 6x slower:
  // its per-particle stores cross the CPU-GPU link in small pieces; the
  // copies spread over several streams were no faster than in one)
  if (!x && !v && !FE && !Jp && !volume) return SNOW_OK;
  float* out[5] = {x, v, FE, Jp, volume};
  const size_t width[5] = {3, 3, 9, 1, 1};
  float* dev[5] = {};
  size_t words = 0;
  for (int k = 0; k < 5; k++)
    if (out[k]) words += width[k] * n;
  std::vector<std::pair<void*, size_t>> tmp;
  size_t tmp_bytes = 0;
  float* stage = nullptr;
  snow_status st = dalloc(ctx, tmp, tmp_bytes, words * sizeof(float), (void**)&stage);
  if (st) return st;
  for (int k = 0; k < 5; k++) {
    if (!out[k]) continue;
    dev[k] = stage;
    stage += width[k] * n;
  }
  fast_unpack(s->sd_dev, n, dev[0], dev[1], dev[2], dev[3], dev[4], ctx->stream);
  cudaError_t e = cudaGetLastError();
  for (int k = 0; k < 5 && e == cudaSuccess; k++)
    if (out[k])
      e = cudaMemcpyAsync(out[k], dev[k], width[k] * n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  dfree_all(ctx, tmp, tmp_bytes);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "snow_scene_download");
  return SNOW_OK;
}

snow_status snow_scene_download_std140(snow_scene* s, float* pxm, int32_t* pv, float* pFE, float* pFP) {
  if (!s) return SNOW_EINVAL;
  snow_ctx* ctx = s->ctx;
  if (s->mode != SNOW_MODE_REFERENCE) return fail(ctx, SNOW_EUNSUPPORTED, "std140 download needs SNOW_MODE_REFERENCE");
  const size_t n = s->n;
  CK(cudaStreamSynchronize(ctx->stream));
  RefArgs& a = ref_args(s);
  if (pxm) CK(cudaMemcpy(pxm, a.pxm, n * sizeof(float4), cudaMemcpyDeviceToHost));
  if (pv) CK(cudaMemcpy(pv, a.pv, n * sizeof(int4), cudaMemcpyDeviceToHost));
  if (pFE) CK(cudaMemcpy(pFE, a.pfe, n * 16 * sizeof(float), cudaMemcpyDeviceToHost));
  if (pFP) CK(cudaMemcpy(pFP, a.pfp, n * 16 * sizeof(float), cudaMemcpyDeviceToHost));
  return SNOW_OK;
}

snow_status snow_scene_download_grid(snow_scene* s, float* mass, float* momentum, float* force, float* vstar) {
  if (!s) return SNOW_EINVAL;
  snow_ctx* ctx = s->ctx;
  CK(cudaStreamSynchronize(ctx->stream));
  const size_t G = (size_t)s->G;
  if (s->mode == SNOW_MODE_REFERENCE) {
    std::vector<int4> gv(G), gf(G);
    std::vector<float4> gvn(G);
    RefArgs& a = ref_args(s);
    CK(cudaMemcpy(gv.data(), a.gv, G * sizeof(int4), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(gf.data(), a.gf, G * sizeof(int4), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(gvn.data(), a.gvn, G * sizeof(float4), cudaMemcpyDeviceToHost));
    for (size_t g = 0; g < G; g++) {
      if (mass) mass[g] = (float)gv[g].w * 1e-8f;
      const float pm[3] = {(float)gv[g].x * 1e-8f, (float)gv[g].y * 1e-8f, (float)gv[g].z * 1e-8f};
      const float fo[3] = {(float)gf[g].x * 1e-6f, (float)gf[g].y * 1e-6f, (float)gf[g].z * 1e-6f};
      const float vs[3] = {gvn[g].x, gvn[g].y, gvn[g].z};
      for (int k = 0; k < 3; k++) {
        if (momentum) momentum[3 * g + k] = pm[k];
        if (force) force[3 * g + k] = fo[k];
        if (vstar) vstar[3 * g + k] = vs[k];
      }
    }
    return SNOW_OK;
  }
  float *dm = nullptr, *dp = nullptr, *df = nullptr, *dv = nullptr;
  std::vector<std::pair<void*, size_t>> tmp;
  size_t tb = 0;
  snow_status r;
  if ((r = dalloc(ctx, tmp, tb, G * sizeof(float), (void**)&dm)) || (r = dalloc(ctx, tmp, tb, 3 * G * sizeof(float), (void**)&dp)) ||
      (r = dalloc(ctx, tmp, tb, 3 * G * sizeof(float), (void**)&df)) || (r = dalloc(ctx, tmp, tb, 3 * G * sizeof(float), (void**)&dv))) {
    dfree_all(ctx, tmp, tb);
    return r;
  }
  cudaMemsetAsync(dm, 0, G * sizeof(float), ctx->stream);
  cudaMemsetAsync(dp, 0, 3 * G * sizeof(float), ctx->stream);
  cudaMemsetAsync(df, 0, 3 * G * sizeof(float), ctx->stream);
  cudaMemsetAsync(dv, 0, 3 * G * sizeof(float), ctx->stream);
  fast_download_grid(s->sd_dev, dm, dp, df, dv, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess && mass) e = cudaMemcpy(mass, dm, G * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && momentum) e = cudaMemcpy(momentum, dp, 3 * G * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && force) e = cudaMemcpy(force, df, 3 * G * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && vstar) e = cudaMemcpy(vstar, dv, 3 * G * sizeof(float), cudaMemcpyDeviceToHost);
  dfree_all(ctx, tmp, tb);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "grid download");
  return SNOW_OK;
}

snow_status snow_scene_download_colliders(snow_scene* s, snow_collider* out) {
  if (!s || !out) return SNOW_EINVAL;
  snow_ctx* ctx = s->ctx;
  CK(cudaStreamSynchronize(ctx->stream));
  if (s->ncoll > 0) CK(cudaMemcpy(out, s->coll_d, s->ncoll * sizeof(snow_collider), cudaMemcpyDeviceToHost));
  return SNOW_OK;
}

static snow_status stats_enqueue(snow_scene* s, int k) {
  snow_ctx* ctx = s->ctx;
  if (s->mode == SNOW_MODE_REFERENCE)
    ref_stats(ref_args(s), ctx->d_stats + k, ctx->d_hstats + k, ctx->stream);
  else
    fast_stats(s->sd_dev, (int)s->n, ctx->d_stats + k, ctx->d_hstats + k, ctx->stream);
  CK(cudaGetLastError());
  return SNOW_OK;
}

static void stats_convert(const StatsAccum& a, size_t n, snow_stats* out) {
  std::memset(out, 0, sizeof *out);
  out->mass = a.mass;
  for (int k = 0; k < 3; k++) {
    out->momentum[k] = a.mom[k];
    out->center_of_mass[k] = a.mass > 0 ? a.com[k] / a.mass : 0.0;
    const int kmin = a.bmin_key[k] >= 0 ? a.bmin_key[k] : a.bmin_key[k] ^ 0x7fffffff;
    const int kmax = a.bmax_key[k] >= 0 ? a.bmax_key[k] : a.bmax_key[k] ^ 0x7fffffff;
    float fmin, fmax;
    std::memcpy(&fmin, &kmin, 4);
    std::memcpy(&fmax, &kmax, 4);
    out->bbox_min[k] = fmin;
    out->bbox_max[k] = fmax;
  }
  out->kinetic_energy = a.ke;
  out->nonfinite = a.nonfinite;
  out->n = n;
  out->mean_jp = n > a.nonfinite ? a.jp / (double)(n - a.nonfinite) : 0.0;
}

snow_status snow_scene_stats(snow_scene* s, snow_stats* out) {
  if (!s || !out) return SNOW_EINVAL;
  snow_ctx* ctx = s->ctx;
  snow_status r = stats_enqueue(s, 0);
  if (r) return r;
  CK(cudaStreamSynchronize(ctx->stream));
  stats_convert(ctx->h_stats[0], s->n, out);
  return SNOW_OK;
}

snow_status snow_scene_stats_enqueue(snow_scene* s, int slot) {
  if (!s || slot < 0 || slot >= SNOW_STATS_SLOTS) return fail(s ? s->ctx : nullptr, SNOW_EINVAL, "stats slot");
  snow_ctx* ctx = s->ctx;
  if (ctx->stat_pending[slot]) CK(cudaEventSynchronize(ctx->stat_ev[slot]));  // reusing an unread slot
  snow_status r = stats_enqueue(s, 1 + slot);
  if (r) return r;
  CK(cudaEventRecord(ctx->stat_ev[slot], ctx->stream));
  ctx->stat_n[slot] = s->n;
  ctx->stat_pending[slot] = true;
  return SNOW_OK;
}

snow_status snow_ctx_stats_read(snow_ctx* ctx, int slot, snow_stats* out) {
  if (!ctx || !out || slot < 0 || slot >= SNOW_STATS_SLOTS) return fail(ctx, SNOW_EINVAL, "stats slot");
  if (!ctx->stat_pending[slot]) return fail(ctx, SNOW_ESTATE, "no statistics queued in this slot");
  CK(cudaEventSynchronize(ctx->stat_ev[slot]));
  ctx->stat_pending[slot] = false;
  stats_convert(ctx->h_stats[1 + slot], ctx->stat_n[slot], out);
  return SNOW_OK;
}

snow_status snow_scene_cell_keys(snow_scene* s, uint32_t* keys, uint32_t* perm) {
  if (!s || !keys) return SNOW_EINVAL;
  snow_ctx* ctx = s->ctx;
  if (s->mode != SNOW_MODE_FAST) return fail(ctx, SNOW_EUNSUPPORTED, "binning runs in SNOW_MODE_FAST");
  const size_t n = s->n;
  cudaStream_t st = ctx->stream;
  // keys of the current positions, then placed at each particle's upload
  // index so the stable sort sees the caller's order
  fast_sort_keys(s->sd, s->sd_dev, s->bin, 0, st);  // keys only (0 bits: no passes)
  std::vector<uint32_t> k(n), pid(n);
  CK(cudaMemcpyAsync(k.data(), s->bin.keys[0], n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(pid.data(), s->sd.pid, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  std::vector<uint32_t> ko(n), vo(n);
  for (size_t i = 0; i < n; i++) {
    ko[pid[i]] = k[i];
    vo[i] = (uint32_t)i;
  }
  std::memcpy(keys, ko.data(), n * sizeof(uint32_t));
  if (perm) {
    CK(cudaMemcpyAsync(s->bin.keys[0], ko.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->bin.vals[0], vo.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    radix_sort_pairs(s->bin.keys, s->bin.vals, n, s->key_bits, s->bin.hist, s->bin.scan_tmp, st);
    CK(cudaMemcpyAsync(perm, s->bin.vals[0], n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  CK(cudaGetLastError());
  return SNOW_OK;
}

snow_status snow_scene_phase_times(snow_scene* s, snow_phase_times* out, int reset) {
  if (!s || !out) return SNOW_EINVAL;
  *out = s->times;
  if (s->mode == SNOW_MODE_FAST && s->sd.fix) {  // the device's cumulative count, relative to the last reset
    snow_ctx* ctx = s->ctx;
    uint32_t wide = 0;
    CK(cudaMemcpyAsync(&wide, &s->sd.fix->wide, sizeof wide, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    out->wide = (uint32_t)(wide - s->wide_base);
    if (reset) s->wide_base = wide;
  }
  if (reset) s->times = snow_phase_times{};
  return SNOW_OK;
}

snow_status snow_scene_set_wait_limit(snow_scene* s, uint32_t wait_ns, uint32_t unsent_bytes) {
  if (!s) return SNOW_EINVAL;
  snow_ctx* ctx = s->ctx;
  if (s->mode != SNOW_MODE_FAST) return fail(ctx, SNOW_EUNSUPPORTED, "bounded copy waits are FAST-mode kernels'");
  if (unsent_bytes > 65536) return fail(ctx, SNOW_EINVAL, "snow_scene_set_wait_limit: unsent_bytes above 65536");
  s->wait_ns = wait_ns ? wait_ns : kDefaultWaitNs;
  s->tx_unsent = unsent_bytes;
  s->sd.wait_ns = s->wait_ns;
  s->sd.tx_unsent = s->tx_unsent;
  if (!s->sd_dev) return SNOW_OK;  // not allocated yet: the first upload pushes the descriptor
  return push_sd(s);
}

snow_status snow_scene_check(snow_scene* s) {
  if (!s) return SNOW_EINVAL;
  snow_ctx* ctx = s->ctx;
  if (s->mode != SNOW_MODE_FAST) {
    CK(cudaStreamSynchronize(ctx->stream));
    return SNOW_OK;
  }
  return fast_check(s);
}

snow_status snow_scene_solver_report(snow_scene* s, snow_solver_report* out) {
  if (!s || !out) return SNOW_EINVAL;
  snow_ctx* ctx = s->ctx;
  if (!s->sd.crs) return fail(ctx, SNOW_EUNSUPPORTED, "the scene steps explicitly");
  CrScalars c;
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(&c, s->sd.crs, sizeof c, cudaMemcpyDeviceToHost));
  out->iterations = c.iters;
  out->max_iters = s->sd.imp_maxit;
  out->initial_residual = c.bb > 0.0 ? std::sqrt(c.rr[0] / c.bb) : 0.0;
  out->residual = c.bb > 0.0 ? std::sqrt(c.rr[c.iters] / c.bb) : 0.0;
  return SNOW_OK;
}

// ---- batches ----------------------------------------------------------------
snow_status snow_batch_create(snow_ctx* ctx, snow_scene* const* scenes, int n, snow_batch** out) {
  if (!ctx || !scenes || n <= 0 || !out) return fail(ctx, SNOW_EINVAL, "snow_batch_create: invalid argument");
  *out = nullptr;
  for (int i = 0; i < n; i++)
    if (!scenes[i] || scenes[i]->mode != SNOW_MODE_FAST || !scenes[i]->initialized || scenes[i]->ctx != ctx)
      return fail(ctx, SNOW_EINVAL, "batch scenes must be initialised SNOW_MODE_FAST scenes of this context");
  snow_batch* b = new snow_batch();
  b->ctx = ctx;
  b->scenes.assign(scenes, scenes + n);
  snow_status st;
  if ((st = dalloc(ctx, b->allocs, b->bytes, sizeof(SceneDev) * n, (void**)&b->d_scenes)) ||
      (st = dalloc(ctx, b->allocs, b->bytes, sizeof(int) * 4 * (n + 1), (void**)&b->d_prefix))) {
    snow_batch_destroy(b);
    return st;
  }
  if (cudaHostAlloc(&b->h_cnt, sizeof(int) * kCounterStride * n, cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer((void**)&b->d_hcnt, b->h_cnt, 0) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->cnt_ev, cudaEventDisableTiming) != cudaSuccess) {
    st = cuda_fail(ctx, cudaGetLastError(), "batch counter snapshot");
    snow_batch_destroy(b);
    return st;
  }
  ctx->batches.insert(b);
  *out = b;
  return SNOW_OK;
}

void snow_batch_destroy(snow_batch* b) {
  if (!b) return;
  cudaStreamSynchronize(b->ctx->stream);
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.second);
  dfree_all(b->ctx, b->allocs, b->bytes);
  if (b->h_cnt) cudaFreeHost(b->h_cnt);
  if (b->cnt_ev) cudaEventDestroy(b->cnt_ev);
  b->ctx->batches.erase(b);
  delete b;
}

namespace {

snow_status batch_refresh(snow_batch* b, const double* dt) {
  snow_ctx* ctx = b->ctx;
  const int n = (int)b->scenes.size();
  bool changed = (int)b->versions.size() != n;
  std::vector<float> want(n);
  for (int i = 0; i < n; i++) {
    snow_scene* s = b->scenes[i];
    want[i] = dt ? (float)dt[i] : s->last_dt;
    if (!changed && b->versions[i] != s->version) changed = true;
  }
  if (want != b->g_dt) changed = true;
  if (!changed) return SNOW_OK;
  std::vector<SceneDev> sds(n);
  std::vector<int> pre(4 * (n + 1), 0);
  long long blocks = 0;
  for (int i = 0; i < n; i++) {
    snow_scene* s = b->scenes[i];
    s->sd.dt = want[i];
    s->last_dt = want[i];
    sds[i] = s->sd;
    pre[3 * (n + 1) + i] = (int)blocks;
    blocks += s->sd.nblocks;
  }
  pre[3 * (n + 1) + n] = (int)blocks;
  b->total_blocks = blocks;
  CK(cudaMemcpyAsync(b->d_scenes, sds.data(), sizeof(SceneDev) * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(b->d_prefix, pre.data(), sizeof(int) * pre.size(), cudaMemcpyHostToDevice, ctx->stream));
  for (int i = 0; i < n; i++) {
    snow_scene* s = b->scenes[i];
    CK(cudaMemcpyAsync(s->sd_dev, &s->sd, sizeof(SceneDev), cudaMemcpyHostToDevice, ctx->stream));
    drop_graphs(s);
    s->version++;
  }
  CK(cudaStreamSynchronize(ctx->stream));
  b->versions.resize(n);
  for (int i = 0; i < n; i++) b->versions[i] = b->scenes[i]->version;
  b->g_dt = want;
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.second);
  b->graphs.clear();
  return SNOW_OK;
}

void batch_enqueue_step(snow_batch* b, bool bin_all, cudaStream_t st) {
  const int n = (int)b->scenes.size();
  int* pre = b->d_prefix;
  int* items = pre;
  int* active = pre + (n + 1);
  int* blocks = pre + 3 * (n + 1);
  fast_begin_step(b->d_scenes, n, true, st);
  // every scene re-binned in the same step, every sort_interval steps, so
  // the other steps run the fused kernel's plain instantiation (re-binning a
  // staggered subset of the scenes each step made every step take the
  // binned one: 3% slower on 16 scenes of 2M-8M particles and on 64 of
  // 10k-500k, A/B on one GPU); the scenes' binnings are independent, so they
  // run on side streams (parallel branches of the step's graph) and join
  // before the compaction
  std::vector<int> bins;
  if (bin_all)
    for (int i = 0; i < n; i++) bins.push_back(i);
  snow_ctx* ctx = b->ctx;
  if (bins.size() < 2) {
    for (int i : bins) fast_bin(b->scenes[i], st, true);
  } else {
    const int lanes = std::min((int)bins.size(), (int)snow_ctx::kAux);
    cudaEventRecord(ctx->fork_ev, st);
    for (int k = 0; k < lanes; k++) cudaStreamWaitEvent(ctx->aux[k], ctx->fork_ev, 0);
    for (size_t k = 0; k < bins.size(); k++) fast_bin(b->scenes[bins[k]], ctx->aux[k % lanes], true);
    for (int k = 0; k < lanes; k++) {
      cudaEventRecord(ctx->join_ev[k], ctx->aux[k]);
      cudaStreamWaitEvent(st, ctx->join_ev[k], 0);
    }
  }
  fast_compact(b->d_scenes, blocks, n, b->total_blocks, items, active, st);
  fast_grid(b->d_scenes, active, n, grid_ctas(), false, st);
  int iters = 0;  // the solve runs while any semi-implicit scene still iterates
  for (snow_scene* s : b->scenes)
    if (s->sd.crs) iters = std::max(iters, s->sd.imp_maxit);
  if (iters > 0)
    fast_implicit_solve(b->d_scenes, items, active, n, iters, item_ctas(b->scenes[0]->tune), grid_ctas(),
                        b->ctx->d_iter, b->ctx->body_stream, b->ctx->gate_stream, st);
  fast_g2p2g(b->d_scenes, items, n, item_ctas(b->scenes[0]->tune), !bins.empty(), st);
}

}  // namespace

snow_status snow_batch_step(snow_batch* b, const double* dt, int n_steps) {
  if (!b || n_steps < 0) return SNOW_EINVAL;
  snow_ctx* ctx = b->ctx;
  if (dt)
    for (size_t i = 0; i < b->scenes.size(); i++)
      if (!(dt[i] >= 0.0) || !std::isfinite(dt[i])) return fail(ctx, SNOW_EINVAL, "snow_batch_step: bad dt");
  cudaStream_t st = ctx->stream;
  for (size_t i = 0; i < b->scenes.size(); i++) {
    snow_scene* s = b->scenes[i];
    if (s->p2g_ready) continue;  // left behind by per-kernel dispatches: scatter its state first
    snow_status r0 = set_dt(s, dt ? (float)dt[i] : s->last_dt);
    if (r0) return r0;
    fast_bin(s, st, false);
    s->steps_since_sort = 0;
    fast_enqueue_p2g(s, false, st);
    s->p2g_ready = true;
  }
  snow_status r = batch_refresh(b, dt);
  if (r) return r;
  const int interval = std::max(1, b->scenes[0]->tune.sort_interval);
  for (int i = 0; i < n_steps; i++) {
    const int phase = b->step_count % interval;
    if (phase == 0 && b->step_count > 0) {
      // the counters gathered at the previous checking point (long landed:
      // no wait for the queued steps), then a new gather for the next one
      if (b->cnt_pending) {
        CK(cudaEventSynchronize(b->cnt_ev));
        b->cnt_pending = false;
        for (size_t k = 0; k < b->scenes.size(); k++) {
          r = check_counters(b->scenes[k], b->h_cnt + k * kCounterStride);
          if (r) return r;
        }
      }
      fast_gather_counters(b->d_scenes, (int)b->scenes.size(), b->d_hcnt, st);
      CK(cudaEventRecord(b->cnt_ev, st));
      b->cnt_pending = true;
      r = batch_refresh(b, dt);
      if (r) return r;
    }
    const int key = phase == 0 ? 0 : 1;  // a step that re-bins every scene, or none
    auto it = b->graphs.find(key);
    if (it == b->graphs.end()) {
      cudaGraph_t graph;
      cudaGraphExec_t exec;
      CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      batch_enqueue_step(b, phase == 0, st);
      CK(cudaStreamEndCapture(st, &graph));
      CK(cudaGraphInstantiate(&exec, graph, 0));
      cudaGraphDestroy(graph);
      it = b->graphs.emplace(key, exec).first;
    }
    CK(cudaGraphLaunch(it->second, st));
    b->step_count++;
  }
  for (snow_scene* s : b->scenes) s->steps_since_sort = 1;  // single-scene stepping re-bins on its own schedule
  CK(cudaGetLastError());
  return SNOW_OK;
}

static bool valid_tuning(const snow_tuning* t) {
  return t && t->sort_interval >= 1 && t->sort_interval <= 64 && t->items_max >= kMinItemMax && t->items_max <= 256 &&
         (t->ctas_per_sm == 1 || t->ctas_per_sm == 2);
}

snow_status snow_scene_set_tuning(snow_scene* s, const snow_tuning* t) {
  if (!s || !valid_tuning(t)) return fail(s ? s->ctx : nullptr, SNOW_EINVAL, "snow_scene_set_tuning: invalid tuning");
  if (s->mode != SNOW_MODE_FAST) return fail(s->ctx, SNOW_EUNSUPPORTED, "tuning applies to SNOW_MODE_FAST scenes");
  snow_ctx* ctx = s->ctx;
  CK(cudaStreamSynchronize(ctx->stream));
  // the captured step graphs bake in the launch shapes: a changed work split
  // needs new ones
  const bool split_changed = s->tune.items_max != t->items_max || s->tune.ctas_per_sm != t->ctas_per_sm;
  s->tune.sort_interval = t->sort_interval;
  s->tune.items_max = t->items_max;
  s->tune.ctas_per_sm = t->ctas_per_sm;
  s->bin_interval = t->sort_interval;
  s->clean_checks = 0;
  // the next step re-bins with the new work split
  if (s->p2g_ready) s->steps_since_sort = s->bin_interval;
  if (split_changed) drop_graphs(s);
  return SNOW_OK;
}

snow_status snow_batch_set_tuning(snow_batch* b, const snow_tuning* t) {
  if (!b || !valid_tuning(t)) return fail(b ? b->ctx : nullptr, SNOW_EINVAL, "snow_batch_set_tuning: invalid tuning");
  snow_ctx* ctx = b->ctx;
  CK(cudaStreamSynchronize(ctx->stream));
  for (snow_scene* s : b->scenes) {
    s->tune.sort_interval = t->sort_interval;
    s->tune.items_max = t->items_max;
    s->tune.ctas_per_sm = t->ctas_per_sm;
    s->bin_interval = t->sort_interval;
    drop_graphs(s);
  }
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.second);
  b->graphs.clear();
  b->step_count = 0;
  return SNOW_OK;
}

// Times each candidate (sort interval x particles per work item x CTAs per
// SM) over real steps of the batch -- one sort interval to re-bin every scene
// with the candidate's work items and capture its graphs, then two intervals
// (at least 32 steps) timed with events -- and keeps the fastest. The scenes
// evolve while the candidates run, so the cost of a step drifts; every
// candidate is timed twice, once in a forward and once in a reversed pass
// over the list, and the two times are averaged, which cancels a drift that
// is linear in the steps taken.
snow_status snow_batch_autotune(snow_batch* b, const double* dt, snow_tuning* out) {
  if (!b) return SNOW_EINVAL;
  snow_ctx* ctx = b->ctx;
  // 1, 2: particles that cross cells in a step or two; 24, 32: slow particles, binning amortised further
  static const int kIntervals[] = {1, 2, 4, 8, 12, 16, 24, 32};
  static const int kItems[] = {128, 256};
  static const int kCtas[] = {1, 2};
  std::vector<snow_tuning> cand;
  for (int si : kIntervals)
    for (int im : kItems)
      for (int cp : kCtas) cand.push_back(snow_tuning{si, im, cp, 0, 0.0});
  const int nc = (int)cand.size();
  snow_tuning best{};
  best.ms_per_step = 1e30;
  int steps = 0;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  snow_status r = SNOW_OK;
  for (int pass = 0; pass < 2; pass++)
    for (int j = 0; j < nc; j++) {
      snow_tuning& t = cand[pass == 0 ? j : nc - 1 - j];
      const int si = t.sort_interval;
      if ((r = snow_batch_set_tuning(b, &t))) goto done;
      if ((r = snow_batch_step(b, dt, si))) goto done;
      const int k = std::max(32, 2 * si);
      if (cudaEventRecord(e0, ctx->stream) != cudaSuccess) { r = cuda_fail(ctx, cudaGetLastError(), "event"); goto done; }
      if ((r = snow_batch_step(b, dt, k))) goto done;
      if (cudaEventRecord(e1, ctx->stream) != cudaSuccess) { r = cuda_fail(ctx, cudaGetLastError(), "event"); goto done; }
      if (cudaEventSynchronize(e1) != cudaSuccess) { r = cuda_fail(ctx, cudaGetLastError(), "event"); goto done; }
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      steps += si + k;
      t.ms_per_step += 0.5 * ms / k;
    }
  for (const snow_tuning& t : cand)
    if (t.ms_per_step < best.ms_per_step) best = t;
  r = snow_batch_set_tuning(b, &best);
done:
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (r) return r;
  for (snow_scene* s : b->scenes) {
    r = fast_check(s);
    if (r) return r;
  }
  best.steps_taken = steps;
  if (out) *out = best;
  return SNOW_OK;
}

}  // extern "C"

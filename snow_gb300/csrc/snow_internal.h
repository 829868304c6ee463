// Internal interfaces between the host runtime (snow_api.cpp) and the CUDA
// kernel files (ref_kernels.cu, fast_kernels.cu, sort.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/snow_mpm.h"

namespace snow {

// ---------------------------------------------------------------------------
// Reference mode: the shaders' buffers, byte for byte (std140).
// ---------------------------------------------------------------------------
struct RefArgs {
  float gpos[3];
  int dim[3];
  float h;
  float young, poisson, hardening, crit_c, crit_s, alpha;
  float grav[3];
  int ncoll;
  snow_collider* coll;
  int n;
  float4* pxm;   // (x, m)
  int4* pv;      // (v * 1e8, rho0 * 1e6)
  float4* pfe;   // mat4 per particle, 4 columns
  float4* pfp;
  int4* pvn;     // G2P accumulators (g2pTransfer.glsl bindings 6, 13-15)
  int4* pd0;
  int4* pd1;
  int4* pd2;
  long long G;
  int4* gv;      // (p * 1e8, m * 1e8)
  int4* gf;      // (f * 1e6, 0)
  float4* gvn;   // (v*, 0)
};

void ref_rigid(snow_collider* coll, int ncoll, float dt, cudaStream_t st);
void ref_reset(const RefArgs& a, cudaStream_t st);
void ref_p2g(const RefArgs& a, bool mass_only, cudaStream_t st);
void ref_volume(const RefArgs& a, cudaStream_t st);
void ref_grid(const RefArgs& a, float dt, cudaStream_t st);
void ref_g2p(const RefArgs& a, cudaStream_t st);
void ref_advance(const RefArgs& a, float dt, cudaStream_t st);

// ---------------------------------------------------------------------------
// Fast mode.
// ---------------------------------------------------------------------------
constexpr int kBlockNodes = 64;            // 4 x 4 x 4 nodes per grid block
constexpr int kAccFields = 7;              // m, p (3), f (3)
constexpr int kOutFields = 6;              // v* (3), d = v* - alpha p/m (3)
// acc holds the P2G sums as integers (fixed point at per-scene power-of-two
// scales): per node seven int64 words (m, p_x, p_y, p_z, f_x, f_y, f_z),
// stored word-major per block. No node sum can leave the int64 range (each
// contribution is below 2^22 or, on the wide path, 2^62), however many
// particles pile into a cell.
constexpr int kAccWords = kAccFields;
constexpr int kAccBlockWords = kAccWords * kBlockNodes;    // 448 (3584 bytes)
constexpr int kOutBlockFloats = kOutFields * kBlockNodes;  // 384

// Fixed-point state of one scene's P2G sums. Magnitudes are the bits of
// non-negative floats (they order like unsigned ints, so atomicMax records
// maxima); every value here is an order-independent function of the state.
struct FixState {
  float scale[3];     // s_m, s_p, s_f of the sums now in acc (integer = round(contribution * s))
  uint32_t m_prev;    // largest particle mass, |v| and force-term bound a of the particles the
  uint32_t v_prev;    //   previous P2G scattered (a = max over rows r of |A_r0| + |A_r1| + |A_r2|)
  uint32_t a_prev;
  uint32_t m_cur;     // the same, recorded by the P2G in flight (moved to *_prev at each step's start)
  uint32_t v_cur;
  uint32_t a_cur;
  uint32_t v0max;     // largest initial particle volume
  uint32_t wide;      // particles scattered with int64 contributions (outgrew the fast range), cumulative
};

// Per-scene counters (int32), one row of kCounterStride per scene.
enum {
  CNT_ACTIVE = 0,     // active grid blocks this step
  CNT_OVERFLOW = 1,   // blocks that found no slot in the pool
  CNT_ITEMS = 2,      // P2G work items since the last binning
  CNT_NONFINITE = 3,  // particles with a non-finite field (cumulative)
  CNT_HOME = 4,       // occupied home blocks at the last binning
  CNT_FALLBACK = 5,   // particles that left their P2G tile (diagnostic, cumulative)
  CNT_TIMEOUT = 6,    // bounded waits that ran out (cumulative)
  CNT_DONE = 7,       // CTAs of the compaction finished (the last forms the prefixes)
  CNT_BINNED = 8,     // 1: this step's binning left the particles in the binned copies
  kCounterStride = 9
};

// Semi-implicit velocity solve: conjugate residuals on the mass-scaled form
// of (M + beta dt^2 K) v = M v* over the active nodes, one record per scene,
// cleared (up to `skipping`) at the start of each step. Iteration k
// (1-based) forms rAr[k] = (r_{k-1}, A r_{k-1}), ApAp[k] = |A p_{k-1}|^2 and
// rr[k] = |r_k|^2. A step whose initial residual is below
// kCrSkipFactor * tolerance makes the next steps skip the solve: they take
// v = v*, which is what a solve that exits at iteration 0 gives, without
// evaluating K v*; the step after them checks again. The skip lasts
// kCrSkipSteps steps, doubled for each further factor of 10 the residual
// lies below the threshold, up to kCrSkipSteps * 2^kCrSkipDoublings.
constexpr int kCrMaxIters = 128;
constexpr int kCrSkipSteps = 15;
constexpr int kCrSkipDoublings = 4;
constexpr double kCrSkipFactor = 1e-3;
struct CrScalars {
  double bb;                   // |M^1/2 v*|^2
  double rr[kCrMaxIters + 1];  // rr[0]: the initial residual
  double rAr[kCrMaxIters + 1];
  double ApAp[kCrMaxIters + 1];
  int iters;                   // iterations taken
  int skipping;                // 1: this step skips the solve
  int skip_left;               // steps still to skip (kept across steps)
  int pad;
};
constexpr int kImpBlockFloats = 3 * kBlockNodes;  // 192: one 3-vector per node
constexpr uint32_t kDefaultWaitNs = 1000000000u;   // one second

// Device-resident description of one FAST scene (read by every kernel).
struct SceneDev {
  float gpos[3];
  float h;
  float inv_h;  // 1 / h (FAST kernels multiply instead of dividing)
  int dim[3];
  int bdim[3];
  int nblocks;
  float young, poisson, hardening, crit_lo, crit_hi, alpha;
  float mu0, lambda0;  // Lame parameters at J_p = 1 (lame.include.glsl:11-27)
  float grav[3];
  float dt;
  int ncoll;
  snow_collider* coll;
  int n;
  // particle streams (SoA): xm = (x, m), vv = (v, V0),
  // fa = (FE00, FE10, FE20, FE01), fb = (FE11, FE21, FE02, FE12),
  // fc = (FE22, Jp); FE stored column-major (m[c][r]).
  float4* xm;
  float4* vv;
  float4* fa;
  float4* fb;
  float2* fc;
  float4* vq;       // FAST: the Jacobi frame (quaternion) of each particle's last SVD
  uint32_t* pid;    // upload index of the particle now stored at each slot
  // the binning's permuted copies of xm, vv, fa, fb, fc, vq: a binning inside
  // a step leaves the particles there (counters[CNT_BINNED] = 1), and the
  // kernels of that step read them from there until the fused kernel, which
  // writes every particle, has put them back into the streams above
  const float4* bxm;
  const float4* bvv;
  const float4* bfa;
  const float4* bfb;
  const float2* bfc;
  const float4* bvq;
  // blocked grid
  int* blk_slot;    // nblocks: pool slot of the block this step, -1 if inactive
  int* blk_flag;    // nblocks: block received P2G sums since the last compaction
  unsigned long long* acc;  // nblocks x 320 words: the fixed-point P2G sums, word-major per block (dense)
  FixState* fix;            // their scales and the magnitudes the next scales are chosen from
  int* active;      // pool_cap: block id of each slot
  float* gout;      // pool_cap x 384: grid-update output, per node (v*, d) as 6 floats
  int pool_cap;
  // P2G work items: (home block, first particle, count, 0)
  int4* items;
  int item_cap;
  int* counters;    // kCounterStride ints
  // bounded waits for bulk copies into shared memory: give up after wait_ns
  // nanoseconds; tx_unsent (0 in normal use) is added to the bytes each such
  // wait expects, so that it runs out (a test of the timeout path)
  uint32_t wait_ns;
  uint32_t tx_unsent;
  // semi-implicit velocity solve (crs == nullptr: the scene steps explicitly)
  float imp_beta;   // beta of (M + beta dt^2 K) v = M v*
  float imp_tol;    // stop once |r| <= imp_tol |M^1/2 v*| (r of the mass-scaled system)
  int imp_maxit;    // at most this many iterations per step
  float4* crv;      // 3 planes of pool_cap x 64 float4 per node: (v, m), (p, 0), (A p, 0)
  float* cru;       // pool_cap x 192: u = M^-1/2 r (the vector K is applied to), 3 floats per node
  CrScalars* crs;
};

struct FastTuning {
  int sort_interval = 8;  // re-bin particles every k steps
  int items_max = 256;    // most particles per work item (kMinItemMax .. 256)
  int ctas_per_sm = 2;    // work-item CTAs launched per SM (1 or 2)
};
constexpr int kMinItemMax = 64;

// Work spaces over a batch: prefix[s] .. prefix[s+1] are scene s's units
// (P2G work items, active blocks, grid blocks). Item and active-block counts
// are only known on the device; fast_prefix() forms both prefixes there.
void fast_prefix(const SceneDev* scenes, int nscenes, int* items_prefix, int* active_prefix, cudaStream_t st);
// Start of a step: resets the per-step counters and, with `rigid`, moves the
// colliders by dt * velocity (rigidAdvance.glsl:14-18).
void fast_begin_step(const SceneDev* scenes, int nscenes, bool rigid, cudaStream_t st);
// Copies every scene's counters into out[s * kCounterStride ...] (mapped
// pinned memory: a batch reads them one re-binning interval later, without
// draining the stream).
void fast_gather_counters(const SceneDev* scenes, int nscenes, int* out, cudaStream_t st);
// Flags -> active list and pool slots; its last CTA then forms the item and
// active-block prefixes (as fast_prefix does).
void fast_compact(const SceneDev* scenes, const int* block_prefix, int nscenes, long long total_blocks,
                  int* items_prefix, int* active_prefix,
                  cudaStream_t st);
// P2G of the stored particle state (set-up, per-kernel dispatches), after a
// pass over the particles that measures the magnitudes its fixed-point
// scales are chosen from.
void fast_p2g(const SceneDev* scenes, const SceneDev& sd_host, const int* item_prefix, int nscenes, int grid_ctas,
              bool mass_only, cudaStream_t st);
void fast_grid(const SceneDev* scenes, const int* active_prefix, int nscenes, int grid_ctas, bool clear_only,
               cudaStream_t st);
void fast_volume(const SceneDev* sd_dev, int n, cudaStream_t st);
void fast_g2p_advance(const SceneDev* scenes, const int* item_prefix, int nscenes, int grid_ctas, cudaStream_t st);
// binned: some scene of the launch was re-binned in this step (its particles
// are in its binned copies)
void fast_g2p2g(const SceneDev* scenes, const int* item_prefix, int nscenes, int grid_ctas, bool binned,
                cudaStream_t st);
// The semi-implicit velocity solve between the grid update (which leaves
// v*, m and u = v* in the solver planes) and G2P: iterations of conjugate
// residuals (each a K u pass over the items and three passes over the active
// nodes) until every scene has converged or reached its cap, then the
// colliders on v and v, d written back into gout. Scenes without a solver
// record are left alone. d_iter is a device int (the iteration counter).
// When `st` is capturing a graph the whole solve is the body of a
// conditional IF node (captured on `gate`), taken when any scene solves in
// this step, and its iterations a conditional WHILE node inside it (body
// captured on `body`; both streams not otherwise in use); otherwise
// max_iters iterations are launched.
void fast_implicit_solve(const SceneDev* scenes, const int* item_prefix, const int* active_prefix, int nscenes,
                         int max_iters, int item_ctas, int grid_ctas, int* d_iter, cudaStream_t body,
                         cudaStream_t gate, cudaStream_t st);
// Kernel attributes of the solve (outside any stream capture).
void fast_implicit_setup();

// While `st` captures a graph: appends a conditional node (IF or WHILE) on
// `cond` after the work captured so far, and captures `fill`'s launches on
// `body` (a stream not otherwise capturing) as the node's body. Returns
// false when `st` is not capturing or a call failed (a failure also
// invalidates the capture, which then fails at its end).
template <class Fill>
bool capture_conditional(cudaStream_t st, cudaGraphConditionalHandle cond, cudaGraphConditionalNodeType type,
                         cudaStream_t body, Fill fill) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  if (cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps) != cudaSuccess ||
      cs != cudaStreamCaptureStatusActive)
    return false;
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = cond;
  p.conditional.type = type;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  if (cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &p) != cudaSuccess ||
      cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess ||
      cudaStreamBeginCaptureToGraph(body, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                    cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return false;
  fill(body);
  cudaGraph_t out = nullptr;
  return cudaStreamEndCapture(body, &out) == cudaSuccess;
}
// A conditional handle on the graph `st` is capturing (false if none).
inline bool capture_handle(cudaStream_t st, cudaGraphConditionalHandle* cond) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  if (cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, nullptr, nullptr, nullptr) != cudaSuccess ||
      cs != cudaStreamCaptureStatusActive)
    return false;
  return cudaGraphConditionalHandleCreate(cond, g, 0, cudaGraphCondAssignDefault) == cudaSuccess;
}

// Binning of one scene (host-side sizes known): keys -> radix sort ->
// permutation of the particle streams -> P2G work items.
struct BinScratch {
  uint32_t* keys[2];
  uint32_t* vals[2];
  uint32_t* hist;      // 256 x tiles
  uint32_t* scan_tmp;  // partial sums of the scan
  int* bstart;         // nblocks
  int* bend;           // nblocks
  int* home;           // nblocks
  float4* tmp4[5];     // permutation targets for xm, vv, fa, fb, vq
  float2* tmp2;        // ... and fc
  uint32_t* tmp_pid;   // ... and pid
  size_t n_cap;
};
size_t radix_tiles(size_t n);
// Sorts (key, index) pairs for the first n particles of scene `sd` (a host
// copy of the device descriptor) and leaves the sorted keys in keys[0] and
// the permutation in vals[0].
void fast_sort_keys(const SceneDev& sd, const SceneDev* sd_dev, BinScratch& b, int key_bits, cudaStream_t st);
// copy_back false: the particles stay in the binned copies (CNT_BINNED) for the
// step's fused kernel; only valid when that kernel follows in the same step.
void fast_apply_bins(const SceneDev& sd, const SceneDev* sd_dev, BinScratch& b, int items_max, bool copy_back,
                     cudaStream_t st);

// Radix sort of arbitrary (key, value) pairs; the result lands in k[0]/v[0].
void radix_sort_pairs(uint32_t* k[2], uint32_t* v[2], size_t n, int key_bits, uint32_t* hist, uint32_t* scan_tmp,
                      cudaStream_t st, int start = 0);  // start: the buffer holding the input

// Bulk statistics of one scene.
struct StatsAccum {
  double mass, mom[3], ke, com[3], jp;
  int bmin_key[3], bmax_key[3];  // order-preserving int keys of the bbox floats
  unsigned long long nonfinite;
};
// Per-block partial sums of one statistics read and the counter of blocks
// that have written theirs. The kernel's last block sums the partials in
// block order (the result does not depend on which block finished when),
// writes the totals to `host` (mapped pinned memory, read after the stream
// passes the kernel) and resets the counter, so a read needs no copy in
// either direction.
constexpr int kStatsMaxBlocks = 1024;
struct StatsBlockSum {
  double acc[9];  // mass, momentum x3, kinetic energy, mass-weighted position x3, sum J_p
  float bmin[3], bmax[3];
  unsigned long long bad;
};
struct StatsSlot {
  StatsBlockSum part[kStatsMaxBlocks];
  unsigned int done;
};
void fast_stats(const SceneDev* sd_dev, int n, StatsSlot* slot, StatsAccum* host, cudaStream_t st);
void ref_stats(const RefArgs& a, StatsSlot* slot, StatsAccum* host, cudaStream_t st);
void fast_download_grid(const SceneDev* sd_dev, float* mass, float* mom, float* force, float* vstar, cudaStream_t st);
void fast_pack(const float* x, const float* v, const float* m, const float* FE, const float* FP, size_t n,
               const SceneDev& sd, cudaStream_t st);
void fast_unpack(const SceneDev* sd_dev, size_t n, float* x, float* v, float* FE, float* Jp, float* volume,
                 cudaStream_t st);

constexpr int kMaxDevices = 64;
// The calling thread's current device (0 .. kMaxDevices - 1).
int current_device();
int num_sms();

}  // namespace snow

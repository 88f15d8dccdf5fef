// libssegpu: kernels and the C-ABI host engine (see include/sse_gpu.h).
//
// Kernels
//   k_walk<INIT>   Carlo.init! for a list of walkers (src/sse.jl:47-60)
//   k_walk<SWEEP>  nsweeps Carlo steps per walker: sweep! + measure!
//                  (src/sse.jl:62-87), persistent: each warp pulls walkers
//                  from a work queue and runs all of their sweeps
//   k_link_debug   vertex list of one walker (src/vertex_list.jl) for export
//   k_gather_*     observable / status gathers for the host
//
// Device memory: one stream-ordered pool (cudaMallocAsync) per engine; each
// walker owns its opstring, compact-record and slot-index arrays sized to a
// capacity that grows (with a relaunch) when the reference's cutoff rule
// (src/sse.jl:138-145) asks for more slots than reserved.
#include <cuda_profiler_api.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "sse_device.cuh"
#include "sse_gpu.h"

using namespace sse;

// ==== kernels: begin (device code only down to the matching end marker) ====
namespace {

constexpr int MODE_INIT = 0;
constexpr int MODE_SWEEP = 1;

// smem: this warp's shared memory; its last stage_bytes (a multiple of 32) may hold the walker's
// compacted records for the worm update when they fit
template <int MODE>
__device__ void process_walker(const DevModel &M, DevWalker *W, uint8_t *smem, int smem_per_warp, int stage_bytes,
                               uint32_t flags, long long add_sweeps, int *flag_counts, int lane) {
  Chain c;
  c.L = W->L;
  c.n = W->n;
  c.cap = W->cap;
  c.ctr = W->ctr;
  c.seed = W->seed;
  c.stream = W->stream;
  c.T = W->T;
  WormCtl wc;
  wc.num_worms = W->num_worms;
  wc.avg_len = W->avg_len;
  wc.att = W->att;
  wc.target_frac = W->target_frac;
  uint32_t *ops = W->ops;
  uint8_t *state = W->state;
  const int N = M.nsites;
  long long sweeps = W->sweeps;
  // first pass of an sse_sweep call sets the target; relaunches after a regrowth keep it
  const long long target = add_sweeps >= 0 ? sweeps + add_sweeps : W->target;
  const long long therm = W->therm;
  long long resize_count = W->resize_after_therm;
  long long slot_visits = W->slot_visits;
  long long worm_steps = W->worm_steps;
  long long need_L = 0;
  int phase = W->phase;
  int warmup_done = W->warmup_done;
  int status = ST_OK;
  uint8_t *sst = smem;
  int32_t *vlast = reinterpret_cast<int32_t *>(smem);
  // the warp's site table sits just below the staging area
  SiteTable *tab = reinterpret_cast<SiteTable *>(smem + smem_per_warp - stage_bytes - (int)sizeof(SiteTable));

  if (MODE == MODE_INIT) {
    if (phase == PH_NEW) {
      // mc.state = [rand(1:dim) for sites] (src/sse.jl:48)
      for (int i = lane; i < N; i += 32)
        state[i] = (uint8_t)urange0(draw64(c.seed, c.stream, c.ctr + i), (unsigned long long)M.site_dims[i]);
      c.ctr += N;
      c.L = W->init_cutoff;
      c.n = 0;
      for (long long p = lane; p < c.L; p += 32) ops[p] = 0u;
      phase = PH_WARMUP;
      warmup_done = 0;
      __syncwarp();
    }
    while (phase == PH_WARMUP && warmup_done < W->warmup) {
      for (int i = lane; i < N; i += 32) sst[i] = state[i];
      __syncwarp();
      status = diag_update(M, c, ops, sst, reinterpret_cast<ulonglong2 *>(tab), false, resize_count, need_L, lane);
      if (status != ST_OK) break;
      slot_visits += c.L;
      warmup_done++;
    }
    if (status == ST_OK && phase == PH_WARMUP) phase = PH_READY;
  } else {
    if (phase != PH_READY) {
      status = ST_STATE;
    } else if (W->status != ST_OK && W->status != ST_NEED_GROW) {
      // a walker stopped by an error (e.g. a worm past the step cap) keeps its status: its
      // opstring was left mid-update and must not be swept again
      status = W->status;
    } else {
      long long cyc0 = 0, cyc1 = 0, cyc2 = 0, cyc3 = 0;
      while (sweeps < target) {
        const bool thermalized = sweeps > therm;
        long long t0 = clock64();
        for (int i = lane; i < N; i += 32) sst[i] = state[i];
        __syncwarp();
        status = diag_update(M, c, ops, sst, reinterpret_cast<ulonglong2 *>(tab), thermalized, resize_count, need_L,
                             lane);
        if (status != ST_OK) break;
        slot_visits += c.L;
        __syncwarp();
        long long t1 = clock64();
        const long long nrec = build_links(M, c.L, ops, W->rec, W->chunk, W->vfirst, vlast, tab, lane);
        // records that fit the staging budget move to shared memory for the pointer chase
        Rec *wrec = W->rec;
        const bool staged = stage_bytes > 0 && nrec * (long long)sizeof(Rec) <= (long long)stage_bytes;
        if (staged) {
          int4 *dst = reinterpret_cast<int4 *>(smem + (smem_per_warp - stage_bytes));
          const int4 *src = reinterpret_cast<const int4 *>(W->rec);
          for (long long i = lane; i < 2 * nrec; i += 32) dst[i] = src[i];
          __syncwarp();
          wrec = reinterpret_cast<Rec *>(dst);
        }
        long long t2 = clock64();
        double wlf = 0.0;
        bool have_wlf = false;
        status = worm_update(M, c, wc, ops, wrec, W->chunk, W->vfirst, state,
                             reinterpret_cast<unsigned long long *>(smem), thermalized, wlf, have_wlf, worm_steps,
                             lane, W->cap_factor);
        // an undone worm phase (thermalisation only) leaves the opstring as the diagonal update made it
        const bool undone = status == ST_WORM_UNDONE;
        if (undone) {  // rare: counted straight in the walker record
          status = ST_OK;
          if (lane == 0) W->worm_undos++;
        }
        if (status != ST_OK) break;
        long long t3 = clock64();
        // measure! after this sweep (Carlo measures once sweeps > thermalization); the records still
        // hold the operators' final codes, and the exact integer measurement runs on them while
        // writing the codes back into the opstring
        // writing the codes back into the opstring.  The sweep at sweeps == thermalization can undo its
        // worm phase and still be measured: it measures the opstring the diagonal update left.
        const bool meas = (flags & SSE_SWEEP_MEASURE) && sweeps + 1 > therm;
        const bool fused = meas && M.est_int && !undone;
        if (fused) measure_records(M, c, W, wrec, ops, state, lane);
        else if (!undone) write_back_ops(c, wrec, ops, lane);
        if (have_wlf && lane == 0) observe(W, 5, wlf);
        sweeps++;
        if (meas && !fused) measure(M, c, W, ops, state, lane);
        __syncwarp();
        long long t4 = clock64();
        cyc0 += t1 - t0;
        cyc1 += t2 - t1;
        cyc2 += t3 - t2;
        cyc3 += t4 - t3;
      }
      if (lane == 0) {
        W->cyc[0] += cyc0;
        W->cyc[1] += cyc1;
        W->cyc[2] += cyc2;
        W->cyc[3] += cyc3;
      }
    }
  }
  if (lane == 0) {
    W->L = c.L;
    W->n = c.n;
    W->ctr = c.ctr;
    W->num_worms = wc.num_worms;
    W->avg_len = wc.avg_len;
    W->sweeps = sweeps;
    W->target = target;
    W->resize_after_therm = resize_count;
    W->slot_visits = slot_visits;
    W->worm_steps = worm_steps;
    W->phase = phase;
    W->warmup_done = warmup_done;
    W->status = status;
    W->need_L = need_L;
    if (status == ST_NEED_GROW) atomicAdd(flag_counts + 0, 1);
    else if (status != ST_OK) atomicAdd(flag_counts + 1, 1);
  }
  __syncwarp();
}

// Persistent: every warp pulls walker indices from `queue` until `work` is exhausted.  With
// single_id >= 0 the launch is one warp working on that walker only (the unbatched path).
template <int MODE>
__global__ void __launch_bounds__(128, 7) k_walk(const DevModel *__restrict__ models, DevWalker *__restrict__ walkers,
                                              const int32_t *__restrict__ work, int nwork, int single_id, int *queue,
                                              uint32_t flags, long long add_sweeps, int smem_per_warp,
                                              int stage_bytes, int *flag_counts) {
  extern __shared__ __align__(32) uint8_t smem[];
  const int lane = threadIdx.x & 31;
  uint8_t *mine = smem + (size_t)(threadIdx.x >> 5) * smem_per_warp;
  if (single_id >= 0) {
    DevWalker *W = walkers + single_id;
    process_walker<MODE>(models[W->model], W, mine, smem_per_warp, stage_bytes, flags, add_sweeps, flag_counts,
                         lane);
    return;
  }
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(queue, 1);
    idx = __shfl_sync(FULL, idx, 0);
    if (idx >= nwork) break;
    DevWalker *W = walkers + work[idx];
    process_walker<MODE>(models[W->model], W, mine, smem_per_warp, stage_bytes, flags, add_sweeps, flag_counts,
                         lane);
  }
}

__global__ void k_set_targets(DevWalker *walkers, const int32_t *ids, const int32_t *nsweeps, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    DevWalker *W = walkers + ids[i];
    W->target = W->sweeps + nsweeps[i];
  }
}

struct GrowEntry {
  int32_t id, pad;
  uint32_t *ops;
  Rec *rec;
  int2 *chunk;
  long long cap;
};

// Points grown walkers at their new arrays (the host copied the opstring prefix beforehand).
__global__ void k_apply_growth(DevWalker *walkers, const GrowEntry *g, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    DevWalker *W = walkers + g[i].id;
    W->ops = g[i].ops;
    W->rec = g[i].rec;
    W->chunk = g[i].chunk;
    W->cap = g[i].cap;
    if (W->status == ST_NEED_GROW) W->status = ST_OK;
    W->need_L = 0;
  }
}

__global__ void k_link_debug(const DevModel *models, DevWalker *walkers, int id, int32_t *vlast_out) {
  extern __shared__ __align__(32) uint8_t smem[];
  const int lane = threadIdx.x & 31;
  DevWalker *W = walkers + id;
  const DevModel &M = models[W->model];
  int32_t *vlast = reinterpret_cast<int32_t *>(smem);
  SiteTable *tab = reinterpret_cast<SiteTable *>(smem + warp_area_bytes(M.nsites));
  build_links(M, W->L, W->ops, W->rec, W->chunk, W->vfirst, vlast, tab, lane);
  for (int i = lane; i < M.nsites; i += 32) vlast_out[i] = vlast[i];
}

__global__ void k_gather_status(const DevWalker *walkers, const int32_t *ids, int n, int32_t *status,
                                long long *need_L) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    status[i] = walkers[ids[i]].status;
    need_L[i] = walkers[ids[i]].need_L;
  }
}

__global__ void k_gather_obs(DevWalker *walkers, const int32_t *ids, int n, const int32_t *offsets, double *sums,
                             long long *counts, double *last, int reset) {
  const int w = blockIdx.x;
  if (w >= n) return;
  DevWalker *W = walkers + ids[w];
  const int off = offsets[w], cnt = offsets[w + 1] - offsets[w];
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
    sums[off + i] = W->obs_sum[i];
    counts[off + i] = W->obs_count[i];
    last[off + i] = W->obs_last[i];
    if (reset) {
      W->obs_sum[i] = 0.0;
      W->obs_count[i] = 0;
    }
  }
}

// ---------------------------------------------------------------------------
// invariant check (test/test_sse.jl:5-28, isconsistent): propagating the spin state through the
// opstring, every operator's lower legs match the state it meets, and the state after the last
// operator is the initial one again (periodic imaginary time).  Also checks the table ranges of
// every operator and the operator count.  One warp per walker; lane 0 walks the opstring.
// ---------------------------------------------------------------------------

constexpr int CHK_OK = 0, CHK_SIZES = 1, CHK_OPERATOR = 2, CHK_COUNT = 3, CHK_LEGS = 4, CHK_PERIODIC = 5,
              CHK_STATE = 6;

__global__ void k_check(const DevModel *models, const DevWalker *walkers, const int32_t *ids, int n,
                        int32_t *result, int smem_per_warp) {
  extern __shared__ __align__(32) uint8_t smem[];
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  uint8_t *sst = smem + (size_t)(threadIdx.x >> 5) * smem_per_warp;
  for (int i = warp; i < n; i += nwarps) {
    const DevWalker &W = walkers[ids[i]];
    const DevModel &M = models[W.model];
    const int N = M.nsites;
    int code = CHK_OK;
    if (W.L < 0 || W.L > W.cap || W.n < 0 || W.n > W.L) code = CHK_SIZES;
    bool bad_state = false;
    for (int s = lane; s < N; s += 32) {
      const uint8_t v = W.state[s];
      bad_state |= v >= M.site_dims[s];
      sst[s] = v;
    }
    if (__any_sync(FULL, bad_state) && code == CHK_OK) code = CHK_STATE;
    __syncwarp();
    if (lane == 0 && code == CHK_OK) {
      long long count = 0;
      for (long long p = 0; p < W.L && code == CHK_OK; p++) {
        const uint32_t op = W.ops[p];
        if (!op) continue;
        count++;
        const int bond = (int)(op >> 11);
        if (!(op & 1u) || bond >= M.nbonds) {
          code = CHK_OPERATOR;
          break;
        }
        const int4 bi = M.bond_info[bond];
        const DevType t = M.types[bi.z];
        const int v = (int)((op >> 2) & 0x1FFu);
        if (v >= t.nverts) {
          code = CHK_OPERATOR;
          break;
        }
        const uint8_t *ls = M.leg_state + 4 * (t.vert_off + v);
        if (sst[bi.x] != ls[0] || sst[bi.y] != ls[1]) {
          code = CHK_LEGS;
          break;
        }
        sst[bi.x] = ls[2];
        sst[bi.y] = ls[3];
      }
      if (code == CHK_OK && count != W.n) code = CHK_COUNT;
      if (code == CHK_OK)
        for (int s = 0; s < N; s++)
          if (sst[s] != W.state[s]) {
            code = CHK_PERIODIC;
            break;
          }
    }
    code = __shfl_sync(FULL, code, 0);
    if (lane == 0) result[i] = code;
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// parallel tempering: Carlo.parallel_tempering_log_weight_ratio and
// parallel_tempering_change_parameter! (src/sse.jl:390-405)
// ---------------------------------------------------------------------------

constexpr int PT_MAX_RUNGS = 1024;

// exp(lwr(a, T_b) + lwr(b, T_a)) with lwr(mc, T') = -n log(T'/T), i.e. (T_a/T_b)^(n_a - n_b), as an
// integer power by binary powering of a correctly rounded base (the same products on any IEEE-754
// machine, so the accept decision replays exactly)
__device__ double pt_swap_weight(double Ta, double Tb, long long na, long long nb) {
  const bool up = na >= nb;
  unsigned long long e = up ? (unsigned long long)(na - nb) : (unsigned long long)(nb - na);
  double b = up ? __ddiv_rn(Ta, Tb) : __ddiv_rn(Tb, Ta);
  double q = 1.0;
  while (e) {
    if (e & 1ull) q = __dmul_rn(q, b);
    e >>= 1;
    if (e) b = __dmul_rn(b, b);
  }
  return q;
}

// One block per ladder of `nrungs` walkers (ids[l*nrungs + k], any order).  The walkers are ranked by
// their current T; step s proposes the rung pairs (k, k+1) with k = s mod 2 (mod 2), accepts one with
// probability min(1, q) using u = rand() from Philox(counter = (s, k, l), key = seed), and exchanges
// the two temperatures together with the observable accumulators, which stay with their temperature.
__global__ void __launch_bounds__(256) k_tempering(DevWalker *walkers, const DevModel *models, const int32_t *ids,
                                                   int nrungs, unsigned long long seed, unsigned long long step,
                                                   int32_t *accepted, long long *acc_count, long long *prop_count,
                                                   int *err) {
  __shared__ double uT[PT_MAX_RUNGS], sT[PT_MAX_RUNGS];
  __shared__ long long sN[PT_MAX_RUNGS];
  __shared__ int32_t sW[PT_MAX_RUNGS];
  __shared__ int dup;
  const int l = blockIdx.x;
  const int32_t *lid = ids + (size_t)l * nrungs;
  if (threadIdx.x == 0) dup = 0;
  for (int k = threadIdx.x; k < nrungs; k += blockDim.x) uT[k] = walkers[lid[k]].T;
  __syncthreads();
  for (int k = threadIdx.x; k < nrungs; k += blockDim.x) {
    const double t = uT[k];
    int r = 0;
    bool same = false;
    for (int j = 0; j < nrungs; j++) {
      r += uT[j] < t;
      same |= (j != k) && (uT[j] == t);
    }
    if (same) dup = 1;
    else {
      sT[r] = t;
      sN[r] = walkers[lid[k]].n;
      sW[r] = lid[k];
    }
  }
  __syncthreads();
  const size_t base = (size_t)l * (nrungs - 1);
  if (dup) {
    if (threadIdx.x == 0) atomicExch(err, 1);
    for (int k = threadIdx.x; k < nrungs - 1; k += blockDim.x) accepted[base + k] = -1;
    return;
  }
  for (int k = threadIdx.x; k < nrungs - 1; k += blockDim.x) {
    int32_t res = -1;
    if ((unsigned long long)(k & 1) == (step & 1ull)) {
      DevWalker *A = walkers + sW[k], *B = walkers + sW[k + 1];
      const bool ok = (A->status == ST_OK || A->status == ST_NEED_GROW) &&
                      (B->status == ST_OK || B->status == ST_NEED_GROW);
      if (ok) {
        const double q = pt_swap_weight(sT[k], sT[k + 1], sN[k], sN[k + 1]);
        const uint4 x = philox_block(seed, ((unsigned long long)(unsigned)l << 32) | (unsigned)k, step);
        const unsigned long long u64 = ((unsigned long long)x.y << 32) | x.x;
        const double u = (double)(u64 >> 11) * 0x1.0p-53;
        res = u < q ? 1 : 0;
        if (res) {
          A->T = sT[k + 1];
          B->T = sT[k];
          const int nobs = models[A->model].nobs;
          for (int i = 0; i < nobs; i++) {
            const double s = A->obs_sum[i], z = A->obs_last[i];
            const long long c = A->obs_count[i];
            A->obs_sum[i] = B->obs_sum[i];
            A->obs_last[i] = B->obs_last[i];
            A->obs_count[i] = B->obs_count[i];
            B->obs_sum[i] = s;
            B->obs_last[i] = z;
            B->obs_count[i] = c;
          }
        }
        prop_count[base + k] += 1;
        acc_count[base + k] += res;
      }
    }
    accepted[base + k] = res;
  }
}

}  // namespace
// ==== kernels: end ====

// ---------------------------------------------------------------------------
// host engine
// ---------------------------------------------------------------------------

struct HostModel {
  DevModel dev{};
  std::vector<void *> allocs;
  int32_t nsites = 0, nobs = 0;
  // host copies used to validate imported walker state
  std::vector<int32_t> bond_type, type_nverts, site_dims;
};

struct HostWalker {
  bool alive = false;
  int32_t model = -1;
  long long cap = 0;
  uint32_t *ops = nullptr;
  Rec *rec = nullptr;
  int2 *chunk = nullptr;  // chunk index: one entry per 32 slots
  int32_t *vfirst = nullptr;
  uint8_t *state = nullptr;
  double *obs_sum = nullptr, *obs_last = nullptr;
  long long *obs_count = nullptr;
};

struct sse_engine {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  int num_sms = 0;
  std::vector<HostModel> models;
  DevModel *d_models = nullptr;
  size_t d_models_cap = 0;
  std::vector<HostWalker> walkers;
  DevWalker *d_walkers = nullptr;
  size_t d_walkers_cap = 0;
  int32_t *d_work = nullptr;
  size_t work_cap = 0;
  int *d_queue = nullptr;      // [0] queue head
  int *d_flags = nullptr;      // [0] need-grow count, [1] error count
  int32_t *d_status = nullptr; // gather buffers
  long long *d_needL = nullptr;
  size_t status_cap = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;
  long long last_launches = 0;
  int warps_per_block = 0, blocks_per_sm = 0;
  int stage_bytes = 0;  // shared-memory staging budget per walker for the worm update (0: off)
  struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    int32_t *d_work = nullptr;
  };
  std::map<std::pair<std::vector<int32_t>, long long>, GraphEntry> graphs;
};

namespace {

int fail(sse_engine *e, int code, const std::string &msg) {
  if (e) e->err = msg;
  return code;
}

#define CUDA_TRY(e, call)                                                                          \
  do {                                                                                             \
    cudaError_t _st = (call);                                                                      \
    if (_st != cudaSuccess)                                                                        \
      return fail((e), SSE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_st));         \
  } while (0)

template <class T>
int dev_alloc(sse_engine *e, T **p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t st = cudaMallocAsync((void **)p, count * sizeof(T), e->stream);
  if (st != cudaSuccess) return fail(e, SSE_ERR_NOMEM, std::string("cudaMallocAsync: ") + cudaGetErrorString(st));
  return SSE_OK;
}

template <class T>
void dev_free(sse_engine *e, T *&p) {
  if (p) cudaFreeAsync(p, e->stream);
  p = nullptr;
}

// Entries of a walker's chunk index for `cap` opstring slots: one per 32-slot chunk.
size_t chunk_count(long long cap) { return (size_t)((cap + 31) / 32); }

// Device buffers of one call, freed (stream-ordered) when the call returns, on every path.
struct Scratch {
  sse_engine *e;
  std::vector<void **> held;
  explicit Scratch(sse_engine *eng) : e(eng) {}
  Scratch(const Scratch &) = delete;
  Scratch &operator=(const Scratch &) = delete;
  template <typename T>
  int alloc(T **p, size_t count) {
    const int rc = dev_alloc(e, p, count);
    if (!rc) held.push_back(reinterpret_cast<void **>(p));
    return rc;
  }
  ~Scratch() {
    for (void **p : held)
      if (*p) {
        cudaFreeAsync(*p, e->stream);
        *p = nullptr;
      }
  }
};

void clear_graphs(sse_engine *e) {
  for (auto &g : e->graphs) {
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
    if (g.second.d_work) cudaFreeAsync(g.second.d_work, e->stream);
  }
  e->graphs.clear();
}

template <class T>
int upload(sse_engine *e, HostModel &hm, const T *src, size_t count, const T **dst) {
  T *d = nullptr;
  int rc = dev_alloc(e, &d, count);
  if (rc) return rc;
  hm.allocs.push_back(d);
  if (count && src) CUDA_TRY(e, cudaMemcpyAsync(d, src, count * sizeof(T), cudaMemcpyHostToDevice, e->stream));
  *dst = d;
  return SSE_OK;
}

void free_walker_buffers(sse_engine *e, HostWalker &h) {
  dev_free(e, h.ops);
  dev_free(e, h.rec);
  dev_free(e, h.chunk);
  dev_free(e, h.vfirst);
  dev_free(e, h.state);
  dev_free(e, h.obs_sum);
  dev_free(e, h.obs_last);
  dev_free(e, h.obs_count);
}

bool valid_id(sse_engine *e, int32_t id) {
  return id >= 0 && (size_t)id < e->walkers.size() && e->walkers[id].alive;
}

// The walkers of one launch: valid and distinct, so that no two warps ever run the same chain.
int check_work_ids(sse_engine *e, int32_t count, const int32_t *ids) {
  std::vector<char> seen(e->walkers.size(), 0);
  for (int i = 0; i < count; i++) {
    if (!valid_id(e, ids[i])) return fail(e, SSE_ERR_ARG, "unknown walker id");
    if (seen[ids[i]]) return fail(e, SSE_ERR_ARG, "walker " + std::to_string(ids[i]) + " appears twice in one call");
    seen[ids[i]] = 1;
  }
  return SSE_OK;
}

int ensure_work(sse_engine *e, size_t n) {
  if (n <= e->work_cap) return SSE_OK;
  size_t cap = std::max<size_t>(n, 2 * e->work_cap);
  // allocate the new buffers before freeing the old ones: a failure leaves the engine as it was
  decltype(e->d_work) work = nullptr;
  decltype(e->d_status) status = nullptr;
  decltype(e->d_needL) needL = nullptr;
  int rc = dev_alloc(e, &work, cap);
  if (!rc) rc = dev_alloc(e, &status, cap);
  if (!rc) rc = dev_alloc(e, &needL, cap);
  if (rc) {
    dev_free(e, work);
    dev_free(e, status);
    dev_free(e, needL);
    return rc;
  }
  dev_free(e, e->d_work);
  dev_free(e, e->d_status);
  dev_free(e, e->d_needL);
  e->d_work = work;
  e->d_status = status;
  e->d_needL = needL;
  e->work_cap = cap;
  e->status_cap = cap;
  return SSE_OK;
}

int read_walker(sse_engine *e, int32_t id, DevWalker &w) {
  CUDA_TRY(e, cudaMemcpyAsync(&w, e->d_walkers + id, sizeof(DevWalker), cudaMemcpyDeviceToHost, e->stream));
  CUDA_TRY(e, cudaStreamSynchronize(e->stream));
  return SSE_OK;
}

int write_walker(sse_engine *e, int32_t id, const DevWalker &w) {
  CUDA_TRY(e, cudaMemcpyAsync(e->d_walkers + id, &w, sizeof(DevWalker), cudaMemcpyHostToDevice, e->stream));
  CUDA_TRY(e, cudaStreamSynchronize(e->stream));
  return SSE_OK;
}

// Grow walker `id` so that at least `need` slots fit; the opstring prefix [0, L) is preserved.
int grow_walker(sse_engine *e, int32_t id, long long need) {
  DevWalker w;
  int rc = read_walker(e, id, w);
  if (rc) return rc;
  HostWalker &h = e->walkers[id];
  if (need <= h.cap) return SSE_OK;
  long long cap = std::max<long long>(need, 2 * h.cap);
  cap = (cap + 63) & ~63LL;
  if (cap >= (1LL << 31) / 4) return fail(e, SSE_ERR_CAPACITY, "walker opstring exceeds 2^29 slots");
  uint32_t *ops = nullptr;
  Rec *rec = nullptr;
  int2 *chunk = nullptr;
  rc = dev_alloc(e, &ops, (size_t)cap);
  if (!rc) rc = dev_alloc(e, &rec, (size_t)cap);
  if (!rc) rc = dev_alloc(e, &chunk, chunk_count(cap));
  if (rc) {
    dev_free(e, ops);
    dev_free(e, rec);
    dev_free(e, chunk);
    return rc;
  }
  if (h.ops && w.L > 0) {
    const cudaError_t st =
        cudaMemcpyAsync(ops, h.ops, sizeof(uint32_t) * (size_t)w.L, cudaMemcpyDeviceToDevice, e->stream);
    if (st != cudaSuccess) {
      dev_free(e, ops);
      dev_free(e, rec);
      dev_free(e, chunk);
      return fail(e, SSE_ERR_CUDA, std::string("cudaMemcpyAsync (opstring prefix): ") + cudaGetErrorString(st));
    }
  }
  dev_free(e, h.ops);
  dev_free(e, h.rec);
  dev_free(e, h.chunk);
  h.ops = ops;
  h.rec = rec;
  h.chunk = chunk;
  h.cap = cap;
  w.ops = ops;
  w.rec = rec;
  w.chunk = chunk;
  w.cap = cap;
  if (w.status == ST_NEED_GROW) w.status = ST_OK;
  w.need_L = 0;
  return write_walker(e, id, w);
}

int choose_launch(sse_engine *e, int max_nsites, int nwork, int &wpb, int &grid, int &smem_per_warp, int &stage,
                  bool init) {
  // per warp: spin state (N bytes, diagonal update), per-site link tails (4N, linking), 64 draws (512 B, worms),
  // the chunk-local site table (1 KB), then the staging area for the records of small walkers (sweeps only)
  stage = init ? 0 : ((e->stage_bytes + 31) & ~31);
  smem_per_warp = warp_area_bytes(max_nsites) + (int)sizeof(SiteTable) + stage;
  wpb = e->warps_per_block > 0 ? e->warps_per_block : 4;
  if (wpb > 4) wpb = 4;  // k_walk is compiled for at most 128 threads per block
  while (wpb > 1 && (size_t)wpb * smem_per_warp > 200 * 1024) wpb >>= 1;
  const size_t smem = (size_t)wpb * smem_per_warp;
  if (smem > 227 * 1024) return fail(e, SSE_ERR_UNSUPPORTED, "per-walker shared memory exceeds the SM limit");
  const void *fn = init ? (const void *)k_walk<MODE_INIT> : (const void *)k_walk<MODE_SWEEP>;
  CUDA_TRY(e, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(smem, 48 * 1024)));
  int per_sm = 0;
  CUDA_TRY(e, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * wpb, smem));
  if (per_sm < 1) return fail(e, SSE_ERR_UNSUPPORTED, "kernel does not fit on an SM with this launch shape");
  if (e->blocks_per_sm > 0) per_sm = std::min(per_sm, e->blocks_per_sm);
  const long long resident = (long long)per_sm * e->num_sms;
  const long long needed = (nwork + wpb - 1) / wpb;
  grid = (int)std::max<long long>(1, std::min(resident, needed));
  return SSE_OK;
}

// Launch one pass: persistent over d_work[0..nwork) when single_id < 0, else one warp on single_id.
int launch_pass(sse_engine *e, int mode, int nwork, int single_id, uint32_t flags, long long add_sweeps,
                int max_nsites) {
  int wpb, grid, spw, stage;
  int rc = choose_launch(e, max_nsites, nwork, wpb, grid, spw, stage, mode == MODE_INIT);
  if (rc) return rc;
  if (single_id >= 0) {
    grid = 1;
    wpb = 1;
  } else {
    CUDA_TRY(e, cudaMemsetAsync(e->d_queue, 0, sizeof(int), e->stream));
  }
  if (mode == MODE_INIT)
    k_walk<MODE_INIT><<<grid, 32 * wpb, (size_t)wpb * spw, e->stream>>>(
        e->d_models, e->d_walkers, e->d_work, nwork, single_id, e->d_queue, flags, add_sweeps, spw, stage, e->d_flags);
  else
    k_walk<MODE_SWEEP><<<grid, 32 * wpb, (size_t)wpb * spw, e->stream>>>(
        e->d_models, e->d_walkers, e->d_work, nwork, single_id, e->d_queue, flags, add_sweeps, spw, stage, e->d_flags);
  CUDA_TRY(e, cudaGetLastError());
  e->last_launches += 1;
  return SSE_OK;
}

int max_nsites_of(sse_engine *e, int n, const int32_t *ids) {
  int m = 1;
  for (int i = 0; i < n; i++) m = std::max(m, e->models[e->walkers[ids[i]].model].nsites);
  return m;
}

// Runs `mode` over the given walkers until none of them needs to grow.  With SSE_SWEEP_PLAIN and a
// single walker the pass is one warp launched for that walker alone.
int run_until_done(sse_engine *e, int mode, std::vector<int32_t> work, long long nsweeps, uint32_t flags) {
  float ms_total = 0.0f;
  e->last_launches = 0;
  bool first = true;
  const bool single = (flags & SSE_SWEEP_PLAIN) && work.size() == 1;
  int first_error = 0, failed = 0;
  std::string err_msg;
  for (int round = 0; round < 64 && !work.empty(); round++) {
    const int n = (int)work.size();
    const int max_ns = max_nsites_of(e, n, work.data());
    int rc = SSE_OK;
    if (!single) {
      // longest walkers first: they bound the makespan of the persistent pass
      std::stable_sort(work.begin(), work.end(),
                       [&](int32_t a, int32_t b) { return e->walkers[a].cap > e->walkers[b].cap; });
      rc = ensure_work(e, work.size());
      if (rc) return rc;
      CUDA_TRY(e, cudaMemcpyAsync(e->d_work, work.data(), sizeof(int32_t) * work.size(), cudaMemcpyHostToDevice,
                                  e->stream));
    }
    const long long add = (mode == MODE_SWEEP && first) ? nsweeps : -1;
    if (!single && mode == MODE_SWEEP && first && (flags & SSE_SWEEP_GRAPH)) {
      // a sweep block replayed from a captured graph: flag and queue resets plus the persistent launch
      auto key = std::make_pair(work, add * 4 + (long long)(flags & SSE_SWEEP_MEASURE));
      auto it = e->graphs.find(key);
      if (it == e->graphs.end()) {
        if (e->graphs.size() >= 16) clear_graphs(e);
        sse_engine::GraphEntry g;
        rc = dev_alloc(e, &g.d_work, work.size());
        if (rc) return rc;
        CUDA_TRY(e, cudaMemcpyAsync(g.d_work, work.data(), sizeof(int32_t) * work.size(), cudaMemcpyHostToDevice,
                                    e->stream));
        CUDA_TRY(e, cudaStreamSynchronize(e->stream));
        int wpb, grid, spw, stage;
        rc = choose_launch(e, max_ns, n, wpb, grid, spw, stage, false);
        if (rc) return rc;
        cudaGraph_t graph = nullptr;
        CUDA_TRY(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t cst = cudaMemsetAsync(e->d_flags, 0, 2 * sizeof(int), e->stream);
        if (cst == cudaSuccess) cst = cudaMemsetAsync(e->d_queue, 0, sizeof(int), e->stream);
        if (cst == cudaSuccess) {
          k_walk<MODE_SWEEP><<<grid, 32 * wpb, (size_t)wpb * spw, e->stream>>>(
              e->d_models, e->d_walkers, g.d_work, n, -1, e->d_queue, flags, add, spw, stage, e->d_flags);
          cst = cudaGetLastError();
        }
        const cudaError_t est = cudaStreamEndCapture(e->stream, &graph);  // always leave capture mode
        if (cst == cudaSuccess) cst = est;
        if (cst == cudaSuccess) cst = cudaGraphInstantiate(&g.exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (cst != cudaSuccess) {
          dev_free(e, g.d_work);
          return fail(e, SSE_ERR_CUDA, std::string("sweep-block graph capture: ") + cudaGetErrorString(cst));
        }
        it = e->graphs.emplace(key, g).first;
      }
      CUDA_TRY(e, cudaEventRecord(e->ev0, e->stream));
      CUDA_TRY(e, cudaGraphLaunch(it->second.exec, e->stream));
      e->last_launches += 1;
    } else {
      CUDA_TRY(e, cudaMemsetAsync(e->d_flags, 0, 2 * sizeof(int), e->stream));
      CUDA_TRY(e, cudaEventRecord(e->ev0, e->stream));
      rc = launch_pass(e, mode, n, single ? work[0] : -1, flags, add, max_ns);
      if (rc) return rc;
    }
    first = false;
    CUDA_TRY(e, cudaEventRecord(e->ev1, e->stream));
    int flags_h[2];
    CUDA_TRY(e, cudaMemcpyAsync(flags_h, e->d_flags, sizeof(flags_h), cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(e, cudaStreamSynchronize(e->stream));
    float ms = 0.0f;
    CUDA_TRY(e, cudaEventElapsedTime(&ms, e->ev0, e->ev1));
    ms_total += ms;
    if (flags_h[0] == 0 && flags_h[1] == 0) break;
    // some walker stopped: collect statuses
    if (single) {
      rc = ensure_work(e, 1);
      if (rc) return rc;
      CUDA_TRY(e, cudaMemcpyAsync(e->d_work, work.data(), sizeof(int32_t), cudaMemcpyHostToDevice, e->stream));
    }
    k_gather_status<<<(n + 255) / 256, 256, 0, e->stream>>>(e->d_walkers, e->d_work, n, e->d_status, e->d_needL);
    CUDA_TRY(e, cudaGetLastError());
    std::vector<int32_t> st(n);
    std::vector<long long> needL(n);
    CUDA_TRY(e, cudaMemcpyAsync(st.data(), e->d_status, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(e, cudaMemcpyAsync(needL.data(), e->d_needL, sizeof(long long) * n, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(e, cudaStreamSynchronize(e->stream));
    std::vector<int32_t> again;
    std::vector<GrowEntry> grow;
    for (int i = 0; i < n; i++) {
      if (st[i] == ST_NEED_GROW) {
        // new arrays for every walker that asked, copies and frees queued on the stream, then
        // one kernel points the walkers at them
        HostWalker &h = e->walkers[work[i]];
        long long cap = std::max<long long>(needL[i], 2 * h.cap);
        cap = (cap + 63) & ~63LL;
        if (cap >= (1LL << 31) / 4) return fail(e, SSE_ERR_CAPACITY, "walker opstring exceeds 2^29 slots");
        GrowEntry g{};
        g.id = work[i];
        rc = dev_alloc(e, &g.ops, (size_t)cap);
        if (!rc) rc = dev_alloc(e, &g.rec, (size_t)cap);
        if (!rc) rc = dev_alloc(e, &g.chunk, chunk_count(cap));
        if (rc) return rc;
        if (h.ops)
          CUDA_TRY(e, cudaMemcpyAsync(g.ops, h.ops, sizeof(uint32_t) * (size_t)h.cap, cudaMemcpyDeviceToDevice,
                                      e->stream));
        dev_free(e, h.ops);
        dev_free(e, h.rec);
        dev_free(e, h.chunk);
        h.ops = g.ops;
        h.rec = g.rec;
        h.chunk = g.chunk;
        h.cap = cap;
        g.cap = cap;
        grow.push_back(g);
        again.push_back(work[i]);
      } else if (st[i] != ST_OK) {
        // the other walkers keep going; the failure is reported when the call returns
        if (!first_error) {
          first_error = st[i];
          char buf[160];
          snprintf(buf, sizeof buf, "walker %d stopped with status %d", work[i], st[i]);
          err_msg = buf;
        }
        failed++;
      }
    }
    if (!grow.empty()) {
      GrowEntry *d_g = nullptr;
      Scratch scratch(e);
      rc = scratch.alloc(&d_g, grow.size());
      if (rc) return rc;
      CUDA_TRY(e, cudaMemcpyAsync(d_g, grow.data(), sizeof(GrowEntry) * grow.size(), cudaMemcpyHostToDevice,
                                  e->stream));
      k_apply_growth<<<((int)grow.size() + 127) / 128, 128, 0, e->stream>>>(e->d_walkers, d_g, (int)grow.size());
      CUDA_TRY(e, cudaGetLastError());
      CUDA_TRY(e, cudaStreamSynchronize(e->stream));
    }
    work.swap(again);
  }
  if (!work.empty() && e->last_launches >= 64) return fail(e, SSE_ERR_CAPACITY, "walkers kept needing regrowth");
  e->last_ms = ms_total;
  if (first_error) {
    if (failed > 1) err_msg += " (" + std::to_string(failed) + " walkers failed)";
    return fail(e, first_error, err_msg);
  }
  return SSE_OK;
}

int upload_models(sse_engine *e) {
  if (e->models.size() > e->d_models_cap) {
    // allocate the new array before freeing the old one: a failure leaves the engine as it was
    size_t cap = std::max<size_t>(8, 2 * e->models.size());
    DevModel *nm = nullptr;
    int rc = dev_alloc(e, &nm, cap);
    if (rc) return rc;
    clear_graphs(e);
    dev_free(e, e->d_models);
    e->d_models = nm;
    e->d_models_cap = cap;
  }
  std::vector<DevModel> h(e->models.size());
  for (size_t i = 0; i < e->models.size(); i++) h[i] = e->models[i].dev;
  CUDA_TRY(e, cudaMemcpyAsync(e->d_models, h.data(), sizeof(DevModel) * h.size(), cudaMemcpyHostToDevice, e->stream));
  CUDA_TRY(e, cudaStreamSynchronize(e->stream));
  return SSE_OK;
}

int ensure_walker_slots(sse_engine *e, size_t n) {
  if (n <= e->d_walkers_cap) return SSE_OK;
  size_t cap = std::max<size_t>(n, std::max<size_t>(64, 2 * e->d_walkers_cap));
  DevWalker *nw = nullptr;
  int rc = dev_alloc(e, &nw, cap);
  if (rc) return rc;
  CUDA_TRY(e, cudaMemsetAsync(nw, 0, sizeof(DevWalker) * cap, e->stream));
  if (e->d_walkers)
    CUDA_TRY(e, cudaMemcpyAsync(nw, e->d_walkers, sizeof(DevWalker) * e->d_walkers_cap, cudaMemcpyDeviceToDevice,
                                e->stream));
  dev_free(e, e->d_walkers);
  e->d_walkers = nw;
  e->d_walkers_cap = cap;
  clear_graphs(e);
  return SSE_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" {

int sse_abi_version(void) { return SSE_GPU_ABI_VERSION; }

int sse_engine_create(int32_t device, sse_engine **out) {
  if (!out) return SSE_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return SSE_ERR_CUDA;
  sse_engine *e = new sse_engine();
  e->device = device;
  if (cudaSetDevice(device) != cudaSuccess) {
    delete e;
    return SSE_ERR_CUDA;
  }
  if (cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      e->num_sms <= 0) {
    delete e;
    return SSE_ERR_CUDA;
  }
  if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e->ev0) != cudaSuccess || cudaEventCreate(&e->ev1) != cudaSuccess) {
    delete e;
    return SSE_ERR_CUDA;
  }
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    unsigned long long thr = ~0ull;  // keep freed blocks cached in the pool
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  if (dev_alloc(e, &e->d_queue, 4) || dev_alloc(e, &e->d_flags, 4)) {
    sse_engine_destroy(e);
    return SSE_ERR_NOMEM;
  }
  *out = e;
  return SSE_OK;
}

int sse_engine_destroy(sse_engine *e) {
  if (!e) return SSE_ERR_ARG;
  cudaSetDevice(e->device);
  clear_graphs(e);
  for (auto &w : e->walkers) free_walker_buffers(e, w);
  for (auto &m : e->models)
    for (void *p : m.allocs) cudaFreeAsync(p, e->stream);
  dev_free(e, e->d_models);
  dev_free(e, e->d_walkers);
  dev_free(e, e->d_work);
  dev_free(e, e->d_status);
  dev_free(e, e->d_needL);
  dev_free(e, e->d_queue);
  dev_free(e, e->d_flags);
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->ev0) cudaEventDestroy(e->ev0);
  if (e->ev1) cudaEventDestroy(e->ev1);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
  return SSE_OK;
}

const char *sse_engine_last_error(const sse_engine *e) { return e ? e->err.c_str() : "null engine"; }

int sse_model_register(sse_engine *e, const sse_model_desc *d, int32_t *model_id) {
  if (!e || !d || !model_id) return SSE_ERR_ARG;
  if (d->nsites <= 0 || d->nbonds <= 0 || d->ntypes <= 0 || d->nest < 0)
    return fail(e, SSE_ERR_ARG, "model sizes must be positive");
  if (d->nbonds >= (1 << 21)) return fail(e, SSE_ERR_UNSUPPORTED, "at most 2^21 - 1 bonds");
  if (d->maxdim < 2 || d->maxdim > 255) return fail(e, SSE_ERR_UNSUPPORTED, "site dimension must be 2..255");
  cudaSetDevice(e->device);
  HostModel hm;
  // every table uploaded below is freed again when the registration fails, on any path
  struct Uploads {
    sse_engine *e;
    HostModel &hm;
    bool keep;
    ~Uploads() {
      if (!keep)
        for (void *p : hm.allocs) cudaFreeAsync(p, e->stream);
    }
  } uploads{e, hm, false};
  hm.nsites = d->nsites;
  hm.nobs = 6 + 5 * d->nest;
  DevModel &m = hm.dev;
  m.nsites = d->nsites;
  m.nbonds = d->nbonds;
  m.ntypes = d->ntypes;
  m.maxdim = d->maxdim;
  m.nest = d->nest;
  m.nobs = hm.nobs;
  m.energy_offset = d->energy_offset;
  m.norm_site_count = d->norm_site_count;
  // validate and pack bonds
  std::vector<int4> bi(d->nbonds);
  for (int b = 0; b < d->nbonds; b++) {
    const int s0 = d->bond_sites[2 * b], s1 = d->bond_sites[2 * b + 1], t = d->bond_type[b];
    if (s0 < 0 || s1 < 0 || s0 >= d->nsites || s1 >= d->nsites || s0 == s1 || t < 0 || t >= d->ntypes)
      return fail(e, SSE_ERR_ARG, "bond " + std::to_string(b) + " has invalid sites or type");
    bi[b] = make_int4(s0, s1, t, 0);
  }
  size_t ndiag = 0, nvert = 0, ntrans = 0, nout = 0;
  std::vector<DevType> types(d->ntypes);
  for (int t = 0; t < d->ntypes; t++) {
    DevType &x = types[t];
    x.d0 = d->type_dims[2 * t];
    x.d1 = d->type_dims[2 * t + 1];
    x.nverts = d->type_nverts[t];
    x.maxworm = d->type_maxworm[t];
    x.diag_off = d->type_diag_off[t];
    x.vert_off = d->type_vert_off[t];
    x.trans_off = d->type_trans_off[t];
    x.pad = 0;
    if (x.nverts <= 0 || x.nverts > 512) return fail(e, SSE_ERR_UNSUPPORTED, "vertex count per type must be 1..512");
    // maxworm and the dimensions share one packed word in the compact records (8 bits each)
    if (x.d0 < 2 || x.d1 < 2 || x.d0 > 255 || x.d1 > 255 || x.maxworm < 1 || x.maxworm > 255)
      return fail(e, SSE_ERR_ARG, "bad type dims");
    if (x.diag_off < 0 || x.vert_off < 0 || x.trans_off < 0) return fail(e, SSE_ERR_ARG, "negative table offset");
    ndiag = std::max(ndiag, (size_t)x.diag_off + (size_t)x.d0 * x.d1);
    nvert = std::max(nvert, (size_t)x.vert_off + x.nverts);
    ntrans = std::max(ntrans, (size_t)x.trans_off + (size_t)x.nverts * 4 * x.maxworm);
  }
  for (size_t i = 0; i < ntrans; i++) {
    if (d->trans_start[i] >= 0) nout = std::max(nout, (size_t)d->trans_start[i] + (size_t)d->trans_count[i]);
  }
  for (int i = 0; i < d->nsites; i++)
    if (d->site_dims[i] < 1 || d->site_dims[i] > d->maxdim)
      return fail(e, SSE_ERR_ARG, "site " + std::to_string(i) + " has a dimension outside 1..maxdim");
  for (int b = 0; b < d->nbonds; b++) {
    const DevType &x = types[bi[b].z];
    if (d->site_dims[bi[b].x] != x.d0 || d->site_dims[bi[b].y] != x.d1)
      return fail(e, SSE_ERR_ARG, "site dimensions inconsistent with bond type dims");
  }
  // every leg state is a valid state of its site (legs 0, 2 on the bond's first site, 1, 3 on the second)
  for (int t = 0; t < d->ntypes; t++)
    for (int v = 0; v < types[t].nverts; v++)
      for (int l = 0; l < 4; l++)
        if (d->leg_state[4 * ((size_t)types[t].vert_off + v) + l] >= ((l & 1) ? types[t].d1 : types[t].d0))
          return fail(e, SSE_ERR_ARG, "leg state outside its site's dimension");
  hm.bond_type.assign(d->bond_type, d->bond_type + d->nbonds);
  hm.type_nverts.assign(d->type_nverts, d->type_nverts + d->ntypes);
  hm.site_dims.assign(d->site_dims, d->site_dims + d->nsites);
  int rc = upload(e, hm, bi.data(), bi.size(), &m.bond_info);
  if (!rc) rc = upload(e, hm, d->site_dims, (size_t)d->nsites, &m.site_dims);
  if (!rc) rc = upload(e, hm, types.data(), types.size(), &m.types);
  if (!rc) rc = upload(e, hm, d->diag_vertex, ndiag, &m.diag_vertex);
  // weight classes: the distinct weights of diagonal vertices; the diagonal update compares
  // random integers against per-class thresholds.  With more than 32 classes it compares against
  // each vertex's own weight instead and uses the class (clamped to 127) only to tell a diagonal
  // vertex from an off-diagonal one, so any number of distinct weights is handled exactly.
  std::vector<double> cls_w;
  std::vector<int8_t> vclass(nvert, (int8_t)-1);
  for (int t = 0; t < d->ntypes; t++) {
    for (int v = 0; v < types[t].nverts; v++) {
      const size_t vo = (size_t)types[t].vert_off + v;
      const uint8_t *ls = d->leg_state + 4 * vo;
      if (ls[0] != ls[2] || ls[1] != ls[3]) continue;
      const double w = d->weight[vo];
      size_t c = 0;
      while (c < cls_w.size() && cls_w[c] != w) c++;
      if (c == cls_w.size()) cls_w.push_back(w);
      vclass[vo] = (int8_t)std::min<size_t>(c, 127);
    }
  }
  std::vector<int32_t> diag_vc(ndiag, -1);
  for (int t = 0; t < d->ntypes; t++) {
    const int nst = types[t].d0 * types[t].d1;
    for (int st = 0; st < nst; st++) {
      const size_t i = (size_t)types[t].diag_off + st;
      const int vc = d->diag_vertex[i];
      if (vc < 0) continue;
      if ((vc >> 1) >= types[t].nverts || !(vc & 1)) return fail(e, SSE_ERR_ARG, "bad diagonal vertex table");
      const int cls = vclass[(size_t)types[t].vert_off + (vc >> 1)];
      if (cls < 0) return fail(e, SSE_ERR_ARG, "diagonal vertex table points at an off-diagonal vertex");
      diag_vc[i] = vc | (cls << 16);
    }
  }
  m.ncls = (int32_t)cls_w.size();
  m.one_worm = 1;
  for (int t = 0; t < d->ntypes; t++)
    if (types[t].maxworm != 1) m.one_worm = 0;
  if (cls_w.empty()) cls_w.push_back(0.0);
  if (!rc) rc = upload(e, hm, diag_vc.data(), ndiag, &m.diag_vc);
  if (!rc) rc = upload(e, hm, vclass.data(), nvert, &m.vclass);
  if (!rc) rc = upload(e, hm, cls_w.data(), cls_w.size(), &m.cls_w);
  if (!rc) rc = upload(e, hm, d->weight, nvert, &m.weight);
  if (!rc) rc = upload(e, hm, d->sign, nvert, &m.sign);
  if (!rc) rc = upload(e, hm, d->leg_state, 4 * nvert, &m.leg_state);
  // scatter tables with integer thresholds: u53 < ceil(cum * 2^53)  <=>  u53 * 2^-53 < cum
  auto threshold = [](double cum) -> unsigned long long {
    if (!(cum > 0.0)) return 0ull;
    if (cum >= 1.0) return 1ull << 53;
    return (unsigned long long)std::ceil(std::ldexp(cum, 53));
  };
  std::vector<Outcome> outc(nout);
  for (size_t o = 0; o < nout; o++) {
    const int leg = d->out_leg[o], worm = d->out_worm[o], tgt = d->out_target[o];
    if (leg < 0 || leg > 3 || worm < 1 || worm > 255 || tgt < 0 || tgt >= 1024)
      return fail(e, SSE_ERR_ARG, "transition outcome out of range");
    outc[o].thr = threshold(d->out_cum[o]);
    outc[o].packed = leg | (worm << 2) | (tgt << 10);
    outc[o].pad = 0;
  }
  // the bond type of every transition row, for the dimension of each outcome's site
  std::vector<int32_t> row_type(ntrans, -1);
  for (int t = 0; t < d->ntypes; t++) {
    const size_t r0 = (size_t)d->type_trans_off[t];
    const size_t r1 = r0 + (size_t)types[t].nverts * 4 * types[t].maxworm;
    for (size_t r = r0; r < r1 && r < ntrans; r++) {
      // a row shared by two types would be checked against one type's tables and walked by the other's
      if (row_type[r] >= 0) return fail(e, SSE_ERR_ARG, "two bond types share transition rows");
      row_type[r] = t;
    }
  }
  std::vector<Trans> trans(ntrans);
  for (size_t i = 0; i < ntrans; i++) {
    const int start = d->trans_start[i], cnt = d->trans_count[i];
    trans[i].thr0 = 0;
    trans[i].packed0 = -1;
    trans[i].rest = 0;
    trans[i].thr1 = 0;
    trans[i].packed1 = -1;
    trans[i].pad = 0;
    if (start < 0 || cnt <= 0) continue;
    if (cnt > 256 || start + 2 >= (1 << 23)) return fail(e, SSE_ERR_UNSUPPORTED, "transition row too long");
    if ((size_t)start + (size_t)cnt > nout || row_type[i] < 0)
      return fail(e, SSE_ERR_ARG, "transition row outside the outcome table");
    const DevType &ty = types[row_type[i]];
    for (int o = start; o < start + cnt; o++) {
      // the next step indexes this type's rows with the target vertex and the outgoing worm
      if (((outc[o].packed >> 11) & 0x1FF) >= ty.nverts || ((outc[o].packed >> 2) & 0xFF) > ty.maxworm)
        return fail(e, SSE_ERR_ARG, "transition outcome outside its bond type's tables");
      const int dim_out = (outc[o].packed & 1) ? ty.d1 : ty.d0;  // leg_out & 1: the bond's second site
      const int worm_out = (outc[o].packed >> 2) & 0xFF;
      outc[o].packed = (outc[o].packed & 0xFFFFF) | (((dim_out - worm_out) & 0xFF) << 20);
    }
    trans[i].thr0 = outc[start].thr;
    trans[i].packed0 = outc[start].packed;
    if (cnt > 1) {
      trans[i].thr1 = outc[start + 1].thr;
      trans[i].packed1 = outc[start + 1].packed;
    }
    if (cnt > 2) trans[i].rest = ((start + 2) << 8) | (cnt - 2);
  }
  if (!rc) rc = upload(e, hm, trans.data(), ntrans, &m.trans);
  if (!rc) rc = upload(e, hm, outc.data(), nout, &m.outc);
  if (!rc) rc = upload(e, hm, d->est_coef, (size_t)d->nest * d->nsites * d->maxdim, &m.est_coef);
  // exact integer measurement when every coefficient is a multiple of 1/2 (all MagnetModel estimators)
  {
    const size_t ncoef = (size_t)d->nest * d->nsites * d->maxdim;
    std::vector<int32_t> c2(ncoef);
    bool ok = d->nsites <= (1 << 20);
    for (size_t i = 0; i < ncoef && ok; i++) {
      const double x = 2.0 * d->est_coef[i];
      if (!(std::fabs(x) <= 1024.0) || x != std::nearbyint(x)) ok = false;
      else c2[i] = (int32_t)x;
    }
    m.est_int = ok ? 1 : 0;
    if (!ok) c2.assign(1, 0);
    if (!rc) rc = upload(e, hm, c2.data(), c2.size(), &m.est_coef2);
  }
  if (rc) return rc;
  e->models.push_back(hm);
  rc = upload_models(e);
  if (rc) {
    e->models.pop_back();
    return rc;
  }
  uploads.keep = true;
  *model_id = (int32_t)e->models.size() - 1;
  return SSE_OK;
}

int sse_model_nobs(sse_engine *e, int32_t model_id, int32_t *nobs) {
  if (!e || !nobs || model_id < 0 || (size_t)model_id >= e->models.size()) return SSE_ERR_ARG;
  *nobs = e->models[model_id].nobs;
  return SSE_OK;
}

int sse_walkers_create(sse_engine *e, int32_t model_id, int32_t count, const sse_walker_params *params,
                       int32_t *ids) {
  if (!e || !params || !ids || count < 0 || model_id < 0 || (size_t)model_id >= e->models.size())
    return SSE_ERR_ARG;
  cudaSetDevice(e->device);
  // all parameters are checked before anything is allocated
  for (int i = 0; i < count; i++) {
    const sse_walker_params &p = params[i];
    // worms per sweep: ceil(num_worms), so a count beyond 2^31 (or infinite) would keep one sweep
    // running for hours
    if (!(p.T > 0) || !std::isfinite(p.T) || p.diagonal_warmup_sweeps < 0 || !(p.init_num_worms >= 0) ||
        !(p.init_num_worms <= SSE_MAX_WORMS_PER_SWEEP))
      return fail(e, SSE_ERR_ARG, "walker parameters out of range");
    // links and slot indices are 32-bit: opstrings stay below 2^29 slots, the initial one included
    const double cut0 = p.init_opstring_cutoff >= 0 ? (double)p.init_opstring_cutoff
                                                    : std::nearbyint((double)e->models[model_id].nsites * p.T);
    if (2.0 * cut0 + 163.0 >= (double)((1LL << 31) / 4))
      return fail(e, SSE_ERR_CAPACITY, "initial opstring cutoff exceeds 2^29 slots");
  }
  const HostModel &hm = e->models[model_id];
  const size_t first = e->walkers.size();
  int rc = ensure_walker_slots(e, first + count);
  if (rc) return rc;
  // on a failure below, the walkers of this call are freed again and their ids never handed out
  struct Created {
    sse_engine *e;
    size_t first;
    bool keep;
    ~Created() {
      if (keep) return;
      for (size_t k = first; k < e->walkers.size(); k++) free_walker_buffers(e, e->walkers[k]);
      e->walkers.resize(first);
    }
  } created{e, first, false};
  std::vector<DevWalker> dw(count);
  for (int i = 0; i < count; i++) {
    const sse_walker_params &p = params[i];
    HostWalker h;
    h.alive = true;
    h.model = model_id;
    long long cutoff = p.init_opstring_cutoff;
    if (cutoff < 0) cutoff = (long long)std::nearbyint((double)hm.nsites * p.T);  // round(Int, N*T), ties to even
    h.cap = std::max<long long>(256, ((2 * cutoff + 100) + 63) & ~63LL);
    rc = dev_alloc(e, &h.ops, (size_t)h.cap);
    if (!rc) rc = dev_alloc(e, &h.rec, (size_t)h.cap);
    if (!rc) rc = dev_alloc(e, &h.chunk, chunk_count(h.cap));
    if (!rc) rc = dev_alloc(e, &h.vfirst, (size_t)hm.nsites);
    if (!rc) rc = dev_alloc(e, &h.state, (size_t)hm.nsites);
    if (!rc) rc = dev_alloc(e, &h.obs_sum, (size_t)hm.nobs);
    if (!rc) rc = dev_alloc(e, &h.obs_last, (size_t)hm.nobs);
    if (!rc) rc = dev_alloc(e, &h.obs_count, (size_t)hm.nobs);
    e->walkers.push_back(h);  // from here on the guard frees its buffers if the call fails
    if (rc) return rc;
    CUDA_TRY(e, cudaMemsetAsync(h.obs_sum, 0, sizeof(double) * hm.nobs, e->stream));
    CUDA_TRY(e, cudaMemsetAsync(h.obs_last, 0, sizeof(double) * hm.nobs, e->stream));
    CUDA_TRY(e, cudaMemsetAsync(h.obs_count, 0, sizeof(long long) * hm.nobs, e->stream));
    CUDA_TRY(e, cudaMemsetAsync(h.state, 0, (size_t)hm.nsites, e->stream));
    DevWalker &w = dw[i];
    memset(&w, 0, sizeof w);
    w.ops = h.ops;
    w.rec = h.rec;
    w.chunk = h.chunk;
    w.vfirst = h.vfirst;
    w.state = h.state;
    w.obs_sum = h.obs_sum;
    w.obs_last = h.obs_last;
    w.obs_count = h.obs_count;
    w.cap = h.cap;
    w.T = p.T;
    w.num_worms = p.init_num_worms;
    w.avg_len = 1.0;
    w.att = p.num_worms_attenuation_factor;
    w.target_frac = p.target_worm_length_fraction;
    w.seed = p.seed;
    w.stream = p.stream;
    w.therm = p.thermalization;
    w.init_cutoff = cutoff;
    w.model = model_id;
    w.phase = PH_NEW;
    w.warmup = p.diagonal_warmup_sweeps;
  }
  if (count)
    CUDA_TRY(e, cudaMemcpyAsync(e->d_walkers + first, dw.data(), sizeof(DevWalker) * count, cudaMemcpyHostToDevice,
                                e->stream));
  CUDA_TRY(e, cudaStreamSynchronize(e->stream));
  created.keep = true;
  for (int i = 0; i < count; i++) ids[i] = (int32_t)(first + i);
  return SSE_OK;
}

int sse_walkers_destroy(sse_engine *e, int32_t count, const int32_t *ids) {
  if (!e || (count && !ids)) return SSE_ERR_ARG;
  cudaSetDevice(e->device);
  const int crc = check_work_ids(e, count, ids);  // all known and distinct, or nothing is destroyed
  if (crc) return crc;
  for (int i = 0; i < count; i++) {
    HostWalker &h = e->walkers[ids[i]];
    free_walker_buffers(e, h);
    h.alive = false;
  }
  clear_graphs(e);
  CUDA_TRY(e, cudaStreamSynchronize(e->stream));
  return SSE_OK;
}

int sse_walkers_reserve(sse_engine *e, int32_t count, const int32_t *ids, int64_t capacity) {
  if (!e || (count && !ids) || capacity < 0) return SSE_ERR_ARG;
  cudaSetDevice(e->device);
  for (int i = 0; i < count; i++) {
    if (!valid_id(e, ids[i])) return fail(e, SSE_ERR_ARG, "unknown walker id");
    int rc = grow_walker(e, ids[i], capacity);
    if (rc) return rc;
  }
  return SSE_OK;
}

int sse_walkers_init(sse_engine *e, int32_t count, const int32_t *ids) {
  if (!e || (count && !ids)) return SSE_ERR_ARG;
  cudaSetDevice(e->device);
  const int rc = check_work_ids(e, count, ids);
  if (rc) return rc;
  std::vector<int32_t> work(ids, ids + count);
  return run_until_done(e, MODE_INIT, work, 0, 0);
}

int sse_sweep(sse_engine *e, int32_t count, const int32_t *ids, int32_t nsweeps, uint32_t flags) {
  if (!e || (count && !ids) || nsweeps < 0) return SSE_ERR_ARG;
  cudaSetDevice(e->device);
  const int crc = check_work_ids(e, count, ids);
  if (crc) return crc;
  std::vector<int32_t> work(ids, ids + count);
  if (flags & SSE_SWEEP_PLAIN) {
    // one launch per walker per sweep
    double ms = 0.0;
    long long launches = 0;
    for (int32_t id : work) {
      for (int s = 0; s < nsweeps; s++) {
        int rc = run_until_done(e, MODE_SWEEP, std::vector<int32_t>{id}, 1, flags);
        if (rc) return rc;
        ms += e->last_ms;
        launches += e->last_launches;
      }
    }
    e->last_ms = ms;
    e->last_launches = launches;
    return SSE_OK;
  }
  return run_until_done(e, MODE_SWEEP, work, nsweeps, flags);
}

int sse_sweep_each(sse_engine *e, int32_t count, const int32_t *ids, const int32_t *nsweeps, uint32_t flags) {
  if (!e || (count && (!ids || !nsweeps))) return SSE_ERR_ARG;
  if (count == 0) return SSE_OK;
  cudaSetDevice(e->device);
  const int crc = check_work_ids(e, count, ids);
  if (crc) return crc;
  std::vector<int32_t> work(ids, ids + count);
  for (int i = 0; i < count; i++)
    if (nsweeps[i] < 0) return fail(e, SSE_ERR_ARG, "negative sweep count");
  if (flags & SSE_SWEEP_PLAIN) return fail(e, SSE_ERR_ARG, "sse_sweep_each runs one batched launch");
  int rc = ensure_work(e, (size_t)count);
  if (rc) return rc;
  int32_t *d_ns = nullptr;
  Scratch scratch(e);
  rc = scratch.alloc(&d_ns, (size_t)count);
  if (rc) return rc;
  CUDA_TRY(e, cudaMemcpyAsync(e->d_work, ids, sizeof(int32_t) * count, cudaMemcpyHostToDevice, e->stream));
  CUDA_TRY(e, cudaMemcpyAsync(d_ns, nsweeps, sizeof(int32_t) * count, cudaMemcpyHostToDevice, e->stream));
  k_set_targets<<<(count + 255) / 256, 256, 0, e->stream>>>(e->d_walkers, e->d_work, d_ns, count);
  CUDA_TRY(e, cudaGetLastError());
  // targets are set: every pass keeps them (nsweeps = -1)
  return run_until_done(e, MODE_SWEEP, work, -1, flags);
}

int sse_observables(sse_engine *e, int32_t count, const int32_t *ids, double *sums, int64_t *counts, double *last,
                    int32_t reset) {
  if (!e || (count && (!ids || !sums || !counts || !last))) return SSE_ERR_ARG;
  if (count == 0) return SSE_OK;
  cudaSetDevice(e->device);
  std::vector<int32_t> off(count + 1, 0);
  for (int i = 0; i < count; i++) {
    if (!valid_id(e, ids[i])) return fail(e, SSE_ERR_ARG, "unknown walker id");
    off[i + 1] = off[i] + e->models[e->walkers[ids[i]].model].nobs;
  }
  const size_t tot = (size_t)off[count];
  int32_t *d_ids = nullptr, *d_off = nullptr;
  double *d_s = nullptr, *d_l = nullptr;
  long long *d_c = nullptr;
  Scratch scratch(e);
  int rc = scratch.alloc(&d_ids, count);
  if (!rc) rc = scratch.alloc(&d_off, count + 1);
  if (!rc) rc = scratch.alloc(&d_s, tot);
  if (!rc) rc = scratch.alloc(&d_l, tot);
  if (!rc) rc = scratch.alloc(&d_c, tot);
  if (rc) return rc;
  CUDA_TRY(e, cudaMemcpyAsync(d_ids, ids, sizeof(int32_t) * count, cudaMemcpyHostToDevice, e->stream));
  CUDA_TRY(e, cudaMemcpyAsync(d_off, off.data(), sizeof(int32_t) * (count + 1), cudaMemcpyHostToDevice, e->stream));
  k_gather_obs<<<count, 64, 0, e->stream>>>(e->d_walkers, d_ids, count, d_off, d_s, d_c, d_l, reset);
  CUDA_TRY(e, cudaGetLastError());
  CUDA_TRY(e, cudaMemcpyAsync(sums, d_s, sizeof(double) * tot, cudaMemcpyDeviceToHost, e->stream));
  CUDA_TRY(e, cudaMemcpyAsync(counts, d_c, sizeof(long long) * tot, cudaMemcpyDeviceToHost, e->stream));
  CUDA_TRY(e, cudaMemcpyAsync(last, d_l, sizeof(double) * tot, cudaMemcpyDeviceToHost, e->stream));
  CUDA_TRY(e, cudaStreamSynchronize(e->stream));
  return SSE_OK;
}

static void info_from(const DevWalker &w, sse_walker_info *info) {
  info->L = w.L;
  info->num_operators = w.n;
  info->capacity = w.cap;
  info->sweeps = w.sweeps;
  info->rng_counter = w.ctr;
  info->num_worms = w.num_worms;
  info->avg_worm_length = w.avg_len;
  info->T = w.T;
  info->status = w.status == ST_NEED_GROW ? SSE_OK : w.status;
  info->model = w.model;
  info->resize_after_thermalization = w.resize_after_therm;
  info->slot_visits = w.slot_visits;
  info->worm_steps = w.worm_steps;
  info->worm_undos = w.worm_undos;
  for (int i = 0; i < 4; i++) info->phase_cycles[i] = w.cyc[i];
}

int sse_walker_info_get(sse_engine *e, int32_t id, sse_walker_info *info) {
  if (!e || !info || !valid_id(e, id)) return SSE_ERR_ARG;
  cudaSetDevice(e->device);
  DevWalker w;
  int rc = read_walker(e, id, w);
  if (rc) return rc;
  info_from(w, info);
  return SSE_OK;
}

int sse_walker_export(sse_engine *e, int32_t id, uint32_t *ops, int64_t ops_len, uint8_t *state,
                      sse_walker_info *info) {
  if (!e || !valid_id(e, id)) return SSE_ERR_ARG;
  cudaSetDevice(e->device);
  DevWalker w;
  int rc = read_walker(e, id, w);
  if (rc) return rc;
  if (ops) {
    if (ops_len < w.L) return fail(e, SSE_ERR_ARG, "ops buffer shorter than L");
    if (w.L) CUDA_TRY(e, cudaMemcpy(ops, w.ops, sizeof(uint32_t) * (size_t)w.L, cudaMemcpyDeviceToHost));
  }
  if (state) CUDA_TRY(e, cudaMemcpy(state, w.state, (size_t)e->models[w.model].nsites, cudaMemcpyDeviceToHost));
  if (info) info_from(w, info);
  return SSE_OK;
}

int sse_walker_import(sse_engine *e, int32_t id, const uint32_t *ops, const uint8_t *state,
                      const sse_walker_info *info) {
  if (!e || !info || !valid_id(e, id) || (info->L > 0 && !ops) || !state) return SSE_ERR_ARG;
  if (info->L < 0 || info->num_operators < 0 || info->num_operators > info->L) return fail(e, SSE_ERR_ARG, "bad L/n");
  if (!(info->num_worms >= 0) || !(info->num_worms <= SSE_MAX_WORMS_PER_SWEEP) || !(info->avg_worm_length >= 0) ||
      !std::isfinite(info->avg_worm_length))
    return fail(e, SSE_ERR_ARG, "worm controller state out of range");
  cudaSetDevice(e->device);
  const HostModel &hm = e->models[e->walkers[id].model];
  long long n = 0;
  for (long long p = 0; p < info->L; p++) {
    const uint32_t op = ops[p];
    if (!op) continue;
    n++;
    const int bond = (int)(op >> 11);
    if (bond >= hm.dev.nbonds || !(op & 1u) || (int)((op >> 2) & 0x1FFu) >= hm.type_nverts[hm.bond_type[bond]])
      return fail(e, SSE_ERR_ARG, "opstring has an invalid operator");
  }
  if (n != info->num_operators) return fail(e, SSE_ERR_ARG, "num_operators does not match the opstring");
  for (int i = 0; i < hm.nsites; i++)
    if ((int)state[i] >= hm.site_dims[i]) return fail(e, SSE_ERR_ARG, "spin state outside its site's dimension");
  int rc = grow_walker(e, id, std::max<long long>(info->L, 1));
  if (rc) return rc;
  DevWalker w;
  rc = read_walker(e, id, w);
  if (rc) return rc;
  if (info->L) CUDA_TRY(e, cudaMemcpy(w.ops, ops, sizeof(uint32_t) * (size_t)info->L, cudaMemcpyHostToDevice));
  CUDA_TRY(e, cudaMemcpy(w.state, state, (size_t)hm.nsites, cudaMemcpyHostToDevice));
  w.L = info->L;
  w.n = info->num_operators;
  w.sweeps = info->sweeps;
  w.ctr = info->rng_counter;
  w.num_worms = info->num_worms;
  w.avg_len = info->avg_worm_length;
  w.status = ST_OK;
  w.phase = PH_READY;
  w.warmup_done = w.warmup;
  return write_walker(e, id, w);
}

int sse_vertex_list(sse_engine *e, int32_t id, int32_t *vertices, int32_t *v_first, int32_t *v_last) {
  if (!e || !valid_id(e, id) || !v_first || !v_last) return SSE_ERR_ARG;
  cudaSetDevice(e->device);
  DevWalker w;
  int rc = read_walker(e, id, w);
  if (rc) return rc;
  const int N = e->models[w.model].nsites;
  int32_t *d_vl = nullptr;
  Scratch scratch(e);
  rc = scratch.alloc(&d_vl, (size_t)N);
  if (rc) return rc;
  const size_t smem = (size_t)warp_area_bytes(N) + sizeof(SiteTable);
  CUDA_TRY(e, cudaFuncSetAttribute(k_link_debug, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)std::max<size_t>(smem, 48 * 1024)));
  k_link_debug<<<1, 32, smem, e->stream>>>(e->d_models, e->d_walkers, id, d_vl);
  CUDA_TRY(e, cudaGetLastError());
  std::vector<Rec> rec((size_t)std::max<long long>(w.n, 1));
  std::vector<int32_t> vf(N), vl(N);
  CUDA_TRY(e, cudaMemcpyAsync(vl.data(), d_vl, sizeof(int32_t) * N, cudaMemcpyDeviceToHost, e->stream));
  CUDA_TRY(e, cudaMemcpyAsync(vf.data(), w.vfirst, sizeof(int32_t) * N, cudaMemcpyDeviceToHost, e->stream));
  if (w.n)
    CUDA_TRY(e, cudaMemcpyAsync(rec.data(), w.rec, sizeof(Rec) * (size_t)w.n, cudaMemcpyDeviceToHost, e->stream));
  CUDA_TRY(e, cudaStreamSynchronize(e->stream));
  auto conv = [&](int32_t x) { return x < 0 ? -1 : 4 * rec[x >> 2].slot + (x & 3); };
  if (vertices) {
    for (long long i = 0; i < 4 * w.L; i++) vertices[i] = -1;
    for (long long k = 0; k < w.n; k++)
      for (int l = 0; l < 4; l++) vertices[4LL * rec[k].slot + l] = conv(rec[k].link[l]);
  }
  for (int i = 0; i < N; i++) {
    v_first[i] = conv(vf[i]);
    v_last[i] = conv(vl[i]);
  }
  return SSE_OK;
}

int sse_last_timing(sse_engine *e, double *ms, int64_t *launches) {
  if (!e) return SSE_ERR_ARG;
  if (ms) *ms = e->last_ms;
  if (launches) *launches = e->last_launches;
  return SSE_OK;
}

int sse_set_launch(sse_engine *e, int32_t warps_per_block, int32_t blocks_per_sm) {
  if (!e || warps_per_block < 0 || warps_per_block > 4 || blocks_per_sm < 0) return SSE_ERR_ARG;
  if (warps_per_block != e->warps_per_block || blocks_per_sm != e->blocks_per_sm) clear_graphs(e);
  e->warps_per_block = warps_per_block;
  e->blocks_per_sm = blocks_per_sm;
  return SSE_OK;
}

int sse_set_staging(sse_engine *e, int32_t stage_bytes) {
  if (!e || stage_bytes < 0 || stage_bytes > SSE_MAX_STAGE_BYTES) return SSE_ERR_ARG;
  const int rounded = (stage_bytes + 31) & ~31;
  if (rounded != e->stage_bytes) clear_graphs(e);
  e->stage_bytes = rounded;
  return SSE_OK;
}

int sse_get_staging(sse_engine *e, int32_t *stage_bytes) {
  if (!e || !stage_bytes) return SSE_ERR_ARG;
  *stage_bytes = e->stage_bytes;
  return SSE_OK;
}

}  // extern "C"

namespace {

// Probes every launch shape and staging budget with real sweeps of the given walkers: nsweeps_probe
// each (sse_sweep), or nsweeps_each[i] for walker i (sse_sweep_each) when that array is given.
int autotune_impl(sse_engine *e, int32_t count, const int32_t *ids, int32_t nsweeps_probe,
                  const int32_t *nsweeps_each, uint32_t flags, int32_t *best_warps_per_block,
                  int32_t *best_stage_bytes, double *best_ms) {
  if (!e || count <= 0 || !ids || (!nsweeps_each && nsweeps_probe <= 0)) return SSE_ERR_ARG;
  const int crc = check_work_ids(e, count, ids);
  if (crc) return crc;
  cudaSetDevice(e->device);
  // staging budgets: off, 8 and 32 KB, and room for the records of the 25th-percentile, median and
  // largest walker (25 % headroom for the operator count's fluctuations), where that fits an SM
  std::vector<long long> n(count);
  for (int i = 0; i < count; i++) {
    DevWalker w;
    int rc = read_walker(e, ids[i], w);
    if (rc) return rc;
    n[i] = w.n;
  }
  std::sort(n.begin(), n.end());
  std::vector<int> stages{0, 8192, 32768};
  for (double q : {0.25, 0.5, 1.0}) {
    const long long nq = n[std::min<size_t>((size_t)count - 1, (size_t)(q * (count - 1)))];
    const long long bytes = ((long long)(1.25 * (double)nq * sizeof(Rec)) + 1024 + 31) & ~31LL;
    if (bytes <= SSE_MAX_STAGE_BYTES && std::find(stages.begin(), stages.end(), (int)bytes) == stages.end())
      stages.push_back((int)bytes);
  }
  const int shapes[3] = {1, 2, 4};
  int best = 0, best_stage = 0;
  double best_t = 0.0;
  for (int st : stages) {
    for (int c : shapes) {
      int rc = sse_set_launch(e, c, 0);
      if (!rc) rc = sse_set_staging(e, st);
      if (rc) return rc;
      int wpb, grid, spw, stage;
      if (choose_launch(e, max_nsites_of(e, count, ids), count, wpb, grid, spw, stage, false) != SSE_OK) continue;
      rc = nsweeps_each ? sse_sweep_each(e, count, ids, nsweeps_each, flags & SSE_SWEEP_MEASURE)
                        : sse_sweep(e, count, ids, nsweeps_probe, flags & SSE_SWEEP_MEASURE);
      if (rc) return rc;
      if (!best || e->last_ms < best_t) {
        best = c;
        best_stage = st;
        best_t = e->last_ms;
      }
    }
  }
  if (!best) return fail(e, SSE_ERR_UNSUPPORTED, "no launch shape fits");
  int rc = sse_set_launch(e, best, 0);
  if (!rc) rc = sse_set_staging(e, best_stage);
  if (rc) return rc;
  if (best_warps_per_block) *best_warps_per_block = best;
  if (best_stage_bytes) *best_stage_bytes = best_stage;
  if (best_ms) *best_ms = best_t;
  return SSE_OK;
}

}  // namespace

extern "C" {

int sse_autotune(sse_engine *e, int32_t count, const int32_t *ids, int32_t nsweeps_probe, uint32_t flags,
                 int32_t *best_warps_per_block, int32_t *best_stage_bytes, double *best_ms) {
  return autotune_impl(e, count, ids, nsweeps_probe, nullptr, flags, best_warps_per_block, best_stage_bytes,
                       best_ms);
}

int sse_autotune_each(sse_engine *e, int32_t count, const int32_t *ids, const int32_t *nsweeps, uint32_t flags,
                      int32_t *best_warps_per_block, int32_t *best_stage_bytes, double *best_ms) {
  if (!nsweeps) return SSE_ERR_ARG;
  return autotune_impl(e, count, ids, 0, nsweeps, flags, best_warps_per_block, best_stage_bytes, best_ms);
}

int sse_get_launch(sse_engine *e, int32_t *warps_per_block, int32_t *blocks_per_sm) {
  if (!e) return SSE_ERR_ARG;
  if (warps_per_block) *warps_per_block = e->warps_per_block;
  if (blocks_per_sm) *blocks_per_sm = e->blocks_per_sm;
  return SSE_OK;
}

int sse_profiler_range(sse_engine *e, int32_t start) {
  if (!e) return SSE_ERR_ARG;
  cudaSetDevice(e->device);
  CUDA_TRY(e, cudaStreamSynchronize(e->stream));
  CUDA_TRY(e, start ? cudaProfilerStart() : cudaProfilerStop());
  return SSE_OK;
}

int sse_check_walkers(sse_engine *e, int32_t count, const int32_t *ids, int32_t *result) {
  if (!e || (count && (!ids || !result))) return SSE_ERR_ARG;
  if (count == 0) return SSE_OK;
  cudaSetDevice(e->device);
  for (int i = 0; i < count; i++)
    if (!valid_id(e, ids[i])) return fail(e, SSE_ERR_ARG, "unknown walker id");
  const int max_ns = max_nsites_of(e, count, ids);
  const int spw = (max_ns + 31) & ~31;
  const int wpb = std::max(1, std::min(8, (int)((48 * 1024) / std::max(spw, 32))));
  if ((size_t)wpb * spw > 227 * 1024) return fail(e, SSE_ERR_UNSUPPORTED, "too many sites for the check");
  CUDA_TRY(e, cudaFuncSetAttribute(k_check, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)std::max<size_t>((size_t)wpb * spw, 48 * 1024)));
  Scratch scratch(e);
  int32_t *d_ids = nullptr, *d_res = nullptr;
  int rc = scratch.alloc(&d_ids, (size_t)count);
  if (!rc) rc = scratch.alloc(&d_res, (size_t)count);
  if (rc) return rc;
  CUDA_TRY(e, cudaMemcpyAsync(d_ids, ids, sizeof(int32_t) * count, cudaMemcpyHostToDevice, e->stream));
  const int grid = (int)std::min<long long>((count + wpb - 1) / wpb, 8LL * e->num_sms);
  k_check<<<grid, 32 * wpb, (size_t)wpb * spw, e->stream>>>(e->d_models, e->d_walkers, d_ids, count, d_res, spw);
  CUDA_TRY(e, cudaGetLastError());
  CUDA_TRY(e, cudaMemcpyAsync(result, d_res, sizeof(int32_t) * count, cudaMemcpyDeviceToHost, e->stream));
  CUDA_TRY(e, cudaStreamSynchronize(e->stream));
  return SSE_OK;
}

int sse_walkers_set_worm_cap(sse_engine *e, int32_t count, const int32_t *ids, int32_t factor) {
  if (!e || (count && !ids)) return SSE_ERR_ARG;
  if (factor < 1 || factor > (1 << 20)) return fail(e, SSE_ERR_ARG, "worm cap factor must be 1..2^20");
  cudaSetDevice(e->device);
  for (int i = 0; i < count; i++) {
    if (!valid_id(e, ids[i])) return fail(e, SSE_ERR_ARG, "unknown walker id");
    char *dst = reinterpret_cast<char *>(e->d_walkers + ids[i]) + offsetof(DevWalker, cap_factor);
    CUDA_TRY(e, cudaMemcpyAsync(dst, &factor, sizeof(int32_t), cudaMemcpyHostToDevice, e->stream));
  }
  CUDA_TRY(e, cudaStreamSynchronize(e->stream));
  return SSE_OK;
}

int sse_walker_set_T(sse_engine *e, int32_t id, double T) {
  if (!e || !valid_id(e, id)) return SSE_ERR_ARG;
  if (!(T > 0) || !std::isfinite(T)) return fail(e, SSE_ERR_ARG, "temperature must be positive and finite");
  cudaSetDevice(e->device);
  char *dst = reinterpret_cast<char *>(e->d_walkers + id) + offsetof(DevWalker, T);
  CUDA_TRY(e, cudaMemcpyAsync(dst, &T, sizeof(double), cudaMemcpyHostToDevice, e->stream));
  CUDA_TRY(e, cudaStreamSynchronize(e->stream));
  return SSE_OK;
}

}  // extern "C"

namespace {

// checks a ladder layout: ids distinct and valid, one model per ladder
int check_ladders(sse_engine *e, int32_t nladders, int32_t nrungs, const int32_t *ids) {
  if (nladders < 0 || nrungs < 2 || nrungs > PT_MAX_RUNGS || (nladders && !ids))
    return fail(e, SSE_ERR_ARG, "ladders need 2..1024 rungs");
  std::vector<char> seen(e->walkers.size(), 0);
  for (int l = 0; l < nladders; l++) {
    const int32_t *lid = ids + (size_t)l * nrungs;
    for (int k = 0; k < nrungs; k++) {
      if (!valid_id(e, lid[k])) return fail(e, SSE_ERR_ARG, "unknown walker id");
      if (seen[lid[k]]) return fail(e, SSE_ERR_ARG, "a walker appears twice in the ladders");
      seen[lid[k]] = 1;
      if (e->walkers[lid[k]].model != e->walkers[lid[0]].model)
        return fail(e, SSE_ERR_ARG, "the walkers of a ladder must share one model");
    }
  }
  return SSE_OK;
}

struct PtBuffers {
  Scratch scratch;
  int32_t *ids = nullptr, *accepted = nullptr;
  long long *acc = nullptr, *prop = nullptr;
  int *err = nullptr;
  size_t npairs = 0;
  explicit PtBuffers(sse_engine *e) : scratch(e) {}
};

int pt_alloc(sse_engine *e, PtBuffers &b, int32_t nladders, int32_t nrungs, const int32_t *ids) {
  b.npairs = (size_t)nladders * (nrungs - 1);
  int rc = b.scratch.alloc(&b.ids, (size_t)nladders * nrungs);
  if (!rc) rc = b.scratch.alloc(&b.accepted, b.npairs);
  if (!rc) rc = b.scratch.alloc(&b.acc, b.npairs);
  if (!rc) rc = b.scratch.alloc(&b.prop, b.npairs);
  if (!rc) rc = b.scratch.alloc(&b.err, 1);
  if (rc) return rc;
  CUDA_TRY(e, cudaMemcpyAsync(b.ids, ids, sizeof(int32_t) * (size_t)nladders * nrungs, cudaMemcpyHostToDevice,
                              e->stream));
  CUDA_TRY(e, cudaMemsetAsync(b.acc, 0, sizeof(long long) * b.npairs, e->stream));
  CUDA_TRY(e, cudaMemsetAsync(b.prop, 0, sizeof(long long) * b.npairs, e->stream));
  CUDA_TRY(e, cudaMemsetAsync(b.err, 0, sizeof(int), e->stream));
  return SSE_OK;
}

int pt_launch(sse_engine *e, PtBuffers &b, int32_t nladders, int32_t nrungs, uint64_t seed, uint64_t step) {
  const int threads = std::min(256, (nrungs + 31) & ~31);
  k_tempering<<<nladders, threads, 0, e->stream>>>(e->d_walkers, e->d_models, b.ids, nrungs, seed, step, b.accepted,
                                                    b.acc, b.prop, b.err);
  CUDA_TRY(e, cudaGetLastError());
  e->last_launches += 1;
  return SSE_OK;
}

int pt_check_err(sse_engine *e, PtBuffers &b) {
  int err = 0;
  CUDA_TRY(e, cudaMemcpyAsync(&err, b.err, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
  CUDA_TRY(e, cudaStreamSynchronize(e->stream));
  if (err) return fail(e, SSE_ERR_ARG, "the temperatures of a ladder must be distinct");
  return SSE_OK;
}

}  // namespace

extern "C" {

int sse_tempering_exchange(sse_engine *e, int32_t nladders, int32_t nrungs, const int32_t *ids, uint64_t seed,
                           uint64_t step, int32_t *accepted) {
  if (!e) return SSE_ERR_ARG;
  int rc = check_ladders(e, nladders, nrungs, ids);
  if (rc || nladders == 0) return rc;
  cudaSetDevice(e->device);
  e->last_launches = 0;
  PtBuffers b(e);
  rc = pt_alloc(e, b, nladders, nrungs, ids);
  if (!rc) {
    CUDA_TRY(e, cudaEventRecord(e->ev0, e->stream));
    rc = pt_launch(e, b, nladders, nrungs, seed, step);
  }
  if (!rc) {
    CUDA_TRY(e, cudaEventRecord(e->ev1, e->stream));
    if (accepted)
      CUDA_TRY(e, cudaMemcpyAsync(accepted, b.accepted, sizeof(int32_t) * b.npairs, cudaMemcpyDeviceToHost,
                                  e->stream));
    rc = pt_check_err(e, b);
    float ms = 0.0f;
    if (!rc && cudaEventElapsedTime(&ms, e->ev0, e->ev1) == cudaSuccess) e->last_ms = ms;
  }
  return rc;
}

int sse_sweep_tempering(sse_engine *e, int32_t nladders, int32_t nrungs, const int32_t *ids, int32_t nblocks,
                        int32_t interval, uint64_t seed, uint64_t first_step, uint32_t flags,
                        int64_t *accepted_counts, int64_t *proposed_counts) {
  if (!e || nblocks < 0 || interval < 0) return SSE_ERR_ARG;
  if (flags & SSE_SWEEP_PLAIN) return fail(e, SSE_ERR_ARG, "sse_sweep_tempering runs batched launches");
  int rc = check_ladders(e, nladders, nrungs, ids);
  if (rc || nladders == 0) return rc;
  cudaSetDevice(e->device);
  PtBuffers b(e);
  rc = pt_alloc(e, b, nladders, nrungs, ids);
  if (rc) return rc;
  const std::vector<int32_t> work(ids, ids + (size_t)nladders * nrungs);
  double ms = 0.0;
  long long launches = 0;
  int first_error = 0;
  std::string err_msg;
  for (int blk = 0; blk < nblocks && !rc; blk++) {
    int r = run_until_done(e, MODE_SWEEP, work, interval, flags);
    ms += e->last_ms;
    launches += e->last_launches;
    if (r == SSE_ERR_INVALID_VERTEX || r == SSE_ERR_WORM_CAP) {
      // walker-level failure: the exchange skips pairs with a stopped walker, the rest go on
      if (!first_error) {
        first_error = r;
        err_msg = e->err;
      }
    } else if (r) {
      rc = r;
      break;
    }
    e->last_launches = 0;
    CUDA_TRY(e, cudaEventRecord(e->ev0, e->stream));
    rc = pt_launch(e, b, nladders, nrungs, seed, first_step + (uint64_t)blk);
    if (rc) break;
    CUDA_TRY(e, cudaEventRecord(e->ev1, e->stream));
    rc = pt_check_err(e, b);
    float t = 0.0f;
    if (!rc && cudaEventElapsedTime(&t, e->ev0, e->ev1) == cudaSuccess) ms += t;
    launches += 1;
  }
  if (!rc && (accepted_counts || proposed_counts)) {
    if (accepted_counts)
      CUDA_TRY(e, cudaMemcpyAsync(accepted_counts, b.acc, sizeof(long long) * b.npairs, cudaMemcpyDeviceToHost,
                                  e->stream));
    if (proposed_counts)
      CUDA_TRY(e, cudaMemcpyAsync(proposed_counts, b.prop, sizeof(long long) * b.npairs, cudaMemcpyDeviceToHost,
                                  e->stream));
    CUDA_TRY(e, cudaStreamSynchronize(e->stream));
  }
  e->last_ms = ms;
  e->last_launches = launches;
  if (rc) return rc;
  if (first_error) return fail(e, first_error, err_msg);
  return SSE_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free sweep (sse_sweep_noalloc): the scratch of k_walk and the tables
// derived from the model live in one static device array.
// ---------------------------------------------------------------------------

namespace {

// ==== noalloc kernels: begin (device code only down to the matching end marker) ====
struct NoAllocScratch {
  Rec rec[SSE_NOALLOC_MAX_SLOTS];
  int2 chunk[SSE_NOALLOC_MAX_SLOTS / 32];
  int32_t vfirst[SSE_NOALLOC_MAX_SITES];
  int4 bond_info[SSE_NOALLOC_MAX_BONDS];
  Trans trans[SSE_NOALLOC_MAX_TRANSITIONS];
  Outcome outc[SSE_NOALLOC_MAX_OUTCOMES];
  DevType types[SSE_NOALLOC_MAX_TYPES];
  int32_t diag_vc[SSE_NOALLOC_MAX_DIAG];
  int8_t vclass[SSE_NOALLOC_MAX_VERTICES];
  int32_t row_owner[SSE_NOALLOC_MAX_TRANSITIONS];
  double cls_w[128];
  DevModel model;
  DevWalker walker;
  int32_t status;
  int32_t flags[2];
};

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

// Derives the engine's model tables from the caller's flat tables (device pointers) and
// loads the caller's walker into the scratch.  One block.  Before anything is derived it checks
// what sse_model_register and sse_walker_import check on the host, so that no later kernel
// indexes outside a table; on failure it writes the status to X->status and to the walker and
// leaves the walker's chain as it was.
__global__ void k_noalloc_prep(NoAllocScratch *X, sse_model_desc d, sse_noalloc_walker *uw, uint32_t *ops,
                               long long ops_capacity, uint8_t *state, double *obs_sum, long long *obs_count,
                               double *obs_last) {
  __shared__ int s_sizes[4];  // ndiag, nvert, ntrans, nout (each at most its limit + 1)
  __shared__ int s_ncls;
  __shared__ int s_bad, s_unsup;
  const int tid = threadIdx.x, nt = blockDim.x;
  const auto clip = [](long long x, int lim) { return (int)(x > lim ? lim + 1 : x); };
  if (tid == 0) {
    X->status = SSE_OK;
    s_bad = 0;
    s_unsup = 0;
    long long ndiag = 0, nvert = 0, ntrans = 0;
    for (int t = 0; t < d.ntypes; t++) {
      const int d0 = d.type_dims[2 * t], d1 = d.type_dims[2 * t + 1];
      const int nv = d.type_nverts[t], mw = d.type_maxworm[t];
      const int doff = d.type_diag_off[t], voff = d.type_vert_off[t], toff = d.type_trans_off[t];
      // maxworm and the dimensions share one packed word in the compact records (8 bits each)
      if (d0 < 2 || d1 < 2 || d0 > 255 || d1 > 255 || mw < 1 || mw > 255 || nv < 1 || nv > 512 || doff < 0 ||
          voff < 0 || toff < 0) {
        X->status = SSE_ERR_ARG;
        continue;
      }
      ndiag = max(ndiag, (long long)doff + d0 * d1);
      nvert = max(nvert, (long long)voff + nv);
      ntrans = max(ntrans, (long long)toff + (long long)nv * 4 * mw);
    }
    s_sizes[0] = clip(ndiag, SSE_NOALLOC_MAX_DIAG);
    s_sizes[1] = clip(nvert, SSE_NOALLOC_MAX_VERTICES);
    s_sizes[2] = clip(ntrans, SSE_NOALLOC_MAX_TRANSITIONS);
    s_sizes[3] = 0;
    if (X->status == SSE_OK && (ndiag > SSE_NOALLOC_MAX_DIAG || nvert > SSE_NOALLOC_MAX_VERTICES ||
                                ntrans > SSE_NOALLOC_MAX_TRANSITIONS))
      X->status = SSE_ERR_CAPACITY;
  }
  __syncthreads();
  if (X->status == SSE_OK) {
    // the outcome table's size: every row that has outcomes ends inside it
    for (int i = tid; i < s_sizes[2]; i += nt) {
      const int st = d.trans_start[i], cnt = d.trans_count[i];
      if (st >= 0 && cnt > 0) atomicMax(&s_sizes[3], clip((long long)st + cnt, SSE_NOALLOC_MAX_OUTCOMES));
    }
  }
  __syncthreads();
  if (tid == 0 && X->status == SSE_OK) {
    if (s_sizes[3] > SSE_NOALLOC_MAX_OUTCOMES) X->status = SSE_ERR_CAPACITY;
  }
  __syncthreads();
  if (X->status != SSE_OK) {
    if (tid == 0) uw->status = X->status;
    return;
  }
  // which bond type owns each transition row (-1: none); a row claimed by two types is refused
  for (int i = tid; i < s_sizes[2]; i += nt) X->row_owner[i] = -1;
  __syncthreads();
  for (int t = 0; t < d.ntypes; t++) {
    const int r0 = d.type_trans_off[t], r1 = r0 + d.type_nverts[t] * 4 * d.type_maxworm[t];
    for (int i = r0 + tid; i < r1; i += nt)
      if (atomicCAS(&X->row_owner[i], -1, t) != -1) s_bad = 1;
  }
  // weight classes of the diagonal vertices, in vertex order (as sse_model_register): with more
  // than 32 classes the diagonal update compares against each vertex's own weight and uses the
  // class (clamped to 127) only to tell a diagonal vertex from an off-diagonal one
  for (int v = tid; v < s_sizes[1]; v += nt) X->vclass[v] = -1;
  __syncthreads();
  if (tid == 0) {
    int ncls = 0;
    for (int t = 0; t < d.ntypes; t++) {
      for (int v = 0; v < d.type_nverts[t]; v++) {
        const int vo = d.type_vert_off[t] + v;
        const uint8_t *ls = d.leg_state + 4 * vo;
        if (ls[0] != ls[2] || ls[1] != ls[3]) continue;
        const double w = d.weight[vo];
        int c = 0;
        while (c < ncls && c < 128 && X->cls_w[c] != w) c++;
        if (c == ncls) {
          if (ncls < 128) X->cls_w[ncls] = w;
          ncls++;
        }
        X->vclass[vo] = (int8_t)min(c, 127);
      }
    }
    s_ncls = ncls;
  }
  __syncthreads();
  // the contents the sweep indexes with: bonds, leg states, the diagonal-vertex table, scatter rows
  // and outcomes and, for a walker past its first call, its opstring and spin state
  for (int b = tid; b < d.nbonds; b += nt) {
    const int s0 = d.bond_sites[2 * b], s1 = d.bond_sites[2 * b + 1], t = d.bond_type[b];
    if (s0 < 0 || s1 < 0 || s0 >= d.nsites || s1 >= d.nsites || s0 == s1 || t < 0 || t >= d.ntypes)
      s_bad = 1;
    else if (d.site_dims[s0] != d.type_dims[2 * t] || d.site_dims[s1] != d.type_dims[2 * t + 1])
      s_bad = 1;
  }
  for (int i = tid; i < d.nsites; i += nt)
    if (d.site_dims[i] < 1 || d.site_dims[i] > d.maxdim) s_bad = 1;
  for (int t = 0; t < d.ntypes; t++) {
    const int d0 = d.type_dims[2 * t], d1 = d.type_dims[2 * t + 1], nv = d.type_nverts[t];
    for (int x = tid; x < 4 * nv; x += nt)
      if (d.leg_state[4 * d.type_vert_off[t] + x] >= ((x & 1) ? d1 : d0)) s_bad = 1;
    for (int st = tid; st < d0 * d1; st += nt) {
      const int vc = d.diag_vertex[d.type_diag_off[t] + st];
      if (vc < 0) continue;
      if (!(vc & 1) || (vc >> 1) >= nv || X->vclass[d.type_vert_off[t] + (vc >> 1)] < 0) s_bad = 1;
    }
    const int r0 = d.type_trans_off[t], r1 = r0 + nv * 4 * d.type_maxworm[t];
    for (int i = r0 + tid; i < r1; i += nt) {
      const int st = d.trans_start[i], cnt = d.trans_count[i];
      if (st < 0 || cnt <= 0) continue;
      if (cnt > 256 || st + 2 >= (1 << 23)) {
        s_unsup = 1;
        continue;
      }
      for (int o = st; o < st + cnt; o++)
        if (d.out_leg[o] < 0 || d.out_leg[o] > 3 || d.out_worm[o] < 1 || d.out_worm[o] > d.type_maxworm[t] ||
            d.out_target[o] < 0 || (d.out_target[o] >> 1) >= nv)
          s_bad = 1;
    }
  }
  // rows with outcomes outside every type's range: the host refuses them too
  for (int i = tid; i < s_sizes[2]; i += nt)
    if (X->row_owner[i] < 0 && d.trans_start[i] >= 0 && d.trans_count[i] > 0) s_bad = 1;
  __syncthreads();
  // the walker's own state, read only once the tables it indexes are known to be valid
  const int phase = uw->phase;
  if (!s_bad && !s_unsup) {
    const double nw = phase == PH_NEW ? uw->init_num_worms : uw->num_worms;
    if ((phase != PH_NEW && phase != PH_WARMUP && phase != PH_READY) || !(uw->T > 0.0) || !(uw->T < INFINITY) ||
        !(nw >= 0.0) || !(nw <= SSE_MAX_WORMS_PER_SWEEP) ||
        (phase != PH_NEW && !(uw->avg_worm_length >= 0.0 && uw->avg_worm_length < INFINITY))) {
      s_bad = 1;
    } else if (phase != PH_NEW) {
      // a walker that went through (part of) Carlo.init! sweeps its own opstring and spin state
      const long long L = uw->L, n = uw->num_operators;
      if (L < 0 || L > ops_capacity || n < 0 || n > L) {
        s_bad = 1;
      } else {
        for (long long p = tid; p < L; p += nt) {
          const uint32_t op = ops[p];
          if (!op) continue;
          const int bond = (int)(op >> 11);
          if (bond >= d.nbonds || !(op & 1u) || (int)((op >> 2) & 0x1FFu) >= d.type_nverts[d.bond_type[bond]])
            s_bad = 1;
        }
      }
      for (int i = tid; i < d.nsites; i += nt)
        if (state[i] >= d.site_dims[i]) s_bad = 1;
    }
  }
  __syncthreads();
  if (s_bad || s_unsup) {
    if (tid == 0) {
      X->status = s_bad ? SSE_ERR_ARG : SSE_ERR_UNSUPPORTED;
      uw->status = X->status;
    }
    return;
  }
  for (int t = tid; t < d.ntypes; t += nt) {
    DevType &x = X->types[t];
    x.d0 = d.type_dims[2 * t];
    x.d1 = d.type_dims[2 * t + 1];
    x.nverts = d.type_nverts[t];
    x.maxworm = d.type_maxworm[t];
    x.diag_off = d.type_diag_off[t];
    x.vert_off = d.type_vert_off[t];
    x.trans_off = d.type_trans_off[t];
    x.pad = 0;
  }
  for (int b = tid; b < d.nbonds; b += nt)
    X->bond_info[b] = make_int4(d.bond_sites[2 * b], d.bond_sites[2 * b + 1], d.bond_type[b], 0);
  // diagonal vertices tagged with their weight class, type by type (a later type wins where two
  // types' ranges overlap, as on the host)
  for (int i = tid; i < s_sizes[0]; i += nt) X->diag_vc[i] = -1;
  for (int t = 0; t < d.ntypes; t++) {
    __syncthreads();
    const int nst = d.type_dims[2 * t] * d.type_dims[2 * t + 1];
    for (int st = tid; st < nst; st += nt) {
      const int i = d.type_diag_off[t] + st;
      const int vc = d.diag_vertex[i];
      X->diag_vc[i] = vc >= 0 ? (vc | ((int)X->vclass[d.type_vert_off[t] + (vc >> 1)] << 16)) : -1;
    }
  }
  for (int o = tid; o < s_sizes[3]; o += nt) {
    const double cum = d.out_cum[o];
    unsigned long long thr = 0ull;
    if (cum >= 1.0) thr = 1ull << 53;
    else if (cum > 0.0) thr = (unsigned long long)ceil(cum * 0x1.0p53);
    X->outc[o].thr = thr;
    X->outc[o].packed = d.out_leg[o] | (d.out_worm[o] << 2) | (d.out_target[o] << 10);
    X->outc[o].pad = 0;
  }
  __syncthreads();
  for (int i = tid; i < s_sizes[2]; i += nt) {
    const int st = d.trans_start[i], cnt = d.trans_count[i];
    Trans &tr = X->trans[i];
    if (st < 0 || cnt <= 0) {
      tr.thr0 = 0;
      tr.packed0 = -1;
      tr.rest = 0;
      tr.thr1 = 0;
      tr.packed1 = -1;
      tr.pad = 0;
    } else {
      const int t = X->row_owner[i];
      for (int o = st; o < st + cnt; o++) {
        const int leg = X->outc[o].packed & 3;
        const int dim_out = (leg & 1) ? d.type_dims[2 * t + 1] : d.type_dims[2 * t];
        const int worm_out = (X->outc[o].packed >> 2) & 0xFF;
        X->outc[o].packed = (X->outc[o].packed & 0xFFFFF) | (((dim_out - worm_out) & 0xFF) << 20);
      }
      tr.thr0 = X->outc[st].thr;
      tr.packed0 = X->outc[st].packed;
      tr.thr1 = cnt > 1 ? X->outc[st + 1].thr : 0;
      tr.packed1 = cnt > 1 ? X->outc[st + 1].packed : -1;
      tr.pad = 0;
      tr.rest = cnt > 2 ? (((st + 2) << 8) | (cnt - 2)) : 0;
    }
  }
  if (tid == 0) {
    DevModel &m = X->model;
    m.nsites = d.nsites;
    m.nbonds = d.nbonds;
    m.ntypes = d.ntypes;
    m.maxdim = d.maxdim;
    m.nest = d.nest;
    m.nobs = 6 + 5 * d.nest;
    m.energy_offset = d.energy_offset;
    m.norm_site_count = d.norm_site_count;
    m.bond_info = X->bond_info;
    m.site_dims = d.site_dims;
    m.types = X->types;
    m.diag_vertex = d.diag_vertex;
    m.weight = d.weight;
    m.sign = d.sign;
    m.leg_state = d.leg_state;
    m.diag_vc = X->diag_vc;
    m.vclass = X->vclass;
    m.cls_w = X->cls_w;
    m.ncls = s_ncls;
    m.one_worm = 0;  // the general chase and slot-order measurement paths
    m.est_int = 0;
    m.trans = X->trans;
    m.outc = X->outc;
    m.est_coef = d.est_coef;
    DevWalker &w = X->walker;
    memset(&w, 0, sizeof w);
    w.ops = ops;
    w.rec = X->rec;
    w.chunk = X->chunk;
    w.vfirst = X->vfirst;
    w.state = state;
    w.obs_sum = obs_sum;
    w.obs_last = obs_last;
    w.obs_count = obs_count;
    w.cap = ops_capacity;
    w.L = uw->L;
    w.n = uw->num_operators;
    w.ctr = uw->rng_counter;
    w.T = uw->T;
    w.num_worms = uw->phase == PH_NEW ? uw->init_num_worms : uw->num_worms;
    w.avg_len = uw->phase == PH_NEW ? 1.0 : uw->avg_worm_length;
    w.att = uw->num_worms_attenuation_factor;
    w.target_frac = uw->target_worm_length_fraction;
    w.seed = uw->seed;
    w.stream = uw->stream;
    w.therm = uw->thermalization;
    w.sweeps = uw->sweeps;
    long long cut = uw->init_opstring_cutoff;
    if (cut < 0) cut = (long long)nearbyint((double)d.nsites * uw->T);
    w.init_cutoff = cut;
    w.slot_visits = uw->slot_visits;
    w.worm_steps = uw->worm_steps;
    w.worm_undos = uw->worm_undos;
    w.model = 0;
    w.phase = uw->phase == PH_READY ? PH_READY : (uw->phase == PH_WARMUP ? PH_WARMUP : PH_NEW);
    w.warmup = uw->diagonal_warmup_sweeps;
    w.warmup_done = uw->warmup_done;
    if (w.phase == PH_NEW && cut > ops_capacity) {
      X->status = SSE_ERR_CAPACITY;
      uw->status = SSE_ERR_CAPACITY;
      uw->need_capacity = cut;
    }
    X->flags[0] = X->flags[1] = 0;
  }
}

// Copies the walker back to the caller and leaves its status in X->status.
__global__ void k_noalloc_finish(NoAllocScratch *X, sse_noalloc_walker *uw) {
  const DevWalker &w = X->walker;
  uw->L = w.L;
  uw->num_operators = w.n;
  uw->sweeps = w.sweeps;
  uw->rng_counter = w.ctr;
  uw->num_worms = w.num_worms;
  uw->avg_worm_length = w.avg_len;
  uw->phase = w.phase;
  uw->warmup_done = w.warmup_done;
  uw->slot_visits = w.slot_visits;
  uw->worm_steps = w.worm_steps;
  uw->worm_undos = w.worm_undos;
  int st = w.status;
  if (st == ST_NEED_GROW) {
    st = SSE_ERR_CAPACITY;
    uw->need_capacity = w.need_L;
  } else {
    uw->need_capacity = 0;
  }
  uw->status = st;
  X->status = st;
}

// ==== noalloc kernels: end ====
void *g_noalloc_ptr[64];
bool g_noalloc_ready[64];

}  // namespace

extern "C" int sse_sweep_noalloc(const sse_model_desc *model, sse_noalloc_walker *walker, uint32_t *ops,
                                 int64_t ops_capacity, uint8_t *state, double *obs_sum, int64_t *obs_count,
                                 double *obs_last, int32_t nsweeps, uint32_t flags) {
  if (!model || !walker || !ops || !state || !obs_sum || !obs_count || !obs_last || nsweeps < 0) return SSE_ERR_ARG;
  if (ops_capacity < 1 || ops_capacity > SSE_NOALLOC_MAX_SLOTS || model->nsites < 1 ||
      model->nsites > SSE_NOALLOC_MAX_SITES || model->nbonds < 1 || model->nbonds > SSE_NOALLOC_MAX_BONDS ||
      model->ntypes < 1 || model->ntypes > SSE_NOALLOC_MAX_TYPES)
    return SSE_ERR_CAPACITY;
  if (model->maxdim < 2 || model->maxdim > 255 || model->nest < 0) return SSE_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return SSE_ERR_CUDA;
  // once per device, with that device current: the device address of the static scratch array
  if (!g_noalloc_ready[dev]) {
    void *ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return SSE_ERR_CUDA;
    g_noalloc_ptr[dev] = ptr;
    g_noalloc_ready[dev] = true;
  }
  NoAllocScratch *X = reinterpret_cast<NoAllocScratch *>(g_noalloc_ptr[dev]);
  k_noalloc_prep<<<1, 256>>>(X, *model, walker, ops, (long long)ops_capacity, state, obs_sum,
                             reinterpret_cast<long long *>(obs_count), obs_last);
  if (cudaGetLastError() != cudaSuccess) return SSE_ERR_CUDA;
  int st = SSE_OK;
  if (cudaMemcpyFromSymbol(&st, g_noalloc_scratch, sizeof(int), offsetof(NoAllocScratch, status)) != cudaSuccess)
    return SSE_ERR_CUDA;
  if (st != SSE_OK) return st;
  const int spw = warp_area_bytes(model->nsites) + (int)sizeof(SiteTable);
  const int smem = std::max(spw, 48 * 1024);
  const DevModel *dm = &X->model;
  DevWalker *dw = &X->walker;
  int *dflags = X->flags;
  // The shared-memory attribute belongs to the k_walk instantiations the engine launches too.  Changing
  // it here is safe because the engine sets it again before each of its own launches (choose_launch).
  if (cudaFuncSetAttribute(k_walk<MODE_INIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess ||
      cudaFuncSetAttribute(k_walk<MODE_SWEEP>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
    return SSE_ERR_CUDA;
  k_walk<MODE_INIT><<<1, 32, spw>>>(dm, dw, nullptr, 1, 0, nullptr, flags, -1, spw, 0, dflags);
  if (cudaGetLastError() != cudaSuccess) return SSE_ERR_CUDA;
  int wst = 0;
  if (cudaMemcpyFromSymbol(&wst, g_noalloc_scratch, sizeof(int),
                           offsetof(NoAllocScratch, walker) + offsetof(DevWalker, status)) != cudaSuccess)
    return SSE_ERR_CUDA;
  if (wst == SSE_OK)
    k_walk<MODE_SWEEP><<<1, 32, spw>>>(dm, dw, nullptr, 1, 0, nullptr, flags, nsweeps, spw, 0, dflags);
  k_noalloc_finish<<<1, 1>>>(X, walker);
  if (cudaGetLastError() != cudaSuccess) return SSE_ERR_CUDA;
  if (cudaMemcpyFromSymbol(&st, g_noalloc_scratch, sizeof(int), offsetof(NoAllocScratch, status)) != cudaSuccess)
    return SSE_ERR_CUDA;
  return st;
}

/*
 * libssegpu -- C ABI of the GB300 SSE update engine.
 *
 * The engine runs the hot path of lukas-weber/StochasticSeriesExpansion.jl,
 * one Carlo.jl MC step per walker:
 *
 *     Carlo.sweep!(mc, ctx)    src/sse.jl:62-68
 *         diagonal_update      src/sse.jl:137-191
 *         make_vertex_list!    src/vertex_list.jl:15-54
 *         worm_update          src/sse.jl:193-303, scatter src/vertex_data.jl:106-125
 *     Carlo.measure!(mc, ctx)  src/sse.jl:70-87, 305-376 (+ MagnetizationEstimator)
 *
 * for many independent walkers (Markov chains) on one GPU.  The library owns
 * all device memory and one CUDA stream per engine; every call below is
 * synchronous with respect to the host and returns an sse_status code.  No
 * exception crosses the boundary; sse_engine_last_error() describes the last
 * failure.  One host thread per engine.
 *
 * Random numbers: walker w with key `seed` and id `stream` draws its i-th
 * 64-bit value from Philox4x32-10(counter = (i/2, stream), key = seed), words
 * (0,1) for even i and (2,3) for odd i.  rand() = (u >> 11) * 2^-53 and
 * rand(1:m) = 1 + floor(u*m / 2^64).  A walker's trajectory therefore depends
 * only on its own (seed, stream) and inputs, never on the batch it runs in.
 *
 * Operator codes (uint32): 0 = identity; bit 0 = 1 otherwise, bit 1 =
 * diagonal, bits 2..10 = vertex index (0-based), bits 11..31 = bond (0-based).
 * Spin states are 0-based uint8 (the reference's StateIndex minus one).
 */
#ifndef SSE_GPU_H
#define SSE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SSE_GPU_ABI_VERSION 3

typedef enum sse_status {
  SSE_OK = 0,
  SSE_ERR_ARG = 1,            /* bad argument (null pointer, unknown id, size out of range) */
  SSE_ERR_CUDA = 2,           /* a CUDA runtime call failed */
  SSE_ERR_CAPACITY = 3,       /* a walker needs more memory than allowed */
  SSE_ERR_INVALID_VERTEX = 4, /* scatter found no outgoing step (src/vertex_data.jl:124) */
  SSE_ERR_TIMEOUT = 5,        /* a bounded device wait gave up */
  SSE_ERR_NOMEM = 6,          /* device or host allocation failed */
  SSE_ERR_STATE = 7,          /* call not valid in the walker's current state */
  SSE_ERR_WORM_CAP = 8,       /* a worm exceeded the step cap (64 * max(L + 16, 65536) unless set otherwise) */
  SSE_ERR_UNSUPPORTED = 9     /* model outside the engine's limits */
} sse_status;

typedef struct sse_engine sse_engine;

/*
 * Flat model tables (the SSEData of src/sse_data.jl with its VertexData of
 * src/vertex_data.jl:13-28, plus the magnetisation-estimator coefficients).
 * Replaces the reference's `generate_sse_data(model)` output
 * (src/abstract_model.jl:31-40, src/models/magnet/magnet.jl:169-184).
 * All arrays are copied to the device by sse_model_register.
 * Limits: two-site bonds only (leg count 4), < 2^21 bonds, <= 512 vertices
 * per bond type, site dimension <= 255.
 */
typedef struct sse_model_desc {
  int32_t nsites, nbonds, ntypes, maxdim, nest;
  double energy_offset;   /* SSEData.energy_offset (sum over bonds) */
  double norm_site_count; /* normalization_site_count(model) */
  const int32_t *site_dims;      /* [nsites] */
  const int32_t *bond_type;      /* [nbonds] 0-based type */
  const int32_t *bond_sites;     /* [2*nbonds] 0-based sites */
  const int32_t *type_dims;      /* [2*ntypes] */
  const int32_t *type_nverts;    /* [ntypes] */
  const int32_t *type_maxworm;   /* [ntypes] */
  const int32_t *type_diag_off;  /* [ntypes] offset into diag_vertex */
  const int32_t *type_vert_off;  /* [ntypes] offset into weight/sign and 4x leg_state */
  const int32_t *type_trans_off; /* [ntypes] offset into trans_start/trans_count */
  const int32_t *diag_vertex;    /* vertex code (diag | idx << 1) for compound state s0 + d0*s1, or -1 */
  const double *weight;
  const int8_t *sign;
  const uint8_t *leg_state;      /* [vertex*4 + leg], 0-based states */
  const int32_t *trans_start;    /* [(v*4 + leg)*maxworm + worm-1] first outcome, -1 invalid */
  const int32_t *trans_count;    /* number of outcomes */
  const double *out_cum;         /* cumulative probabilities */
  const int32_t *out_target;     /* vertex code after the step */
  const int8_t *out_leg;         /* outgoing leg, 0-based */
  const int8_t *out_worm;        /* outgoing worm, 1-based */
  const double *est_coef;        /* [(e*nsites + site)*maxdim + s] staggered sign * magnetization_state */
} sse_model_desc;

/* MC(params) + the SSE-level task parameters of docs/src/parameters.md (src/sse.jl:26-45) */
typedef struct sse_walker_params {
  double T;
  uint64_t seed;
  uint64_t stream;
  int64_t init_opstring_cutoff;        /* < 0: round(nsites*T), ties to even */
  int32_t diagonal_warmup_sweeps;      /* reference default 5 */
  double init_num_worms;               /* reference default 5 */
  double num_worms_attenuation_factor; /* reference default 0.01 */
  double target_worm_length_fraction;  /* reference default 2.0 */
  int64_t thermalization;              /* Carlo thermalization sweeps */
} sse_walker_params;

/* scalar walker state: the checkpoint fields of src/sse.jl:89-107 plus the replay counter */
typedef struct sse_walker_info {
  int64_t L;             /* opstring cutoff, length(mc.operators) */
  int64_t num_operators; /* mc.num_operators */
  int64_t capacity;      /* device slots reserved for the opstring */
  int64_t sweeps;        /* Carlo ctx.sweeps */
  uint64_t rng_counter;  /* draws consumed */
  double num_worms;
  double avg_worm_length;
  double T;
  int32_t status;        /* sse_status of the walker's last device work */
  int32_t model;
  int64_t resize_after_thermalization; /* count of "spin array resized after thermalization" */
  int64_t slot_visits;   /* diagonal-update slot visits, cumulative */
  int64_t worm_steps;    /* worm vertex visits (scatter calls), cumulative */
  int64_t phase_cycles[4]; /* SM clock cycles in diagonal update, linking, worm update, measurement */
  int64_t worm_undos;    /* thermalisation sweeps whose worm phase was undone at the worm step cap */
} sse_walker_info;

/* sse_sweep flags */
#define SSE_SWEEP_MEASURE 1u /* Carlo.measure! after every sweep that leaves the walker thermalized */
#define SSE_SWEEP_PLAIN 2u   /* one kernel launch per walker per sweep (the unbatched path) */
#define SSE_SWEEP_GRAPH 4u   /* replay the sweep block from a captured CUDA graph */

/* ---- engine ---- */
int sse_engine_create(int32_t device, sse_engine **out);
int sse_engine_destroy(sse_engine *eng);
const char *sse_engine_last_error(const sse_engine *eng);
int sse_abi_version(void);

/* ---- models: replaces generate_sse_data / SSEData (src/sse_data.jl:34-42) ---- */
int sse_model_register(sse_engine *eng, const sse_model_desc *desc, int32_t *model_id);
/* number of observables per walker of a model: 6 + 5*nest (names in the same order as
 * Sign, OperatorCount, SignOperatorCount, SignOperatorCount2, SignEnergy, WormLengthFraction,
 * then per estimator SignMag, SignAbsMag, SignMag2, SignMag4, SignMagChi) */
int sse_model_nobs(sse_engine *eng, int32_t model_id, int32_t *nobs);

/* A sweep runs ceil(num_worms) worms (src/sse.jl:195-198); creation, import and the allocation-free
 * entry point refuse a worm count outside [0, SSE_MAX_WORMS_PER_SWEEP] with SSE_ERR_ARG. */
#define SSE_MAX_WORMS_PER_SWEEP 2147483648.0 /* 2^31 */

/* ---- walkers: replaces MC(params) (src/sse.jl:26-45) ----
 * Refuses (before allocating anything) T that is not positive and finite, negative warm-up sweeps,
 * an initial worm count outside [0, SSE_MAX_WORMS_PER_SWEEP] (SSE_ERR_ARG), and an initial cutoff
 * whose opstring would reach 2^29 slots, the limit of the engine's 32-bit links and slot indices
 * (SSE_ERR_CAPACITY). */
int sse_walkers_create(sse_engine *eng, int32_t model_id, int32_t count, const sse_walker_params *params,
                       int32_t *ids);
int sse_walkers_destroy(sse_engine *eng, int32_t count, const int32_t *ids);
/* reserve opstring capacity up front so that no regrowth happens later */
int sse_walkers_reserve(sse_engine *eng, int32_t count, const int32_t *ids, int64_t capacity);

/* ---- Carlo.init! (src/sse.jl:47-60) ---- */
int sse_walkers_init(sse_engine *eng, int32_t count, const int32_t *ids);

/* ---- Carlo.sweep! + Carlo.measure! (src/sse.jl:62-87), nsweeps Carlo steps per walker:
 *      is_thermalized = sweeps > thermalization; sweep!; sweeps += 1;
 *      measure! if SSE_SWEEP_MEASURE and sweeps > thermalization ---- */
int sse_sweep(sse_engine *eng, int32_t count, const int32_t *ids, int32_t nsweeps, uint32_t flags);

/* as sse_sweep, with its own number of Carlo steps for every walker (nsweeps[i] >= 0), all in one
 * persistent launch: the continuous-batching step of a request loop */
int sse_sweep_each(sse_engine *eng, int32_t count, const int32_t *ids, const int32_t *nsweeps, uint32_t flags);

/* observable sums/counts/last values, nobs per walker, walker-major; reset clears sums and counts */
int sse_observables(sse_engine *eng, int32_t count, const int32_t *ids, double *sums, int64_t *counts, double *last,
                    int32_t reset);

/* ---- walker state: Carlo.write_checkpoint / read_checkpoint (src/sse.jl:89-107) ---- */
int sse_walker_info_get(sse_engine *eng, int32_t id, sse_walker_info *info);
/* ops: at least info.L entries; state: nsites entries */
int sse_walker_export(sse_engine *eng, int32_t id, uint32_t *ops, int64_t ops_len, uint8_t *state,
                      sse_walker_info *info);
/* sets L, num_operators, sweeps, rng_counter, num_worms, avg_worm_length from info; capacity grows as needed.
 * Refuses operators, spin states, num_worms outside [0, SSE_MAX_WORMS_PER_SWEEP] and a negative or
 * infinite avg_worm_length with SSE_ERR_ARG, leaving the walker unchanged. */
int sse_walker_import(sse_engine *eng, int32_t id, const uint32_t *ops, const uint8_t *state,
                      const sse_walker_info *info);

/* ---- the vertex list of a walker's current opstring, reference layout (src/vertex_list.jl:1-54):
 *      vertices[4*p + leg] = 4*p' + leg' or -1 (L*4 entries), v_first/v_last per site ---- */
int sse_vertex_list(sse_engine *eng, int32_t id, int32_t *vertices, int32_t *v_first, int32_t *v_last);

/* ---- instrumentation ---- */
/* device time (ms) of the kernels of the last sse_sweep / sse_walkers_init, and the number of kernel launches */
int sse_last_timing(sse_engine *eng, double *ms, int64_t *launches);
/* launch shape of the batched kernel: warps (walkers) per block, 1..4; 0 = automatic (4) */
int sse_set_launch(sse_engine *eng, int32_t warps_per_block, int32_t blocks_per_sm);
int sse_get_launch(sse_engine *eng, int32_t *warps_per_block, int32_t *blocks_per_sm);
/* shared-memory staging: a walker whose compacted operator records (32 bytes per non-identity
 * operator) fit in stage_bytes runs its worm update on a copy in shared memory instead of chasing
 * links through HBM; 0 (default) turns it off.  Every warp of the sweep kernel then holds
 * stage_bytes of shared memory, which lowers the number of resident walkers. */
#define SSE_MAX_STAGE_BYTES (192 * 1024)
int sse_set_staging(sse_engine *eng, int32_t stage_bytes);
int sse_get_staging(sse_engine *eng, int32_t *stage_bytes);
/* times nsweeps_probe sweeps of the given walkers for each launch shape (1, 2, 4 walkers per block)
 * and staging budget (off, 8 KB, 32 KB, and room for the 25th-percentile, median and largest walker's
 * records)
 * and keeps the fastest; the probe sweeps are ordinary Carlo steps of those walkers (run it during
 * thermalisation) */
int sse_autotune(sse_engine *eng, int32_t count, const int32_t *ids, int32_t nsweeps_probe, uint32_t flags,
                 int32_t *best_warps_per_block, int32_t *best_stage_bytes, double *best_ms);
/* as sse_autotune, each probe an sse_sweep_each with nsweeps[i] Carlo steps for walker i (the
 * cost-balanced blocks of an uneven batch) */
int sse_autotune_each(sse_engine *eng, int32_t count, const int32_t *ids, const int32_t *nsweeps, uint32_t flags,
                      int32_t *best_warps_per_block, int32_t *best_stage_bytes, double *best_ms);
/* brackets a profiled region (cudaProfilerStart / cudaProfilerStop) for profilers started with
 * collection off; start != 0 opens the region, 0 closes it */
int sse_profiler_range(sse_engine *eng, int32_t start);

/* ---- invariant check (test/test_sse.jl:5-28, isconsistent) ----
 * For each walker: propagating its spin state through its opstring, every operator's lower legs
 * match the state they meet and the state after the last operator is the initial one (periodic
 * imaginary time); every operator's bond and vertex exist; the operator count is num_operators.
 * result[i]: 0 consistent, 1 sizes (L, num_operators, capacity), 2 invalid operator, 3 operator
 * count, 4 leg state mismatch, 5 not periodic, 6 spin state outside its site's dimension. */
int sse_check_walkers(sse_engine *eng, int32_t count, const int32_t *ids, int32_t *result);

/* ---- worm step cap (no counterpart in the reference, whose worm_traverse! has no limit) ----
 * A worm that has not closed after factor * max(L + 16, 65536) steps
 *  - in a thermalisation sweep (sweeps <= thermalization) undoes the sweep's worm phase: the
 *    opstring returns to its state after the diagonal update, the worm-count controller and the
 *    spin state stay as they were, the draws the worms consumed stay consumed, worm_undos counts
 *    it, and the walker goes on (thermalisation sweeps need no detailed balance);
 *  - in a measured sweep stops its walker with SSE_ERR_WORM_CAP (the walker keeps that status;
 *    the other walkers go on).
 * The default factor is 64, so the cap is at least about 4.2 million steps.  With S >= 1 and
 * cluster-basis vertex tables, worms of the first thermalisation sweeps (while L is still small)
 * can run for orders of magnitude longer than the opstring before they close, over 10^9 steps in
 * some chains; the cap bounds how long one walker holds up its batch.  Small systems at low
 * temperature run worms of hundreds of times L + 16 even after thermalisation, hence the minimum
 * of 65536 slots.  A smaller factor undoes or stops long worms sooner and more often. */
int sse_walkers_set_worm_cap(sse_engine *eng, int32_t count, const int32_t *ids, int32_t factor);

/* ---- parallel tempering between resident walkers (src/sse.jl:390-405) ----
 *
 * Carlo.parallel_tempering_change_parameter!(mc, :T, T): sets the walker's temperature. */
int sse_walker_set_T(sse_engine *eng, int32_t id, double T);

/* One exchange step over nladders ladders of nrungs walkers (2 <= nrungs <= 1024); ladder l is
 * ids[l*nrungs .. l*nrungs + nrungs - 1] in any order, all of one model, with distinct temperatures;
 * a walker may appear in one ladder only.  Within a ladder the walkers are ranked by their current T
 * (ascending) and `step` proposes the rung pairs (k, k+1) with k = step (mod 2).  For a pair (a, b),
 * T_a < T_b, the swap weight is exp(lwr(a, T_b) + lwr(b, T_a)) with Carlo's
 * parallel_tempering_log_weight_ratio lwr(mc, T') = -num_operators * log(T'/T), i.e.
 * q = (T_a/T_b)^(n_a - n_b), computed as an integer power by binary powering of the correctly
 * rounded quotient (T_a/T_b if n_a >= n_b, else T_b/T_a).  The swap is accepted when u < q with
 * u = (x >> 11) * 2^-53, x = words (0,1) of Philox4x32-10(counter = (step, k, l), key = seed).
 * An accepted swap exchanges the two walkers' temperatures and their observable accumulators
 * (sums, counts, last values), so a walker's accumulators always hold the measurements taken at
 * its current temperature.  Pairs with a walker whose status is not SSE_OK are not proposed.
 * accepted (may be NULL): nladders*(nrungs-1) entries, pair k of ladder l at l*(nrungs-1) + k:
 * 1 accepted, 0 rejected, -1 not proposed. */
int sse_tempering_exchange(sse_engine *eng, int32_t nladders, int32_t nrungs, const int32_t *ids, uint64_t seed,
                           uint64_t step, int32_t *accepted);

/* nblocks times: `interval` Carlo steps of every ladder walker (as sse_sweep with `flags`), then
 * sse_tempering_exchange with step first_step + block.  accepted_counts / proposed_counts (may be
 * NULL): nladders*(nrungs-1) entries, this call's accepted and proposed swaps per rung pair.
 * A walker that stops (SSE_ERR_WORM_CAP, SSE_ERR_INVALID_VERTEX) leaves the others running; the
 * call then returns its status after the last block. */
int sse_sweep_tempering(sse_engine *eng, int32_t nladders, int32_t nrungs, const int32_t *ids, int32_t nblocks,
                        int32_t interval, uint64_t seed, uint64_t first_step, uint32_t flags,
                        int64_t *accepted_counts, int64_t *proposed_counts);

/* ---- allocation-free sweep (no counterpart in the reference) ----
 *
 * For callers that cannot call cudaMalloc: code that lives inside a host
 * whose device memory belongs to someone else's pool (a Julia CUDA.jl or
 * PyTorch caching allocator, a serving process with a fixed memory budget),
 * and latency-critical loops that cannot afford the implicit device
 * synchronisation of cudaMalloc/cudaFree.  The caller owns every input and
 * output buffer in device memory; the per-sweep scratch (compacted operator
 * records, slot index, per-site heads) and the tables derived from the model
 * live in one static device array of about 13 MB (its size follows from the
 * SSE_NOALLOC_MAX_* limits below), which every GPU that loads this library
 * holds until the process exits.
 *
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  All calls share the one array and leave the
 * last call's contents in it; everything a call reads from it is rewritten
 * by that call first.  Calls whose device work overlaps (several host
 * threads, several streams) race on the array and must be serialised by the
 * caller.  The call is synchronous and returns the walker's sse_status.
 *
 * Streams: the call launches its kernels on the legacy default stream and
 * waits for them before it returns.  The legacy default stream is ordered
 * after work on ordinary (blocking) streams, but not after work on streams
 * created with cudaStreamNonBlocking -- PyTorch's side streams, CUDA.jl's
 * per-task streams and most library streams are of that kind.  A caller
 * whose buffers (model tables, walker, opstring, state, observables) were
 * written on such a stream must synchronise that stream before the call.
 *
 * Input checks: before it sweeps, the call checks on the device what the
 * engine's sse_model_register and sse_walker_import check on the host --
 * bond sites and types, type sizes and table offsets, leg states, the
 * diagonal-vertex table, every transition row and scatter outcome, and for a
 * walker past Carlo.init! its cutoff, opstring and spin state -- and returns
 * SSE_ERR_ARG (SSE_ERR_UNSUPPORTED for a transition row longer than 256
 * outcomes) without touching the walker's chain when one fails. */
#define SSE_NOALLOC_MAX_SLOTS (1 << 18)    /* opstring capacity (cutoff L) */
#define SSE_NOALLOC_MAX_SITES (1 << 14)
#define SSE_NOALLOC_MAX_BONDS (1 << 16)
#define SSE_NOALLOC_MAX_TYPES 64
#define SSE_NOALLOC_MAX_VERTICES 4096      /* summed over bond types */
#define SSE_NOALLOC_MAX_DIAG 4096          /* summed d0*d1 over bond types */
#define SSE_NOALLOC_MAX_TRANSITIONS (1 << 16)
#define SSE_NOALLOC_MAX_OUTCOMES (1 << 16)

/* one walker for sse_sweep_noalloc, kept by the caller in device memory */
typedef struct sse_noalloc_walker {
  /* parameters, as sse_walker_params */
  double T;
  uint64_t seed;
  uint64_t stream;
  int64_t init_opstring_cutoff;
  int32_t diagonal_warmup_sweeps;
  int32_t phase;       /* 0: Carlo.init! still to run (set by the caller), 1: its diagonal warm-up
                          sweeps under way (left by a call stopped for capacity), 2: initialised;
                          any other value is refused with SSE_ERR_ARG */
  double init_num_worms;
  double num_worms_attenuation_factor;
  double target_worm_length_fraction;
  int64_t thermalization;
  /* chain state, updated by every call */
  int64_t L;
  int64_t num_operators;
  int64_t sweeps;
  uint64_t rng_counter;
  double num_worms;
  double avg_worm_length;
  int32_t warmup_done;
  int32_t status;        /* sse_status of the last call */
  int64_t need_capacity; /* with SSE_ERR_CAPACITY: opstring slots the walker needs next */
  int64_t slot_visits;
  int64_t worm_steps;
  int64_t worm_undos;    /* thermalisation worm phases undone at the worm step cap */
} sse_noalloc_walker;

/* Runs Carlo.init! (when walker->phase == 0) and then nsweeps Carlo steps of one walker,
 * like sse_walkers_init + sse_sweep, without allocating anything.
 *   model       host struct whose array pointers are DEVICE pointers to the flat tables
 *   walker      device pointer
 *   ops         device, ops_capacity uint32 slots (<= SSE_NOALLOC_MAX_SLOTS)
 *   state       device, nsites uint8
 *   obs_*       device, 6 + 5*nest entries each (accumulated, never cleared here)
 * Sizes beyond the SSE_NOALLOC_MAX_* limits are rejected with SSE_ERR_CAPACITY.  When the
 * reference's cutoff growth needs more than ops_capacity slots, the walker stops at a sweep
 * boundary with status SSE_ERR_CAPACITY and need_capacity set; grow ops and call again. */
int sse_sweep_noalloc(const sse_model_desc *model, sse_noalloc_walker *walker, uint32_t *ops,
                      int64_t ops_capacity, uint8_t *state, double *obs_sum, int64_t *obs_count,
                      double *obs_last, int32_t nsweeps, uint32_t flags);

#ifdef __cplusplus
}
#endif
#endif

// Device side of the GB300 SSE update engine.
//
// One warp owns one walker (Markov chain) at a time and runs its whole Carlo
// step -- diagonal update, vertex linking, worm update, measurement -- with
// the walker's opstring in HBM and its spin state / per-site link heads in
// shared memory.  Reference functions restated here:
//
//   diagonal_update    src/sse.jl:137-191
//   make_vertex_list!  src/vertex_list.jl:15-54
//   worm_update        src/sse.jl:193-231
//   worm_traverse!     src/sse.jl:233-303, scatter src/vertex_data.jl:106-125
//   measure!           src/sse.jl:70-87, 305-376,
//                      MagnetizationEstimator magnetization_estimator.jl:96-230
//
// Compile with -fmad=false: every floating-point expression that decides an
// accept/reject or feeds the worm-count controller must round exactly as the
// reference's one-operation-at-a-time evaluation.
#pragma once

#include <stdint.h>

namespace sse {

constexpr unsigned FULL = 0xFFFFFFFFu;

// internal walker status codes (public ones are sse_status values)
constexpr int ST_OK = 0;
constexpr int ST_INVALID_VERTEX = 4;
constexpr int ST_TIMEOUT = 5;
constexpr int ST_STATE = 7;
constexpr int ST_WORM_CAP = 8;
// a worm's step cap is cap_factor * max(L + 16, WORM_CAP_MIN_SLOTS)
constexpr long long WORM_CAP_MIN_SLOTS = 1 << 16;
// worm_update only: a thermalisation worm passed the step cap and the sweep's worm phase was
// undone; the caller counts it and carries on with ST_OK (never stored in a walker)
constexpr int ST_WORM_UNDONE = -8;
constexpr int ST_NEED_GROW = 100;

// walker phases
constexpr int PH_NEW = 0;     // spin state not drawn yet
constexpr int PH_WARMUP = 1;  // diagonal warm-up sweeps in progress
constexpr int PH_READY = 2;   // Carlo.init! done

struct __align__(16) DevType {
  int32_t d0, d1, nverts, maxworm;
  int32_t diag_off, vert_off, trans_off, pad;
};

struct DevModel {
  int32_t nsites, nbonds, ntypes, maxdim;
  int32_t nest, nobs, pad0, pad1;
  double energy_offset, norm_site_count;
  const int4 *bond_info;  // (site0, site1, type, 0)
  const int32_t *site_dims;
  const DevType *types;
  const int32_t *diag_vertex;
  const double *weight;
  const int8_t *sign;
  const uint8_t *leg_state;
  const int32_t *diag_vc;   // diag_vertex with the weight class in bits 16+: vcode | cls << 16, or -1
  const int8_t *vclass;     // weight class of every vertex (-1: off-diagonal)
  const double *cls_w;      // weight of each class
  int32_t ncls, pad2, pad3, pad4;
  const int32_t *est_coef2;  // 2 * est_coef as integers when est_int (every coefficient a multiple of 1/2)
  int32_t est_int;
  int32_t one_worm;  // every bond type has maxworm 1 (one worm type): the chase's row index needs no worm
  int32_t pad6, pad7;
  const struct Trans *trans;  // one per (type, vertex, leg_in, worm_in)
  const struct Outcome *outc;
  const double *est_coef;
};

// Scatter tables (src/vertex_data.jl:106-125) with integer thresholds: for
// r = u53 * 2^-53 (u53 = u >> 11) the reference's test `r < cum` holds
// exactly when u53 < ceil(cum * 2^53), so the worm compares integers.
// packed = leg_out | worm_out << 2 | target vertex code << 10 | ((dim_out - worm_out) & 0xFF) << 20,
// dim_out the dimension of the site of leg_out: the worm closes at the exit leg of its start
// operator when worm_out == dim_out - worm_0 (src/worms.jl worm_inverse), i.e. when this field
// equals worm_0 (worm_0 is 1..254, so a table whose worm_out >= dim_out never closes there, as in
// the reference).
struct __align__(16) Outcome {
  unsigned long long thr;
  int32_t packed;
  int32_t pad;
};

// A transition row with its first two outcomes inline (packed1 < 0: the row has
// one); `rest` = index of the third outcome << 8 | number of further outcomes.
// packed0 < 0: invalid row.
struct __align__(32) Trans {
  unsigned long long thr0;
  int32_t packed0;
  int32_t rest;
  unsigned long long thr1;
  int32_t packed1;
  int32_t pad;
};

// One non-identity operator of the compacted opstring, 32 bytes = one DRAM
// sector: its four leg links (4*k' + leg'), its code, its slot, and what the
// worm needs of its bond type (transition-table offset; maxworm | d0 << 8 |
// d1 << 16) so that a worm step costs one dependent DRAM access.
struct __align__(32) Rec {
  int32_t link[4];
  uint32_t op;
  int32_t slot;
  int32_t trans_off;
  int32_t tpack;
};

struct DevWalker {
  // device arrays
  uint32_t *ops;   // [cap]   opstring
  Rec *rec;        // [cap]   compacted operators + links (rebuilt every sweep)
  int2 *chunk;     // [cap/32] per 32-slot chunk: compact index of its first operator, bitmask of
                   //          its operator slots (slot p -> operator chunk.x + popc(bits below p))
  int32_t *vfirst; // [nsites] first leg per site (4k + leg) or -1
  uint8_t *state;  // [nsites]
  double *obs_sum;
  double *obs_last;
  long long *obs_count;
  long long cap;
  // Markov chain
  long long L, n;
  unsigned long long ctr;
  double T, num_worms, avg_len, att, target_frac;
  unsigned long long seed, stream;
  long long therm, sweeps, target;
  long long init_cutoff, need_L;
  long long resize_after_therm, slot_visits, worm_steps;
  long long worm_undos;  // thermalisation worm phases undone at the step cap
  long long cyc[4];  // clock cycles spent in diagonal update, linking, worms, measurement
  int32_t model, status, phase, warmup, warmup_done;
  int32_t cap_factor;  // worm step cap: cap_factor * max(L + 16, WORM_CAP_MIN_SLOTS); 0: 64
};

// ---------------------------------------------------------------------------
// replay stream: Philox4x32-10 (Salmon et al., SC'11)
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint4 philox10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    if (r) {
      k.x += 0x9E3779B9u;
      k.y += 0xBB67AE85u;
    }
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
  }
  return c;
}

__device__ __forceinline__ uint4 philox_block(unsigned long long seed, unsigned long long stream,
                                              unsigned long long blk) {
  return philox10(make_uint4((uint32_t)blk, (uint32_t)(blk >> 32), (uint32_t)stream, (uint32_t)(stream >> 32)),
                  make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
}

__device__ __forceinline__ unsigned long long draw64(unsigned long long seed, unsigned long long stream,
                                                     unsigned long long idx) {
  const uint4 x = philox_block(seed, stream, idx >> 1);
  return (idx & 1ull) ? (((unsigned long long)x.w << 32) | x.z) : (((unsigned long long)x.y << 32) | x.x);
}

// draws idx and idx+1 with one Philox block when idx is even
__device__ __forceinline__ void draw2(unsigned long long seed, unsigned long long stream, unsigned long long idx,
                                      unsigned long long &u1, unsigned long long &u2) {
  const uint4 x = philox_block(seed, stream, idx >> 1);
  if (!(idx & 1ull)) {
    u1 = ((unsigned long long)x.y << 32) | x.x;
    u2 = ((unsigned long long)x.w << 32) | x.z;
  } else {
    u1 = ((unsigned long long)x.w << 32) | x.z;
    const uint4 y = philox_block(seed, stream, (idx >> 1) + 1);
    u2 = ((unsigned long long)y.y << 32) | y.x;
  }
}

__device__ __forceinline__ double u01(unsigned long long u) { return (double)(u >> 11) * 0x1.0p-53; }

// rand(1:m) - 1
__device__ __forceinline__ unsigned long long urange0(unsigned long long u, unsigned long long m) {
  return __umul64hi(u, m);
}

// ---------------------------------------------------------------------------
// tanh for the worm-count controller (src/sse.jl:213).  expm1 by its Taylor
// series below 0.5, otherwise exp by Cody-Waite reduction y = k ln2 + r and a
// degree-13 Taylor polynomial for exp(r).  Only +, -, *, / and floor, with
// coefficients given as exact binary constants (1/k! correctly rounded), so
// the result is the same bit pattern on any IEEE-754 machine without FMA
// contraction.
// ---------------------------------------------------------------------------

__device__ __constant__ double c_inv_fact[20] = {
    0x1.0000000000000p+0,  0x1.0000000000000p+0,  0x1.0000000000000p-1,  0x1.5555555555555p-3,
    0x1.5555555555555p-5,  0x1.1111111111111p-7,  0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13,
    0x1.a01a01a01a01ap-16, 0x1.71de3a556c734p-19, 0x1.27e4fb7789f5cp-22, 0x1.ae64567f544e4p-26,
    0x1.1eed8eff8d898p-29, 0x1.6124613a86d09p-33, 0x1.93974a8c07c9dp-37, 0x1.ae7f3e733b81fp-41,
    0x1.ae7f3e733b81fp-45, 0x1.952c77030ad4ap-49, 0x1.6827863b97d97p-53, 0x1.2f49b46814157p-57};

__device__ inline double expm1_pos(double y) {
  if (y < 0.5) {
    double q = c_inv_fact[17];
    for (int k = 16; k >= 1; k--) q = __dadd_rn(__dmul_rn(q, y), c_inv_fact[k]);
    return __dmul_rn(q, y);
  }
  const double k = floor(__dadd_rn(__dmul_rn(y, 0x1.71547652b82fep+0), 0.5));
  const double r = __dsub_rn(__dsub_rn(y, __dmul_rn(k, 0x1.62e42fee00000p-1)), __dmul_rn(k, 0x1.a39ef35793c76p-33));
  double p = c_inv_fact[13];
  for (int j = 12; j >= 0; j--) p = __dadd_rn(__dmul_rn(p, r), c_inv_fact[j]);
  const double scale = __longlong_as_double((long long)((unsigned long long)((long long)k + 1023) << 52));
  return __dsub_rn(__dmul_rn(p, scale), 1.0);
}

__device__ inline double ctl_tanh(double x) {
  const double ax = fabs(x);
  if (!(ax < 20.0)) {
    if (x > 0) return 1.0;
    if (x < 0) return -1.0;
    return x;
  }
  if (ax == 0.0) return x;
  const double e = expm1_pos(__dmul_rn(2.0, ax));
  const double t = __ddiv_rn(e, __dadd_rn(e, 2.0));
  return x < 0 ? -t : t;
}

// ---------------------------------------------------------------------------
// warp helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned r;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
  return r;
}

__device__ __forceinline__ long long shfl_ll(long long v, int src) {
  return (long long)__shfl_sync(FULL, (unsigned long long)v, src);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(FULL, v, o));
  return v;
}

__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// Chunk-local site table (vertex linking).  A 32-slot chunk touches at most 64 sites; each operator
// lane enters its two sites into a small open-addressing table in the warp's shared memory, with its
// lane bit in the site's mask.  A lane then finds the operators of the chunk on each of its sites --
// the last one before it, whether any comes after it -- from that mask, instead of a loop over every
// operator of the chunk (ncu on 1024 walkers of the 32x32, beta = 16 batch: about 230 instead of 770
// warp instructions per chunk).  Slots are emptied by the lanes that filled them before the next chunk.
// The diagonal update keeps its loop over the chunk's off-diagonal operators (about half as many):
// the table's extra barriers made it slower there.
// ---------------------------------------------------------------------------

constexpr int SITE_TABLE_SLOTS = 128;

struct SiteTable {
  int32_t key[SITE_TABLE_SLOTS];    // site, or -1 when the slot is empty
  uint32_t mask[SITE_TABLE_SLOTS];  // lanes that entered the site
};

// bytes of a warp's shared memory before its site table: spin state (diagonal update), per-site
// link tails (linking) or the worm's 64-draw buffer, whichever is largest
__host__ __device__ inline int warp_area_bytes(int nsites) {
  const int b = 4 * (nsites > 1 ? nsites : 1);
  return ((b > 512 ? b : 512) + 31) & ~31;
}

__device__ __forceinline__ int site_slot(int s) { return (int)(((uint32_t)s * 0x9E3779B1u) >> 25); }

__device__ __forceinline__ void site_table_clear(SiteTable *t, int lane) {
  for (int i = lane; i < SITE_TABLE_SLOTS; i += 32) {
    t->key[i] = -1;
    t->mask[i] = 0u;
  }
}

// Enters site s with this lane's bit; returns the slot.  At most 64 sites in 128 slots, so a free
// slot or the site itself is always found within the probe limit.
__device__ __forceinline__ int site_insert(SiteTable *t, int s, int lane) {
  int h = site_slot(s);
  for (int i = 0; i < SITE_TABLE_SLOTS; i++) {
    const int old = atomicCAS(&t->key[h], -1, s);
    if (old == -1 || old == s) {
      atomicOr(&t->mask[h], 1u << lane);
      return h;
    }
    h = (h + 1) & (SITE_TABLE_SLOTS - 1);
  }
  return -1;
}

__device__ __forceinline__ void site_release(SiteTable *t, int h) {
  t->key[h] = -1;
  t->mask[h] = 0u;
}

// Chain scalars, held identically in every lane of the owning warp.
struct Chain {
  long long L, n, cap;
  unsigned long long ctr, seed, stream;
  double T;
};

// ---------------------------------------------------------------------------
// diagonal update, src/sse.jl:137-191
//
// Slots are processed 32 at a time, one per lane.  Draw indices are an
// exclusive prefix sum of the per-slot draw counts (identity 2, diagonal 1,
// off-diagonal 0), which depend only on the input opstring.  The spin state
// seen by a slot is the shared-memory state before the chunk, patched by the
// earlier off-diagonal operators of the chunk.  The operator count n seen by
// a slot lies in [n - #diagonal before, n + #identity before]; acceptance is
// monotone in n (insertion: (N_b/T)/(L-n)*w grows with n; removal:
// (L-n+1)*(T/N_b) shrinks), so a lane whose decision is equal at both ends
// of its window is fixed, and the rare remaining lanes are resolved in slot
// order with the exact n.  Every decision evaluates the reference's own
// expression at the reference's n, so the result is bit-identical.
//
// Most lanes never touch FP64: with r = u53 * 2^-53, the tests
// `r < q(n)*w` and `r*w < P(n)` are prefixes in u53, so integer thresholds
// computed for the window n_c +- 48 (recomputed when n drifts by more than
// 16) classify a lane as surely accepted or surely rejected for every n its
// chunk can see.  Only lanes between the two thresholds run the exact FP64
// expressions.  Opcodes are loaded two chunks ahead and the next chunk's
// random numbers and bond lookups are issued before the current chunk's
// decisions.
// ---------------------------------------------------------------------------

constexpr unsigned long long U53_ALL = 1ull << 53;

// u53 < thr_lt(X)  <=>  u53 * 2^-53 < X
__device__ __forceinline__ unsigned long long thr_lt(double X) {
  if (!(X > 0.0)) return 0ull;
  if (X >= 1.0) return U53_ALL;
  return (unsigned long long)ceil(__dmul_rn(X, 0x1.0p53));
}

// u53 < result  <=>  fl(u53 * 2^-53 * w) < P, for w > 0 (multiplication by w is monotone).
// Returns `fallback` if the boundary is not found within a few steps of the estimate.
__device__ unsigned long long thr_mul_lt(double w, double P, unsigned long long fallback) {
  if (!(P > 0.0)) return 0ull;
  const double t = __dmul_rn(__ddiv_rn(P, w), 0x1.0p53);
  unsigned long long u = (t < 0x1.0p53) ? (unsigned long long)floor(t) : U53_ALL;
#define PRED(x) (__dmul_rn(__dmul_rn((double)(x), 0x1.0p-53), w) < P)
  for (int it = 0; it < 8 && u < U53_ALL && PRED(u); it++) u++;
  for (int it = 0; it < 8 && u > 0 && !PRED(u - 1); it++) u--;
  const bool ok = (u == 0 || PRED(u - 1)) && (u == U53_ALL || !PRED(u));
#undef PRED
  return ok ? u : fallback;
}

struct DiagStage {  // per-lane data of one chunk after the first pipeline stage
  uint32_t opb;  // the opcode, or for an identity slot its drawn bond << 11
  int kind;      // 0 none, 1 identity, 2 diagonal, 3 off-diagonal
  unsigned long long u53;
  int4 bi;
};

// Stage A: classify the chunk's slots and draw their random numbers.  The chunk
// consumes draws [ctr, ctr + tot); lane l computes Philox block ctr/2 + l (one
// block per lane, no divergence) and every slot fetches its draws with
// shuffles.  At most 33 blocks are needed; the 33rd is computed only when a
// chunk needs it.
__device__ __forceinline__ void diag_stage_a(DiagStage &a, uint32_t op, bool inr, unsigned long long &ctr,
                                             unsigned long long seed, unsigned long long stream, uint32_t nb,
                                             const int4 *__restrict__ bond_info, unsigned lt, int lane) {
  const bool id = inr && op == 0u;
  const bool dg = inr && op != 0u && (op & 2u);
  const bool od = inr && op != 0u && !(op & 2u);
  const unsigned idm = __ballot_sync(FULL, id);
  const unsigned dgm = __ballot_sync(FULL, dg);
  const unsigned tot = 2u * __popc(idm) + __popc(dgm);
  const unsigned long long d0 = ctr + 2u * __popc(idm & lt) + __popc(dgm & lt);
  const unsigned long long b0 = ctr >> 1;
  a.opb = op;
  a.kind = id ? 1 : dg ? 2 : od ? 3 : 0;
  a.u53 = 0;
  if (tot) {
    const uint4 x = philox_block(seed, stream, b0 + lane);
    uint4 x32 = make_uint4(0, 0, 0, 0);
    if (((ctr + tot - 1) >> 1) - b0 >= 32) x32 = philox_block(seed, stream, b0 + 32);
    const int s0 = (int)((d0 >> 1) - b0);  // block of this slot's first draw, 0..32
    const int s1 = s0 + 1;
    const uint32_t p0 = __shfl_sync(FULL, x.x, s0 & 31), p1 = __shfl_sync(FULL, x.y, s0 & 31);
    const uint32_t p2 = __shfl_sync(FULL, x.z, s0 & 31), p3 = __shfl_sync(FULL, x.w, s0 & 31);
    const uint32_t q0 = __shfl_sync(FULL, x.x, s1 & 31), q1 = __shfl_sync(FULL, x.y, s1 & 31);
    const uint4 blk0 = s0 < 32 ? make_uint4(p0, p1, p2, p3) : x32;
    const uint2 blk1 = s1 < 32 ? make_uint2(q0, q1) : make_uint2(x32.x, x32.y);
    unsigned long long u1, u2;
    if (!(d0 & 1ull)) {
      u1 = ((unsigned long long)blk0.y << 32) | blk0.x;
      u2 = ((unsigned long long)blk0.w << 32) | blk0.z;
    } else {
      u1 = ((unsigned long long)blk0.w << 32) | blk0.z;
      u2 = ((unsigned long long)blk1.y << 32) | blk1.x;
    }
    if (id) {
      a.opb = (uint32_t)urange0(u1, (unsigned long long)nb) << 11;
      a.u53 = u2 >> 11;
    } else if (dg) {
      a.u53 = u1 >> 11;
    }
  }
  ctr += tot;
  a.bi = a.kind ? __ldg(bond_info + (a.opb >> 11)) : make_int4(-1, -1, 0, 0);
}

// The exact test of one slot at operator count nj (src/sse.jl:150-186) in FP64, with the reference's
// operations in its order: insertion of the diagonal vertex of weight index vo at an identity slot,
// or removal of a diagonal operator.  Only the rare lanes the integer thresholds cannot classify get
// here, so the two rates are recomputed (bit-identical IEEE divisions) instead of occupying registers
// through the chunk loop (A/B at 4096 walkers of 32x32, beta = 16, with the 32-bit slot indices:
// 201 instead of 230 cycles per slot under load).
__device__ __forceinline__ bool diag_exact(const DevModel &M, const Chain &c, int L, int nj, bool insert,
                                           unsigned long long u53, int vo) {
  const double r = (double)u53 * 0x1.0p-53;
  const double w = M.weight[vo];
  if (insert) return r < __dmul_rn(__ddiv_rn(__ddiv_rn((double)M.nbonds, c.T), (double)(L - nj)), w);
  return __dmul_rn(r, w) < __dmul_rn((double)(L - nj + 1), __ddiv_rn(c.T, (double)M.nbonds));
}

// Per-class integer thresholds for the window n_c +- 48, written by lane cls for class cls (lanes
// below ncls): thr[2 cls] = (insert surely / insert never), thr[2 cls + 1] = (remove surely / never).
__device__ __forceinline__ void diag_thresholds(const DevModel &M, const Chain &c, int L, int n_c,
                                                ulonglong2 *thr, int lane) {
  const double pmake_raw = __ddiv_rn((double)M.nbonds, c.T);
  const double premove_raw = __ddiv_rn(c.T, (double)M.nbonds);
  const double wc = M.cls_w[lane];
  const int nlo = n_c - 48, nhi = n_c + 48;
  const unsigned long long ti_a = thr_lt(__dmul_rn(__ddiv_rn(pmake_raw, (double)(L - nlo)), wc));
  const unsigned long long ti_r =
      (L - nhi > 0) ? thr_lt(__dmul_rn(__ddiv_rn(pmake_raw, (double)(L - nhi)), wc)) : U53_ALL;
  const unsigned long long tr_a = thr_mul_lt(wc, __dmul_rn((double)(L - nhi + 1), premove_raw), 0ull);
  const unsigned long long tr_r = thr_mul_lt(wc, __dmul_rn((double)(L - nlo + 1), premove_raw), U53_ALL);
  thr[2 * lane] = make_ulonglong2(ti_a, ti_r);
  thr[2 * lane + 1] = make_ulonglong2(tr_a, tr_r);
}

// thr: 1 KB of the warp's shared memory (the site table's, idle during this phase) for the per-class
// thresholds.  Slot indices, the cutoff and the operator count are 32-bit here: the engine keeps
// opstrings below 2^29 slots.
__device__ __noinline__ int diag_update(const DevModel &M, Chain &c, uint32_t *__restrict__ ops, uint8_t *sst,
                                        ulonglong2 *thr, bool thermalized, long long &resize_count,
                                        long long &need_L, int lane) {
  if (2 * c.n >= c.L) {
    const long long Lnew = c.L + c.L / 2 + 100;  // floor(1.5 L + 100)
    if (Lnew > c.cap) {
      need_L = Lnew;
      return ST_NEED_GROW;
    }
    for (long long p = c.L + lane; p < Lnew; p += 32) ops[p] = 0u;
    c.L = Lnew;
    if (thermalized) resize_count++;
    __syncwarp();
  }
  const unsigned lt = lanemask_lt();
  const int L = (int)c.L;
  int n = (int)c.n;
  unsigned long long ctr = c.ctr;
  const uint32_t nb = (uint32_t)M.nbonds;
  const unsigned long long seed = c.seed, stream = c.stream;
  const int4 *__restrict__ bond_info = M.bond_info;
  const DevType *__restrict__ types = M.types;
  const int32_t *__restrict__ diag_vc = M.diag_vc;
  const int8_t *__restrict__ vclass = M.vclass;
  const uint8_t *__restrict__ leg_state = M.leg_state;
  const int ncls = M.ncls;
  const bool use_thr = ncls <= 32;

  // per-class integer thresholds (in thr[]), valid while |n - n_c| <= 16
  int n_c = -(1 << 30);

  // two chunks of opcodes in flight, the first chunk's stage A done before the loop
  uint32_t op_n1 = (lane < L) ? ops[lane] : 0u;
  uint32_t op_n2 = (32 + lane < L) ? ops[32 + lane] : 0u;
  DiagStage cur;
  diag_stage_a(cur, op_n1, lane < L, ctr, seed, stream, nb, bond_info, lt, lane);

  for (int base = 0; base < L; base += 32) {
    const int p = base + lane;
    // stage A of the next chunk and the opcode load two chunks ahead
    const uint32_t op_next = op_n2;
    op_n2 = (base + 64 + lane < L) ? ops[base + 64 + lane] : 0u;
    DiagStage nxt;
    diag_stage_a(nxt, op_next, base + 32 + lane < L, ctr, seed, stream, nb, bond_info, lt, lane);

    // stage B of this chunk
    const bool id = cur.kind == 1, dg = cur.kind == 2, od = cur.kind == 3;
    const unsigned idm = __ballot_sync(FULL, id);
    const unsigned dgm = __ballot_sync(FULL, dg);
    const unsigned odm = __ballot_sync(FULL, od);
    const int si = cur.bi.x, sj = cur.bi.y, type = cur.bi.z;
    int vcode = -1, cls = -1, ups = 0;
    if (dg || od) {
      vcode = (int)((cur.opb >> 1) & 0x3FFu);
      const int vo = types[type].vert_off + (vcode >> 1);
      if (dg) cls = vclass[vo];
      else {
        const uchar4 ls = *reinterpret_cast<const uchar4 *>(leg_state + 4 * vo);
        ups = (int)ls.z | ((int)ls.w << 8);
      }
    }
    int s0 = 0, s1 = 0;
    if (id) {
      s0 = sst[si];
      s1 = sst[sj];
    }
    bool lastA = true, lastB = true;
    for (unsigned m = odm; m; m &= m - 1) {
      const int j = __ffs(m) - 1;
      const int aj = __shfl_sync(FULL, si, j);
      const int bj = __shfl_sync(FULL, sj, j);
      const int uj = __shfl_sync(FULL, ups, j);
      if (id && j < lane) {
        if (si == aj) s0 = uj & 0xFF;
        else if (si == bj) s0 = uj >> 8;
        if (sj == aj) s1 = uj & 0xFF;
        else if (sj == bj) s1 = uj >> 8;
      }
      if (od && j > lane) {
        if (aj == si || bj == si) lastA = false;
        if (aj == sj || bj == sj) lastB = false;
      }
    }
    if (id) {
      const DevType t = types[type];
      const int dv = __ldg(diag_vc + t.diag_off + s0 + t.d0 * s1);
      vcode = dv >= 0 ? (dv & 0xFFFF) : -1;
      cls = dv >= 0 ? (dv >> 16) : -1;
    }
    // thresholds for the window around n
    if (use_thr && (n - n_c > 16 || n_c - n > 16)) {
      n_c = n;
      if (lane < ncls) diag_thresholds(M, c, L, n_c, thr, lane);
      __syncwarp();
    }
    // classify: surely accepted / surely rejected / maybe
    ulonglong2 ti = make_ulonglong2(0ull, U53_ALL), tr = make_ulonglong2(0ull, U53_ALL);
    if (use_thr && cls >= 0) {
      ti = thr[2 * cls];
      tr = thr[2 * cls + 1];
    }
    const int nlo = n - __popc(dgm & lt);
    const int nhi = n + __popc(idm & lt);
    bool alo = false, ahi = false;
    if (id) {
      if (cls < 0) {
        alo = ahi = false;  // invalid diagonal vertex: weight 0, never accepted
      } else if (use_thr && cur.u53 < ti.x) {
        alo = ahi = true;
      } else if (use_thr && cur.u53 >= ti.y) {
        alo = ahi = false;
      } else {
        const int vo = types[type].vert_off + (vcode >> 1);
        alo = diag_exact(M, c, L, nlo, true, cur.u53, vo);
        ahi = diag_exact(M, c, L, nhi, true, cur.u53, vo);
      }
    } else if (dg) {
      if (use_thr && cur.u53 < tr.x) {
        alo = ahi = true;
      } else if (use_thr && cur.u53 >= tr.y) {
        alo = ahi = false;
      } else {
        const int vo = types[type].vert_off + (vcode >> 1);
        alo = diag_exact(M, c, L, nlo, false, cur.u53, vo);
        ahi = diag_exact(M, c, L, nhi, false, cur.u53, vo);
      }
    }
    const bool amb = (id || dg) && (alo != ahi);
    unsigned plus = __ballot_sync(FULL, id && !amb && alo);
    unsigned minus = __ballot_sync(FULL, dg && !amb && alo);
    for (unsigned am = __ballot_sync(FULL, amb); am; am &= am - 1) {
      const int j = __ffs(am) - 1;
      const unsigned below = (1u << j) - 1u;
      const int nj = n + __popc(plus & below) - __popc(minus & below);
      bool acc = false;
      if (lane == j) acc = diag_exact(M, c, L, nj, id, cur.u53, types[type].vert_off + (vcode >> 1));
      const unsigned b = __ballot_sync(FULL, acc);
      if (idm & (1u << j)) plus |= b;
      else minus |= b;
    }
    if ((plus >> lane) & 1u) ops[p] = 1u | ((uint32_t)vcode << 1) | (cur.opb & 0xFFFFF800u);
    if ((minus >> lane) & 1u) ops[p] = 0u;
    n += __popc(plus) - __popc(minus);
    __syncwarp();
    if (od) {
      if (lastA) sst[si] = (uint8_t)(ups & 0xFF);
      if (lastB) sst[sj] = (uint8_t)(ups >> 8);
    }
    __syncwarp();
    cur = nxt;
  }
  c.n = n;
  c.ctr = ctr;
  return ST_OK;
}

// ---------------------------------------------------------------------------
// vertex list, src/vertex_list.jl:15-54, on the compacted opstring.
//
// Non-identity operators get compact indices k in slot order (ballot +
// popcount).  Each operator's lower leg on site s links to the upper leg of
// the previous operator on s -- found among the earlier lanes of the chunk
// through the chunk's site table, else in the per-site tail table vlast
// (shared memory).
// The first and last legs of every site are joined at the end, exactly like
// the reference's wrap loop.  Links are stored as 4*k + leg.
// ---------------------------------------------------------------------------

__device__ __noinline__ long long build_links(const DevModel &M, long long L, const uint32_t *__restrict__ ops,
                                              Rec *__restrict__ rec, int2 *__restrict__ chunk,
                                              int32_t *__restrict__ vfirst, int32_t *vlast, SiteTable *tab,
                                              int lane) {
  const int N = M.nsites;
  for (int i = lane; i < N; i += 32) {
    vlast[i] = -1;
    vfirst[i] = -1;
  }
  site_table_clear(tab, lane);
  __syncwarp();
  const unsigned lt = lanemask_lt();
  const int4 *__restrict__ bond_info = M.bond_info;
  const DevType *__restrict__ types = M.types;
  long long kbase = 0;
  // opcodes two chunks ahead, bond lookups one chunk ahead
  uint32_t op_c = (lane < L) ? ops[lane] : 0u;
  uint32_t op_n = (32 + lane < L) ? ops[32 + lane] : 0u;
  int4 bi_c = op_c ? __ldg(bond_info + (op_c >> 11)) : make_int4(-1, -1, 0, 0);
  for (long long base = 0; base < L; base += 32) {
    const long long p = base + lane;
    const uint32_t op_nn = (base + 64 + lane < L) ? ops[base + 64 + lane] : 0u;
    const int4 bi_n = op_n ? __ldg(bond_info + (op_n >> 11)) : make_int4(-1, -1, 0, 0);
    const uint32_t op = op_c;
    const bool nonid = op != 0u;
    const unsigned mask = __ballot_sync(FULL, nonid);
    const int k = (int)(kbase + __popc(mask & lt));
    if (lane == 0) chunk[base >> 5] = make_int2((int)kbase, (int)mask);
    const int a = nonid ? bi_c.x : -1, b = nonid ? bi_c.y : -1, type = bi_c.z;
    // the previous operator of the chunk on each site (its upper leg 2 when the site is its first
    // site, else 3) and whether a later one of the chunk is on the site, from the site table
    int hA = -1, hB = -1;
    if (nonid) {
      hA = site_insert(tab, a, lane);
      hB = site_insert(tab, b, lane);
    }
    __syncwarp();
    const uint32_t mA = nonid ? tab->mask[hA] : 0u, mB = nonid ? tab->mask[hB] : 0u;
    const unsigned gt = ~lt & ~(1u << lane);
    const bool lastA = (mA & gt) == 0u, lastB = (mB & gt) == 0u;
    const int jA = (mA & lt) ? 31 - __clz(mA & lt) : lane;
    const int jB = (mB & lt) ? 31 - __clz(mB & lt) : lane;
    const int aA = __shfl_sync(FULL, a, jA), kA = __shfl_sync(FULL, k, jA);
    const int aB = __shfl_sync(FULL, a, jB), kB = __shfl_sync(FULL, k, jB);
    const int predA = (mA & lt) ? 4 * kA + (aA == a ? 2 : 3) : -1;
    const int predB = (mB & lt) ? 4 * kB + (aB == b ? 2 : 3) : -1;
    if (nonid) {
      const int pa = predA >= 0 ? predA : vlast[a];
      const int pb = predB >= 0 ? predB : vlast[b];
      int la = -1, lb = -1;
      if (pa >= 0) {
        la = pa;
        rec[pa >> 2].link[pa & 3] = 4 * k + 0;
      } else {
        vfirst[a] = 4 * k + 0;
      }
      if (pb >= 0) {
        lb = pb;
        rec[pb >> 2].link[pb & 3] = 4 * k + 1;
      } else {
        vfirst[b] = 4 * k + 1;
      }
      const DevType t = types[type];
      int2 *r2 = reinterpret_cast<int2 *>(rec + k);
      r2[0] = make_int2(la, lb);
      r2[2] = make_int2((int)op, (int)p);
      r2[3] = make_int2(t.trans_off, t.maxworm | (t.d0 << 8) | (t.d1 << 16));
    }
    __syncwarp();
    if (nonid) {
      if (lastA) vlast[a] = 4 * k + 2;
      if (lastB) vlast[b] = 4 * k + 3;
      site_release(tab, hA);
      site_release(tab, hB);
    }
    kbase += __popc(mask);
    __syncwarp();
    op_c = op_n;
    op_n = op_nn;
    bi_c = bi_n;
  }
  for (int i = lane; i < N; i += 32) {
    const int f = vfirst[i];
    if (f >= 0) {
      const int l = vlast[i];
      rec[f >> 2].link[f & 3] = l;
      rec[l >> 2].link[l & 3] = f;
    }
  }
  __syncwarp();
  return kbase;
}

// ---------------------------------------------------------------------------
// worm update, src/sse.jl:193-303
// ---------------------------------------------------------------------------

struct WormCtl {
  double num_worms, avg_len, att, target_frac;
};

// Lane 0's chase of one worm between draw-buffer refills.
struct Chase {
  int k, leg_in, wf;
  long long len;
  int4 ra, rb;  // record of operator k: links, then (op, slot, transition offset, type info)
};

// What one call of worm_chase needs besides the tables: the draw position in the 64-draw buffer
// (in and out), the worm's start (k0, l0, wf0) and the steps left before the cap.
struct ChaseWindow {
  int pos, k0, l0, wf0, room, done;
};

// Steps of one worm run by lane 0 while draws remain in the buffer (src/sse.jl:262-303 with
// scatter, src/vertex_data.jl:106-125).  Per step: one 32-byte record (its links, code and type
// info) and the first 16 bytes of one transition row from L1 (threshold and packed outcome of the
// row's first outcome; the second half only when the first outcome is not taken).
//
// The records of the worm's possible next operators are not prefetched: at 4096 walkers the three
// extra random sector reads per step cost the diagonal and link phases more than the ~110 cycles
// they save the step (A/B on the 32x32, beta = 16 batch: 75.9k vs 75.4k walker-sweeps/s).
//
// CAPPED: the worm can reach its step cap within this window, so every step is counted against
// `room`; a window (at most 64 steps) that cannot reach it skips the test.
// ONE_WORM: every bond type has a single worm type (maxworm 1, e.g. every S=1/2 model), so the worm
// is always 1 and the row of (vertex, leg) needs no worm term.
template <bool CAPPED, bool ONE_WORM>
__device__ __forceinline__ int worm_chase_loop(const Trans *__restrict__ trans, const Outcome *__restrict__ outc,
                                               Rec *__restrict__ rec, const unsigned long long *__restrict__ dbuf,
                                               Chase *cs, ChaseWindow *win) {
  int k = cs->k, leg_in = cs->leg_in, wf = cs->wf;
  int4 ra = cs->ra;
  uint32_t op = (uint32_t)cs->rb.x;
  int slot = cs->rb.y, toff = cs->rb.z, tp = cs->rb.w;
  int pos = win->pos;
  const int k0 = win->k0, room = win->room;
  // the closing tests compare (leg, worm) pairs packed as leg | worm << 2
  const int lw0 = win->l0 | (win->wf0 << 2);
  const int4 *rq = reinterpret_cast<const int4 *>(rec);
  uint32_t *rop = reinterpret_cast<uint32_t *>(rec);  // rec[k].op = rop[8 k + 4]
  int used = 0, status = ST_OK, done = 0;
  while (pos < 64) {
    const unsigned long long u53 = dbuf[pos];
    pos++;
    const int ti = ONE_WORM ? toff + (int)((op >> 2) & 0x1FFu) * 4 + leg_in
                            : toff + ((int)((op >> 2) & 0x1FFu) * 4 + leg_in) * (tp & 0xFF) + (wf - 1);
    const int4 *tr = reinterpret_cast<const int4 *>(trans + ti);
    const int4 h0 = __ldg(tr);  // thr0, packed0, rest
    int packed = h0.z;
    if (packed >= 0 && !(u53 < (((unsigned long long)(uint32_t)h0.y << 32) | (uint32_t)h0.x))) {
      const int4 h1 = __ldg(tr + 1);  // thr1, packed1
      packed = h1.z;
      if (packed >= 0 && !(u53 < (((unsigned long long)(uint32_t)h1.y << 32) | (uint32_t)h1.x))) {
        packed = -1;
        const int o0 = h0.w >> 8, on = h0.w & 0xFF;
        for (int o = o0; o < o0 + on; o++) {
          const Outcome oc = outc[o];
          if (u53 < oc.thr) {
            packed = oc.packed;
            break;
          }
        }
      }
    }
    if (packed < 0) {
      status = ST_INVALID_VERTEX;
      break;
    }
    // the store precedes the next load of the same record, so a revisit sees the new code; the
    // opstring itself is written once after the worms (slot order, coalesced)
    rop[8 * k + 4] = 1u | ((uint32_t)((packed >> 10) & 0x3FF) << 1) | (op & 0xFFFFF800u);
    // closed at the exit leg: the start operator, the start leg, and worm_out == dim_out - worm_0,
    // i.e. dim_out - worm_out (bits 20..27 of the outcome) == worm_0
    if (k == k0 && ((packed & 3) | ((packed >> 18) & 0x3FC)) == lw0) {
      done = 1;
      break;
    }
    used++;
    if (!ONE_WORM) wf = (packed >> 2) & 0xFF;
    const int l01 = (packed & 1) ? ra.y : ra.x, l23 = (packed & 1) ? ra.w : ra.z;
    const int link = (packed & 2) ? l23 : l01;
    leg_in = link & 3;
    k = link >> 2;
    if (k == k0 && (ONE_WORM ? leg_in == (lw0 & 3) : (leg_in | (wf << 2)) == lw0)) {
      done = 1;
      break;
    }
    if (CAPPED && used > room) {  // len0 + used > cap
      status = ST_WORM_CAP;
      break;
    }
    ra = rq[2 * k];
    const int4 rb = rq[2 * k + 1];
    op = (uint32_t)rb.x;
    slot = rb.y;
    toff = rb.z;
    tp = rb.w;
  }
  cs->k = k;
  cs->leg_in = leg_in;
  cs->wf = wf;
  cs->len += used;
  cs->ra = ra;
  cs->rb = make_int4((int)op, slot, toff, tp);
  win->pos = pos;
  win->done = done;
  return status;
}

// Kept out of line, with its state in a handful of registers, so that the chase does not share the
// register budget of the worm update's other phases.  Returns the status; sets win.done when the
// worm closed; win.pos == 64 when the buffer ran dry.
__device__ __noinline__ int worm_chase(const Trans *__restrict__ trans, const Outcome *__restrict__ outc,
                                       Rec *__restrict__ rec, const unsigned long long *__restrict__ dbuf,
                                       Chase *cs, ChaseWindow *win, bool one_worm) {
  if (one_worm) {
    if (win->room >= 64) return worm_chase_loop<false, true>(trans, outc, rec, dbuf, cs, win);
    return worm_chase_loop<true, true>(trans, outc, rec, dbuf, cs, win);
  }
  if (win->room >= 64) return worm_chase_loop<false, false>(trans, outc, rec, dbuf, cs, win);
  return worm_chase_loop<true, false>(trans, outc, rec, dbuf, cs, win);
}

__device__ __noinline__ int worm_update(const DevModel &M, Chain &c, WormCtl &wc, uint32_t *__restrict__ ops,
                                        Rec *__restrict__ rec, const int2 *__restrict__ chunk,
                                        const int32_t *__restrict__ vfirst, uint8_t *__restrict__ state,
                                        unsigned long long *dbuf, bool thermalized, double &wlf, bool &have_wlf,
                                        long long &steps, int lane, int cap_factor) {
  double total = 1.0;
  const double ceil_nw = ceil(wc.num_worms);
  const long long nworms = (long long)ceil_nw;
  // the cap counts at least WORM_CAP_MIN_SLOTS slots: small systems run long worms relative to L
  const long long cap =
      (long long)(cap_factor > 0 ? cap_factor : 64) * (c.L + 16 > WORM_CAP_MIN_SLOTS ? c.L + 16 : WORM_CAP_MIN_SLOTS);
  const unsigned long long L = (unsigned long long)c.L;
  for (long long wi = 0; wi < nworms; wi++) {
    if (c.n == 0) continue;  // worm_traverse! returns 0 without drawing
    // rejection-sample the start (src/sse.jl:241-247): 32 tries side by side, first success wins
    int l0 = 0, k0 = -1;
    for (int guard = 0;; guard++) {
      if (guard >= (1 << 26)) return ST_TIMEOUT;
      unsigned long long u1, u2;
      draw2(c.seed, c.stream, c.ctr + 2ull * lane, u1, u2);
      const long long pp = (long long)urange0(u1, L);
      const int ll = (int)urange0(u2, 4ull);
      const int2 ch = chunk[pp >> 5];  // the operator at slot pp, if any (compact index)
      const unsigned bit = 1u << (pp & 31);
      const int kk = ((unsigned)ch.y & bit) ? ch.x + __popc((unsigned)ch.y & (bit - 1u)) : -1;
      const unsigned okm = __ballot_sync(FULL, kk >= 0);
      if (okm) {
        const int t = __ffs(okm) - 1;
        c.ctr += 2ull * (t + 1);
        l0 = __shfl_sync(FULL, ll, t);
        k0 = __shfl_sync(FULL, kk, t);
        break;
      }
      c.ctr += 64ull;
    }
    // worm function (src/sse.jl:249-251)
    const uint32_t op0 = rec[k0].op;  // the start operator's code (src/sse.jl:249)
    const int4 bi0 = M.bond_info[op0 >> 11];
    const int site0 = (l0 & 1) ? bi0.y : bi0.x;
    const int dim0 = M.site_dims[site0];
    const int wf0 = 1 + (int)urange0(draw64(c.seed, c.stream, c.ctr), (unsigned long long)(dim0 - 1));
    c.ctr++;
    // the worm: lane 0 walks, the whole warp refills 64 draws at a time (one Philox block per lane)
    Chase cs;
    cs.k = k0;
    cs.leg_in = l0;
    cs.wf = wf0;
    cs.len = 1;
    if (lane == 0) {
      const int4 *rq = reinterpret_cast<const int4 *>(rec);
      cs.ra = rq[2 * k0];
      cs.rb = rq[2 * k0 + 1];
    }
    unsigned long long ctr = c.ctr;
    int status = ST_OK;
    bool done = false;
    for (;;) {
      const unsigned long long b = ctr & ~1ull;
      const uint4 x = philox_block(c.seed, c.stream, (b >> 1) + lane);
      dbuf[2 * lane] = (((unsigned long long)x.y << 32) | x.x) >> 11;
      dbuf[2 * lane + 1] = (((unsigned long long)x.w << 32) | x.z) >> 11;
      __syncwarp();
      int pos = (int)(ctr - b);
      if (lane == 0) {
        // steps left before the worm exceeds the cap (a draw window has at most 64 steps)
        ChaseWindow win;
        win.pos = pos;
        win.k0 = k0;
        win.l0 = l0;
        win.wf0 = wf0;
        win.room = (cap - cs.len) > 0x3FFFFFFFLL ? 0x3FFFFFFF : (int)(cap - cs.len);
        win.done = 0;
        status = worm_chase(M.trans, M.outc, rec, dbuf, &cs, &win, M.one_worm != 0);
        pos = win.pos;
        done = win.done != 0;
      }
      __syncwarp();
      status = __shfl_sync(FULL, status, 0);
      done = __shfl_sync(FULL, (int)done, 0) != 0;
      ctr = b + (unsigned long long)__shfl_sync(FULL, pos, 0);
      if (status != ST_OK || done) break;
    }
    steps += (long long)(ctr - c.ctr);  // one draw per scatter
    c.ctr = ctr;
    const long long len = shfl_ll(cs.len, 0);
    if (status == ST_WORM_CAP && !thermalized) {
      // undo the worm phase: the worms rewrote only the records, so ops[] still holds the
      // opstring of the diagonal update; the controller and the spin state stay as they were
      // and the draws the worms consumed stay consumed
      return ST_WORM_UNDONE;
    }
    if (status != ST_OK) {
      for (long long k = lane; k < c.n; k += 32) {
        const int2 os = reinterpret_cast<const int2 *>(rec + k)[2];
        ops[os.y] = (uint32_t)os.x;
      }
      __syncwarp();
      return status;
    }
    total = __dadd_rn(total, (double)len);
  }

  // the operators' final codes are still only in the records: the caller writes them back into the
  // opstring (write_back_ops, or fused with the measurement in measure_records)
  have_wlf = thermalized && c.n != 0;
  if (have_wlf) wlf = __ddiv_rn(total, (double)c.n);

  const double avg_worm_length = __ddiv_rn(total, ceil_nw);
  if (!thermalized) {
    const double a = wc.att;
    wc.avg_len = __dadd_rn(wc.avg_len, __dmul_rn(a, __dsub_rn(avg_worm_length, wc.avg_len)));
    const double target_worms = __ddiv_rn(__dmul_rn(wc.target_frac, (double)c.n), wc.avg_len);
    const double diff = __dsub_rn(target_worms, wc.num_worms);
    wc.num_worms = __dadd_rn(wc.num_worms, __dmul_rn(a, __dadd_rn(diff, __dmul_rn(100.0, ctl_tanh(diff)))));
    if (a != 0) {
      const double hi = __dadd_rn(1.0, __ddiv_rn((double)c.n, 2.0));
      const double x = wc.num_worms;
      wc.num_worms = x > hi ? hi : (x < 1.0 ? 1.0 : x);
    }
  }

  // re-derive the spin state from the first leg of every site (src/sse.jl:219-228)
  const unsigned lt = lanemask_lt();
  const int N = M.nsites;
  for (int i0 = 0; i0 < N; i0 += 32) {
    const int i = i0 + lane;
    const bool inr = i < N;
    const int vf = inr ? vfirst[i] : 0;
    const bool freeb = inr && vf < 0;
    const unsigned fm = __ballot_sync(FULL, freeb);
    if (freeb) {
      const unsigned long long u = draw64(c.seed, c.stream, c.ctr + __popc(fm & lt));
      state[i] = (uint8_t)urange0(u, (unsigned long long)M.site_dims[i]);
    } else if (inr) {
      const uint32_t op = rec[vf >> 2].op;
      const int type = M.bond_info[op >> 11].z;
      state[i] = M.leg_state[4 * (M.types[type].vert_off + (int)((op >> 1) & 0x3FFu) / 2) + (vf & 3)];
    }
    c.ctr += __popc(fm);
  }
  __syncwarp();
  return ST_OK;
}

// ---------------------------------------------------------------------------
// measure!, src/sse.jl:70-87 with measure_sign (305-314) and the fused
// MagnetizationEstimator loop (321-376, magnetization_estimator.jl:96-230).
// Running magnetisations are an inclusive warp scan of the per-operator
// changes; sums are accumulated per lane and reduced at the end.
// ---------------------------------------------------------------------------

__device__ __forceinline__ void observe(DevWalker *W, int idx, double v) {
  W->obs_sum[idx] += v;
  W->obs_last[idx] = v;
  W->obs_count[idx] += 1;
}

// Exact pass for models whose coefficients are multiples of 1/2 (every MagnetModel): running
// magnetisations are integers in units of 1/2, sums are exact (m^4 in 128 bits), and the result
// is converted to double once.  Handles estimators e0 .. e0+ne-1 (ne <= 2) and, on the first
// pass, the sign parity.
__device__ __forceinline__ long long warp_sum_i64(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

__device__ __forceinline__ unsigned __int128 warp_sum_u128(unsigned __int128 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long lo = __shfl_xor_sync(FULL, (unsigned long long)v, o);
    const unsigned long long hi = __shfl_xor_sync(FULL, (unsigned long long)(v >> 64), o);
    v += ((unsigned __int128)hi << 64) | lo;
  }
  return v;
}

__device__ __forceinline__ double u128_to_double(unsigned __int128 v) {
  const unsigned long long hi = (unsigned long long)(v >> 64), lo = (unsigned long long)v;
  return __dadd_rn(__dmul_rn(__ull2double_rn(hi), 0x1.0p64), __ull2double_rn(lo));
}

__device__ void finish_estimator(const DevModel &M, const Chain &c, DevWalker *W, int e, double sign, double mag,
                                 double absmag, double mag2, double mag4) {
  const double n = (double)c.n;
  const double est_n = __dadd_rn(1.0, n);
  const double norm = __ddiv_rn(1.0, M.norm_site_count);
  const double norm2 = __dmul_rn(norm, norm);
  mag = __dmul_rn(mag, norm);
  absmag = __dmul_rn(absmag, norm);
  mag2 = __dmul_rn(mag2, norm2);
  mag4 = __dmul_rn(mag4, __dmul_rn(norm2, norm2));
  const int base = 6 + 5 * e;
  observe(W, base + 0, __ddiv_rn(__dmul_rn(sign, mag), est_n));
  observe(W, base + 1, __ddiv_rn(__dmul_rn(sign, absmag), est_n));
  observe(W, base + 2, __ddiv_rn(__dmul_rn(sign, mag2), est_n));
  observe(W, base + 3, __ddiv_rn(__dmul_rn(sign, mag4), est_n));
  const double chi =
      __dmul_rn(__dmul_rn(__ddiv_rn(__ddiv_rn(__ddiv_rn(1.0, c.T), __dadd_rn(est_n, 1.0)), est_n),
                          __dadd_rn(__dmul_rn(mag, mag), mag2)),
                M.norm_site_count);
  observe(W, base + 4, __dmul_rn(sign, chi));
}

__device__ void observe_base(const DevModel &M, const Chain &c, DevWalker *W, double sign) {
  const double n = (double)c.n;
  observe(W, 0, sign);
  observe(W, 1, n);
  observe(W, 2, __dmul_rn(sign, n));
  observe(W, 3, __dmul_rn(sign, __dmul_rn(n, n)));
  observe(W, 4, __ddiv_rn(__dmul_rn(-sign, __dadd_rn(__dmul_rn(n, c.T), M.energy_offset)), M.norm_site_count));
}

template <int NE>
__device__ long long measure_pass_int(const DevModel &M, const Chain &c, DevWalker *W, const uint32_t *__restrict__ ops,
                                      const uint8_t *__restrict__ state, int e0, bool count_sign, double sign_in,
                                      int lane) {
  const long long L = c.L;
  const int N = M.nsites, md = M.maxdim;
  const int4 *__restrict__ bond_info = M.bond_info;
  const DevType *__restrict__ types = M.types;
  const int8_t *__restrict__ vsign = M.sign;
  const uint8_t *__restrict__ leg_state = M.leg_state;
  const int32_t *__restrict__ cf[2];
  int t0[2], carry[2];
  long long s1[2], s2[2], s3[2];
  unsigned __int128 s4[2];
#pragma unroll
  for (int q = 0; q < NE; q++) {
    cf[q] = M.est_coef2 + (long long)(e0 + q) * N * md;
    int acc = 0;
    for (int i = lane; i < N; i += 32) acc += cf[q][(long long)i * md + state[i]];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(FULL, acc, o);
    t0[q] = acc;
    carry[q] = acc;
    s1[q] = s2[q] = s3[q] = 0;
    s4[q] = 0;
  }
  long long negs = 0;
  uint32_t op_n = (lane < L) ? ops[lane] : 0u;
  for (long long base = 0; base < L; base += 32) {
    const uint32_t op = op_n;
    op_n = (base + 32 + lane < L) ? ops[base + 32 + lane] : 0u;
    int d[2] = {0, 0};
    if (op != 0u) {
      const int4 bi = __ldg(bond_info + (op >> 11));
      const int vo = types[bi.z].vert_off + (int)((op >> 1) & 0x3FFu) / 2;
      if (count_sign) negs += vsign[vo] < 0;
      if (!(op & 2u)) {
        const uchar4 ls = *reinterpret_cast<const uchar4 *>(leg_state + 4 * vo);
#pragma unroll
        for (int q = 0; q < NE; q++) {
          d[q] = (cf[q][(long long)bi.x * md + ls.z] - cf[q][(long long)bi.x * md + ls.x]) +
                 (cf[q][(long long)bi.y * md + ls.w] - cf[q][(long long)bi.y * md + ls.y]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < NE; q++) {
      int x = d[q];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
      }
      const int t = carry[q] + x;
      if (op != 0u) {
        const long long tl = t;
        s1[q] += tl;
        s2[q] += tl < 0 ? -tl : tl;
        const long long t2 = tl * tl;
        s3[q] += t2;
        s4[q] += (unsigned __int128)((unsigned long long)t2) * (unsigned long long)t2;
      }
      carry[q] = __shfl_sync(FULL, t, 31);
    }
  }
  if (count_sign) negs = warp_sum_i64(negs);
  const double sign = count_sign ? ((negs & 1) ? -1.0 : 1.0) : sign_in;
  if (count_sign && lane == 0) observe_base(M, c, W, sign);
#pragma unroll
  for (int q = 0; q < NE; q++) {
    const long long S1 = warp_sum_i64(s1[q]), S2 = warp_sum_i64(s2[q]), S3 = warp_sum_i64(s3[q]);
    const unsigned __int128 S4 = warp_sum_u128(s4[q]);
    if (lane == 0) {
      const long long a = t0[q];
      const long long a2 = a * a;
      const double mag = __dmul_rn(__ll2double_rn(a + S1), 0.5);
      const double absmag = __dmul_rn(__ll2double_rn((a < 0 ? -a : a) + S2), 0.5);
      const double mag2 = __dmul_rn(__ll2double_rn(a2 + S3), 0.25);
      const double mag4 = __dmul_rn(u128_to_double(S4 + (unsigned __int128)((unsigned long long)a2) * (unsigned long long)a2),
                                    0.0625);
      finish_estimator(M, c, W, e0 + q, sign, mag, absmag, mag2, mag4);
    }
  }
  __syncwarp();
  return (long long)(sign < 0 ? 1 : 0);
}

// The operators' final codes from the compacted records back into the opstring (slot order).
__device__ __noinline__ void write_back_ops(const Chain &c, const Rec *__restrict__ rec, uint32_t *__restrict__ ops,
                                            int lane) {
  for (long long k = lane; k < c.n; k += 32) {
    const int2 os = reinterpret_cast<const int2 *>(rec + k)[2];
    ops[os.y] = (uint32_t)os.x;
  }
  __syncwarp();
}

// measure_pass_int over the compacted records instead of the opstring: the non-identity operators
// in slot order, n entries instead of L slots (identity slots add no term to any sum).  With
// `first` the pass also writes every operator's code back into the opstring and counts the sign.
template <int NE>
__device__ long long measure_pass_rec(const DevModel &M, const Chain &c, DevWalker *W, const Rec *__restrict__ rec,
                                      uint32_t *__restrict__ ops, const uint8_t *__restrict__ state, int e0,
                                      bool first, double sign_in, int lane) {
  const long long n = c.n;
  const int N = M.nsites, md = M.maxdim;
  const int4 *__restrict__ bond_info = M.bond_info;
  const DevType *__restrict__ types = M.types;
  const int8_t *__restrict__ vsign = M.sign;
  const uint8_t *__restrict__ leg_state = M.leg_state;
  const int2 *__restrict__ r2 = reinterpret_cast<const int2 *>(rec);  // r2[4 k + 2] = (op, slot) of record k
  const int32_t *__restrict__ cf[2];
  int t0[2], carry[2];
  long long s1[2], s2[2], s3[2];
  unsigned __int128 s4[2];
#pragma unroll
  for (int q = 0; q < NE; q++) {
    cf[q] = M.est_coef2 + (long long)(e0 + q) * N * md;
    int acc = 0;
    for (int i = lane; i < N; i += 32) acc += cf[q][(long long)i * md + state[i]];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(FULL, acc, o);
    t0[q] = acc;
    carry[q] = acc;
    s1[q] = s2[q] = s3[q] = 0;
    s4[q] = 0;
  }
  long long negs = 0;
  int2 os_n = (lane < n) ? r2[4 * (long long)lane + 2] : make_int2(0, 0);
  for (long long base = 0; base < n; base += 32) {
    const int2 os = os_n;
    os_n = (base + 32 + lane < n) ? r2[4 * (base + 32 + lane) + 2] : make_int2(0, 0);
    const uint32_t op = (uint32_t)os.x;  // 0 past the last operator
    if (first && op != 0u) ops[os.y] = op;
    int d[2] = {0, 0};
    if (op != 0u) {
      const int4 bi = __ldg(bond_info + (op >> 11));
      const int vo = types[bi.z].vert_off + (int)((op >> 2) & 0x1FFu);
      if (first) negs += vsign[vo] < 0;
      if (!(op & 2u)) {
        const uchar4 ls = *reinterpret_cast<const uchar4 *>(leg_state + 4 * vo);
#pragma unroll
        for (int q = 0; q < NE; q++) {
          d[q] = (cf[q][(long long)bi.x * md + ls.z] - cf[q][(long long)bi.x * md + ls.x]) +
                 (cf[q][(long long)bi.y * md + ls.w] - cf[q][(long long)bi.y * md + ls.y]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < NE; q++) {
      int x = d[q];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
      }
      const int t = carry[q] + x;
      if (op != 0u) {
        const long long tl = t;
        s1[q] += tl;
        s2[q] += tl < 0 ? -tl : tl;
        const long long t2 = tl * tl;
        s3[q] += t2;
        s4[q] += (unsigned __int128)((unsigned long long)t2) * (unsigned long long)t2;
      }
      carry[q] = __shfl_sync(FULL, t, 31);
    }
  }
  if (first) negs = warp_sum_i64(negs);
  const double sign = first ? ((negs & 1) ? -1.0 : 1.0) : sign_in;
  if (first && lane == 0) observe_base(M, c, W, sign);
#pragma unroll
  for (int q = 0; q < NE; q++) {
    const long long S1 = warp_sum_i64(s1[q]), S2 = warp_sum_i64(s2[q]), S3 = warp_sum_i64(s3[q]);
    const unsigned __int128 S4 = warp_sum_u128(s4[q]);
    if (lane == 0) {
      const long long a = t0[q];
      const long long a2 = a * a;
      const double mag = __dmul_rn(__ll2double_rn(a + S1), 0.5);
      const double absmag = __dmul_rn(__ll2double_rn((a < 0 ? -a : a) + S2), 0.5);
      const double mag2 = __dmul_rn(__ll2double_rn(a2 + S3), 0.25);
      const double mag4 = __dmul_rn(u128_to_double(S4 + (unsigned __int128)((unsigned long long)a2) * (unsigned long long)a2),
                                    0.0625);
      finish_estimator(M, c, W, e0 + q, sign, mag, absmag, mag2, mag4);
    }
  }
  __syncwarp();
  return (long long)(sign < 0 ? 1 : 0);
}

// measure! (exact integer estimators, M.est_int) right after the worm update, on the compacted
// records, fused with writing the operators' codes back into the opstring.
__device__ __noinline__ void measure_records(const DevModel &M, const Chain &c, DevWalker *W,
                                             const Rec *__restrict__ rec, uint32_t *__restrict__ ops,
                                             const uint8_t *__restrict__ state, int lane) {
  if (M.nest == 0) {
    measure_pass_rec<0>(M, c, W, rec, ops, state, 0, true, 1.0, lane);
    return;
  }
  double sign = 1.0;
  for (int e0 = 0; e0 < M.nest; e0 += 2) {
    const bool first = e0 == 0;
    long long neg;
    if (M.nest - e0 >= 2) neg = measure_pass_rec<2>(M, c, W, rec, ops, state, e0, first, sign, lane);
    else neg = measure_pass_rec<1>(M, c, W, rec, ops, state, e0, first, sign, lane);
    if (first) sign = neg ? -1.0 : 1.0;
  }
}

__device__ __noinline__ void measure(const DevModel &M, const Chain &c, DevWalker *W, const uint32_t *__restrict__ ops,
                                     const uint8_t *__restrict__ state, int lane) {
  if (M.est_int) {
    // one fused pass per pair of estimators; the first also measures the sign
    double sign = 1.0;
    if (M.nest == 0) {
      sign = measure_pass_int<0>(M, c, W, ops, state, 0, true, 1.0, lane) ? -1.0 : 1.0;
      return;
    }
    for (int e0 = 0; e0 < M.nest; e0 += 2) {
      const bool first = e0 == 0;
      long long neg;
      if (M.nest - e0 >= 2) neg = measure_pass_int<2>(M, c, W, ops, state, e0, first, sign, lane);
      else neg = measure_pass_int<1>(M, c, W, ops, state, e0, first, sign, lane);
      if (first) sign = neg ? -1.0 : 1.0;
    }
    return;
  }
  const long long L = c.L;
  long long negs = 0;
  for (long long base = 0; base < L; base += 32) {
    const long long p = base + lane;
    const uint32_t op = p < L ? ops[p] : 0u;
    if (op != 0u) {
      const int type = M.bond_info[op >> 11].z;
      negs += M.sign[M.types[type].vert_off + (int)((op >> 1) & 0x3FFu) / 2] < 0;
    }
  }
  negs = warp_sum_ll(negs);
  const double sign = (negs & 1) ? -1.0 : 1.0;
  if (lane == 0) observe_base(M, c, W, sign);
  const int N = M.nsites, md = M.maxdim;
  for (int e = 0; e < M.nest; e++) {
    const double *coef = M.est_coef + (long long)e * N * md;
    double t0 = 0.0;
    for (int i = lane; i < N; i += 32) t0 = __dadd_rn(t0, coef[(long long)i * md + state[i]]);
    t0 = warp_sum(t0);
    double carry = t0, s1 = 0.0, s2 = 0.0, s3 = 0.0, s4 = 0.0;
    for (long long base = 0; base < L; base += 32) {
      const long long p = base + lane;
      const uint32_t op = p < L ? ops[p] : 0u;
      double d = 0.0;
      if (op != 0u && !(op & 2u)) {
        const int4 bi = M.bond_info[op >> 11];
        const uchar4 ls =
            *reinterpret_cast<const uchar4 *>(M.leg_state + 4 * (M.types[bi.z].vert_off + (int)((op >> 1) & 0x3FFu) / 2));
        const double d0 = __dsub_rn(coef[(long long)bi.x * md + ls.z], coef[(long long)bi.x * md + ls.x]);
        const double d1 = __dsub_rn(coef[(long long)bi.y * md + ls.w], coef[(long long)bi.y * md + ls.y]);
        d = __dadd_rn(d0, d1);
      }
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const double y = __shfl_up_sync(FULL, d, o);
        if (lane >= o) d = __dadd_rn(d, y);
      }
      const double t = __dadd_rn(carry, d);
      if (op != 0u) {
        s1 = __dadd_rn(s1, t);
        s2 = __dadd_rn(s2, fabs(t));
        const double t2 = __dmul_rn(t, t);
        s3 = __dadd_rn(s3, t2);
        s4 = __dadd_rn(s4, __dmul_rn(t2, t2));
      }
      carry = __shfl_sync(FULL, t, 31);
    }
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    s3 = warp_sum(s3);
    s4 = warp_sum(s4);
    if (lane == 0) {
      const double t02 = __dmul_rn(t0, t0);
      finish_estimator(M, c, W, e, sign, __dadd_rn(t0, s1), __dadd_rn(fabs(t0), s2), __dadd_rn(t02, s3),
                       __dadd_rn(__dmul_rn(t02, t02), s4));
    }
    __syncwarp();
  }
}

}  // namespace sse

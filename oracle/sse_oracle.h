/*
 * CPU oracle for the SSE update engine -- TEST INFRASTRUCTURE ONLY.
 *
 * A statement-by-statement restatement in C of the reference's sweep
 * (lukas-weber/StochasticSeriesExpansion.jl):
 *   init!            src/sse.jl:47-60
 *   sweep!           src/sse.jl:62-68
 *   diagonal_update  src/sse.jl:137-191
 *   make_vertex_list src/vertex_list.jl:15-54
 *   worm_update      src/sse.jl:193-231, worm_traverse! src/sse.jl:233-303
 *   scatter          src/vertex_data.jl:106-125
 *   measure!         src/sse.jl:70-87, measure_sign src/sse.jl:305-314,
 *                    measure_opstring! src/sse.jl:321-376 with
 *                    MagnetizationEstimator (magnetization_estimator.jl:96-230)
 *
 * Random numbers come from a counter-based replay stream (Philox4x32-10,
 * key = seed, counter = (draw index / 2, walker id)); every draw the
 * reference makes from ctx.rng consumes exactly one 64-bit value in the same
 * order.  The value mappings are fixed by this project:
 *   rand()     = (u >> 11) * 2^-53
 *   rand(1:m)  = 1 + floor(u * m / 2^64)
 *
 * Only the tests, the smoke check and the benchmark's CPU baseline link this
 * library.  The GPU engine never does.
 */
#ifndef SSE_ORACLE_H
#define SSE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_OK = 0,
  ORC_ERR_ARG = 1,
  ORC_ERR_INVALID_VERTEX = 4,
  ORC_ERR_WORM_CAP = 8,
  ORC_ERR_NOMEM = 6,
};

/* flat model tables, layout documented in the host package's tables.py */
typedef struct orc_model {
  int32_t nsites, nbonds, ntypes, maxdim, nest;
  double energy_offset, norm_site_count;
  const int32_t *site_dims, *bond_type, *bond_sites;
  const int32_t *type_dims, *type_nverts, *type_maxworm;
  const int32_t *type_diag_off, *type_vert_off, *type_trans_off;
  const int32_t *diag_vertex;
  const double *weight;
  const int8_t *sign;
  const uint8_t *leg_state;
  const int32_t *trans_start, *trans_count;
  const double *out_cum;
  const int32_t *out_target;
  const int8_t *out_leg, *out_worm;
  const double *est_coef;
} orc_model;

#define ORC_OBS_BASE 6 /* Sign, OperatorCount, SignOperatorCount, SignOperatorCount2, SignEnergy, WormLengthFraction */
#define ORC_OBS_PER_EST 5 /* SignMag, SignAbsMag, SignMag2, SignMag4, SignMagChi */

typedef struct orc_walker {
  /* parameters */
  double T;
  double target_worm_length_fraction;
  double num_worms_attenuation_factor;
  uint64_t seed, stream;
  int64_t thermalization;
  /* Markov chain state (checkpoint fields of src/sse.jl:89-107 + replay counter) */
  double avg_worm_length;
  double num_worms;
  int64_t num_operators;
  int64_t L;
  uint64_t ctr;
  int64_t sweeps;
  uint32_t *ops;
  int64_t ops_cap;
  uint8_t *state;
  /* vertex list, reference layout: vertices[p*4 + leg] = 4*p' + leg' or -1 */
  int32_t *vertices;
  int64_t vertices_len;
  int32_t *v_first, *v_last;
  /* diagnostics */
  int32_t status;
  int64_t resize_after_thermalization;
  int64_t worm_steps_total; /* scatter calls */
  int64_t slot_visits_total;
  /* observables: sums, counts and last values, ORC_OBS_BASE + 5*nest entries */
  int32_t nobs;
  double *obs_sum;
  double *obs_last;
  int64_t *obs_count;
  /* a worm stops the walker (ORC_ERR_WORM_CAP) after worm_cap_factor * max(L + 16, ORC_WORM_CAP_MIN_SLOTS)
   * steps; default 64.
   * During thermalisation the sweep's worm phase is undone instead: the opstring returns to its
   * state after the diagonal update, the controller and the spin state are left as they were,
   * and the walker goes on (no counterpart in the reference, whose worms have no limit). */
  int32_t worm_cap_factor;
  int64_t worm_undos; /* thermalisation worm phases undone at the cap */
  uint32_t *ops_saved; /* the opstring before the worm phase, kept during thermalisation */
  int64_t ops_saved_cap;
} orc_walker;

/* the worm step cap counts at least this many opstring slots (small systems run long worms relative to L) */
#define ORC_WORM_CAP_MIN_SLOTS 65536

orc_walker *orc_walker_create(const orc_model *m, double T, uint64_t seed, uint64_t stream,
                              double init_num_worms, double attenuation, double target_fraction,
                              int64_t thermalization);
void orc_walker_destroy(orc_walker *w);

/* Carlo.init!: random state, identity opstring of length init_cutoff (<0: round(N*T)), warm-up diagonal sweeps */
int orc_init(const orc_model *m, orc_walker *w, int64_t init_cutoff, int32_t warmup_sweeps);
/* Carlo.sweep! with an explicit is_thermalized flag */
int orc_sweep(const orc_model *m, orc_walker *w, int32_t thermalized);
/* Carlo.measure! */
int orc_measure(const orc_model *m, orc_walker *w);
/* one Carlo step: sweep!(is_thermalized = sweeps > therm); sweeps += 1; measure! if sweeps > therm */
int orc_step(const orc_model *m, orc_walker *w, int32_t do_measure);
int orc_run(const orc_model *m, orc_walker *w, int64_t nsteps, int32_t do_measure);

/* pieces, exposed for unit tests */
int orc_diagonal_update(const orc_model *m, orc_walker *w, int32_t thermalized);
int orc_make_vertex_list(const orc_model *m, orc_walker *w);
int orc_worm_update(const orc_model *m, orc_walker *w, int32_t thermalized);
int orc_set_opstring(orc_walker *w, const uint32_t *ops, int64_t L, int64_t num_operators);
int orc_set_state(const orc_model *m, orc_walker *w, const uint8_t *state);

/* independent chains, one per thread (CPU baseline) */
int orc_run_parallel(const orc_model *m, orc_walker **ws, int32_t nwalkers, int64_t nsteps,
                     int32_t do_measure, int32_t nthreads);

/* Parallel-tempering exchange step over nladders ladders of nrungs walkers (ws[l*nrungs + k]):
 * walkers ranked by T; step proposes rung pairs (k, k+1) with k = step mod 2; the swap weight is
 * exp of the summed log weight ratios of src/sse.jl:390-396, q = (T_a/T_b)^(n_a - n_b) by binary
 * powering; accept when u < q, u from Philox(counter = (step, k, l), key = seed) words 0,1; an
 * accepted swap exchanges T and the observable accumulators.  accepted: nladders*(nrungs-1)
 * entries, 1/0, or -1 for pairs not proposed. */
double orc_tempering_weight(double Ta, double Tb, int64_t na, int64_t nb);
int orc_tempering_exchange(orc_walker **ws, int32_t nladders, int32_t nrungs, uint64_t seed, uint64_t step,
                           int32_t *accepted);

/* replay stream primitives (tests) */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
uint64_t orc_draw(uint64_t seed, uint64_t stream, uint64_t index);
double orc_tanh(double x);

#ifdef __cplusplus
}
#endif
#endif

/*
 * CPU oracle for the SSE update engine -- TEST INFRASTRUCTURE ONLY.
 * See sse_oracle.h for the reference functions restated here.
 *
 * Build with -ffp-contract=off: every floating-point expression below is
 * evaluated as the reference writes it, one IEEE-754 double operation at a
 * time, and must not be fused into FMAs.
 */
#include "sse_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* replay stream                                                             */
/* ------------------------------------------------------------------------ */

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    if (r > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0;
    c1 = n1;
    c2 = n2;
    c3 = n3;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

uint64_t orc_draw(uint64_t seed, uint64_t stream, uint64_t index) {
  uint64_t blk = index >> 1;
  uint32_t ctr[4] = {(uint32_t)blk, (uint32_t)(blk >> 32), (uint32_t)stream, (uint32_t)(stream >> 32)};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t x[4];
  orc_philox4x32_10(ctr, key, x);
  if (index & 1) return (uint64_t)x[2] | ((uint64_t)x[3] << 32);
  return (uint64_t)x[0] | ((uint64_t)x[1] << 32);
}

static inline uint64_t next_u64(orc_walker *w) { return orc_draw(w->seed, w->stream, w->ctr++); }

/* rand(rng) */
static inline double rand01(orc_walker *w) { return (double)(next_u64(w) >> 11) * 0x1.0p-53; }

/* rand(rng, 1:m) */
static inline int64_t rand_range(orc_walker *w, uint64_t m) {
  unsigned __int128 prod = (unsigned __int128)next_u64(w) * m;
  return 1 + (int64_t)(uint64_t)(prod >> 64);
}

/* ------------------------------------------------------------------------ */
/* tanh for the worm-count controller (src/sse.jl:213)                       */
/* expm1 by Taylor series near 0, otherwise exp by Cody-Waite reduction       */
/* (y = k ln2 + r) with a degree-13 Taylor polynomial for exp(r).  Only        */
/* +, -, *, / and floor, so the GPU engine can reproduce it bit for bit.      */
/* ------------------------------------------------------------------------ */

static const double inv_fact[20] = {
    0x1.0000000000000p+0,  0x1.0000000000000p+0,  0x1.0000000000000p-1,  0x1.5555555555555p-3,
    0x1.5555555555555p-5,  0x1.1111111111111p-7,  0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13,
    0x1.a01a01a01a01ap-16, 0x1.71de3a556c734p-19, 0x1.27e4fb7789f5cp-22, 0x1.ae64567f544e4p-26,
    0x1.1eed8eff8d898p-29, 0x1.6124613a86d09p-33, 0x1.93974a8c07c9dp-37, 0x1.ae7f3e733b81fp-41,
    0x1.ae7f3e733b81fp-45, 0x1.952c77030ad4ap-49, 0x1.6827863b97d97p-53, 0x1.2f49b46814157p-57};

static double orc_expm1_pos(double y) {
  if (y < 0.5) {
    double q = inv_fact[17];
    for (int k = 16; k >= 1; k--) q = q * y + inv_fact[k];
    return q * y;
  }
  double k = floor(y * 0x1.71547652b82fep+0 + 0.5);
  double r = (y - k * 0x1.62e42fee00000p-1) - k * 0x1.a39ef35793c76p-33;
  double p = inv_fact[13];
  for (int j = 12; j >= 0; j--) p = p * r + inv_fact[j];
  uint64_t bits = (uint64_t)((int64_t)k + 1023) << 52;
  double scale;
  memcpy(&scale, &bits, sizeof scale);
  return p * scale - 1.0;
}

double orc_tanh(double x) {
  double ax = fabs(x);
  if (!(ax < 20.0)) {
    if (x > 0) return 1.0;
    if (x < 0) return -1.0;
    return x;
  }
  if (ax == 0.0) return x;
  double e = orc_expm1_pos(2.0 * ax);
  double t = e / (e + 2.0);
  return x < 0 ? -t : t;
}

/* ------------------------------------------------------------------------ */
/* walker lifetime                                                           */
/* ------------------------------------------------------------------------ */

orc_walker *orc_walker_create(const orc_model *m, double T, uint64_t seed, uint64_t stream,
                              double init_num_worms, double attenuation, double target_fraction,
                              int64_t thermalization) {
  orc_walker *w = (orc_walker *)calloc(1, sizeof(orc_walker));
  if (!w) return NULL;
  w->T = T;
  w->seed = seed;
  w->stream = stream;
  w->target_worm_length_fraction = target_fraction;
  w->num_worms_attenuation_factor = attenuation;
  w->avg_worm_length = 1.0;
  w->num_worms = init_num_worms;
  w->thermalization = thermalization;
  w->worm_cap_factor = 64;
  w->state = (uint8_t *)calloc((size_t)m->nsites, 1);
  w->v_first = (int32_t *)malloc(sizeof(int32_t) * (size_t)m->nsites);
  w->v_last = (int32_t *)malloc(sizeof(int32_t) * (size_t)m->nsites);
  w->nobs = ORC_OBS_BASE + ORC_OBS_PER_EST * m->nest;
  w->obs_sum = (double *)calloc((size_t)w->nobs, sizeof(double));
  w->obs_last = (double *)calloc((size_t)w->nobs, sizeof(double));
  w->obs_count = (int64_t *)calloc((size_t)w->nobs, sizeof(int64_t));
  if (!w->state || !w->v_first || !w->v_last || !w->obs_sum || !w->obs_last || !w->obs_count) {
    orc_walker_destroy(w);
    return NULL;
  }
  return w;
}

void orc_walker_destroy(orc_walker *w) {
  if (!w) return;
  free(w->ops);
  free(w->ops_saved);
  free(w->state);
  free(w->vertices);
  free(w->v_first);
  free(w->v_last);
  free(w->obs_sum);
  free(w->obs_last);
  free(w->obs_count);
  free(w);
}

static int reserve_ops(orc_walker *w, int64_t L) {
  if (L <= w->ops_cap) return ORC_OK;
  int64_t cap = L + L / 2 + 16;
  uint32_t *p = (uint32_t *)realloc(w->ops, sizeof(uint32_t) * (size_t)cap);
  if (!p) return ORC_ERR_NOMEM;
  w->ops = p;
  w->ops_cap = cap;
  return ORC_OK;
}

int orc_set_opstring(orc_walker *w, const uint32_t *ops, int64_t L, int64_t num_operators) {
  int rc = reserve_ops(w, L);
  if (rc) return rc;
  memcpy(w->ops, ops, sizeof(uint32_t) * (size_t)L);
  w->L = L;
  w->num_operators = num_operators;
  return ORC_OK;
}

int orc_set_state(const orc_model *m, orc_walker *w, const uint8_t *state) {
  memcpy(w->state, state, (size_t)m->nsites);
  return ORC_OK;
}

static void observe(orc_walker *w, int idx, double value) {
  w->obs_sum[idx] += value;
  w->obs_last[idx] = value;
  w->obs_count[idx] += 1;
}

/* ------------------------------------------------------------------------ */
/* helpers on the device opcode layout (bit0 non-identity, bit1 diagonal,    */
/* bits 2..10 vertex index, bits 11..31 bond)                                 */
/* ------------------------------------------------------------------------ */

static inline uint32_t op_bond(uint32_t op) { return op >> 11; }
static inline int32_t op_vcode(uint32_t op) { return (int32_t)((op >> 1) & 0x3FFu); }
static inline uint32_t make_op(uint32_t bond, int32_t vcode) { return 1u | ((uint32_t)vcode << 1) | (bond << 11); }

static inline const uint8_t *vertex_legs(const orc_model *m, int32_t type, int32_t vcode) {
  return m->leg_state + 4 * ((int64_t)m->type_vert_off[type] + (vcode >> 1));
}

/* ------------------------------------------------------------------------ */
/* diagonal update, src/sse.jl:137-191                                       */
/* ------------------------------------------------------------------------ */

int orc_diagonal_update(const orc_model *m, orc_walker *w, int32_t thermalized) {
  /* 138-145: grow the cutoff */
  if ((double)w->num_operators >= (double)w->L * 0.5) {
    if (thermalized) w->resize_after_thermalization++;
    int64_t old_length = w->L;
    int64_t new_length = (int64_t)floor((double)old_length * 1.5 + 100);
    int rc = reserve_ops(w, new_length);
    if (rc) return rc;
    for (int64_t p = old_length; p < new_length; p++) w->ops[p] = 0;
    w->L = new_length;
  }

  const double p_make_bond_raw = (double)m->nbonds / w->T;
  const double p_remove_bond_raw = w->T / (double)m->nbonds;
  const int64_t L = w->L;

  for (int64_t iop = 0; iop < L; iop++) {
    uint32_t op = w->ops[iop];
    w->slot_visits_total++;
    if (op == 0) {
      int64_t bond = rand_range(w, (uint64_t)m->nbonds) - 1;
      int32_t type = m->bond_type[bond];
      int32_t si = m->bond_sites[2 * bond], sj = m->bond_sites[2 * bond + 1];
      /* join_idx(dims, (state[i], state[j])) -- first site fastest */
      int32_t state_idx = (int32_t)w->state[si] + m->type_dims[2 * type] * (int32_t)w->state[sj];
      int32_t new_vert = m->diag_vertex[m->type_diag_off[type] + state_idx];
      double weight = new_vert < 0 ? 0.0 : m->weight[m->type_vert_off[type] + (new_vert >> 1)];
      double p_make_bond = p_make_bond_raw / (double)(L - w->num_operators);
      if (rand01(w) < p_make_bond * weight) {
        w->ops[iop] = make_op((uint32_t)bond, new_vert);
        w->num_operators += 1;
      }
    } else {
      uint32_t bond = op_bond(op);
      int32_t type = m->bond_type[bond];
      int32_t vc = op_vcode(op);
      if (vc & 1) {
        double weight = m->weight[m->type_vert_off[type] + (vc >> 1)];
        double p_remove_bond = (double)(L - w->num_operators + 1) * p_remove_bond_raw;
        if (rand01(w) * weight < p_remove_bond) {
          w->ops[iop] = 0;
          w->num_operators -= 1;
        }
      } else {
        const uint8_t *ls = vertex_legs(m, type, vc);
        w->state[m->bond_sites[2 * bond]] = ls[2];
        w->state[m->bond_sites[2 * bond + 1]] = ls[3];
      }
    }
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* vertex list, src/vertex_list.jl:15-54                                     */
/* ------------------------------------------------------------------------ */

int orc_make_vertex_list(const orc_model *m, orc_walker *w) {
  if (w->vertices_len != w->L) {
    free(w->vertices);
    w->vertices = (int32_t *)malloc(sizeof(int32_t) * 4 * (size_t)(w->L > 0 ? w->L : 1));
    if (!w->vertices) return ORC_ERR_NOMEM;
    w->vertices_len = w->L;
  }
  for (int64_t i = 0; i < 4 * w->L; i++) w->vertices[i] = -1;
  for (int32_t i = 0; i < m->nsites; i++) w->v_first[i] = w->v_last[i] = -1;

  for (int64_t p = 0; p < w->L; p++) {
    uint32_t op = w->ops[p];
    if (op == 0) continue;
    uint32_t bond = op_bond(op);
    for (int s = 0; s < 2; s++) {
      int32_t site = m->bond_sites[2 * bond + s];
      int32_t last = w->v_last[site];
      if (last >= 0) {
        w->vertices[last] = (int32_t)(4 * p + s);
        w->vertices[4 * p + s] = last;
      } else {
        w->v_first[site] = (int32_t)(4 * p + s);
      }
      w->v_last[site] = (int32_t)(4 * p + 2 + s);
    }
  }
  for (int32_t i = 0; i < m->nsites; i++) {
    if (w->v_first[i] >= 0) {
      w->vertices[w->v_first[i]] = w->v_last[i];
      w->vertices[w->v_last[i]] = w->v_first[i];
    }
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* worm update, src/sse.jl:193-303                                           */
/* ------------------------------------------------------------------------ */

static int64_t worm_traverse(const orc_model *m, orc_walker *w) {
  if (w->num_operators == 0) return 0;
  int64_t p0;
  int32_t l0;
  for (;;) {
    p0 = rand_range(w, (uint64_t)w->L) - 1;
    l0 = (int32_t)rand_range(w, 4) - 1;
    if (w->vertices[4 * p0 + l0] >= 0) break;
  }
  uint32_t op0 = w->ops[p0];
  int32_t site0 = m->bond_sites[2 * op_bond(op0) + (l0 & 1)];
  int32_t wormfunc0 = (int32_t)rand_range(w, (uint64_t)(m->site_dims[site0] - 1));

  int32_t leg_in = l0, wormfunc = wormfunc0;
  int64_t p = p0;
  int64_t worm_length = 1;
  const int64_t cap = (int64_t)w->worm_cap_factor * (w->L + 16 > ORC_WORM_CAP_MIN_SLOTS ? w->L + 16 : ORC_WORM_CAP_MIN_SLOTS);
  for (;;) {
    uint32_t op = w->ops[p];
    uint32_t bond = op_bond(op);
    int32_t type = m->bond_type[bond];
    int32_t vc = op_vcode(op);
    double random = rand01(w);
    w->worm_steps_total++;
    /* scatter, vertex_data.jl:106-125 */
    int64_t ti = (int64_t)m->type_trans_off[type] +
                 ((int64_t)(vc >> 1) * 4 + leg_in) * m->type_maxworm[type] + (wormfunc - 1);
    int32_t start = m->trans_start[ti], count = m->trans_count[ti];
    int32_t found = -1;
    if (start >= 0) {
      for (int32_t o = start; o < start + count; o++) {
        if (random < m->out_cum[o]) {
          found = o;
          break;
        }
      }
    }
    if (found < 0) {
      w->status = ORC_ERR_INVALID_VERTEX;
      return -1;
    }
    int32_t leg_out = m->out_leg[found];
    int32_t wormfunc_out = m->out_worm[found];
    w->ops[p] = make_op(bond, m->out_target[found]);
    int32_t dim_out = m->site_dims[m->bond_sites[2 * bond + (leg_out & 1)]];

    if (p == p0 && leg_out == l0 && wormfunc_out == dim_out - wormfunc0) break;
    worm_length += 1;
    if (worm_length > cap) {
      w->status = ORC_ERR_WORM_CAP;
      return -1;
    }
    wormfunc = wormfunc_out;
    int32_t link = w->vertices[4 * p + leg_out];
    leg_in = link & 3;
    p = link >> 2;
    if (p == p0 && leg_in == l0 && wormfunc == wormfunc0) break;
  }
  return worm_length;
}

int orc_worm_update(const orc_model *m, orc_walker *w, int32_t thermalized) {
  double total_worm_length = 1.0;
  int64_t nworms = (int64_t)ceil(w->num_worms);
  /* thermalisation: keep the opstring of the diagonal update, to undo the worm phase at the cap */
  if (!thermalized && nworms > 0 && w->num_operators > 0) {
    if (w->L > w->ops_saved_cap) {
      uint32_t *p = (uint32_t *)realloc(w->ops_saved, sizeof(uint32_t) * (size_t)w->ops_cap);
      if (!p) return w->status = ORC_ERR_NOMEM;
      w->ops_saved = p;
      w->ops_saved_cap = w->ops_cap;
    }
    memcpy(w->ops_saved, w->ops, sizeof(uint32_t) * (size_t)w->L);
  }
  for (int64_t i = 0; i < nworms; i++) {
    int64_t len = worm_traverse(m, w);
    if (len < 0 && w->status == ORC_ERR_WORM_CAP && !thermalized) {
      memcpy(w->ops, w->ops_saved, sizeof(uint32_t) * (size_t)w->L);
      w->status = ORC_OK;
      w->worm_undos++;
      return ORC_OK;
    }
    if (len < 0) return w->status;
    total_worm_length += (double)len;
  }
  if (thermalized && w->num_operators != 0)
    observe(w, 5, total_worm_length / (double)w->num_operators);

  double avg_worm_length = total_worm_length / ceil(w->num_worms);
  if (!thermalized) {
    const double a = w->num_worms_attenuation_factor;
    w->avg_worm_length += a * (avg_worm_length - w->avg_worm_length);
    double target_worms = w->target_worm_length_fraction * (double)w->num_operators / w->avg_worm_length;
    double diff = target_worms - w->num_worms;
    w->num_worms += a * (diff + 100.0 * orc_tanh(diff));
    if (a != 0) {
      double hi = 1.0 + (double)w->num_operators / 2.0;
      double x = w->num_worms;
      w->num_worms = x > hi ? hi : (x < 1.0 ? 1.0 : x);
    }
  }

  for (int32_t i = 0; i < m->nsites; i++) {
    int32_t vf = w->v_first[i];
    if (vf < 0) {
      w->state[i] = (uint8_t)(rand_range(w, (uint64_t)m->site_dims[i]) - 1);
    } else {
      uint32_t op = w->ops[vf >> 2];
      w->state[i] = vertex_legs(m, m->bond_type[op_bond(op)], op_vcode(op))[vf & 3];
    }
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* init! / sweep! / measure!                                                  */
/* ------------------------------------------------------------------------ */

int orc_init(const orc_model *m, orc_walker *w, int64_t init_cutoff, int32_t warmup_sweeps) {
  for (int32_t i = 0; i < m->nsites; i++) w->state[i] = (uint8_t)(rand_range(w, (uint64_t)m->site_dims[i]) - 1);
  if (init_cutoff < 0) init_cutoff = (int64_t)nearbyint((double)m->nsites * w->T); /* round-half-even */
  int rc = reserve_ops(w, init_cutoff > 0 ? init_cutoff : 1);
  if (rc) return rc;
  for (int64_t p = 0; p < init_cutoff; p++) w->ops[p] = 0;
  w->L = init_cutoff;
  w->num_operators = 0;
  for (int32_t s = 0; s < warmup_sweeps; s++) {
    rc = orc_diagonal_update(m, w, 0);
    if (rc) return rc;
  }
  return ORC_OK;
}

int orc_sweep(const orc_model *m, orc_walker *w, int32_t thermalized) {
  int rc = orc_diagonal_update(m, w, thermalized);
  if (rc) return rc;
  rc = orc_make_vertex_list(m, w);
  if (rc) return rc;
  return orc_worm_update(m, w, thermalized);
}

int orc_measure(const orc_model *m, orc_walker *w) {
  /* measure_sign, src/sse.jl:305-314 */
  int64_t negs = 0;
  for (int64_t p = 0; p < w->L; p++) {
    uint32_t op = w->ops[p];
    if (op == 0) continue;
    int32_t type = m->bond_type[op_bond(op)];
    negs += m->sign[m->type_vert_off[type] + (op_vcode(op) >> 1)] < 0;
  }
  const double sign = (negs & 1) ? -1.0 : 1.0;
  const double n = (double)w->num_operators;
  observe(w, 0, sign);
  observe(w, 1, n);
  observe(w, 2, sign * n);
  observe(w, 3, sign * (n * n));
  observe(w, 4, -sign * (n * w->T + m->energy_offset) / m->norm_site_count);

  /* measure_opstring! with MagnetizationEstimator, one pass per estimator */
  const int32_t N = m->nsites, md = m->maxdim;
  uint8_t *st = (uint8_t *)malloc((size_t)N);
  if (!st) return ORC_ERR_NOMEM;
  for (int32_t e = 0; e < m->nest; e++) {
    const double *coef = m->est_coef + (int64_t)e * N * md;
    memcpy(st, w->state, (size_t)N);
    double tmpmag = 0.0;
    for (int32_t i = 0; i < N; i++) tmpmag += coef[(int64_t)i * md + st[i]];
    double mag = tmpmag, absmag = fabs(tmpmag), mag2 = tmpmag * tmpmag, mag4 = (tmpmag * tmpmag) * (tmpmag * tmpmag);
    double est_n = 1.0;
    for (int64_t p = 0; p < w->L; p++) {
      uint32_t op = w->ops[p];
      if (op == 0) continue;
      uint32_t bond = op_bond(op);
      int32_t vc = op_vcode(op);
      if (!(vc & 1)) {
        const uint8_t *ls = vertex_legs(m, m->bond_type[bond], vc);
        for (int l = 0; l < 2; l++) {
          int32_t site = m->bond_sites[2 * bond + l];
          st[site] = ls[2 + l];
          tmpmag += coef[(int64_t)site * md + ls[2 + l]] - coef[(int64_t)site * md + ls[l]];
        }
      }
      mag += tmpmag;
      absmag += fabs(tmpmag);
      double t2 = tmpmag * tmpmag;
      mag2 += t2;
      mag4 += t2 * t2;
      est_n += 1.0;
    }
    const double norm = 1.0 / m->norm_site_count;
    mag *= norm;
    absmag *= norm;
    mag2 *= norm * norm;
    mag4 *= (norm * norm) * (norm * norm);
    const int base = ORC_OBS_BASE + ORC_OBS_PER_EST * e;
    observe(w, base + 0, sign * mag / est_n);
    observe(w, base + 1, sign * absmag / est_n);
    observe(w, base + 2, sign * mag2 / est_n);
    observe(w, base + 3, sign * mag4 / est_n);
    double chi = 1.0 / w->T / (est_n + 1.0) / est_n * (mag * mag + mag2) * m->norm_site_count;
    observe(w, base + 4, sign * chi);
  }
  free(st);
  return ORC_OK;
}

int orc_step(const orc_model *m, orc_walker *w, int32_t do_measure) {
  int rc = orc_sweep(m, w, w->sweeps > w->thermalization);
  if (rc) return rc;
  w->sweeps += 1;
  if (do_measure && w->sweeps > w->thermalization) return orc_measure(m, w);
  return ORC_OK;
}

int orc_run(const orc_model *m, orc_walker *w, int64_t nsteps, int32_t do_measure) {
  for (int64_t i = 0; i < nsteps; i++) {
    int rc = orc_step(m, w, do_measure);
    if (rc) return rc;
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* one chain per thread                                                       */
/* ------------------------------------------------------------------------ */

typedef struct {
  const orc_model *m;
  orc_walker **ws;
  int32_t nwalkers, tid, nthreads, do_measure;
  int64_t nsteps;
  int rc;
} par_arg;

static void *par_main(void *p) {
  par_arg *a = (par_arg *)p;
  for (int32_t i = a->tid; i < a->nwalkers; i += a->nthreads) {
    int rc = orc_run(a->m, a->ws[i], a->nsteps, a->do_measure);
    if (rc) a->rc = rc;
  }
  return NULL;
}

int orc_run_parallel(const orc_model *m, orc_walker **ws, int32_t nwalkers, int64_t nsteps,
                     int32_t do_measure, int32_t nthreads) {
  if (nthreads < 1) nthreads = 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
  par_arg *args = (par_arg *)calloc((size_t)nthreads, sizeof(par_arg));
  if (!th || !args) {
    free(th);
    free(args);
    return ORC_ERR_NOMEM;
  }
  for (int32_t t = 0; t < nthreads; t++) {
    args[t] = (par_arg){m, ws, nwalkers, t, nthreads, do_measure, nsteps, 0};
    pthread_create(&th[t], NULL, par_main, &args[t]);
  }
  int rc = 0;
  for (int32_t t = 0; t < nthreads; t++) {
    pthread_join(th[t], NULL);
    if (args[t].rc) rc = args[t].rc;
  }
  free(th);
  free(args);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* parallel tempering: Carlo.parallel_tempering_log_weight_ratio and         */
/* parallel_tempering_change_parameter! (src/sse.jl:390-405)                 */
/* ------------------------------------------------------------------------ */

/* exp(lwr(a, T_b) + lwr(b, T_a)), lwr(mc, T') = -n log(T'/T) (src/sse.jl:390-396), written as the
 * integer power (T_a/T_b)^(n_a - n_b) and evaluated by binary powering */
double orc_tempering_weight(double Ta, double Tb, int64_t na, int64_t nb) {
  uint64_t e;
  double b;
  if (na >= nb) {
    e = (uint64_t)(na - nb);
    b = Ta / Tb;
  } else {
    e = (uint64_t)(nb - na);
    b = Tb / Ta;
  }
  double q = 1.0;
  while (e) {
    if (e & 1u) q = q * b;
    e >>= 1;
    if (e) b = b * b;
  }
  return q;
}

int orc_tempering_exchange(orc_walker **ws, int32_t nladders, int32_t nrungs, uint64_t seed, uint64_t step,
                           int32_t *accepted) {
  if (nrungs < 2) return ORC_ERR_ARG;
  int32_t *order = (int32_t *)malloc(sizeof(int32_t) * (size_t)nrungs);
  if (!order) return ORC_ERR_NOMEM;
  int rc = ORC_OK;
  for (int32_t l = 0; l < nladders; l++) {
    orc_walker **lw = ws + (size_t)l * nrungs;
    int32_t *acc = accepted + (size_t)l * (nrungs - 1);
    /* rank the ladder by temperature (insertion sort), distinct temperatures required */
    int dup = 0;
    for (int32_t k = 0; k < nrungs; k++) {
      int32_t j = k;
      while (j > 0 && lw[order[j - 1]]->T > lw[k]->T) {
        order[j] = order[j - 1];
        j--;
      }
      order[j] = k;
    }
    for (int32_t k = 0; k + 1 < nrungs; k++)
      if (lw[order[k]]->T == lw[order[k + 1]]->T) dup = 1;
    for (int32_t k = 0; k + 1 < nrungs; k++) acc[k] = -1;
    if (dup) {
      rc = ORC_ERR_ARG;
      continue;
    }
    for (int32_t k = (int32_t)(step & 1u); k + 1 < nrungs; k += 2) {
      orc_walker *a = lw[order[k]], *b = lw[order[k + 1]];
      if (a->status != ORC_OK || b->status != ORC_OK) continue;
      const double q = orc_tempering_weight(a->T, b->T, a->num_operators, b->num_operators);
      const uint32_t ctr[4] = {(uint32_t)step, (uint32_t)(step >> 32), (uint32_t)k, (uint32_t)l};
      const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
      uint32_t x[4];
      orc_philox4x32_10(ctr, key, x);
      const double u = (double)((((uint64_t)x[1] << 32) | x[0]) >> 11) * 0x1.0p-53;
      acc[k] = u < q;
      if (acc[k]) {
        /* parallel_tempering_change_parameter! on both walkers (src/sse.jl:399-405); the
         * observable accumulators stay with their temperature */
        const double t = a->T;
        a->T = b->T;
        b->T = t;
        for (int32_t i = 0; i < a->nobs; i++) {
          const double s = a->obs_sum[i], z = a->obs_last[i];
          const int64_t c = a->obs_count[i];
          a->obs_sum[i] = b->obs_sum[i];
          a->obs_last[i] = b->obs_last[i];
          a->obs_count[i] = b->obs_count[i];
          b->obs_sum[i] = s;
          b->obs_last[i] = z;
          b->obs_count[i] = c;
        }
      }
    }
  }
  free(order);
  return rc;
}

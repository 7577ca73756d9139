/*
 * pt_oracle.c -- CPU restatement of PySA's parallel-tempering Metropolis core.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the CUDA path is compared
 * against (tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg); the
 * product never links or calls it.
 *
 * It follows the reference algorithm step for step, with one substitution: the
 * random numbers come from the counter-based stream spec shared with the GPU
 * (Philox4x32-10 keyed by instance/read/replica/sweep/spin), so a GPU run and
 * an oracle run on the same seed make the same decisions.  The reference draws
 * from numba's Mersenne Twister instead; the golden vectors in tests/golden
 * pin this restatement to the reference's own update rule by feeding that same
 * stream into pysa.ising.update_spin / pysa.qubo.update_spin.
 *
 * Reference lines restated (paths inside nasa/PySA):
 *   pysa/ising.py:32-37, pysa/qubo.py:32-37   get_energy  E = s.(J s / 2 + h)
 *   pysa/ising.py:40-63, pysa/qubo.py:40-63   update_spin (dense dot per attempt)
 *   pysa/ising.py:66-92, pysa/qubo.py:66-92   update_spin_ref (AIS rule)
 *   pysa/simulation.py:41-76                  random_sweep / sequential_sweep
 *   pysa/simulation.py:123-181                simulation_parallel (per-replica best)
 *   pysa/simulation.py:184-236                simulation_sequential (global best)
 *   pysa/simulation.py:293-317                ais_sample
 *   pysa/utils.py:26-58                       pt (replica exchange of beta_idx)
 *   pysa/ais.py:79-112                        get_log_omega
 *   pysa/sa.py:204-205                         float_type='float64' runs
 *                                              (orc_pt_run64, f64 throughout)
 *
 * Numeric spec (identical on the GPU):
 *   u(x)      = (x + 0.5) * 2^-32 for a Philox output word x  (exact in f64)
 *   accept    = dn >= 0  ||  log(u) < (double)beta * (double)dn
 *   PT swap   = de >= 0  ||  u < exp((double)de), de = f32((E1-E2)*(b1-b2))
 *   sweep energy delta accumulated in f64, added to the f32 energy per sweep.
 * Build with -ffp-contract=off so x86 and Arm builds round identically.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_ISING 0
#define ORC_QUBO 1

/* ---------------------------------------------------------------- Philox */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).  Round: (hi,lo) of the two
 * 32x32 products of counter words 0 and 2 with the multipliers, words mixed
 * with the key; key bumped by the Weyl constants between rounds. */
static inline uint32_t mulhi32(uint32_t a, uint32_t b) {
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
}

void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint32_t lo0 = 0xD2511F53u * c0, hi0 = mulhi32(0xD2511F53u, c0);
    uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = mulhi32(0xCD9E8D57u, c2);
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

/* Stream tags in the top counter word: (instance << 4) | tag. */
#define ORC_TAG_SWEEP 0u
#define ORC_TAG_PT 1u
#define ORC_TAG_PERM 2u
#define ORC_TAG_AIS 3u

/* One 32-bit draw: word (idx & 3) of Philox(ctr = (idx >> 2, a, b, inst<<4|tag)). */
uint32_t orc_draw(uint64_t seed, uint32_t tag, uint32_t inst, uint32_t a,
                  uint32_t b, uint32_t idx) {
  uint32_t ctr[4] = {idx >> 2, a, b, (inst << 4) | tag};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t out[4];
  orc_philox(ctr, key, out);
  return out[idx & 3];
}

static inline double u_of(uint32_t x) { return ((double)x + 0.5) * 0x1p-32; }

/* Fisher-Yates visiting order for one (instance, sweep); shared by all chains
 * of the instance.  j = floor(x * (i+1) / 2^32). */
void orc_permutation(uint64_t seed, uint32_t inst, uint32_t sweep, int n,
                     int32_t *perm) {
  for (int i = 0; i < n; ++i) perm[i] = i;
  for (int i = n - 1; i > 0; --i) {
    uint32_t x = orc_draw(seed, ORC_TAG_PERM, inst, sweep, 0, (uint32_t)i);
    int j = (int)(((uint64_t)x * (uint64_t)(i + 1)) >> 32);
    int32_t t = perm[i];
    perm[i] = perm[j];
    perm[j] = t;
  }
}

/* ---------------------------------------------------------------- energy */
/* E = s.(J s/2 + h) accumulated in f64 (reference: pysa/ising.py:32-37). */
double orc_energy64(int n, int ld, const float *J, const float *h,
                    const float *s) {
  double e = 0.0;
  for (int i = 0; i < n; ++i) {
    if (s[i] == 0.0f) continue;
    double f = 0.0;
    const float *row = J + (size_t)i * ld;
    for (int j = 0; j < n; ++j) f += (double)row[j] * (double)s[j];
    e += (double)s[i] * (0.5 * f + (double)h[i]);
  }
  return e;
}

/* f32 dot in a fixed order: eight interleaved partial sums, then summed in
 * index order.  Deterministic on every host; exact for integer couplings. */
static inline float dot8(const float *a, const float *b, int n) {
  float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int j = 0;
  for (; j + 8 <= n; j += 8)
    for (int k = 0; k < 8; ++k) acc[k] += a[j + k] * b[j + k];
  for (; j < n; ++j) acc[j & 7] += a[j] * b[j];
  float s = 0.0f;
  for (int k = 0; k < 8; ++k) s += acc[k];
  return s;
}

/* Metropolis rule of pysa/ising.py:40-63 and pysa/qubo.py:40-63.  Returns the
 * energy change (-dn) of the attempt, 0 on reject. */
static inline float attempt(int ptype, int n, int ld, const float *J,
                            const float *h, float *s, int pos, float beta,
                            uint32_t x) {
  float field = dot8(J + (size_t)pos * ld, s, n) + h[pos];
  float dn = (ptype == ORC_ISING) ? 2.0f * s[pos] * field
                                  : (2.0f * s[pos] - 1.0f) * field;
  int acc = dn >= 0.0f;
  if (!acc) acc = log(u_of(x)) < (double)beta * (double)dn;
  if (!acc) return 0.0f;
  if (ptype == ORC_ISING)
    s[pos] = -s[pos];
  else
    s[pos] = (s[pos] != 0.0f) ? 0.0f : 1.0f;
  return -dn;
}

/* ------------------------------------------------------ PT driver (batch) */
typedef struct {
  int32_t problem_type; /* 0 ising, 1 qubo */
  int32_t n;            /* spins */
  int32_t ld;           /* row stride of J (>= n) */
  int32_t replicas;     /* R */
  int32_t reads;        /* Rd; chain = read * R + replica */
  int32_t inst;         /* instance index used in the RNG counter */
  int32_t update;       /* 0 sequential, 1 random */
  int32_t use_pt;
  int32_t best_mode;    /* 0 per replica (simulation_parallel), 1 global */
  int32_t log_omega;    /* 1: record get_log_omega per sweep */
  int32_t exchange_every; /* <= 1: exchange after every sweep (the
                             reference); k: only after sweeps with
                             (s + 1) % k == 0 (the GPU's opt-in knob) */
  uint64_t seed;
} orc_pt_args;

static inline int exchange_after(const orc_pt_args *a, int64_t sw) {
  return a->exchange_every <= 1 || (sw + 1) % a->exchange_every == 0;
}

typedef struct {
  float *spins;       /* [reads*R, n] values +-1 or {0,1} */
  float *energies;    /* [reads*R] */
  int32_t *beta_idx;  /* [reads, R]  slot -> replica */
  float *best_energy; /* [reads*R] per chain */
  int32_t *best_sweep;/* [reads*R] */
  float *best_spins;  /* [reads*R, n] */
  double *log_omega;  /* [reads, lo_stride] */
  int32_t lo_stride;
} orc_pt_state;

/* utils.pt restated (pysa/utils.py:44-58): hottest slot pair first, swaps the
 * slot -> replica map, uniform drawn per pair index whether used or not. */
static void pt_step(const orc_pt_args *a, const float *betas, const float *E,
                    int32_t *bidx, uint32_t read, uint32_t sweep) {
  int R = a->replicas;
  for (int k = 0; k < R - 1; ++k) {
    int k1 = R - k - 1, k2 = R - k - 2;
    float de = (E[bidx[k1]] - E[bidx[k2]]) * (betas[k1] - betas[k2]);
    int swap = de >= 0.0f;
    if (!swap) {
      uint32_t x = orc_draw(a->seed, ORC_TAG_PT, a->inst, sweep, read, k);
      swap = u_of(x) < exp((double)de);
    }
    if (swap) {
      int32_t t = bidx[k1];
      bidx[k1] = bidx[k2];
      bidx[k2] = t;
    }
  }
}

/* get_log_omega restated (pysa/ais.py:79-112); sorted_slots = argsort(betas). */
static double log_omega_of(int R, const float *betas, const int32_t *sorted,
                           const int32_t *bidx, const float *E) {
  double lw = 0.0;
  float beta_old = 0.0f;
  for (int r = 1; r < R; ++r) {
    float b = betas[sorted[r]];
    float e = E[bidx[sorted[r]]];
    float t1 = -b * e, t2 = -beta_old * e;
    lw += (double)(float)(t1 - t2);
    beta_old = b;
  }
  return lw;
}

/* Run sweeps [first_sweep, first_sweep + num_sweeps) over every read.
 * Mirrors simulation_parallel: sweep all replicas at their slot's beta, update
 * per-chain bests (strict <), exchange, then log-omega.  nthreads <= 0 uses
 * all OpenMP threads; chains of a sweep run in parallel like numba.prange. */
int orc_pt_run(const orc_pt_args *a, const float *J, const float *h,
               const float *betas, const int32_t *sorted_slots,
               orc_pt_state *st, int64_t first_sweep, int32_t num_sweeps,
               int nthreads) {
  const int n = a->n, R = a->replicas, Rd = a->reads;
  const int64_t C = (int64_t)R * Rd;
  int32_t *perm = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  float *cbeta = (float *)malloc(sizeof(float) * (size_t)(C > 0 ? C : 1));
  if (!perm || !cbeta) {
    free(perm);
    free(cbeta);
    return -1;
  }
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  (void)nthreads;
#endif
  for (int64_t sw = first_sweep; sw < first_sweep + num_sweeps; ++sw) {
    uint32_t sweep = (uint32_t)sw;
    if (a->update == 1) orc_permutation(a->seed, a->inst, sweep, n, perm);
    /* betas_sorted[beta_idx[k]] = betas[k] per read (simulation.py:151-152) */
    for (int rd = 0; rd < Rd; ++rd)
      for (int k = 0; k < R; ++k)
        cbeta[(int64_t)rd * R + st->beta_idx[(int64_t)rd * R + k]] = betas[k];
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (int64_t c = 0; c < C; ++c) {
      float *s = st->spins + c * n;
      double dE = 0.0;
      for (int t = 0; t < n; ++t) {
        int pos = (a->update == 1) ? perm[t] : t;
        uint32_t x = orc_draw(a->seed, ORC_TAG_SWEEP, a->inst, sweep,
                              (uint32_t)c, (uint32_t)t);
        dE += (double)attempt(a->problem_type, n, a->ld, J, h, s, pos,
                              cbeta[c], x);
      }
      st->energies[c] = (float)((double)st->energies[c] + dE);
      if (st->energies[c] < st->best_energy[c]) {
        st->best_energy[c] = st->energies[c];
        st->best_sweep[c] = (int32_t)sw;
        memcpy(st->best_spins + c * n, s, sizeof(float) * (size_t)n);
      }
    }
    for (int rd = 0; rd < Rd; ++rd) {
      int32_t *bidx = st->beta_idx + (int64_t)rd * R;
      const float *E = st->energies + (int64_t)rd * R;
      if (a->use_pt && exchange_after(a, sw))
        pt_step(a, betas, E, bidx, (uint32_t)rd, sweep);
      if (a->log_omega)
        st->log_omega[(int64_t)rd * st->lo_stride + sw] =
            log_omega_of(R, betas, sorted_slots, bidx, E);
    }
  }
  free(perm);
  free(cbeta);
  return 0;
}

/* --------------------------------------------- PT driver in f64 (batch) */
/* The same driver with the arithmetic the reference uses when the Solver is
 * built with float_type='float64' (pysa/sa.py:204-205 casts couplings, fields,
 * states and betas to it): f64 couplings and states, field J_pos.s + h_pos in
 * f64 (pysa/ising.py:48-49, pysa/qubo.py:48-49), dn and the acceptance test
 * in f64, f64 energies, exchange with de = (E1 - E2)(b1 - b2) in f64
 * (pysa/utils.py:44-58).  Same random stream and visiting orders as
 * orc_pt_run; per-replica best (simulation_parallel). */
typedef struct {
  double *spins, *energies;
  int32_t *beta_idx;
  double *best_energy;
  int32_t *best_sweep;
  double *best_spins;
} orc_pt_state64;

static inline double dot8_64(const double *a, const double *b, int n) {
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int j = 0;
  for (; j + 8 <= n; j += 8)
    for (int k = 0; k < 8; ++k) acc[k] += a[j + k] * b[j + k];
  for (; j < n; ++j) acc[j & 7] += a[j] * b[j];
  double s = 0.0;
  for (int k = 0; k < 8; ++k) s += acc[k];
  return s;
}

int orc_pt_run64(const orc_pt_args *a, const double *J, const double *h,
                 const double *betas, orc_pt_state64 *st, int64_t first_sweep,
                 int32_t num_sweeps, int nthreads) {
  const int n = a->n, R = a->replicas, Rd = a->reads;
  const int64_t C = (int64_t)R * Rd;
  int32_t *perm = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  double *cbeta = (double *)malloc(sizeof(double) * (size_t)(C > 0 ? C : 1));
  if (!perm || !cbeta) {
    free(perm);
    free(cbeta);
    return -1;
  }
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  (void)nthreads;
#endif
  for (int64_t sw = first_sweep; sw < first_sweep + num_sweeps; ++sw) {
    uint32_t sweep = (uint32_t)sw;
    if (a->update == 1) orc_permutation(a->seed, a->inst, sweep, n, perm);
    for (int rd = 0; rd < Rd; ++rd)
      for (int k = 0; k < R; ++k)
        cbeta[(int64_t)rd * R + st->beta_idx[(int64_t)rd * R + k]] = betas[k];
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (int64_t c = 0; c < C; ++c) {
      double *sp = st->spins + c * n;
      double dE = 0.0;
      for (int t = 0; t < n; ++t) {
        const int pos = (a->update == 1) ? perm[t] : t;
        const uint32_t x = orc_draw(a->seed, ORC_TAG_SWEEP, a->inst, sweep,
                                    (uint32_t)c, (uint32_t)t);
        const double field = dot8_64(J + (size_t)pos * a->ld, sp, n) + h[pos];
        const double dn = (a->problem_type == ORC_ISING)
                              ? 2.0 * sp[pos] * field
                              : (2.0 * sp[pos] - 1.0) * field;
        int acc = dn >= 0.0;
        if (!acc) acc = log(u_of(x)) < cbeta[c] * dn;
        if (!acc) continue;
        if (a->problem_type == ORC_ISING)
          sp[pos] = -sp[pos];
        else
          sp[pos] = (sp[pos] != 0.0) ? 0.0 : 1.0;
        dE -= dn;
      }
      st->energies[c] += dE;
      if (st->energies[c] < st->best_energy[c]) {
        st->best_energy[c] = st->energies[c];
        st->best_sweep[c] = (int32_t)sw;
        memcpy(st->best_spins + c * n, sp, sizeof(double) * (size_t)n);
      }
    }
    if (!a->use_pt || !exchange_after(a, sw)) continue;
    for (int rd = 0; rd < Rd; ++rd) {
      int32_t *bidx = st->beta_idx + (int64_t)rd * R;
      const double *E = st->energies + (int64_t)rd * R;
      for (int k = 0; k < R - 1; ++k) {
        const int k1 = R - k - 1, k2 = R - k - 2;
        const double de = (E[bidx[k1]] - E[bidx[k2]]) * (betas[k1] - betas[k2]);
        int swap = de >= 0.0;
        if (!swap) {
          const uint32_t x =
              orc_draw(a->seed, ORC_TAG_PT, a->inst, sweep, (uint32_t)rd, k);
          swap = u_of(x) < exp(de);
        }
        if (swap) {
          const int32_t t = bidx[k1];
          bidx[k1] = bidx[k2];
          bidx[k2] = t;
        }
      }
    }
  }
  free(perm);
  free(cbeta);
  return 0;
}

/* ------------------------------------------------------------------- AIS */
/* ais_sample restated (pysa/simulation.py:293-317) with update_spin_ref
 * (pysa/ising.py:66-92).  ref: 0 uniform, 1 bernoulli(p = P(bit 0 / spin -1)).
 * order: 0 = reference (weight after each sweep), 1 = standard (weight before).
 * J and h arrive already scaled by the target beta. */
typedef struct {
  int32_t problem_type, n, ld, num_temps, samples, inst, update, ref, order;
  double p;
  uint64_t seed;
} orc_ais_args;

static double ref_energy_of(const orc_ais_args *a, const float *s) {
  if (a->ref == 0) return 0.0;
  int c = 0;
  for (int i = 0; i < a->n; ++i) c += (s[i] == 1.0f);
  /* -log(p^(n-c) (1-p)^c) */
  return -((double)(a->n - c) * log((double)a->p) +
           (double)c * log(1.0 - (double)a->p));
}

int orc_ais_run(const orc_ais_args *a, const float *J, const float *h,
                const float *temps, float *samples, double *log_w,
                int nthreads) {
  const int n = a->n;
  int32_t *perms = NULL;
  if (a->update == 1) {
    perms = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * a->num_temps);
    if (!perms) return -1;
    for (int k = 0; k < a->num_temps; ++k)
      orc_permutation(a->seed, a->inst, (uint32_t)k, n, perms + (size_t)k * n);
  }
  const double lr = (a->ref == 1)
                        ? log((1.0 - (double)a->p) / (double)a->p)
                        : 0.0; /* log p0(bit->1)/p0(bit->0) */
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#else
  (void)nthreads;
#endif
  for (int smp = 0; smp < a->samples; ++smp) {
    float *s = samples + (size_t)smp * n;
    double lw = 0.0;
    float beta_old = 0.0f;
    for (int k = 0; k < a->num_temps; ++k) {
      float beta = temps[k];
      if (a->order == 1) {
        float e = (float)orc_energy64(n, a->ld, J, h, s);
        double re = ref_energy_of(a, s);
        double lk = (double)(-beta * e) - (1.0 - (double)beta) * re;
        double lm = (double)(-beta_old * e) - (1.0 - (double)beta_old) * re;
        lw += lk - lm;
      }
      for (int t = 0; t < n; ++t) {
        int pos = (a->update == 1) ? perms[(size_t)k * n + t] : t;
        uint32_t x = orc_draw(a->seed, ORC_TAG_AIS, a->inst, (uint32_t)k,
                              (uint32_t)smp, (uint32_t)t);
        float field = dot8(J + (size_t)pos * a->ld, s, n) + h[pos];
        float dn = (a->problem_type == ORC_ISING)
                       ? 2.0f * s[pos] * field
                       : (2.0f * s[pos] - 1.0f) * field;
        /* bit goes to 1 (spin +1) when s[pos] is the "0/-1" value */
        int up = (a->problem_type == ORC_ISING) ? (s[pos] < 0.0f)
                                                 : (s[pos] == 0.0f);
        double refd = up ? lr : -lr;
        double full = (double)beta * (double)dn + (1.0 - (double)beta) * refd;
        int acc = full >= 0.0;
        if (!acc) acc = log(u_of(x)) < full;
        if (acc) {
          if (a->problem_type == ORC_ISING)
            s[pos] = -s[pos];
          else
            s[pos] = (s[pos] != 0.0f) ? 0.0f : 1.0f;
        }
      }
      if (a->order == 0) {
        float e = (float)orc_energy64(n, a->ld, J, h, s);
        double re = ref_energy_of(a, s);
        double lk = (double)(-beta * e) - (1.0 - (double)beta) * re;
        double lm = (double)(-beta_old * e) - (1.0 - (double)beta_old) * re;
        lw += lk - lm;
      }
      beta_old = beta;
    }
    log_w[smp] = lw;
  }
  free(perms);
  return 0;
}

/* omegas_to_partition restated (pysa/ais.py:115-131). */
double orc_omegas_to_partition(const double *lw, int64_t ns, double logz0) {
  double m = -INFINITY;
  for (int64_t i = 0; i < ns; ++i)
    if (lw[i] > m) m = lw[i];
  double s = 0.0;
  for (int64_t i = 0; i < ns; ++i) s += exp(lw[i] - m);
  return m - log((double)ns) + logz0 + log(s);
}

/* Exact log Z = log sum_s exp(-beta E(s)) by Gray-code enumeration in f64. */
double orc_logz_exact(int ptype, int n, int ld, const float *J, const float *h,
                      double beta) {
  double *f = (double *)malloc(sizeof(double) * (size_t)n);
  double *s = (double *)malloc(sizeof(double) * (size_t)n);
  if (!f || !s) {
    free(f);
    free(s);
    return NAN;
  }
  double lo = (ptype == ORC_ISING) ? -1.0 : 0.0;
  for (int i = 0; i < n; ++i) s[i] = lo;
  double e = 0.0;
  for (int i = 0; i < n; ++i) {
    double acc = 0.0;
    for (int j = 0; j < n; ++j) acc += (double)J[(size_t)i * ld + j] * s[j];
    f[i] = acc;
  }
  for (int i = 0; i < n; ++i) e += s[i] * (0.5 * f[i] + (double)h[i]);
  /* two passes: max of -beta E, then the sum, both over the same Gray walk */
  double best = -INFINITY, total = 0.0;
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = 0; i < n; ++i) s[i] = lo;
    for (int i = 0; i < n; ++i) {
      double acc = 0.0;
      for (int j = 0; j < n; ++j) acc += (double)J[(size_t)i * ld + j] * s[j];
      f[i] = acc;
    }
    e = 0.0;
    for (int i = 0; i < n; ++i) e += s[i] * (0.5 * f[i] + (double)h[i]);
    uint64_t count = (uint64_t)1 << n;
    for (uint64_t g = 0; g < count; ++g) {
      double w = -beta * e;
      if (pass == 0) {
        if (w > best) best = w;
      } else {
        total += exp(w - best);
      }
      if (g + 1 == count) break;
      int i = __builtin_ctzll(g + 1); /* Gray code: flip bit ctz(g+1) */
      double ns = (ptype == ORC_ISING) ? -s[i] : 1.0 - s[i];
      double d = ns - s[i];
      e += d * (f[i] + (double)h[i]);
      for (int j = 0; j < n; ++j) f[j] += (double)J[(size_t)j * ld + i] * d;
      s[i] = ns;
    }
  }
  free(f);
  free(s);
  return best + log(total);
}

/*
 * pysa_gb.h -- C ABI of the GB300 parallel-tempering simulated-annealing core.
 *
 * Drop-in boundary for the hot path of nasa/PySA: the driver call
 *     simulation(update_spin, sweep, couplings, local_fields, states,
 *                energies, beta_idx, betas, n_sweeps, get_part_fun, use_pt)
 * made by pysa/sa.py:329-332 and pysa/sa.py:349-352 (drivers
 * pysa/simulation.py:123-236, update rules pysa/ising.py:40-63 and
 * pysa/qubo.py:40-63, exchange pysa/utils.py:26-58), the energy function
 * pysa/ising.py:32-37, and the AIS sampler of pysa/sa.py:432-553
 * (pysa/simulation.py:239-317, pysa/ais.py:79-131).
 *
 * Conventions
 *   - Every pointer in the structs below is DEVICE memory owned by the caller;
 *     the library allocates nothing and keeps no per-call state.
 *   - All work is enqueued on the given cudaStream_t (passed as void*);
 *     entry points return immediately.  They are reentrant per stream.
 *   - Return value: 0 on success, a negative PYSA_GB_ERR_* code otherwise;
 *     pysa_gb_last_error() returns a message for the calling thread.
 *     Device-side failures (a bounded wait that ran out) are reported in the
 *     caller's status word, read after the stream synchronises.
 *   - Spins are bit-packed: bit (j % 32) of word (j / 32) of a chain holds
 *     spin j; 1 means +1 (Ising) or 1 (QUBO), 0 means -1 (Ising) or 0 (QUBO).
 *   - A chain is one replica of one read of one instance; the chains of an
 *     instance are numbered read-major (read * R + replica) from
 *     chain_off[instance].
 */
#ifndef PYSA_GB_H
#define PYSA_GB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PYSA_GB_ABI_VERSION 2

enum {
  PYSA_GB_ISING = 0,
  PYSA_GB_QUBO = 1
};

enum {
  PYSA_GB_SEQUENTIAL = 0, /* sequential_sweep, pysa/simulation.py:60-76 */
  PYSA_GB_RANDOM = 1      /* random_sweep, pysa/simulation.py:41-57 */
};

enum {
  PYSA_GB_OK = 0,
  PYSA_GB_ERR_ARG = -1,     /* invalid argument */
  PYSA_GB_ERR_SIZE = -2,    /* size beyond what the kernels support */
  PYSA_GB_ERR_CUDA = -3,    /* a CUDA runtime call failed */
  PYSA_GB_ERR_TIMEOUT = -4, /* (status word) a bounded device wait ran out */
  PYSA_GB_ERR_NOBETA0 = -5, /* log-omega requested without a beta = 0 slot */
  PYSA_GB_ERR_DRIFT = -6    /* (status word) a chain's accumulated energy left
                               its recomputed value by more than 1e-3 of
                               max(1, |E|), or is not finite */
};

/* Largest number of spins per instance the sweep kernels accept.  Dense
 * instances up to 4096 spins keep their fields in registers (plain kernel);
 * wider ones keep them in the workspace's fields array (wide-instance
 * kernel); 64 <= n <= 2048 can take the tensor cores. */
#define PYSA_GB_MAX_N 65536

/* A batch of dense problems (one or many instances, uneven sizes allowed). */
typedef struct {
  int32_t problem_type;   /* PYSA_GB_ISING or PYSA_GB_QUBO */
  int32_t num_instances;
  int32_t max_n;          /* largest n over the instances */
  int32_t words;          /* spin words per chain = ceil(max_n / 32) */
  int64_t num_chains;     /* sum over instances of reads * replicas */
  int64_t num_reads;      /* sum over instances of reads */
  /* per-instance tables [num_instances] */
  const int32_t *n;         /* spins */
  const int32_t *replicas;  /* R */
  const int32_t *reads;     /* Rd */
  const int64_t *j_off;     /* element offset of J (n x ld, f32, row-major) */
  const int32_t *ld;        /* row stride of J, >= n, multiple of 4 */
  const int64_t *h_off;     /* element offset of h (n entries) */
  const int64_t *chain_off; /* first chain of the instance */
  const int64_t *read_off;  /* first read of the instance */
  const int64_t *ladder_off;/* offset of the instance's R betas (slot order) */
  /* per-read table [num_reads] */
  const int32_t *read_inst; /* instance of each read */
  /* data */
  const float *J;           /* couplings with zero diagonal (pysa/sa.py:67-70),
                               stored TRANSPOSED: row j of this buffer is
                               column j of the coupling matrix, i.e. the
                               field change when spin j flips (the same
                               thing for the symmetric problems accepted by
                               pysa/sa.py:64-65 up to allclose tolerance) */
  const float *h;           /* local fields = diagonal of the problem */
  const float *ladder;      /* inverse temperatures, slot order */
  const int32_t *ladder_sorted; /* per instance: argsort of its R betas */
  /* sparse rows of the instances flagged in pysa_gb_host_tables.sparse
   * (all NULL when none is).  Row i of instance k (row i of the transposed
   * couplings above, as every kernel reads them) has its nonzero entries
   * grouped by column % 8, ascending column inside a group; group g is
   * entries csr_rows[9 (csr_row_off[k] + i) + g] ..
   * csr_rows[9 (csr_row_off[k] + i) + g + 1] - 1, counted from the
   * instance's first entry csr_ent_off[k]. */
  const int64_t *csr_row_off; /* [num_instances] first row record (-1 dense) */
  const int64_t *csr_ent_off; /* [num_instances] first entry */
  const int32_t *csr_rows;    /* 9 int32 per row */
  const int32_t *csr_col;     /* column of each entry */
  const float *csr_val;       /* coupling of each entry */
  int32_t csr_width;          /* layout of the sparse rows, as
                                 pysa_gb_workspace.csr_width (0 grouped rows,
                                 4/8/16/32 fixed records); read by
                                 pysa_gb_prepare and pysa_gb_energy64_tables,
                                 which take sparse instances' fields and
                                 energies from these rows (their dense J is
                                 never read: j_off may point anywhere, ld >=
                                 n) */
  int32_t pad_;
} pysa_gb_problems;

/* Chain state, updated in place by the sweeps. */
typedef struct {
  uint32_t *spins;        /* [num_chains, words] */
  float *energies;        /* [num_chains] accumulated energies */
  int32_t *beta_idx;      /* [num_chains]: per read, slot k -> replica */
  float *chain_beta;      /* [num_chains] beta each chain runs at */
  float *best_energy;     /* [num_chains] lowest energy seen (strict <) */
  int32_t *best_sweep;    /* [num_chains] sweep index of best_energy */
  uint32_t *best_spins;   /* [num_chains, words] state at best_energy */
  double *log_omega;      /* [num_reads, log_omega_stride] or NULL */
  int64_t *sweep_counter; /* [1] index of the next sweep */
  int32_t *status;        /* [1] 0 or a PYSA_GB_ERR_* code from the device */
  uint32_t *ticket;       /* [1] zero-initialised scratch word */
  uint32_t *stream_key;   /* [num_chains] or NULL: per-chain change of the
                             sweep stream's key (0 = the plain stream);
                             pysa_gb_propose advances a chain's entry on every
                             proposal it accepts, so its later sweeps draw
                             fresh uniforms instead of replaying the ones
                             that would undo the move */
} pysa_gb_state;

/* Per-call workspace, caller-allocated (sizes from pysa_gb_workspace_bytes). */
typedef struct {
  float *fields;          /* local fields, [num_chains, field_ld] */
  int32_t field_ld;       /* row stride of fields (>= 32 * ceil(max_n/32),
                             a multiple of 4; fields 16-byte aligned) */
  int32_t perm_slots;     /* visiting orders held (sweeps per batch) */
  int32_t *perm;          /* [perm_slots, num_instances, max_n] */
  float *packed_j;        /* couplings in the sweep kernel's row layout */
  int64_t packed_j_elems; /* capacity of packed_j */
  int32_t *items;         /* [num_items, 8] work list of the sweep kernel */
  int32_t num_items;      /* capacity of items, in work items */
  int32_t variant_start[8]; /* host: first work item of each kernel variant */
  int32_t variant_count[8]; /* host: work items of each kernel variant */
  /* tensor-core blocked sweep (pysa_gb_tc_setup); tc_enabled = 0 disables */
  uint16_t *tc_b;           /* BF16 J tiles (hi[, lo]) in MMA operand order */
  int64_t tc_b_elems;
  float *tc_diag;           /* FP32 64x64 diagonal blocks of J */
  int64_t tc_diag_elems;
  int32_t *tc_items;        /* [tc_num_items, 8] work list (128/F chains) */
  int32_t tc_num_items;
  int32_t tc_terms;         /* 1: J exact in BF16, 2: J = J_hi + J_lo */
  int32_t tc_enabled;       /* 1: sequential sweeps use the tensor cores */
  int32_t tc_variant_start[3]; /* host: items of fold F = 1, 2, 4 */
  int32_t tc_variant_count[3];
  int32_t tc_min_n;         /* instances with tc_min_n <= n <= 2048 take the
                               tensor-core sweep, the others the plain kernel
                               in the same sweep (0 means 64) */
  int32_t *tc_inst;         /* [num_instances] device flags written by
                               pysa_gb_tc_setup: 1 = tensor-core instance */
  int32_t plain_live;       /* host, from pysa_gb_tc_setup: bit v set when
                               plain variant v still has instances */
  int32_t tc_fusable;       /* host, from pysa_gb_tc_setup: 1 when every
                               tensor-core instance's R divides its chains
                               per CTA (exchange can run inside the kernel) */
  int32_t *tc_sched;        /* [2 + tc_num_items] device scratch of the
                               persistent tensor-core kernel */
  int32_t tc_unit_sweeps;   /* sweeps per work unit of that kernel (0: 8) */
  int32_t tc_launch_sweeps; /* most sweeps one launch of it covers (0: 128) */
  /* random visiting order on the tensor cores: J tiles and diagonal blocks
   * repacked in each sweep's order, tc_rand_slots sweeps at a time (0: random
   * sweeps run on the plain kernel); needs perm_slots >= tc_rand_slots */
  uint16_t *tc_b_rand;      /* [tc_rand_slots, tc_b_elems] */
  float *tc_diag_rand;      /* [tc_rand_slots, tc_diag_elems] */
  int64_t *tc_inst_off;     /* [2 * num_instances] device, written by
                               pysa_gb_tc_setup when not NULL: offsets of each
                               instance's tiles and diagonal blocks, -1 for
                               plain-kernel instances */
  int32_t tc_rand_slots;
  /* host, from pysa_gb_setup: work items of the sparse-row sweep (one per
   * csr_chains chains of each sparse instance) within items */
  int32_t csr_item_start;
  int32_t csr_item_count;
  /* caller: 0 = the sparse tables are grouped rows (csr_rows); 4, 8, 16 or
   * 32 = every sparse row is a fixed record of that many entries at
   * csr_ent_off + width * i (csr_rows unused): the row's entries in the
   * same group order, bit 31 of csr_col set on the last entry of each
   * group, padding entries with value 0 */
  int32_t csr_width;
  int32_t csr_chains;     /* host, from pysa_gb_setup: chains per work item
                             (128, or 64 / 32 while that leaves SMs idle) */
  /* host, from pysa_gb_setup: work items of the wide-instance sweep (dense
   * instances with n > 4096: fields in this workspace's fields array, J
   * read in place, so j_off and ld of those instances must be multiples
   * of 4 and J 16-byte aligned) within items, 8 chains each */
  int32_t wide_item_start;
  int32_t wide_item_count;
  /* caller: chains per tensor-core work item (0: automatic -- a CTA's full
   * tensor memory, 128 / F chains, halved while the batch would leave SMs
   * idle); otherwise the largest multiple of each instance's granule (R
   * when R divides 128 / F, else 32) not above min(this, 128 / F).  Read
   * by pysa_gb_tc_setup; pysa_gb_tc_workspace sizes for the smallest
   * items any value can give. */
  int32_t tc_item_chains;
  /* host, from pysa_gb_tc_setup: bit v set when every work item of fold
   * variant v (F = 1, 2, 4) belongs to an instance of the same n.  Fused
   * launches of such a variant, with tc_unit_sweeps = 0, split the launch's
   * item-sweeps evenly over the CTAs (wrap-around units) instead of running
   * fixed-length units from a queue. */
  int32_t tc_uniform;
  /* caller, read by pysa_gb_tc_setup: 1 = the tensor-core tiles in FP8 E4M3
   * (half the bytes and MMA instructions of BF16; results identical).  Only
   * valid when every tensor-core instance's couplings are exact in E4M3
   * (integers up to 16 in magnitude, for instance) and tc_terms = 1; random
   * visiting order keeps BF16 tiles. */
  int32_t tc_fp8;
} pysa_gb_workspace;

/* Host copies of the per-instance tables, used to plan the work list. */
typedef struct {
  const int32_t *n;
  const int32_t *replicas;
  const int32_t *reads;
  const int64_t *chain_off;
  const int64_t *j_off;
  const int32_t *ld;
  const int32_t *sparse;  /* [num_instances] 1: the instance sweeps on the
                             sparse-row kernel (pysa_gb_problems.csr_*);
                             NULL: none does */
} pysa_gb_host_tables;

typedef struct {
  uint64_t seed;           /* key of the Philox stream */
  int32_t update;          /* PYSA_GB_SEQUENTIAL or PYSA_GB_RANDOM */
  int32_t use_pt;          /* 1: replica exchange after every sweep */
  int32_t log_omega_stride;/* 0: off; else row stride of state.log_omega */
  int32_t best_global;     /* 0: per-replica best (simulation_parallel);
                              1: energies start at +inf best (sequential) */
  int32_t phases;          /* 0 = all; bit 0: visiting order + sweep kernel,
                              bit 1: exchange (lets a caller time each) */
  int32_t recompute_every; /* tensor-core sweep: rebuild fields and energies
                              from the spins at the start of every sweep whose
                              index is a multiple of this (0 = never) */
  int32_t exchange_every;  /* 0 or 1: replica exchange after every sweep, as
                              pysa/simulation.py:167-168 does; k > 1: only
                              after sweeps s with (s + 1) % k == 0 (an opt-in
                              tuning knob with no counterpart in the
                              reference; log-omega is still taken every
                              sweep) */
  int32_t pad_;
} pysa_gb_options;

/* ABI version (PYSA_GB_ABI_VERSION) and the last error of this thread. */
int pysa_gb_abi_version(void);
const char *pysa_gb_last_error(void);

/* Diagnostics: when `device_buffer` (>= 24 x 64 uint64) is not NULL, the
 * tensor-core sweep records a per-block timeline (SM clock cycles) of its first CTA
 * there: [0] decision start, [1] fields ready, [2] decisions done, [3] A free,
 * [4] A published, [5] MMA start, [6] next-block fields committed, [7] stages
 * issued, [8 + 3g .. 10 + 3g] sub-block g: fields loaded, lazy corrections
 * applied, decided.  NULL turns it off.  Recorded only by builds with
 * PYSA_GB_TRACE defined (PYSA_GB_TRACE=1 in the environment of the build
 * script).  No counterpart in the reference. */
int pysa_gb_set_trace(void *device_buffer);

/* Diagnostics: bound, in nanoseconds, of the tensor-core sweep's wait for a
 * work item's previous unit (0 restores the default of one second).  A
 * unit waits only at its start, with nothing in flight, so a tiny bound
 * makes a run end cleanly with PYSA_GB_ERR_TIMEOUT in the status word: the
 * way tests exercise the timeout path.  Applies to launches enqueued after
 * the call, process-wide.  No counterpart in the reference. */
int pysa_gb_set_unit_wait_limit(uint64_t ns);

/* Decision mode of the tensor-core sweep's 64-spin blocks: 0 (default)
 * chooses per block -- rounds over the whole block while the previous
 * block's largest flip count of a chain was small, sequential 16-spin
 * sub-blocks otherwise; 1 always rounds; 2 always sub-blocks.  Every mode
 * makes the same decisions (the rule of pysa/ising.py:40-63 and
 * pysa/qubo.py:40-63 in the visiting order); only the speed differs, and
 * tests pin both forms.  Applies to launches enqueued after the call,
 * process-wide.  No counterpart in the reference. */
int pysa_gb_set_decision_mode(int32_t mode);

/* Decision mode 0's switch point: a block is decided in rounds while the
 * previous block's largest flip count of a chain was at most `flips`
 * (0..64, default 12), in sequential sub-blocks otherwise.  Same decisions
 * for every value; process-wide, for launches enqueued after the call.  No
 * counterpart in the reference. */
int pysa_gb_set_block_round_limit(int32_t flips);

/* Most CTAs of a tensor-core sweep launch (0, the default: one per SM).
 * Results do not depend on it; a smaller value leaves SMs to other work and
 * lets tests split few work items over fewer CTAs.  Process-wide, for
 * launches enqueued after the call.  No counterpart in the reference. */
int pysa_gb_set_tc_max_ctas(int32_t ctas);

/* The tensor-core sweep's wrap-around schedule, as the kernel computes it
 * (host copy of the same code, for tests and tools): piece `piece` of share
 * `share` when `ctas` CTAs split `items` work items x `sweeps` sweeps of a
 * launch (ctas <= items).  Returns 1 and out = {item, first sweep, sweeps},
 * 0 past the share's last piece, or an error.  No counterpart in the
 * reference. */
int pysa_gb_tc_wrap_piece(int32_t items, int32_t sweeps, int32_t ctas,
                          int32_t share, int32_t piece, int32_t out[3]);

/* Workspace sizing and set-up.
 *   pysa_gb_workspace_bytes: sizes of the workspace arrays for a batch
 *     described by host tables (n, replicas, reads are read); returns the
 *     number of work items (>= 0) or an error.  out[0] packed_j elements,
 *     out[1] items int32 entries, out[2] minimum field_ld.
 *   pysa_gb_setup: packs J into the sweep kernel's row layout and writes the
 *     work list; fills ws->variant_start / variant_count. */
int pysa_gb_workspace_bytes(int32_t num_instances,
                            const pysa_gb_host_tables *host, int64_t out[3]);
int pysa_gb_setup(const pysa_gb_problems *p, const pysa_gb_host_tables *host,
                  pysa_gb_workspace *ws, void *stream);

/* Tensor-core blocked sweep (sequential order, 64 <= n <= 2048): sizes of
 * tc_b, tc_diag and tc_items (int32 entries) for `terms` BF16 terms over the
 * instances with min_n <= n <= 2048 (min_n < 64 means 64), and the set-up
 * that packs them (instances selected by ws->tc_min_n; the others stay on
 * the plain kernel, which skips the tensor-core instances in sequential
 * sweeps).  Returns the number of tc work items. */
int pysa_gb_tc_workspace(int32_t num_instances,
                         const pysa_gb_host_tables *host, int32_t terms,
                         int32_t min_n, int64_t out[3]);
int pysa_gb_tc_setup(const pysa_gb_problems *p,
                     const pysa_gb_host_tables *host, pysa_gb_workspace *ws,
                     void *stream);

/* Local fields H = J s + h for every chain, accumulated in f64 from f32
 * products, and (if set_energies) energies E = s.(J s / 2 + h)
 * (pysa/ising.py:32-37, pysa/qubo.py:32-37).  Also sets chain_beta from
 * beta_idx and, if init_best, best_* from the current state
 * (best_global: best_energy = +inf). */
int pysa_gb_prepare(const pysa_gb_problems *p, pysa_gb_state *s,
                    pysa_gb_workspace *ws, int32_t set_energies,
                    int32_t init_best, int32_t best_global, void *stream);

/* num_sweeps Metropolis sweeps, each followed by the replica exchange
 * (pysa/utils.py:44-58) and, when enabled, the log-omega of the sorted ladder
 * (pysa/ais.py:79-112).  Replaces the loop of simulation_parallel
 * (pysa/simulation.py:150-171).  Sweep indices come from
 * state.sweep_counter, so the same enqueued work can be replayed by a CUDA
 * graph. */
int pysa_gb_sweeps(const pysa_gb_problems *p, pysa_gb_state *s,
                   pysa_gb_workspace *ws, const pysa_gb_options *o,
                   int32_t num_sweeps, void *stream);

/* Allocation-free form of pysa_gb_prepare + pysa_gb_sweeps on the plain
 * CUDA-core kernel.  No counterpart in the reference: it exists for callers
 * that cannot allocate device memory themselves (a plugin inside a host
 * application whose device memory is owned by the host's pool, a loop that
 * cannot afford cudaMalloc's implicit synchronisation, C code without a
 * device allocator).  The caller passes only inputs and outputs; the local
 * fields, visiting orders, packed couplings and work list live in one
 * library-owned device array of 64 MiB, held on every GPU that loads the
 * library until the process exits.  Batches needing more scratch are
 * rejected with PYSA_GB_ERR_SIZE.  `init` = 1 computes energies from the
 * spins and resets best_*; 0 continues from the caller's energies and best_*.
 * Fields are rebuilt from the spins on every call.  All calls share the
 * array: calls that overlap on the GPU race.  The first call on each device
 * resolves the array's address and should come before any stream capture;
 * the address stays cached, so after cudaDeviceReset the entry point must
 * not be called again on that device.  Dense couplings only: a batch with a
 * sparse-row instance (host->sparse) is rejected with PYSA_GB_ERR_ARG, one
 * with more than 4096 spins in an instance with PYSA_GB_ERR_SIZE, before
 * anything is enqueued.  Sequential and random order; never the
 * tensor-core kernel. */
int pysa_gb_sweeps_noalloc(const pysa_gb_problems *p, pysa_gb_state *s,
                           const pysa_gb_host_tables *host,
                           const pysa_gb_options *o, int32_t init,
                           int32_t num_sweeps, void *stream);

/* Energies in f64 of `count` bit-packed states of instance `inst`
 * (get_energy, pysa/ising.py:32-37) with f64 couplings J64 (n x ld64). */
int pysa_gb_energy64(int32_t problem_type, int32_t n, int32_t ld64,
                     const double *J64, const double *h64,
                     const uint32_t *spins, int32_t words, int64_t count,
                     double *out, void *stream);

/* The same f64 energies with the couplings and fields of instance inst of
 * the problem tables (f32, J stored transposed, values taken exactly). */
int pysa_gb_energy64_tables(const pysa_gb_problems *p,
                            const pysa_gb_host_tables *host, int32_t inst,
                            const uint32_t *spins, int32_t words,
                            int64_t count, double *out, void *stream);

/* Unpack bit-packed spins into float32 values (+-1 or 0/1), [count, n]. */
int pysa_gb_unpack(int32_t problem_type, int32_t n, const uint32_t *spins,
                   int32_t words, int64_t count, float *out, int32_t out_ld,
                   void *stream);

/* Pack float32 states on the device ([count, x_ld], +-1 or 0/1; the bit is
 * x > 0 for Ising, x != 0 for QUBO) into bit-packed words [count, words]:
 * the device-side form of the initial states handed to
 * simulation_parallel (pysa/sa.py:303-313). */
int pysa_gb_pack(int32_t problem_type, int32_t n, const float *x,
                 int32_t x_ld, int64_t count, uint32_t *spins, int32_t words,
                 void *stream);

/* Replace instance inst's couplings and local fields (writes p->J and p->h,
 * which must be writable device memory) from a dense symmetric problem
 * matrix P in device memory (n x n, row stride p_ld), split as
 * Solver.__init__ does (pysa/sa.py:66-69): couplings = P with a zero
 * diagonal, fields = diag(P).  The caller then re-runs pysa_gb_setup (and
 * pysa_gb_tc_setup) so the sweep kernels' copies of J follow. */
int pysa_gb_load_problem(const pysa_gb_problems *p,
                         const pysa_gb_host_tables *host, int32_t inst,
                         const float *P, int32_t p_ld, void *stream);

/* Annealed importance sampling (Solver.annealed_importance, pysa/sa.py:432-553;
 * ais_sample, pysa/simulation.py:293-317; update_spin_ref,
 * pysa/ising.py:66-92).  Every instance of the batch (one replica each; its
 * reads are its samples) anneals in one launch on the same temperature
 * schedule; state.spins holds the initial samples [chains, words],
 * state.energies their energies and ws.fields their local fields (from
 * pysa_gb_prepare, with the couplings already scaled by the target beta).
 * Writes final samples, energies and the f64 log weights [chains].  Random
 * order needs ws.perm_slots >= num_temps.  An instance with more than one
 * replica sets PYSA_GB_ERR_ARG in the status word. */
typedef struct {
  uint64_t seed;
  int32_t update;     /* PYSA_GB_SEQUENTIAL or PYSA_GB_RANDOM */
  int32_t reference;  /* 0 uniform (pysa/ais.py:137-169),
                         1 bernoulli (pysa/ais.py:175-226) */
  int32_t order;      /* 0: weight after each sweep (pysa/simulation.py:305-316);
                         1: weight before each sweep (standard AIS) */
  int32_t num_temps;
  double p;           /* bernoulli: probability of bit 0 / spin -1 */
  int32_t max_samples;/* largest reads of an instance (0: num_chains) */
  int32_t pad_;
} pysa_gb_ais_options;

int pysa_gb_ais(const pysa_gb_problems *p, pysa_gb_state *s,
                pysa_gb_workspace *ws, const pysa_gb_ais_options *o,
                const float *temps, double *log_w, void *stream);

/* Exact log Z(beta) = log sum_s exp(-beta E(s)) of every instance by
 * enumeration of all 2^n states in f64 (n <= 34).  part_max / part_sum are
 * caller buffers of pysa_gb_logz_parts(...) doubles each; the host combines
 * them: logZ = M + log(sum_b part_sum[b] exp(part_max[b] - M)). */
int64_t pysa_gb_logz_parts(int32_t num_instances, int32_t max_n);
int pysa_gb_logz_exact(const pysa_gb_problems *p, double beta,
                       double *part_max, double *part_sum, void *stream);

/* ------------------------------------------------------------------------
 * Learned flip proposal.  No counterpart in the reference: these entry
 * points add a Metropolis-Hastings move for the coldest replica of every
 * read, proposed by a per-instance MLP  nn -> hidden -> nn  (ReLU hidden
 * layer, one Bernoulli flip logit per spin) that is trained online on pairs
 * of cold states.  Weights are FP32 masters with BF16 copies for the tensor
 * cores; GEMMs accumulate in FP32.  Every array is device memory, stacked
 * over instances with the sizes given beside it (I = num_instances,
 * B = batch, H = hidden).  nn % 256 == 0, hidden % 256 == 0,
 * batch % 128 == 0, nn >= max_n of the problems.
 * ---------------------------------------------------------------------- */
typedef struct {
  int32_t num_instances, n, hidden, batch;
  float *w1, *b1, *w2, *b2;          /* [I][H][nn], [I][H], [I][nn][H], [I][nn] */
  float *m1, *v1, *mb1, *vb1;        /* Adam moments of w1, b1 */
  float *m2, *v2, *mb2, *vb2;        /* Adam moments of w2, b2 */
  float *dw1, *db1, *dw2, *db2;      /* gradients, shapes of w1, b1, w2, b2 */
  uint16_t *w1_p, *w2_p, *w2t_p;     /* BF16 tiles of w1, w2, w2^T [I][H*nn] */
  float *x, *a1, *z2, *dz2, *da1;    /* [I][B][nn], [I][B][H], [I][B][nn] x2,
                                        [I][B][H] */
  uint16_t *pa, *pb;                 /* operand tiles [I][B*max(nn,H)] each */
  float *loss;                       /* [I] mean BCE of the last backward */
  int32_t *status;                   /* bounded-wait status word */
} pysa_gb_mlp;

/* Per-proposal scratch: flip masks, delta = s' - s and J delta [I][B][nn];
 * log q forward / reverse and accepted dE [I][B]. */
typedef struct {
  float *flip, *delta, *jd;
  float *logq_fwd, *logq_rev, *de;
} pysa_gb_proposal_scratch;

/* BF16 copies of w1, w2 and w2^T after the masters changed. */
int pysa_gb_mlp_sync_weights(const pysa_gb_mlp *m, void *stream);
/* z2 = W2 relu(W1 x + b1) + b2 for the B rows of x of every instance. */
int pysa_gb_mlp_forward(const pysa_gb_mlp *m, void *stream);
/* Gradients of the row-weighted mean (weights [I][B]) of the per-row sum of
 * binary cross-entropies between sigmoid(z2) and target [I][B][nn]; uses
 * the activations of the last forward.  loss[i] = that mean. */
int pysa_gb_mlp_backward(const pysa_gb_mlp *m, const float *target,
                         const float *row_weight, void *stream);
/* One Adam step (Kingma & Ba 2015) on every parameter; step >= 1 is the
 * bias-correction count.  Refreshes the BF16 copies. */
int pysa_gb_mlp_adam(const pysa_gb_mlp *m, float lr, float beta1, float beta2,
                     float eps, int32_t step, void *stream);
/* Training pairs from two snapshots [I][B][words]: x = snapshot a as spin
 * values, target = (a != b) per spin. */
int pysa_gb_mlp_pairs(const pysa_gb_mlp *m, int32_t problem_type,
                      const int32_t *n_inst, const uint32_t *snap_a,
                      const uint32_t *snap_b, int32_t words, float *target,
                      void *stream);
/* rows[i][r] = chain holding the largest beta of read r of instance i
 * (first on ties), -1 for r >= reads[i] or when enabled[i] == 0 (enabled
 * may be NULL: all instances). */
int pysa_gb_cold_rows(const pysa_gb_problems *p, const pysa_gb_state *s,
                      const int32_t *enabled, int32_t batch, int32_t *rows,
                      void *stream);
/* out[i][r][:] = spins of chain rows[i][r] (zeros for -1). */
int pysa_gb_snapshot(const pysa_gb_problems *p, const pysa_gb_state *s,
                     const int32_t *rows, int32_t batch, uint32_t *out,
                     void *stream);
/* BF16 copies of the couplings as the B operand of J delta:
 * out[i][t] (t < terms) = tile(J_field^T), J_field[j][k] = change of field j
 * per unit change of spin k; terms = 2 adds the residual J - bf16(J). */
int64_t pysa_gb_proposal_j_elems(int32_t num_instances, int32_t nn,
                                 int32_t terms);
int pysa_gb_pack_proposal_j(const pysa_gb_problems *p,
                            const pysa_gb_host_tables *host, int32_t nn,
                            int32_t terms, uint16_t *out, void *stream);
/* One proposal for every row: s' from the flip mask sampled from
 * sigmoid(z2(s) + c(s)) with uniforms of stream (PROPOSAL, inst, round,
 * chain, j); c(s) = 0 when target_flips <= 0, else the shift that makes the
 * expected number of flips target_flips (same rule for the reverse pass);
 * accept iff log u < -beta dE + log q(s|s') - log q(s'|s) (u from index
 * 0xFFFFFFFF of the same stream), dE = delta.(H + J delta / 2) in f32.
 * Accepted rows get new spins, fields, energies and best_* (best_sweep =
 * sweep_counter - 1).  accepted[i] += accepted rows of instance i. */
int pysa_gb_propose(const pysa_gb_problems *p, pysa_gb_state *s,
                    pysa_gb_workspace *ws, const pysa_gb_mlp *m,
                    const int32_t *rows, const uint16_t *j_packed,
                    int32_t terms, const pysa_gb_proposal_scratch *sc,
                    uint64_t seed, uint32_t round, float target_flips,
                    int32_t *accepted, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PYSA_GB_H */

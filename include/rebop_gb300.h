/*
 * rebop_gb300.h -- C ABI of the GB300 ensemble engine for rebop's run-time
 * Gillespie direct method.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns an
 * int status (RB_OK = 0) and never aborts: where the reference panics or
 * raises, this library returns RB_ERR_INVALID and keeps a message that
 * rb_last_error() copies out (per calling thread).  Host buffers stay owned
 * by the caller; device buffers, streams and the per-device tables belong to
 * the library unless a *_device entry point is used, in which case the
 * caller owns the device buffers and the stream.
 *
 * Arithmetic contract: species counts are int64 (the reference's isize),
 * propensities, their running sums and the clock are IEEE binary64 evaluated
 * in the reference's order, and the random stream is the reference's
 * generator stack (xoshiro256++ seeded by SplitMix64, a 256-layer ziggurat for
 * Exp1, 53-bit uniforms), one stream per trajectory seed.  A trajectory run
 * with seed s therefore follows the reference's
 * `Gillespie::new_with_seed(x0, sparse, s)` event for event.
 *
 * Citations are to files of the rebop v0.9.7 source tree.
 */
#ifndef REBOP_GB300_H
#define REBOP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define RB_OK 0
#define RB_ERR_INVALID 1     /* bad argument: the reference's assert!/ValueError */
#define RB_ERR_CUDA 2        /* a CUDA runtime call failed (message has details) */
#define RB_ERR_NOMEM 3       /* host or device allocation failed */
#define RB_ERR_PARSE 4       /* define_system! text not understood */
#define RB_ERR_UNSUPPORTED 5 /* network shape outside every kernel's range */
#define RB_ERR_TIMEOUT 6     /* a kernel ran out of its wall-clock budget
                              * (RB_KERNEL_BUDGET_S seconds, default 120);
                              * results of that call are incomplete */

/* Library version string ("<major>.<minor>.<patch>"). */
const char *rb_version(void);

/* Copy the calling thread's last error message into buf (always
 * NUL-terminated when len > 0).  Returns the message length. */
size_t rb_last_error(char *buf, size_t len);

/* Per-call statistics, filled when a non-NULL pointer is passed. */
typedef struct {
    uint64_t events;       /* accepted reaction events, all trajectories    */
    double kernel_ms;      /* device time of the simulation kernel(s)       */
    double total_ms;       /* wall time of the whole call                   */
    uint64_t h2d_bytes;    /* host->device bytes copied by the call         */
    uint64_t d2h_bytes;    /* device->host bytes copied by the call         */
    int32_t kernel_launches;
    int32_t mapping;       /* kernel that ran: 0 generic thread-per-trajectory,
                            * 2 lockstep exact, 3 speculative float-pair,
                            * 4 speculative generated for the network (NVRTC),
                            * 5 warp per trajectory, 6 batch graph,
                            * 7 thread unit of a batch's persistent launch */
    uint64_t exact_reruns; /* sample intervals the speculative kernel re-ran
                            * exactly because a decision fell inside its
                            * error margin */
} rb_run_stats;

/* ------------------------------------------------- reaction network -----
 * A network is the packed reaction descriptor every kernel reads.  It is
 * built the way the reference builds a Gillespie's reaction list
 * (src/gillespie.rs:225-244): each reaction is a mass-action rate and a
 * vector of species differences. */
typedef struct rb_network rb_network;

/* Empty network over n_species species.  Replaces the species-count part of
 * Gillespie::new (src/gillespie.rs:168-176). */
int rb_network_create(int32_t n_species, rb_network **out);
void rb_network_destroy(rb_network *net);
int32_t rb_network_nb_species(const rb_network *net);   /* gillespie.rs:199-201 */
int32_t rb_network_nb_reactions(const rb_network *net); /* gillespie.rs:209-211 */

/* add_reaction(Rate::lma(rate, exponents), differences):
 * src/gillespie.rs:24-26 and :225-244.  n_exponents and n_differences must
 * both equal the species count (the reference's assert_eq!). */
int rb_network_add_reaction_lma(rb_network *net, double rate, const uint32_t *exponents,
                                int32_t n_exponents, const int64_t *differences,
                                int32_t n_differences);

/* add_reaction(Rate::lma_sparse(rate, pairs), differences):
 * src/gillespie.rs:29-31 and :225-244.  The (species, exponent) pairs are
 * multiplied in the order given, as Rate::rate's sparse arm does
 * (gillespie.rs:79-86); an index out of range is RB_ERR_INVALID (the
 * reference's issue-85 assert, gillespie.rs:229-233 and :496-502). */
int rb_network_add_reaction_lma_sparse(rb_network *net, double rate, const uint32_t *species,
                                       const uint32_t *exponents, int32_t n_pairs,
                                       const int64_t *differences, int32_t n_differences);

/* add_reaction(Rate::expr(expr), differences): src/gillespie.rs:33-35, :88
 * and :225-244; the expression tree of src/expr.rs:8-21 in postfix form.
 * Each code word is op | argument << 8 with op
 *   0 push constant consts[argument]   1 push species count [argument] as f64
 *   2 negate   3 add   4 subtract   5 multiply   6 divide   7 powf
 *   8 max   9 min   10 exp
 * (binary operations pop y then x and push x op y).  The propensity is the
 * program's value, evaluated in binary64 as Expr::eval does (expr.rs:23-39).
 * A malformed program, an index out of range or a stack deeper than 16 is
 * RB_ERR_INVALID.  Networks with such reactions run on the generic exact
 * kernel; the no-allocation entry point refuses them (RB_ERR_UNSUPPORTED). */
int rb_network_add_reaction_expr(rb_network *net, const int32_t *code, int32_t n_code,
                                 const double *consts, int32_t n_consts, const int64_t *differences,
                                 int32_t n_differences);

/* Lower a define_system! body (src/gillespie_macro.rs:50-58):
 *     p1 p2 ...;  Name { A, B, ... }  rname: [k] A + ... => [k] B + ... @ rate ...
 * `rate` is a parameter name or a numeric literal.  Parameters start as NaN,
 * as the macro's `new()` leaves them (gillespie_macro.rs:71-78); set them with
 * rb_network_set_param.  The network keeps the macro's arithmetic: integer
 * falling factorials per reactant term in written order, and the
 * first-match choice chain (gillespie_macro.rs:106, :133-171). */
int rb_network_from_dsl(const char *text, rb_network **out);
int rb_network_set_param(rb_network *net, const char *name, double value);
int32_t rb_network_nb_params(const rb_network *net);
int rb_network_param_name(const rb_network *net, int32_t idx, char *buf, size_t len);
int rb_network_species_name(const rb_network *net, int32_t idx, char *buf, size_t len);
int rb_network_name(const rb_network *net, char *buf, size_t len);
/* Rate constant of reaction r (after parameter substitution). */
int rb_network_reaction_rate(const rb_network *net, int32_t r, double *rate);

/* ---------------------------------------------------- ensemble runs -----
 * The batched entry point: n_traj independent trajectories of one network,
 * each the reference's Python-API run (src/pyo3_gillespie.rs:168-208) with its
 * own seed: t starts at 0, and for i = 0..nb_steps the trajectory is
 * advanced to tmax*i/nb_steps (gillespie.rs:315-344) and the saved species
 * are recorded.
 *
 *   x0        [S] shared initial counts, or [n_traj][S] when x0_per_traj
 *   rates     NULL: the network's rate constants; else [R] or
 *             [n_traj][R] (rates_per_traj) per-trajectory rate constants
 *   seeds     [n_traj] one u64 seed per trajectory
 *   save_idx  [n_save] species to record (NULL with n_save < 0: all)
 *   out       [nb_steps+1][n_save][n_traj] recorded counts
 *   times     [nb_steps+1] sample times, may be NULL
 *   events    [n_traj] accepted events per trajectory, may be NULL
 *   final_species [n_traj][S], may be NULL
 *
 * rb_ensemble_run takes host buffers and does the copies itself (page-locked
 * out/events buffers may be written by the kernel in place, over the host
 * link, when the network's previous run wrote its samples slowly; the call
 * returns only once every result is in place either way);
 * rb_ensemble_run_device takes device buffers and a cudaStream_t (NULL:
 * the legacy default stream) and returns once the work is enqueued. */
int rb_ensemble_run(const rb_network *net, int64_t n_traj, const int64_t *x0, int32_t x0_per_traj,
                    const double *rates, int32_t rates_per_traj, const uint64_t *seeds, double tmax,
                    int64_t nb_steps, const int32_t *save_idx, int32_t n_save, int64_t *out,
                    double *times, uint64_t *events, int64_t *final_species, rb_run_stats *stats);

int rb_ensemble_run_device(const rb_network *net, int64_t n_traj, const int64_t *d_x0,
                           int32_t x0_per_traj, const double *d_rates, int32_t rates_per_traj,
                           const uint64_t *d_seeds, double tmax, int64_t nb_steps,
                           const int32_t *save_idx, int32_t n_save, int64_t *d_out,
                           uint64_t *d_events, int64_t *d_final_species, void *stream);

/* rb_ensemble_run_device for callers that cannot let a library allocate device
 * memory -- hosts whose own pool allocator owns all GPU memory, or
 * latency-critical callers that cannot take cudaMalloc's implicit device
 * synchronisation.  No counterpart in the reference, which runs on the CPU and
 * never allocates device memory.
 *
 * The call allocates nothing: the engine's own device data (counters, Exp1
 * tables, packed descriptor, sample times, saved list) goes into one fixed
 * 64 KiB array compiled into the library, which every GPU that loads the
 * library keeps until the process exits.  A network and sampling grid that
 * do not fit return RB_ERR_INVALID with the needed size in the message.
 * The first call on a device looks up that array's device address (with the
 * device current); make that first call before any stream capture.  The address
 * is kept for the life of the process, so it is stale after a cudaDeviceReset of
 * that device.  The call's own data reaches the array as launch parameters of
 * small staging kernels, so no host buffer is read after the call returns.  Arguments
 * are those of rb_ensemble_run_device (device buffers, host save_idx), plus
 * d_status: NULL or a device pointer to 2 uint64 receiving the run's event
 * total and its time-budget flag (1 = ran out, results incomplete).  Work is
 * enqueued on `stream` and the call returns.  All calls share the one array
 * and each rewrites it, so calls whose work overlaps on the GPU (e.g. on two
 * streams) race; issue them on one stream or wait between them. */
int rb_ensemble_run_device_noalloc(const rb_network *net, int64_t n_traj, const int64_t *d_x0,
                                   int32_t x0_per_traj, const double *d_rates,
                                   int32_t rates_per_traj, const uint64_t *d_seeds, double tmax,
                                   int64_t nb_steps, const int32_t *save_idx, int32_t n_save,
                                   int64_t *d_out, uint64_t *d_events, uint64_t *d_status,
                                   void *stream);

/* Sum of accepted events of the last rb_ensemble_run_device on this network
 * (synchronises with that run's stream); RB_ERR_TIMEOUT if that run ran out
 * of its time budget. */
int rb_ensemble_last_events(const rb_network *net, uint64_t *events);

/* ------------------------------------------------------------ autotuner ---
 * No counterpart in the reference, which has one CPU code path.  The kernels
 * that can run an ensemble map it differently (a kernel generated for the
 * network, the speculative kernel over the packed descriptor, the lockstep
 * exact kernel -- a thread per trajectory -- or a warp per trajectory), and
 * the fastest, with its block size, phase length and slot scheduler, depends
 * on the network and the ensemble.  rb_ensemble_tune times pilot runs of this
 * workload (the arguments of rb_ensemble_run, internal seeds) for every
 * kernel that covers it, then the launch shapes of the fastest, and keeps the
 * winner for networks of the same shape (species, reactions, reactant
 * orders, macro arithmetic, log2 of the trajectory count, per-trajectory
 * rates) on this GPU, in memory and in a cache file ($RB_TUNE_CACHE, default
 * $HOME/.cache/rebop_gb300/tune_cache.txt).  Later runs of such networks use
 * it (RB_TUNE=0: never).  Results are the same bit for bit whichever kernel
 * runs. */
typedef struct {
    int32_t mapping;      /* rb_run_stats.mapping code of the kernel */
    int32_t block;        /* lanes per block of the generated kernel (0: 384) */
    int32_t phase_steps;  /* steps per phase of the speculative kernels (0: 128) */
    int32_t sched;        /* their slot scheduler: 0 lagging clocks first, 1 rotation, -1 default */
    double ms;            /* pilot run time (best of two); < 0: the shape failed */
} rb_tune_result;
/* best: the winner; trials[0 .. min(max_trials, *n_trials)): every shape timed. */
int rb_ensemble_tune(const rb_network *net, int64_t n_traj, const int64_t *x0, int32_t x0_per_traj,
                     const double *rates, int32_t rates_per_traj, double tmax, int64_t nb_steps,
                     rb_tune_result *best, rb_tune_result *trials, int32_t max_trials, int32_t *n_trials);
/* The remembered shape for this network and ensemble size on the current GPU
 * (RB_ERR_INVALID: none). */
int rb_tune_lookup(const rb_network *net, int64_t n_traj, int32_t rates_per_traj, rb_tune_result *out);
/* Path of the cache file (length returned; copied NUL-terminated into buf). */
size_t rb_tune_cache_path(char *buf, size_t len);
/* Forget the tuned shapes held in memory (the next lookup reads the cache file
 * again), and delete the cache file when remove_file. */
void rb_tune_clear(int32_t remove_file);

/* Every-event run of one trajectory, src/pyo3_gillespie.rs:209-223: records
 * (t, saved species) at t = 0 and after each reaction while t < tmax; the
 * last record is the first event at or after tmax, or t = +inf when the
 * total propensity vanishes (gillespie.rs:275-297).  Writes at most `cap`
 * records and returns their full number in *n_records. */
int rb_run_all_events(const rb_network *net, const int64_t *x0, uint64_t seed, double tmax,
                      const int32_t *save_idx, int32_t n_save, double *times, int64_t *out,
                      int64_t cap, int64_t *n_records);

/* One trajectory whose state the caller keeps: species[S], *t and the
 * 4-word generator state are read and updated in place by one GPU
 * advance_until(tmax).  The define_system! struct's advance_until
 * (src/gillespie_macro.rs:98-126) maps here, as does any checkpoint/resume. */
int rb_trajectory_advance_until(const rb_network *net, int64_t *species, double *t, uint64_t *rng_state,
                                double tmax);
/* The generator state SmallRng::seed_from_u64(seed) starts from
 * (src/gillespie.rs:184; gillespie_macro.rs:81-84). */
void rb_rng_state_from_seed(uint64_t seed, uint64_t *state);

/* ------------------------------------------------ heterogeneous batch ---
 * No counterpart in the reference, which runs one network and one parameter
 * set per call.  A batch holds many ensembles -- different networks, rate
 * constants, initial counts, horizons, trajectory counts -- and runs them all
 * with one CUDA graph around one persistent launch: its warps take work from
 * one queue, a trajectory of a large network (a warp per trajectory, items
 * with the most estimated work first) or a thread unit -- 32 trajectories of
 * a network of at most 16 species and 16 reactions, one per lane, with the
 * exact per-lane step.  Items with rate expressions, define_system! items
 * whose arithmetic differs from the launch's and per-trajectory rates on
 * networks too large for a thread unit run as launches of their own in the
 * same graph.  (RB_BATCH_MODE=merged: ensembles of one network structure and
 * sample grid merge into one thread-per-trajectory launch instead.)  Every
 * result equals what rb_ensemble_run gives for the same item, bit for bit. */
typedef struct rb_batch rb_batch;
int rb_batch_create(rb_batch **out);
void rb_batch_destroy(rb_batch *b);
/* Add one ensemble.  Arguments mean what they mean for rb_ensemble_run; the
 * host buffers (x0, rates, seeds, save_idx, out, events) are kept by pointer
 * and must outlive the batch: every rb_batch_run reads the inputs' current
 * contents and writes the outputs.  out may be null: the results then stay
 * with the batch (rb_batch_item_results), with no copy into caller memory.
 * A network must not change after it is added (RB_ERR_INVALID at run time). */
int rb_batch_add(rb_batch *b, const rb_network *net, int64_t n_traj, const int64_t *x0, int32_t x0_per_traj,
                 const double *rates, int32_t rates_per_traj, const uint64_t *seeds, double tmax,
                 int64_t nb_steps, const int32_t *save_idx, int32_t n_save, int64_t *out, uint64_t *events);
/* Run every ensemble.  The first run plans, uploads the tables and captures
 * the graph; later runs replay it.  stats->kernel_ms is the graph's device
 * time (copies included), stats->kernel_launches its kernel count. */
int rb_batch_run(rb_batch *b, rb_run_stats *stats);
/* The plan (no GPU needed): launches of their own, and items of the
 * persistent launch; and the kernel an item runs on (rb_run_stats.mapping
 * codes: 5 warp per trajectory and 7 thread unit in the persistent launch;
 * 4 for a merged class until the first run confirms whether the generated
 * kernel compiled). */
int rb_batch_plan(rb_batch *b, int32_t *n_own_launches, int32_t *n_persistent_items);
int rb_batch_item_mapping(const rb_batch *b, int32_t item, int32_t *mapping);
/* After a run: where item's results lie -- out [nb_steps + 1][n_save][n_traj]
 * and events [n_traj] -- in the batch's page-locked staging buffer (items of
 * the persistent launch: no copy at all), in the batch's own copy (items of a
 * merged class added without an output buffer), or in the caller's buffers
 * given to rb_batch_add.  Valid until the next rb_batch_run, rb_batch_add or
 * rb_batch_destroy; RB_ERR_INVALID before the first run.  (No reference
 * counterpart.) */
int rb_batch_item_results(const rb_batch *b, int32_t item, const int64_t **out, const uint64_t **events);

/* ------------------------------------------ stateful single trajectory ---
 * The Rust API's `Gillespie` object (src/gillespie.rs:157-344) with the same
 * methods; every advance runs on the GPU. */
typedef struct rb_gillespie rb_gillespie;

/* Gillespie::new (gillespie.rs:168-176): seed drawn from OS entropy. */
int rb_gillespie_new(const int64_t *species, int32_t n_species, int32_t sparse, rb_gillespie **out);
/* Gillespie::new_with_seed (gillespie.rs:179-187). */
int rb_gillespie_new_with_seed(const int64_t *species, int32_t n_species, int32_t sparse,
                               uint64_t seed, rb_gillespie **out);
void rb_gillespie_free(rb_gillespie *g);
int rb_gillespie_seed(rb_gillespie *g, uint64_t seed);         /* gillespie.rs:189-191 */
int32_t rb_gillespie_nb_species(const rb_gillespie *g);        /* gillespie.rs:199-201 */
int32_t rb_gillespie_nb_reactions(const rb_gillespie *g);      /* gillespie.rs:209-211 */
int rb_gillespie_add_reaction_lma(rb_gillespie *g, double rate, const uint32_t *exponents,
                                  int32_t n_exponents, const int64_t *differences,
                                  int32_t n_differences);      /* gillespie.rs:225-244 */
int rb_gillespie_add_reaction_lma_sparse(rb_gillespie *g, double rate, const uint32_t *species,
                                         const uint32_t *exponents, int32_t n_pairs,
                                         const int64_t *differences, int32_t n_differences);
int rb_gillespie_add_reaction_expr(rb_gillespie *g, const int32_t *code, int32_t n_code,
                                   const double *consts, int32_t n_consts, const int64_t *differences,
                                   int32_t n_differences);     /* Rate::expr, as above */
double rb_gillespie_get_time(const rb_gillespie *g);           /* gillespie.rs:246-248 */
void rb_gillespie_set_time(rb_gillespie *g, double t);         /* gillespie.rs:250-252 */
int rb_gillespie_get_species(const rb_gillespie *g, int32_t s, int64_t *value); /* :260-262 */
int rb_gillespie_set_species(rb_gillespie *g, const int64_t *species, int32_t n); /* :264-267 */
int rb_gillespie_advance_until(rb_gillespie *g, double tmax);  /* gillespie.rs:315-344 */
int rb_gillespie_advance_one_reaction(rb_gillespie *g);        /* gillespie.rs:269-272 */

#ifdef __cplusplus
}
#endif
#endif /* REBOP_GB300_H */

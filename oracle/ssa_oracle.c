/*
 * ssa_oracle.c -- CPU restatement of rebop's run-time Gillespie path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm load it.
 * The product (rebop_gb300/) never links, imports or calls it.
 *
 * What it restates (paths are within the rebop v0.9.7 source tree):
 *   - Rate::rate LMA fold ................ src/gillespie.rs:71-90
 *   - Jump::affect ....................... src/gillespie.rs:142-152
 *   - add_reaction shape checks .......... src/gillespie.rs:225-244
 *   - _advance_one_reaction .............. src/gillespie.rs:275-297
 *   - advance_until ...................... src/gillespie.rs:315-344
 *   - make_cumrates ...................... src/gillespie.rs:357-364
 *   - choose_cumrate_sum ................. src/gillespie.rs:402-407
 *   - sampling loop (nb_steps > 0) ....... src/pyo3_gillespie.rs:200-208
 *   - every-event loop (nb_steps == 0) ... src/pyo3_gillespie.rs:209-223
 *   - define_system! arithmetic .......... src/gillespie_macro.rs:106-120,133-171
 *
 * The random stream is the reference's third-party generator stack, which is
 * not vendored in the reference tree; each piece below restates the published
 * algorithm of the pinned crate version (Cargo.lock):
 *   - rand 0.10.2 `SmallRng` on 64-bit targets = xoshiro256++
 *     (Blackman & Vigna, "Scrambled linear pseudorandom number generators",
 *     2018/2021), seeded by `seed_from_u64` = four SplitMix64 outputs
 *     (Steele, Lea & Flood 2014).  Call sites: gillespie.rs:173,184,190.
 *   - rand 0.10.2 `StandardUniform` for f64: the top 53 bits of next_u64()
 *     times 2^-53, i.e. a multiple of 2^-53 in [0, 1).  Call sites:
 *     gillespie.rs:286,332.
 *   - rand_distr 0.6.0 `Exp1`: 256-layer ziggurat (Marsaglia & Tsang 2000)
 *     with the ZIGNOR table construction of Doornik (2005); layer index from
 *     the low 8 bits of one next_u64(), the layer abscissa u in (0,1) from its
 *     top 52 bits, the tail sampled as R - ln(U).  Call sites:
 *     gillespie.rs:285,327; gillespie_macro.rs:114.
 * Parity pin: with numpy's seed derivation (python/rebop/gillespie.py:139-140)
 * this stack reproduces the reference's only fixed-seed golden,
 * tests/test_rebop.py:30-36 (SIR, rng=42 -> S,I,R = 0,227,773).
 *
 * Build with -ffp-contract=off: the reference never fuses a*b+c, and the
 * ziggurat's rejection test must round like it.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* RNG: xoshiro256++ / SplitMix64 / 53-bit uniform / ziggurat Exp1          */
/* ------------------------------------------------------------------------ */

typedef struct { uint64_t s[4]; } orc_rng;

static inline uint64_t orc_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

/* seed_from_u64: four SplitMix64 outputs fill the 256-bit state. */
void orc_rng_seed(orc_rng *g, uint64_t seed) {
    uint64_t st = seed;
    for (int i = 0; i < 4; i++) {
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        g->s[i] = z ^ (z >> 31);
    }
}

uint64_t orc_next_u64(orc_rng *g) {
    uint64_t *s = g->s;
    uint64_t out = orc_rotl(s[0] + s[3], 23) + s[0];
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = orc_rotl(s[3], 45);
    return out;
}

double orc_uniform(orc_rng *g) { return (double)(orc_next_u64(g) >> 11) * 0x1.0p-53; }

/* ZIGNOR tables for the unit exponential, 256 layers. */
#define ORC_ZIG_R 7.69711747013104972
#define ORC_ZIG_V 0.0039496598225815571993
static double ZX[257], ZF[257];
static pthread_once_t zig_once = PTHREAD_ONCE_INIT;

static void zig_init(void) {
    ZX[0] = ORC_ZIG_V / exp(-ORC_ZIG_R);
    ZX[1] = ORC_ZIG_R;
    for (int i = 2; i < 256; i++) ZX[i] = -log(ORC_ZIG_V / ZX[i - 1] + exp(-ZX[i - 1]));
    ZX[256] = 0.0;
    for (int i = 0; i < 257; i++) ZF[i] = exp(-ZX[i]);
}

void orc_zig_tables(double *x_out, double *f_out) {
    pthread_once(&zig_once, zig_init);
    memcpy(x_out, ZX, sizeof ZX);
    memcpy(f_out, ZF, sizeof ZF);
}

double orc_exp1(orc_rng *g) {
    for (;;) {
        uint64_t bits = orc_next_u64(g);
        int i = (int)(bits & 0xff);
        uint64_t ubits = (bits >> 12) | 0x3FF0000000000000ull; /* [1, 2) */
        double one_two;
        memcpy(&one_two, &ubits, 8);
        double u = one_two - (1.0 - 0x1.0p-53); /* (0, 1) */
        double x = u * ZX[i];
        if (x < ZX[i + 1]) return x;
        if (i == 0) return ORC_ZIG_R - log(orc_uniform(g));
        if (ZF[i + 1] + (ZF[i] - ZF[i + 1]) * orc_uniform(g) < exp(-x)) return x;
    }
}

/* ------------------------------------------------------------------------ */
/* Reaction network, as the reference stores it                              */
/* ------------------------------------------------------------------------ */

/* One reaction: a Rate (dense LMA vector, or sparse (index, exponent) list)
 * and a Jump (dense difference vector, or its non-zero entries).
 * gillespie.rs:12-19 and :95-100. */
typedef struct {
    int32_t n_species;
    int32_t n_reactions;
    const double *rate;        /* [R] rate constants                              */
    const int32_t *rate_kind;  /* [R] 0 = Rate::LMA (dense), 1 = Rate::LMASparse,
                                  2 = Rate::Expr                                  */
    const uint32_t *lma;       /* [R*S] dense exponents (kind 0)                  */
    const int32_t *sp_off;     /* [R+1] offsets into sp_idx/sp_exp (kind 1)       */
    const uint32_t *sp_idx;
    const uint32_t *sp_exp;
    const int64_t *jump;       /* [R*S] dense differences                         */
    int32_t macro_mode;        /* 1 = define_system! arithmetic (see rate_macro)  */
    const int32_t *mfac_off;   /* macro mode: [R+1] offsets of (species, order)   */
    const uint32_t *mfac_idx;  /*   factors in the order written in the reaction  */
    const uint32_t *mfac_ord;
    const int32_t *ex_off;     /* kind 2: [R+1] offsets into ex_code              */
    const int32_t *ex_code;    /*   postfix program: op | argument << 8           */
    const double *ex_const;    /*   constants the program pushes                  */
} orc_net;

/* Postfix form of an Expr tree (expr.rs:8-21): each word is op | arg << 8. */
enum { EX_CONST = 0, EX_SPECIES, EX_NEG, EX_ADD, EX_SUB, EX_MUL, EX_DIV, EX_POW, EX_MAX, EX_MIN, EX_EXP };
#define EX_MAX_DEPTH 64

/* Expr::eval, expr.rs:23-39: species counts as f64, IEEE operations, powf
 * and exp from the C library, max/min returning the non-NaN operand. */
static double expr_eval(const orc_net *net, int r, const int64_t *sp) {
    double st[EX_MAX_DEPTH];
    int top = 0;
    for (int k = net->ex_off[r]; k < net->ex_off[r + 1]; k++) {
        const int32_t w = net->ex_code[k];
        const int op = w & 0xff, arg = w >> 8;
        if (op == EX_CONST) {
            st[top++] = net->ex_const[arg];
        } else if (op == EX_SPECIES) {
            st[top++] = (double)sp[arg];
        } else if (op == EX_NEG) {
            st[top - 1] = -st[top - 1];
        } else if (op == EX_EXP) {
            st[top - 1] = exp(st[top - 1]);
        } else {
            const double b = st[--top], a = st[top - 1];
            double v;
            switch (op) {
            case EX_ADD: v = a + b; break;
            case EX_SUB: v = a - b; break;
            case EX_MUL: v = a * b; break;
            case EX_DIV: v = a / b; break;
            case EX_POW: v = pow(a, b); break;
            case EX_MAX: v = fmax(a, b); break;
            default: v = fmin(a, b); break;
            }
            st[top - 1] = v;
        }
    }
    return st[0];
}

/* Rate::rate for LMA, gillespie.rs:71-87: a fold over species in index order,
 * multiplying the running product by each factor of n(n-1)...(n-e+1) taken
 * from the lowest factor up, each converted to f64 on its own. */
static double rate_lma(const orc_net *net, const double *rates, int r, const int64_t *sp) {
    if (net->rate_kind[r] == 2) return expr_eval(net, r, sp);  /* gillespie.rs:88 */
    double acc = rates[r];
    if (net->rate_kind[r] == 0) {
        const uint32_t *e = net->lma + (size_t)r * net->n_species;
        for (int s = 0; s < net->n_species; s++) {
            int64_t n = sp[s];
            for (int64_t x = n + 1 - (int64_t)e[s]; x <= n; x++) acc *= (double)x;
        }
    } else {
        for (int p = net->sp_off[r]; p < net->sp_off[r + 1]; p++) {
            int64_t n = sp[net->sp_idx[p]];
            for (int64_t x = n + 1 - (int64_t)net->sp_exp[p]; x <= n; x++) acc *= (double)x;
        }
    }
    return acc;
}

/* define_system! propensity, gillespie_macro.rs:106 and :133-146: the rate
 * parameter times, for each reactant in the order written, the integer
 * falling factorial n(n-1)...(n-k+1) computed in isize and cast once. */
static double rate_macro(const orc_net *net, const double *rates, int r, const int64_t *sp) {
    if (net->rate_kind[r] == 2) return expr_eval(net, r, sp);
    double acc = rates[r];
    for (int p = net->mfac_off[r]; p < net->mfac_off[r + 1]; p++) {
        int64_t n = sp[net->mfac_idx[p]];
        int64_t ff = n;
        for (int64_t i = 1; i < (int64_t)net->mfac_ord[p]; i++) ff *= n - i;
        acc *= (double)ff;
    }
    return acc;
}

/* make_cumrates, gillespie.rs:357-364. */
static double make_cumrates(const orc_net *net, const double *rates, const int64_t *sp, double *cum) {
    double total = 0.0;
    for (int r = 0; r < net->n_reactions; r++) {
        double a = net->macro_mode ? rate_macro(net, rates, r, sp) : rate_lma(net, rates, r, sp);
        cum[r] = total + a;
        total = cum[r];
    }
    return total;
}

/* choose_cumrate_sum, gillespie.rs:402-407: the number of cumulative rates
 * strictly below the chosen value, over all reactions. */
static int choose_cumrate_sum(const orc_net *net, double chosen, const double *cum) {
    int n = 0;
    for (int r = 0; r < net->n_reactions; r++) n += (cum[r] < chosen) ? 1 : 0;
    return n;
}

/* define_system! choice chain, gillespie_macro.rs:150-171: the first
 * reaction k with chosen < carry_k + a_k, none if no such k. */
static int choose_macro(const orc_net *net, double chosen, const double *cum) {
    for (int r = 0; r < net->n_reactions; r++)
        if (chosen < cum[r]) return r;
    return net->n_reactions;
}

/* Jump::affect, gillespie.rs:142-152 (dense form; the sparse form adds the
 * same non-zero entries). */
static void affect(const orc_net *net, int r, int64_t *sp) {
    if (r >= net->n_reactions) return;
    const int64_t *d = net->jump + (size_t)r * net->n_species;
    for (int s = 0; s < net->n_species; s++) sp[s] += d[s];
}

/* Trajectory state: Gillespie { species, t, rng } (gillespie.rs:157-163). */
typedef struct {
    int64_t *species;
    double t;
    orc_rng rng;
} orc_state;

/* advance_until, gillespie.rs:315-344 (API) or gillespie_macro.rs:98-126
 * (macro mode: the same loop with the macro's propensity and choice). */
static int64_t advance_until(const orc_net *net, const double *rates, orc_state *st, double tmax,
                             double *cum, int32_t *log_r, double *log_t, int64_t log_cap,
                             int64_t *log_n) {
    int64_t events = 0;
    for (;;) {
        double total = make_cumrates(net, rates, st->species, cum);
        if (!(0.0 < total)) {
            st->t = tmax;
            return events;
        }
        st->t += orc_exp1(&st->rng) / total;
        if (st->t > tmax) {
            st->t = tmax;
            return events;
        }
        double chosen = total * orc_uniform(&st->rng);
        int r = net->macro_mode ? choose_macro(net, chosen, cum) : choose_cumrate_sum(net, chosen, cum);
        affect(net, r, st->species);
        if (log_n && *log_n < log_cap) {
            log_r[*log_n] = r;
            log_t[*log_n] = st->t;
        }
        if (log_n) (*log_n)++;
        events++;
    }
}

/* _advance_one_reaction, gillespie.rs:275-297: one event, no horizon;
 * a non-positive (or NaN) total sends the clock to +inf. */
static int advance_one(const orc_net *net, const double *rates, orc_state *st, double *cum) {
    double total = make_cumrates(net, rates, st->species, cum);
    if (!(0.0 < total)) {
        st->t = INFINITY;
        return 0;
    }
    st->t += orc_exp1(&st->rng) / total;
    double chosen = total * orc_uniform(&st->rng);
    int r = choose_cumrate_sum(net, chosen, cum);
    affect(net, r, st->species);
    return 1;
}

/* ------------------------------------------------------------------------ */
/* Exported entry points (ctypes)                                           */
/* ------------------------------------------------------------------------ */

/* Validation mirrors add_reaction's asserts (gillespie.rs:227-237): sparse
 * indices in range; the reference panics, the oracle returns -1. */
int orc_validate(const orc_net *net) {
    if (net->n_species < 0 || net->n_reactions < 0) return -1;
    for (int r = 0; r < net->n_reactions; r++) {
        if (net->rate_kind[r] == 1) {
            for (int p = net->sp_off[r]; p < net->sp_off[r + 1]; p++)
                if ((int64_t)net->sp_idx[p] >= net->n_species) return -1;
        }
        if (net->macro_mode) {
            for (int p = net->mfac_off[r]; p < net->mfac_off[r + 1]; p++)
                if ((int64_t)net->mfac_idx[p] >= net->n_species) return -1;
        }
        if (net->rate_kind[r] == 2) {
            /* a well-formed postfix program leaves exactly one value */
            int depth = 0;
            for (int k = net->ex_off[r]; k < net->ex_off[r + 1]; k++) {
                const int op = net->ex_code[k] & 0xff, arg = net->ex_code[k] >> 8;
                if (op == EX_SPECIES && (arg < 0 || arg >= net->n_species)) return -1;
                if (op > EX_EXP) return -1;
                depth += (op <= EX_SPECIES) ? 1 : (op == EX_NEG || op == EX_EXP) ? 0 : -1;
                if (depth < 1 || depth > EX_MAX_DEPTH) return -1;
            }
            if (depth != 1) return -1;
        }
    }
    return 0;
}

/* Rate::rate of one reaction at a given state (the rate_lma known-answer
 * test, gillespie.rs:448-472, calls this). */
double orc_rate(const orc_net *net, int r, const int64_t *species) {
    return net->macro_mode ? rate_macro(net, net->rate, r, species) : rate_lma(net, net->rate, r, species);
}

/* Jump::affect of one reaction (jump_affect test, gillespie.rs:484-494). */
void orc_affect(const orc_net *net, int r, int64_t *species) { affect(net, r, species); }

/* One stateful trajectory, as Gillespie::advance_until.  `state_rng` is the
 * 4-word xoshiro state (in/out); `species` in/out; returns the events. */
int64_t orc_advance_until(const orc_net *net, int64_t *species, double *t, uint64_t *state_rng,
                          double tmax, int32_t *log_r, double *log_t, int64_t log_cap, int64_t *log_n) {
    pthread_once(&zig_once, zig_init);
    double *cum = (double *)malloc(sizeof(double) * (net->n_reactions ? net->n_reactions : 1));
    orc_state st;
    st.species = species;
    st.t = *t;
    memcpy(st.rng.s, state_rng, 32);
    int64_t ev = advance_until(net, net->rate, &st, tmax, cum, log_r, log_t, log_cap, log_n);
    *t = st.t;
    memcpy(state_rng, st.rng.s, 32);
    free(cum);
    return ev;
}

void orc_seed_state(uint64_t seed, uint64_t *state_rng) {
    orc_rng g;
    orc_rng_seed(&g, seed);
    memcpy(state_rng, g.s, 32);
}

/* Draw helpers for RNG known-answer tests. */
void orc_draw_u64(uint64_t seed, uint64_t *out, int64_t n) {
    orc_rng g;
    orc_rng_seed(&g, seed);
    for (int64_t i = 0; i < n; i++) out[i] = orc_next_u64(&g);
}
void orc_draw_exp1(uint64_t seed, double *out, int64_t n) {
    pthread_once(&zig_once, zig_init);
    orc_rng g;
    orc_rng_seed(&g, seed);
    for (int64_t i = 0; i < n; i++) out[i] = orc_exp1(&g);
}

/* The regular-sampling run of one trajectory, pyo3_gillespie.rs:200-208:
 * sample i at t = tmax * i / nb_steps (left to right in f64).  Writes
 * out[i * out_stride_sample + k * out_stride_save] for saved species k. */
static int64_t run_sampled(const orc_net *net, const double *rates, orc_state *st, double tmax,
                           int64_t nb_steps, const int32_t *save_idx, int32_t n_save, int64_t *out,
                           int64_t stride_sample, int64_t stride_save, double *cum) {
    int64_t events = 0;
    for (int64_t i = 0; i <= nb_steps; i++) {
        double t = tmax * (double)i / (double)nb_steps;
        events += advance_until(net, rates, st, t, cum, NULL, NULL, 0, NULL);
        for (int k = 0; k < n_save; k++)
            out[i * stride_sample + k * stride_save] = st->species[save_idx[k]];
    }
    return events;
}

typedef struct {
    const orc_net *net;
    const double *rates;       /* [R] or [n_traj][R] */
    int64_t rates_stride;      /* 0 or R             */
    const int64_t *x0;
    int64_t x0_stride;         /* 0 or S             */
    const uint64_t *seeds;
    int64_t n_traj;
    double tmax;
    int64_t nb_steps;
    const int32_t *save_idx;
    int32_t n_save;
    int64_t *out;              /* [nb_steps+1][n_save][n_traj] */
    int64_t *final_species;    /* [n_traj][S] or NULL           */
    uint64_t *events;          /* [n_traj] or NULL              */
    int64_t next;              /* shared work counter           */
    int64_t chunk;             /* trajectories per work item    */
    int64_t total_events;
    pthread_mutex_t lock;
} ens_job;

static void *ens_worker(void *arg) {
    ens_job *job = (ens_job *)arg;
    const orc_net *net = job->net;
    int S = net->n_species;
    double *cum = (double *)malloc(sizeof(double) * (net->n_reactions ? net->n_reactions : 1));
    int64_t *sp = (int64_t *)malloc(sizeof(int64_t) * (S ? S : 1));
    int64_t local_events = 0;
    for (;;) {
        int64_t begin = __atomic_fetch_add(&job->next, job->chunk, __ATOMIC_RELAXED);
        if (begin >= job->n_traj) break;
        int64_t end = begin + job->chunk < job->n_traj ? begin + job->chunk : job->n_traj;
        for (int64_t j = begin; j < end; j++) {
            orc_state st;
            st.species = sp;
            memcpy(sp, job->x0 + j * job->x0_stride, sizeof(int64_t) * S);
            st.t = 0.0;
            orc_rng_seed(&st.rng, job->seeds[j]);
            const double *rates = job->rates + j * job->rates_stride;
            int64_t ev = run_sampled(net, rates, &st, job->tmax, job->nb_steps, job->save_idx, job->n_save,
                                     job->out + j, (int64_t)job->n_save * job->n_traj, job->n_traj, cum);
            if (job->events) job->events[j] = (uint64_t)ev;
            if (job->final_species) memcpy(job->final_species + j * S, sp, sizeof(int64_t) * S);
            local_events += ev;
        }
    }
    pthread_mutex_lock(&job->lock);
    job->total_events += local_events;
    pthread_mutex_unlock(&job->lock);
    free(cum);
    free(sp);
    return NULL;
}

/* An ensemble of independent trajectories, each exactly the reference's
 * `Gillespie::new_with_seed(x0, sparse, seeds[j])` followed by the
 * sampling loop -- the reference runs such ensembles as a serial loop
 * (examples/sir.rs:13-21, benchmarks/benches/vilar/vilar.rs:28-51); the
 * oracle spreads them over `n_threads` host threads.  Returns the total
 * number of reaction events, or -1 on invalid input. */
int64_t orc_run_ensemble(const orc_net *net, const double *rates, int64_t rates_stride, const int64_t *x0,
                         int64_t x0_stride, const uint64_t *seeds, int64_t n_traj, double tmax,
                         int64_t nb_steps, const int32_t *save_idx, int32_t n_save, int64_t *out,
                         int64_t *final_species, uint64_t *events, int32_t n_threads) {
    if (orc_validate(net) != 0 || nb_steps <= 0) return -1;
    pthread_once(&zig_once, zig_init);
    ens_job job;
    job.net = net;
    job.rates = rates ? rates : net->rate;
    job.rates_stride = rates ? rates_stride : 0;
    job.x0 = x0;
    job.x0_stride = x0_stride;
    job.seeds = seeds;
    job.n_traj = n_traj;
    job.tmax = tmax;
    job.nb_steps = nb_steps;
    job.save_idx = save_idx;
    job.n_save = n_save;
    job.out = out;
    job.final_species = final_species;
    job.events = events;
    job.next = 0;
    job.total_events = 0;
    pthread_mutex_init(&job.lock, NULL);
    if (n_threads < 1) n_threads = 1;
    /* up to 64 trajectories per work item, but at least four items per thread */
    job.chunk = n_traj / (4 * (int64_t)n_threads);
    if (job.chunk > 64) job.chunk = 64;
    if (job.chunk < 1) job.chunk = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * n_threads);
    for (int i = 0; i < n_threads; i++) pthread_create(&th[i], NULL, ens_worker, &job);
    for (int i = 0; i < n_threads; i++) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&job.lock);
    return job.total_events;
}

/* Every-event run of one trajectory, pyo3_gillespie.rs:209-223: record
 * (t, species) at t = 0 and after each _advance_one_reaction while t < tmax.
 * Returns the number of records (which may exceed `cap`; only the first
 * `cap` are written). */
int64_t orc_run_all_events(const orc_net *net, const int64_t *x0, uint64_t seed, double tmax,
                           const int32_t *save_idx, int32_t n_save, double *times, int64_t *out,
                           int64_t cap) {
    if (orc_validate(net) != 0) return -1;
    pthread_once(&zig_once, zig_init);
    int S = net->n_species;
    double *cum = (double *)malloc(sizeof(double) * (net->n_reactions ? net->n_reactions : 1));
    int64_t *sp = (int64_t *)malloc(sizeof(int64_t) * (S ? S : 1));
    memcpy(sp, x0, sizeof(int64_t) * S);
    orc_state st;
    st.species = sp;
    st.t = 0.0;
    orc_rng_seed(&st.rng, seed);
    int64_t n = 0;
    for (;;) {
        if (n < cap) {
            times[n] = st.t;
            for (int k = 0; k < n_save; k++) out[n * n_save + k] = sp[save_idx[k]];
        }
        n++;
        if (!(st.t < tmax)) break;
        advance_one(net, net->rate, &st, cum);
    }
    free(cum);
    free(sp);
    return n;
}

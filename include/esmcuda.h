/*
 * esmcuda.h -- C ABI of libesmcuda.so, the GB300 (sm_103a) replica-sampler hot path.
 *
 * The reference (a Julia package) has no FFI on this path; the seam this library replaces is
 * the body of the replica step `replica_step!` (src/replicas.jl:676-707) and `init_replicas`
 * (src/replicas.jl:785), i.e. the per-replica operation sweeps, the capacity scores, the
 * replica-averaged Langevin capacity step with dispatch following, and the weather process.
 * The host keeps the run loop, the gate, the weights and the probe bookkeeping
 * (src/replicas.jl:841-1000 run_replicas), as the reference's GPU port does
 * (device/src/replica_run.jl:309 replica_device_step!).
 *
 * Conventions
 *  - Every entry point returns an int status: ESM_OK (0) or a negative ESM_E* code; the
 *    message of the last failure of a context is `esm_last_error(ctx)`. Nothing aborts or traps.
 *  - Host arrays are caller-owned and copied at call time. Device buffers are owned by the
 *    context and freed by esm_destroy.
 *  - State arrays are (X, T, R) with the replica index fastest: element (x, t, r) at
 *    (x*T + t)*R + r. X is N (angles), D (dispatchable units), S (storage units) or n0 (weather
 *    series). This is the layout of the reference port's DeviceState (device/src/core.jl).
 *  - One context per host thread; one CUDA stream per context.
 *  - Random numbers: counter-based Philox4x32-10 streams keyed by the context seed and a tag per
 *    stream; the exact stream layout (tags and counter words) is part of the contract, so that a
 *    CPU restatement of the algorithm can replay every draw.
 */
#ifndef ESMCUDA_H
#define ESMCUDA_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ESM_OK = 0,
    ESM_EINVAL = -1,      /* bad argument or model */
    ESM_ECUDA = -2,       /* CUDA runtime error */
    ESM_ENOMEM = -3,      /* device allocation failed */
    ESM_ETIMEOUT = -4,    /* a bounded device wait ran out */
    ESM_ESTATE = -5       /* call out of order (e.g. no state uploaded) */
};

/* unit kinds of the flat capacity vector */
enum { ESM_UNIT_REN = 0, ESM_UNIT_DISP = 1, ESM_UNIT_STOR = 2 };
/* v-field roles (src/local.jl:36) */
enum { ESM_ROLE_THETA = 1, ESM_ROLE_GEN = 3, ESM_ROLE_SE = 6 };
/* the plain local families (src/local.jl:1912 plain_families), in this order, then the two
   compensated transport families of the flow design that need no flow basis (flow_families,
   src/flowmoves.jl:333, rate 0.1 each there; 0 in the plain sweep): TPOT (prep_tpot!,
   src/local.jl:1741, one node angle with the dispatch at the ends of its lines following pro
   rata) and TSOC (prep_tsoc!, :1849, one unit's state of charge with the dispatch at its node
   following pro rata at tau - 1 and tau) */
enum { ESM_FAM_UNIT = 0, ESM_FAM_PAIR, ESM_FAM_XPAIR, ESM_FAM_XLOCC, ESM_FAM_XLOC, ESM_FAM_POTENTIAL,
       ESM_FAM_CELLPAIR, ESM_FAM_CELL, ESM_FAM_SPAIR, ESM_FAM_TPOT, ESM_FAM_TSOC, ESM_NFAM };

/*
 * Static model: network, units, prices, weather prior and the move tables.
 * Reference: EnergyModel (src/energy.jl:219), LocalModel (src/local.jl:193), WeatherModel
 * (src/weather.jl:22). Index arrays are 0-based.
 */
typedef struct esm_model {
    int32_t N, L, T;            /* nodes, lines, steps of the year */
    double dt;                  /* step length (h) */
    /* lines: flow b (theta_a - theta_b), hard limit s (src/energy.jl:590) */
    const int32_t *bus0, *bus1;
    const double *line_b, *line_s;
    /* capacity units, flat; kind ESM_UNIT_* */
    int32_t K;
    const int32_t *unit_kind, *unit_group, *unit_bus, *unit_series;
    const double *unit_mc, *unit_capex, *unit_lo, *unit_hi, *unit_avail;
    const double *unit_hours, *unit_eta_in, *unit_eta_out, *unit_qt;
    int32_t D, S;               /* dispatchable and storage units */
    const int32_t *disp, *stor; /* their flat capacity indices */
    /* weather: n0 series (load per node, then availability series), single-level
       regime-switching VAR(1) with diagonal coefficients (src/weather.jl:22) */
    int32_t n0, nreg;
    const int32_t *series_field; /* 0 = load, > 0 availability */
    const int32_t *series_node;
    const double *xbar;          /* [n0*T] climatology */
    const double *wscale;        /* [n0] */
    const double *Ptr, *pi0;     /* [nreg*nreg], [nreg] */
    const double *phi;           /* [nreg*n0] diagonal AR coefficient */
    const double *mu;            /* [nreg*n0*3] harmonic regime mean (1, cos, sin) */
    const double *sig;           /* [nreg*n0] innovation sd */
    const double *sig0;          /* [n0] sd of the first step */
    /* prices and temperatures (src/run.jl:14-16,54-55; src/energy.jl:279) */
    double c_shed, c_dump, c_viol, gamma_k, kappa0, beta_v, beta_k;
    int32_t physical;            /* reference measure "physical" (src/energy.jl:811) */
    /* v fields: theta, g per dispatchable carrier, se per storage carrier; atoms are the
       node-space columns of their graph-Haar bases (src/spatial.jl:112) */
    int32_t nfields;
    const int32_t *field_role;   /* [nfields] ESM_ROLE_* */
    const int32_t *field_atom_ptr; /* [nfields+1] -> atoms */
    const int32_t *atom_ptr;     /* [natoms+1] -> entries */
    const int32_t *atom_idx;     /* node (theta) or index into disp/stor */
    const double *atom_val;
    /* incidence and unit lists (src/local.jl:248-285) */
    const int32_t *nodelines_ptr, *nodelines;
    const int32_t *units_ptr, *units_at;   /* dispatchable units per node (index into disp) */
    const int32_t *stor_ptr, *stor_at;     /* storage units per node (index into stor) */
    /* cell moves (src/local.jl:265-283) */
    int32_t nlev;
    const double *qcum;                    /* [nlev] cumulative level probabilities */
    const int32_t *cell_level_ptr;         /* [nlev+1] -> cells */
    const int32_t *cell_ptr, *cell_units;  /* cells -> dispatchable units */
    /* xloc templates (src/local.jl:122 xloc_directions), per node and partner */
    const int32_t *xpart_ptr, *xpart;
    const int32_t *xnod_ptr, *xnod;        /* per pair: re-routing angle changes */
    const double *xval;
    const int32_t *xlk_ptr, *xlkn;         /* per pair: leak nodes and requirement change */
    const double *xlkg;
    /* global re-routing (src/local.jl:44 GridSolver): column n of the grounded inverse */
    const double *reroute;                 /* [N*N], element (i, n) at i*N + n */
    const int32_t *comp;                   /* AC component per node */
    /* storage multiscale sweep (src/flowmoves.jl:255 storage_ms_sweep!): the storage units grouped
       by (cell of their node in the country partition, carrier) -- the cell-class aggregates of its
       plateau moves -- as CSR over indices into stor */
    int32_t nsgroups;
    const int32_t *sgroup_ptr, *sgroup_units;
} esm_model;

/* Sampler options (src/run.jl:20 local_extra; src/local.jl:1294 maxnats; ReplicaCtl defaults
   src/replicas.jl:484-519). */
typedef struct esm_opts {
    int32_t R;                 /* replicas per chain */
    int32_t precision;         /* 32: FP32 evaluations (production), 64: FP64 (parity) */
    uint64_t seed;
    double extra;              /* random moves per node, step and sweep (4.0) */
    double maxnats;            /* walk stop (40.0) */
    double kappa_min;          /* move validity and reflection floor (1.0) */
    int32_t max_points;        /* walk points per direction; beyond: t = 0, counted (guard); 0: automatic,
                                  esm_auto_max_points of the largest state-of-charge atom */
    int32_t span;              /* class steps sharing one move list (0: max(1, 32/R)) */
    double family_rates[ESM_NFAM];
    int32_t storage_ms;        /* 1: an operation sweep runs, after the local sweep, the storage multiscale
                                  sweep with probability 1/2 (operation_sweep!, src/local.jl:2417);
                                  0: the local sweep only */
    int32_t storage_long;      /* 1: then the long-range storage sweep (storage_long_sweep!,
                                  src/storage_long.jl:245; probability 1, the default of src/run.jl:27) */
    int32_t probe;             /* 1: create the one-replica context of esm_lag_probe (its streams are
                                  keyed by esm_probe_seed(seed)) */
} esm_opts;

/* The seed of the lag probe's streams (the reference's separate probe stream, src/replicas.jl:873). */
static inline uint64_t esm_probe_seed(uint64_t seed) { return seed ^ 0x50524F4245000000ull; }

/* The automatic point cap: 192, or 4 points per unit of the largest state-of-charge atom when that
   is more (measured guard rates: 0 at 40 nodes with 192; 0.06 % at 256 nodes with 1024). */
static inline int32_t esm_auto_max_points(int32_t max_storage_atom_units) {
    int32_t p = 4 * max_storage_atom_units;
    return p > 192 ? p : 192;
}

typedef struct esm_ctx esm_ctx;

/* Create a context: uploads the model, allocates the state for R replicas. */
int esm_create(const esm_model *model, const esm_opts *opts, esm_ctx **out);
int esm_destroy(esm_ctx *ctx);
const char *esm_last_error(const esm_ctx *ctx);

/* Upload / download the state (host arrays in double, layouts as above):
   theta [N*T*R], g [D*T*R], e [S*T*R], z [n0*T*R] (weather anomaly), reg [T*R], k [K]
   (capacities shared by the replicas; State in src/hierarchy.jl:28). Any pointer may be NULL
   to skip that array on download. */
int esm_upload_state(esm_ctx *ctx, const double *theta, const double *g, const double *e,
                     const double *z, const int32_t *reg, const double *k);
int esm_download_state(esm_ctx *ctx, double *theta, double *g, double *e, double *z,
                       int32_t *reg, double *k);

/* Caches (residual r [N*T*R], flows F [L*T*R]) rebuilt from the state; as LocalCost
   (src/local.jl:313, rebuild_step! :332). */
int esm_rebuild_caches(esm_ctx *ctx);
int esm_download_caches(esm_ctx *ctx, double *r, double *F);

/* `n` operation sweeps of every replica: local_sweep! (src/local.jl:1927) with the plain
   families; sweep counters start at `sweep0` (the Philox counter of the sweep). stats (may be
   NULL): [ESM_NFAM+1][2] moves tried / moved per family (last row: atoms) and, at index
   2*(ESM_NFAM+1), the number of guard events (walk beyond max_points). */
int esm_operation_sweeps(esm_ctx *ctx, int32_t n, int64_t sweep0, int64_t *stats);

/* One colour class of one sweep (parity tests): class cls (0: even 0-based steps, 1: odd, 2: the
   last step of an odd year); only the first move_limit entries of every move list when > 0. */
int esm_class_pass(esm_ctx *ctx, int64_t sweep, int32_t cls, int32_t move_limit, int64_t *stats);

/* The storage multiscale sweep of sweep `sweep` (storage_ms_sweep!, src/flowmoves.jl:255) in its
   plateau form: for the dyadic lengths 2 .. 128 below T/2 (random order, random offset), blocks of
   one parity at a time, 8 moves per block, each raising the state of charge of one storage unit or
   of a cell-class aggregate (esm_model.sgroup_*) over the block's instants with pro-rata
   compensation at its end steps and the Jacobian test. It runs with probability 1/2 per sweep
   (operation_sweep!, src/local.jl:2417) unless force is set; esm_operation_sweeps calls it after
   the local sweep when esm_opts.storage_ms is 1. max_passes > 0 runs only the first class passes
   of the sweep (a diagnostic, as move_limit of esm_class_pass). stats (may be NULL) += (moves
   tried, moves taken, guard events). */
int esm_storage_ms(esm_ctx *ctx, int64_t sweep, int32_t force, int32_t max_passes, int64_t *stats);

/* The long-range storage sweep of sweep `sweep` (storage_long_sweep!, src/storage_long.jl:245): for
   every storage unit with at least 24 h of storage and kappa_s >= kappa_min, the level move (every
   instant of the year rises) and 4 long-range plateaus (prep_slong!, :77: the cyclic instants
   a+1 .. a+L rise, energy moved from step a to step a+L with pro-rata compensation at both and the
   Jacobian test), in random order. esm_operation_sweeps calls it after the local (and multiscale)
   sweep when esm_opts.storage_long is 1. stats (may be NULL) += (moves tried, taken, guard events). */
int esm_storage_long(esm_ctx *ctx, int64_t sweep, int64_t *stats);

/* Capacity scores per replica: sk [R*K] (s_k = -beta_v dC/dk + dlogJ/dk, node space) and the
   capex force fk [K] (beta_k dK/dk), capacity_scores (src/replicas.jl:329) on energy_cost with
   grad (src/energy.jl:551) and log_measure_grad (:811). parts (may be NULL): [R*8] cost parts
   per replica: capex, op, gen, storage, shed, dump, penalty, 0 (CostParts, src/energy.jl:531).
   One pass over the state, summed in a fixed order: the same state gives the same scores bit for
   bit. The FP64 build forms every node balance and term in FP64. The FP32 production build forms
   them in FP32 from its FP32 state and sums them with compensated (Neumaier) sums; the sign of a
   node balance within its rounding bound of 0 is taken from the FP64 balance. Every score and cost
   part carries a bound on its distance from the exact sums (esm_score_errors). */
int esm_capacity_scores(esm_ctx *ctx, double *sk, double *fk, double *parts);

/* The error bounds of the last esm_capacity_scores (or _static) call: sk_err [R*K] bounds
   |sk - s_exact|, parts_err [R*8] bounds the cost parts, where s_exact are the same sums taken
   exactly over the same state (running error analysis of the terms' and the sums' rounding).
   Either may be NULL. ESM_ESTATE when the state changed since the last scores. */
int esm_score_errors(esm_ctx *ctx, double *sk_err, double *parts_err);

/* esm_capacity_scores without allocating in the call (no counterpart in the reference): for a
   caller that must not allocate device memory here -- one whose device memory is held by a caching
   allocator or a capped pool, or whose step must not stall on cudaMalloc/cudaFree. The score
   accumulators -- the partial sums of the score pass over step chunks and the 2*R*(K+8) totals
   and bounds --
   live in a file-scope device array of ESM_SCORE_SCRATCH_DOUBLES doubles (8 MiB); the pass takes
   fewer chunks where that is needed to fit (the same chunks as esm_capacity_scores, so both give the
   same scores bit for bit), and contexts that do not fit even with one chunk (2*R*(K+8) near 2^20)
   are rejected with ESM_EINVAL. esm_create, which allocates anyway, resolves
   the array's address on the context's device and loads the score kernels, so the call places
   nothing on the device; it must be made with the context's device current (else ESM_EINVAL). The
   array is shared by all contexts on a device, so overlapping calls race: serialise them. Same
   outputs and effect as esm_capacity_scores (a following esm_langevin_step uses these scores). */
#define ESM_SCORE_SCRATCH_DOUBLES (1 << 20)
int esm_capacity_scores_static(esm_ctx *ctx, double *sk, double *fk, double *parts);

/* The Langevin step of the shared capacities from the replica-weighted score
   (src/replicas.jl:697 sbar = sum_j w_j sk_j; langevin_capacities :391, langevin_update :368)
   followed by the dispatch following of every replica (follow_capacities! :448:
   set_dispatchable_capacity! :412 and the kop curve of renewables and storage, src/kop.jl).
   w [R] replica weights; eta [nkf], kappa_s [nkf] per capacity group; xi [K] standard normals
   (NULL: drawn from the context's Philox stream at counter `it`); knew_out [K] (may be NULL);
   nclip_out (may be NULL). */
int esm_langevin_step(esm_ctx *ctx, const double *w, const double *eta, const double *kappa_s,
                      double kappa_min, double clip, int32_t box, const double *xi, int64_t it,
                      double *knew_out, int32_t *nclip_out);

/* The dispatch following of esm_langevin_step for given capacities: every replica follows the
   capacities from the current k to knew [K] (follow_capacities!, src/replicas.jl:448), which then
   become the context's k (k_out [K], may be NULL: the followed values, knew within the box). */
int esm_follow_capacities(esm_ctx *ctx, const double *knew, double kappa_min, double *k_out);

/* Snapshot of the sampler state (fields, weather, regimes, k) into device buffers of the context
   (allocated by the first call), and its restoration (caches rebuilt). No reference counterpart:
   the delayed-acceptance capacity step restores the state of a rejected proposal. */
int esm_state_save(esm_ctx *ctx);
int esm_state_restore(esm_ctx *ctx);

/* The line-move grid. k_move runs as blocks of 1, 2 or 4 warps whose warps take work items from a
   per-move counter, so any grid is correct. The block shape sets the register budget (80, 64 and
   48 registers per thread) and with it the warps an SM holds (up to 24, 32 and 40); the warp count
   trades latency hiding against the cache footprint of the warps' walk scratch. esm_set_move_grid
   sets warps_per_block (1, 2, 4) and warps_per_sm (0: the resident limit of that shape; capped at
   it) and drops the captured class graphs; the default is one-warp blocks at their limit. Models
   whose walk scratch exceeds the lanes' local arrays keep it in device memory, first sized for at
   most 1 GB (never below the default grid) and grown (reallocated) by esm_set_move_grid when a
   larger grid is set.
   esm_move_grid reads the current shape, warps per SM and the limits of the three shapes
   (limits_per_sm[3]). No reference counterpart (the reference threads the steps of a class on the
   host, src/local.jl:1954). */
int esm_set_move_grid(esm_ctx *ctx, int32_t warps_per_block, int32_t warps_per_sm);
int esm_move_grid(const esm_ctx *ctx, int32_t *warps_per_block, int32_t *warps_per_sm, int32_t *limits_per_sm);

/* Move log (diagnostics of parity tests; no reference counterpart): with nreps > 0 every class pass
   of esm_class_pass records the t that each line move took for the replicas below nreps (device
   memory: moves x longest class x nreps doubles); 0 switches it off. esm_move_log copies the log of
   the last class pass, which must have been class cls, as [(move * nsteps + q) * nreps + replica]
   for the class's q-th step (nsteps its steps); moves whose selection made no move read NaN. With
   cls = -1 it copies the log of the last esm_storage_long: [(unit * 5 + move) * nreps + replica]
   over the sweep's eligible units in plan order (at most 5 moves each). */
int esm_set_move_log(esm_ctx *ctx, int32_t nreps);
int esm_move_log(esm_ctx *ctx, int32_t cls, double *out);

/* The cooperative walk of the separable moves. A move whose terms are storage units at distinct
   nodes and nothing else (the state-of-charge atoms, walk!, src/local.jl:1294, on a potential that
   is a sum of per-unit functions) with at least min_units units runs one (step, replica) task per
   warp: the lanes generate the units' breakpoints, a window's breakpoints are sorted in shared memory
   and the potential follows from warp scans. Smaller and other moves keep one task per lane (k_move).
   min_units 0 switches it off. Same draws and the same points as the per-lane walk, up to the
   order of floating-point sums. esm_set_sep_walk drops the captured class graphs; esm_sep_walk
   reads the setting and the kernel's warps. No reference counterpart. */
#define ESM_SEP_MIN_DEFAULT 0
int esm_set_sep_walk(esm_ctx *ctx, int32_t min_units);
int esm_sep_walk(const esm_ctx *ctx, int32_t *min_units, int32_t *warps);

/* How the line moves of a class pass are launched. ESM_MOVES_PER_MOVE (the default): one k_move
   launch per move, all tasks of move mi before any task of move mi + 1. ESM_MOVES_PER_CLASS: the
   whole class pass in one launch, whose warps take (move, 32-task item) pairs in move-major order
   and run an item's move mi + 1 as soon as its move mi is done (the tasks of a colour class are
   independent, so a task's moves and their results are the same: bit-identical states), without
   the idle tail each per-move launch ends with; each of its waits for an item's previous move is
   bounded, and one that runs out makes the next esm_sync or statistics read return ESM_ETIMEOUT.
   Not combined with the cooperative walk (esm_set_sep_walk > 0 keeps the per-move launches). No
   reference counterpart. */
enum { ESM_MOVES_PER_MOVE = 0, ESM_MOVES_PER_CLASS = 1 };
int esm_set_move_schedule(esm_ctx *ctx, int32_t schedule);
int esm_move_schedule(const esm_ctx *ctx, int32_t *schedule);

/* Autotuner of the line-move grid: for each candidate (warps_per_block, warps_per_sm) -- the three
   block shapes at their resident limits and at 8, 16, 24, 32, 40 warps per SM below them -- one
   colour class of sweep `sweep` is run and timed (CUDA events on the context's stream) from the
   current state, which is then restored, and the fastest grid is kept. The chain state is
   unchanged; the esm_state_save slot is overwritten. Outputs (each may be NULL): the chosen pair
   best[2], the candidate pairs cand[2*ESM_TUNE_MAX], their times in ms ms[ESM_TUNE_MAX], their count. */
#define ESM_TUNE_MAX 16
int esm_autotune_moves(esm_ctx *ctx, int64_t sweep, int32_t *best, int32_t *cand, double *ms, int32_t *ncand);

/* Lag probe (lag_probe, src/replicas.jl:733): a copy of replica j, at the chain's capacities and
   with its weather frozen, runs nsweeps operation sweeps (sweep indices sweep0 ... sweep0 +
   nsweeps - 1 of the probe context's streams: give every probe its own range, e.g. sweep0 = step *
   nsweeps, as the reference's probe stream advances from probe to probe) and sk_mean [K]
   receives the mean capacity score of the last `tail` sweeps, fk
   [K] (may be NULL) the prior term of the last; the chain is unchanged. The host forms the gap
   against the replica's in-flight scores and adapts the step (adapt_step!, :758). Needs
   esm_opts.probe = 1. */
int esm_lag_probe(esm_ctx *ctx, int32_t j, int32_t nsweeps, int32_t tail, int64_t sweep0, double *sk_mean,
                  double *fk);

/* Fraction of (step, replica) pairs in each (regime, season): occ [nreg*4], regime-major, the
   season of a step as season (src/weather.jl:50). The regime summary fed to the surrogate. */
int esm_regime_occupancy(esm_ctx *ctx, double *occ);

/* Weather features of every replica (replica_features / weather_features, src/replicas.jl:246-276),
   from its weather anomalies through the model's data map: per replica r, out[r * nfeat + i] is
   [0] the annual mean system load (GW: the sum over nodes of the positive load, / 1e3), [1 .. C]
   the annual mean availability of each weather-dependent carrier (the carriers of the renewable
   units in increasing group order, averaged over their units), [1 + C] the annual mean residual
   load at the reference capacities kref [K] (load minus the sum over renewable units of kref times
   availability, GW), [2 + C] its peak step, [3 + C] its worst cyclic 7-step mean, [4 + C .. 3 + C +
   nreg] the frequency of each regime over the steps, [4 + C + nreg] the number of regime switches;
   nfeat = 5 + C + nreg (written whenever nfeat is not NULL; out NULL: only nfeat). The declared
   tilt functional of the replica step (TiltFunctional, :278) is the standardised feature [1 + C]. */
int esm_replica_features(esm_ctx *ctx, const double *kref, double *out, int32_t *nfeat);

/* Weather step of the replicas flagged in `moved` [R] (0/1): pCN of angle theta[r] in the VAR
   innovations (src/replicas.jl:105 pcn_weather), then with window[r] > 0 a regime window move of
   that length starting at wstart[r] (:156 regime_window, uniforms from the stream), then the
   compensated initialisation of the operation (:207 compensate_weather!). xi (may be NULL):
   injected normals [R*n0*T]. */
int esm_weather_step(esm_ctx *ctx, const int32_t *moved, const double *theta,
                     const int32_t *window, const int32_t *wstart, const double *xi, int64_t it);

/* Kernel families of the device timing (esm_timing). */
enum { ESM_KT_CLASS = 0, ESM_KT_REBUILD, ESM_KT_SCORE, ESM_KT_LANGEVIN, ESM_KT_WEATHER, ESM_KT_STORAGE, ESM_KT_N };

/* Device timing: while on, every launch of the library is bracketed by CUDA events on the
   context's stream. esm_timing writes out[2*i] = accumulated milliseconds and out[2*i+1] = launches
   of family i (ESM_KT_*) since timing was switched on, then resets the counters. */
int esm_set_timing(esm_ctx *ctx, int32_t on);
int esm_timing(esm_ctx *ctx, double *out);

/* The context's CUDA stream (a cudaStream_t), for callers that order their own work after it. */
void *esm_stream(esm_ctx *ctx);

/* Synchronise the context's stream with a bounded wait (ESM_ETIMEOUT after timeout_s). */
int esm_sync(esm_ctx *ctx, double timeout_s);

/* Device launches recorded since creation (kernels of this library). */
int64_t esm_launch_count(const esm_ctx *ctx);

/* ------------------------------------------------------------------------------------------
 * A batch of independent chains (models of any sizes, one context each, one precision) whose
 * operation sweeps run together: the batch axis of the reference's GPU port (a batch of models
 * in one program, device/src/replica_run.jl:84-108) over the local sweep (local_sweep!,
 * src/local.jl:1927, as esm_operation_sweeps runs it without the storage sweeps). A sweep is one
 * CUDA graph captured at the batch's first sweep: the caching rebuild of every model, then per
 * colour-class pass one launch that builds every model's move descriptors and one line-move launch
 * per move index, whose work items are the tasks of every model that has that move. Each task
 * runs the arithmetic of the model's own class pass, so every model's state after
 * esm_batch_sweeps equals the state esm_operation_sweeps gives it on its own context.
 * ------------------------------------------------------------------------------------------ */
typedef struct esm_batch esm_batch;
/* ctxs [n]: contexts created by esm_create with the same precision, states uploaded, the storage
   sweeps off (esm_opts.storage_ms = storage_long = 0); they stay owned by the caller and must
   outlive the batch. The batch runs on its own stream, ordered after and before each context's. */
int esm_batch_create(esm_ctx *const *ctxs, int32_t n, esm_batch **out);
int esm_batch_destroy(esm_batch *b);
const char *esm_batch_last_error(const esm_batch *b);
/* n operation sweeps (sweep indices sweep0 ... sweep0 + n - 1) of every chain; stats (may be NULL):
   [n_models * (2 * (ESM_NFAM + 1) + 1)], chain i's counts at row i (the order of ctxs) in
   esm_operation_sweeps' layout (tried and moved per family, then the guard events) */
int esm_batch_sweeps(esm_batch *b, int32_t n, int64_t sweep0, int64_t *stats);
/* The grid of the batch's line-move launches: warps per block (1 or 2) and warps per SM (0: the
   resident limit); esm_batch_grid reads it back with the resident limit of that block shape. */
int esm_batch_set_grid(esm_batch *b, int32_t warps_per_block, int32_t warps_per_sm);
int esm_batch_grid(const esm_batch *b, int32_t *warps_per_block, int32_t *warps_per_sm, int32_t *limit_per_sm);
/* Autotuner of the batch's grid: for both block shapes at 8, 16, 24, 32 warps per SM and at their
   resident limits, the first ESM_BATCH_TUNE_MOVES line moves of the first colour-class pass of
   sweep `sweep` of every chain are run twice and the second run is timed (CUDA events on the
   batch's stream), each run from the current states, which are then restored; the fastest grid is
   kept. The chains are unchanged; every context's esm_state_save slot is overwritten. Outputs as
   esm_autotune_moves. */
#define ESM_BATCH_TUNE_MOVES 64
int esm_batch_autotune(esm_batch *b, int64_t sweep, int32_t *best, int32_t *cand, double *ms, int32_t *ncand);
/* CUDA-event time of the batch's last esm_batch_sweeps call (ms, the device time of its sweeps). */
int esm_batch_time(const esm_batch *b, double *ms);
/* Kernels launched by the batch's sweeps since creation. */
int64_t esm_batch_launch_count(const esm_batch *b);

/* ------------------------------------------------------------------------------------------
 * Surrogate of the replica-averaged capacity score (no counterpart in the reference: the
 * learned proposal is an addition of this library). An MLP with nlayers linear layers of widths
 * dims[0] -> dims[1] -> ... -> dims[nlayers], SiLU between them, BF16 weights and activations
 * with FP32 accumulation on the tensor cores, trained by Adam on the mean-squared error.
 * ------------------------------------------------------------------------------------------ */
typedef struct esm_mlp esm_mlp;
int esm_mlp_create(int32_t nlayers, const int32_t *dims, int32_t batch_max, uint64_t seed, esm_mlp **out);
int esm_mlp_destroy(esm_mlp *mlp);
const char *esm_mlp_last_error(const esm_mlp *mlp);
/* layer l: W [dims[l+1], dims[l]] row-major and b [dims[l+1]], FP32 (either may be NULL) */
int esm_mlp_set_layer(esm_mlp *mlp, int32_t l, const float *w, const float *b);
int esm_mlp_get_layer(esm_mlp *mlp, int32_t l, float *w, float *b);
/* y [B, dims[nlayers]] = MLP(x [B, dims[0]]) */
int esm_mlp_forward(esm_mlp *mlp, int32_t B, const float *x, float *y);
/* one Adam step (lr) on the minibatch; loss_out: (1/2B) sum (y - t)^2 before the step;
   grads_out (may be NULL): the gradients, layer by layer, W then b */
int esm_mlp_train_step(esm_mlp *mlp, int32_t B, const float *x, const float *target, float lr,
                       double *loss_out, float *grads_out);
int64_t esm_mlp_launch_count(const esm_mlp *mlp);
/* the GEMM kernels of the MLP: 1 (default) the 5th-generation tensor cores (tcgen05.mma, FP32
   accumulator in tensor memory, one 128 x 64 tile per CTA), 0 the warp-level mma.sync kernel */
int esm_mlp_set_gemm(esm_mlp *mlp, int32_t kind);

#ifdef __cplusplus
}
#endif
#endif /* ESMCUDA_H */

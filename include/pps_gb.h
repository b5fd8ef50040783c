/* pps_gb.h - C ABI of the GB300-native postflop DCFR solver (libpps_gb.so).
 *
 * This is the drop-in boundary: every entry point mirrors one method of the
 * reference's pps::gpu::GpuPostflopSolver (cuda/gpu_cfr.h:141-264), which
 * the reference's own FFI (the pybind module, python/pps_native.cpp:514-551)
 * binds. Plain pointers and sizes only; results go into caller buffers
 * whose maximum sizes are fixed by PPS_GB_MAX_ACTIONS and PPS_GB_COMBOS.
 *
 * Every call returns PPS_GB_OK (0) or an error code; pps_gb_last_error()
 * gives the calling thread's message for its last failed call. The library
 * never exits the process. A handle is not thread-safe: drive one solver
 * from one thread at a time (the reference has the same rule,
 * python/pps_native.cpp:256-259).
 */
#ifndef PPS_GB_H
#define PPS_GB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PPS_GB_ABI_VERSION 1
#define PPS_GB_MAX_ACTIONS 32 /* reference kMaxNa, cuda/gpu_cfr.cu:41 */
#define PPS_GB_COMBOS 1326    /* reference kCombos, src/range.h:14 */
#define PPS_GB_MAX_SIZES 16

enum {
  PPS_GB_OK = 0,
  PPS_GB_E_ARG = 1,         /* invalid argument (bad board, config, algo) */
  PPS_GB_E_INDEX = 2,       /* node / action / player index out of range */
  PPS_GB_E_STATE = 3,       /* call not valid in the current state */
  PPS_GB_E_IO = 4,          /* file cannot be opened / written */
  PPS_GB_E_FORMAT = 5,      /* corrupt, truncated or mismatched file */
  PPS_GB_E_CUDA = 6,        /* CUDA runtime error (message has details) */
  PPS_GB_E_MEMORY = 7,      /* host or device allocation failed */
  PPS_GB_E_DEVICE = 8,      /* a kernel raised its device error flag */
  PPS_GB_E_BUDGET = 9,      /* admission refused: over the HBM budget */
  PPS_GB_E_TOO_WIDE = 10,   /* more than PPS_GB_MAX_ACTIONS actions */
  PPS_GB_PENDING = 11       /* batch request not finished yet (not an error) */
};

typedef struct pps_gb_solver pps_gb_solver;

/* pf::BetConfig (src/postflop_cfr.h:24-42). */
typedef struct {
  double bet_fracs[PPS_GB_MAX_SIZES];
  int n_bet_fracs;
  double raise_mults[PPS_GB_MAX_SIZES];
  int n_raise_mults;
  int bet_allin;
  int bet_geometric;
  int max_raises;
  double add_allin_threshold;
  double force_allin_threshold;
  double merging_threshold;
} pps_gb_bet_config;

/* gpu::PostflopSpot (cuda/gpu_cfr.h:35-42); card id = suit*13 + rank. */
typedef struct {
  uint8_t board[5];
  int n_board; /* 3, 4 or 5 */
  double oop[PPS_GB_COMBOS];
  double ip[PPS_GB_COMBOS];
  int64_t pot;
  int64_t stack;
} pps_gb_spot;

/* gpu::ActionLabel (cuda/gpu_cfr.h:48-51); kind = pf::ActionKind value
 * (0 fold, 1 check, 2 call, 3 bet, 4 raise, 5 all-in). */
typedef struct {
  int32_t kind;
  int64_t amount;
} pps_gb_action;

/* pf::NodeStats (src/postflop_cfr.h:55-60). */
typedef struct {
  double ev0;
  double ev1;
  double expl;
  int64_t pair_mass;
} pps_gb_node_stats;

/* Scalars of a compiled solver (numNodes/maxDepth/iterationsRun/... of
 * cuda/gpu_cfr.h:176-241). */
typedef struct {
  int32_t num_nodes;
  int32_t max_depth;
  int32_t num_decide_nodes;
  int32_t iterations_run;
  int64_t total_iterations;
  int32_t n_base[2];
  int64_t row_total; /* regret (= strategy) row entries, reference regTotal */
  int32_t empty;     /* 1 when a range compiled to no combos */
  int32_t launches_per_iteration;
  int64_t device_bytes;
  int64_t h2d_bytes; /* host->device bytes copied since creation */
  int64_t d2h_bytes; /* device->host bytes copied since creation */
  int32_t engine;    /* 0 terminal groups (default), 1 per-node terminal kernels */
  int32_t compensated; /* 1: two-float cumulative-strategy sums (pps_gb_set_compensated) */
} pps_gb_info;

/* Per kernel class of one profile pass (pps_gb_profile). */
typedef struct {
  char name[32];
  int64_t launches;
  double ms;          /* summed CUDA-event time of the launches */
  double algo_bytes;  /* summed algorithmic bytes (see the byte model) */
} pps_gb_kernel_stat;

/* gpu::DecideNodeInfo (cuda/gpu_cfr.h:54-62). */
typedef struct {
  int32_t node_id;
  int32_t player;
  int32_t depth;
  int32_t n_board;
  int32_t n_combos;
  int32_t n_actions;
  pps_gb_action actions[PPS_GB_MAX_ACTIONS];
  int32_t children[PPS_GB_MAX_ACTIONS];
} pps_gb_decide_info;

const char* pps_gb_last_error(void);
int pps_gb_abi_version(void);
/* The bet config defaults of pf::BetConfig (src/postflop_cfr.h:24-42). */
void pps_gb_bet_config_default(pps_gb_bet_config* cfg);

/* GpuPostflopSolver(spot, cfg) - cuda/gpu_cfr.h:144. */
int pps_gb_create(const pps_gb_spot* spot, const pps_gb_bet_config* cfg,
                  pps_gb_solver** out);
/* Extension: one bet config per street (cfgs[k] where the board has 3+k
 * cards); no reference counterpart (the reference shares one config,
 * cuda/gpu_cfr.cu:1254-1256). */
int pps_gb_create_streets(const pps_gb_spot* spot,
                          const pps_gb_bet_config cfgs[3],
                          pps_gb_solver** out);
/* GpuPostflopSolver(solutionPath) - cuda/gpu_cfr.h:149. */
int pps_gb_load(const char* path, pps_gb_solver** out);
/* ~GpuPostflopSolver - cuda/gpu_cfr.h:150. NULL is ignored. */
void pps_gb_destroy(pps_gb_solver* h);

/* solve(iterations, algo, target) - cuda/gpu_cfr.h:160. */
int pps_gb_solve(pps_gb_solver* h, int iterations, const char* algo,
                 double target);
/* continueSolve(iterations, target) - cuda/gpu_cfr.h:168. */
int pps_gb_continue(pps_gb_solver* h, int iterations, double target);
/* reset() - cuda/gpu_cfr.h:172. */
int pps_gb_reset(pps_gb_solver* h);
/* numNodes/maxDepth/numDecideNodes/iterationsRun/totalIterations. */
int pps_gb_get_info(pps_gb_solver* h, pps_gb_info* out);

/* stats() - cuda/gpu_cfr.h:184 (FP64 walks on the device). */
int pps_gb_stats(pps_gb_solver* h, pps_gb_node_stats* out);
/* rootStrategy() - cuda/gpu_cfr.h:187; freq[PPS_GB_MAX_ACTIONS]. */
int pps_gb_root_strategy(pps_gb_solver* h, double* freq, int* n_actions);
/* nodeStrategy(i) - cuda/gpu_cfr.h:196; *n_actions = 0 where the reference
 * returns {} (nodes past a chance node). */
int pps_gb_node_strategy(pps_gb_solver* h, int decide_idx, double* freq,
                         int* n_actions);
/* decideNode(i) - cuda/gpu_cfr.h:201. */
int pps_gb_decide_node(pps_gb_solver* h, int decide_idx,
                       pps_gb_decide_info* out);
/* comboStrategy(i) - cuda/gpu_cfr.h:208: actions[PPS_GB_MAX_ACTIONS],
 * combos[PPS_GB_COMBOS], freqs[PPS_GB_MAX_ACTIONS * PPS_GB_COMBOS]
 * (action-major, row stride = *n_combos). */
int pps_gb_combo_strategy(pps_gb_solver* h, int decide_idx, int* n_actions,
                          int* n_combos, pps_gb_action* actions,
                          int* combos, double* freqs);
/* rootEvPerCombo() - cuda/gpu_cfr.h:211, one player per call; combos, ev,
 * mass hold PPS_GB_COMBOS entries. */
int pps_gb_root_ev(pps_gb_solver* h, int player, int* n, int* combos,
                   double* ev, double* mass);
/* nodeEv(i) - cuda/gpu_cfr.h:216. Per side p (0, 1): n_combos[p],
 * combos/ev/mass[p * PPS_GB_COMBOS + i], agg_ev[p]. Per action a:
 * action_ev[a * PPS_GB_COMBOS + i] over the decider's combos and
 * action_agg[a]. */
int pps_gb_node_ev(pps_gb_solver* h, int decide_idx, int* decider,
                   int* n_actions, pps_gb_action* actions, int* n_combos,
                   int* combos, double* ev, double* mass, double* agg_ev,
                   double* action_ev, double* action_agg);
/* runoutSummary(i, a) - cuda/gpu_cfr.h:222. Per branch b (< 52):
 * cards[b], next_decide[b], n_freq[b], freq[b * PPS_GB_MAX_ACTIONS + k],
 * agg_ev[b * 2 + p]. */
int pps_gb_runout_summary(pps_gb_solver* h, int decide_idx, int action_idx,
                          int* decider, int* n_actions,
                          pps_gb_action* actions, int* n_branches,
                          int* cards, int* next_decide, int* n_freq,
                          double* freq, double* agg_ev);
/* playerCards(p) / numBaseCombos(p) - cuda/gpu_cfr.h:227-230:
 * cards[2 * PPS_GB_COMBOS]. */
int pps_gb_player_cards(pps_gb_solver* h, int player, uint8_t* cards, int* n);
/* playerWeights(p) - cuda/gpu_cfr.h:234: w[PPS_GB_COMBOS]. */
int pps_gb_player_weights(pps_gb_solver* h, int player, double* w, int* n);
/* treeStructure() - cuda/gpu_cfr.h:238. Pass NULL arrays to get the sizes
 * (*n_nodes, *n_children); then kinds[n_nodes], child_base[n_nodes],
 * children[n_children], boards[5 * n_nodes]. */
int pps_gb_tree_structure(pps_gb_solver* h, uint8_t* kinds, int* child_base,
                          int* children, uint8_t* boards, int* n_nodes,
                          int* n_children);
/* save(path) - cuda/gpu_cfr.h:246 ("PPS1" file, cuda/gpu_cfr.cu:2686-2785). */
int pps_gb_save(pps_gb_solver* h, const char* path);
/* Extension (no reference counterpart): save with compressed rows, each
 * action row as 16-bit codes plus one f32 scale (file version 3, or 4 with
 * per-street configs), about half the size; pps_gb_load reads every
 * version. Decoded entries are within half a code step of the saved ones. */
int pps_gb_save_compressed(pps_gb_solver* h, const char* path);
/* debugDump() - cuda/gpu_cfr.h:249. */
int pps_gb_debug_dump(pps_gb_solver* h);

/* Row access in the reference's dense layout (decide nodes in node order,
 * each na x nC action-major at the reference regOff, cuda/gpu_cfr.cu:
 * 1476-1481). which: 0 = cumulative regrets, 1 = cumulative strategy.
 * Replaces the reference's debug hooks on the same rows (GPU_CFR_SEED_STRAT,
 * cuda/gpu_cfr.cu:2066-2097, writes the strategy rows). */
int pps_gb_read_rows(pps_gb_solver* h, int which, float* out, int64_t cap,
                     int64_t* n);
int pps_gb_write_rows(pps_gb_solver* h, int which, const float* in,
                      int64_t n);
/* One value walk (reference rootValue, cuda/gpu_cfr.cu:894-916): mode 0 =
 * EV vs the average strategy, 1 = best response; FP64 on the device.
 * root_cfv receives the traverser's root row (n_base[tr] entries) and
 * *value the range-weighted root value in chips. */
int pps_gb_walk(pps_gb_solver* h, int traverser, int mode, double* root_cfv,
                double* value);
/* Extension: the iteration graph's plan. 0 = staged: decide records and
 * chance tasks per level, showdown and fold nodes of one level and board
 * state in groups of four (one CTA each, float4 lanes) on side streams; 1 =
 * one CTA per terminal node; 2 = fused (lists of at most 1023 combos): one
 * launch per backward level for all its tasks, on one stream. 0 and 2
 * compute identical rows, 1 agrees to f32 rounding. By default the first
 * solve of 32 or more iterations times 0 and 2 on the tree and keeps the
 * faster; setting an engine turns that off. */
int pps_gb_set_engine(pps_gb_solver* h, int engine);

/* Extension: the launch shape of the iteration graph, which the first solve
 * of 32 or more iterations picks by timing candidates on the tree (or takes
 * from the autotuner's cache for the tree's size class: file
 * PPS_GB_TUNE_FILE, "off" for none, else $XDG_CACHE_HOME or $HOME/.cache
 * pps_gb/launch_shapes). plan: 0 staged, 2 fused backward levels (lists of
 * at most 1023 combos). Each cap gives a launch kind's grid: 0, one CTA per
 * task; k (1..64), a persistent grid of k x SM-count CTAs striding over the
 * level's (spot, node-range) tasks. Shapes change timing only: the rows are
 * identical under every shape. Setting a shape turns the autotuner off. No
 * reference counterpart (its launch geometry is fixed: block 128, one block
 * per node, cuda/gpu_cfr.cu:806-816). */
typedef struct {
  int32_t plan;
  int32_t fwd_cap, bwd_cap, sd_cap, fd_cap;
} pps_gb_launch_shape;
int pps_gb_set_launch_shape(pps_gb_solver* h, const pps_gb_launch_shape* shape);
int pps_gb_get_launch_shape(pps_gb_solver* h, pps_gb_launch_shape* out);

/* Extension: compensated (two-float) cumulative-strategy sums, the update
 * strat = strat * avg + sigma of cuda/gpu_cfr.cu:512-523 carried as an
 * unevaluated sum of two floats (a row of low words beside the strategy
 * rows, device memory allocated on first use). The strategy rows keep the
 * sum rounded to f32, so every reader - walks, queries, files - is
 * unchanged; turning the option on keeps the current sums (low words 0).
 * Off by default (the reference's plain f32 sums). */
int pps_gb_set_compensated(pps_gb_solver* h, int on);

/* Benchmark helper: enqueues n further DCFR iterations (graph replays that
 * continue the current DCFR schedule) bracketed by CUDA events recorded on
 * the solver's own stream, waits, and returns the elapsed milliseconds.
 * Plays the role of the reference's solve-loop timing in tools/gpu_pfflop.cu:
 * 169-180. */
int pps_gb_time_iterations(pps_gb_solver* h, int n, double* ms);
/* Profile pass (the reference's GPU_CFR_PROFILE mode, cuda/gpu_cfr.cu:
 * 1895-1987): runs n further iterations launch by launch, each launch
 * bracketed by CUDA events, and sums time and algorithmic bytes per kernel
 * class into out[cap]; *n_out = classes written. flags bit 0: issue each
 * backward level once per node kind (showdown / fold / chance / decide)
 * and report the kinds separately (the reference's kindMask breakdown). */
int pps_gb_profile(pps_gb_solver* h, int n, int flags, pps_gb_kernel_stat* out,
                   int cap, int* n_out);
/* Diagnostic of the bounded device waits (no counterpart in the reference):
 * on the solver's stream, one warp waits on its shared-memory barrier for a
 * copy that is never issued, with the same bounded wait and give-up path
 * as the iteration's bulk-copied records (`spins` polls per round, one
 * round plus four drain rounds; 1 <= spins <= 65536, the records' own
 * bound, else PPS_GB_E_ARG). The give-up sets the solver's device error
 * word, so the call returns PPS_GB_E_CUDA ("a device wait timed out"); the
 * solver stays usable. No GPU fault is involved. */
int pps_gb_probe_bounded_wait(pps_gb_solver* h, int spins);

/* Size in bytes of the static device array behind pps_gb_solve_noalloc. */
#define PPS_GB_NOALLOC_SCRATCH_BYTES (64ull << 20)

/* No-allocation solve. No counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc - processes whose device memory is
 * owned by another allocator (a framework's caching allocator holding the
 * GPU, a fixed budget carved out at start-up) and callers that must not
 * trigger cudaMalloc's implicit device-wide synchronization.
 *
 * Runs `iterations` DCFR iterations (the "dcfr" schedule, absolute indices
 * first_iteration .. first_iteration + iterations - 1) of the spot over the
 * caller's cumulative regret and strategy rows: device memory in the
 * reference's dense layout (see pps_gb_read_rows), row_capacity floats
 * each, read at entry and written back at exit. Every other device buffer
 * (tree tables, reach and value rows, schedule) lives in ONE static device
 * array of PPS_GB_NOALLOC_SCRATCH_BYTES (64 MiB), held by every GPU that
 * loads the library until the process exits; spots that need more are
 * rejected with PPS_GB_E_BUDGET and a message giving both sizes (the
 * schedule table counts too: it holds this call's `iterations` entries, so
 * a very long call may need splitting). The call allocates no device memory
 * (no cudaMalloc, cudaFree or allocating library routine), issues its work
 * on `stream` (NULL: the legacy default stream) and waits for it. The first
 * call on a device looks up the array's device address with
 * cudaGetSymbolAddress and keeps it for the device's current context (after
 * a cudaDeviceReset the next call looks it up again); make that first call
 * before any stream capture. All calls share the array and leave their
 * contents in it: calls that overlap on a GPU (other threads or streams)
 * race - serialize them. A spot without decide nodes (zero behind-stack)
 * has no rows: the buffers may then be NULL. A CUDA error left pending by
 * the caller's earlier work is reported as such (PPS_GB_E_CUDA) and left
 * pending.
 * *n_rows (may be NULL) receives the row count the spot needs as soon as
 * the spot is compiled - also when the call then fails because
 * row_capacity is too small or the scratch too small - so a call with
 * row_capacity 0 is a size query. */
int pps_gb_solve_noalloc(const pps_gb_spot* spot, const pps_gb_bet_config* cfg,
                         float* d_regret, float* d_strat, int64_t row_capacity,
                         int first_iteration, int iterations, void* stream,
                         int64_t* n_rows);

/* ---------------------------------------------------------------------
 * Batched and served solving. No reference counterpart: the reference
 * solves one spot per GpuPostflopSolver (cuda/gpu_cfr.h:141-264) and its
 * API server serialises solves behind one lock (python/pps_api.py). Here
 * many spots are resident on the GPU at once and share every launch:
 * submit() queues a spot (compiled on host threads), a driver admits
 * compiled spots in submission order while the device memory the batch
 * maps stays within the HBM budget, runs check_every DCFR iterations of all
 * resident spots per epoch (one CUDA graph), checks each spot's
 * exploitability with FP64 best-response walks and retires it once it is
 * at or below its target (or at max_iterations), with FP64 EV walks.
 * Requests submitted while others run are admitted as memory frees up, so
 * their work overlaps on the device. A spot's result does not depend on the
 * other resident spots (same rows, same checks, same iteration count).
 * All pps_gb_batch_* calls may come from any thread.
 * --------------------------------------------------------------------- */
typedef struct pps_gb_batch pps_gb_batch;

typedef struct {
  int64_t hbm_budget;      /* device bytes resident spots may occupy (0: 80% of free) */
  int32_t check_every;     /* most DCFR iterations between two checks of a spot (0: 64) */
  int32_t fixed_checks;    /* 1: check every check_every iterations; 0 (default):
                              adaptive, first check after min(32, check_every), the
                              next where exploitability ~ 1/t^2 would meet the target,
                              in steps of 16 iterations */
  int32_t max_iterations;  /* per spot, rounded up to a multiple of 16 (0: 4096) */
  int32_t compile_threads; /* host compile threads (0: hardware threads, at most 16) */
  char algo[16];           /* "dcfr" (default), "dcfr-g2", "dcfr-noreset", "dcfr-g2-noreset" */
} pps_gb_batch_config;

typedef struct {
  int64_t ticket;
  int32_t status;      /* PPS_GB_OK, or this request's error (pps_gb_batch_result.error) */
  int32_t converged;   /* 1: exploitability <= target at the last check */
  int32_t iterations;  /* DCFR iterations run */
  int32_t num_nodes;
  double ev0, ev1, exploitability, target; /* chips (pf::NodeStats fields) */
  int64_t pair_mass;                        /* pf::NodeStats::pairMass */
  double submit_ms, admit_ms, finish_ms;    /* ms since the batch was created */
  int64_t device_bytes;                     /* the spot's device footprint */
  int32_t root_actions; /* actions at the root decide node (0: root is no decision) */
  int32_t root_combos;  /* root actor's combos (rows of pps_gb_batch_root_rows) */
  pps_gb_action root_action[PPS_GB_MAX_ACTIONS];
  double root_freqs[PPS_GB_MAX_ACTIONS];    /* range-weighted root strategy */
  char error[160];
} pps_gb_batch_result;

typedef struct {
  int64_t submitted, compiling, waiting, active, done, failed;
  int64_t used_bytes;   /* footprints of the resident spots */
  int64_t device_bytes; /* pool capacity held on the device */
  int64_t budget;
  int64_t epochs, spot_iterations, captures, peak_active;
  int64_t peak_used_bytes; /* largest used_bytes seen (never above budget) */
  int32_t check_every, max_iterations;
  /* Driver time split (ms): admission (uploads), DCFR iterations (CUDA
   * events), iterations plus best-response checks (wall), EV walks and
   * retirement, waiting for compiles. */
  double admit_ms, iterate_ms, check_ms, retire_ms, idle_ms;
} pps_gb_batch_info;

void pps_gb_batch_config_default(pps_gb_batch_config* cfg);
/* Creates a batch on the current CUDA device. */
int pps_gb_batch_create(const pps_gb_batch_config* cfg, pps_gb_batch** out);
/* Stops the serve thread (if any) and frees everything. NULL is ignored. */
void pps_gb_batch_destroy(pps_gb_batch* b);
int pps_gb_batch_set_budget(pps_gb_batch* b, int64_t bytes);
/* Queues a spot (target: exploitability in chips; <= 0 runs to
 * max_iterations). cfgs holds 1 config (all streets) or 3 (per street). */
int pps_gb_batch_submit(pps_gb_batch* b, const pps_gb_spot* spot,
                        const pps_gb_bet_config* cfgs, int n_cfgs,
                        double target, int64_t* ticket);
/* Drives the batch on the calling thread until every submitted request has
 * finished (PPS_GB_OK) or timeout_s (> 0) passed (PPS_GB_PENDING). */
int pps_gb_batch_run(pps_gb_batch* b, double timeout_s);
/* Serve mode: a library thread drives the batch until pps_gb_batch_stop. */
int pps_gb_batch_start(pps_gb_batch* b);
int pps_gb_batch_stop(pps_gb_batch* b);
/* PPS_GB_OK with *out filled once the request finished, else PPS_GB_PENDING. */
int pps_gb_batch_poll(pps_gb_batch* b, int64_t ticket, pps_gb_batch_result* out);
/* Blocks until the request finished or timeout_s (> 0) passed. */
int pps_gb_batch_wait(pps_gb_batch* b, int64_t ticket, double timeout_s,
                      pps_gb_batch_result* out);
/* Moves up to cap finished results (ticket order) into out; their tickets
 * are forgotten afterwards. */
int pps_gb_batch_collect(pps_gb_batch* b, pps_gb_batch_result* out, int cap,
                         int* n_out);
/* Cumulative root strategy rows of a finished, uncollected request
 * (root_actions x root_combos floats, action-major). */
int pps_gb_batch_root_rows(pps_gb_batch* b, int64_t ticket, float* out,
                           int64_t cap, int64_t* n_out);
int pps_gb_batch_get_info(pps_gb_batch* b, pps_gb_batch_info* out);
/* Host only: the device bytes a spot occupies in a batch. */
int pps_gb_batch_footprint(const pps_gb_spot* spot,
                           const pps_gb_bet_config* cfgs, int n_cfgs,
                           int64_t* bytes);

/* Host only (tests): a 64-bit FNV-1a digest of the device layout the
 * library builds for a spot (every node, row, table, task list and record
 * array), 0 for an empty spot. Equal digests mean byte-identical layouts. */
int pps_gb_layout_digest(const pps_gb_spot* spot,
                         const pps_gb_bet_config* cfgs, int n_cfgs,
                         uint64_t* digest);

/* Host-only compile (no device use): runs the tree compiler and reports
 * every artifact in the reference's own layout (cuda/gpu_cfr.cu:1331-1827)
 * through cb(user, name, dtype, data, count); dtype 'i' int32, 'q' int64,
 * 'B' uint8, 'f' float32, 'd' float64. cfgs holds 1 config (all streets)
 * or 3 (per street). */
typedef void (*pps_gb_array_cb)(void* user, const char* name, char dtype,
                                const void* data, int64_t count);
int pps_gb_compile_export(const pps_gb_spot* spot,
                          const pps_gb_bet_config* cfgs, int n_cfgs,
                          pps_gb_array_cb cb, void* user);

/* Evaluator entry (tests): strength keys of n 7-card hands (cards[7*i]). */
int pps_gb_hand_keys(const uint8_t* cards, int n, uint64_t* keys);
/* Bet abstraction entry (tests): pf::betActions (src/postflop_cfr.h:47-51);
 * out[PPS_GB_MAX_ACTIONS]. */
int pps_gb_bet_actions(int64_t pot_base, int64_t stack,
                       const pps_gb_bet_config* cfg, int64_t sc0,
                       int64_t sc1, int actor, int after_allin,
                       int num_bets, int num_streets, pps_gb_action* out,
                       int* n);
/* Range parser entry (tests): parseRange (src/range.h:41). */
int pps_gb_parse_range(const char* text, double* w /* PPS_GB_COMBOS */);

#ifdef __cplusplus
}
#endif

#endif /* PPS_GB_H */

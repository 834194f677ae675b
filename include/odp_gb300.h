/*
 * odp_gb300.h -- entry points of libodp_gb300 beyond the reference's odp.h.
 * None of these has a counterpart in the reference; each evaluates graphs
 * exactly as ODP_Init_aspl_* + ODP_Set_aspl would (same diameter, sum and
 * ASPL bits), and returns an error code instead of exiting.
 *
 *   ODP_Set_aspl_batch   many graphs of any size/degree/symmetry in one
 *                        persistent launch (replayed as a CUDA graph when the
 *                        same shapes come back)
 *   ODPX_Batch_*         the same with an explicit, reusable plan
 *   ODPX_Serve_*         device-resident graphs updated by 2-opt deltas,
 *                        evaluated in continuous batches (serving mode)
 *   ODPX_Anneal_*        simulated-annealing chains whose proposals,
 *                        evaluations and decisions all run on the GPU
 *   ODPX_Generate_*      the reference generators on a private random stream
 *                        (same graphs for the same seed, thread-safe)
 */
#ifndef ODP_GB300_H_INCLUDED
#define ODP_GB300_H_INCLUDED
#include <stddef.h>
#include "odp.h"
#ifdef __cplusplus
extern "C" {
#endif

/* Error codes (0 = success). */
#define ODPX_OK            0
#define ODPX_ERR_INVALID   1   /* bad shape: n % s != 0, bad grid symmetry, ... */
#define ODPX_ERR_CUDA      2   /* a CUDA call failed */
#define ODPX_ERR_ADJACENCY 3   /* adjacency entry outside [0, n) or degree > d */
#define ODPX_ERR_TIMEOUT   4   /* a device-side wait ran past its limit */
#define ODPX_ERR_MEMORY    5   /* admission refused: over the memory budget */
#define ODPX_ERR_STATE     6   /* call out of order (e.g. no plan) */
#define ODPX_PENDING       7   /* ODPX_Serve_poll: not finished yet */

/* One graph of a batch: the arguments of the matching ODP_Init_aspl_* call
 * plus the adjacency of ODP_Set_aspl. */
typedef struct {
  int grid;                  /* 0: ODP_Init_aspl_general[_s], 1: ODP_Init_aspl_grid[_s] */
  int nodes;                 /* general graphs: number of vertices */
  int width, height;         /* grid graphs */
  int degree;
  int symmetries;            /* 1 for the non-_s variants */
  const int *num_degrees;    /* as for ODP_Init_aspl_*, or NULL */
  const int *adjacency;      /* host int[nodes/symmetries][degree] */
} ODP_Graph;

/* Evaluates `count` graphs; results written per graph.  Returns ODPX_*. */
int ODP_Set_aspl_batch(int count, const ODP_Graph *graphs, int *diameter, long *sum, double *ASPL);

/* Reusable batch plan (same shapes every run).  ODPX_Batch_run evaluates
 * adjacency[i] (int[n_i/s_i][d_i] each) for graph i and returns when the
 * results are written; the arrays are read during the call only. */
typedef struct odp_plan ODPX_Batch;
int  ODPX_Batch_create(int count, const ODP_Graph *graphs, ODPX_Batch **batch);
int  ODPX_Batch_run(ODPX_Batch *batch, const int *const *adjacency, int *diameter, long *sum, double *ASPL);
void ODPX_Batch_destroy(ODPX_Batch *batch);
/* Device time of the plan's GPU work in ms per run (CUDA events on the
 * plan's stream).  A non-NULL adjacency is handed over first; with NULL the
 * arrays of the previous run or timing call are read again, so they must
 * still be valid and unchanged (on devices that read host memory directly
 * the plan keeps only their addresses). */
int  ODPX_Batch_time(ODPX_Batch *batch, const int *const *adjacency, int repeats, float *ms_per_run);
/* mode 0: whole per-call sequence (upload, expand, engine, read back);
 * mode 1: engine on resident inputs.  flush_mb > 0 overwrites a buffer of
 * that size before each run, outside the timed interval. */
int  ODPX_Batch_time_mode(ODPX_Batch *batch, const int *const *adjacency, int repeats, int mode, int flush_mb,
                          float *ms_per_run);
unsigned long long ODPX_Batch_tiles(const ODPX_Batch *batch);
/* Introspection for benchmarks: jobs, slots, chunk width (log2 words) of graph i. */
int  ODPX_Batch_info(const ODPX_Batch *batch, int graph, int *njobs, int *nslots, int *wc_log2, int *tile_rows);
/* Which kernel evaluates the plan: 1 when every graph has at most
 * ODP_GB300_SMALL_N (default 8192) vertices, both bitset buffers of a column
 * chunk of at least 128 sources fit in one CTA's shared memory beside its
 * share of the row table, and the plan's CTAs fit on the SMs in one wave, so
 * each job runs in the small-graph kernel, on the CTAs
 * of one thread-block cluster; 0 for the persistent engine (larger or mixed
 * plans, explicit schedule settings, change tracking).  Results are the same
 * either way. */
int  ODPX_Batch_kernel(const ODPX_Batch *batch);
/* For a plan on the small-graph kernel: the CTAs of the thread-block cluster
 * that runs each job (1, 2, 4 or 8; each CTA computes its share of the
 * rows), the threads per CTA, and whether the bitsets are partitioned over
 * the cluster (1: each CTA holds its own rows and reads the others' from
 * their shared memory; 0: each CTA holds the whole level).  Returns 0, or
 * ODPX_ERR_INVALID for a plan on the persistent engine.
 * ODP_GB300_SMALL_CLUSTER forces the cluster size of plans created
 * afterwards (halved until the shape fits), ODP_GB300_SMALL_PART=0 or 1 the
 * layout. */
int  ODPX_Batch_small_shape(const ODPX_Batch *batch, int *cluster, int *threads, int *partitioned);
/* Level at which each job (graph x column chunk, plan order) of the last run
 * finished (negative: stalled, i.e. unreachable pairs).  Returns the job count. */
int  ODPX_Batch_job_levels(const ODPX_Batch *batch, int *levels, int max_jobs);
/* Per job of the last run (plan order): its graph and the device times (us,
 * from the start of the engine kernel) at which it was loaded into a slot
 * (0: before the launch) and finished.  Returns the job count.  After the
 * first run of a plan the jobs are ordered by their measured durations,
 * longest first (ODP_GB300_REORDER=0 keeps the first order). */
int  ODPX_Batch_job_profile(const ODPX_Batch *batch, int *graph, double *loaded_us, double *done_us, int max_jobs);
/* Time limit of the engine's idle waits (default 60 s); past it the run
 * stops with ODPX_ERR_TIMEOUT instead of waiting on. */
void ODPX_Batch_set_wait_limit(ODPX_Batch *batch, unsigned long long ns);
/* Algorithmic bytes of the last run (roofline numerator): sum over jobs of
 * levels x 8 x the chunk's source words x sum over the graph's vertices of
 * (degree + 2). */
double ODPX_Batch_bytes_alg(const ODPX_Batch *batch);
/* Read bandwidth (GB/s) of 16-byte L2-only loads streaming an L2-resident
 * buffer of `megabytes`, `reps` times: the L2 ceiling of the roofline. */
double ODPX_Measure_l2_read_gbs(int megabytes, int reps);

/* Tuning knobs for plans created after the call, batch plans and the
 * drop-in ODP_Init_aspl_* alike (0 = automatic; use_graph: -1 automatic,
 * 0 off, 1 on). */
void ODPX_Set_tuning(int wc_log2, int slots, int tile_rows, int l2_budget_mb, int local_kb, int use_graph);

/* Per-bucket tuning table consulted when plans are created (the autotuner
 * in odp_gb300/autotune.py fills it).  A graph matches an entry by
 * ceil(log2 n), degree class (ODPX_Degree_class) and grid flag; fields <= 0
 * keep the built-in choice.  ODPX_Set_tuning overrides take precedence. */
typedef struct {
  int n_log2, degree_class, grid;
  int wc_log2;               /* chunk width: 2^wc_log2 words, i.e. 2^wc_log2 / 2 lanes per row (<= 32) */
  int tile_kb;               /* traffic per row tile */
  int local_kb;              /* per-level traffic at or below which one CTA runs the whole job */
} ODPX_Tune_entry;
int ODPX_Set_tuning_table(const ODPX_Tune_entry *entries, int count);
int ODPX_Degree_class(int degree);

/* Drop-in introspection: the plan behind the current ODP_Init_aspl_* state. */
ODPX_Batch *ODPX_Current_plan(void);

/* Seeded generators on a private stream (bit-identical to ODP_Srand(seed)
 * followed by the ODP_Generate_* call). */
void ODPX_Generate_random_general_seeded(unsigned int seed, int nodes, int degree, int symmetries, int (*edge)[2]);
void ODPX_Generate_random_grid_seeded(unsigned int seed, int width, int height, int degree, int length,
                                      int symmetries, int (*edge)[2]);
/* Private random streams for per-chain 2-opt proposals. */
size_t ODPX_Rng_size(void);
void   ODPX_Rng_seed(void *rng_state, unsigned int seed);
int    ODPX_Rng_next(void *rng_state);
void   ODPX_Mutate_adjacency_general_s_rng(void *rng_state, int nodes, int degree, const int *num_degrees,
                                           int symmetries, ODP_Restore *r, int *adjacency);
/* ODP_Restore_adjacency_general with the graph's shape given explicitly. */
void   ODPX_Restore_adjacency_general_s(int nodes, int degree, int symmetries, ODP_Restore r, int *adjacency);
/* The same two for grids (ODP_Mutate_adjacency_grid_s, ODP_Restore_adjacency_grid). */
void   ODPX_Mutate_adjacency_grid_s_rng(void *rng_state, int width, int height, int degree, const int *num_degrees,
                                        int length, int symmetries, ODP_Restore *r, int *adjacency);
void   ODPX_Restore_adjacency_grid_s(int width, int height, int degree, int symmetries, ODP_Restore r, int *adjacency);

/* ODPX_Set_aspl_noalloc: no counterpart in the reference.  Evaluates one
 * regular general graph (the arguments of ODP_Init_aspl_general[_s] with
 * num_degrees == NULL, plus ODP_Set_aspl's host adjacency and outputs)
 * without allocating any memory, host or device: for callers that must not
 * allocate while they run, such as an annealing loop on a latency budget
 * (cudaMalloc and cudaFree synchronise the device and stall its other
 * streams) or a process whose device memory is already reserved by another
 * framework's pool allocator.  All working memory comes from one fixed
 * array of ODPX_NOALLOC_SCRATCH_BYTES in the library's device image, which
 * every GPU context that loads the library holds until the process exits.
 * Graphs whose working set does not fit are refused with ODPX_ERR_MEMORY
 * (a line on stderr says so); as a guide, n = 8192 with degree 32 fits, and
 * n = 262144 with degree 16 does not.  The first call on each device looks
 * up the array's device address, so make that first call before any stream
 * capture.  Every call uses the same array (each call rewrites the state it
 * needs): calls that overlap on the GPU, from several host threads, race.
 * Results equal ODP_Set_aspl's bit for bit.  Returns ODPX_*. */
#define ODPX_NOALLOC_SCRATCH_BYTES (16u << 20)
int ODPX_Set_aspl_noalloc(int nodes, int degree, int symmetries, const int *adjacency,
                          int *diameter, long *sum, double *ASPL);

/* ---- Serving: device-resident graphs, in-place 2-opt deltas, continuous
 * batching (ODPX_Serve_*).  No counterpart in the reference. ---- */

/* One compact-adjacency update, adjacency[row][slot] = value (row < n/s). */
typedef struct { int row, slot, value; } ODPX_Delta;

typedef struct {
  int lanes;                 /* concurrent batches on the GPU (streams); default 4 */
  int max_batch;             /* requests per batch; default 16 */
  int max_nodes;             /* largest graph admitted; sizes the bitset slots; default 32768 */
  int memory_mb;             /* device memory for bitset slots, all lanes; default 1024 */
  int wc_log2;               /* column chunk width, log2 of 64-bit words; default 4 */
} ODPX_Serve_config;

typedef struct {
  long long requests_done, batches, batched_requests;
  int max_batch, max_inflight_lanes, slots_per_lane, blocks_per_lane;
} ODPX_Serve_counters;

typedef struct odp_server ODPX_Server;
int  ODPX_Serve_create(const ODPX_Serve_config *config, ODPX_Server **server);
/* Uploads a graph (the adjacency stays on the GPU); *handle names it. */
int  ODPX_Serve_register(ODPX_Server *server, const ODP_Graph *graph, int *handle);
/* Queues an evaluation of graph `handle` after applying `ndelta` updates to
 * its resident adjacency (they persist).  Returns at once with a request id.
 * A delta must name a local row, a slot below that row's degree (its
 * num_degrees entry, when the graph has one) and a vertex in [0, n);
 * otherwise nothing is queued and ODPX_ERR_ADJACENCY is returned. */
int  ODPX_Serve_submit(ODPX_Server *server, int handle, int ndelta, const ODPX_Delta *deltas, long long *request);
/* Blocks until the request is done; latency_s = submit -> result. */
int  ODPX_Serve_wait(ODPX_Server *server, long long request, int *diameter, long *sum, double *ASPL,
                     double *latency_s);
/* ODPX_PENDING while the request runs, else as ODPX_Serve_wait. */
int  ODPX_Serve_poll(ODPX_Server *server, long long request, int *diameter, long *sum, double *ASPL,
                     double *latency_s);
int  ODPX_Serve_stats(ODPX_Server *server, ODPX_Serve_counters *stats);
/* Copies the graph's resident adjacency back to the host (checkpoint). */
int  ODPX_Serve_adjacency(ODPX_Server *server, int handle, int *adjacency);
void ODPX_Serve_destroy(ODPX_Server *server);

/* Library version string. */
/* ---- Annealing chains on the GPU ----
 * The reference runs its annealing loop on the host (sample/SA/general.c:
 * 160-191, general_s.c:170-191): Mutate, Set_aspl, accept_s, Restore when
 * rejected, temp *= cooling_rate.  ODPX_Anneal runs the same loop for many
 * chains at once with every step on the GPU: the 2-opt proposal (the
 * ODP_Mutate_adjacency_general_s rule, drawn from the chain's own stream, the
 * one ODP_Srand(seed) would give), the evaluation, the acceptance (accept_s:
 * one more draw from the stream when a move is worse at equal diameter) and
 * the undo.  A chain given the same seed and temperatures as the reference's
 * client makes the same moves, except that the acceptance uses the GPU's
 * exp(), which may differ from the host's in the last bit (a decision can
 * flip only when the uniform draw falls within that bit).  General(_s) and
 * grid(_s) graphs (sample/SA/grid.c, grid_s.c: ODP_Mutate_adjacency_grid_s
 * with its length limit). */
typedef struct {
  int nodes, degree, symmetries;
  const int *num_degrees;      /* per local row, or NULL (regular) */
  const int *adjacency;        /* int[nodes/symmetries][degree]: the starting graph */
  unsigned int seed;           /* the proposal stream, as ODP_Srand(seed) */
  double max_temp, min_temp;   /* temperature from max_temp towards min_temp ... */
  long long ncalcs;            /* ... over ncalcs steps: cooling = pow(min/max, 1/ncalcs) */
  int hill_climbing;           /* accept only ASPL <= current (the samples' -Y) */
  int aspl_priority;           /* compare ASPL before diameter (the samples' -A) */
  int grid;                    /* 1: a grid graph of width x height (nodes is ignored) ... */
  int width, height, length;   /* ... with edges at most `length` long (the grid samples' -L) */
} ODPX_Chain;

typedef struct {
  long long steps, accepted;
  int status;                  /* 0 running; 1 a proposal ran out of draws; 2 an evaluation failed */
  int diameter;                /* the current graph */
  long sum;
  double aspl;
  int best_diameter;           /* the best graph seen (diameter first, then ASPL) */
  long best_sum;
  double best_aspl;
  double temp;                 /* the next step's temperature */
} ODPX_Chain_state;

typedef struct odpx_anneal ODPX_Anneal;
/* Uploads and evaluates the starting graphs (the samples' first Set_aspl). */
int  ODPX_Anneal_create(const ODPX_Chain *chains, int count, ODPX_Anneal **anneal);
/* Runs `steps` steps of every chain; returns when they are done. */
int  ODPX_Anneal_run(ODPX_Anneal *anneal, int steps);
/* A chain's counters and results, and optionally its current and best
 * graphs (int[nodes/symmetries][degree] each; NULL to skip). */
int  ODPX_Anneal_state(ODPX_Anneal *anneal, int chain, ODPX_Chain_state *state, int *adjacency,
                       int *best_adjacency);
void ODPX_Anneal_destroy(ODPX_Anneal *anneal);

const char *ODPX_Version(void);

#ifdef __cplusplus
}
#endif
#endif

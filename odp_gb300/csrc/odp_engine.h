/*
 * odp_engine.h -- the thin C ABI between the host C driver (odp_aspl.c,
 * odp_batch.c, odp_serve.c) and the CUDA layer (aspl_engine.cu).
 * Plain pointers and sizes only; every device pointer here was allocated by
 * gbx_malloc.  All calls are asynchronous on the given stream unless named
 * *_sync.  Return values are cudaError_t codes (0 = success).
 */
#ifndef ODP_ENGINE_H
#define ODP_ENGINE_H
#include <stddef.h>
#include <stdint.h>
#include "odp.h"
#ifdef __cplusplus
extern "C" {
#endif

/* One graph whose compact adjacency is turned into a row-space neighbour
 * table nbr[n][dp]: row r lists the rows of r's neighbours, -1 padded. */
typedef struct {
  const int *adj;          /* int[n/s][d] as passed to ODP_Set_aspl: a device copy, or the caller's
                              host array itself when kernels can read pageable host memory */
  int *adj_dev;            /* NULL, or the device copy that gbx_pull fills from the host array `adj`
                              and that expand then reads */
  const int *ndeg;         /* device int[n] per-vertex degree, or NULL (regular) */
  const int *itable;       /* device int[n] vertex -> row (grid symmetry), or NULL */
  int *nbr;                /* device out int[n][dp] */
  int n, d, dp, s;
  int width, height;       /* grid symmetry only */
  int grid_s;              /* 1: rows are itable-permuted, grid rotation rules */
  int pad;
  long long first_vertex;  /* prefix of n over the descriptors before this one */
} gbx_expand_desc;

/* One (graph, column chunk) BFS job: sources [src0, src0 + nsrc). */
typedef struct {
  const int *nbr;          /* device int[n][dp]; an entry that is no neighbour holds the row itself */
  const int *srcpos;       /* device int[n]: row -> source ordinal (-1: not a source), or NULL: row itself */
  int n, dp;
  int wc_log2;             /* words (uint64) per row in this chunk = 1 << wc_log2, 1..7 */
  int src0, nsrc;          /* source ordinals [src0, src0 + nsrc) */
  int sym;                 /* symmetries: sums are scaled by it */
  int graph;               /* index into the graph accumulators */
  int tile_rows, ntiles;
  int flags;               /* GBX_JOB_ACTIVE: gather only words that changed at the previous level */
  int d;                   /* neighbour columns per row; [d, dp) is padding */
} gbx_job;

#define GBX_JOB_ACTIVE 1

/* Largest degree the engine takes: its row tables are staged in blocks of
 * a few thousand neighbour entries that must hold several rows; rows are at
 * most 512 entries (the degree rounded up to a multiple of 4). */
#define GBX_MAX_DEGREE 508

/* Shared memory a job of the small-graph kernel may use: its two bitset
 * buffers (2 x n x wc x 8 bytes) and its neighbour table (n x dp x 4). */
#define GBX_SMALL_SMEM_MAX (200 * 1024)
#define GBX_SMALL_CLUSTER_MAX 8   /* CTAs (one thread-block cluster) per small-kernel job */

/* Per-slot mutable state, two 128-byte lines each.  The slot holds a copy
 * of its job's descriptor, so a CTA that takes a tile reads everything it
 * needs from the slot's first 144 bytes in one round trip. */
typedef struct {
  unsigned long long ticket;   /* (ntiles << 32) | next tile */
  unsigned int done;           /* tiles finished at the current level */
  int job;                     /* job index */
  int level;                   /* BFS level being computed (>= 1) */
  int pad0;
  unsigned long long count;    /* bits set at this level (with change tracking after level 1: bits added) */
  unsigned long long prev;     /* bits set at the previous level */
  long long sum;               /* this job's share of the ordered distance sum */
  unsigned long long *buf0, *buf1;
  unsigned int *mask0, *mask1; /* per row: which lanes' words changed at a level */
  gbx_job desc;                /* jobs[job], written before the ticket that publishes it */
  unsigned long long pad1[14];
} gbx_slot;

#define GBX_SLOT_HEAD_BYTES 144  /* ticket .. desc: what a CTA taking a tile reads */
#ifdef __cplusplus
static_assert(sizeof(gbx_job) == 64 && sizeof(gbx_slot) == 256, "slot layout");
#else
_Static_assert(sizeof(gbx_job) == 64 && sizeof(gbx_slot) == 256, "slot layout");
#endif

typedef struct {
  unsigned int next_job;       /* next job index to load into a freed slot */
  unsigned int retired;        /* slots with no job left */
  unsigned int error;          /* GBX_ERR_* bits */
  unsigned int pad;
  unsigned long long tiles;    /* tiles processed */
  unsigned long long t_start;  /* %globaltimer when CTA 0 started */
  unsigned long long pad1[4];  /* 64 bytes */
} gbx_ctrl;

typedef struct {
  unsigned long long sum;      /* ordered distance sum (before halving) */
  int levels;                  /* max over chunks of the level that completed */
  int flags;                   /* 1: some chunk stalled (disconnected) */
} gbx_graph_acc;

/* Per-job outcome: the level at which the job finished (negative: it
 * stalled) and %globaltimer stamps of when it was loaded into a slot (0 for
 * jobs loaded by the host before the launch) and when it finished. */
typedef struct {
  int level;
  int pad;
  unsigned long long t_loaded, t_done;
} gbx_job_out;

/* One int write into device memory (served-graph updates). */
typedef struct {
  int *at;
  int value;
  int pad;
} gbx_write;

#define GBX_ERR_BAD_ADJ   1u   /* adjacency entry outside [0, n) */
#define GBX_ERR_TIMEOUT   2u   /* an idle wait exceeded its time limit */

/* Device / memory / stream plumbing. */
int  gbx_device_init(int *sm_count);
int  gbx_malloc(void **p, size_t bytes);
int  gbx_free(void *p);
int  gbx_host_alloc(void **p, size_t bytes);
int  gbx_host_free(void *p);
int  gbx_stream_create(void **stream);
int  gbx_stream_destroy(void *stream);
int  gbx_memcpy_h2d(void *dst, const void *src, size_t bytes, void *stream);
int  gbx_memcpy_d2h(void *dst, const void *src, size_t bytes, void *stream);
int  gbx_memcpy_d2d(void *dst, const void *src, size_t bytes, void *stream);
int  gbx_memset(void *dst, int value, size_t bytes, void *stream);
int  gbx_stream_sync(void *stream);
const char *gbx_error_string(int err);

/* Kernels. */
int  gbx_expand(const gbx_expand_desc *d_descs, int ndesc, long long total_vertices, int max_dp,
                unsigned int *d_error, void *stream);
/* Persistent grid size (SMs x resident CTAs) for the launch's staging size
 * (active nonzero: some job tracks changes). */
int  gbx_engine_blocks(int active);
/* 1 when kernels can read pageable host memory directly (after gbx_device_init). */
int  gbx_pageable_access(void);
/* Streaming read bandwidth of an L2-resident buffer of `bytes` (GB/s). */
int  gbx_l2_read_probe(size_t bytes, int reps, double *gbs);
/* The persistent engine over jobs [0, njobs).  active: 0 when no job
 * tracks changes, 1 when every job does, 2 when some do (each launches an
 * engine built for exactly those passes). */
int  gbx_engine_launch(const gbx_job *d_jobs, int njobs, gbx_slot *d_slots, int nslots,
                       gbx_ctrl *d_ctrl, gbx_graph_acc *d_acc, gbx_job_out *d_job_out,
                       unsigned long long spin_limit_ns, int blocks, int active, void *stream);

/* Copies every descriptor's host array `adj` into its `adj_dev` with
 * coalesced 16-byte loads over the CPU-GPU link (pageable host memory).  The
 * descriptors are read from pinned host memory (`h_descs`, a device address)
 * and stored into `d_descs` for gbx_expand; the same launch copies the
 * initial engine state `d_state_init` over `d_state` (state_bytes, a multiple
 * of 8), so a call needs no separate uploads for either. */
int  gbx_pull(const gbx_expand_desc *h_descs, gbx_expand_desc *d_descs, int ndesc, void *d_state,
              const void *d_state_init, size_t state_bytes, void *stream);
/* Outcome of one job of the small-graph kernel, written to pinned host
 * memory: its last level (negative: stalled), error bits (GBX_ERR_*), its
 * share of the graph's ordered distance sum, and %globaltimer stamps. */
typedef struct {
  int level;
  unsigned int err;
  long long sum;
  unsigned long long t_loaded, t_done;
} gbx_small_rec;

/* Jobs [0, njobs) of d_jobs, one thread-block cluster of `cluster` CTAs
 * (1, 2, 4 or 8) of `threads` threads each per job, every level in shared
 * memory (smem_bytes per CTA, at most GBX_SMALL_SMEM_MAX: both bitset
 * buffers of the job and the row table of the CTA's 1/cluster of the rows).
 * The CTAs read their graph's descriptor descs[job.graph] and the compact
 * adjacency it names (`adj`) from host memory and build the row tables in
 * shared memory; the job's record goes to rec[job].  `descs` and `rec` are
 * device addresses of pinned host memory (gbx_host_device_ptr).  With
 * `descs` NULL every job belongs to graph 0, whose descriptor `*desc0` is
 * passed by value in the launch's parameters (no host-memory read for it).
 * With `part` set each CTA holds only its own rows of the bitset buffers
 * (1/cluster of them) and gathers the others' rows from their shared memory. */
int  gbx_small_launch(const gbx_job *d_jobs, int njobs, const gbx_expand_desc *descs, const gbx_expand_desc *desc0,
                      gbx_small_rec *rec, size_t smem_bytes, int cluster, int threads, int part, void *stream);
/* How many clusters of that shape the GPU holds at once (0: the shape does
 * not fit; then it cannot be launched). */
int  gbx_small_clusters(int cluster, int threads, size_t smem_bytes, int *active);
/* Device address of pinned host memory. */
int  gbx_host_device_ptr(void *host, void **dev);
/* Allows the small-graph kernel GBX_SMALL_SMEM_MAX bytes of shared memory
 * (once per process; call before the first launch or capture). */
int  gbx_small_prepare(void);

/* Applies `count` writes, in stream order. */
int  gbx_scatter(const gbx_write *d_writes, int count, void *stream);
int  gbx_event_query(void *ev);        /* 0: complete, 1: not yet, else an error */

/* CUDA graphs: capture everything issued on `stream` between begin and end. */
int  gbx_capture_begin(void *stream);
int  gbx_capture_end(void *stream, void **graph_exec);
int  gbx_graph_launch(void *graph_exec, void *stream);
int  gbx_graph_destroy(void *graph_exec);

/* Timing with CUDA events on a stream. */
int  gbx_event_create(void **ev);
int  gbx_event_destroy(void *ev);
int  gbx_event_record(void *ev, void *stream);
int  gbx_event_elapsed_ms(void *start, void *stop, float *ms);

/* One simulated-annealing chain on a general(_s) graph, resident on the
 * device (anneal.cu).  Its graph is evaluated by the engine as graph `graph`
 * of a plan whose tables `adj` and `nbr` point into. */
typedef struct {
  int n, d, dp, s, base, graph;
  int grid, width, height, len;  /* grid chains: vertex x*height + y, edges up to len long */
  const int *itable;           /* grid symmetry: vertex -> neighbour-table row, else NULL */
  int *adj;                    /* compact int[base][d] */
  int *nbr;                    /* neighbour table int[n][dp] */
  const int *ndeg;             /* degree per base row, or NULL (regular) */
  int *best_adj;               /* int[base][d]: the best graph seen */
  unsigned int ring[31];       /* proposal stream: the last 31 words of glibc's TYPE_3 recurrence, */
  int ring_pos;                /*   ring[ring_pos] the oldest */
  int status;                  /* 0 running, else GBX_CHAIN_ERR_* (the chain stops) */
  ODP_Restore last;            /* the last swap, for its undo */
  int cur_diameter, best_diameter;
  long long cur_sum, best_sum;
  double cur_aspl, best_aspl;
  double temp, cooling;        /* temp *= cooling after every step */
  long long steps, accepted;
  int hill_climbing, aspl_priority;
} gbx_chain;

#define GBX_CHAIN_ERR_SWAP 1   /* a proposal found no back slot or ran out of draws */
#define GBX_CHAIN_ERR_EVAL 2   /* an evaluation reported an error (bad adjacency, timeout) */

/* One proposal per running chain: a 2-opt swap applied to adj and nbr. */
int  gbx_anneal_propose(gbx_chain *d_chains, int count, void *stream);
/* One decision per running chain from its evaluation: best tracking (copying
 * adj to best_adj), acceptance, the undo of a rejected swap, cooling. */
int  gbx_anneal_decide(gbx_chain *d_chains, int count, const gbx_graph_acc *d_acc, const gbx_ctrl *d_ctrl,
                       const unsigned int *d_err, void *stream);

#ifdef __cplusplus
}
#endif
#endif

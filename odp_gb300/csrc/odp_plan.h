/*
 * odp_plan.h -- execution plans for ASPL evaluation on the GPU.
 *
 * A plan holds everything needed to evaluate a fixed list of graph shapes
 * (one graph for ODP_Set_aspl, many for ODP_Set_aspl_batch): packed device
 * copies of the adjacency / degree / row tables, the neighbour tables, the
 * job list (graph x column chunk), the slot bitset buffers and a CUDA graph
 * that replays [upload, expand, reset state, engine, read back] per call.
 */
#ifndef ODP_PLAN_H
#define ODP_PLAN_H
#include <stddef.h>
#include "odp_engine.h"

typedef struct {
  int grid;                    /* 0 general, 1 grid */
  int nodes;                   /* general: n; grid: ignored */
  int width, height;           /* grid only */
  int degree, symmetries;
  const int *num_degrees;      /* as given to ODP_Init_aspl_* (NULL: regular) */
} odp_shape;

typedef struct {
  int wc_log2;                 /* chunk width, log2 of uint64 words; 0 = automatic */
  int slots;                   /* concurrently active jobs; 0 = automatic */
  int tile_rows;               /* rows per tile; 0 = automatic */
  int l2_budget_mb;            /* bitset working set to keep under (L2 residency) */
  int local_kb;                /* per-level traffic at or below which a job runs in one CTA */
  int use_graph;               /* replay through a CUDA graph */
  int blocks;                  /* persistent grid size; 0 = SMs x occupancy */
  int activity;                /* change tracking: -2 automatic (default), 0 never, 1 always, -1 grids only */
  int local_kb_explicit;       /* local_kb was set by the caller: the tuning table does not override it */
  int reorder;                 /* after the first run, order jobs by their measured duration (1, default) */
  int direct;                  /* pull callers' adjacency from host memory when the device can (1, default) */
  int small_n;                 /* graphs of at most this many vertices may run in shared memory (0: never) */
  int small_cluster;           /* CTAs per small-kernel job: 1, 2, 4 or 8; 0 = automatic */
  int small_part;              /* small-kernel rows partitioned over the cluster: -1 when needed, 0 never, 1 always */
} odp_tuning;

typedef struct {
  int grid, n, d, dp, s, grid_s, width, height;
  int B, W;                    /* sources (n/s) and uint64 words per full row */
  int wc_log2, nchunks, tile_rows, ntiles;
  size_t adj_off, ndeg_off, itable_off, nbr_off, srcpos_off;   /* int offsets into packed arrays */
  size_t adj_ints;
  int has_ndeg, has_itable, has_srcpos;
  double row_reads;            /* sum over vertices of (degree + 2): rows touched per row per level */
} odp_plan_graph;

typedef struct odp_plan {
  int ngraphs, njobs, nslots;
  odp_plan_graph *g;
  odp_tuning tuning;
  size_t adj_ints, ndeg_ints, itable_ints, nbr_ints, srcpos_ints, slot_words, slot_rows;
  long long total_vertices;
  /* device */
  int *d_adj, *d_ndeg, *d_itable, *d_nbr, *d_srcpos;
  unsigned long long *d_slotbuf;
  unsigned int *d_slotmask;
  gbx_expand_desc *d_expand;
  gbx_job *d_jobs;
  char *d_state;               /* slots | ctrl | error | accumulators */
  /* host (pinned) */
  int *h_adj;
  char *h_state_init, *h_state_out;
  size_t state_bytes, out_off, out_bytes;
  size_t acc_off, levels_off;    /* offsets of the accumulators / per-job levels in the state */
  gbx_job *h_jobs;
  void *stream, *graph_exec;
  unsigned long long spin_limit_ns;
  int blocks;
  int any_active;              /* some job tracks changes: launch with the full staging area */
  int some_plain;              /* some job does not (with any_active: the engine built for both) */
  double bytes_alg_last;       /* algorithmic bytes of the last run (roofline) */
  int reordered;               /* the job order was learned from a run */
  int direct;                  /* the device pulls the callers' arrays (h_expand holds their pointers) */
  gbx_expand_desc *h_expand;   /* pinned copy of the expand descriptors (direct plans) */
  int small;                   /* every job runs in the small-graph kernel, in shared memory */
  size_t small_smem;           /* shared memory per CTA of the small-graph kernel */
  int small_cluster;           /* CTAs (one thread-block cluster) per job of the small-graph kernel */
  int small_threads;           /* threads per CTA of the small-graph kernel */
  int small_part;              /* 1: each CTA holds only its rows of the bitsets (partitioned layout) */
  int max_dp;                  /* widest neighbour-table row of the plan */
  gbx_expand_desc *d_hexpand;  /* device address of h_expand (direct engine plans) */
  char *d_state_init;          /* device copy of h_state_init (direct engine plans) */
  gbx_small_rec *h_small_rec;  /* small plans: per-job records, pinned; the kernel writes them */
  gbx_small_rec *d_small_rec;  /*   the same memory, as the device addresses it */
  gbx_expand_desc *d_small_desc; /* small plans: h_expand as the device addresses it */
} odp_plan;

typedef struct {
  int diameter;
  long sum;
  double aspl;
} odp_result;

void odp_tuning_defaults(odp_tuning *t, int batch);
/* The defaults for `count` graphs with the ODPX_Set_tuning overrides applied. */
void odp_tuning_for(int count, odp_tuning *t);
/* Returns 0 on success, else an ODPX_ERR_* code (include/odp_gb300.h). */
int  odp_plan_create(const odp_shape *shapes, int count, const odp_tuning *tuning, odp_plan **out);
void odp_plan_destroy(odp_plan *p);
/* adjacency[i] = host int[n_i/s_i][d_i]; results per graph. */
int  odp_plan_run(odp_plan *p, const int *const *adjacency, odp_result *results);
/* Split form used for timing: stage copies host adjacency into the pinned
 * buffer, launch enqueues the GPU work, finish waits and decodes. */
void odp_plan_stage(odp_plan *p, const int *const *adjacency);
int  odp_plan_launch(odp_plan *p);
int  odp_plan_finish(odp_plan *p, odp_result *results);
/* Last run's device counters. */
unsigned long long odp_plan_tiles(const odp_plan *p);
unsigned int odp_plan_error(const odp_plan *p);
/* Outcome of each job (plan order): level (negative if it stalled) and
 * device timestamps of its load and finish. */
const gbx_job_out *odp_plan_job_out(const odp_plan *p);
int odp_plan_enqueue_engine(odp_plan *p);
/* Algorithmic bytes of the last run: sum over jobs of |level| x 8 x the
 * chunk's source words (ceil(nsrc / 64)) x row_reads of the job's graph. */
double odp_plan_bytes_alg(const odp_plan *p);

/* Device bring-up shared by every entry point; exits through ODP_FAIL-like
 * reporting on failure when `fatal`. */
int odp_device_ready(void);

#endif

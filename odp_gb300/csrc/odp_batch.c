/*
 * odp_batch.c -- ODP_Set_aspl_batch and the ODPX_Batch_* plan API: many
 * graphs of uneven size, degree and symmetry evaluated in one persistent
 * engine launch.  Each graph's results are bit-identical to evaluating it
 * alone through ODP_Init_aspl_* + ODP_Set_aspl.  No counterpart in the
 * reference, whose clients evaluate one graph per call.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "odp_plan.h"
#include "odp_gb300.h"

static odp_tuning g_override;
static int g_override_set = 0;

void ODPX_Set_tuning(int wc_log2, int slots, int tile_rows, int l2_budget_mb, int local_kb, int use_graph)
{
  g_override.wc_log2 = wc_log2;
  g_override.slots = slots;
  g_override.tile_rows = tile_rows;
  g_override.l2_budget_mb = l2_budget_mb;
  g_override.local_kb = local_kb;
  g_override.use_graph = use_graph;
  g_override_set = 1;
}

/* Plan tuning for `count` graphs: the defaults, then the ODPX_Set_tuning
 * overrides.  The drop-in ODP_Init_aspl_* plans use it too. */
void odp_tuning_for(int count, odp_tuning *t)
{
  odp_tuning_defaults(t, count > 1);
  if(!g_override_set) return;
  if(g_override.wc_log2 > 0) t->wc_log2 = g_override.wc_log2;
  if(g_override.slots > 0) t->slots = g_override.slots;
  if(g_override.tile_rows > 0) t->tile_rows = g_override.tile_rows;
  if(g_override.l2_budget_mb > 0) t->l2_budget_mb = g_override.l2_budget_mb;
  if(g_override.local_kb > 0){ t->local_kb = g_override.local_kb; t->local_kb_explicit = 1; }
  if(g_override.use_graph >= 0) t->use_graph = g_override.use_graph;
}

/* A grid with symmetries other than 2 and 4 follows the general rule, as
 * ODP_Init_aspl_grid_s does. */
static void to_shape(const ODP_Graph *g, odp_shape *sh)
{
  sh->grid = g->grid;
  sh->nodes = g->grid ? g->width * g->height : g->nodes;
  sh->width = g->width;
  sh->height = g->height;
  sh->degree = g->degree;
  sh->symmetries = g->symmetries;
  sh->num_degrees = g->num_degrees;
  if(g->grid && g->symmetries != 1 && g->symmetries != 2 && g->symmetries != 4) sh->grid = 0;
}

int ODPX_Batch_create(int count, const ODP_Graph *graphs, ODPX_Batch **batch)
{
  if(count <= 0 || !graphs || !batch) return ODPX_ERR_INVALID;
  odp_shape *sh = malloc(sizeof(odp_shape) * (size_t)count);
  for(int i = 0; i < count; i++) to_shape(&graphs[i], &sh[i]);
  odp_tuning t;
  odp_tuning_for(count, &t);
  int rc = odp_plan_create(sh, count, &t, batch);
  free(sh);
  return rc;
}

void ODPX_Batch_destroy(ODPX_Batch *batch) { odp_plan_destroy(batch); }

static void store_results(const odp_result *r, int count, int *diameter, long *sum, double *ASPL)
{
  for(int i = 0; i < count; i++){
    diameter[i] = r[i].diameter;
    sum[i] = r[i].sum;
    ASPL[i] = r[i].aspl;
  }
}

int ODPX_Batch_run(ODPX_Batch *batch, const int *const *adjacency, int *diameter, long *sum, double *ASPL)
{
  if(!batch) return ODPX_ERR_STATE;
  odp_result *r = malloc(sizeof(odp_result) * (size_t)batch->ngraphs);
  int rc = odp_plan_run(batch, adjacency, r);
  if(!rc) store_results(r, batch->ngraphs, diameter, sum, ASPL);
  free(r);
  return rc;
}

unsigned long long ODPX_Batch_tiles(const ODPX_Batch *batch) { return batch ? odp_plan_tiles(batch) : 0; }

int ODPX_Batch_info(const ODPX_Batch *batch, int graph, int *njobs, int *nslots, int *wc_log2, int *tile_rows)
{
  if(!batch || graph < 0 || graph >= batch->ngraphs) return ODPX_ERR_INVALID;
  if(njobs) *njobs = batch->njobs;
  if(nslots) *nslots = batch->nslots;
  if(wc_log2) *wc_log2 = batch->g[graph].wc_log2;
  if(tile_rows) *tile_rows = batch->g[graph].tile_rows;
  return 0;
}

int ODPX_Batch_kernel(const ODPX_Batch *batch) { return batch ? batch->small : ODPX_ERR_INVALID; }

int ODPX_Batch_small_shape(const ODPX_Batch *batch, int *cluster, int *threads, int *partitioned)
{
  if(!batch || !batch->small) return ODPX_ERR_INVALID;
  if(cluster) *cluster = batch->small_cluster;
  if(threads) *threads = batch->small_threads;
  if(partitioned) *partitioned = batch->small_part;
  return 0;
}

/* ODP_Set_aspl_batch keeps the last plan and reuses it (and its CUDA graph)
 * while the shapes and degree tables stay the same. */
static struct {
  ODPX_Batch *plan;
  int count;
  ODP_Graph *shapes;
  int **degrees;
} g_cache;

static void cache_clear(void)
{
  if(g_cache.plan) odp_plan_destroy(g_cache.plan);
  for(int i = 0; i < g_cache.count; i++) free(g_cache.degrees[i]);
  free(g_cache.degrees);
  free(g_cache.shapes);
  memset(&g_cache, 0, sizeof(g_cache));
}

static size_t degree_entries(const ODP_Graph *g)
{
  int n = g->grid ? g->width * g->height : g->nodes;
  return (size_t)(n / (g->symmetries > 0 ? g->symmetries : 1));
}

static int cache_matches(int count, const ODP_Graph *graphs)
{
  if(!g_cache.plan || g_cache.count != count) return 0;
  for(int i = 0; i < count; i++){
    const ODP_Graph *a = &g_cache.shapes[i], *b = &graphs[i];
    if(a->grid != b->grid || a->nodes != b->nodes || a->width != b->width || a->height != b->height ||
       a->degree != b->degree || a->symmetries != b->symmetries) return 0;
    if((g_cache.degrees[i] == NULL) != (b->num_degrees == NULL)) return 0;
    if(b->num_degrees && memcmp(g_cache.degrees[i], b->num_degrees, sizeof(int) * degree_entries(b))) return 0;
  }
  return 1;
}

int ODP_Set_aspl_batch(int count, const ODP_Graph *graphs, int *diameter, long *sum, double *ASPL)
{
  if(count <= 0 || !graphs) return ODPX_ERR_INVALID;
  if(!cache_matches(count, graphs)){
    cache_clear();
    ODPX_Batch *b = NULL;
    int rc = ODPX_Batch_create(count, graphs, &b);
    if(rc) return rc;
    g_cache.plan = b;
    g_cache.count = count;
    g_cache.shapes = malloc(sizeof(ODP_Graph) * (size_t)count);
    memcpy(g_cache.shapes, graphs, sizeof(ODP_Graph) * (size_t)count);
    g_cache.degrees = calloc((size_t)count, sizeof(int *));
    for(int i = 0; i < count; i++){
      g_cache.shapes[i].adjacency = NULL;
      if(graphs[i].num_degrees){
        size_t k = degree_entries(&graphs[i]);
        g_cache.degrees[i] = malloc(sizeof(int) * k);
        memcpy(g_cache.degrees[i], graphs[i].num_degrees, sizeof(int) * k);
      }
    }
  }
  const int **adj = malloc(sizeof(int *) * (size_t)count);
  for(int i = 0; i < count; i++) adj[i] = graphs[i].adjacency;
  int rc = ODPX_Batch_run(g_cache.plan, adj, diameter, sum, ASPL);
  free(adj);
  return rc;
}

/* Device time per run of the plan's GPU work, averaged over `repeats` runs
 * timed with CUDA events on the plan's stream.  mode 0: the whole per-call
 * sequence (adjacency upload, expand, engine, read back); mode 1: the engine
 * alone on resident inputs (state reset + engine kernel).  When flush_mb > 0
 * a buffer of that size is overwritten before every run, outside the timed
 * interval, so no run starts with the previous run's data in L2. */
static void *g_flush = NULL;
static size_t g_flush_bytes = 0;

int ODPX_Batch_time_mode(ODPX_Batch *p, const int *const *adjacency, int repeats, int mode, int flush_mb,
                         float *ms_per_run)
{
  if(!p || repeats <= 0) return ODPX_ERR_INVALID;
  if(adjacency) odp_plan_stage(p, adjacency);
  odp_result *tmp = malloc(sizeof(odp_result) * (size_t)p->ngraphs);
  int rc = odp_plan_launch(p);                 /* warm: builds the CUDA graph, expands tables */
  if(!rc) rc = odp_plan_finish(p, tmp);
  free(tmp);
  if(rc) return rc;
  size_t fb = (size_t)(flush_mb > 0 ? flush_mb : 0) << 20;
  if(fb > g_flush_bytes){
    if(g_flush) gbx_free(g_flush);
    g_flush = NULL; g_flush_bytes = 0;
    if(gbx_malloc(&g_flush, fb)) return ODPX_ERR_CUDA;
    g_flush_bytes = fb;
  }
  void **ev = malloc(sizeof(void *) * 2 * (size_t)repeats);
  for(int i = 0; i < 2 * repeats; i++) gbx_event_create(&ev[i]);
  for(int r = 0; r < repeats && !rc; r++){
    if(fb) gbx_memset(g_flush, r & 0xff, fb, p->stream);
    gbx_event_record(ev[2 * r], p->stream);
    if(mode == 0 || p->small) rc = odp_plan_launch(p);   /* a small plan's call is its one kernel */
    else{
      if(gbx_memcpy_h2d(p->d_state, p->h_state_init, p->state_bytes, p->stream)) rc = ODPX_ERR_CUDA;
      else if(odp_plan_enqueue_engine(p)) rc = ODPX_ERR_CUDA;
      else if(gbx_memcpy_d2h(p->h_state_out, p->d_state + p->out_off, p->out_bytes, p->stream)) rc = ODPX_ERR_CUDA;
    }
    gbx_event_record(ev[2 * r + 1], p->stream);
  }
  if(gbx_stream_sync(p->stream)) rc = ODPX_ERR_CUDA;
  double total = 0;
  for(int r = 0; r < repeats && !rc; r++){
    float ms = 0;
    if(gbx_event_elapsed_ms(ev[2 * r], ev[2 * r + 1], &ms)) rc = ODPX_ERR_CUDA;
    total += ms;
  }
  for(int i = 0; i < 2 * repeats; i++) gbx_event_destroy(ev[i]);
  free(ev);
  if(!rc && (odp_plan_error(p) & GBX_ERR_TIMEOUT)) rc = ODPX_ERR_TIMEOUT;
  *ms_per_run = (float)(total / repeats);
  return rc;
}

int ODPX_Batch_time(ODPX_Batch *batch, const int *const *adjacency, int repeats, float *ms_per_run)
{
  return ODPX_Batch_time_mode(batch, adjacency, repeats, 1, 0, ms_per_run);
}

int ODPX_Batch_job_levels(const ODPX_Batch *batch, int *levels, int max_jobs)
{
  if(!batch) return ODPX_ERR_STATE;
  const gbx_job_out *jo = odp_plan_job_out(batch);
  int n = batch->njobs < max_jobs ? batch->njobs : max_jobs;
  for(int i = 0; i < n; i++) levels[i] = jo[i].level;
  return batch->njobs;
}

int ODPX_Batch_job_profile(const ODPX_Batch *batch, int *graph, double *loaded_us, double *done_us, int max_jobs)
{
  if(!batch) return ODPX_ERR_STATE;
  const gbx_job_out *jo = odp_plan_job_out(batch);
  int n = batch->njobs < max_jobs ? batch->njobs : max_jobs;
  /* time origin: the engine's start, or the earliest stamp (the small-graph
   * kernel does not set the engine's) */
  unsigned long long t0 = ((const gbx_ctrl *)batch->h_state_out)->t_start;
  if(t0 == 0) t0 = ~0ull;
  for(int i = 0; i < batch->njobs; i++){
    if(jo[i].t_loaded && jo[i].t_loaded < t0) t0 = jo[i].t_loaded;
    if(jo[i].t_done && jo[i].t_done < t0) t0 = jo[i].t_done;
  }
  if(t0 == ~0ull) t0 = 0;
  for(int i = 0; i < n; i++){
    if(graph) graph[i] = batch->h_jobs[i].graph;
    loaded_us[i] = jo[i].t_loaded ? (double)(jo[i].t_loaded - t0) * 1e-3 : 0.0;
    done_us[i] = (double)(jo[i].t_done - t0) * 1e-3;
  }
  return batch->njobs;
}

void ODPX_Batch_set_wait_limit(ODPX_Batch *batch, unsigned long long ns)
{
  if(!batch || batch->spin_limit_ns == ns) return;
  batch->spin_limit_ns = ns;
  /* the limit is an argument of the captured engine launch: capture anew */
  if(batch->graph_exec){
    gbx_stream_sync(batch->stream);
    gbx_graph_destroy(batch->graph_exec);
    batch->graph_exec = NULL;
  }
}

double ODPX_Batch_bytes_alg(const ODPX_Batch *batch) { return batch ? odp_plan_bytes_alg(batch) : 0.0; }

double ODPX_Measure_l2_read_gbs(int megabytes, int reps)
{
  double gbs = 0;
  if(odp_device_ready()) return -1.0;
  if(gbx_l2_read_probe((size_t)megabytes << 20, reps, &gbs)) return -1.0;
  return gbs;
}

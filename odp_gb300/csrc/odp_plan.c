/*
 * odp_plan.c -- builds and runs execution plans (odp_plan.h) on the CUDA
 * layer.  This is the host runtime of the library: it sizes column chunks so
 * the live bitsets stay in L2, orders jobs, lays out device memory, and
 * replays one CUDA graph per evaluation so a call costs one host->device
 * copy, two kernels and one small device->host copy, with no host round trip
 * per BFS level (the reference does one per level, aspl_cuda.cu:62-82).
 *
 * Result semantics follow the reference exactly (aspl_cuda.cu:84-85,
 * 121-125, 256-260): the ordered sum is accumulated in 64-bit integers,
 * ASPL = sum / ((double)n - 1) / n computed as sum / (((double)n-1)*n), the
 * returned sum is (long)(sum / 2.0), the diameter is the largest level at
 * which a chunk became complete, and a graph with unreachable pairs returns
 * INT_MAX / LONG_MAX / DBL_MAX.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#include <float.h>
#include <pthread.h>
#include <unistd.h>
#include "odp_plan.h"
#include "odp_gb300.h"

#define ALIGN_UP(x, a) ((((x) + (a) - 1) / (a)) * (a))

static int g_device_ready = 0, g_sm_count = 0;

int odp_device_ready(void)
{
  if(g_device_ready) return 0;
  int e = gbx_device_init(&g_sm_count);
  if(e) return e;
  g_device_ready = 1;
  return 0;
}

static int env_int(const char *name, int fallback)
{
  const char *v = getenv(name);
  return (v && *v) ? atoi(v) : fallback;
}

void odp_tuning_defaults(odp_tuning *t, int batch)
{
  t->wc_log2 = env_int("ODP_GB300_WC_LOG2", 0);
  t->slots = env_int("ODP_GB300_SLOTS", 0);
  t->tile_rows = env_int("ODP_GB300_TILE_ROWS", 0);
  t->l2_budget_mb = env_int("ODP_GB300_L2_MB", 80);
  t->local_kb = env_int("ODP_GB300_LOCAL_KB", batch ? 2048 : 96);
  t->use_graph = env_int("ODP_GB300_GRAPH", 1);
  t->blocks = env_int("ODP_GB300_BLOCKS", 0);
  t->activity = env_int("ODP_GB300_ACTIVITY", -2);
  t->local_kb_explicit = getenv("ODP_GB300_LOCAL_KB") != NULL;
  t->reorder = env_int("ODP_GB300_REORDER", 1);
  t->direct = env_int("ODP_GB300_DIRECT", 1);
  t->small_n = env_int("ODP_GB300_SMALL_N", 8192);
  t->small_cluster = env_int("ODP_GB300_SMALL_CLUSTER", 0);
  t->small_part = env_int("ODP_GB300_SMALL_PART", -1);
}

/* Chunk width (log2 words) for a graph whose whole level runs in shared
 * memory on a cluster of `cluster` CTAs: the widest of at most 16 words, and
 * at most the graph's own width, whose two bitset buffers (whole in every
 * CTA, or with `part` only the CTA's rows) and row table (1/cluster of the
 * rows per CTA) fit; 0 if none does. */
static int small_wc_log2(int n, int dp, int full_l2, int cluster, int part)
{
  const size_t rows = (size_t)(n + cluster - 1) / (size_t)cluster;
  const size_t buf_rows = part ? rows : (size_t)n;
  for(int wl = full_l2 < 4 ? full_l2 : 4; wl >= 1; wl--){
    size_t bytes = 2 * buf_rows * ((size_t)8 << wl) + rows * (size_t)dp * 4;
    if(bytes <= GBX_SMALL_SMEM_MAX) return wl;
  }
  return 0;
}

/* Shared memory per CTA of the small kernel when `cluster` CTAs share a job:
 * both bitset buffers (whole, or with `part` the CTA's 1/cluster of the
 * rows) and the row table of 1/cluster of the rows. */
static size_t small_bytes(int n, int dp, int wl, int cluster, int part)
{
  const size_t rows = (size_t)(n + cluster - 1) / (size_t)cluster;
  return 2 * (part ? rows : (size_t)n) * ((size_t)8 << wl) + rows * (size_t)dp * 4;
}

/* Threads per CTA for a CTA's rows: one lane per 16 bytes of a row (at most
 * a warp per row), rounded up to whole warps, 64 to 512. */
static int small_threads_for(int n, int wl, int cluster)
{
  const int rows = (n + cluster - 1) / cluster;
  const int lanes = (1 << wl) / 2 < 32 ? (1 << wl) / 2 : 32;
  long long t = ((long long)rows * lanes + 31) / 32 * 32;
  if(t < 64) t = 64;
  if(t > 512) t = 512;
  return (int)t;
}

static int ilog2_ceil(long long x)
{
  int l = 0;
  while((1LL << l) < x) l++;
  return l;
}

/* Rows one CTA pass covers for a chunk of 2^wl words (see RowShape in the .cu). */
static int rows_per_pass(int wl)
{
  int vpr = (1 << wl) / 2;
  int g = vpr < 32 ? vpr : 32;
  return 8 * (32 / g);
}

static int validate_shape(const odp_shape *sh)
{
  int n = sh->grid ? sh->width * sh->height : sh->nodes;
  if(n <= 0 || sh->degree < 0 || sh->degree > GBX_MAX_DEGREE || sh->symmetries <= 0) return ODPX_ERR_INVALID;
  if(n % sh->symmetries != 0) return ODPX_ERR_INVALID;
  if(sh->grid && sh->symmetries != 1){
    int s = sh->symmetries, w = sh->width, h = sh->height;
    if(s != 2 && s != 4) return ODPX_ERR_INVALID;
    if(s == 2 && w % 2 != 0) return ODPX_ERR_INVALID;
    if(s == 4 && (w % 2 != 0 || h % 2 != 0 || w != h)) return ODPX_ERR_INVALID;
  }
  return 0;
}

/* ODP_ROTATE (reference utils.c:67-88) on the host, for row tables. */
static int rotate_host(int v, int width, int height, int s, int deg)
{
  int x = v / height, y = v % height;
  if(s == 2) return (width - x - 1) * height + (height - y - 1);
  if(deg == 90)  return y * height + (height - x - 1);
  if(deg == 180) return (height - x - 1) * height + (height - y - 1);
  return (height - y - 1) * height + x;
}

/* Vertex -> row table of a rotation-symmetric grid (ODP_Create_itable, utils.c:2103-2124). */
static void fill_itable(int width, int height, int s, int *itable)
{
  int base = (width * height) / s;
  if(s == 2){
    for(int i = 0; i < base; i++){
      itable[i] = i;
      itable[rotate_host(i, width, height, s, 180)] = i + base;
    }
  }
  else{
    int bh = height / 2;
    for(int i = 0; i < base; i++){
      int v = (i / bh) * height + (i % bh);
      itable[v] = i;
      itable[rotate_host(v, width, height, s, 90)]  = i + base;
      itable[rotate_host(v, width, height, s, 180)] = i + base * 2;
      itable[rotate_host(v, width, height, s, 270)] = i + base * 3;
    }
  }
}

/* Per-vertex degrees over all n vertices, as the reference's Init variants
 * expand them (aspl_cuda.cu:164-179 tiling, :200-217 rotation).  For s = 4
 * grids the base vertex of local index i is placed with the inverse of the
 * local index map, as the row table does. */
static void fill_degrees(const odp_shape *sh, int n, int *out)
{
  int s = sh->symmetries, base = n / s;
  const int *nd = sh->num_degrees;
  if(!sh->grid || s == 1){
    for(int t = 0; t < s; t++)
      for(int j = 0; j < base; j++) out[t * base + j] = nd[j];
    return;
  }
  int w = sh->width, h = sh->height;
  if(s == 2){
    for(int i = 0; i < base; i++){
      out[i] = nd[i];
      out[rotate_host(i, w, h, 2, 180)] = nd[i];
    }
  }
  else{
    for(int i = 0; i < base; i++){
      int v = (i / (h / 2)) * h + i % (h / 2);
      out[v] = nd[i];
      out[rotate_host(v, w, h, 4, 90)]  = nd[i];
      out[rotate_host(v, w, h, 4, 180)] = nd[i];
      out[rotate_host(v, w, h, 4, 270)] = nd[i];
    }
  }
}

/* Source ordinals of a grid graph, ordered by square tiles of the base
 * region (the whole grid, the left half for s = 2, the lower-left quadrant
 * for s = 4), so that each column chunk's sources are close together and its
 * BFS wavefront stays narrow.  Indexed by row; rows that are not sources get
 * -1.  Any assignment of sources to bits gives the same results: the sum and
 * the diameter do not depend on which sources share a chunk. */
static void fill_srcpos(const odp_plan_graph *g, int *srcpos)
{
  int bw = g->s == 1 ? g->width : g->width / 2;
  int bh = g->s == 4 ? g->height / 2 : g->height;
  int cap = 64 << g->wc_log2, ts = 1;
  while((ts + 1) * (ts + 1) <= cap) ts++;
  for(int r = 0; r < g->n; r++) srcpos[r] = -1;
  int ord = 0;
  for(int tx = 0; tx < bw; tx += ts)
    for(int ty = 0; ty < bh; ty += ts)
      for(int x = tx; x < tx + ts && x < bw; x++)
        for(int y = ty; y < ty + ts && y < bh; y++){
          /* rows of base vertices: v itself for s = 1, 2 (x < w/2); the local
           * index x * (h/2) + y for s = 4 */
          int row = (g->s == 4) ? x * bh + y : x * g->height + y;
          srcpos[row] = ord++;
        }
}

/* Per-bucket tuning table (ODPX_Set_tuning_table), filled by the autotuner:
 * a graph whose (ceil log2 n, degree class, grid) matches an entry takes its
 * chunk width, tile traffic and local-job threshold. */
#define TUNE_MAX 256
static ODPX_Tune_entry g_table[TUNE_MAX];
static int g_table_len = 0;

int ODPX_Set_tuning_table(const ODPX_Tune_entry *entries, int count)
{
  if(count < 0 || count > TUNE_MAX || (count > 0 && !entries)) return ODPX_ERR_INVALID;
  if(count) memcpy(g_table, entries, sizeof(ODPX_Tune_entry) * (size_t)count);
  g_table_len = count;
  return 0;
}

int ODPX_Degree_class(int degree) { return degree <= 8 ? 0 : degree <= 16 ? 1 : degree <= 32 ? 2 : 3; }

static const ODPX_Tune_entry *table_lookup(int n, int degree, int grid)
{
  int nl = ilog2_ceil(n);
  int dc = ODPX_Degree_class(degree);
  for(int i = 0; i < g_table_len; i++)
    if(g_table[i].n_log2 == nl && g_table[i].degree_class == dc && g_table[i].grid == grid) return &g_table[i];
  return NULL;
}

typedef struct { int job; double work; } job_order;

static int cmp_work_desc(const void *a, const void *b)
{
  double wa = ((const job_order *)a)->work, wb = ((const job_order *)b)->work;
  if(wa > wb) return -1;
  if(wa < wb) return 1;
  return ((const job_order *)a)->job - ((const job_order *)b)->job;
}

/* Initial engine state: the first nslots jobs loaded into the slots, the
 * job queue at nslots, everything else zero. */
static void fill_state_init(odp_plan *p)
{
  memset(p->h_state_init, 0, p->state_bytes);
  gbx_slot *sl = (gbx_slot *)p->h_state_init;
  for(int k = 0; k < p->nslots; k++){
    const gbx_job *j = &p->h_jobs[k];
    sl[k].ticket = (unsigned long long)j->ntiles << 32;
    sl[k].job = k;
    sl[k].desc = *j;
    sl[k].level = 1;
    sl[k].prev = (unsigned long long)j->nsrc;
    sl[k].sum = ((long long)j->n * j->nsrc - j->nsrc) * j->sym;
    sl[k].buf0 = p->d_slotbuf + (size_t)k * 2 * p->slot_words;
    sl[k].buf1 = sl[k].buf0 + p->slot_words;
    sl[k].mask0 = p->d_slotmask + (size_t)k * 2 * p->slot_rows;
    sl[k].mask1 = sl[k].mask0 + p->slot_rows;
  }
  gbx_ctrl *ctrl = (gbx_ctrl *)(p->h_state_init + p->out_off);
  ctrl->next_job = (unsigned)p->nslots;
}

/* Whether a graph's jobs track changes (gather only words that changed at
 * the previous level).  It is exact for every graph.  Without it, lanes whose
 * words are saturated already skip their gathers; with it, every row stages
 * its neighbours' change masks, which pays where levels are many and each
 * changes few words: single grids.  Plans whose every job tracks changes run
 * the engine built for those passes alone, with two vectors per lane.
 * Measured on GB300, on against off (ms): 100 x 100, d = 4: 1.27 / 1.10;
 * 128 x 128, d = 6: 1.63 / 1.42, but d = 4: 1.87 / 2.04; 160 x 160: 3.62 /
 * 3.96; 192 x 192: 6.26 / 9.15; 224 x 224: 12.9 / 17.4; 256 x 256, s = 4:
 * 6.86 / 7.04; 256 x 256, d = 8, s = 2: 9.76 / 13.3.  In batches the larger
 * staging area of every job cost more than it saved (the 512-graph batch:
 * 9.0 against 7.15 ms tuned).  So by default it is on for a single grid of
 * at least 20000 vertices. */
static int tracks_changes(const odp_tuning *t, int count, int grid, int n, int s)
{
  (void)s;
  if(t->activity == -2) return count == 1 && grid && n >= 20000;
  return t->activity == -1 ? grid : t->activity;
}

static int shape_n(const odp_shape *sh) { return sh->grid ? sh->width * sh->height : sh->nodes; }
static int shape_dp(const odp_shape *sh) { return ALIGN_UP(sh->degree > 0 ? sh->degree : 1, 4); }
static int shape_words(const odp_shape *sh) { return (shape_n(sh) / sh->symmetries + 63) / 64; }

/* Jobs of the small kernel with these chunk widths. */
static long long small_job_count(const odp_shape *shapes, int count, const int *wl)
{
  long long jobs = 0;
  for(int i = 0; i < count; i++) jobs += (shape_words(&shapes[i]) + (1 << wl[i]) - 1) >> wl[i];
  return jobs;
}

/* Whether a plan runs on the small-graph kernel, and its shape: the chunk
 * width of each graph (wl), the CTAs per job (one thread-block cluster), the
 * threads and shared memory per CTA.  Every graph must have at most small_n
 * vertices and no schedule setting or change tracking may ask for the
 * engine.  The cluster is the largest power of two up to 8 at which every
 * graph fits and every CTA of the plan gets its own SM; for each graph the
 * widest chunk that fits is halved, widest first, while the jobs still fit on
 * the SMs (the n = 1024, d = 8 graph: 8 jobs of 2 words on clusters of 8
 * CTAs, 64 SMs).  Plans that would need more than one wave of CTAs stay on
 * the persistent engine: every job reads its graph's adjacency from host
 * memory, and on GB300 the n = 4096, d = 24 and 32 graphs (32 jobs on
 * clusters of 8, two waves) took 151 and 257 us in the small kernel against
 * 84 and 95 us in the engine, while one-wave graphs up to n = 4096 gained
 * (n = 4096, d = 8: 55 against 85 us; a 64 x 64 grid: 176 against 418 us).
 * The replicated layout (every CTA holds the whole level) is tried first.
 * Plans of grid graphs whose whole level does not fit in one CTA take the
 * partitioned layout (each CTA holds its rows, neighbour rows are read from
 * the CTA that owns them through distributed shared memory), which fits
 * graphs up to `cluster` times larger.  Its gathers run at about one 16-byte
 * request per clock per SM, so it pays only where levels are many and
 * light: on GB300, grids of n = 5184, 6400 and 8100 (diameters 49 to 74)
 * took 265, 301 and 655 us against 547, 626 and 888 us in the engine, while
 * general graphs lost (n = 8192, d = 8: 339 against 122 us; n = 4096,
 * d = 24: 304 against 83 us).  A cluster size forced by
 * ODP_GB300_SMALL_CLUSTER is used if the graphs fit at it (else halved),
 * whatever the SM count; ODP_GB300_SMALL_PART=0 or 1 forces the layout. */
static int choose_small(const odp_shape *shapes, int count, const odp_tuning *t, int sms, int *wl,
                        int *cluster_out, int *threads_out, size_t *smem_out, int *part_out)
{
  if(count <= 0 || t->small_n <= 0 || t->wc_log2 > 0 || t->slots > 0 || t->tile_rows > 0 || t->local_kb_explicit)
    return 0;
  for(int i = 0; i < count; i++){
    const int n = shape_n(&shapes[i]);
    const ODPX_Tune_entry *te = table_lookup(n, shapes[i].degree, shapes[i].grid);
    if(n > t->small_n || (te && te->wc_log2 > 0) || tracks_changes(t, count, shapes[i].grid, n, shapes[i].symmetries))
      return 0;
  }
  if(gbx_small_prepare()) return 0;
  const int want = t->small_cluster > 0 && t->small_cluster <= GBX_SMALL_CLUSTER_MAX ? t->small_cluster : 0;
  int all_grids = 1;
  for(int i = 0; i < count; i++) all_grids &= shapes[i].grid != 0;
  for(int part = t->small_part > 0 ? 1 : 0; part <= (t->small_part == 0 ? 0 : 1); part++){
    for(int c = want ? want : GBX_SMALL_CLUSTER_MAX; c >= 1; c >>= 1){
      if(part && c == 1) continue;                 /* one CTA: the replicated layout */
      if(part && t->small_part < 0 && !all_grids) continue;
      int ok = 1;
      for(int i = 0; i < count && ok; i++){
        const int W = shape_words(&shapes[i]);
        wl[i] = small_wc_log2(shape_n(&shapes[i]), shape_dp(&shapes[i]), ilog2_ceil(W < 2 ? 2 : W), c, part);
        if(!wl[i]) ok = 0;
      }
      if(!ok) continue;
      long long jobs = small_job_count(shapes, count, wl);
      if(!want && jobs * c > sms) continue;
      for(;;){                                   /* narrower chunks while the jobs fit on the SMs */
        int k = -1;
        for(int i = 0; i < count; i++)
          if(wl[i] > 1 && (k < 0 || wl[i] > wl[k])) k = i;
        if(k < 0) break;
        wl[k]--;
        const long long more = small_job_count(shapes, count, wl);
        if(more * c > sms){ wl[k]++; break; }
        jobs = more;
      }
      size_t smem = 0;
      int threads = 64;
      for(int i = 0; i < count; i++){
        const size_t b = small_bytes(shape_n(&shapes[i]), shape_dp(&shapes[i]), wl[i], c, part);
        const int th = small_threads_for(shape_n(&shapes[i]), wl[i], c);
        if(b > smem) smem = b;
        if(th > threads) threads = th;
      }
      int active = 0;
      if(smem <= GBX_SMALL_SMEM_MAX && gbx_small_clusters(c, threads, smem, &active) == 0 && active > 0){
        *cluster_out = c;
        *threads_out = threads;
        *smem_out = smem;
        *part_out = part;
        return 1;
      }
    }
  }
  return 0;
}

#define CK(call) do{ int _e = (call); if(_e){ rc = ODPX_ERR_CUDA; goto fail; } }while(0)

int odp_plan_create(const odp_shape *shapes, int count, const odp_tuning *tuning, odp_plan **out)
{
  int rc = 0;
  *out = NULL;
  if(count <= 0) return ODPX_ERR_INVALID;
  for(int i = 0; i < count; i++){          /* arguments first: refused the same with or without a device */
    rc = validate_shape(&shapes[i]);
    if(rc) return rc;
  }
  if(odp_device_ready()) return ODPX_ERR_CUDA;

  odp_plan *p = calloc(1, sizeof(odp_plan));
  p->tuning = *tuning;
  p->ngraphs = count;
  p->g = calloc((size_t)count, sizeof(odp_plan_graph));
  p->blocks = tuning->blocks;          /* 0: chosen per launch from the staging size */
  p->spin_limit_ns = 60ull * 1000000000ull;
  const double budget = (double)tuning->l2_budget_mb * 1024.0 * 1024.0;
  const double local_bytes = (double)tuning->local_kb * 1024.0;

  /* A small plan: every job runs in the small-graph kernel, its bitsets and
   * row table in the shared memory of one thread-block cluster, with no
   * device-wide hand-off per level.  Mixed plans keep every job in the
   * persistent engine, whose short jobs fill the end of a run. */
  const int sms = g_sm_count > 0 ? g_sm_count : 1;
  int *small_wl = calloc((size_t)count, sizeof(int));
  int small = choose_small(shapes, count, tuning, sms, small_wl, &p->small_cluster, &p->small_threads,
                           &p->small_smem, &p->small_part);

  /* Shapes, chunk widths, tiles. */
  int njobs = 0;
  for(int i = 0; i < count; i++){
    const odp_shape *sh = &shapes[i];
    odp_plan_graph *g = &p->g[i];
    g->grid = sh->grid;
    g->n = sh->grid ? sh->width * sh->height : sh->nodes;
    g->d = sh->degree;
    g->dp = ALIGN_UP(sh->degree > 0 ? sh->degree : 1, 4);
    if(g->dp > p->max_dp) p->max_dp = g->dp;
    g->s = sh->symmetries;
    g->grid_s = sh->grid && sh->symmetries != 1;
    g->width = sh->width;
    g->height = sh->height;
    g->B = g->n / g->s;
    g->W = (g->B + 63) / 64;
    int full_l2 = ilog2_ceil(g->W < 2 ? 2 : g->W);
    const ODPX_Tune_entry *te = table_lookup(g->n, g->d, g->grid);
    int wl;
    if(tuning->wc_log2 > 0) wl = tuning->wc_log2;
    else if(te && te->wc_log2 > 0) wl = te->wc_log2;
    else if(tracks_changes(tuning, count, sh->grid, g->n, g->s)){
      /* 512-byte rows for a grid with change tracking (the 256 x 256 grid:
       * 24.4 ms with 64 words and 16 slots against 28.8 ms with 32 and 8) */
      wl = full_l2 < 6 ? full_l2 : 6;
    }
    else{
      /* 256-byte rows (32 words): measured best on GB300 for the 512-graph
       * batch and for single graphs (n = 1024, 65536, the 262144-vertex s = 64
       * graph and grids without change tracking) */
      wl = full_l2 < 5 ? full_l2 : 5;
    }
    if(wl < 1) wl = 1;
    if(wl > 7) wl = 7;                 /* rows of at most 1 KB per chunk */
    if(wl > full_l2 && full_l2 >= 1) wl = full_l2;
    if(small) wl = small_wl[i];
    g->wc_log2 = wl;
    const int wc = 1 << wl;
    g->nchunks = (g->W + wc - 1) / wc;
    g->has_ndeg = sh->num_degrees != NULL;
    g->has_itable = g->grid_s;
    g->has_srcpos = sh->grid;             /* grids: spatially compact source chunks */
    g->adj_ints = (size_t)g->B * g->d;
    g->adj_off = p->adj_ints;       p->adj_ints += ALIGN_UP(g->adj_ints, 4);
    g->ndeg_off = p->ndeg_ints;     if(g->has_ndeg) p->ndeg_ints += ALIGN_UP((size_t)g->n, 4);
    g->itable_off = p->itable_ints; if(g->has_itable) p->itable_ints += ALIGN_UP((size_t)g->n, 4);
    g->nbr_off = p->nbr_ints;       p->nbr_ints += (size_t)g->n * g->dp;
    g->srcpos_off = p->srcpos_ints; if(g->has_srcpos) p->srcpos_ints += ALIGN_UP((size_t)g->n, 4);
    p->total_vertices += g->n;
    njobs += g->nchunks;
  }
  p->njobs = njobs;
  p->small = small;
  free(small_wl);

  /* Tiles: about 640 KB of traffic each, measured best on GB300 for large
   * single graphs and for most size buckets of the batch.  A plan with few
   * jobs for the grid (a single graph, a group of annealing chains) takes
   * smaller tiles, and splits jobs it would otherwise run in one CTA, so
   * that its concurrently active jobs give every CTA about two tiles per
   * level.  A graph with change tracking, whose tiles mostly have little to
   * do, takes tiles of about 1.6 MB (the 256 x 256 grid: 400-row tiles,
   * 21.9 ms, against 23.6 ms with 160 rows and 24.0 ms with 640 on GB300). */
  const int grid_blocks = tuning->blocks > 0 ? tuning->blocks : gbx_engine_blocks(0);
  double fill_tile = 0;
  if(njobs * 4 <= grid_blocks){
    double active = 0;
    for(int i = 0; i < count; i++){
      const odp_plan_graph *g = &p->g[i];
      double lb = (double)g->n * (1 << g->wc_log2) * 8.0 * (g->d + 2);
      int conc = g->nchunks;
      if(count == 1){
        int cap = !g->grid ? 4 : tracks_changes(tuning, 1, 1, g->n, g->s) ? 16 : 8;
        if(conc > cap) conc = cap;
      }
      active += lb * conc;
    }
    fill_tile = active / (2.0 * (grid_blocks > 0 ? grid_blocks : 1));
    if(fill_tile < 32.0 * 1024.0) fill_tile = 32.0 * 1024.0;
  }
  for(int i = 0; i < count; i++){
    odp_plan_graph *g = &p->g[i];
    const ODPX_Tune_entry *te = table_lookup(g->n, g->d, g->grid);
    const int wc = 1 << g->wc_log2;
    double level_bytes = (double)g->n * wc * 8.0 * (g->d + 2);
    int rpp = rows_per_pass(g->wc_log2);
    double local_here = (te && te->local_kb > 0 && tuning->local_kb_explicit == 0) ? te->local_kb * 1024.0
                                                                                   : local_bytes;
    double tile_bytes = tracks_changes(tuning, count, g->grid, g->n, g->s) ? 1600.0 * 1024.0 : 640.0 * 1024.0;
    if(te && te->tile_kb > 0) tile_bytes = te->tile_kb * 1024.0;
    else if(fill_tile > 0 && fill_tile < tile_bytes){
      tile_bytes = fill_tile;
      if(!tuning->local_kb_explicit && fill_tile < local_here) local_here = fill_tile;
    }
    if(tuning->tile_rows > 0) g->tile_rows = ALIGN_UP(tuning->tile_rows, 4);   /* blocks start on 16-byte mask boundaries */
    else if(level_bytes <= local_here) g->tile_rows = g->n;
    else{
      double per_row = (double)wc * 8.0 * (g->d + 2);
      int tr = (int)(tile_bytes / per_row);
      g->tile_rows = ALIGN_UP(tr < rpp ? rpp : tr, rpp);
    }
    if(g->tile_rows > g->n) g->tile_rows = g->n;
    if(g->tile_rows < 1) g->tile_rows = 1;
    g->ntiles = (g->n + g->tile_rows - 1) / g->tile_rows;
  }

  /* Jobs, largest first so the long ones start early. */
  gbx_job *jobs = calloc((size_t)njobs, sizeof(gbx_job));
  job_order *ord = calloc((size_t)njobs, sizeof(job_order));
  {
    int k = 0;
    for(int i = 0; i < count; i++){
      odp_plan_graph *g = &p->g[i];
      int wc = 1 << g->wc_log2;
      for(int c = 0; c < g->nchunks; c++, k++){
        gbx_job *j = &jobs[k];
        j->n = g->n; j->dp = g->dp; j->d = g->d; j->wc_log2 = g->wc_log2;
        j->src0 = c * wc * 64;
        j->nsrc = g->B - j->src0 < wc * 64 ? g->B - j->src0 : wc * 64;
        j->sym = g->s; j->graph = i;
        j->tile_rows = g->tile_rows; j->ntiles = g->ntiles;
        j->flags = tracks_changes(tuning, count, g->grid, g->n, g->s) ? GBX_JOB_ACTIVE : 0;
        ord[k].job = k;
        ord[k].work = (double)g->n * wc * (g->d + 2) * (count > 1 ? 1.0 : 0.0);
      }
    }
  }
  qsort(ord, (size_t)njobs, sizeof(job_order), cmp_work_desc);
  p->h_jobs = calloc((size_t)njobs, sizeof(gbx_job));
  for(int k = 0; k < njobs; k++){
    p->h_jobs[k] = jobs[ord[k].job];
    if(p->h_jobs[k].flags & GBX_JOB_ACTIVE) p->any_active = 1;
    else p->some_plain = 1;
  }
  free(jobs);
  free(ord);

  /* Slots: for batches, as many concurrent jobs as the L2 budget holds, at
   * least 64; for a single graph a fixed count measured best on GB300 (4 for
   * general graphs; 8 for grids, whose many short levels leave hand-offs to
   * hide, 16 for grids with change tracking).  Capped by the job count. */
  size_t max_words = 0, max_rows = 0;
  double sum_fp = 0;
  int fit = 0;
  for(int k = 0; k < njobs; k++){
    size_t w = (size_t)p->h_jobs[k].n << p->h_jobs[k].wc_log2;
    if(w > max_words) max_words = w;
    if((size_t)p->h_jobs[k].n > max_rows) max_rows = (size_t)p->h_jobs[k].n;
    double fp = 2.0 * 8.0 * (double)w;
    if(sum_fp + fp <= budget){ sum_fp += fp; fit++; }
  }
  int nslots = tuning->slots > 0 ? tuning->slots : fit;
  if(tuning->slots <= 0){
    if(nslots < 2) nslots = 2;
    if(count == 1){
      const int n0 = shapes[0].grid ? shapes[0].width * shapes[0].height : shapes[0].nodes;
      nslots = !shapes[0].grid ? 4 : tracks_changes(tuning, 1, 1, n0, shapes[0].symmetries) ? 16 : 8;
    }
    if(count > 1 && nslots < 64) nslots = 64;
    if(nslots > 512) nslots = 512;
  }
  if(nslots > njobs) nslots = njobs;
  if(nslots < 1) nslots = 1;
  p->nslots = nslots;
  p->slot_words = ALIGN_UP(max_words, 32);
  p->slot_rows = ALIGN_UP(max_rows, 64);

  /* Device memory. */
  p->out_off = sizeof(gbx_slot) * (size_t)nslots;
  p->acc_off = p->out_off + sizeof(gbx_ctrl) + 64;
  p->levels_off = p->acc_off + ALIGN_UP(sizeof(gbx_graph_acc) * (size_t)count, 64);
  p->state_bytes = p->levels_off + ALIGN_UP(sizeof(gbx_job_out) * (size_t)njobs, 64);
  p->out_bytes = p->state_bytes - p->out_off;

  CK(gbx_stream_create(&p->stream));
  CK(gbx_malloc((void **)&p->d_adj, sizeof(int) * (p->adj_ints ? p->adj_ints : 4)));
  if(p->ndeg_ints) CK(gbx_malloc((void **)&p->d_ndeg, sizeof(int) * p->ndeg_ints));
  if(p->itable_ints) CK(gbx_malloc((void **)&p->d_itable, sizeof(int) * p->itable_ints));
  CK(gbx_malloc((void **)&p->d_nbr, sizeof(int) * (p->nbr_ints ? p->nbr_ints : 4)));
  CK(gbx_malloc((void **)&p->d_slotbuf, sizeof(unsigned long long) * p->slot_words * 2 * (size_t)nslots));
  CK(gbx_malloc((void **)&p->d_slotmask, sizeof(unsigned int) * p->slot_rows * 2 * (size_t)nslots));
  if(p->srcpos_ints) CK(gbx_malloc((void **)&p->d_srcpos, sizeof(int) * p->srcpos_ints));
  CK(gbx_malloc((void **)&p->d_expand, sizeof(gbx_expand_desc) * (size_t)count));
  CK(gbx_malloc((void **)&p->d_jobs, sizeof(gbx_job) * (size_t)njobs));
  CK(gbx_malloc((void **)&p->d_state, p->state_bytes));
  p->direct = tuning->direct && gbx_pageable_access();
  /* Small plans read their descriptors (and through them the adjacency)
   * from pinned host memory and write per-job records there. */
  if(p->direct || small) CK(gbx_host_alloc((void **)&p->h_expand, sizeof(gbx_expand_desc) * (size_t)count));
  if(!p->direct) CK(gbx_host_alloc((void **)&p->h_adj, sizeof(int) * (p->adj_ints ? p->adj_ints : 4)));
  if(small){
    CK(gbx_host_alloc((void **)&p->h_small_rec, sizeof(gbx_small_rec) * (size_t)njobs));
    memset(p->h_small_rec, 0, sizeof(gbx_small_rec) * (size_t)njobs);
    CK(gbx_host_device_ptr(p->h_small_rec, (void **)&p->d_small_rec));
    CK(gbx_host_device_ptr(p->h_expand, (void **)&p->d_small_desc));
  }
  else if(p->direct){
    /* the pull kernel reads this call's descriptors from pinned memory and
     * resets the engine state from a device copy of its initial value */
    CK(gbx_host_device_ptr(p->h_expand, (void **)&p->d_hexpand));
    CK(gbx_malloc((void **)&p->d_state_init, p->state_bytes));
  }
  CK(gbx_host_alloc((void **)&p->h_state_init, p->state_bytes));
  CK(gbx_host_alloc((void **)&p->h_state_out, p->out_bytes));

  /* Static tables: degrees, row tables, expand descriptors, jobs. */
  {
    int *h_nd = p->ndeg_ints ? malloc(sizeof(int) * p->ndeg_ints) : NULL;
    int *h_it = p->itable_ints ? malloc(sizeof(int) * p->itable_ints) : NULL;
    int *h_sp = p->srcpos_ints ? malloc(sizeof(int) * p->srcpos_ints) : NULL;
    gbx_expand_desc *ed = calloc((size_t)count, sizeof(gbx_expand_desc));
    long long first = 0;
    for(int i = 0; i < count; i++){
      odp_plan_graph *g = &p->g[i];
      if(g->has_ndeg){
        fill_degrees(&shapes[i], g->n, h_nd + g->ndeg_off);
        g->row_reads = 0;
        for(int v = 0; v < g->n; v++) g->row_reads += (double)h_nd[g->ndeg_off + v] + 2.0;
      }
      else g->row_reads = (double)g->n * (g->d + 2);
      if(g->has_itable) fill_itable(g->width, g->height, g->s, h_it + g->itable_off);
      if(g->has_srcpos) fill_srcpos(g, h_sp + g->srcpos_off);
      gbx_expand_desc *e = &ed[i];
      e->adj = p->d_adj + g->adj_off;
      e->ndeg = g->has_ndeg ? p->d_ndeg + g->ndeg_off : NULL;
      e->itable = g->has_itable ? p->d_itable + g->itable_off : NULL;
      e->nbr = p->d_nbr + g->nbr_off;
      e->n = g->n; e->d = g->d; e->dp = g->dp; e->s = g->s;
      e->width = g->width; e->height = g->height; e->grid_s = g->grid_s;
      e->first_vertex = first;
      first += g->n;
    }
    for(int k = 0; k < njobs; k++){
      const odp_plan_graph *g = &p->g[p->h_jobs[k].graph];
      p->h_jobs[k].nbr = p->d_nbr + g->nbr_off;
      p->h_jobs[k].srcpos = g->has_srcpos ? p->d_srcpos + g->srcpos_off : NULL;
    }
    if(h_sp) CK(gbx_memcpy_h2d(p->d_srcpos, h_sp, sizeof(int) * p->srcpos_ints, p->stream));
    if(h_nd) CK(gbx_memcpy_h2d(p->d_ndeg, h_nd, sizeof(int) * p->ndeg_ints, p->stream));
    if(h_it) CK(gbx_memcpy_h2d(p->d_itable, h_it, sizeof(int) * p->itable_ints, p->stream));
    CK(gbx_memcpy_h2d(p->d_expand, ed, sizeof(gbx_expand_desc) * (size_t)count, p->stream));
    if(small){
      /* the small-graph kernel reads `adj` itself: the caller's array (set
       * per call) or this plan's pinned staging copy */
      memcpy(p->h_expand, ed, sizeof(gbx_expand_desc) * (size_t)count);
      for(int i = 0; i < count; i++){
        p->h_expand[i].adj_dev = NULL;
        p->h_expand[i].adj = p->direct ? NULL : p->h_adj + p->g[i].adj_off;
      }
    }
    else if(p->direct){
      /* per call: `adj` names the caller's host array, `adj_dev` the device
       * copy that gbx_pull fills and expand reads */
      memcpy(p->h_expand, ed, sizeof(gbx_expand_desc) * (size_t)count);
      for(int i = 0; i < count; i++) p->h_expand[i].adj_dev = (int *)ed[i].adj;
    }
    CK(gbx_memcpy_h2d(p->d_jobs, p->h_jobs, sizeof(gbx_job) * (size_t)njobs, p->stream));
    CK(gbx_stream_sync(p->stream));
    free(h_nd); free(h_it); free(h_sp); free(ed);
  }

  fill_state_init(p);
  if(p->d_state_init){
    CK(gbx_memcpy_h2d(p->d_state_init, p->h_state_init, p->state_bytes, p->stream));
    CK(gbx_stream_sync(p->stream));
  }
  *out = p;
  return 0;

fail:
  odp_plan_destroy(p);
  return rc;
}

void odp_plan_destroy(odp_plan *p)
{
  if(!p) return;
  if(p->graph_exec) gbx_graph_destroy(p->graph_exec);
  gbx_free(p->d_adj); gbx_free(p->d_ndeg); gbx_free(p->d_itable); gbx_free(p->d_nbr);
  gbx_free(p->d_slotbuf); gbx_free(p->d_slotmask); gbx_free(p->d_srcpos); gbx_free(p->d_expand); gbx_free(p->d_jobs); gbx_free(p->d_state);
  gbx_free(p->d_state_init);
  gbx_host_free(p->h_adj); gbx_host_free(p->h_expand); gbx_host_free(p->h_state_init); gbx_host_free(p->h_state_out);
  gbx_host_free(p->h_small_rec);
  if(p->stream) gbx_stream_destroy(p->stream);
  free(p->h_jobs);
  free(p->g);
  free(p);
}

/* The per-call GPU work, in stream order.  A small plan is one kernel: it
 * reads the adjacency from host memory and writes its records there. */
static int enqueue(odp_plan *p)
{
  int e;
  if(p->small) return odp_plan_enqueue_engine(p);
  if(p->direct){
    /* one kernel: this call's descriptors (their host pointers) from pinned
     * memory, the callers' arrays into the device copy that expand reads,
     * and the engine state reset */
    if((e = gbx_pull(p->d_hexpand, p->d_expand, p->ngraphs, p->d_state, p->d_state_init, p->state_bytes, p->stream)))
      return e;
  }
  else{
    if((e = gbx_memcpy_h2d(p->d_adj, p->h_adj, sizeof(int) * (p->adj_ints ? p->adj_ints : 4), p->stream))) return e;
    if((e = gbx_memcpy_h2d(p->d_state, p->h_state_init, p->state_bytes, p->stream))) return e;
  }
  if((e = gbx_expand(p->d_expand, p->ngraphs, p->total_vertices, p->max_dp,
                     (unsigned int *)(p->d_state + p->out_off + sizeof(gbx_ctrl)), p->stream))) return e;
  if((e = odp_plan_enqueue_engine(p))) return e;
  return gbx_memcpy_d2h(p->h_state_out, p->d_state + p->out_off, p->out_bytes, p->stream);
}

int odp_plan_enqueue_engine(odp_plan *p)
{
  if(p->small){
    /* one graph: its descriptor (this call's adjacency pointer) travels in
     * the launch's parameters, so the plan is launched directly each call */
    const int one = p->ngraphs == 1;
    return gbx_small_launch(p->d_jobs, p->njobs, one ? NULL : p->d_small_desc, one ? &p->h_expand[0] : NULL,
                            p->d_small_rec, p->small_smem, p->small_cluster, p->small_threads, p->small_part,
                            p->stream);
  }
  return gbx_engine_launch(p->d_jobs, p->njobs, (gbx_slot *)p->d_state, p->nslots,
                           (gbx_ctrl *)(p->d_state + p->out_off), (gbx_graph_acc *)(p->d_state + p->acc_off),
                           (gbx_job_out *)(p->d_state + p->levels_off), p->spin_limit_ns, p->blocks,
                           !p->any_active ? 0 : p->some_plain ? 2 : 1, p->stream);
}

const gbx_job_out *odp_plan_job_out(const odp_plan *p)
{
  return (const gbx_job_out *)(p->h_state_out + (p->levels_off - p->out_off));
}

typedef struct {
  odp_plan *p;
  const int *const *adjacency;
  int first, last;
} stage_part;

static void *stage_worker(void *arg)
{
  stage_part *w = arg;
  for(int i = w->first; i < w->last; i++){
    const odp_plan_graph *g = &w->p->g[i];
    memcpy(w->p->h_adj + g->adj_off, w->adjacency[i], sizeof(int) * g->adj_ints);
  }
  return NULL;
}

/* Hands this call's adjacency arrays to the device.  When kernels can read
 * pageable host memory, a pull kernel reads the callers' arrays in place
 * (coalesced 16-byte loads over the CPU-GPU link) and only their pointers are
 * recorded here: no host-side copy.  Otherwise the arrays
 * are copied into the pinned staging buffer that the upload reads; large
 * batches are split over host threads by bytes, since one thread copies at a
 * fraction of the memory bandwidth. */
void odp_plan_stage(odp_plan *p, const int *const *adjacency)
{
  if(p->direct){
    /* The device reads pageable host memory: no staging copy, only the
     * pointers (the arrays must stay unchanged until the run is finished). */
    for(int i = 0; i < p->ngraphs; i++) p->h_expand[i].adj = adjacency[i];
    return;
  }
  size_t total = sizeof(int) * p->adj_ints;
  long cpus = sysconf(_SC_NPROCESSORS_ONLN);
  int nt = total < (4u << 20) ? 1 : (int)(cpus < 16 ? cpus : 16);
  if(nt > p->ngraphs) nt = p->ngraphs;
  if(nt <= 1){
    stage_part w = { p, adjacency, 0, p->ngraphs };
    stage_worker(&w);
    return;
  }
  stage_part parts[16];
  pthread_t th[16];
  size_t per = total / (size_t)nt, acc = 0;
  int start = 0, k = 0;
  for(int i = 0; i < p->ngraphs && k < nt - 1; i++){
    acc += sizeof(int) * p->g[i].adj_ints;
    if(acc >= per * (size_t)(k + 1)){
      parts[k] = (stage_part){ p, adjacency, start, i + 1 };
      start = i + 1;
      k++;
    }
  }
  parts[k++] = (stage_part){ p, adjacency, start, p->ngraphs };
  int launched[16] = {0};
  for(int t = 1; t < k; t++) launched[t] = pthread_create(&th[t], NULL, stage_worker, &parts[t]) == 0;
  stage_worker(&parts[0]);
  for(int t = 1; t < k; t++){
    if(launched[t]) pthread_join(th[t], NULL);
    else stage_worker(&parts[t]);
  }
}

int odp_plan_launch(odp_plan *p)
{
  /* a single-graph small plan passes this call's descriptor by value: never captured */
  if(p->tuning.use_graph && !(p->small && p->ngraphs == 1)){
    if(!p->graph_exec){
      if(gbx_capture_begin(p->stream)) return ODPX_ERR_CUDA;
      int e = enqueue(p);
      void *ge = NULL;
      int e2 = gbx_capture_end(p->stream, &ge);
      if(e || e2) return ODPX_ERR_CUDA;
      p->graph_exec = ge;
    }
    return gbx_graph_launch(p->graph_exec, p->stream) ? ODPX_ERR_CUDA : 0;
  }
  return enqueue(p) ? ODPX_ERR_CUDA : 0;
}

/* Longest-processing-time order learned from a finished run.  The first
 * order sorts jobs by their per-level traffic, which does not know how many
 * levels each job will run; a graph with a long diameter (a grid with a short
 * length limit) then starts late and ends the batch alone.  After the first
 * run the jobs are re-sorted by their measured device time (load to finish),
 * so the next runs start the longest ones first.  Results do not depend on
 * the order.  The per-job records of the finished run are permuted the same
 * way so that they stay matched with the job table.  Runs with the stream
 * idle (after the synchronisation in odp_plan_finish), so neither the job
 * table nor the initial state is being read by the device. */
static int reorder_by_duration(odp_plan *p)
{
  gbx_job_out *jo = (gbx_job_out *)(p->h_state_out + (p->levels_off - p->out_off));
  unsigned long long t0 = ((const gbx_ctrl *)p->h_state_out)->t_start;
  for(int k = 0; k < p->njobs; k++){
    if(jo[k].t_loaded && jo[k].t_loaded < t0) t0 = jo[k].t_loaded;
    if(jo[k].t_done && jo[k].t_done < t0) t0 = jo[k].t_done;
  }
  job_order *ord = malloc(sizeof(job_order) * (size_t)p->njobs);
  gbx_job *nj = malloc(sizeof(gbx_job) * (size_t)p->njobs);
  gbx_job_out *no = malloc(sizeof(gbx_job_out) * (size_t)p->njobs);
  if(!ord || !nj || !no){ free(ord); free(nj); free(no); return ODPX_ERR_MEMORY; }
  for(int k = 0; k < p->njobs; k++){
    unsigned long long a = jo[k].t_loaded ? jo[k].t_loaded : t0;
    ord[k].job = k;
    ord[k].work = jo[k].t_done > a ? (double)(jo[k].t_done - a) : 0.0;
  }
  qsort(ord, (size_t)p->njobs, sizeof(job_order), cmp_work_desc);
  for(int k = 0; k < p->njobs; k++){
    nj[k] = p->h_jobs[ord[k].job];
    no[k] = jo[ord[k].job];
  }
  memcpy(p->h_jobs, nj, sizeof(gbx_job) * (size_t)p->njobs);
  memcpy(jo, no, sizeof(gbx_job_out) * (size_t)p->njobs);
  free(ord); free(nj); free(no);
  fill_state_init(p);
  if(gbx_memcpy_h2d(p->d_jobs, p->h_jobs, sizeof(gbx_job) * (size_t)p->njobs, p->stream)) return ODPX_ERR_CUDA;
  if(p->d_state_init && gbx_memcpy_h2d(p->d_state_init, p->h_state_init, p->state_bytes, p->stream))
    return ODPX_ERR_CUDA;
  if(gbx_stream_sync(p->stream)) return ODPX_ERR_CUDA;
  return 0;
}

/* Small plans: the per-job records folded per graph, as the engine's
 * accumulators fold them (sum of the jobs' sums, the largest level, stalled
 * if any job stalled); the levels and stamps also go to the per-job outcome
 * table that the introspection calls read. */
static int finish_small(odp_plan *p, odp_result *results)
{
  gbx_job_out *jo = (gbx_job_out *)(p->h_state_out + (p->levels_off - p->out_off));
  unsigned int err = 0;
  for(int k = 0; k < p->njobs; k++){
    err |= p->h_small_rec[k].err;
    jo[k].level = p->h_small_rec[k].level;
    jo[k].t_loaded = p->h_small_rec[k].t_loaded;
    jo[k].t_done = p->h_small_rec[k].t_done;
  }
  if(err & GBX_ERR_BAD_ADJ) return ODPX_ERR_ADJACENCY;
  for(int i = 0; i < p->ngraphs; i++){
    unsigned long long sum = 0;
    int level = 0, stalled = 0;
    for(int k = 0; k < p->njobs; k++){
      const gbx_small_rec *r = &p->h_small_rec[k];
      if(p->h_jobs[k].graph != i) continue;
      sum += (unsigned long long)r->sum;
      const int l = r->level < 0 ? -r->level : r->level;
      if(l > level) level = l;
      if(r->level < 0) stalled = 1;
    }
    const odp_plan_graph *g = &p->g[i];
    odp_result *res = &results[i];
    if(stalled){
      res->diameter = INT_MAX;
      res->sum = LONG_MAX;
      res->aspl = DBL_MAX;
      continue;
    }
    long total = (long)sum;
    res->diameter = level;
    res->aspl = total / (((double)g->n - 1) * g->n);
    res->sum = (long)(total / 2.0);
  }
  return 0;
}

int odp_plan_finish(odp_plan *p, odp_result *results)
{
  if(gbx_stream_sync(p->stream)) return ODPX_ERR_CUDA;
  if(p->small) return finish_small(p, results);
  const gbx_ctrl *ctrl = (const gbx_ctrl *)p->h_state_out;
  unsigned int err = *(const unsigned int *)(p->h_state_out + sizeof(gbx_ctrl)) | ctrl->error;
  if(err & GBX_ERR_TIMEOUT) return ODPX_ERR_TIMEOUT;
  if(err & GBX_ERR_BAD_ADJ) return ODPX_ERR_ADJACENCY;
  if(p->tuning.reorder && !p->small && !p->reordered && p->njobs > p->nslots){
    p->reordered = 1;
    int e = reorder_by_duration(p);
    if(e) return e;
  }
  const gbx_graph_acc *acc = (const gbx_graph_acc *)(p->h_state_out + (p->acc_off - p->out_off));
  p->bytes_alg_last = 0;
  for(int i = 0; i < p->ngraphs; i++){
    const odp_plan_graph *g = &p->g[i];
    odp_result *r = &results[i];
    if(acc[i].flags & 1){
      r->diameter = INT_MAX;
      r->sum = LONG_MAX;
      r->aspl = DBL_MAX;
      continue;
    }
    long sum = (long)acc[i].sum;
    r->diameter = acc[i].levels;
    r->aspl = sum / (((double)g->n - 1) * g->n);
    r->sum = (long)(sum / 2.0);
  }
  return 0;
}

int odp_plan_run(odp_plan *p, const int *const *adjacency, odp_result *results)
{
  odp_plan_stage(p, adjacency);
  int rc = odp_plan_launch(p);
  if(rc) return rc;
  return odp_plan_finish(p, results);
}

unsigned long long odp_plan_tiles(const odp_plan *p)
{
  return ((const gbx_ctrl *)p->h_state_out)->tiles;
}

unsigned int odp_plan_error(const odp_plan *p)
{
  if(p->small){
    unsigned int err = 0;
    for(int k = 0; k < p->njobs; k++) err |= p->h_small_rec[k].err;
    return err;
  }
  const gbx_ctrl *ctrl = (const gbx_ctrl *)p->h_state_out;
  return *(const unsigned int *)(p->h_state_out + sizeof(gbx_ctrl)) | ctrl->error;
}

double odp_plan_bytes_alg(const odp_plan *p)
{
  const gbx_job_out *jo = odp_plan_job_out(p);
  double total = 0;
  for(int k = 0; k < p->njobs; k++){
    const gbx_job *j = &p->h_jobs[k];
    int l = jo[k].level < 0 ? -jo[k].level : jo[k].level;
    /* only the chunk's words that hold sources count; padding words of a
     * narrow last chunk are moved but are not algorithmic */
    double words = (double)((j->nsrc + 63) / 64);
    total += (double)l * 8.0 * words * p->g[j->graph].row_reads;
  }
  return total;
}

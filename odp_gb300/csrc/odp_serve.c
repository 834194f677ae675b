/*
 * odp_serve.c -- serving mode: device-resident graphs updated in place by
 * 2-opt deltas and evaluated in continuous batches (ODPX_Serve_*).  No
 * counterpart in the reference, whose simulated-annealing clients re-upload
 * and re-evaluate the whole adjacency for every proposal
 * (sample/SA/general.c:149-181, aspl_cuda.cu:247).
 *
 * A client registers its graph once (adjacency and neighbour table stay on
 * the GPU), then submits requests that carry the adjacency slots its last
 * move changed: the 2-opt swap, plus the previous swap's undo when that move
 * was rejected.  A scheduler thread admits pending requests into lanes.  A
 * lane is a CUDA stream with its own pool of bitset slots (the memory budget
 * is divided among lanes) and a persistent engine launch sized to its share of
 * the GPU, so a batch admitted while others are running overlaps with them on
 * the device.  Per batch, in stream order: the deltas are applied by one
 * scatter kernel (to the compact adjacency and to every neighbour-table row
 * they touch), the jobs and engine state are uploaded, the engine runs, and
 * the per-graph accumulators come back.  A graph is never in two batches at
 * once, so a delta never races an evaluation of the same graph.
 *
 * Results are bit-identical to ODP_Init_aspl_* + ODP_Set_aspl on the updated
 * adjacency.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#include <float.h>
#include <pthread.h>
#include <time.h>
#include <math.h>
#include <sys/prctl.h>
#include "odp_plan.h"
#include "odp_gb300.h"

#define ALIGN_UP(x, a) ((((x) + (a) - 1) / (a)) * (a))

typedef struct {
  int grid, grid_s, n, d, dp, s, B, W, width, height;
  int wc_log2, nchunks, tile_rows, ntiles;
  double cost;                 /* bytes one level of all its chunks moves: the batching class */
  int *d_adj, *d_nbr, *d_ndeg, *d_itable;
  gbx_expand_desc *d_desc;
  int *h_adj;                  /* host mirror of the compact adjacency */
  int *h_itable;               /* grid symmetry: vertex -> row */
  int *h_rowdeg;               /* num_degrees of the local rows, or NULL (regular) */
  int busy;                    /* part of an in-flight batch */
} serve_graph;

typedef struct {
  int graph, ndelta;
  ODPX_Delta *deltas;
  double t_submit, t_done;
  int state;                   /* 0 pending, 1 running, 2 done */
  int rc, diameter;
  long sum;
  double aspl;
  pthread_cond_t *waiter;      /* the condition the one thread waiting for it sleeps on, or NULL */
} serve_req;

/* A lane's per-batch state block, laid out anew for every batch so that one
 * small copy carries all of it: control block and error word | per-graph
 * accumulators | the active slots | the jobs | per-job outcomes (device
 * only).  The host copy is pinned; the device reads the batch's writes
 * (delta updates) straight from pinned memory. */
#define LANE_ACC_OFF 128       /* after gbx_ctrl (64 B) and the error word */
typedef struct {
  void *stream, *ev;
  int busy, nslots, max_jobs, max_batch, max_writes, blocks;
  size_t slot_words, slot_rows, block_bytes;
  unsigned long long *d_slotbuf;
  unsigned *d_slotmask;
  char *d_block, *h_block;     /* the state block, device and pinned host */
  char *h_out;                 /* pinned: control block and accumulators of the finished batch */
  gbx_write *h_writes, *dh_writes; /* pinned writes of the batch, and their device address */
  gbx_job *h_jobs;             /* jobs as they are formed (host) */
  long long *members;          /* request ids of the running batch */
  int nmembers;
  /* the batch formed and not yet issued */
  int b_nw, b_njobs, b_nslots;
  size_t b_slots_off, b_jobs_off, b_outcomes_off, b_acc_bytes;
} serve_lane;

typedef struct odp_server odp_server;

struct odp_server {
  ODPX_Serve_config cfg;
  pthread_t thread;
  pthread_mutex_t mu;
  pthread_cond_t cv_work, cv_done;   /* cv_done: the shared wake-up of shared_waiters */
  int shared_waiters;          /* threads sleeping on cv_done */
  int stop, started;
  void *ctl_stream;
  serve_graph *graphs;
  int ngraphs, cap_graphs;
  serve_req *reqs;             /* indexed by request id */
  long long nreqs, cap_reqs, next_pending;
  serve_lane *lanes;
  double l2_lane_bytes;        /* bitset working set a lane keeps active at once (L2 share) */
  double min_cost, max_cost;   /* over the registered graphs */
  ODPX_Serve_counters stats;
};

static double now_s(void)
{
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t.tv_sec + 1e-9 * t.tv_nsec;
}

static int ilog2_ceil(long long x)
{
  int l = 0;
  while((1LL << l) < x) l++;
  return l;
}

static int rotate(int v, int width, int height, int s, int deg)   /* ODP_ROTATE, utils.c:67-88 */
{
  int x = v / height, y = v % height;
  if(s == 2) return (width - x - 1) * height + (height - y - 1);
  if(deg == 90)  return y * height + (height - x - 1);
  if(deg == 180) return (height - x - 1) * height + (height - y - 1);
  return (height - y - 1) * height + x;
}

/* ---------------------------------------------------------------------- */

static void lane_free(serve_lane *l)
{
  if(l->stream) gbx_stream_sync(l->stream);
  gbx_free(l->d_slotbuf); gbx_free(l->d_slotmask); gbx_free(l->d_block);
  gbx_host_free(l->h_block); gbx_host_free(l->h_out); gbx_host_free(l->h_writes);
  free(l->h_jobs);
  if(l->ev) gbx_event_destroy(l->ev);
  if(l->stream) gbx_stream_destroy(l->stream);
  free(l->members);
}

static int lane_init(serve_lane *l, const ODPX_Serve_config *c, int nslots, int blocks)
{
  memset(l, 0, sizeof(*l));
  l->nslots = nslots;
  l->blocks = blocks;
  l->max_batch = c->max_batch;
  l->max_jobs = c->max_batch * 64;
  l->max_writes = c->max_batch * 4096;
  l->slot_words = ALIGN_UP((size_t)c->max_nodes << c->wc_log2, 32);
  l->slot_rows = ALIGN_UP((size_t)c->max_nodes, 64);
  l->block_bytes = LANE_ACC_OFF + ALIGN_UP(sizeof(gbx_graph_acc) * (size_t)l->max_batch, 256) +
                   sizeof(gbx_slot) * (size_t)nslots + sizeof(gbx_job) * (size_t)l->max_jobs +
                   ALIGN_UP(sizeof(gbx_job_out) * (size_t)l->max_jobs, 64);
  l->h_jobs = malloc(sizeof(gbx_job) * (size_t)l->max_jobs);
  l->members = malloc(sizeof(long long) * (size_t)l->max_batch);
  if(!l->h_jobs || !l->members || gbx_stream_create(&l->stream) || gbx_event_create(&l->ev) ||
     gbx_malloc((void **)&l->d_slotbuf, sizeof(unsigned long long) * l->slot_words * 2 * (size_t)nslots) ||
     gbx_malloc((void **)&l->d_slotmask, sizeof(unsigned) * l->slot_rows * 2 * (size_t)nslots) ||
     gbx_malloc((void **)&l->d_block, l->block_bytes) ||
     gbx_host_alloc((void **)&l->h_block, l->block_bytes) ||
     gbx_host_alloc((void **)&l->h_out, LANE_ACC_OFF + sizeof(gbx_graph_acc) * (size_t)l->max_batch) ||
     gbx_host_alloc((void **)&l->h_writes, sizeof(gbx_write) * (size_t)l->max_writes) ||
     gbx_host_device_ptr(l->h_writes, (void **)&l->dh_writes))
    return ODPX_ERR_CUDA;
  return 0;
}

/* ---------------------------------------------------------------------- */

/* Device writes for one compact-adjacency update of graph g: the compact
 * entry itself and the neighbour-table entry of every row in its orbit
 * (the expand rules of the engine, evaluated on the host). */
static int delta_writes(serve_graph *g, const ODPX_Delta *dl, gbx_write *w)
{
  int k = 0, m = dl->row, j = dl->slot, a = dl->value;
  w[k].at = g->d_adj + (size_t)m * g->d + j; w[k].value = a; k++;
  g->h_adj[(size_t)m * g->d + j] = a;
  if(!g->grid_s){
    for(int t = 0; t < g->s; t++){
      int row = m + t * g->B, nb = a + t * g->B;
      if(nb >= g->n) nb -= g->n;
      w[k].at = g->d_nbr + (size_t)row * g->dp + j; w[k].value = nb; k++;
    }
  }
  else{
    int h = g->height, bh = h / 2;
    int bv = g->s == 2 ? m : (m / bh) * h + (m % bh);      /* base vertex of local row m */
    for(int t = 0; t < g->s; t++){
      int v = bv, u = a;
      if(t > 0){
        int deg = g->s == 2 ? 180 : 90 * t;
        v = rotate(bv, g->width, h, g->s, deg);
        u = rotate(a, g->width, h, g->s, deg);
      }
      w[k].at = g->d_nbr + (size_t)g->h_itable[v] * g->dp + j; w[k].value = g->h_itable[u]; k++;
    }
  }
  return k;
}

/* Results of lane l's finished batch go to its requests, and each request's
 * waiting thread, if any, is woken.  Called with the mutex held. */
static void finish_batch(odp_server *s, serve_lane *l)
{
  const gbx_ctrl *ctrl = (const gbx_ctrl *)l->h_out;
  unsigned err = *(const unsigned *)(l->h_out + sizeof(gbx_ctrl)) | ctrl->error;
  const gbx_graph_acc *acc = (const gbx_graph_acc *)(l->h_out + LANE_ACC_OFF);
  double t = now_s();
  for(int i = 0; i < l->nmembers; i++){
    serve_req *r = &s->reqs[l->members[i]];
    serve_graph *g = &s->graphs[r->graph];
    r->rc = (err & GBX_ERR_TIMEOUT) ? ODPX_ERR_TIMEOUT : (err & GBX_ERR_BAD_ADJ) ? ODPX_ERR_ADJACENCY : 0;
    if(acc[i].flags & 1){ r->diameter = INT_MAX; r->sum = LONG_MAX; r->aspl = DBL_MAX; }
    else{
      long sum = (long)acc[i].sum;
      r->diameter = acc[i].levels;
      r->aspl = sum / (((double)g->n - 1) * g->n);
      r->sum = (long)(sum / 2.0);
    }
    r->t_done = t;
    r->state = 2;
    g->busy = 0;
    if(r->waiter) pthread_cond_signal(r->waiter);
  }
  s->stats.requests_done += l->nmembers;
  l->busy = 0;
  l->nmembers = 0;
}

/* Forms a batch from the oldest pending requests whose graphs are idle on
 * lane l: its writes, jobs and state block, ready for issue_batch.  Called
 * with the mutex held; returns the number of requests taken. */
static int form_batch(odp_server *s, serve_lane *l, double max_seed_cost)
{
  int nreq = 0, njobs = 0, nw = 0;
  double seed_cost = 0;
  for(long long id = s->next_pending; id < s->nreqs && nreq < l->max_batch; id++){
    serve_req *r = &s->reqs[id];
    if(r->state != 0) continue;
    serve_graph *g = &s->graphs[r->graph];
    int need_w = r->ndelta * (1 + g->s);
    /* A batch holds requests of similar cost (within 4x of the oldest one it
     * takes): a request completes only when its whole batch does, so a small
     * graph batched with a large one would wait for it. */
    int other_class = nreq > 0 ? (g->cost > 4.0 * seed_cost || 4.0 * g->cost < seed_cost)
                               : g->cost > max_seed_cost;
    if(g->busy || other_class || njobs + g->nchunks > l->max_jobs || nw + need_w > l->max_writes) continue;
    if(nreq == 0) seed_cost = g->cost;
    for(int k = 0; k < r->ndelta; k++) nw += delta_writes(g, &r->deltas[k], l->h_writes + nw);
    free(r->deltas);
    r->deltas = NULL;
    const int wc = 1 << g->wc_log2;
    for(int c = 0; c < g->nchunks; c++){
      gbx_job *j = &l->h_jobs[njobs++];
      memset(j, 0, sizeof(*j));
      j->nbr = g->d_nbr; j->n = g->n; j->dp = g->dp; j->d = g->d; j->wc_log2 = g->wc_log2;
      j->src0 = c * wc * 64;
      j->nsrc = g->B - j->src0 < wc * 64 ? g->B - j->src0 : wc * 64;
      j->sym = g->s; j->graph = nreq; j->tile_rows = g->tile_rows; j->ntiles = g->ntiles;
    }
    g->busy = 1;
    r->state = 1;
    l->members[nreq++] = id;
  }
  /* the pending cursor moves past the prefix that is no longer pending */
  while(s->next_pending < s->nreqs && s->reqs[s->next_pending].state != 0) s->next_pending++;
  if(nreq == 0) return 0;

  /* Active slots: as many leading jobs as fit the lane's share of L2 (at
   * least one).  Lanes run at the same time, so their bitsets together must
   * stay L2-resident; the rest of the jobs queue for a free slot. */
  int nslots = 0;
  double fp = 0;
  while(nslots < njobs && nslots < l->nslots){
    const gbx_job *j = &l->h_jobs[nslots];
    double f = 16.0 * (double)((size_t)j->n << j->wc_log2);
    if(nslots > 0 && fp + f > s->l2_lane_bytes) break;
    fp += f;
    nslots++;
  }
  l->b_acc_bytes = sizeof(gbx_graph_acc) * (size_t)nreq;
  l->b_slots_off = LANE_ACC_OFF + ALIGN_UP(l->b_acc_bytes, 256);
  l->b_jobs_off = l->b_slots_off + sizeof(gbx_slot) * (size_t)nslots;
  l->b_outcomes_off = ALIGN_UP(l->b_jobs_off + sizeof(gbx_job) * (size_t)njobs, 64);
  memset(l->h_block, 0, l->b_jobs_off);
  gbx_slot *sl = (gbx_slot *)(l->h_block + l->b_slots_off);
  for(int k = 0; k < nslots; k++){
    const gbx_job *j = &l->h_jobs[k];
    sl[k].ticket = (unsigned long long)j->ntiles << 32;
    sl[k].job = k;
    sl[k].desc = *j;
    sl[k].level = 1;
    sl[k].prev = (unsigned long long)j->nsrc;
    sl[k].sum = ((long long)j->n * j->nsrc - j->nsrc) * j->sym;
    sl[k].buf0 = l->d_slotbuf + (size_t)k * 2 * l->slot_words;
    sl[k].buf1 = sl[k].buf0 + l->slot_words;
    sl[k].mask0 = l->d_slotmask + (size_t)k * 2 * l->slot_rows;
    sl[k].mask1 = sl[k].mask0 + l->slot_rows;
  }
  memcpy(l->h_block + l->b_jobs_off, l->h_jobs, sizeof(gbx_job) * (size_t)njobs);
  ((gbx_ctrl *)l->h_block)->next_job = (unsigned)nslots;
  l->b_nw = nw;
  l->b_njobs = njobs;
  l->b_nslots = nslots;
  l->nmembers = nreq;
  l->busy = 1;
  s->stats.batches++;
  s->stats.batched_requests += nreq;
  if(nreq > s->stats.max_batch) s->stats.max_batch = nreq;
  return nreq;
}

/* Issues lane l's formed batch on its stream: the delta writes (read by the
 * scatter kernel from pinned memory), one copy of the state block, the
 * engine, one copy back of the control block and accumulators, and the
 * completion event.  Touches only the lane, so it runs without the mutex. */
static int issue_batch(serve_lane *l)
{
  int e = 0;
  if(l->b_nw) e |= gbx_scatter(l->dh_writes, l->b_nw, l->stream);
  e |= gbx_memcpy_h2d(l->d_block, l->h_block, l->b_outcomes_off, l->stream);
  e |= gbx_engine_launch((const gbx_job *)(l->d_block + l->b_jobs_off), l->b_njobs,
                         (gbx_slot *)(l->d_block + l->b_slots_off), l->b_nslots, (gbx_ctrl *)l->d_block,
                         (gbx_graph_acc *)(l->d_block + LANE_ACC_OFF),
                         (gbx_job_out *)(l->d_block + l->b_outcomes_off), 60ull * 1000000000ull, l->blocks, 0,
                         l->stream);
  e |= gbx_memcpy_d2h(l->h_out, l->d_block, LANE_ACC_OFF + l->b_acc_bytes, l->stream);
  e |= gbx_event_record(l->ev, l->stream);
  return e;
}

/* A batch that could not be issued fails its requests.  Mutex held. */
static void fail_batch(odp_server *s, serve_lane *l)
{
  for(int i = 0; i < l->nmembers; i++){
    serve_req *r = &s->reqs[l->members[i]];
    r->rc = ODPX_ERR_CUDA; r->state = 2; r->t_done = now_s();
    s->graphs[r->graph].busy = 0;
    if(r->waiter) pthread_cond_signal(r->waiter);
  }
  l->busy = 0;
  l->nmembers = 0;
}

/* The scheduler thread.  Lanes belong to it alone: their CUDA calls (event
 * queries, copies, launches) run with the mutex released, so clients that
 * submit or wait are not held up by them; requests and graphs are touched
 * only with the mutex held. */
#define MAX_LANES 64
static void *scheduler(void *arg)
{
  odp_server *s = arg;
  /* the completion polling sleeps for microseconds: keep the kernel from
   * stretching them by its default 50 us timer slack */
  prctl(PR_SET_TIMERSLACK, 1UL, 0, 0, 0);
  const int nl = s->cfg.lanes < MAX_LANES ? s->cfg.lanes : MAX_LANES;
  int q[MAX_LANES];
  serve_lane *formed[MAX_LANES];
  pthread_mutex_lock(&s->mu);
  while(!s->stop){
    int progress = 0;
    /* completions: queried without the mutex */
    pthread_mutex_unlock(&s->mu);
    for(int i = 0; i < nl; i++) q[i] = s->lanes[i].busy ? gbx_event_query(s->lanes[i].ev) : 1;
    for(int i = 0; i < nl; i++)
      if(s->lanes[i].busy && q[i] != 0 && q[i] != 1) gbx_stream_sync(s->lanes[i].stream);  /* a CUDA error */
    pthread_mutex_lock(&s->mu);
    for(int i = 0; i < nl; i++)
      if(s->lanes[i].busy && q[i] != 1){ finish_batch(s, &s->lanes[i]); progress = 1; }
    if(progress && s->shared_waiters) pthread_cond_broadcast(&s->cv_done);
    /* With several lanes, lane 0 takes only the cheaper half of the cost
     * range (below the geometric mean of the registered graphs' costs), so
     * small requests always find a lane that large batches cannot hold. */
    const double small = nl > 1 ? sqrt(s->min_cost * s->max_cost) : HUGE_VAL;
    int nformed = 0;
    for(int i = 0; i < nl && s->next_pending < s->nreqs; i++){
      serve_lane *l = &s->lanes[i];
      if(!l->busy && form_batch(s, l, i == 0 ? small : HUGE_VAL) > 0) formed[nformed++] = l;
    }
    if(nformed){
      /* issued without the mutex; failures are handed back with it */
      pthread_mutex_unlock(&s->mu);
      int failed[MAX_LANES];
      for(int k = 0; k < nformed; k++) failed[k] = issue_batch(formed[k]) != 0;
      pthread_mutex_lock(&s->mu);
      for(int k = 0; k < nformed; k++) if(failed[k]) fail_batch(s, formed[k]);
      progress = 1;
    }
    int inflight = 0;
    for(int i = 0; i < nl; i++) inflight += s->lanes[i].busy;
    if(inflight > s->stats.max_inflight_lanes) s->stats.max_inflight_lanes = inflight;
    const int have_pending = s->next_pending < s->nreqs;
    if(!inflight && !have_pending){
      pthread_cond_wait(&s->cv_work, &s->mu);
    }
    else if(!progress){
      pthread_mutex_unlock(&s->mu);
      struct timespec ts = {0, 4000};                /* completion polling period */
      nanosleep(&ts, NULL);
      pthread_mutex_lock(&s->mu);
    }
  }
  pthread_mutex_unlock(&s->mu);
  return NULL;
}

/* ---------------------------------------------------------------------- */

int ODPX_Serve_create(const ODPX_Serve_config *cfg, ODPX_Server **out)
{
  *out = NULL;
  if(odp_device_ready()) return ODPX_ERR_CUDA;
  odp_server *s = calloc(1, sizeof(odp_server));
  ODPX_Serve_config c = cfg ? *cfg : (ODPX_Serve_config){0};
  if(c.lanes <= 0) c.lanes = 4;
  if(c.max_batch <= 0) c.max_batch = 16;
  if(c.max_nodes <= 0) c.max_nodes = 32768;
  if(c.memory_mb <= 0) c.memory_mb = 1024;
  if(c.wc_log2 <= 0) c.wc_log2 = 4;
  if(c.wc_log2 > 7) c.wc_log2 = 7;
  s->cfg = c;
  pthread_mutex_init(&s->mu, NULL);
  pthread_cond_init(&s->cv_work, NULL);
  pthread_cond_init(&s->cv_done, NULL);
  double per_slot = 2.0 * 8.0 * (double)((size_t)c.max_nodes << c.wc_log2);
  int slots_total = (int)((double)c.memory_mb * 1024.0 * 1024.0 / per_slot);
  int per_lane = slots_total / c.lanes;
  if(per_lane < 1){
    pthread_mutex_destroy(&s->mu);
    pthread_cond_destroy(&s->cv_work);
    pthread_cond_destroy(&s->cv_done);
    free(s);
    return ODPX_ERR_MEMORY;
  }
  if(per_lane > 256) per_lane = 256;
  int blocks = gbx_engine_blocks(0) / c.lanes;
  if(blocks < 1) blocks = 1;
  {
    const char *v = getenv("ODP_GB300_L2_MB");
    double mb = (v && *v) ? atof(v) : 80.0;
    s->l2_lane_bytes = mb * 1024.0 * 1024.0 / c.lanes;
  }
  s->lanes = calloc((size_t)c.lanes, sizeof(serve_lane));
  for(int i = 0; i < c.lanes; i++){
    int e = lane_init(&s->lanes[i], &c, per_lane, blocks);
    if(e){
      for(int k = 0; k <= i; k++) lane_free(&s->lanes[k]);
      free(s->lanes);
      free(s);
      return e;
    }
  }
  /* from here on a failure releases everything through ODPX_Serve_destroy,
   * which handles a server whose scheduler thread never started */
  if(gbx_stream_create(&s->ctl_stream)){
    s->ctl_stream = NULL;
    ODPX_Serve_destroy(s);
    return ODPX_ERR_CUDA;
  }
  s->stats.slots_per_lane = per_lane;
  s->stats.blocks_per_lane = blocks;
  if(pthread_create(&s->thread, NULL, scheduler, s) != 0){
    ODPX_Serve_destroy(s);
    return ODPX_ERR_STATE;
  }
  s->started = 1;
  *out = s;
  return 0;
}

int ODPX_Serve_register(ODPX_Server *s, const ODP_Graph *gr, int *handle)
{
  if(!s || !gr || !gr->adjacency || !handle) return ODPX_ERR_INVALID;
  int n = gr->grid ? gr->width * gr->height : gr->nodes;
  int sym = gr->symmetries;
  if(n <= 0 || sym <= 0 || n % sym || gr->degree < 1 || gr->degree > GBX_MAX_DEGREE) return ODPX_ERR_INVALID;
  int grid_s = gr->grid && sym != 1;
  if(grid_s && (sym != 2 && sym != 4)) grid_s = 0;           /* the general rule, as ODP_Init_aspl_grid_s */
  if(grid_s && ((gr->width % 2) || (sym == 4 && (gr->height % 2 || gr->width != gr->height)))) return ODPX_ERR_INVALID;
  if(n > s->cfg.max_nodes) return ODPX_ERR_MEMORY;          /* admission: the slot pools hold max_nodes rows */
  serve_graph g = {0};
  g.grid = gr->grid; g.grid_s = grid_s; g.n = n; g.d = gr->degree; g.dp = ALIGN_UP(gr->degree, 4);
  g.s = sym; g.B = n / sym; g.W = (g.B + 63) / 64; g.width = gr->width; g.height = gr->height;
  int full = ilog2_ceil(g.W < 2 ? 2 : g.W);
  g.wc_log2 = full < s->cfg.wc_log2 ? full : s->cfg.wc_log2;
  if(g.wc_log2 < 1) g.wc_log2 = 1;
  int wc = 1 << g.wc_log2;
  g.nchunks = (g.W + wc - 1) / wc;
  double level_bytes = (double)n * wc * 8.0 * (g.d + 2);
  int vpr = wc / 2, lanes_per_row = vpr < 32 ? vpr : 32, rpp = 8 * (32 / lanes_per_row);
  /* Tiles of about 640 KB; a smaller graph takes tiles small enough for
   * about two per CTA of its lane when it runs alone, so that a request does
   * not wait on one CTA while the rest of the lane idles. */
  int lane_blocks = s->lanes[0].blocks > 0 ? s->lanes[0].blocks : 1;
  double tile_bytes = level_bytes * g.nchunks / (2.0 * lane_blocks);
  if(tile_bytes > 640.0 * 1024.0) tile_bytes = 640.0 * 1024.0;
  if(tile_bytes < 32.0 * 1024.0) tile_bytes = 32.0 * 1024.0;
  if(level_bytes <= tile_bytes) g.tile_rows = n;
  else{
    int tr = (int)(tile_bytes / ((double)wc * 8.0 * (g.d + 2)));
    if(tr < rpp) tr = rpp;
    g.tile_rows = ALIGN_UP(tr, rpp);
    if(g.tile_rows > n) g.tile_rows = n;
  }
  g.ntiles = (n + g.tile_rows - 1) / g.tile_rows;
  g.cost = level_bytes * g.nchunks;
  if(g.nchunks > s->lanes[0].max_jobs) return ODPX_ERR_MEMORY;   /* one request must fit a batch */
  size_t adj_ints = (size_t)g.B * g.d;
  g.h_adj = malloc(sizeof(int) * adj_ints);
  memcpy(g.h_adj, gr->adjacency, sizeof(int) * adj_ints);
  int *h_nd = NULL;
  int e = 0;
  e |= gbx_malloc((void **)&g.d_adj, sizeof(int) * adj_ints);
  e |= gbx_malloc((void **)&g.d_nbr, sizeof(int) * (size_t)n * g.dp);
  e |= gbx_malloc((void **)&g.d_desc, sizeof(gbx_expand_desc));
  if(gr->num_degrees){
    g.h_rowdeg = malloc(sizeof(int) * (size_t)g.B);
    memcpy(g.h_rowdeg, gr->num_degrees, sizeof(int) * (size_t)g.B);
    /* per-vertex degrees as the Init variants expand them (odp_plan.c) */
    h_nd = malloc(sizeof(int) * (size_t)n);
    if(!grid_s || sym == 1){
      for(int t = 0; t < sym; t++) for(int j = 0; j < g.B; j++) h_nd[t * g.B + j] = gr->num_degrees[j];
    }
    else if(sym == 2){
      for(int i = 0; i < g.B; i++){ h_nd[i] = gr->num_degrees[i]; h_nd[rotate(i, g.width, g.height, 2, 180)] = gr->num_degrees[i]; }
    }
    else{
      for(int i = 0; i < g.B; i++){
        int v = (i / (g.height / 2)) * g.height + i % (g.height / 2);
        h_nd[v] = gr->num_degrees[i];
        for(int r = 90; r <= 270; r += 90) h_nd[rotate(v, g.width, g.height, 4, r)] = gr->num_degrees[i];
      }
    }
    e |= gbx_malloc((void **)&g.d_ndeg, sizeof(int) * (size_t)n);
    e |= gbx_memcpy_h2d(g.d_ndeg, h_nd, sizeof(int) * (size_t)n, s->ctl_stream);
  }
  if(grid_s){
    g.h_itable = malloc(sizeof(int) * (size_t)n);
    int base = n / sym;
    if(sym == 2){
      for(int i = 0; i < base; i++){ g.h_itable[i] = i; g.h_itable[rotate(i, g.width, g.height, 2, 180)] = i + base; }
    }
    else{
      int bh = g.height / 2;
      for(int i = 0; i < base; i++){
        int v = (i / bh) * g.height + (i % bh);
        g.h_itable[v] = i;
        for(int t = 1; t < 4; t++) g.h_itable[rotate(v, g.width, g.height, 4, 90 * t)] = i + base * t;
      }
    }
    e |= gbx_malloc((void **)&g.d_itable, sizeof(int) * (size_t)n);
    e |= gbx_memcpy_h2d(g.d_itable, g.h_itable, sizeof(int) * (size_t)n, s->ctl_stream);
  }
  gbx_expand_desc desc = {0};
  desc.adj = g.d_adj; desc.ndeg = g.d_ndeg; desc.itable = g.d_itable; desc.nbr = g.d_nbr;
  desc.n = n; desc.d = g.d; desc.dp = g.dp; desc.s = sym; desc.width = g.width; desc.height = g.height;
  desc.grid_s = grid_s;
  unsigned *d_err = NULL, h_err = 0;
  e |= gbx_malloc((void **)&d_err, sizeof(unsigned));
  e |= gbx_memset(d_err, 0, sizeof(unsigned), s->ctl_stream);
  e |= gbx_memcpy_h2d(g.d_adj, gr->adjacency, sizeof(int) * adj_ints, s->ctl_stream);
  e |= gbx_memcpy_h2d(g.d_desc, &desc, sizeof(desc), s->ctl_stream);
  e |= gbx_expand(g.d_desc, 1, n, g.dp, d_err, s->ctl_stream);
  e |= gbx_memcpy_d2h(&h_err, d_err, sizeof(unsigned), s->ctl_stream);
  e |= gbx_stream_sync(s->ctl_stream);
  gbx_free(d_err);
  free(h_nd);
  if(e || h_err){
    gbx_free(g.d_adj); gbx_free(g.d_nbr); gbx_free(g.d_desc); gbx_free(g.d_ndeg); gbx_free(g.d_itable);
    free(g.h_adj); free(g.h_itable); free(g.h_rowdeg);
    return e ? ODPX_ERR_CUDA : ODPX_ERR_ADJACENCY;
  }
  pthread_mutex_lock(&s->mu);
  if(s->ngraphs == s->cap_graphs){
    s->cap_graphs = s->cap_graphs ? 2 * s->cap_graphs : 16;
    s->graphs = realloc(s->graphs, sizeof(serve_graph) * (size_t)s->cap_graphs);
  }
  s->graphs[s->ngraphs] = g;
  if(s->ngraphs == 0 || g.cost < s->min_cost) s->min_cost = g.cost;
  if(s->ngraphs == 0 || g.cost > s->max_cost) s->max_cost = g.cost;
  *handle = s->ngraphs++;
  pthread_mutex_unlock(&s->mu);
  return 0;
}

int ODPX_Serve_submit(ODPX_Server *s, int handle, int ndelta, const ODPX_Delta *deltas, long long *request)
{
  if(!s || !request || ndelta < 0 || (ndelta > 0 && !deltas)) return ODPX_ERR_INVALID;
  pthread_mutex_lock(&s->mu);
  if(handle < 0 || handle >= s->ngraphs){ pthread_mutex_unlock(&s->mu); return ODPX_ERR_INVALID; }
  serve_graph *g = &s->graphs[handle];
  if((long long)ndelta * (1 + g->s) > s->lanes[0].max_writes){   /* one request must fit a batch */
    pthread_mutex_unlock(&s->mu);
    return ODPX_ERR_INVALID;
  }
  for(int k = 0; k < ndelta; k++){
    const ODPX_Delta *dl = &deltas[k];
    /* a slot beyond the row's degree holds no edge (the reference ignores
     * adjacency entries past num_degrees), so a delta may not target it */
    if(dl->row < 0 || dl->row >= g->B || dl->slot < 0 || dl->slot >= g->d || dl->value < 0 || dl->value >= g->n ||
       (g->h_rowdeg && dl->slot >= g->h_rowdeg[dl->row])){
      pthread_mutex_unlock(&s->mu);
      return ODPX_ERR_ADJACENCY;
    }
  }
  if(s->nreqs == s->cap_reqs){
    s->cap_reqs = s->cap_reqs ? 2 * s->cap_reqs : 1024;
    s->reqs = realloc(s->reqs, sizeof(serve_req) * (size_t)s->cap_reqs);
  }
  serve_req *r = &s->reqs[s->nreqs];
  memset(r, 0, sizeof(*r));
  r->graph = handle;
  if(ndelta){
    /* Deltas apply in order, but the device writes them all at once: keep
     * only the last update of each slot (an undo followed by a new swap may
     * touch the same one). */
    r->deltas = malloc(sizeof(ODPX_Delta) * (size_t)ndelta);
    int kept = 0;
    for(int k = 0; k < ndelta; k++){
      int later = 0;
      for(int q = k + 1; q < ndelta && !later; q++)
        later = deltas[q].row == deltas[k].row && deltas[q].slot == deltas[k].slot;
      if(!later) r->deltas[kept++] = deltas[k];
    }
    r->ndelta = kept;
  }
  r->t_submit = now_s();
  *request = s->nreqs++;
  pthread_cond_signal(&s->cv_work);
  pthread_mutex_unlock(&s->mu);
  return 0;
}

static void copy_result(const serve_req *r, int *diameter, long *sum, double *ASPL, double *latency_s)
{
  if(diameter) *diameter = r->diameter;
  if(sum) *sum = r->sum;
  if(ASPL) *ASPL = r->aspl;
  if(latency_s) *latency_s = r->t_done - r->t_submit;
}

int ODPX_Serve_wait(ODPX_Server *s, long long request, int *diameter, long *sum, double *ASPL, double *latency_s)
{
  if(!s) return ODPX_ERR_INVALID;
  pthread_mutex_lock(&s->mu);
  if(request < 0 || request >= s->nreqs){ pthread_mutex_unlock(&s->mu); return ODPX_ERR_INVALID; }
  /* the thread that waits for a request sleeps on a condition of its own,
   * which only that request's completion signals; a second thread waiting
   * for the same request uses the shared one */
  pthread_cond_t cv;
  int own = s->reqs[request].waiter == NULL && s->reqs[request].state != 2;
  if(own){
    pthread_cond_init(&cv, NULL);
    s->reqs[request].waiter = &cv;
    while(s->reqs[request].state != 2) pthread_cond_wait(&cv, &s->mu);
    s->reqs[request].waiter = NULL;
    pthread_cond_destroy(&cv);
  }
  else{
    s->shared_waiters++;
    while(s->reqs[request].state != 2) pthread_cond_wait(&s->cv_done, &s->mu);
    s->shared_waiters--;
  }
  serve_req *r = &s->reqs[request];
  copy_result(r, diameter, sum, ASPL, latency_s);
  int rc = r->rc;
  pthread_mutex_unlock(&s->mu);
  return rc;
}

int ODPX_Serve_poll(ODPX_Server *s, long long request, int *diameter, long *sum, double *ASPL, double *latency_s)
{
  if(!s) return ODPX_ERR_INVALID;
  pthread_mutex_lock(&s->mu);
  if(request < 0 || request >= s->nreqs){ pthread_mutex_unlock(&s->mu); return ODPX_ERR_INVALID; }
  serve_req *r = &s->reqs[request];
  int rc = ODPX_PENDING;
  if(r->state == 2){
    copy_result(r, diameter, sum, ASPL, latency_s);
    rc = r->rc;
  }
  pthread_mutex_unlock(&s->mu);
  return rc;
}

int ODPX_Serve_stats(ODPX_Server *s, ODPX_Serve_counters *st)
{
  if(!s || !st) return ODPX_ERR_INVALID;
  pthread_mutex_lock(&s->mu);
  *st = s->stats;
  pthread_mutex_unlock(&s->mu);
  return 0;
}

int ODPX_Serve_adjacency(ODPX_Server *s, int handle, int *adjacency)
{
  if(!s || !adjacency) return ODPX_ERR_INVALID;
  pthread_mutex_lock(&s->mu);
  if(handle < 0 || handle >= s->ngraphs){ pthread_mutex_unlock(&s->mu); return ODPX_ERR_INVALID; }
  serve_graph *g = &s->graphs[handle];
  s->shared_waiters++;
  while(g->busy) pthread_cond_wait(&s->cv_done, &s->mu);
  s->shared_waiters--;
  /* also wait until no pending request carries deltas for it */
  size_t bytes = sizeof(int) * (size_t)g->B * g->d;
  int e = gbx_memcpy_d2h(adjacency, g->d_adj, bytes, s->ctl_stream) | gbx_stream_sync(s->ctl_stream);
  pthread_mutex_unlock(&s->mu);
  return e ? ODPX_ERR_CUDA : 0;
}

void ODPX_Serve_destroy(ODPX_Server *s)
{
  if(!s) return;
  pthread_mutex_lock(&s->mu);
  s->stop = 1;
  pthread_cond_broadcast(&s->cv_work);
  pthread_mutex_unlock(&s->mu);
  if(s->started) pthread_join(s->thread, NULL);
  for(int i = 0; i < s->cfg.lanes; i++) lane_free(&s->lanes[i]);
  free(s->lanes);
  for(int i = 0; i < s->ngraphs; i++){
    serve_graph *g = &s->graphs[i];
    gbx_free(g->d_adj); gbx_free(g->d_nbr); gbx_free(g->d_desc); gbx_free(g->d_ndeg); gbx_free(g->d_itable);
    free(g->h_adj); free(g->h_itable); free(g->h_rowdeg);
  }
  free(s->graphs);
  for(long long i = 0; i < s->nreqs; i++) free(s->reqs[i].deltas);
  free(s->reqs);
  if(s->ctl_stream) gbx_stream_destroy(s->ctl_stream);
  pthread_mutex_destroy(&s->mu);
  pthread_cond_destroy(&s->cv_work);
  pthread_cond_destroy(&s->cv_done);
  free(s);
}

/*
 * odp_anneal.c -- host side of the device-resident annealing chains
 * (ODPX_Anneal_*, kernels in anneal.cu).
 *
 * A set of chains is one batch plan (odp_plan.c): every chain's graph is a
 * graph of the plan, uploaded and expanded once.  A step is four stream-ordered
 * operations and no host round trip: the proposal kernel, a device-to-device
 * reset of the engine state, the engine, and the decision kernel.  The host
 * only reads state back when asked.
 *
 * Each chain follows the reference's annealing client (sample/SA/general.c:
 * 130-191, general_s.c:152-191): temp starts at max_temp and is multiplied by
 * cooling_rate = pow(min_temp / max_temp, 1.0 / ncalcs) after every step
 * (0 for hill climbing), the best graph is kept, and accept_s decides.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "odp_plan.h"
#include "odp_rng.h"
#include "odp_gb300.h"

#define ANNEAL_GRAPH_STEPS 8   /* steps per replayed CUDA graph */

struct odpx_anneal {
  odp_plan *p;
  int count;
  gbx_chain *h_chains, *d_chains;
  int *d_best, *d_rowdeg;
  char *d_state_init;
  void *steps_exec;            /* ANNEAL_GRAPH_STEPS steps captured as one CUDA graph */
};

static int chain_nodes(const ODPX_Chain *c)
{
  return c->grid ? c->width * c->height : c->nodes;
}

static int check_chain(const ODPX_Chain *c)
{
  if(!c->adjacency || c->degree <= 0 || c->symmetries <= 0) return ODPX_ERR_INVALID;
  if(c->grid){
    /* the grid 2-opt takes s = 1, 2 or 4 (utils.c:125-133), 4 on square grids */
    if(c->width <= 0 || c->height <= 0 || c->length <= 0) return ODPX_ERR_INVALID;
    if(c->symmetries != 1 && c->symmetries != 2 && c->symmetries != 4) return ODPX_ERR_INVALID;
    if(c->symmetries > 1 && c->width % 2) return ODPX_ERR_INVALID;
    if(c->symmetries == 4 && (c->height % 2 || c->width != c->height)) return ODPX_ERR_INVALID;
  }
  else if(c->nodes <= 0) return ODPX_ERR_INVALID;
  if(chain_nodes(c) % c->symmetries) return ODPX_ERR_INVALID;
  if(!c->hill_climbing && (!(c->max_temp > 0) || !(c->min_temp > 0) || c->ncalcs <= 0)) return ODPX_ERR_INVALID;
  if(c->num_degrees){
    int base = chain_nodes(c) / c->symmetries;
    for(int i = 0; i < base; i++)
      if(c->num_degrees[i] < 0 || c->num_degrees[i] > c->degree) return ODPX_ERR_INVALID;
  }
  return 0;
}

void ODPX_Anneal_destroy(ODPX_Anneal *a)
{
  if(!a) return;
  if(a->steps_exec) gbx_graph_destroy(a->steps_exec);
  if(a->p) odp_plan_destroy(a->p);
  gbx_free(a->d_chains); gbx_free(a->d_best); gbx_free(a->d_rowdeg); gbx_free(a->d_state_init);
  free(a->h_chains);
  free(a);
}

#define CK(call) do{ if(call){ rc = ODPX_ERR_CUDA; goto fail; } }while(0)

int ODPX_Anneal_create(const ODPX_Chain *chains, int count, ODPX_Anneal **out)
{
  if(!out || !chains || count <= 0) return ODPX_ERR_INVALID;
  *out = NULL;
  for(int i = 0; i < count; i++){
    int e = check_chain(&chains[i]);
    if(e) return e;
  }
  if(odp_device_ready()) return ODPX_ERR_CUDA;
  int rc = 0;
  ODPX_Anneal *a = calloc(1, sizeof(ODPX_Anneal));
  odp_shape *shapes = calloc((size_t)count, sizeof(odp_shape));
  const int **adj = calloc((size_t)count, sizeof(int *));
  odp_result *res = calloc((size_t)count, sizeof(odp_result));
  if(!a || !shapes || !adj || !res){ rc = ODPX_ERR_MEMORY; goto fail; }
  a->count = count;
  for(int i = 0; i < count; i++){
    shapes[i].grid = chains[i].grid != 0;
    shapes[i].nodes = chain_nodes(&chains[i]);
    shapes[i].width = chains[i].width;
    shapes[i].height = chains[i].height;
    shapes[i].degree = chains[i].degree;
    shapes[i].symmetries = chains[i].symmetries;
    shapes[i].num_degrees = chains[i].num_degrees;
    adj[i] = chains[i].adjacency;
  }
  odp_tuning t;
  odp_tuning_defaults(&t, count > 1);
  t.reorder = 0;                      /* the job order is fixed once the steps run on the device */
  t.direct = 0;                       /* the chains update the plan's device copy of the adjacency */
  /* Chain groups run side by side on parts of the GPU.  The small-graph
   * kernel's CTAs (512 threads, up to 200 KB of shared memory) do not fit on
   * SMs that hold other groups' engine CTAs: with four groups on four
   * streams, 1024-vertex chains ran at 52k instead of 121k evals/s. */
  t.small_n = 0;
  if((rc = odp_plan_create(shapes, count, &t, &a->p))) goto fail;
  odp_plan *p = a->p;
  /* the starting graphs' evaluation; it also uploads and expands them */
  if((rc = odp_plan_run(p, adj, res))) goto fail;

  size_t best_ints = 0, deg_ints = 0;
  for(int i = 0; i < count; i++){
    best_ints += ((size_t)p->g[i].B * p->g[i].d + 3) & ~(size_t)3;   /* 16-byte aligned copies */
    if(chains[i].num_degrees) deg_ints += (size_t)p->g[i].B;
  }
  CK(gbx_malloc((void **)&a->d_best, sizeof(int) * (best_ints ? best_ints : 1)));
  if(deg_ints) CK(gbx_malloc((void **)&a->d_rowdeg, sizeof(int) * deg_ints));
  CK(gbx_malloc((void **)&a->d_state_init, p->state_bytes));
  CK(gbx_malloc((void **)&a->d_chains, sizeof(gbx_chain) * (size_t)count));
  a->h_chains = calloc((size_t)count, sizeof(gbx_chain));
  if(!a->h_chains){ rc = ODPX_ERR_MEMORY; goto fail; }

  size_t boff = 0, doff = 0;
  for(int i = 0; i < count; i++){
    const ODPX_Chain *in = &chains[i];
    const odp_plan_graph *g = &p->g[i];
    gbx_chain *c = &a->h_chains[i];
    size_t words = (size_t)g->B * g->d;
    c->n = g->n; c->d = g->d; c->dp = g->dp; c->s = g->s; c->base = g->B; c->graph = i;
    c->grid = in->grid != 0;
    c->width = in->width; c->height = in->height; c->len = in->length;
    c->itable = g->has_itable ? p->d_itable + g->itable_off : NULL;
    c->adj = p->d_adj + g->adj_off;
    c->nbr = p->d_nbr + g->nbr_off;
    c->best_adj = a->d_best + boff;
    CK(gbx_memcpy_h2d(c->best_adj, in->adjacency, sizeof(int) * words, p->stream));
    boff += (words + 3) & ~(size_t)3;
    if(in->num_degrees){
      CK(gbx_memcpy_h2d(a->d_rowdeg + doff, in->num_degrees, sizeof(int) * (size_t)g->B, p->stream));
      c->ndeg = a->d_rowdeg + doff;
      doff += (size_t)g->B;
    }
    odp_rng rng;
    odp_rng_seed(&rng, in->seed);     /* ODP_Srand(seed): no output drawn yet */
    for(int k = 0; k < 31; k++) c->ring[k] = rng.line[k];
    c->ring_pos = 0;
    c->cur_diameter = c->best_diameter = res[i].diameter;
    c->cur_sum = c->best_sum = res[i].sum;
    c->cur_aspl = c->best_aspl = res[i].aspl;
    c->temp = in->hill_climbing ? 0.0 : in->max_temp;
    c->cooling = in->hill_climbing ? 0.0 : pow(in->min_temp / in->max_temp, (double)1.0 / in->ncalcs);
    c->hill_climbing = in->hill_climbing != 0;
    c->aspl_priority = in->aspl_priority != 0;
  }
  CK(gbx_memcpy_h2d(a->d_state_init, p->h_state_init, p->state_bytes, p->stream));
  CK(gbx_memcpy_h2d(a->d_chains, a->h_chains, sizeof(gbx_chain) * (size_t)count, p->stream));
  CK(gbx_stream_sync(p->stream));
  free(shapes); free(adj); free(res);
  *out = a;
  return 0;

fail:
  free(shapes); free(adj); free(res);
  ODPX_Anneal_destroy(a);
  return rc;
}

/* One step in stream order: propose, reset the engine state, evaluate, decide. */
static int enqueue_step(ODPX_Anneal *a)
{
  odp_plan *p = a->p;
  gbx_ctrl *ctrl = (gbx_ctrl *)(p->d_state + p->out_off);
  const unsigned int *err = (const unsigned int *)(p->d_state + p->out_off + sizeof(gbx_ctrl));
  const gbx_graph_acc *acc = (const gbx_graph_acc *)(p->d_state + p->acc_off);
  if(gbx_anneal_propose(a->d_chains, a->count, p->stream)) return ODPX_ERR_CUDA;
  if(gbx_memcpy_d2d(p->d_state, a->d_state_init, p->state_bytes, p->stream)) return ODPX_ERR_CUDA;
  if(odp_plan_enqueue_engine(p)) return ODPX_ERR_CUDA;
  if(gbx_anneal_decide(a->d_chains, a->count, acc, ctrl, err, p->stream)) return ODPX_ERR_CUDA;
  return 0;
}

int ODPX_Anneal_run(ODPX_Anneal *a, int steps)
{
  if(!a || steps < 0) return ODPX_ERR_INVALID;
  odp_plan *p = a->p;
  int s = 0;
  if(steps >= ANNEAL_GRAPH_STEPS){
    /* full groups of steps replay one captured graph: a launch per group
     * instead of four operations per step */
    if(!a->steps_exec){
      if(gbx_capture_begin(p->stream)) return ODPX_ERR_CUDA;
      int e = 0;
      for(int k = 0; k < ANNEAL_GRAPH_STEPS && !e; k++) e = enqueue_step(a);
      void *ge = NULL;
      int e2 = gbx_capture_end(p->stream, &ge);
      if(e || e2) return ODPX_ERR_CUDA;
      a->steps_exec = ge;
    }
    for(; s + ANNEAL_GRAPH_STEPS <= steps; s += ANNEAL_GRAPH_STEPS)
      if(gbx_graph_launch(a->steps_exec, p->stream)) return ODPX_ERR_CUDA;
  }
  for(; s < steps; s++)
    if(enqueue_step(a)) return ODPX_ERR_CUDA;
  return gbx_stream_sync(p->stream) ? ODPX_ERR_CUDA : 0;
}

int ODPX_Anneal_state(ODPX_Anneal *a, int chain, ODPX_Chain_state *st, int *adjacency, int *best_adjacency)
{
  if(!a || chain < 0 || chain >= a->count) return ODPX_ERR_INVALID;
  odp_plan *p = a->p;
  gbx_chain *c = &a->h_chains[chain];
  if(gbx_memcpy_d2h(c, a->d_chains + chain, sizeof(gbx_chain), p->stream)) return ODPX_ERR_CUDA;
  size_t words = (size_t)c->base * c->d;
  if(adjacency && gbx_memcpy_d2h(adjacency, c->adj, sizeof(int) * words, p->stream)) return ODPX_ERR_CUDA;
  if(best_adjacency && gbx_memcpy_d2h(best_adjacency, c->best_adj, sizeof(int) * words, p->stream))
    return ODPX_ERR_CUDA;
  if(gbx_stream_sync(p->stream)) return ODPX_ERR_CUDA;
  if(st){
    st->steps = c->steps;
    st->accepted = c->accepted;
    st->status = c->status;
    st->diameter = c->cur_diameter;
    st->sum = (long)c->cur_sum;
    st->aspl = c->cur_aspl;
    st->best_diameter = c->best_diameter;
    st->best_sum = (long)c->best_sum;
    st->best_aspl = c->best_aspl;
    st->temp = c->temp;
  }
  return 0;
}

/*
 * serve_load.c -- a native client of the serving API (ODPX_Serve_*), used by
 * bench.py to drive the served simulated-annealing workload without a
 * Python client in the loop.  Not part of the library: a separate program
 * linked against libodp_gb300.so.
 *
 * Each chain is a host thread that runs the annealing loop of the
 * reference's samples (sample/SA/general.c:149-181) against a served graph:
 * a 2-opt proposal from its own random stream (ODPX_Mutate_adjacency_
 * general_s_rng), an evaluation request carrying the adjacency slots the
 * proposal rewrote (and the undo of the previous proposal when that one was
 * rejected), Metropolis acceptance at a fixed temperature, and the host-side
 * undo (ODPX_Restore_adjacency_general_s) of a rejected move.  Closed loop:
 * one request outstanding per chain, with an exponentially distributed think
 * time before each proposal (mean THINK_US; 0: none, the chains saturate the
 * server).  At the end every chain's served graph is evaluated once more and
 * compared bit for bit with the same graph evaluated alone by a fresh plan.
 *
 *   serve_load SECONDS THINK_US LANES MAX_BATCH MEMORY_MB TEMPERATURE N:D:SEED:PSEED ...
 *
 * Prints one JSON object: completed requests, seconds, evals/s, latency
 * percentiles overall and per n, and how many final results were checked.
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "odp.h"
#include "odp_gb300.h"

typedef struct {
  int n, d;
  unsigned seed, pseed;
  int handle;
  int *adj;                  /* the client's copy, kept equal to the served graph */
  void *rng;
  double *lat;               /* latency of every request (s) */
  long long nlat, cap;
  ODPX_Delta undo[4];
  int nundo;
  int final_d; long final_s; double final_a;
  int error;
} chain_t;

static ODPX_Server *g_srv;
static double g_stop, g_think_s, g_temp;

static double now_s(void)
{
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* Uniform in (0, 1) from the chain's stream (31-bit draws). */
static double uniform(void *rng) { return ((double)ODPX_Rng_next(rng) + 0.5) / 2147483648.0; }

/* The slots a 2-opt move (its ODP_Restore record) touched, with their current values. */
static int move_deltas(const chain_t *c, const ODP_Restore *r, ODPX_Delta *out)
{
  int k = 0;
  for(int i = 0; i < 2; i++){
    out[k].row = r->u[i]; out[k].slot = r->u_d[i]; out[k].value = c->adj[(size_t)r->u[i] * c->d + r->u_d[i]]; k++;
    out[k].row = r->v[i]; out[k].slot = r->v_d[i]; out[k].value = c->adj[(size_t)r->v[i] * c->d + r->v_d[i]]; k++;
  }
  return k;
}

static void record(chain_t *c, double lat)
{
  if(c->nlat == c->cap){
    c->cap = c->cap ? 2 * c->cap : 4096;
    c->lat = realloc(c->lat, sizeof(double) * (size_t)c->cap);
  }
  c->lat[c->nlat++] = lat;
}

static void *chain_main(void *arg)
{
  chain_t *c = arg;
  int dm; long sm; double current, lat;
  long long req;
  if(ODPX_Serve_submit(g_srv, c->handle, 0, NULL, &req) || ODPX_Serve_wait(g_srv, req, &dm, &sm, &current, &lat)){
    c->error = 1;
    return NULL;
  }
  const double pairs = (double)c->n * (c->n - 1) / 2.0;
  while(now_s() < g_stop){
    if(g_think_s > 0){
      double t = -g_think_s * log(uniform(c->rng));
      struct timespec ts = { (time_t)t, (long)((t - floor(t)) * 1e9) };
      nanosleep(&ts, NULL);
    }
    ODP_Restore r;
    ODPX_Mutate_adjacency_general_s_rng(c->rng, c->n, c->d, NULL, 1, &r, c->adj);
    ODPX_Delta deltas[8];
    int nd = 0;
    for(int i = 0; i < c->nundo; i++) deltas[nd++] = c->undo[i];
    nd += move_deltas(c, &r, deltas + nd);
    double a;
    if(ODPX_Serve_submit(g_srv, c->handle, nd, deltas, &req) || ODPX_Serve_wait(g_srv, req, &dm, &sm, &a, &lat)){
      c->error = 1;
      return NULL;
    }
    record(c, lat);
    if(a <= current || uniform(c->rng) < exp(-(a - current) * pairs / g_temp)){
      current = a;
      c->nundo = 0;
    }
    else{
      ODPX_Restore_adjacency_general_s(c->n, c->d, 1, r, c->adj);
      c->nundo = move_deltas(c, &r, c->undo);
    }
  }
  /* the served graph brought back to the client's copy, evaluated once more */
  if(ODPX_Serve_submit(g_srv, c->handle, c->nundo, c->undo, &req) ||
     ODPX_Serve_wait(g_srv, req, &c->final_d, &c->final_s, &c->final_a, &lat))
    c->error = 1;
  return NULL;
}

static int cmp_double(const void *a, const void *b)
{
  double x = *(const double *)a, y = *(const double *)b;
  return x < y ? -1 : x > y;
}

static double pct(const double *v, long long n, double p)
{
  if(n == 0) return 0.0;
  double pos = p / 100.0 * (double)(n - 1);
  long long i = (long long)pos;
  double f = pos - (double)i;
  return i + 1 < n ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

int main(int argc, char **argv)
{
  if(argc < 8){
    fprintf(stderr, "usage: serve_load SECONDS THINK_US LANES MAX_BATCH MEMORY_MB TEMPERATURE N:D:SEED:PSEED ...\n");
    return 2;
  }
  const double seconds = atof(argv[1]);
  g_think_s = atof(argv[2]) * 1e-6;
  g_temp = atof(argv[6]);
  const int nchains = argc - 7;
  chain_t *ch = calloc((size_t)nchains, sizeof(chain_t));
  int max_n = 0;
  for(int i = 0; i < nchains; i++){
    if(sscanf(argv[7 + i], "%d:%d:%u:%u", &ch[i].n, &ch[i].d, &ch[i].seed, &ch[i].pseed) != 4) return 2;
    if(ch[i].n > max_n) max_n = ch[i].n;
  }
  ODPX_Serve_config cfg = { atoi(argv[3]), atoi(argv[4]), max_n, atoi(argv[5]), 0 };
  if(ODPX_Serve_create(&cfg, &g_srv)){ fprintf(stderr, "serve_load: ODPX_Serve_create failed\n"); return 3; }
  for(int i = 0; i < nchains; i++){
    chain_t *c = &ch[i];
    const int lines = c->n * c->d / 2;
    int (*edge)[2] = malloc(sizeof(int) * 2 * (size_t)lines);
    c->adj = malloc(sizeof(int) * (size_t)c->n * c->d);
    ODPX_Generate_random_general_seeded(c->seed, c->n, c->d, 1, edge);
    ODP_Conv_edge2adjacency_general(c->n, lines, c->d, edge, c->adj);
    free(edge);
    ODP_Graph g = { 0, c->n, 0, 0, c->d, 1, NULL, c->adj };
    if(ODPX_Serve_register(g_srv, &g, &c->handle)){ fprintf(stderr, "serve_load: register failed\n"); return 3; }
    c->rng = malloc(ODPX_Rng_size());
    ODPX_Rng_seed(c->rng, c->pseed);
  }
  pthread_t *th = malloc(sizeof(pthread_t) * (size_t)nchains);
  const double t0 = now_s();
  g_stop = t0 + seconds;
  for(int i = 0; i < nchains; i++) pthread_create(&th[i], NULL, chain_main, &ch[i]);
  for(int i = 0; i < nchains; i++) pthread_join(th[i], NULL);
  const double wall = now_s() - t0;
  ODPX_Serve_counters st;
  ODPX_Serve_stats(g_srv, &st);
  ODPX_Serve_destroy(g_srv);

  /* every chain's last served result against its graph evaluated alone */
  int checked = 0, mismatched = 0, errors = 0;
  for(int i = 0; i < nchains; i++){
    chain_t *c = &ch[i];
    if(c->error){ errors++; continue; }
    ODP_Graph g = { 0, c->n, 0, 0, c->d, 1, NULL, c->adj };
    ODPX_Batch *b = NULL;
    int dm; long sm; double a;
    const int *adjp = c->adj;
    if(ODPX_Batch_create(1, &g, &b) || ODPX_Batch_run(b, &adjp, &dm, &sm, &a)){ errors++; ODPX_Batch_destroy(b); continue; }
    ODPX_Batch_destroy(b);
    checked++;
    if(dm != c->final_d || sm != c->final_s || memcmp(&a, &c->final_a, sizeof(double)) != 0) mismatched++;
  }

  long long total = 0;
  for(int i = 0; i < nchains; i++) total += ch[i].nlat;
  double *all = malloc(sizeof(double) * (size_t)(total ? total : 1));
  long long k = 0;
  for(int i = 0; i < nchains; i++){ memcpy(all + k, ch[i].lat, sizeof(double) * (size_t)ch[i].nlat); k += ch[i].nlat; }
  qsort(all, (size_t)total, sizeof(double), cmp_double);
  printf("{\"completed\": %lld, \"seconds\": %.6f, \"evals_per_s\": %.3f, \"latency_ms\": {\"p50\": %.6f, "
         "\"p99\": %.6f}, \"checked\": %d, \"mismatched\": %d, \"errors\": %d, \"batches\": %lld, "
         "\"mean_batch\": %.4f, \"max_batch\": %d, \"max_concurrent_lanes\": %d, \"by_n\": {",
         total, wall, (double)total / wall, 1e3 * pct(all, total, 50), 1e3 * pct(all, total, 99), checked, mismatched,
         errors, st.batches, st.batches ? (double)st.batched_requests / (double)st.batches : 0.0, st.max_batch,
         st.max_inflight_lanes);
  /* per graph size */
  int first = 1;
  for(int i = 0; i < nchains; i++){
    int seen = 0;
    for(int j = 0; j < i; j++) if(ch[j].n == ch[i].n) seen = 1;
    if(seen) continue;
    long long m = 0;
    for(int j = 0; j < nchains; j++) if(ch[j].n == ch[i].n) m += ch[j].nlat;
    double *v = malloc(sizeof(double) * (size_t)(m ? m : 1));
    long long q = 0;
    for(int j = 0; j < nchains; j++)
      if(ch[j].n == ch[i].n){ memcpy(v + q, ch[j].lat, sizeof(double) * (size_t)ch[j].nlat); q += ch[j].nlat; }
    qsort(v, (size_t)m, sizeof(double), cmp_double);
    printf("%s\"%d\": {\"requests\": %lld, \"evals_per_s\": %.3f, \"p50\": %.6f, \"p99\": %.6f}", first ? "" : ", ",
           ch[i].n, m, (double)m / wall, 1e3 * pct(v, m, 50), 1e3 * pct(v, m, 99));
    first = 0;
    free(v);
  }
  printf("}}\n");
  return (mismatched || errors) ? 4 : 0;
}

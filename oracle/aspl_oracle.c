/*
 * aspl_oracle.c -- TEST INFRASTRUCTURE ONLY.  A CPU restatement of the
 * reference ODP ASPL evaluation, used as the parity checker for the GPU
 * library and as the timed CPU baseline ("port").  The product never links,
 * loads or calls this file.
 *
 * It follows the reference CPU driver step for step:
 *   - state set-up and num_degrees expansion      aspl.c:121-164, 223-288
 *   - MATRIX kind: identity, level loop, sums     aspl.c:35-75
 *   - MATRIX_SAVING kind: CPU_CHUNK columns       aspl.c:77-119
 *   - the OR-gather ("matmul") for s == 1, general symmetry and grid
 *     symmetry                                    utils.c:1815-1861, 1938-1984
 *   - grid index maps and the row table           utils.c:67-88, 189-247, 2103-2124
 *   - disconnected graphs -> INT_MAX/LONG_MAX/DBL_MAX   aspl.c:332-336
 * with plain C loops (the reference's AVX2 variant computes the same words)
 * and OpenMP over rows, as libodp_threads.a does.  Pinned against the
 * reference library's own outputs by tests/test_oracle.py and the committed
 * fixtures in tests/golden/.
 *
 * C ABI (ctypes): oracle_new / oracle_set / oracle_free, see below.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <limits.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KIND_MATRIX 1
#define KIND_SAVING 2
#define ORACLE_CHUNK 24        /* CPU_CHUNK, parameter.h:9 */

typedef struct {
  int nodes, degree, symmetries, height, grid_s, kind;
  int *num_degrees;            /* n entries, expanded like the reference, or NULL */
  int *itable;                 /* grid symmetry only */
  unsigned elements;           /* 64-bit words per row (MATRIX) */
  uint64_t *A, *B;
} oracle_t;

static int rot(int v, int width, int height, int s, int deg)        /* utils.c:67-88 */
{
  int w = v / height, h = v % height;
  if(s == 2) return (width - w - 1) * height + (height - h - 1);
  if(deg == 90)  return h * height + (height - w - 1);
  if(deg == 180) return (height - w - 1) * height + (height - h - 1);
  return (height - h - 1) * height + w;
}

static int local_index(int x, int height, int s)                     /* utils.c:189-211 */
{
  if(s != 4) return x;
  return (x / height) * (height / 2) + x % height;
}

static int grid_adj(int width, int height, int degree, int s, const int *adj, int v, int j)  /* utils.c:214-247 */
{
  if(s == 1) return adj[v * degree + j];
  int w = v / height, h = v % height, bw = width / 2, bh = height / 2;
  if(s == 2){
    if(w < bw) return adj[v * degree + j];
    return rot(adj[rot(v, width, height, s, 180) * degree + j], width, height, s, 180);
  }
  if(w < bw && h < bh) return adj[local_index(v, height, s) * degree + j];
  if(w < bw)  return rot(adj[local_index(rot(v, width, height, s, 270), height, s) * degree + j], width, height, s, 90);
  if(h >= bh) return rot(adj[local_index(rot(v, width, height, s, 180), height, s) * degree + j], width, height, s, 180);
  return rot(adj[local_index(rot(v, width, height, s, 90), height, s) * degree + j], width, height, s, 270);
}

static void make_itable(int width, int height, int s, int *itable)   /* utils.c:2103-2124 */
{
  int base = (width * height) / s;
  if(s == 2){
    for(int i = 0; i < base; i++){
      itable[i] = i;
      itable[rot(i, width, height, s, 180)] = i + base;
    }
  }
  else{
    int bh = height / 2;
    for(int i = 0; i < base; i++){
      int v = (i / bh) * height + (i % bh);
      itable[v] = i;
      itable[rot(v, width, height, s, 90)]  = i + base;
      itable[rot(v, width, height, s, 180)] = i + base * 2;
      itable[rot(v, width, height, s, 270)] = i + base * 3;
    }
  }
}

/* kind: 0 = reference default (MATRIX when its estimate is <= 2048 MB,
 * utils.c:1238-1266 with is_cpu), 1 = MATRIX, 2 = MATRIX_SAVING.
 * grid: 0 general, 1 grid.  num_degrees as passed to ODP_Init_aspl_* (may be NULL). */
oracle_t *oracle_new(int grid, int width_or_nodes, int height, int degree, const int *num_degrees,
                     int symmetries, int kind)
{
  oracle_t *o = calloc(1, sizeof(oracle_t));
  int nodes = grid ? width_or_nodes * height : width_or_nodes;
  int width = grid ? width_or_nodes : 0;
  if(symmetries <= 0 || nodes % symmetries != 0){
    fprintf(stderr, "nodes(%d) must be divisible by symmetries(%d)\n", nodes, symmetries);
    free(o);
    return NULL;
  }
  o->nodes = nodes; o->degree = degree; o->symmetries = symmetries;
  o->height = grid ? height : -1;
  o->grid_s = grid && (symmetries == 2 || symmetries == 4);
  if(o->grid_s){
    o->itable = malloc(sizeof(int) * (size_t)nodes);
    make_itable(width, height, symmetries, o->itable);
  }
  if(num_degrees){                                   /* aspl.c:226-280 */
    o->num_degrees = malloc(sizeof(int) * (size_t)nodes);
    int base = nodes / symmetries;
    if(!grid || symmetries == 1){
      for(int i = 0; i < symmetries; i++)
        for(int j = 0; j < base; j++) o->num_degrees[i * base + j] = num_degrees[j];
    }
    else if(symmetries == 2){
      for(int i = 0; i < base; i++){
        o->num_degrees[i] = num_degrees[i];
        o->num_degrees[rot(i, width, height, 2, 180)] = num_degrees[i];
      }
    }
    else{
      for(int i = 0; i < base; i++){
        int v = (i / (height / 2)) * height + i % (height / 2);
        o->num_degrees[v] = num_degrees[i];
        o->num_degrees[rot(v, width, height, 4, 90)]  = num_degrees[i];
        o->num_degrees[rot(v, width, height, 4, 180)] = num_degrees[i];
        o->num_degrees[rot(v, width, height, 4, 270)] = num_degrees[i];
      }
    }
  }
  if(kind == 0){
    double mb = nodes * ((double)nodes / (4.0 * symmetries));
    if(o->grid_s) mb += sizeof(int) * (double)nodes;
    mb /= 1024.0 * 1024.0;
    kind = (mb <= 2048) ? KIND_MATRIX : KIND_SAVING;
  }
  o->kind = kind;
  o->elements = (unsigned)((nodes / symmetries + 63) / 64);
  size_t words = (size_t)nodes * (kind == KIND_MATRIX ? o->elements : ORACLE_CHUNK);
  o->A = malloc(words * sizeof(uint64_t));
  o->B = malloc(words * sizeof(uint64_t));
  if(!o->A || !o->B){ free(o->A); free(o->B); free(o); return NULL; }
  return o;
}

void oracle_free(oracle_t *o)
{
  if(!o) return;
  free(o->A); free(o->B); free(o->num_degrees); free(o->itable); free(o);
}

int oracle_kind(const oracle_t *o) { return o->kind; }

/* B[row(i)] |= OR_j A[row(nbr(i, j))] over `words` words per row. */
static void or_gather(const oracle_t *o, const int *adj, const uint64_t *A, uint64_t *B, unsigned words)
{
  const int nodes = o->nodes, degree = o->degree, s = o->symmetries;
  const int base = nodes / s;
  const int width = o->grid_s ? nodes / o->height : 0;
#pragma omp parallel for schedule(static)
  for(int i = 0; i < nodes; i++){
    int d = o->num_degrees ? o->num_degrees[i] : degree;
    size_t row = o->grid_s ? (size_t)o->itable[i] : (size_t)i;
    uint64_t *b = B + row * words;
    for(int j = 0; j < d; j++){
      int nb;
      if(s == 1)         nb = adj[(size_t)i * degree + j];
      else if(o->grid_s) nb = o->itable[grid_adj(width, o->height, degree, s, adj, i, j)];
      else{
        int p = i / base, m = i - p * base;
        nb = adj[(size_t)m * degree + j] + p * base;
        if(nb >= nodes) nb -= nodes;
      }
      const uint64_t *a = A + (size_t)nb * words;
      for(unsigned k = 0; k < words; k++) b[k] |= a[k];
    }
  }
}

static uint64_t count_bits(const uint64_t *B, size_t words)
{
  uint64_t num = 0;
#pragma omp parallel for reduction(+:num) schedule(static)
  for(size_t i = 0; i < words; i++) num += (uint64_t)__builtin_popcountll(B[i]);
  return num;
}

static void run_matrix(oracle_t *o, const int *adj, int *diameter, long *sum, double *ASPL)   /* aspl.c:35-75 */
{
  const int nodes = o->nodes, s = o->symmetries;
  const unsigned el = o->elements;
  size_t total = (size_t)nodes * el;
  memset(o->A, 0, total * sizeof(uint64_t));
  memset(o->B, 0, total * sizeof(uint64_t));
  for(int i = 0; i < nodes / s; i++){
    size_t off = (size_t)i * el + i / 64;
    o->A[off] = o->B[off] = 1ULL << (i % 64);
  }
  *sum = (long)nodes * (nodes - 1);
  *diameter = 1;
  for(int kk = 0; kk < nodes; kk++){
    or_gather(o, adj, o->A, o->B, el);
    uint64_t num = count_bits(o->B, total) * (uint64_t)s;
    if(num == (uint64_t)nodes * nodes) break;
    uint64_t *t = o->A; o->A = o->B; o->B = t;
    *sum += (long)nodes * nodes - (long)num;
    (*diameter)++;
  }
  *ASPL = *sum / (((double)nodes - 1) * nodes);
  *sum /= 2.0;
}

static void run_saving(oracle_t *o, const int *adj, int *diameter, long *sum, double *ASPL)   /* aspl.c:77-119 */
{
  const int nodes = o->nodes, s = o->symmetries, base = nodes / s;
  const int parsize = (int)((o->elements + ORACLE_CHUNK - 1) / ORACLE_CHUNK);
  size_t total = (size_t)nodes * ORACLE_CHUNK;
  *sum = (long)nodes * (nodes - 1);
  *diameter = 1;
  for(int t = 0; t < parsize; t++){
    unsigned kk, l;
    memset(o->A, 0, total * sizeof(uint64_t));
    memset(o->B, 0, total * sizeof(uint64_t));
    for(l = 0; l < 64 * ORACLE_CHUNK && 64 * t * ORACLE_CHUNK + (int)l < base; l++){
      size_t off = (size_t)(64 * t * ORACLE_CHUNK + l) * ORACLE_CHUNK + l / 64;
      o->A[off] = o->B[off] = 1ULL << (l % 64);
    }
    for(kk = 0; kk < (unsigned)nodes; kk++){
      or_gather(o, adj, o->A, o->B, ORACLE_CHUNK);
      uint64_t num = count_bits(o->B, total);
      if(num == (uint64_t)nodes * l) break;
      uint64_t *tmp = o->A; o->A = o->B; o->B = tmp;
      *sum += ((long)nodes * l - (long)num) * s;
    }
    if((int)(kk + 1) > *diameter) *diameter = (int)(kk + 1);
  }
  *ASPL = *sum / (((double)nodes - 1) * nodes);
  *sum /= 2.0;
}

/* ODP_Set_aspl (aspl.c:319-339) for one adjacency int[nodes/s][degree]. */
void oracle_set(oracle_t *o, const int *adjacency, int *diameter, long *sum, double *ASPL)
{
  if(o->kind == KIND_MATRIX) run_matrix(o, adjacency, diameter, sum, ASPL);
  else                       run_saving(o, adjacency, diameter, sum, ASPL);
  if(*diameter > o->nodes){
    *diameter = INT_MAX;
    *sum = LONG_MAX;
    *ASPL = DBL_MAX;
  }
}

int oracle_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

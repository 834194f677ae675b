/*
 * odp_graph.c -- the graph utilities that sit on either side of the ASPL hot
 * path: seeded random generators, edge-list <-> adjacency conversion, and the
 * 2-opt Mutate/Restore edge swaps that simulated-annealing clients issue
 * between ASPL evaluations.
 *
 * These are the odp.h utility entry points that the reference ships inside
 * every libodp*.a next to the ASPL driver (utils.c).  The generators must
 * reproduce the reference's graphs exactly for a given seed, which fixes the
 * order of every random draw and every accept/reject decision; the code below
 * restates those steps (cited per function) in our own structure.  Two
 * deliberate differences, neither visible in the results:
 *   - the random stream is an explicit odp_rng (odp_rng.h), so graphs can be
 *     generated concurrently (ODPX_* seeded variants); the public ODP_*
 *     functions bind it to libc rand() exactly like the reference;
 *   - the reverse-slot search of a 2-opt proposal (get_degree_index_*) is
 *     done only once a proposal is known to be accepted: it draws no random
 *     numbers, so skipping it for rejected proposals changes nothing but time.
 *
 * Errors print to stderr and exit(1), as the reference's ERROR macro does
 * (common.h:32).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdbool.h>
#include <math.h>
#include "odp_rng.h"
#include "odp_internal.h"

#define ODP_FAIL(...) do{ fprintf(stderr, __VA_ARGS__); exit(1); }while(0)
#define GEN_ITERS 10          /* GEN_GRAPH_ITERS, parameter.h:17 */
#define UNSET (-1)            /* NOT_DEFINED, common.h:41 */

/* ------------------------------------------------------------------------ */
/* Index arithmetic shared by the general (circulant) and grid symmetries.   */
/* ------------------------------------------------------------------------ */

/* The general (circulant) 2-opt swap is shared with the device annealing
 * kernels (odp_mutate.h); here it draws from an odp_rng and, like the
 * reference, retries without a bound. */
typedef odp_rng mut_rng;
#define MUT_BELOW(rng, max) odp_rng_below((rng), (max))
#define MUT_TRIES 0
#include "odp_mutate.h"

typedef mut_general gen_ctx;  /* a symmetric general graph: n vertices, s orbits */

typedef mut_grid grid_ctx;     /* a (possibly rotation-symmetric) grid graph */

static inline int wrap(int x, int n) { return mut_wrap(x, n); }  /* NORM, utils.c:171-177 */

static inline int gen_rel(const gen_ctx *g, int v, int pos) { return mut_rel(g, v, pos); }

static void fill_restore(ODP_Restore *r, const int u[2], const int us[2], const int v[2], const int vs[2])
{
  mut_fill_restore(r, u, us, v, vs);
}

/* One 2-opt attempt on a general(_s) graph; false when the attempt is
 * rejected and the caller retries. */
static bool gen_two_opt(odp_rng *rng, gen_ctx *g, ODP_Restore *r)
{
  int e = mut_two_opt(rng, g, r);
  if(e < 0) ODP_FAIL("Something Wrong ! [id=4]\n");
  return e == 1;
}

/* ------------------------------------------------------------------------ */
/* Grid graphs: vertex v = x*h + y; symmetric grids store the base block.    */
/* ------------------------------------------------------------------------ */

static int *grid_coords(int w, int h)
{
  int *xy = malloc(sizeof(int) * 2 * (size_t)w * h);
  for(int v = 0; v < w * h; v++){ xy[2 * v] = v / h; xy[2 * v + 1] = v % h; }
  return xy;
}

/* One 2-opt attempt on a grid(_s) graph; false when the attempt is rejected
 * and the caller retries. */
static bool grid_two_opt(odp_rng *rng, grid_ctx *g, ODP_Restore *r)
{
  int e = mut_grid_two_opt(rng, g, r);
  if(e < 0) ODP_FAIL("Something Wrong ! [id=5]\n");
  return e == 1;
}

/* ------------------------------------------------------------------------ */
/* Connectivity probe used by the generators (simple_bfs, utils.c:273-353).  */
/* ------------------------------------------------------------------------ */

static bool has_unreached_general(const gen_ctx *g)
{
  int n = g->n;
  char *seen = calloc((size_t)n, 1);
  int *queue = malloc(sizeof(int) * (size_t)n);
  int head = 0, tail = 0;
  queue[tail++] = 0; seen[0] = 1;
  while(head < tail){
    int v = queue[head++];
    int p = v / g->base, m = v - p * g->base;
    for(int j = 0; j < g->d; j++){
      int x = g->adj[(size_t)m * g->d + j] + p * g->base;
      if(x >= n) x -= n;
      if(!seen[x]){ seen[x] = 1; queue[tail++] = x; }
    }
  }
  free(queue); free(seen);
  return tail != n;
}

static bool has_unreached_grid(const grid_ctx *g)
{
  int n = g->n;
  char *seen = calloc((size_t)n, 1);
  int *queue = malloc(sizeof(int) * (size_t)n);
  int head = 0, tail = 0;
  queue[tail++] = 0; seen[0] = 1;
  while(head < tail){
    int v = queue[head++];
    for(int j = 0; j < g->d; j++){
      int x = grid_nbr(g, v, j);
      if(!seen[x]){ seen[x] = 1; queue[tail++] = x; }
    }
  }
  free(queue); free(seen);
  return tail != n;
}

/* ------------------------------------------------------------------------ */
/* Conversions.                                                              */
/* ------------------------------------------------------------------------ */

/* ODP_Conv_edge2adjacency_general_s, utils.c:1012-1034 */
static void edges_to_rows_general(int n, int lines, int d, const int (*edge)[2], int s, int *adj)
{
  int base = n / s;
  int *cnt = calloc((size_t)base, sizeof(int));
  for(size_t i = 0; i < (size_t)base * d; i++) adj[i] = UNSET;
  for(int i = 0; i < lines; i++){
    int a = edge[i][0], b = edge[i][1];
    if(a < base) adj[(size_t)a * d + cnt[a]++] = b;
    if(b < base) adj[(size_t)b * d + cnt[b]++] = a;
  }
  free(cnt);
}

/* ODP_Conv_edge2adjacency_grid_s, utils.c:1116-1151 (s = 2 or 4) */
static void edges_to_rows_grid(int w, int h, int lines, int d, const int (*edge)[2], int s, int *adj)
{
  grid_ctx g = { .w = w, .h = h, .d = d, .s = s, .n = w * h, .bw = w / 2, .bh = (s == 2) ? h : h / 2 };
  int base = g.n / s;
  int *cnt = calloc((size_t)base, sizeof(int));
  for(size_t i = 0; i < (size_t)base * d; i++) adj[i] = UNSET;
  for(int i = 0; i < lines; i++){
    int a = edge[i][0], b = edge[i][1];
    if(gx(a, h) < g.bw && gy(a, h) < g.bh){ int r = grid_row(&g, a); adj[(size_t)r * d + cnt[r]++] = b; }
    if(gx(b, h) < g.bw && gy(b, h) < g.bh){ int r = grid_row(&g, b); adj[(size_t)r * d + cnt[r]++] = a; }
  }
  free(cnt);
}

static int expected_lines(int n, int d, const int *ndeg)
{
  if(!ndeg) return (n * d) / 2;
  long total = 0;
  for(int i = 0; i < n; i++) total += ndeg[i];
  if(total % 2 == 1) ODP_FAIL("Something Wrong ! [id=2]\n");
  return (int)(total / 2);
}

/* ODP_Conv_adjacency2edge_general, utils.c:1506-1533 */
static void rows_to_edges_full(int n, int d, const int *ndeg, const int *adj, int (*edge)[2])
{
  int lines = 0, loops = 0;
  for(int i = 0; i < n; i++){
    int dd = ndeg ? ndeg[i] : d;
    for(int j = 0; j < dd; j++){
      int v = adj[(size_t)i * d + j];
      if(i < v){ edge[lines][0] = i; edge[lines][1] = v; lines++; }
      else if(i == v){
        loops++;
        if(loops % 2 == 0){ edge[lines][0] = i; edge[lines][1] = v; lines++; }
      }
    }
  }
  if(loops % 2 == 1 || lines != expected_lines(n, d, ndeg))
    ODP_FAIL("Something Wrong ! [id=1]\n");
}

/* ODP_Conv_adjacency2edge_general_s, utils.c:991-1010 */
static void rows_to_edges_general(int n, int d, const int *ndeg, const int *adj, int s, int (*edge)[2])
{
  int base = n / s;
  int *full = malloc(sizeof(int) * (size_t)n * d);
  int *full_deg = ndeg ? malloc(sizeof(int) * (size_t)n) : NULL;
  for(int i = 0; i < s; i++)
    for(int j = 0; j < base; j++){
      int dd = ndeg ? ndeg[j] : d;
      if(full_deg) full_deg[i * base + j] = dd;
      for(int k = 0; k < dd; k++)
        full[(size_t)(i * base + j) * d + k] = wrap(adj[(size_t)j * d + k] + i * base, n);
    }
  /* The reference passes the base-sized num_degrees on to the n-row
   * conversion (utils.c:1009); the per-row degrees are tiled here instead. */
  rows_to_edges_full(n, d, full_deg, full, edge);
  free(full_deg);
  free(full);
}

/* ODP_Conv_adjacency2edge_grid_s, utils.c:152-169 / 154-168 */
static void rows_to_edges_grid(int w, int h, int d, const int *ndeg, const int *adj, int s, int (*edge)[2])
{
  int n = w * h;
  if(s == 1){ rows_to_edges_full(n, d, ndeg, adj, edge); return; }
  grid_ctx g = { .w = w, .h = h, .d = d, .s = s, .n = n, .bw = w / 2, .bh = (s == 2) ? h : h / 2 };
  int *full = malloc(sizeof(int) * (size_t)n * d);
  int *full_deg = ndeg ? malloc(sizeof(int) * (size_t)n) : NULL;
  int base = n / s;
  for(int i = 0; i < base; i++){
    int dd = ndeg ? ndeg[i] : d;
    if(s == 2){
      if(full_deg){ full_deg[i] = dd; full_deg[grid_rot(&g, i, 180)] = dd; }
      for(int k = 0; k < dd; k++){
        int v = adj[(size_t)i * d + k];
        full[(size_t)i * d + k] = v;
        full[(size_t)grid_rot(&g, i, 180) * d + k] = grid_rot(&g, v, 180);
      }
    }
    else{
      int j = (i / g.bh) * h + (i % g.bh);
      if(full_deg){
        full_deg[j] = dd;
        for(int r = 90; r <= 270; r += 90) full_deg[grid_rot(&g, j, r)] = dd;
      }
      for(int k = 0; k < dd; k++){
        int v = adj[(size_t)i * d + k];
        full[(size_t)j * d + k] = v;
        full[(size_t)grid_rot(&g, j, 90) * d + k]  = grid_rot(&g, v, 90);
        full[(size_t)grid_rot(&g, j, 180) * d + k] = grid_rot(&g, v, 180);
        full[(size_t)grid_rot(&g, j, 270) * d + k] = grid_rot(&g, v, 270);
      }
    }
  }
  rows_to_edges_full(n, d, full_deg, full, edge);
  free(full_deg);
  free(full);
}

/* ------------------------------------------------------------------------ */
/* Generators.                                                               */
/* ------------------------------------------------------------------------ */

static void check_nd(int n, int d)                    /* CHECK_PARAMETERS, utils.c:355-359 */
{
  if(n % 2 == 1 && d % 2 == 1)
    ODP_FAIL("Nodes(%d) or Degree(%d) must be a multiple of 2.\n", n, d);
}

static void check_sym(int n, int s)
{
  if(s <= 0 || n % s != 0) ODP_FAIL("nodes(%d) must be divisible by symmetries(%d)\n", n, s);
}

static void check_grid_sym(int w, int h, int s)
{
  if(s != 1 && s != 2 && s != 4) ODP_FAIL("symmetries(%d) must be 1 or 2 or 4\n", s);
  if(s == 2 && w % 2 != 0) ODP_FAIL("width(%d) must be divisible by 2\n", w);
  else if(s == 4 && (w % 2 != 0 || h % 2 != 0)) ODP_FAIL("width(%d) and height(%d) must be divisible by 2\n", w, h);
  else if(s == 4 && w != h) ODP_FAIL("Must be the same as width(%d) and height(%d)\n", w, h);
}

/* Ring with d/2 parallel edges per consecutive pair, plus antipodal chords
 * when d is odd (create_simple_graph, utils.c:1041-1063). */
static void ring_multigraph(int n, int d, int (*edge)[2])
{
  int hd = d / 2;
  for(int i = 0; i < n - 1; i++)
    for(int j = 0; j < hd; j++){ edge[i * hd + j][0] = i; edge[i * hd + j][1] = i + 1; }
  for(int j = 0; j < hd; j++){ edge[(n - 1) * hd + j][0] = n - 1; edge[(n - 1) * hd + j][1] = 0; }
  if(d % 2 == 1){
    int half = n / 2;
    for(int i = 0; i < half; i++){ edge[hd * n + i][0] = i; edge[hd * n + i][1] = i + half; }
  }
}

/* ODP_Generate_random_general(_s), utils.c:1065-1114 */
void odpx_generate_general(odp_rng *rng, int n, int d, int s, int (*edge)[2])
{
  check_sym(n, s);
  check_nd(n, d);
  ring_multigraph(n, d, edge);
  int lines = (n * d) / 2;
  gen_ctx g = { .n = n, .d = d, .s = s, .base = n / s, .ndeg = NULL };
  g.adj = malloc(sizeof(int) * (size_t)g.base * d);
  edges_to_rows_general(n, lines, d, (const int (*)[2])edge, s, g.adj);
  for(long i = 0; i < (long)lines * GEN_ITERS; i++)
    while(!gen_two_opt(rng, &g, NULL)) {}
  while(has_unreached_general(&g))
    while(!gen_two_opt(rng, &g, NULL)) {}
  if(s == 1) rows_to_edges_full(n, d, NULL, g.adj, edge);
  else       rows_to_edges_general(n, d, NULL, g.adj, s, edge);
  free(g.adj);
}

static void grid_mutate_until(odp_rng *rng, grid_ctx *g, ODP_Restore *r)
{
  while(!grid_two_opt(rng, g, r)) {}
}

/* ODP_Generate_random_grid, utils.c:1577-1625 */
static void generate_grid_plain(odp_rng *rng, int w, int h, int d, int len, int (*edge)[2])
{
  int n = w * h;
  check_nd(n, d);
  int i = 0;
  for(int x = 0; x < w / 2; x++)
    for(int y = 0; y < h; y++)
      for(int k = 0; k < d; k++){
        edge[i][0] = y + 2 * x * h;
        edge[i][1] = edge[i][0] + h;
        i++;
      }
  if(w % 2 == 1){
    for(int y = 0; y < h / 2; y++)
      for(int k = 0; k < d; k++){
        edge[i][0] = (w - 1) * h + 2 * y;
        edge[i][1] = edge[i][0] + 1;
        i++;
      }
    if(h % 2 == 1)
      for(int k = 0; k < d / 2; k++){ edge[i][0] = edge[i][1] = n - 1; i++; }
  }
  int lines = (n * d) / 2;
  int *xy = grid_coords(w, h);
  grid_ctx g = { .w = w, .h = h, .d = d, .s = 1, .len = len, .n = n, .bw = w / 2, .bh = h / 2, .ndeg = NULL, .xy = xy };
  g.adj = malloc(sizeof(int) * (size_t)n * d);
  edges_to_rows_general(n, lines, d, (const int (*)[2])edge, 1, g.adj);
  for(long it = 0; it < (long)lines * GEN_ITERS; it++) grid_mutate_until(rng, &g, NULL);
  gen_ctx probe = { .n = n, .d = d, .s = 1, .base = n, .adj = g.adj };
  while(has_unreached_general(&probe)) grid_mutate_until(rng, &g, NULL);
  rows_to_edges_full(n, d, NULL, g.adj, edge);
  free(g.adj);
  free(xy);
}

/* ODP_Generate_random_grid_s, utils.c:1627-1749 */
void odpx_generate_grid(odp_rng *rng, int w, int h, int d, int len, int s, int (*edge)[2])
{
  check_nd(w * h, d);
  check_grid_sym(w, h, s);
  if(s == 1){ generate_grid_plain(rng, w, h, d, len, edge); return; }

  grid_ctx g = { .w = w, .h = h, .d = d, .s = s, .len = len, .n = w * h, .bw = w / 2, .bh = (s == 2) ? h : h / 2 };
  int n = g.n, lines = (n * d) / 2, base_lines = lines / s, base = n / s;
  int bw = g.bw, bh = g.bh;
  int deg_base = (base % 2 == 0 || d % 2 == 0) ? d : d - 1;
  generate_grid_plain(rng, bw, bh, deg_base, len, edge);
  int made = (deg_base == d) ? base_lines : (base * (d - 1)) / 2;
  for(int i = 0; i < made; i++)
    for(int j = 0; j < 2; j++)
      edge[i][j] = gx(edge[i][j], bh) * h + gy(edge[i][j], bh);
  if(s == 2){
    for(int i = 0; i < made; i++)
      for(int j = 0; j < 2; j++) edge[made + i][j] = grid_rot(&g, edge[i][j], 180);
  }
  else{
    for(int i = 0; i < made; i++)
      for(int j = 0; j < 2; j++){
        edge[made + i][j]     = grid_rot(&g, edge[i][j], 90);
        edge[made * 2 + i][j] = grid_rot(&g, edge[i][j], 180);
        edge[made * 3 + i][j] = grid_rot(&g, edge[i][j], 270);
      }
  }
  if(deg_base != d){                      /* odd base and odd degree: add a perfect matching */
    int k = made * s;
    if(s == 2){
      for(int x = 0; x < w; x += 2)
        for(int y = 0; y < h; y++){ edge[k][0] = y + x * h; edge[k][1] = edge[k][0] + h; k++; }
    }
    else{
      for(int x = 0; x < bw / 2; x++)
        for(int y = 0; y < bh; y++){
          edge[k][0] = x * 2 * h + y;
          edge[k][1] = edge[k][0] + h;
          for(int r = 1; r < 4; r++){
            edge[k + r][0] = grid_rot(&g, edge[k][0], 90 * r);
            edge[k + r][1] = grid_rot(&g, edge[k][1], 90 * r);
          }
          k += 4;
        }
      if(bw % 2 == 1){
        for(int y = 0; y < bh / 2; y++){
          edge[k][0] = (bw - 1) * h + y * 2;
          edge[k][1] = edge[k][0] + 1;
          for(int r = 1; r < 4; r++){
            edge[k + r][0] = grid_rot(&g, edge[k][0], 90 * r);
            edge[k + r][1] = grid_rot(&g, edge[k][1], 90 * r);
          }
          k += 4;
        }
        if(bh % 2 == 1){
          if(len <= 1) ODP_FAIL("Graphs with odd width/2 and length/2 and length 1 cannot be created.");
          edge[k][0]     = (bw - 1) * h + (bh - 1);
          edge[k][1]     = bw * h + bh;
          edge[k + 1][0] = (bw - 1) * h + bh;
          edge[k + 1][1] = bw * h + (bh - 1);
        }
      }
    }
  }
  int *xy = grid_coords(w, h);
  g.xy = xy;
  g.adj = malloc(sizeof(int) * (size_t)base * d);
  edges_to_rows_grid(w, h, lines, d, (const int (*)[2])edge, s, g.adj);
  for(long it = 0; it < (long)base_lines * GEN_ITERS; it++) grid_mutate_until(rng, &g, NULL);
  while(has_unreached_grid(&g)) grid_mutate_until(rng, &g, NULL);
  rows_to_edges_grid(w, h, d, NULL, g.adj, s, edge);
  free(g.adj);
  free(xy);
}

/* ------------------------------------------------------------------------ */
/* Public odp.h utility surface.                                             */
/* ------------------------------------------------------------------------ */

static odp_rng g_libc_rng = { .libc = 1 };

/* Parameters of the last Mutate call, which Restore reuses
 * (the reference keeps the same file-scope state, utils.c:2). */
static int m_nodes, m_degree, m_width, m_height, m_symmetries;

void ODP_Srand(unsigned int seed) { srand(seed); }

void ODP_Generate_random_general(int nodes, int degree, int (*edge)[2])
{
  odpx_generate_general(&g_libc_rng, nodes, degree, 1, edge);
}

void ODP_Generate_random_general_s(int nodes, int degree, int symmetries, int (*edge)[2])
{
  odpx_generate_general(&g_libc_rng, nodes, degree, symmetries, edge);
}

void ODP_Generate_random_grid(int width, int height, int degree, int length, int (*edge)[2])
{
  odpx_generate_grid(&g_libc_rng, width, height, degree, length, 1, edge);
}

void ODP_Generate_random_grid_s(int width, int height, int degree, int length, int symmetries, int (*edge)[2])
{
  odpx_generate_grid(&g_libc_rng, width, height, degree, length, symmetries, edge);
}

void ODPX_Generate_random_general_seeded(unsigned int seed, int nodes, int degree, int symmetries, int (*edge)[2])
{
  odp_rng g; odp_rng_seed(&g, seed);
  odpx_generate_general(&g, nodes, degree, symmetries, edge);
}

void ODPX_Generate_random_grid_seeded(unsigned int seed, int width, int height, int degree, int length,
                                      int symmetries, int (*edge)[2])
{
  odp_rng g; odp_rng_seed(&g, seed);
  odpx_generate_grid(&g, width, height, degree, length, symmetries, edge);
}

void ODP_Conv_edge2adjacency_general(int nodes, int lines, int degree, int (*edge)[2], void *adjacency)
{
  edges_to_rows_general(nodes, lines, degree, (const int (*)[2])edge, 1, adjacency);
}

void ODP_Conv_edge2adjacency_general_s(int nodes, int lines, int degree, int (*edge)[2], int symmetries, void *adjacency)
{
  check_sym(nodes, symmetries);
  edges_to_rows_general(nodes, lines, degree, (const int (*)[2])edge, symmetries, adjacency);
}

void ODP_Conv_edge2adjacency_grid(int width, int height, int lines, int degree, int (*edge)[2], void *adjacency)
{
  edges_to_rows_general(width * height, lines, degree, (const int (*)[2])edge, 1, adjacency);
}

void ODP_Conv_edge2adjacency_grid_s(int width, int height, int lines, int degree, int (*edge)[2], int symmetries,
                                    void *adjacency)
{
  check_grid_sym(width, height, symmetries);
  if(symmetries == 1) edges_to_rows_general(width * height, lines, degree, (const int (*)[2])edge, 1, adjacency);
  else edges_to_rows_grid(width, height, lines, degree, (const int (*)[2])edge, symmetries, adjacency);
}

void ODP_Conv_adjacency2edge_general(int nodes, int degree, int *num_degrees, void *adjacency, int (*edge)[2])
{
  rows_to_edges_full(nodes, degree, num_degrees, adjacency, edge);
}

void ODP_Conv_adjacency2edge_grid(int width, int height, int degree, int *num_degrees, void *adjacency, int (*edge)[2])
{
  rows_to_edges_full(width * height, degree, num_degrees, adjacency, edge);
}

void ODP_Conv_adjacency2edge_general_s(int nodes, int degree, int *num_degrees, void *adjacency, int symmetries,
                                       int (*edge)[2])
{
  check_sym(nodes, symmetries);
  rows_to_edges_general(nodes, degree, num_degrees, adjacency, symmetries, edge);
}

void ODP_Conv_adjacency2edge_grid_s(int width, int height, int degree, int *num_degrees, void *adjacency,
                                    int symmetries, int (*edge)[2])
{
  check_grid_sym(width, height, symmetries);
  rows_to_edges_grid(width, height, degree, num_degrees, adjacency, symmetries, edge);
}

/* ODP_Mutate_adjacency_general(_s), utils.c:752-788 */
void odpx_mutate_general(odp_rng *rng, int nodes, int degree, const int *num_degrees, int symmetries,
                         ODP_Restore *r, int *adjacency)
{
  check_sym(nodes, symmetries);
  gen_ctx g = { .n = nodes, .d = degree, .s = symmetries, .base = nodes / symmetries,
                .ndeg = num_degrees, .adj = adjacency };
  while(!gen_two_opt(rng, &g, r)) {}
}

/* ODP_Mutate_adjacency_grid(_s), utils.c:973-989, 2105-2113 */
void odpx_mutate_grid(odp_rng *rng, int width, int height, int degree, const int *num_degrees, int length,
                      int symmetries, ODP_Restore *r, int *adjacency)
{
  check_nd(width * height, degree);
  check_grid_sym(width, height, symmetries);
  grid_ctx g = { .w = width, .h = height, .d = degree, .s = symmetries, .len = length, .n = width * height,
                 .bw = width / 2, .bh = (symmetries == 2) ? height : height / 2,
                 .ndeg = num_degrees, .adj = adjacency };
  grid_mutate_until(rng, &g, r);
}

void ODP_Mutate_adjacency_general_s(int nodes, int degree, int *num_degrees, int symmetries, ODP_Restore *r,
                                    int (*adjacency)[degree])
{
  m_nodes = nodes; m_degree = degree; m_symmetries = symmetries;
  odpx_mutate_general(&g_libc_rng, nodes, degree, num_degrees, symmetries, r, (int *)adjacency);
}

void ODP_Mutate_adjacency_general(int nodes, int degree, int *num_degrees, ODP_Restore *r, int (*adjacency)[degree])
{
  ODP_Mutate_adjacency_general_s(nodes, degree, num_degrees, 1, r, adjacency);
}

void ODP_Mutate_adjacency_grid_s(int width, int height, int degree, int *num_degrees, int length, int symmetries,
                                 ODP_Restore *r, int (*adjacency)[degree])
{
  m_width = width; m_height = height; m_degree = degree; m_symmetries = symmetries;
  odpx_mutate_grid(&g_libc_rng, width, height, degree, num_degrees, length, symmetries, r, (int *)adjacency);
}

void ODP_Mutate_adjacency_grid(int width, int height, int degree, int *num_degrees, int length, ODP_Restore *r,
                               int (*adjacency)[degree])
{
  /* The reference's grid Mutate leaves the Restore state untouched unless
   * the _s variant is used (utils.c:2105-2113); it is set here as well so that
   * Restore after a plain grid Mutate writes through the right shape. */
  m_width = width; m_height = height; m_degree = degree; m_symmetries = 1;
  odpx_mutate_grid(&g_libc_rng, width, height, degree, num_degrees, length, 1, r, (int *)adjacency);
}

/* ODP_Restore_adjacency_general, utils.c:500-507 */
void odpx_restore_general(int nodes, int degree, int symmetries, ODP_Restore r, int *adjacency)
{
  gen_ctx g = { .n = nodes, .d = degree, .s = symmetries, .base = nodes / symmetries };
  for(int i = 0; i < 2; i++){
    adjacency[(size_t)(r.u[i] % g.base) * degree + r.u_d[i]] = gen_rel(&g, r.v[i], r.u[i]);
    adjacency[(size_t)(r.v[i] % g.base) * degree + r.v_d[i]] = gen_rel(&g, r.u[i], r.v[i]);
  }
}

/* ODP_Restore_adjacency_grid, utils.c:461-467 */
void odpx_restore_grid(int width, int height, int degree, int symmetries, ODP_Restore r, int *adjacency)
{
  grid_ctx g = { .w = width, .h = height, .d = degree, .s = symmetries, .n = width * height,
                 .bw = width / 2, .bh = (symmetries == 2) ? height : height / 2, .adj = adjacency };
  for(int i = 0; i < 2; i++){
    grid_put(&g, r.u[i], r.u_d[i], r.v[i]);
    grid_put(&g, r.v[i], r.v_d[i], r.u[i]);
  }
}

/* Restore uses the shape of the last Mutate call, as the reference does
 * (utils.c:500-507, 461-467); without one there is no shape to use. */
void ODP_Restore_adjacency_general(ODP_Restore r, void *adjacency)
{
  if(m_nodes <= 0 || m_symmetries <= 0) ODP_FAIL("ODP_Restore_adjacency_general called before ODP_Mutate_adjacency_general\n");
  odpx_restore_general(m_nodes, m_degree, m_symmetries, r, adjacency);
}

void ODP_Restore_adjacency_grid(ODP_Restore r, void *adjacency)
{
  if(m_width <= 0 || m_height <= 0 || m_symmetries <= 0)
    ODP_FAIL("ODP_Restore_adjacency_grid called before ODP_Mutate_adjacency_grid\n");
  odpx_restore_grid(m_width, m_height, m_degree, m_symmetries, r, adjacency);
}

/* Restore with an explicit shape, for callers that mutate through their own
 * random streams (ODPX_Mutate_adjacency_general_s_rng). */
void ODPX_Restore_adjacency_general_s(int nodes, int degree, int symmetries, ODP_Restore r, int *adjacency)
{
  if(nodes <= 0 || symmetries <= 0 || nodes % symmetries) ODP_FAIL("nodes(%d) must be divisible by symmetries(%d)\n", nodes, symmetries);
  odpx_restore_general(nodes, degree, symmetries, r, adjacency);
}

/* Thread-safe, explicitly parameterised mutate for callers that keep one
 * stream per annealing chain (the serving workload). */
void ODPX_Mutate_adjacency_general_s_rng(void *rng_state, int nodes, int degree, const int *num_degrees,
                                         int symmetries, ODP_Restore *r, int *adjacency)
{
  odpx_mutate_general((odp_rng *)rng_state, nodes, degree, num_degrees, symmetries, r, adjacency);
}

/* The grid counterparts (ODP_Mutate_adjacency_grid_s / ODP_Restore_adjacency_grid
 * with an explicit stream and shape). */
void ODPX_Mutate_adjacency_grid_s_rng(void *rng_state, int width, int height, int degree, const int *num_degrees,
                                      int length, int symmetries, ODP_Restore *r, int *adjacency)
{
  odpx_mutate_grid((odp_rng *)rng_state, width, height, degree, num_degrees, length, symmetries, r, adjacency);
}

void ODPX_Restore_adjacency_grid_s(int width, int height, int degree, int symmetries, ODP_Restore r, int *adjacency)
{
  check_grid_sym(width, height, symmetries);
  odpx_restore_grid(width, height, degree, symmetries, r, adjacency);
}

size_t ODPX_Rng_size(void) { return sizeof(odp_rng); }

void ODPX_Rng_seed(void *rng_state, unsigned int seed) { odp_rng_seed((odp_rng *)rng_state, seed); }

int ODPX_Rng_next(void *rng_state) { return odp_rng_next((odp_rng *)rng_state); }

/*
 * odp_mutate.h -- the 2-opt edge swap of a general (circulant-symmetric)
 * graph, shared by the host graph utilities (odp_graph.c: generators and
 * ODP_Mutate_adjacency_general_s) and the device annealing kernels
 * (anneal.cu), so that both draw the same random numbers in the same order
 * and make the same swap.
 *
 * It restates mutate_adjacency_2opt_general_s and its helpers
 * (reference utils.c:509-532, 572-750) over an explicit context.  The reference's
 * multiple-edge check (check_multiple_edges_general_s, utils.c:469-482) always
 * succeeds and is left out.
 *
 * The includer defines, before including this header:
 *   mut_rng                  the random stream type;
 *   MUT_BELOW(rng, max)      a uniform integer in [0, max) drawn from it, as the
 *                            reference's get_random (utils.c:361-364);
 *   MUT_TRIES                0 for retry loops without a bound (as the
 *                            reference), or the number of draws after which a
 *                            proposal gives up with an error (device code
 *                            must not spin without a bound);
 * and may define MUT_FN, the functions' qualifiers (device-only code).
 */
#ifndef ODP_MUTATE_H
#define ODP_MUTATE_H

#include "odp.h"
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifndef MUT_FN
#define MUT_FN static inline
#endif

typedef struct {
  int n, d, s, base;          /* base = n / s rows stored */
  const int *ndeg;            /* per base row degree, or NULL (regular) */
  int *adj;                   /* int[base][d] */
  int nw;                     /* the last successful swap's writes: */
  int wrow[4], wslot[4];      /*   adj[wrow][wslot] was set (base rows) */
} mut_general;

MUT_FN int mut_wrap(int x, int n)                 /* NORM, utils.c:171-177 */
{
  if(n <= 0) return x;
  while(x < 0 || x >= n) x = (x < 0) ? x + n : x - n;
  return x;
}

/* adjacency[v][j] of the expanded graph (GLOBAL_ADJ_GENERAL, utils.c:180-186) */
MUT_FN int mut_nbr(const mut_general *g, int v, int j)
{
  return mut_wrap(g->adj[(long long)(v % g->base) * g->d + j] + (v / g->base) * g->base, g->n);
}

/* value to store in the row of `pos` so that it names global vertex v
 * (LOCAL_INDEX_GENERAL, utils.c:266-270) */
MUT_FN int mut_rel(const mut_general *g, int v, int pos)
{
  return mut_wrap(v - (pos / g->base) * g->base, g->n);
}

MUT_FN int mut_antipodal(const mut_general *g, int u, int v)   /* IS_DIAMETER_GENERAL, utils.c:96-102 */
{
  int x = u - v;
  return (g->s % 2 == 0) && (x < 0 ? -x : x) == g->n / 2;
}

MUT_FN int mut_deg(const mut_general *g, int v)
{
  return g->ndeg ? g->ndeg[v % g->base] : g->d;
}

/* The slot of v's row that points back at u (get_degree_index_general,
 * utils.c:509-532); -1 when there is none (the reference stops there). */
MUT_FN int mut_back_slot(const mut_general *g, int u, int v, int u_slot)
{
  if(u == v){
    int dd = mut_deg(g, v);
    for(int i = 0; i < dd; i++)
      if(mut_nbr(g, v, i) == u && i != u_slot) return i;
  }
  else if(mut_antipodal(g, u, v)){
    return u_slot;
  }
  else{
    int dd = mut_deg(g, v);
    for(int i = 0; i < dd; i++)
      if(mut_nbr(g, v, i) == u) return i;
  }
  return -1;
}

/* Two edges that are images of each other under the rotation
 * (check_rotated_edges_overlap_general, utils.c:603-621). */
MUT_FN int mut_same_orbit(const mut_general *g, int u0, int v0, int u1, int v1)
{
  int n = g->n;
  int d0 = (u0 > v0) ? v0 - u0 + n : v0 - u0;
  int d1 = (u1 > v1) ? v1 - u1 + n : v1 - u1;
  int d2 = (u1 < v1) ? u1 - v1 + n : u1 - v1;
  if(d0 == d1 && u0 % g->base == u1 % g->base) return 1;
  if(d0 == d2 && u0 % g->base == v1 % g->base) return 1;
  return 0;
}

MUT_FN void mut_put(mut_general *g, int v, int slot, int value)
{
  int row = v % g->base;
  g->adj[(long long)row * g->d + slot] = value;
  if(g->nw < 4){ g->wrow[g->nw] = row; g->wslot[g->nw] = slot; g->nw++; }
}

MUT_FN void mut_fill_restore(ODP_Restore *r, const int u[2], const int us[2], const int v[2], const int vs[2])
{
  if(!r) return;
  for(int i = 0; i < 2; i++){
    r->u[i] = u[i]; r->v[i] = v[i]; r->u_d[i] = us[i]; r->v_d[i] = vs[i];
  }
}

/* Rotate a single edge to another orbit position (mutate_adjacency_1opt_general_s,
 * utils.c:572-601).  1: done; 0: rejected; -1: no back slot or out of tries. */
MUT_FN int mut_one_opt(mut_rng *rng, mut_general *g, int u, int us)
{
  int base = g->base, s = g->s, n = g->n;
  int v = mut_nbr(g, u, us);
  if(mut_antipodal(g, u, v)) return 0;
  int vs = mut_back_slot(g, u, v, us);
  if(vs < 0) return -1;
  int nv;
  if((u - v) % base == 0){
    if(s <= 4) return 0;
    for(long long tries = 0;; tries++){
      if(MUT_TRIES && tries >= MUT_TRIES) return -1;
      nv = v + base * MUT_BELOW(rng, s);
      if(u == nv || v == nv) continue;
      if(mut_wrap(u - v, n) == mut_wrap(nv - u, n)) continue;
      if(n % 2 == 1) break;
      if((u - nv) % (n / 2) != 0) break;
    }
  }
  else{
    int k = (s % 2 == 1) ? MUT_BELOW(rng, s - 1) : MUT_BELOW(rng, s);
    nv = (k != s - 1) ? v + base * (k + 1) : u + base * (s / 2);
  }
  int nu = v - (nv - u);
  int a = mut_rel(g, nv, u), b = mut_rel(g, nu, v);
  mut_put(g, u, us, a);
  mut_put(g, v, vs, b);
  return 1;
}

/* One 2-opt attempt (mutate_adjacency_2opt_general_s, utils.c:623-750).
 * 1: the swap was made (g->nw writes, *r filled); 0: the attempt was
 * rejected and the caller retries; -1: the graph has no back slot for a
 * drawn edge, or the draws ran out of tries. */
MUT_FN int mut_two_opt(mut_rng *rng, mut_general *g, ODP_Restore *r)
{
  int u[2], v[2], us[2], vs[2];
  const int n = g->n;
  g->nw = 0;
  for(long long tries = 0;; tries++){
    if(MUT_TRIES && tries >= MUT_TRIES) return -1;
    u[0] = MUT_BELOW(rng, n);
    u[1] = MUT_BELOW(rng, n);
    if(u[0] == u[1]) continue;
    us[0] = MUT_BELOW(rng, mut_deg(g, u[0]));
    v[0] = mut_nbr(g, u[0], us[0]);
    if(v[0] == u[1]) continue;
    us[1] = MUT_BELOW(rng, mut_deg(g, u[1]));
    v[1] = mut_nbr(g, u[1], us[1]);
    if(v[1] == u[0] || v[0] == v[1]) continue;
    break;
  }
  vs[0] = mut_back_slot(g, u[0], v[0], us[0]);
  vs[1] = mut_back_slot(g, u[1], v[1], us[1]);
  if(vs[0] < 0 || vs[1] < 0) return -1;
  mut_fill_restore(r, u, us, v, vs);

  int a0 = mut_antipodal(g, u[0], v[0]), a1 = mut_antipodal(g, u[1], v[1]);
  if(a0 && a1){
    if((u[0] - u[1]) % g->base == 0) return 0;
    int t0, t1;
    if(MUT_BELOW(rng, 2)){ t0 = mut_rel(g, u[1], u[0]); t1 = mut_rel(g, u[0], u[1]); }
    else                 { t0 = mut_rel(g, v[1], u[0]); t1 = mut_rel(g, v[0], u[1]); }
    mut_put(g, u[0], us[0], t0);
    mut_put(g, u[1], us[1], t1);
    return 1;
  }
  if(a0 || a1){
    if(a1){
      int t;
      t = u[0]; u[0] = u[1]; u[1] = t;
      t = us[0]; us[0] = us[1]; us[1] = t;
      t = v[0]; v[0] = v[1]; v[1] = t;
      t = vs[0]; vs[0] = vs[1]; vs[1] = t;
    }
    int opp = n / 2, k = MUT_BELOW(rng, 4), t[4];
    switch(k){
    case 0:
      t[0] = mut_rel(g, v[1], u[0]);        t[1] = mut_rel(g, u[1] + opp, u[1]);
      t[2] = mut_rel(g, v[1] + opp, v[0]);  t[3] = mut_rel(g, u[0], v[1]);
      break;
    case 1:
      t[0] = mut_rel(g, v[1] + opp, u[0]);  t[1] = mut_rel(g, u[1] + opp, u[1]);
      t[2] = mut_rel(g, v[1], v[0]);        t[3] = mut_rel(g, v[0], v[1]);
      break;
    case 2:
      t[0] = mut_rel(g, u[1], u[0]);        t[1] = mut_rel(g, u[0], u[1]);
      t[2] = mut_rel(g, u[1] + opp, v[0]);  t[3] = mut_rel(g, v[1] + opp, v[1]);
      break;
    default:
      t[0] = mut_rel(g, u[1] + opp, u[0]);  t[1] = mut_rel(g, v[0], u[1]);
      t[2] = mut_rel(g, u[1], v[0]);        t[3] = mut_rel(g, v[1] + opp, v[1]);
      break;
    }
    mut_put(g, u[0], us[0], t[0]);
    mut_put(g, u[1], us[1], t[1]);
    mut_put(g, v[0], vs[0], t[2]);
    mut_put(g, v[1], vs[1], t[3]);
    return 1;
  }

  if(mut_same_orbit(g, u[0], v[0], u[1], v[1]))
    return mut_one_opt(rng, g, u[0], us[0]);

  int t[4];
  if(MUT_BELOW(rng, 2)){                /* u0--v1, v0--u1 */
    if(mut_antipodal(g, u[0], v[1]) || mut_antipodal(g, v[0], u[1])) return 0;
    if(mut_same_orbit(g, u[0], v[1], v[0], u[1])) return 0;
    t[0] = mut_rel(g, v[1], u[0]); t[1] = mut_rel(g, v[0], u[1]);
    t[2] = mut_rel(g, u[1], v[0]); t[3] = mut_rel(g, u[0], v[1]);
  }
  else{                                 /* u0--u1, v0--v1 */
    if(mut_antipodal(g, u[0], u[1]) || mut_antipodal(g, v[0], v[1])) return 0;
    if(mut_same_orbit(g, u[0], u[1], v[0], v[1])) return 0;
    t[0] = mut_rel(g, u[1], u[0]); t[1] = mut_rel(g, u[0], u[1]);
    t[2] = mut_rel(g, v[1], v[0]); t[3] = mut_rel(g, v[0], v[1]);
  }
  mut_put(g, u[0], us[0], t[0]);
  mut_put(g, u[1], us[1], t[1]);
  mut_put(g, v[0], vs[0], t[2]);
  mut_put(g, v[1], vs[1], t[3]);
  return 1;
}

/* ODP_Restore_adjacency_general (utils.c:500-507): puts back the two edges a
 * swap replaced, recording the writes like a swap. */
MUT_FN void mut_restore(mut_general *g, const ODP_Restore *r)
{
  g->nw = 0;
  for(int i = 0; i < 2; i++){
    mut_put(g, r->u[i], r->u_d[i], mut_rel(g, r->v[i], r->u[i]));
    mut_put(g, r->v[i], r->v_d[i], mut_rel(g, r->u[i], r->v[i]));
  }
}

/* ------------------------------------------------------------------------ */
/* Grid graphs: vertex v = x*h + y; symmetric grids store the base block.    */
/* Restates mutate_adjacency_2opt_grid_s and its helpers (utils.c:52-56,     */
/* 67-88, 104-110, 189-247, 392-459, 534-557, 766-971).                      */
/* ------------------------------------------------------------------------ */

typedef struct {              /* a (possibly rotation-symmetric) grid graph */
  int w, h, d, s, len, n;
  int bw, bh;                 /* base block: x < bw, y < bh */
  const int *ndeg;            /* per local row degree, or NULL */
  int *adj;                   /* int[n/s][d], rows in local-index order */
  const int *xy;              /* optional (x, y) per vertex: saves divisions */
  int nw;                     /* the last successful swap's writes: */
  int wrow[4], wslot[4];      /*   adj[wrow][wslot] was set (local rows) */
} mut_grid;

MUT_FN int mut_abs(int x) { return x < 0 ? -x : x; }

MUT_FN int gx(int v, int h) { return v / h; }
MUT_FN int gy(int v, int h) { return v % h; }

/* ODP_ROTATE (utils.c:67-88) for s = 2 (180 degrees) and s = 4 (90/180/270, w == h). */
MUT_FN int grid_rot(const mut_grid *g, int v, int deg)
{
  int x = gx(v, g->h), y = gy(v, g->h), h = g->h;
  if(g->s == 2) return (g->w - x - 1) * h + (h - y - 1);
  if(deg == 90)  return y * h + (h - x - 1);
  if(deg == 180) return (h - x - 1) * h + (h - y - 1);
  return (h - y - 1) * h + x;
}

/* Row of a base-block vertex (ODP_LOCAL_INDEX_GRID, utils.c:189-211). */
MUT_FN int grid_row(const mut_grid *g, int v)
{
  if(g->s != 4) return v;
  return gx(v, g->h) * g->bh + gy(v, g->h);
}

/* adjacency[v][j] of the expanded grid (GLOBAL_ADJ_GRID, utils.c:214-247). */
MUT_FN int grid_nbr(const mut_grid *g, int v, int j)
{
  const int d = g->d;
  if(g->s == 1) return g->adj[(size_t)v * d + j];
  int x = gx(v, g->h), y = gy(v, g->h);
  if(g->s == 2){
    if(x < g->bw) return g->adj[(size_t)v * d + j];
    return grid_rot(g, g->adj[(size_t)grid_rot(g, v, 180) * d + j], 180);
  }
  if(x < g->bw && y < g->bh) return g->adj[(size_t)grid_row(g, v) * d + j];
  if(x < g->bw)  return grid_rot(g, g->adj[(size_t)grid_row(g, grid_rot(g, v, 270)) * d + j], 90);
  if(y >= g->bh) return grid_rot(g, g->adj[(size_t)grid_row(g, grid_rot(g, v, 180)) * d + j], 180);
  return grid_rot(g, g->adj[(size_t)grid_row(g, grid_rot(g, v, 90)) * d + j], 270);
}

/* Base row that stores vertex v's orbit (global2local_vertex_grid, utils.c:392-423). */
MUT_FN int grid_orbit_row(const mut_grid *g, int v)
{
  if(g->s == 1) return v;
  int x = gx(v, g->h), y = gy(v, g->h);
  if(g->s == 2) return (x < g->bw) ? v : grid_rot(g, v, 180);
  if(x < g->bw && y < g->bh) return grid_row(g, v);
  if(x < g->bw)  return grid_row(g, grid_rot(g, v, 270));
  if(y >= g->bh) return grid_row(g, grid_rot(g, v, 180));
  return grid_row(g, grid_rot(g, v, 90));
}

/* adjacency[v][slot] = u through the symmetry (set_adjacency, utils.c:425-459). */
MUT_FN void grid_record(mut_grid *g, int row, int slot)
{
  if(g->nw < 4){ g->wrow[g->nw] = row; g->wslot[g->nw] = slot; g->nw++; }
}

MUT_FN void grid_put(mut_grid *g, int v, int slot, int u)
{
  const int d = g->d;
  int row, val;
  if(g->s == 1){ row = v; val = u; }
  else{
    int x = gx(v, g->h), y = gy(v, g->h);
    if(g->s == 2){
      if(x < g->bw){ row = v; val = u; }
      else{ row = grid_rot(g, v, 180); val = grid_rot(g, u, 180); }
    }
    else if(x < g->bw && y < g->bh){ row = grid_row(g, v); val = u; }
    else if(x < g->bw){ row = grid_row(g, grid_rot(g, v, 270)); val = grid_rot(g, u, 270); }
    else if(y >= g->bh){ row = grid_row(g, grid_rot(g, v, 180)); val = grid_rot(g, u, 180); }
    else{ row = grid_row(g, grid_rot(g, v, 90)); val = grid_rot(g, u, 90); }
  }
  g->adj[(long long)row * d + slot] = val;
  grid_record(g, row, slot);
}

MUT_FN int grid_deg(const mut_grid *g, int v)
{
  return g->ndeg ? g->ndeg[grid_orbit_row(g, v)] : g->d;
}

MUT_FN bool grid_short(const mut_grid *g, int u, int v)      /* CHECK_LENGTH, utils.c:52-56 */
{
  if(g->xy)
    return mut_abs(g->xy[2 * u] - g->xy[2 * v]) + mut_abs(g->xy[2 * u + 1] - g->xy[2 * v + 1]) <= g->len;
  return mut_abs(gx(u, g->h) - gx(v, g->h)) + mut_abs(gy(u, g->h) - gy(v, g->h)) <= g->len;
}

MUT_FN bool grid_is_antipodal(const mut_grid *g, int u, int v)  /* IS_DIAMETER_GRID, utils.c:104-110 */
{
  return g->s != 1 && u == grid_rot(g, v, 180);
}

/* get_degree_index_grid, utils.c:534-557 */
MUT_FN int grid_back_slot(const mut_grid *g, int u, int v, int u_slot)
{
  if(u == v){
    int dd = grid_deg(g, v);
    for(int i = 0; i < dd; i++)
      if(grid_nbr(g, v, i) == u && i != u_slot) return i;
  }
  else if(g->s != 1 && u == grid_rot(g, v, 180)){
    return u_slot;
  }
  else{
    int dd = grid_deg(g, v);
    for(int i = 0; i < dd; i++)
      if(grid_nbr(g, v, i) == u) return i;
  }
  return -1;
}

/* check_rotated_edges_overlap_grid, utils.c:766-782 */
MUT_FN bool grid_same_orbit(const mut_grid *g, int u0, int v0, int u1, int v1)
{
  if(g->s == 2)
    return (u0 == grid_rot(g, u1, 180) && v0 == grid_rot(g, v1, 180)) ||
           (u0 == grid_rot(g, v1, 180) && v0 == grid_rot(g, u1, 180));
  if(g->s == 4){
    for(int deg = 90; deg <= 270; deg += 90)
      if(u0 == grid_rot(g, u1, deg) && v0 == grid_rot(g, v1, deg)) return true;
    for(int deg = 90; deg <= 270; deg += 90)
      if(u0 == grid_rot(g, v1, deg) && v0 == grid_rot(g, u1, deg)) return true;
  }
  return false;
}

/* mutate_adjacency_1opt_grid_s, utils.c:790-822 */
MUT_FN int grid_one_opt(mut_rng *rng, mut_grid *g, int u, int us)
{
  int s = g->s;
  int v = grid_nbr(g, u, us);
  if(grid_is_antipodal(g, u, v)) return 0;
  if(s == 2 && u == grid_rot(g, v, 180)) return 0;
  if(s == 4 && (u == grid_rot(g, v, 90) || u == grid_rot(g, v, 270))) return 0;
  int vs = grid_back_slot(g, u, v, us);
  if(vs < 0) return -1;
  int k = MUT_BELOW(rng, s);
  if(k != s - 1){
    int nv = grid_rot(g, v, (k + 1) * (360 / s));
    int nu = grid_rot(g, u, (s - k - 1) * (360 / s));
    if(!grid_short(g, u, nv)) return 0;
    grid_put(g, nv, vs, u);
    grid_put(g, nu, us, v);
  }
  else{
    int nv = grid_rot(g, u, 180);
    int nu = grid_rot(g, v, 180);
    if(!grid_short(g, u, nv) || !grid_short(g, v, nu)) return 0;
    grid_put(g, nv, us, u);
    grid_put(g, nu, vs, v);
  }
  return 1;
}

/* One 2-opt attempt on a grid(_s) graph (mutate_adjacency_2opt_grid_s,
 * utils.c:824-971).  1: the swap was made (g->nw writes, *r filled); 0: the
 * attempt was rejected and the caller retries; -1: no back slot for a drawn
 * edge, or the draws ran out of tries. */
MUT_FN int mut_grid_two_opt(mut_rng *rng, mut_grid *g, ODP_Restore *r)
{
  int u[2], v[2], us[2], vs[2];
  const int n = g->n;
  g->nw = 0;
  for(long long tries = 0;; tries++){
    if(MUT_TRIES && tries >= MUT_TRIES) return -1;
    u[0] = MUT_BELOW(rng, n);
    u[1] = MUT_BELOW(rng, n);
    if(u[0] == u[1]) continue;
    us[0] = MUT_BELOW(rng, grid_deg(g, u[0]));
    v[0] = grid_nbr(g, u[0], us[0]);
    if(v[0] == u[1]) continue;
    us[1] = MUT_BELOW(rng, grid_deg(g, u[1]));
    v[1] = grid_nbr(g, u[1], us[1]);
    if(v[1] == u[0] || v[0] == v[1]) continue;
    break;
  }
  /* The reverse slots draw no random numbers, so they are looked up only
   * once a proposal has passed its cheap tests; vs_ready tracks it. */
  bool vs_ready = false;
#define RESOLVE_BACK_SLOTS() do{ if(!vs_ready){ \
    vs[0] = grid_back_slot(g, u[0], v[0], us[0]); \
    vs[1] = grid_back_slot(g, u[1], v[1], us[1]); \
    if(vs[0] < 0 || vs[1] < 0) return -1; \
    mut_fill_restore(r, u, us, v, vs); vs_ready = true; } }while(0)

  bool a0 = grid_is_antipodal(g, u[0], v[0]), a1 = grid_is_antipodal(g, u[1], v[1]);
  if(a0 && a1){
    if(g->s == 4 && (u[0] == grid_rot(g, u[1], 90) || u[0] == grid_rot(g, u[1], 270))) return 0;
    int t0, t1;
    if(MUT_BELOW(rng, 2)){ if(!grid_short(g, u[0], u[1])) return 0; t0 = u[1]; t1 = u[0]; }
    else                     { if(!grid_short(g, u[0], v[1])) return 0; t0 = v[1]; t1 = v[0]; }
    RESOLVE_BACK_SLOTS();
    grid_put(g, u[0], us[0], t0);
    grid_put(g, u[1], us[1], t1);
    return 1;
  }
  if(a0 || a1){
    RESOLVE_BACK_SLOTS();       /* the restore record keeps the unswapped order */
    if(a1){
      int t;
      t = u[0]; u[0] = u[1]; u[1] = t;
      t = us[0]; us[0] = us[1]; us[1] = t;
      t = v[0]; v[0] = v[1]; v[1] = t;
      t = vs[0]; vs[0] = vs[1]; vs[1] = t;
    }
    int k = MUT_BELOW(rng, 4), t[4];
    int u1o = grid_rot(g, u[1], 180), v1o = grid_rot(g, v[1], 180);
    switch(k){
    case 0:
      if(!grid_short(g, u[0], v[1]) || !grid_short(g, u[1], u1o)) return 0;
      t[0] = v[1]; t[1] = u1o; t[2] = v1o; t[3] = u[0];
      break;
    case 1:
      if(!grid_short(g, u[0], v1o) || !grid_short(g, u[1], u1o)) return 0;
      t[0] = v1o; t[1] = u1o; t[2] = v[1]; t[3] = v[0];
      break;
    case 2:
      if(!grid_short(g, u[0], u[1]) || !grid_short(g, v[1], v1o)) return 0;
      t[0] = u[1]; t[1] = u[0]; t[2] = u1o; t[3] = v1o;
      break;
    default:
      if(!grid_short(g, u[0], u1o) || !grid_short(g, v[1], v1o)) return 0;
      t[0] = u1o; t[1] = v[0]; t[2] = u[1]; t[3] = v1o;
      break;
    }
    grid_put(g, u[0], us[0], t[0]);
    grid_put(g, u[1], us[1], t[1]);
    grid_put(g, v[0], vs[0], t[2]);
    grid_put(g, v[1], vs[1], t[3]);
    return 1;
  }

  if(grid_same_orbit(g, u[0], v[0], u[1], v[1])){
    RESOLVE_BACK_SLOTS();
    return grid_one_opt(rng, g, u[0], us[0]);
  }

  int t[4];
  int cross = MUT_BELOW(rng, 2);
  {
    /* Length test first and without a data-dependent branch: almost every
     * proposal on a large grid fails here. */
    int pu = cross ? v[1] : u[1], pv = cross ? u[1] : v[1];
    if(!(grid_short(g, u[0], pu) & grid_short(g, v[0], pv))) return 0;
  }
  if(cross){                            /* u0--v1, v0--u1 */
    if(grid_is_antipodal(g, u[0], v[1]) || grid_is_antipodal(g, v[0], u[1])) return 0;
    if(grid_same_orbit(g, u[0], v[1], v[0], u[1])) return 0;
    t[0] = v[1]; t[1] = v[0]; t[2] = u[1]; t[3] = u[0];
  }
  else{                                 /* u0--u1, v0--v1 */
    if(grid_is_antipodal(g, u[0], u[1]) || grid_is_antipodal(g, v[0], v[1])) return 0;
    if(grid_same_orbit(g, u[0], u[1], v[0], v[1])) return 0;
    t[0] = u[1]; t[1] = u[0]; t[2] = v[1]; t[3] = v[0];
  }
  RESOLVE_BACK_SLOTS();
  grid_put(g, u[0], us[0], t[0]);
  grid_put(g, u[1], us[1], t[1]);
  grid_put(g, v[0], vs[0], t[2]);
  grid_put(g, v[1], vs[1], t[3]);
  return 1;
#undef RESOLVE_BACK_SLOTS
}


/* ODP_Restore_adjacency_grid (utils.c:461-467), recording the writes. */
MUT_FN void mut_grid_restore(mut_grid *g, const ODP_Restore *r)
{
  g->nw = 0;
  for(int i = 0; i < 2; i++){
    grid_put(g, r->u[i], r->u_d[i], r->v[i]);
    grid_put(g, r->v[i], r->v_d[i], r->u[i]);
  }
}

#endif

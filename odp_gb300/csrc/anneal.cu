/*
 * anneal.cu -- simulated-annealing chains that live on the GPU.
 *
 * The reference's annealing clients (sample/SA/general.c:160-191,
 * general_s.c:170-191, grid.c:170-191, grid_s.c:180-201) loop on the host:
 * ODP_Mutate_adjacency_general_s (or _grid_s),
 * ODP_Set_aspl (which uploads the whole adjacency), then accept_s
 * (sample/SA/common.c:15-37) and ODP_Restore_adjacency_general when the move
 * is rejected, then temp *= cooling_rate.  Here every part of that step runs
 * on the device for many chains at once, with no host round trip:
 *
 *   propose  one thread per chain draws a 2-opt swap from the chain's own
 *            glibc-compatible stream (the same swap rule as the host utilities,
 *            odp_mutate.h) and writes it into the compact adjacency and the
 *            engine's neighbour table (s orbit rows per changed slot);
 *   evaluate the persistent engine evaluates every chain's graph as one batch;
 *   decide   one block per chain reads its graph's accumulator, tracks the
 *            best graph (copied by the block), applies accept_s (one draw
 *            from the stream when the move is worse at equal diameter), undoes
 *            a rejected swap and cools the temperature.
 *
 * Each proposal's retry loops are bounded; a chain whose draws run out (a
 * graph on which the reference would loop for ever) stops with
 * GBX_CHAIN_ERR_SWAP instead of spinning.
 */
#include <cuda_runtime.h>
#include <climits>
#include <cstdint>
#include <cfloat>
#include "odp_engine.h"

namespace {

/* glibc's TYPE_3 stream (r[i] = r[i-31] + r[i-3], output r[i] >> 1) over a
 * ring of its last 31 words, ring[pos] = r[i-31]. */
struct dev_rng {
  unsigned int ring[31];
  int pos;
};

__device__ __forceinline__ int rng_next(dev_rng *g)
{
  const int p = g->pos;
  const unsigned int x = g->ring[p] + g->ring[p >= 3 ? p - 3 : p + 28];
  g->ring[p] = x;
  g->pos = (p == 30) ? 0 : p + 1;
  return (int)(x >> 1);
}

/* get_random (utils.c:361-364): the integer form is exact where the double
 * product is (max <= 2^22); above it the same double arithmetic. */
__device__ __forceinline__ int rng_below(dev_rng *g, int max)
{
  const int x = rng_next(g);
  if(max >= 0 && max <= (1 << 22))
    return (int)(((unsigned long long)(unsigned)x * (unsigned long long)max) >> 31);
  return (int)(x * ((double)max) / (1.0 + 2147483647.0));
}

}  // namespace

typedef dev_rng mut_rng;
#define MUT_BELOW(rng, max) rng_below((rng), (max))
#define MUT_TRIES (1LL << 22)
#define MUT_FN static __device__ inline
#include "odp_mutate.h"

namespace {

#define ANNEAL_MAX_ATTEMPTS (1 << 20)   /* rejected 2-opt attempts per proposal */
#define DECIDE_THREADS 256

/* The neighbour-table rows of the slots a swap (or its undo) wrote: orbit
 * row t of base row m is vertex m + t*base, whose entry is the stored value
 * shifted by t*base (the expansion rule of the engine's neighbour table). */
__device__ void apply_to_nbr(const gbx_chain &c, const mut_general &g)
{
  for(int k = 0; k < g.nw; k++){
    const int row = g.wrow[k], slot = g.wslot[k];
    const int a = c.adj[(long long)row * c.d + slot];
    for(int t = 0; t < c.s; t++){
      const int v = row + t * c.base;
      int nb = a + t * c.base;
      if(nb >= c.n) nb -= c.n;
      c.nbr[(long long)v * c.dp + slot] = nb;
    }
  }
}

__device__ __forceinline__ mut_general chain_graph(const gbx_chain &c)
{
  mut_general g;
  g.n = c.n; g.d = c.d; g.s = c.s; g.base = c.base;
  g.ndeg = c.ndeg; g.adj = c.adj; g.nw = 0;
  return g;
}

__device__ __forceinline__ mut_grid chain_grid(const gbx_chain &c)
{
  mut_grid g;
  g.w = c.width; g.h = c.height; g.d = c.d; g.s = c.s; g.len = c.len; g.n = c.n;
  g.bw = c.width / 2; g.bh = (c.s == 2) ? c.height : c.height / 2;
  g.ndeg = c.ndeg; g.adj = c.adj; g.xy = nullptr; g.nw = 0;
  return g;
}

/* The same for a grid chain.  Without symmetry a row is its vertex.  With
 * symmetry s (2 or 4) local row m stores base vertex bv (the inverse of
 * ODP_LOCAL_INDEX_GRID); the orbit member rotated by t steps is vertex
 * rot(bv), its neighbour rot(a), and the table indexes both through itable,
 * as expand_kernel builds it. */
__device__ void apply_to_nbr_grid(const gbx_chain &c, const mut_grid &g)
{
  for(int k = 0; k < g.nw; k++){
    const int m = g.wrow[k], slot = g.wslot[k];
    const int a = c.adj[(long long)m * c.d + slot];
    if(c.s == 1){
      c.nbr[(long long)m * c.dp + slot] = a;
      continue;
    }
    const int bv = (c.s == 2) ? m : (m / g.bh) * c.height + (m % g.bh);
    for(int t = 0; t < c.s; t++){
      int v = bv, u = a;
      if(t > 0){
        const int deg = (c.s == 2) ? 180 : 90 * t;
        v = grid_rot(&g, bv, deg);
        u = grid_rot(&g, a, deg);
      }
      c.nbr[(long long)c.itable[v] * c.dp + slot] = c.itable[u];
    }
  }
}

__global__ void anneal_propose_kernel(gbx_chain *chains, int count)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= count) return;
  gbx_chain &c = chains[i];
  if(c.status) return;
  dev_rng rng;
  for(int k = 0; k < 31; k++) rng.ring[k] = c.ring[k];
  rng.pos = c.ring_pos;
  ODP_Restore r;
  int e = 0;
  if(c.grid){
    mut_grid g = chain_grid(c);
    for(int attempt = 0; attempt < ANNEAL_MAX_ATTEMPTS && e == 0; attempt++) e = mut_grid_two_opt(&rng, &g, &r);
    if(e == 1) apply_to_nbr_grid(c, g);
  }
  else{
    mut_general g = chain_graph(c);
    for(int attempt = 0; attempt < ANNEAL_MAX_ATTEMPTS && e == 0; attempt++) e = mut_two_opt(&rng, &g, &r);
    if(e == 1) apply_to_nbr(c, g);
  }
  for(int k = 0; k < 31; k++) c.ring[k] = rng.ring[k];
  c.ring_pos = rng.pos;
  if(e != 1){
    c.status = GBX_CHAIN_ERR_SWAP;
    return;
  }
  c.last = r;
}

/* accept_s (sample/SA/common.c:15-37); uniform_rand (common.c:10-13) is
 * (random() + 1) / (RAND_MAX + 2) from the same stream as the proposals. */
__device__ bool accept_move(gbx_chain &c, dev_rng *rng, int diameter, double aspl)
{
  if(c.hill_climbing) return aspl <= c.cur_aspl;
  if(diameter < c.cur_diameter && !c.aspl_priority) return true;
  if(diameter > c.cur_diameter && !c.aspl_priority) return false;
  if(aspl <= c.cur_aspl) return true;
  const double diff = ((c.cur_aspl - aspl) * c.n * (c.n - 1)) / c.s;
  const double u = ((double)rng_next(rng) + 1.0) / ((double)2147483647 + 2.0);
  return exp(diff / c.temp) > u;
}

__global__ void __launch_bounds__(DECIDE_THREADS)
anneal_decide_kernel(gbx_chain *chains, int count, const gbx_graph_acc *acc, const gbx_ctrl *ctrl,
                     const unsigned int *err)
{
  __shared__ int sh_run, sh_copy, sh_accept;
  gbx_chain &c = chains[blockIdx.x];
  if(threadIdx.x == 0){
    sh_run = (c.status == 0);
    sh_copy = 0;
    sh_accept = 0;
    if(sh_run && ((ctrl->error | *err) & (GBX_ERR_TIMEOUT | GBX_ERR_BAD_ADJ))){
      c.status = GBX_CHAIN_ERR_EVAL;
      sh_run = 0;
    }
    if(sh_run){
      /* the result as ODP_Set_aspl reports it (aspl_cuda.cu:84-85, 256-260) */
      const gbx_graph_acc a = acc[c.graph];
      int diameter;
      long long sum;
      double aspl;
      if(a.flags & 1){ diameter = INT_MAX; sum = LLONG_MAX; aspl = DBL_MAX; }
      else{
        const long long total = (long long)a.sum;
        diameter = a.levels;
        aspl = total / (((double)c.n - 1) * c.n);
        sum = (long long)(total / 2.0);
      }
      c.steps++;
      if(diameter < c.best_diameter || (diameter == c.best_diameter && aspl < c.best_aspl)){
        c.best_diameter = diameter;
        c.best_sum = sum;
        c.best_aspl = aspl;
        sh_copy = 1;
      }
      dev_rng rng;
      for(int k = 0; k < 31; k++) rng.ring[k] = c.ring[k];
      rng.pos = c.ring_pos;
      sh_accept = accept_move(c, &rng, diameter, aspl);
      for(int k = 0; k < 31; k++) c.ring[k] = rng.ring[k];
      c.ring_pos = rng.pos;
      if(sh_accept){
        c.cur_diameter = diameter;
        c.cur_sum = sum;
        c.cur_aspl = aspl;
        c.accepted++;
      }
    }
  }
  __syncthreads();
  if(sh_copy){
    /* the pointers are read once: a store through best_adj could otherwise
     * alias the chain record and force a reload per element */
    const int *__restrict__ src = c.adj;
    int *__restrict__ dst = c.best_adj;
    const long long words = (long long)c.base * c.d;
    if(((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0){
      const long long q = words >> 2;
      const int4 *s4 = reinterpret_cast<const int4 *>(src);
      int4 *d4 = reinterpret_cast<int4 *>(dst);
      for(long long k = threadIdx.x; k < q; k += blockDim.x) d4[k] = s4[k];
      for(long long k = (q << 2) + threadIdx.x; k < words; k += blockDim.x) dst[k] = src[k];
    }
    else{
      for(long long k = threadIdx.x; k < words; k += blockDim.x) dst[k] = src[k];
    }
  }
  __syncthreads();                       /* the copy has read adj before an undo rewrites it */
  if(threadIdx.x == 0 && sh_run){
    if(!sh_accept){
      if(c.grid){
        mut_grid g = chain_grid(c);
        mut_grid_restore(&g, &c.last);
        apply_to_nbr_grid(c, g);
      }
      else{
        mut_general g = chain_graph(c);
        mut_restore(&g, &c.last);
        apply_to_nbr(c, g);
      }
    }
    c.temp *= c.cooling;
  }
}

}  // namespace

extern "C" int gbx_anneal_propose(gbx_chain *d_chains, int count, void *stream)
{
  if(count <= 0) return 0;
  anneal_propose_kernel<<<(count + 127) / 128, 128, 0, (cudaStream_t)stream>>>(d_chains, count);
  return (int)cudaGetLastError();
}

extern "C" int gbx_anneal_decide(gbx_chain *d_chains, int count, const gbx_graph_acc *d_acc, const gbx_ctrl *d_ctrl,
                                 const unsigned int *d_err, void *stream)
{
  if(count <= 0) return 0;
  anneal_decide_kernel<<<count, DECIDE_THREADS, 0, (cudaStream_t)stream>>>(d_chains, count, d_acc, d_ctrl, d_err);
  return (int)cudaGetLastError();
}

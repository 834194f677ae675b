/*
 * aspl_engine.cu -- the GB300 (sm_103a) kernels of the ODP ASPL/diameter
 * evaluation and the thin extern "C" layer the host C driver calls.
 *
 * The computation is the reference's bitset BFS (aspl_cuda.cu:53-126,
 * utils_cuda.cu:97-211): rows are vertices, bits are source vertices (the
 * n/s base vertices of a symmetric graph), and level k sets bit (v, src)
 * when src is within distance k of v:
 *
 *     P_k[v] = P_{k-1}[v] | OR_{u in N(v)} P_{k-1}[u],     P_0 = identity
 *
 * which is what the reference's A/B double buffer computes (its B keeps
 * P_{k-2}, and P_{k-2}[v] | OR P_{k-1}[u] = P_k[v] because P only grows).
 * popcount(P_k) decides termination and the sum exactly as the reference's
 * host loop does (aspl_cuda.cu:62-82, 102-121).
 *
 * GB300 design, instead of the reference's per-level kernel + popcount
 * kernel + blocking D2H copy:
 *  - expand_kernel turns the compact adjacency (n/s rows, symmetry-relative
 *    ids, grid rotations) into a row-space neighbour table nbr[n][dp] once
 *    per upload; the rotation/itable arithmetic of utils_cuda.cu:3-59 and
 *    :117-151 runs there, not once per (row, word, level).
 *  - engine_kernel is persistent (grid = SMs x resident CTAs).  Work is a
 *    queue of jobs = (graph, column chunk); active jobs sit in slots, each
 *    slot runs BFS levels, and each level is split into row tiles handed out
 *    through a 64-bit ticket (ntiles << 32 | next).  The CTA finishing a
 *    level's last tile decides, on the device, whether the job is complete,
 *    stalled (disconnected) or opens the next level; a finished job folds its
 *    sum into the graph's accumulator and the slot loads the next job.  CTAs
 *    never wait on each other except when idle (bounded by a time limit that
 *    raises GBX_ERR_TIMEOUT).
 *  - Level 1 is built straight from the neighbour table (no clear/identity
 *    pass); levels >= 2 OR-gather 128-bit vectors of the d neighbour rows
 *    (L2-only loads: the buffers are rewritten by other SMs between levels),
 *    and the popcount is fused: warp __reduce_add_sync, one 64-bit atomic per
 *    tile.
 *  - A job whose level fits in one tile (small graphs) is run to completion
 *    by the CTA that took it, with no device-wide handshake per level.
 */
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>
#include "odp_engine.h"
#include <cooperative_groups.h>

namespace cg = cooperative_groups;

#define ENGINE_THREADS 256
#define ENGINE_WARPS (ENGINE_THREADS / 32)
#ifndef ENGINE_MIN_BLOCKS
#define ENGINE_MIN_BLOCKS 4         /* resident CTAs per SM the register budget is sized for */
#endif

namespace {

__device__ __forceinline__ unsigned popc4(const uint4 &v)
{
  return __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
}

__device__ __forceinline__ void or_into(uint4 &a, const uint4 &b)
{
  a.x |= b.x; a.y |= b.y; a.z |= b.z; a.w |= b.w;
}

template <typename T>
__device__ __forceinline__ T vload(const T *p) { return *(const volatile T *)p; }

__device__ __forceinline__ unsigned long long globaltimer()
{
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

/* ---------------------------------------------------------------------- */
/* Neighbour-table expansion.                                              */
/* ---------------------------------------------------------------------- */

/* ODP_ROTATE for the grid symmetries (reference utils_cuda.cu:3-14). */
__device__ __forceinline__ int grid_rotate(int v, int width, int height, int s, int deg)
{
  int x = v / height, y = v % height;
  if(s == 2) return (width - x - 1) * height + (height - y - 1);
  if(deg == 90)  return y * height + (height - x - 1);
  if(deg == 180) return (height - x - 1) * height + (height - y - 1);
  return (height - y - 1) * height + x;
}

/* Row of a base-quadrant vertex (utils_cuda.cu:16-23). */
__device__ __forceinline__ int grid_base_row(int x, int height, int s)
{
  if(s == 2) return x;
  return (x / height) * (height / 2) + x % height;
}

/* Neighbour j of global vertex v of a rotation-symmetric grid
 * (utils_cuda.cu:25-59), read from the compact adjacency `adj`; -1 when the
 * stored entry is out of range. */
__device__ __forceinline__ int grid_source_row(const gbx_expand_desc &e, int v, int &back)
{
  const int w = e.width, h = e.height, s = e.s;
  int x = v / h, y = v % h, bw = w / 2, bh = h / 2;
  if(s == 2){
    if(x < bw){ back = 0; return v; }
    back = 180;
    return grid_rotate(v, w, h, s, 180);
  }
  if(x < bw && y < bh){ back = 0; return grid_base_row(v, h, s); }
  if(x < bw)          { back = 90; return grid_base_row(grid_rotate(v, w, h, s, 270), h, s); }
  if(y >= bh)         { back = 180; return grid_base_row(grid_rotate(v, w, h, s, 180), h, s); }
  back = 270;
  return grid_base_row(grid_rotate(v, w, h, s, 90), h, s);
}

/* Compact-adjacency position of entry j of global vertex v, and the
 * rotation that maps the stored value back (grid symmetry) or the shift
 * that does (general symmetry). */
__device__ __forceinline__ size_t entry_source(const gbx_expand_desc &e, int v, int j, int &back)
{
  if(e.grid_s) return (size_t)grid_source_row(e, v, back) * e.d + j;
  const int base = e.n / e.s;
  back = (v / base) * base;
  return (size_t)(v % base) * e.d + j;
}

/* Row-table entry from the stored value `a` of entry (v, j) (entries at or
 * past the vertex's degree hold the row itself, and so does an out-of-range
 * value, which also sets `bad`): the rotated vertex's row for symmetric
 * grids, the shifted vertex (mod n) for general symmetry. */
__device__ __forceinline__ int expand_value(const gbx_expand_desc &e, int a, int back, int j, int deg, int row,
                                            bool &bad)
{
  if(j >= deg) return row;
  if(a < 0 || a >= e.n){ bad = true; return row; }
  if(e.grid_s) return e.itable[back ? grid_rotate(a, e.width, e.height, e.s, back) : a];
  const int nb = a + back;
  return nb >= e.n ? nb - e.n : nb;
}

/* One descriptor per blockIdx.y: its compact adjacency, read from host
 * memory by consecutive threads in 16-byte pieces when both ends are 16-byte
 * aligned, else in 4-byte pieces.  The descriptors come from pinned host
 * memory (`hdescs`: this call's adjacency pointers); block (0, y) stores
 * descriptor y into `ddescs` for expand_kernel.  All blocks together also
 * copy the plan's initial engine state (`state_init`, `state_words` 8-byte
 * words, device memory) over `state`. */
__global__ void pull_kernel(const gbx_expand_desc *hdescs, gbx_expand_desc *ddescs,
                            unsigned long long *__restrict__ state, const unsigned long long *__restrict__ state_init,
                            long long state_words)
{
  __shared__ gbx_expand_desc s_desc;
  const long long nthreads = (long long)gridDim.x * gridDim.y * blockDim.x;
  const long long tid = ((long long)blockIdx.y * gridDim.x + blockIdx.x) * blockDim.x + threadIdx.x;
  for(long long i = tid; i < state_words; i += nthreads) state[i] = state_init[i];
  if(threadIdx.x == 0){
    s_desc = hdescs[blockIdx.y];
    if(blockIdx.x == 0) ddescs[blockIdx.y] = s_desc;
  }
  __syncthreads();
  const gbx_expand_desc &e = s_desc;
  if(!e.adj_dev) return;
  const long long ints = (long long)(e.n / e.s) * e.d;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(((reinterpret_cast<uintptr_t>(e.adj) | reinterpret_cast<uintptr_t>(e.adj_dev)) & 15) == 0){
    const int4 *src = reinterpret_cast<const int4 *>(e.adj);
    int4 *dst = reinterpret_cast<int4 *>(e.adj_dev);
    const long long q = ints >> 2;
    for(long long i = t0; i < q; i += stride) dst[i] = src[i];
    for(long long i = (q << 2) + t0; i < ints; i += stride) e.adj_dev[i] = e.adj[i];
  }
  else{
    for(long long i = t0; i < ints; i += stride) e.adj_dev[i] = e.adj[i];
  }
}

#define EXPAND_GROUP 8         /* neighbour entries per thread, loaded before any is stored */

/* Thread (global vertex gv, group blockIdx.y) writes entries [8y, 8y + 8)
 * of gv's row of its graph's neighbour table: all eight compact-adjacency
 * loads are issued before the first store. */
__global__ void expand_kernel(const gbx_expand_desc *__restrict__ descs, int ndesc, long long total,
                              unsigned int *err)
{
  const int j0 = (int)blockIdx.y * EXPAND_GROUP;
  for(long long gv = blockIdx.x * (long long)blockDim.x + threadIdx.x; gv < total;
      gv += (long long)gridDim.x * blockDim.x){
    int lo = 0, hi = ndesc - 1;
    while(lo < hi){
      int mid = (lo + hi + 1) >> 1;
      if(descs[mid].first_vertex <= gv) lo = mid; else hi = mid - 1;
    }
    const gbx_expand_desc &e = descs[lo];
    const int d = e.d, dp = e.dp;
    if(j0 >= dp) continue;
    const int *adj = e.adj_dev ? e.adj_dev : e.adj;
    const int v = (int)(gv - e.first_vertex);
    bool bad = false;
    int deg = e.ndeg ? e.ndeg[v] : d;
    if(deg < 0 || deg > d){ bad = true; deg = deg < 0 ? 0 : d; }
    const int row = e.grid_s ? e.itable[v] : v;
    int *out = e.nbr + (size_t)row * dp;
    /* Entries that are not neighbours (beyond the vertex's degree, padding,
     * or out of range, which is also reported) hold the row itself: OR-ing a
     * row into itself changes nothing, so the gather needs no test. */
    int val[EXPAND_GROUP], back[EXPAND_GROUP];
#pragma unroll
    for(int k = 0; k < EXPAND_GROUP; k++){
      const int j = j0 + k;
      back[k] = 0;
      val[k] = j < deg ? adj[entry_source(e, v, j, back[k])] : 0;
    }
#pragma unroll
    for(int k = 0; k < EXPAND_GROUP; k++){
      const int j = j0 + k;
      if(j < dp) out[j] = expand_value(e, val[k], back[k], j, deg, row, bad);
    }
    if(bad) atomicOr(err, GBX_ERR_BAD_ADJ);
  }
}

/* ---------------------------------------------------------------------- */
/* Row passes.  WC = uint64 words per row of the chunk (a power of two).   */
/* A row is covered by G lanes, each holding V 16-byte vectors.            */
/* ---------------------------------------------------------------------- */

template <int WC>
struct RowShape {
  static constexpr int VPR = WC / 2;                 /* uint4 vectors per row */
  static constexpr int G = VPR < 32 ? VPR : 32;      /* lanes per row */
  static constexpr int V = VPR / G;                  /* vectors per lane */
  static constexpr int RPW = 32 / G;                 /* rows per warp pass */
  static constexpr bool LEAN = false;                /* change tests by comparing words */
};

/* The shape of the row passes the engine runs: half as many lanes per row,
 * two vectors each, so a warp pass covers twice the rows and each lane
 * issues both vectors of every neighbour it gathers back to back.  On
 * GB300 it cut the 512-graph batch from 6.90 to 6.21 ms (tuned), the
 * n = 65536 graph from 2.81 to 2.60 ms and the 256 x 256 grid, where few
 * neighbours of a row change per level, from 21.2 to 18.4 ms.  (RowShape,
 * one vector per lane up to 32 lanes per row, remains for change-tracking
 * jobs in plans that mix both kinds and for the small-graph kernel, where
 * two vectors per lane made the partitioned grids 10-33 % slower: their
 * gathers from other CTAs' shared memory go one 16-byte request at a time.) */
template <int WC>
struct RowShapeWide {
  static constexpr int VPR = WC / 2;
  static constexpr int G = VPR >= 64 ? 32 : (VPR >= 2 ? VPR / 2 : 1);
  static constexpr int V = VPR / G;
  static constexpr int RPW = 32 / G;
  static constexpr bool LEAN = true;                 /* change tests by popcount: words only grow */
};

/* Set local source bit b (0 <= b < nsrc) if it lands in this lane's vectors. */
template <class S>
__device__ __forceinline__ void mark_source(uint4 (&acc)[S::V], int b, int nsrc, int gl)
{
  if((unsigned)b >= (unsigned)nsrc) return;
  const int vec = b >> 7;
  const unsigned bit = 1u << (b & 31);
  const int comp = (b >> 5) & 3;
#pragma unroll
  for(int k = 0; k < S::V; k++){
    if(vec == gl + k * S::G){
      acc[k].x |= (comp == 0) ? bit : 0u;
      acc[k].y |= (comp == 1) ? bit : 0u;
      acc[k].z |= (comp == 2) ? bit : 0u;
      acc[k].w |= (comp == 3) ? bit : 0u;
    }
  }
}

/* Shared-memory budget for one block of neighbour lists (ints). */
#define IDX_SMEM_INTS 4096
#define BLOCK_ROWS_MAX (IDX_SMEM_INTS / 4)

/* Per-block staging area: the block's neighbour lists and two per-row lane
 * masks.  Without change tracking, `own` holds the lanes whose words were
 * saturated (every source bit of the lane set) at the previous level and
 * `act` those saturated two levels back.  With change tracking, `nmask`
 * holds the previous level's change masks of the neighbours, `own` the row's
 * own and `act` the union of both (rows whose lanes have nothing to do are
 * skipped).  Launches without change tracking get the area up to `nmask`. */
struct Stage {
  int idx[IDX_SMEM_INTS];
  unsigned own[BLOCK_ROWS_MAX];
  unsigned act[BLOCK_ROWS_MAX];
  unsigned nmask[IDX_SMEM_INTS];
};

/* Source bits a lane holds in one row of a chunk of nsrc sources: its
 * vectors gl, gl + G, ... each cover 128 source ordinals. */
template <int WC, class S = RowShape<WC>>
__device__ __forceinline__ int lane_sources(int nsrc, int gl)
{
  int v = 0;
#pragma unroll
  for(int k = 0; k < S::V; k++) v += min(max(nsrc - 128 * (gl + k * S::G), 0), 128);
  return v;
}

/* Source ordinal of a row (the bit it owns across the chunks): the row
 * itself, or from the graph's source table (SP). */
template <bool SP>
__device__ __forceinline__ int source_of(const int *srcpos, int row)
{
  if(!SP) return row;
  return row < 0 ? -1 : __ldg(srcpos + row);
}

/* Level 1: P_1[v] = {v} u N(v), restricted to the chunk's sources, and the
 * lanes of each row whose words differ from the identity P_0. */
template <int WC, bool ACT, bool SP, class S = RowShape<WC>>
__device__ unsigned rows_level1(const Stage &st, int dp, const gbx_job &jb, unsigned long long *Y,
                                unsigned *Mcur, int row0, int nrows)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane / S::G, gl = lane % S::G;
  const int src0 = jb.src0, nsrc = jb.nsrc;
  unsigned cnt = 0;
  for(int base = 0; base < nrows; base += ENGINE_WARPS * S::RPW){
    const int r = base + warp * S::RPW + sub;
    const bool valid = r < nrows;
    bool changed = false;
    if(valid){
      const int row = row0 + r;
      constexpr bool IDW = ACT && !S::LEAN;             /* the identity kept as words */
      uint4 acc[S::V], id[IDW ? S::V : 1];
#pragma unroll
      for(int k = 0; k < S::V; k++) acc[k] = make_uint4(0u, 0u, 0u, 0u);
      const int self = source_of<SP>(jb.srcpos, row) - src0;
      mark_source<S>(acc, self, nsrc, gl);
      if(IDW){
#pragma unroll
        for(int k = 0; k < S::V; k++) id[k] = acc[k];
      }
      /* LEAN: the identity's bits in this lane (0 or 1) */
      unsigned id_bits = 0;
      if(ACT && S::LEAN){
#pragma unroll
        for(int k = 0; k < S::V; k++) id_bits += popc4(acc[k]);
      }
      const int4 *ip = reinterpret_cast<const int4 *>(st.idx + r * dp);
      for(int j = 0; j < (dp >> 2); j++){
        int4 q = ip[j];
        mark_source<S>(acc, source_of<SP>(jb.srcpos, q.x) - src0, nsrc, gl);
        mark_source<S>(acc, source_of<SP>(jb.srcpos, q.y) - src0, nsrc, gl);
        mark_source<S>(acc, source_of<SP>(jb.srcpos, q.z) - src0, nsrc, gl);
        mark_source<S>(acc, source_of<SP>(jb.srcpos, q.w) - src0, nsrc, gl);
      }
      uint4 *yr = reinterpret_cast<uint4 *>(Y) + (size_t)row * S::VPR + gl;
      unsigned c = 0;
#pragma unroll
      for(int k = 0; k < S::V; k++){
        __stcg(yr + k * S::G, acc[k]);
        c += popc4(acc[k]);
        if(IDW)
          changed |= (acc[k].x != id[k].x) | (acc[k].y != id[k].y) | (acc[k].z != id[k].z) |
                     (acc[k].w != id[k].w);
      }
      if(ACT && S::LEAN) changed = c != id_bits;
      cnt += c;
      if(!ACT) changed = c == (unsigned)lane_sources<WC, S>(nsrc, gl);    /* saturated */
    }
    const unsigned bal = __ballot_sync(0xffffffffu, changed);
    if(valid && gl == 0)
      Mcur[row0 + r] = S::G == 32 ? bal : (bal >> (sub * S::G)) & ((1u << S::G) - 1u);
  }
  return cnt;
}

/* Level k >= 2 without change tracking: P_k[v] = P_{k-1}[v] | OR_j
 * P_{k-1}[nbr[v][j]] over the d neighbour columns.  Eight 16-byte loads per
 * lane are in flight per step (NB neighbours x V vectors).  Columns that
 * hold no neighbour hold the row itself, so only the step past the last
 * column needs a test.  A lane whose words were saturated at level k-1 stays
 * so: it gathers nothing, and copies its words from X only if they were not
 * already saturated at level k-2 (Y then still holds them).  Lanes past the chunk's
 * last source are saturated from level 1 on.  Returns the bits set at this
 * level; the row's saturated lanes replace its entry of `own` (the group's
 * lanes have all read it before the ballot). */
template <int WC, class S = RowShape<WC>>
__device__ unsigned rows_levelk_all(Stage &st, int dp, int d, int nsrc, const unsigned long long *X,
                                    unsigned long long *Y, int row0, int nrows)
{
  constexpr int NB = S::V >= 8 ? 1 : 8 / S::V;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane / S::G, gl = lane % S::G;
  const unsigned lane_bits = (unsigned)lane_sources<WC, S>(nsrc, gl);
  const uint4 *Xv = reinterpret_cast<const uint4 *>(X);
  unsigned cnt = 0;
  for(int r = warp * S::RPW + sub; r < nrows; r += ENGINE_WARPS * S::RPW){
    const int row = row0 + r;
    uint4 *yr = reinterpret_cast<uint4 *>(Y) + (size_t)row * S::VPR + gl;
    bool sat = (st.own[r] >> gl) & 1u;
    if(sat){
      if(!((st.act[r] >> gl) & 1u)){
#pragma unroll
        for(int k = 0; k < S::V; k++)
          __stcg(yr + k * S::G, __ldcg(Xv + (size_t)row * S::VPR + gl + k * S::G));
      }
      cnt += lane_bits;
    }
    else{
      uint4 acc[S::V];
      const uint4 *xr = Xv + (size_t)row * S::VPR + gl;
#pragma unroll
      for(int k = 0; k < S::V; k++) acc[k] = __ldcg(xr + k * S::G);
      const int *ip = st.idx + r * dp;
      for(int j = 0; j < d; j += NB){
        uint4 t[NB][S::V];
#pragma unroll
        for(int i = 0; i < NB; i++){
          const bool ok = j + i < d;
          const uint4 *nr = Xv + (size_t)ip[ok ? j + i : j] * S::VPR + gl;
#pragma unroll
          for(int k = 0; k < S::V; k++)
            t[i][k] = ok ? __ldcg(nr + k * S::G) : make_uint4(0u, 0u, 0u, 0u);
        }
#pragma unroll
        for(int i = 0; i < NB; i++)
#pragma unroll
          for(int k = 0; k < S::V; k++) or_into(acc[k], t[i][k]);
      }
      unsigned c = 0;
#pragma unroll
      for(int k = 0; k < S::V; k++){
        __stcg(yr + k * S::G, acc[k]);
        c += popc4(acc[k]);
      }
      cnt += c;
      sat = c == lane_bits;
    }
    const unsigned bal = __ballot_sync(S::G == 32 ? 0xffffffffu : (((1u << S::G) - 1u) << (sub * S::G)), sat);
    if(gl == 0) st.own[r] = S::G == 32 ? bal : (bal >> (sub * S::G)) & ((1u << S::G) - 1u);
  }
  return cnt;
}

/* Level k >= 2: P_k[v] = P_{k-1}[v] | OR over neighbours u whose lane words
 * changed at level k-1 of P_{k-1}[u] (the other neighbours' words are
 * already in P_{k-1}[v]).  Y still holds P_{k-2}; a lane writes only when
 * its words differ from that (changed at k-1 or at k), except at level 2,
 * where Y has never been written and every word is stored.  Returns the bits
 * added at this level; the row's new change mask goes to Mcur. */
template <int WC, class S = RowShape<WC>, bool LEAN = S::LEAN>
__device__ unsigned rows_levelk(const Stage &st, int dp, const unsigned long long *X, unsigned long long *Y,
                                unsigned *Mcur, int row0, int nrows, bool write_all)
{
  constexpr int NB = S::V >= 8 ? 1 : 8 / S::V;       /* neighbours gathered per step */
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane / S::G, gl = lane % S::G;
  const uint4 *Xv = reinterpret_cast<const uint4 *>(X);
  unsigned cnt = 0;
  for(int base = 0; base < nrows; base += ENGINE_WARPS * S::RPW){
    const int r = base + warp * S::RPW + sub;
    const bool valid = r < nrows;
    bool changed = false;
    if(valid && (write_all || ((st.act[r] >> gl) & 1u))){
      const int row = row0 + r;
      const bool own = (st.own[r] >> gl) & 1u;
      /* LEAN: the words only grow, so they changed exactly when their
       * popcount did; the previous words need not be kept */
      uint4 acc[S::V], old[LEAN ? 1 : S::V];
      unsigned pold = 0;
      const uint4 *xr = Xv + (size_t)row * S::VPR + gl;
#pragma unroll
      for(int k = 0; k < S::V; k++){
        acc[k] = __ldcg(xr + k * S::G);
        if(LEAN) pold += popc4(acc[k]);
        else old[k] = acc[k];
      }
      const int *ip = st.idx + r * dp;
      const unsigned *mp = st.nmask + r * dp;
      for(int j = 0; j < dp; j += NB){
        uint4 t[NB][S::V];
#pragma unroll
        for(int i = 0; i < NB; i++){
          const bool take = (j + i < dp) && ((mp[j + i] >> gl) & 1u);
          const int idx = take ? ip[j + i] : 0;
          const uint4 *nr = Xv + (size_t)idx * S::VPR + gl;
#pragma unroll
          for(int k = 0; k < S::V; k++)
            t[i][k] = take ? __ldcg(nr + k * S::G) : make_uint4(0u, 0u, 0u, 0u);
        }
#pragma unroll
        for(int i = 0; i < NB; i++)
#pragma unroll
          for(int k = 0; k < S::V; k++) or_into(acc[k], t[i][k]);
      }
      unsigned added = 0;
      if(LEAN){
#pragma unroll
        for(int k = 0; k < S::V; k++) added += popc4(acc[k]);
        added -= pold;
        changed = added != 0;
      }
      else{
#pragma unroll
        for(int k = 0; k < S::V; k++){
          added += popc4(acc[k]) - popc4(old[k]);
          changed |= (acc[k].x != old[k].x) | (acc[k].y != old[k].y) | (acc[k].z != old[k].z) |
                     (acc[k].w != old[k].w);
        }
      }
      if(own || changed || write_all){
        uint4 *yr = reinterpret_cast<uint4 *>(Y) + (size_t)row * S::VPR + gl;
#pragma unroll
        for(int k = 0; k < S::V; k++) __stcg(yr + k * S::G, acc[k]);
      }
      cnt += added;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, changed);
    if(valid && gl == 0)
      Mcur[row0 + r] = S::G == 32 ? bal : (bal >> (sub * S::G)) & ((1u << S::G) - 1u);
  }
  return cnt;
}

/* Engine instantiations by change tracking: MODE_ACTIVE compiles only the
 * passes with it (plans whose every job tracks changes), MODE_MIXED both
 * (every other plan).  An instantiation with only the passes without change
 * tracking is not built: at the 64 registers of four CTAs per SM it spilled
 * (60 bytes), where the one with both passes does not. */
#define MODE_PLAIN 0
#define MODE_ACTIVE 1
#define MODE_MIXED 2

template <int MODE>
__device__ __forceinline__ bool job_active(const gbx_job &jb)
{
  return MODE == MODE_ACTIVE || (MODE == MODE_MIXED && (jb.flags & GBX_JOB_ACTIVE));
}

template <int WC, int MODE>
__device__ unsigned run_block(Stage &st, int dp, const gbx_job &jb, int level, const unsigned long long *X,
                              unsigned long long *Y, unsigned *Mcur, int row0, int nrows)
{
  if(job_active<MODE>(jb)){
    if(MODE == MODE_ACTIVE){
      typedef RowShapeWide<WC> SW;
      if(level > 1) return rows_levelk<WC, SW>(st, dp, X, Y, Mcur, row0, nrows, level == 2);
      return jb.srcpos ? rows_level1<WC, true, true, SW>(st, dp, jb, Y, Mcur, row0, nrows)
                       : rows_level1<WC, true, false, SW>(st, dp, jb, Y, Mcur, row0, nrows);
    }
    if(level > 1) return rows_levelk<WC>(st, dp, X, Y, Mcur, row0, nrows, level == 2);
    return jb.srcpos ? rows_level1<WC, true, true>(st, dp, jb, Y, Mcur, row0, nrows)
                     : rows_level1<WC, true, false>(st, dp, jb, Y, Mcur, row0, nrows);
  }
  if(MODE == MODE_ACTIVE) return 0;
  typedef RowShapeWide<WC> SW;
  if(level > 1) return rows_levelk_all<WC, SW>(st, dp, jb.d, jb.nsrc, X, Y, row0, nrows);
  return jb.srcpos ? rows_level1<WC, false, true, SW>(st, dp, jb, Y, Mcur, row0, nrows)
                   : rows_level1<WC, false, false, SW>(st, dp, jb, Y, Mcur, row0, nrows);
}

/* Rows [r0, r1) of one level, block by block: stage the block's neighbour
 * lists (and, after level 1, the neighbours' and rows' change masks of the
 * previous level) in shared memory, then process the rows.  Returns this
 * thread's share of the level's count (level 1: bits set; later: added). */
template <int MODE>
__device__ unsigned run_rows(Stage &st, const gbx_job &jb, int level, const unsigned long long *X,
                             unsigned long long *Y, const unsigned *Mprev, unsigned *Mcur, int r0, int r1)
{
  const int dp = jb.dp;
  const int block_rows = IDX_SMEM_INTS / dp;
  unsigned cnt = 0;
  for(int b0 = r0; b0 < r1; b0 += block_rows){
    const int nr = min(block_rows, r1 - b0);
    const int4 *src = reinterpret_cast<const int4 *>(jb.nbr + (size_t)b0 * dp);
    int4 *dst = reinterpret_cast<int4 *>(st.idx);
    for(int i = threadIdx.x; i < (nr * dp) >> 2; i += ENGINE_THREADS) dst[i] = __ldg(src + i);
    if(level > 1 && !job_active<MODE>(jb)){
      /* saturated lanes at k-1, and at k-2 (Mcur still holds that level's
       * masks; at level 2 it holds nothing of this job) */
      for(int r = threadIdx.x; r < nr; r += ENGINE_THREADS){
        st.own[r] = __ldcg(Mprev + b0 + r);
        st.act[r] = level >= 3 ? __ldcg(Mcur + b0 + r) : 0u;
      }
    }
    if(level > 1 && job_active<MODE>(jb)){
      for(int r = threadIdx.x; r < nr; r += ENGINE_THREADS) st.own[r] = __ldcg(Mprev + b0 + r);
      __syncthreads();
      /* the neighbours' masks: eight independent gathers in flight per thread */
      const int total = nr * dp;
      for(int i0 = threadIdx.x; i0 < total; i0 += ENGINE_THREADS * 8){
        unsigned v[8];
#pragma unroll
        for(int k = 0; k < 8; k++){
          const int i = i0 + k * ENGINE_THREADS;
          const int q = i < total ? st.idx[i] : -1;
          v[k] = q >= 0 ? __ldcg(Mprev + q) : 0u;
        }
#pragma unroll
        for(int k = 0; k < 8; k++){
          const int i = i0 + k * ENGINE_THREADS;
          if(i < total) st.nmask[i] = v[k];
        }
      }
      __syncthreads();
      for(int r = threadIdx.x; r < nr; r += ENGINE_THREADS){
        unsigned a = st.own[r];
        for(int j = 0; j < dp; j++) a |= st.nmask[r * dp + j];
        st.act[r] = a;
      }
    }
    __syncthreads();
#define ODP_WC_CASE(L) case L: cnt += run_block<(1 << L), MODE>(st, dp, jb, level, X, Y, Mcur, b0, nr); break;
    switch(jb.wc_log2){
      ODP_WC_CASE(1) ODP_WC_CASE(2) ODP_WC_CASE(3) ODP_WC_CASE(4)
      ODP_WC_CASE(5) ODP_WC_CASE(6) ODP_WC_CASE(7)
      default: break;
    }
#undef ODP_WC_CASE
    __syncthreads();
    /* saturation masks of this level out; each thread copies the entries it
     * staged, so the next block's staging needs no barrier first */
    if(level > 1 && !job_active<MODE>(jb))
      for(int r = threadIdx.x; r < nr; r += ENGINE_THREADS) __stcg(Mcur + b0 + r, st.own[r]);
  }
  return cnt;
}

/* Warp 0 takes one tile from the first slot (from `cursor` on) that has one
 * left.  Each lane reads the tickets of up to four slots, so 128 slots cost
 * one L2 round trip; the candidates are then tried in slot order, one atomic
 * at a time.  A ticket is read before it is incremented, so slots without
 * tiles are never pushed past their tile count by idle CTAs.  Every lane of
 * warp 0 calls this and gets the same answer. */
__device__ __forceinline__ bool take_tile(gbx_slot *slots, int nslots, int &cursor, int &slot, int &tile)
{
  const int lane = threadIdx.x & 31;
  for(int base = 0; base < nslots; base += 128){
    unsigned long long t[4];
    int si[4];
#pragma unroll
    for(int k = 0; k < 4; k++){
      const int i = base + k * 32 + lane;
      int s = cursor + i;
      if(s >= nslots) s -= nslots;
      si[k] = s;
      t[k] = i < nslots ? vload(&slots[s].ticket) : 0ull;
    }
#pragma unroll
    for(int k = 0; k < 4; k++){
      unsigned m = __ballot_sync(0xffffffffu, (unsigned)t[k] < (unsigned)(t[k] >> 32));
      while(m){
        const int l = __ffs(m) - 1;
        const int s = __shfl_sync(0xffffffffu, si[k], l);
        unsigned long long r = 0;
        if(lane == 0) r = atomicAdd(&slots[s].ticket, 1ull);
        r = __shfl_sync(0xffffffffu, r, 0);
        if((unsigned)r < (unsigned)(r >> 32)){
          slot = s;
          tile = (int)(unsigned)r;
          cursor = s;
          return true;
        }
        m &= m - 1;
      }
    }
  }
  return false;
}

template <int MODE>
__global__ void __launch_bounds__(ENGINE_THREADS, ENGINE_MIN_BLOCKS)
engine_kernel(const gbx_job *__restrict__ jobs, int njobs, gbx_slot *slots, int nslots, gbx_ctrl *ctrl,
              gbx_graph_acc *acc, gbx_job_out *job_out, unsigned long long spin_limit_ns)
{
  __shared__ gbx_job sh_job;
  __shared__ int sh_state, sh_slot, sh_tile, sh_level;
  __shared__ unsigned long long *sh_buf0, *sh_buf1;
  __shared__ unsigned *sh_mask0, *sh_mask1;
  __shared__ __align__(16) gbx_slot sh_head;        /* head of the slot taken */
  __shared__ unsigned sh_warp[ENGINE_WARPS];
  /* Staging area in dynamic shared memory: the launch gives the whole Stage
   * when some job tracks changes, else only its index block. */
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  Stage &sh_stage = *reinterpret_cast<Stage *>(dyn_smem);

  int cursor = blockIdx.x % nslots;
  unsigned long long idle_since = 0;
  if(blockIdx.x == 0 && threadIdx.x == 0) ctrl->t_start = globaltimer();

  for(;;){
    if(threadIdx.x < 32){
      int slot = -1, tile = 0;
      const bool got = take_tile(slots, nslots, cursor, slot, tile);
      if(got){
        /* acquire the level's inputs, then read the slot's head (its level,
         * buffers and job descriptor) with one 16-byte load per lane */
        __threadfence();
        const int lane = threadIdx.x;
        if(lane < GBX_SLOT_HEAD_BYTES / 16)
          reinterpret_cast<uint4 *>(&sh_head)[lane] = __ldcg(reinterpret_cast<const uint4 *>(slots + slot) + lane);
        __syncwarp();
      }
      if(threadIdx.x == 0){
        int state = got ? 1 : 0;
        if(state == 1){
          sh_slot = slot;
          sh_tile = tile;
          sh_level = sh_head.level;
          sh_job = sh_head.desc;
          sh_buf0 = sh_head.buf0;
          sh_buf1 = sh_head.buf1;
          sh_mask0 = sh_head.mask0;
          sh_mask1 = sh_head.mask1;
          idle_since = 0;
        }
        else{
          if(vload(&ctrl->retired) >= (unsigned)nslots || (vload(&ctrl->error) & GBX_ERR_TIMEOUT)){
            state = 2;
          }
          else{
            unsigned long long now = globaltimer();
            if(idle_since == 0) idle_since = now;
            if(now - idle_since > spin_limit_ns){
              atomicOr(&ctrl->error, GBX_ERR_TIMEOUT);
              state = 2;
            }
            else __nanosleep(256);
          }
        }
        sh_state = state;
      }
    }
    __syncthreads();
    const int state = sh_state;
    if(state == 2) return;
    if(state == 0){ __syncthreads(); continue; }

    const gbx_job jb = sh_job;
    gbx_slot *sl = &slots[sh_slot];
    unsigned long long *buf0 = sh_buf0, *buf1 = sh_buf1;
    unsigned *mask0 = sh_mask0, *mask1 = sh_mask1;
    int level = sh_level, tile = sh_tile;
    __syncthreads();

    for(;;){
      /* level k writes buffer k&1 and reads buffer (k-1)&1 */
      const unsigned long long *X = (level & 1) ? buf0 : buf1;
      unsigned long long *Y = (level & 1) ? buf1 : buf0;
      const unsigned *Mprev = (level & 1) ? mask0 : mask1;
      unsigned *Mcur = (level & 1) ? mask1 : mask0;
      const int r0 = tile * jb.tile_rows;
      const int r1 = min(r0 + jb.tile_rows, jb.n);
      /* Thread 0 asks for the slot's next tile now; the answer is read after
       * the rows, so its round trip overlaps them.  While this CTA holds a
       * tile of the level the level cannot close, so a tile obtained here
       * belongs to the same level and needs no new set-up. */
      unsigned long long pre = 0;
      if(threadIdx.x == 0 && jb.ntiles > 1) pre = atomicAdd(&sl->ticket, 1ull);
      unsigned cnt = run_rows<MODE>(sh_stage, jb, level, X, Y, Mprev, Mcur, r0, r1);
      cnt = __reduce_add_sync(0xffffffffu, cnt);
      if((threadIdx.x & 31) == 0) sh_warp[threadIdx.x >> 5] = cnt;
      __syncthreads();
      if(threadIdx.x == 0){
        unsigned long long c_tile = 0;
        for(int w = 0; w < ENGINE_WARPS; w++) c_tile += sh_warp[w];
        atomicAdd(&sl->count, c_tile);
        atomicAdd(&ctrl->tiles, 1ull);
        /* Releases the CTA's row writes (ordered before this thread by the
         * barrier) and the ticket request before the done count. */
        __threadfence();
        unsigned old = atomicAdd(&sl->done, 1u);
        int next = 0;
        if(jb.ntiles > 1 && (unsigned)pre < (unsigned)(pre >> 32)){
          next = 1;                                    /* same slot, same level */
          sh_tile = (int)(unsigned)pre;
          sh_level = level;
        }
        else if(old + 1 == (unsigned)jb.ntiles){      /* this CTA closes the level */
          __threadfence();
          /* level 1 and the full-gather pass count bits set; the pass with
           * change tracking counts bits added */
          const bool delta = level > 1 && job_active<MODE>(jb);
          const unsigned long long c = (delta ? vload(&sl->prev) : 0ull) + vload(&sl->count);
          const unsigned long long full = (unsigned long long)jb.n * (unsigned long long)jb.nsrc;
          const bool complete = (c == full);
          const bool stalled = !complete && (c == vload(&sl->prev) || level >= jb.n);
          if(!complete && !stalled){
            sl->sum += (long long)(full - c) * jb.sym;
            sl->prev = c;
            sl->count = 0;
            sl->done = 0;
            sl->level = level + 1;
            if(jb.ntiles == 1){ next = 1; sh_level = level + 1; sh_tile = 0; }
            else{
              __threadfence();
              atomicExch(&sl->ticket, (unsigned long long)jb.ntiles << 32);
            }
          }
          else{
            gbx_graph_acc *ga = &acc[jb.graph];
            job_out[sl->job].level = stalled ? -level : level;
            job_out[sl->job].t_done = globaltimer();
            atomicAdd(&ga->sum, (unsigned long long)sl->sum);
            atomicMax(&ga->levels, level);
            if(stalled) atomicOr(&ga->flags, 1);
            unsigned j = atomicAdd(&ctrl->next_job, 1u);
            if(j < (unsigned)njobs){
              const gbx_job nj = jobs[j];
              job_out[j].t_loaded = globaltimer();
              sl->job = (int)j;
              sl->desc = nj;
              sl->level = 1;
              sl->count = 0;
              sl->done = 0;
              sl->prev = (unsigned long long)nj.nsrc;
              sl->sum = ((long long)nj.n * nj.nsrc - nj.nsrc) * nj.sym;
              __threadfence();
              atomicExch(&sl->ticket, (unsigned long long)nj.ntiles << 32);
            }
            else{
              atomicExch(&sl->ticket, 0ull);
              __threadfence();
              atomicAdd(&ctrl->retired, 1u);
            }
          }
        }
        sh_state = next;
      }
      __syncthreads();
      const int more = sh_state;
      level = sh_level;
      tile = sh_tile;
      __syncthreads();
      if(!more) break;
    }
  }
}

/* ---------------------------------------------------------------------- */
/* Small graphs: one CTA per job, its neighbour table and both bitset        */
/* buffers in shared memory, every level in the CTA.  The kernel reads the  */
/* caller's compact adjacency from host memory itself and writes its        */
/* outcome to pinned host memory, so a call is this one launch.             */
/* ---------------------------------------------------------------------- */

#define SMALL_THREADS 512        /* most threads per CTA (launches use fewer when the rows are few) */
#define SMALL_LOADS 8            /* host loads in flight per thread while the table is built */
#define SMALL_CLUSTER_MAX GBX_SMALL_CLUSTER_MAX   /* CTAs sharing one job (portable cluster size) */

struct SmallOutcome {
  long long sum;
  int level;
  int stalled;
};

/* Per-CTA bookkeeping of the small kernel (static shared memory). */
struct SmallShared {
  gbx_expand_desc desc;
  unsigned long long total[3];                       /* bits of level k in total[k % 3], from every CTA */
  unsigned bad[SMALL_CLUSTER_MAX];                   /* rank 0: every CTA's error flag */
};

/* Distributed shared memory: the address of a CTA-local shared address in
 * CTA `rank` of the cluster, and a 16-byte load from such an address. */
__device__ __forceinline__ unsigned dsmem_map(unsigned local, unsigned rank)
{
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
  return r;
}

__device__ __forceinline__ uint4 dsmem_ld16(unsigned addr)
{
  uint4 v;
  asm volatile("ld.shared::cluster.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(addr) : "memory");
  return v;
}

/* Row-table entries of the partitioned small kernel: the owning CTA in the
 * top bits, the row within the owner's range below. */
#define SMALL_OWNER_SHIFT 24
#define SMALL_LOCAL_MASK ((1 << SMALL_OWNER_SHIFT) - 1)

/* One job (chunk of sources) of a graph whose level fits in shared memory,
 * run by the C CTAs of one thread-block cluster; CTA q computes rows
 * [r0, r1) of each level.  Two layouts:
 *  - replicated (PART false): every CTA holds both bitset buffers whole,
 *    gathers from its own copy of the previous level and stores each row it
 *    computes into the new level's buffer of every CTA of the cluster;
 *  - partitioned (PART true): every CTA holds only its own rows of both
 *    buffers and gathers each neighbour row from the CTA that owns it
 *    (row-table entries name the owner and the row within its range), so a
 *    graph C times larger fits.  Every gather goes through the cluster's
 *    shared-memory window, own rows included: on GB300 a separate local path
 *    (a branch, or a generic address) measured no faster.
 * The same recurrence and bookkeeping as the engine: level 1 from the
 * neighbour lists, then P_k[v] = P_{k-1}[v] | OR_j P_{k-1}[nbr[v][j]], the
 * bits set per level counted, the job complete when all n * nsrc bits are
 * set and stalled when a level adds none (or the level reaches n).  Each warp
 * adds its count of a level into the level's total in every CTA (remote
 * atomics) and one cluster barrier per level orders the rows and the counts;
 * each CTA then reads the same total and takes the same decision.  The
 * totals rotate over three slots: the slot of level k + 1 is cleared during
 * level k, after the barrier that ended every read of it (level k - 2) and
 * before the barrier after which level k + 1 adds into it.  A CTA reads or
 * writes another's shared memory only between two barriers that both pass,
 * so none exits while another may still access it.  Thread 0 of each CTA
 * returns the job's outcome. */
template <int WC, bool SP, bool PART>
__device__ void small_job(const gbx_job &jb, const int *idx, uint4 *b0, uint4 *b1, int r0, int r1, int R,
                          SmallShared &sh, SmallOutcome &out)
{
  typedef RowShape<WC> S;
  constexpr int NB = S::V >= 8 ? 1 : 8 / S::V;
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks();
  const int n = jb.n, dp = jb.dp, d = jb.d, nsrc = jb.nsrc, src0 = jb.src0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int sub = lane / S::G, gl = lane % S::G;
  const int nrows = r1 - r0;

  const unsigned long long full = (unsigned long long)n * (unsigned long long)nsrc;
  unsigned long long prev = (unsigned long long)nsrc;
  long long sum = ((long long)n * nsrc - nsrc) * jb.sym;
  for(int level = 1;; level++){
    const uint4 *X = (level & 1) ? b0 : b1;
    uint4 *Y = (level & 1) ? b1 : b0;
    const unsigned xs = (unsigned)__cvta_generic_to_shared(X) + 16u * (unsigned)gl;
    unsigned cnt = 0;
    for(int lr = warp * S::RPW + sub; lr < nrows; lr += nwarps * S::RPW){
      const int r = r0 + lr;
      const int own = PART ? lr : r;                 /* the row's place in this CTA's buffers */
      uint4 a[S::V];
      const int *ip = idx + lr * dp;
      if(level == 1){
#pragma unroll
        for(int k = 0; k < S::V; k++) a[k] = make_uint4(0u, 0u, 0u, 0u);
        mark_source<S>(a, source_of<SP>(jb.srcpos, r) - src0, nsrc, gl);
        for(int j = 0; j < dp; j++){
          int u = ip[j];
          if(PART) u = (u >> SMALL_OWNER_SHIFT) * R + (u & SMALL_LOCAL_MASK);
          mark_source<S>(a, source_of<SP>(jb.srcpos, u) - src0, nsrc, gl);
        }
      }
      else{
#pragma unroll
        for(int k = 0; k < S::V; k++) a[k] = X[(size_t)own * S::VPR + gl + k * S::G];
        for(int j = 0; j < d; j += NB){
          uint4 t[NB][S::V];
#pragma unroll
          for(int i = 0; i < NB; i++){
            const bool ok = j + i < d;
            const int u = ip[ok ? j + i : j];
            if(PART){
              /* a generic address: this CTA's own shared window for its own
               * rows, the owner's window in the cluster for the others' */
              const unsigned base = dsmem_map(xs + 16u * (unsigned)((u & SMALL_LOCAL_MASK) * S::VPR),
                                              (unsigned)(u >> SMALL_OWNER_SHIFT));
#pragma unroll
              for(int k = 0; k < S::V; k++)
                t[i][k] = ok ? dsmem_ld16(base + 16u * (unsigned)(k * S::G)) : make_uint4(0u, 0u, 0u, 0u);
            }
            else{
              const uint4 *nr = X + (size_t)u * S::VPR + gl;
#pragma unroll
              for(int k = 0; k < S::V; k++) t[i][k] = ok ? nr[k * S::G] : make_uint4(0u, 0u, 0u, 0u);
            }
          }
#pragma unroll
          for(int i = 0; i < NB; i++)
#pragma unroll
            for(int k = 0; k < S::V; k++) or_into(a[k], t[i][k]);
        }
      }
      uint4 *yr = Y + (size_t)own * S::VPR + gl;
#pragma unroll
      for(int k = 0; k < S::V; k++){
        if(PART) yr[k * S::G] = a[k];
        else
          for(int q = 0; q < C; q++) *cl.map_shared_rank(yr + k * S::G, (unsigned)q) = a[k];
        cnt += popc4(a[k]);
      }
    }
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    unsigned long long *tot = &sh.total[level % 3];
    if(lane == 0 && cnt)
      for(int q = 0; q < C; q++) atomicAdd(cl.map_shared_rank(tot, (unsigned)q), (unsigned long long)cnt);
    if(threadIdx.x == 0) sh.total[(level + 1) % 3] = 0;
    cl.sync();
    const unsigned long long c = *tot;
    const bool complete = c == full;
    const bool stalled = !complete && (c == prev || level >= n);
    if(complete || stalled){
      out.sum = sum;
      out.level = level;
      out.stalled = stalled;
      break;
    }
    sum += (long long)(full - c) * jb.sym;
    prev = c;
  }
}

/* One cluster of C CTAs per job (blockIdx.x / C).  The job's graph
 * descriptor and the caller's compact adjacency are read from host memory
 * (pinned, or pageable where the device reads it through the host page
 * tables); each CTA reads 1/C of the adjacency, eight independent host loads
 * in flight per thread, expands it with the rules of expand_kernel and
 * stores each entry into the row table of the CTA that owns the row (rows
 * are split into C equal ranges; with `part` set the entries name the owner
 * of each neighbour row and the bitset buffers hold only the CTA's own rows).
 * Rank 0 writes the job's record (level,
 * error bits, sum, timestamps) to pinned host memory.  With `descs` NULL
 * every job belongs to one graph, whose descriptor is the parameter `desc0`
 * (a single-graph call then reads no descriptor from host memory). */
__global__ void __launch_bounds__(SMALL_THREADS, 1)
small_kernel(const gbx_job *__restrict__ jobs, const gbx_expand_desc *descs, gbx_small_rec *rec,
             const gbx_expand_desc desc0, const int part)
{
  extern __shared__ __align__(16) unsigned char small_smem[];
  __shared__ SmallShared sh;
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks(), rank = (int)cl.block_rank();
  const int job = blockIdx.x / C;
  const gbx_job jb = jobs[job];
  unsigned long long t_loaded = 0;
  if(threadIdx.x == 0){
    t_loaded = globaltimer();
    sh.desc = descs ? descs[jb.graph] : desc0;
    sh.total[0] = sh.total[1] = sh.total[2] = 0;
  }
  /* every CTA of the cluster is running (its shared memory may be written)
   * and the descriptor is visible to the whole CTA */
  cl.sync();
  const gbx_expand_desc &e = sh.desc;
  const int n = jb.n, dp = jb.dp;
  const int R = (n + C - 1) / C;
  const int r0 = min(n, rank * R), r1 = min(n, r0 + R);
  const size_t vecs = (size_t)(part ? R : n) << (jb.wc_log2 - 1);  /* uint4 per bitset buffer */
  uint4 *b0 = reinterpret_cast<uint4 *>(small_smem);
  uint4 *b1 = b0 + vecs;
  int *idx = reinterpret_cast<int *>(b1 + vecs);                   /* rows [r0, r1) */

  bool bad = false;
  const int total = n * dp;
  const int per = (total + C - 1) / C;
  const int e0 = min(total, rank * per), e1 = min(total, e0 + per);
  for(int t0 = e0 + (int)threadIdx.x; t0 < e1; t0 += (int)blockDim.x * SMALL_LOADS){
    int val[SMALL_LOADS], back[SMALL_LOADS];
#pragma unroll
    for(int k = 0; k < SMALL_LOADS; k++){
      const int t = t0 + k * (int)blockDim.x;
      const int v = t / dp, j = t - v * dp;
      back[k] = 0;
      val[k] = (t < e1 && j < e.d) ? e.adj[entry_source(e, v, j, back[k])] : 0;
    }
#pragma unroll
    for(int k = 0; k < SMALL_LOADS; k++){
      const int t = t0 + k * (int)blockDim.x;
      if(t < e1){
        const int v = t / dp, j = t - v * dp;
        int deg = e.ndeg ? e.ndeg[v] : e.d;
        if(deg < 0 || deg > e.d){ bad = true; deg = deg < 0 ? 0 : e.d; }
        const int row = e.grid_s ? e.itable[v] : v;
        int value = expand_value(e, val[k], back[k], j, deg, row, bad);
        if(part){
          const int vo = value / R;
          value = (vo << SMALL_OWNER_SHIFT) | (value - vo * R);
        }
        if((unsigned)row < (unsigned)n){
          const int owner = row / R;
          *cl.map_shared_rank(idx + (row - owner * R) * dp + j, (unsigned)owner) = value;
        }
        else bad = true;
      }
    }
  }
  const unsigned bad_cta = __syncthreads_or(bad);
  if(threadIdx.x == 0) *cl.map_shared_rank(&sh.bad[rank], 0u) = bad_cta;
  cl.sync();                                   /* every row table complete */

  SmallOutcome o = {0, 0, 0};
#define ODP_SMALL_CASE(L) case L: \
    if(part){ \
      if(jb.srcpos) small_job<(1 << L), true, true>(jb, idx, b0, b1, r0, r1, R, sh, o); \
      else small_job<(1 << L), false, true>(jb, idx, b0, b1, r0, r1, R, sh, o); \
    } \
    else{ \
      if(jb.srcpos) small_job<(1 << L), true, false>(jb, idx, b0, b1, r0, r1, R, sh, o); \
      else small_job<(1 << L), false, false>(jb, idx, b0, b1, r0, r1, R, sh, o); \
    } \
    break;
  switch(jb.wc_log2){
    ODP_SMALL_CASE(1) ODP_SMALL_CASE(2) ODP_SMALL_CASE(3) ODP_SMALL_CASE(4)
    default: break;
  }
#undef ODP_SMALL_CASE
  if(rank == 0 && threadIdx.x == 0){
    unsigned b = 0;
    for(int q = 0; q < C; q++) b |= sh.bad[q];
    gbx_small_rec r;
    r.level = o.stalled ? -o.level : o.level;
    r.err = b ? GBX_ERR_BAD_ADJ : 0u;
    r.sum = o.sum;
    r.t_loaded = t_loaded;
    r.t_done = globaltimer();
    rec[job] = r;
  }
}

/* L2 read ceiling for the roofline: every CTA streams an L2-resident buffer
 * with the same 16-byte ld.global.cg loads the engine uses, `reps` times. */
__global__ void __launch_bounds__(256) l2_read_probe_kernel(const uint4 *__restrict__ buf, size_t vecs, int reps,
                                                             unsigned *sink)
{
  uint4 acc = make_uint4(0u, 0u, 0u, 0u);
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for(int r = 0; r < reps; r++)
    for(size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < vecs; i += stride){
      uint4 v = __ldcg(buf + i);
      acc.x ^= v.x; acc.y ^= v.y; acc.z ^= v.z; acc.w ^= v.w;
    }
  if((acc.x ^ acc.y ^ acc.z ^ acc.w) == 0x9e3779b9u) sink[0] = 1;   /* keeps the loads */
}

/* Applies (address, value) int writes: the in-place 2-opt updates of a
 * served graph's adjacency and neighbour table, in stream order before the
 * evaluation that must see them. */
__global__ void scatter_kernel(const gbx_write *__restrict__ w, int count)
{
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) *w[i].at = w[i].value;
}

int g_engine_blocks = 0, g_engine_blocks_active = 0;
int g_pageable_access = 0;

constexpr size_t STAGE_BYTES_PLAIN = offsetof(Stage, nmask);
constexpr size_t STAGE_BYTES_ACTIVE = sizeof(Stage);

}  // namespace

/* ---------------------------------------------------------------------- */
/* extern "C" layer.                                                       */
/* ---------------------------------------------------------------------- */

extern "C" {

int gbx_device_init(int *sm_count)
{
  cudaError_t e = cudaFree(0);
  if(e != cudaSuccess) return (int)e;
  int dev = 0;
  e = cudaGetDevice(&dev);
  if(e != cudaSuccess) return (int)e;
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if(e != cudaSuccess) return (int)e;
  if(sm_count) *sm_count = sms;
  {
    /* Kernels may read pageable host memory (through the host page tables,
     * as on Grace systems) only when both attributes say so. */
    int pageable = 0, host_tables = 0;
    if(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) pageable = 0;
    if(cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess)
      host_tables = 0;
    g_pageable_access = pageable == 1 && host_tables == 1;
    cudaGetLastError();
  }
  if(g_engine_blocks == 0){
    int per_sm = 0, per_sm_active = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, engine_kernel<MODE_MIXED>, ENGINE_THREADS,
                                                      STAGE_BYTES_PLAIN);
    if(e != cudaSuccess) return (int)e;
    int per_sm_a = 0, per_sm_m = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_a, engine_kernel<MODE_ACTIVE>, ENGINE_THREADS,
                                                      STAGE_BYTES_ACTIVE);
    if(e != cudaSuccess) return (int)e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_m, engine_kernel<MODE_MIXED>, ENGINE_THREADS,
                                                      STAGE_BYTES_ACTIVE);
    per_sm_active = per_sm_a < per_sm_m ? per_sm_a : per_sm_m;
    if(e != cudaSuccess) return (int)e;
    g_engine_blocks = (per_sm < 1 ? 1 : per_sm) * sms;
    g_engine_blocks_active = (per_sm_active < 1 ? 1 : per_sm_active) * sms;
  }
  return 0;
}

int gbx_engine_blocks(int active) { return active ? g_engine_blocks_active : g_engine_blocks; }

int gbx_pageable_access(void) { return g_pageable_access; }

int gbx_l2_read_probe(size_t bytes, int reps, double *gbs)
{
  void *buf = nullptr, *sink = nullptr;
  cudaEvent_t a, b;
  cudaError_t e = cudaMalloc(&buf, bytes);
  if(e != cudaSuccess) return (int)e;
  if((e = cudaMalloc(&sink, 64)) != cudaSuccess){ cudaFree(buf); return (int)e; }
  cudaMemset(buf, 0x5a, bytes);
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t vecs = bytes / 16;
  l2_read_probe_kernel<<<sms * 8, 256>>>((const uint4 *)buf, vecs, 1, (unsigned *)sink);   /* warm L2 */
  cudaEventRecord(a);
  l2_read_probe_kernel<<<sms * 8, 256>>>((const uint4 *)buf, vecs, reps, (unsigned *)sink);
  cudaEventRecord(b);
  e = cudaEventSynchronize(b);
  float ms = 0;
  if(e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  if(e == cudaSuccess) *gbs = (double)bytes * reps / (ms * 1e-3) / 1e9;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(sink);
  cudaFree(buf);
  return (int)e;
}

int gbx_malloc(void **p, size_t bytes) { return (int)cudaMalloc(p, bytes ? bytes : 256); }
int gbx_free(void *p) { return p ? (int)cudaFree(p) : 0; }
int gbx_host_alloc(void **p, size_t bytes) { return (int)cudaMallocHost(p, bytes ? bytes : 64); }
int gbx_host_free(void *p) { return p ? (int)cudaFreeHost(p) : 0; }

int gbx_stream_create(void **stream)
{
  cudaStream_t s;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  *stream = (void *)s;
  return (int)e;
}

int gbx_stream_destroy(void *stream) { return (int)cudaStreamDestroy((cudaStream_t)stream); }

int gbx_memcpy_h2d(void *dst, const void *src, size_t bytes, void *stream)
{
  return (int)cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream);
}

int gbx_memcpy_d2d(void *dst, const void *src, size_t bytes, void *stream)
{
  return (int)cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)stream);
}

int gbx_memcpy_d2h(void *dst, const void *src, size_t bytes, void *stream)
{
  return (int)cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream);
}

int gbx_memset(void *dst, int value, size_t bytes, void *stream)
{
  return (int)cudaMemsetAsync(dst, value, bytes, (cudaStream_t)stream);
}

int gbx_stream_sync(void *stream) { return (int)cudaStreamSynchronize((cudaStream_t)stream); }

const char *gbx_error_string(int err) { return cudaGetErrorString((cudaError_t)err); }

int gbx_small_prepare(void)
{
  static int configured = 0;
  if(configured) return 0;
  cudaError_t e = cudaFuncSetAttribute(small_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       GBX_SMALL_SMEM_MAX);
  if(e != cudaSuccess) return (int)e;
  configured = 1;
  return 0;
}

static cudaLaunchConfig_t small_config(int njobs, int cluster, int threads, size_t smem_bytes, cudaStream_t stream,
                                       cudaLaunchAttribute *attr)
{
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(njobs * cluster), 1, 1);
  cfg.blockDim = dim3((unsigned)threads, 1, 1);
  cfg.dynamicSmemBytes = smem_bytes;
  cfg.stream = stream;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

static int small_shape_ok(int cluster, int threads, size_t smem_bytes)
{
  return cluster >= 1 && cluster <= SMALL_CLUSTER_MAX && (cluster & (cluster - 1)) == 0 && threads >= 32 &&
         threads <= SMALL_THREADS && threads % 32 == 0 && smem_bytes <= GBX_SMALL_SMEM_MAX;
}

int gbx_small_clusters(int cluster, int threads, size_t smem_bytes, int *active)
{
  *active = 0;
  if(!small_shape_ok(cluster, threads, smem_bytes)) return (int)cudaErrorInvalidValue;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = small_config(1, cluster, threads, smem_bytes, 0, attr);
  return (int)cudaOccupancyMaxActiveClusters(active, small_kernel, &cfg);
}

int gbx_small_launch(const gbx_job *d_jobs, int njobs, const gbx_expand_desc *descs, const gbx_expand_desc *desc0,
                     gbx_small_rec *rec, size_t smem_bytes, int cluster, int threads, int part, void *stream)
{
  if(njobs <= 0) return 0;
  if(!small_shape_ok(cluster, threads, smem_bytes) || (!descs && !desc0)) return (int)cudaErrorInvalidValue;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = small_config(njobs, cluster, threads, smem_bytes, (cudaStream_t)stream, attr);
  gbx_expand_desc d0;
  if(desc0) d0 = *desc0;
  else memset(&d0, 0, sizeof(d0));
  return (int)cudaLaunchKernelEx(&cfg, small_kernel, d_jobs, descs, rec, d0, part ? 1 : 0);
}

int gbx_host_device_ptr(void *host, void **dev)
{
  return (int)cudaHostGetDevicePointer(dev, host, 0);
}

int gbx_pull(const gbx_expand_desc *h_descs, gbx_expand_desc *d_descs, int ndesc, void *d_state,
             const void *d_state_init, size_t state_bytes, void *stream)
{
  if(ndesc <= 0) return 0;
  if(state_bytes % 8) return (int)cudaErrorInvalidValue;
  pull_kernel<<<dim3(32, (unsigned)ndesc), 256, 0, (cudaStream_t)stream>>>(
      h_descs, d_descs, (unsigned long long *)d_state, (const unsigned long long *)d_state_init,
      (long long)(state_bytes / 8));
  return (int)cudaGetLastError();
}

int gbx_expand(const gbx_expand_desc *d_descs, int ndesc, long long total_vertices, int max_dp, unsigned int *d_error,
               void *stream)
{
  if(total_vertices <= 0) return 0;
  if(max_dp <= 0 || max_dp > 65535 * EXPAND_GROUP) return (int)cudaErrorInvalidValue;
  long long blocks = (total_vertices + 255) / 256;
  if(blocks > 65535LL * 8) blocks = 65535LL * 8;
  const unsigned groups = (unsigned)((max_dp + EXPAND_GROUP - 1) / EXPAND_GROUP);
  expand_kernel<<<dim3((unsigned)blocks, groups), 256, 0, (cudaStream_t)stream>>>(d_descs, ndesc, total_vertices,
                                                                                d_error);
  return (int)cudaGetLastError();
}

int gbx_engine_launch(const gbx_job *d_jobs, int njobs, gbx_slot *d_slots, int nslots, gbx_ctrl *d_ctrl,
                      gbx_graph_acc *d_acc, gbx_job_out *d_job_out, unsigned long long spin_limit_ns, int blocks,
                      int active, void *stream)
{
  if(njobs <= 0 || nslots <= 0) return 0;
  if(blocks <= 0) blocks = gbx_engine_blocks(active);
  if(blocks <= 0) blocks = 1;
  const size_t smem = active ? STAGE_BYTES_ACTIVE : STAGE_BYTES_PLAIN;
  cudaStream_t st = (cudaStream_t)stream;
  if(active == 1)
    engine_kernel<MODE_ACTIVE><<<blocks, ENGINE_THREADS, smem, st>>>(d_jobs, njobs, d_slots, nslots, d_ctrl, d_acc,
                                                                     d_job_out, spin_limit_ns);
  else
    engine_kernel<MODE_MIXED><<<blocks, ENGINE_THREADS, smem, st>>>(d_jobs, njobs, d_slots, nslots, d_ctrl, d_acc,
                                                                    d_job_out, spin_limit_ns);
  return (int)cudaGetLastError();
}

int gbx_scatter(const gbx_write *d_writes, int count, void *stream)
{
  if(count <= 0) return 0;
  int blocks = (count + 255) / 256;
  if(blocks > 1024) blocks = 1024;
  scatter_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_writes, count);
  return (int)cudaGetLastError();
}

int gbx_capture_begin(void *stream)
{
  return (int)cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal);
}

int gbx_capture_end(void *stream, void **graph_exec)
{
  cudaGraph_t g;
  cudaError_t e = cudaStreamEndCapture((cudaStream_t)stream, &g);
  if(e != cudaSuccess) return (int)e;
  cudaGraphExec_t ge;
  e = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  if(e != cudaSuccess) return (int)e;
  *graph_exec = (void *)ge;
  return 0;
}

int gbx_graph_launch(void *graph_exec, void *stream)
{
  return (int)cudaGraphLaunch((cudaGraphExec_t)graph_exec, (cudaStream_t)stream);
}

int gbx_graph_destroy(void *graph_exec)
{
  return graph_exec ? (int)cudaGraphExecDestroy((cudaGraphExec_t)graph_exec) : 0;
}

int gbx_event_create(void **ev)
{
  cudaEvent_t e;
  cudaError_t r = cudaEventCreate(&e);
  *ev = (void *)e;
  return (int)r;
}

int gbx_event_destroy(void *ev) { return (int)cudaEventDestroy((cudaEvent_t)ev); }

int gbx_event_query(void *ev)
{
  cudaError_t e = cudaEventQuery((cudaEvent_t)ev);
  if(e == cudaSuccess) return 0;
  if(e == cudaErrorNotReady){ cudaGetLastError(); return 1; }
  return (int)e;
}
int gbx_event_record(void *ev, void *stream) { return (int)cudaEventRecord((cudaEvent_t)ev, (cudaStream_t)stream); }

int gbx_event_elapsed_ms(void *start, void *stop, float *ms)
{
  cudaError_t e = cudaEventSynchronize((cudaEvent_t)stop);
  if(e != cudaSuccess) return (int)e;
  return (int)cudaEventElapsedTime(ms, (cudaEvent_t)start, (cudaEvent_t)stop);
}

}  /* extern "C" */

/* ---------------------------------------------------------------------- */
/* Evaluation without any memory allocation: ODPX_Set_aspl_noalloc.        */
/*                                                                         */
/* Some callers cannot allocate device memory while they run: an annealing  */
/* loop on a latency budget, where cudaMalloc/cudaFree synchronise the      */
/* device and stall its other streams, or a process whose device memory is  */
/* already reserved by another framework's pool allocator, so an allocation */
/* could fail in the middle of a run.  This entry point runs the same two   */
/* kernels as ODP_Set_aspl (expand_kernel, engine_kernel) with all of their */
/* working memory -- the adjacency copy, the neighbour table, the engine    */
/* state and the bitset buffers -- carved out of one fixed array that is    */
/* part of the library's device image.  Every GPU context that loads the    */
/* library holds that array (ODPX_NOALLOC_SCRATCH_BYTES) until the process  */
/* exits.                                                                   */
/* ---------------------------------------------------------------------- */

#include <stdio.h>
#include <string.h>
#include <float.h>
#include <limits.h>
#include "odp_gb300.h"

#define NOALLOC_MAX_JOBS 256
#define NOALLOC_MAX_DEVICES 64

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[ODPX_NOALLOC_SCRATCH_BYTES];

struct NoallocDevice {
  int ready;
  int blocks;
  unsigned char *scratch;    /* device address of g_noalloc_scratch on this device */
};
NoallocDevice g_noalloc_dev[NOALLOC_MAX_DEVICES];

/* Once per device, with that device current: look up the array's device
 * address (the name is only a host-side stand-in) and the persistent grid
 * size.  No allocation is involved. */
int noalloc_device(NoallocDevice **out)
{
  int dev = 0;
  if(cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) return ODPX_ERR_CUDA;
  NoallocDevice *nd = &g_noalloc_dev[dev];
  if(!nd->ready){
    void *p = nullptr;
    if(cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return ODPX_ERR_CUDA;
    int sms = 0, per_sm = 0;
    if(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return ODPX_ERR_CUDA;
    if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, engine_kernel<MODE_MIXED>, ENGINE_THREADS,
                                                     STAGE_BYTES_PLAIN) != cudaSuccess)
      return ODPX_ERR_CUDA;
    nd->scratch = (unsigned char *)p;
    nd->blocks = (per_sm < 1 ? 1 : per_sm) * sms;
    nd->ready = 1;
  }
  *out = nd;
  return 0;
}

inline size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

extern "C" int ODPX_Set_aspl_noalloc(int nodes, int degree, int symmetries, const int *adjacency,
                                     int *diameter, long *sum, double *ASPL)
{
  if(nodes <= 0 || degree < 0 || degree > GBX_MAX_DEGREE || symmetries <= 0 || nodes % symmetries != 0 ||
     !adjacency || !diameter || !sum || !ASPL)
    return ODPX_ERR_INVALID;
  const int n = nodes, d = degree, s = symmetries, B = n / s, W = (B + 63) / 64;
  const int dp = ((d > 0 ? d : 1) + 3) & ~3;
  int full_l2 = 1;
  while((1 << full_l2) < W) full_l2++;

  /* Layout of the scratch array for the widest chunk (<= 64 words) that fits. */
  size_t off_adj = 0, off_nbr = 0, off_desc = 0, off_jobs = 0, off_state = 0, off_buf = 0, off_mask = 0, total = 0;
  size_t out_off = 0, acc_off = 0, levels_off = 0, state_bytes = 0;
  int wl = full_l2 < 6 ? full_l2 : 6, njobs = 0, nslots = 0, fits = 0;
  const int mask_rows = (n + 63) & ~63;          /* each mask buffer starts on a 256-byte boundary */
  for(; wl >= 1; wl--){
    njobs = (W + (1 << wl) - 1) >> wl;
    if(njobs > NOALLOC_MAX_JOBS) break;
    nslots = njobs < 2 ? njobs : 2;
    off_adj = 0;
    off_nbr = up256(off_adj + sizeof(int) * (size_t)B * d);
    off_desc = up256(off_nbr + sizeof(int) * (size_t)n * dp);
    off_jobs = up256(off_desc + sizeof(gbx_expand_desc));
    off_state = up256(off_jobs + sizeof(gbx_job) * (size_t)njobs);
    out_off = sizeof(gbx_slot) * (size_t)nslots;
    acc_off = out_off + sizeof(gbx_ctrl) + 64;
    levels_off = acc_off + 64;
    state_bytes = levels_off + sizeof(gbx_job_out) * (size_t)njobs;
    off_buf = up256(off_state + state_bytes);
    off_mask = up256(off_buf + sizeof(unsigned long long) * 2 * (size_t)nslots * ((size_t)n << wl));
    total = off_mask + sizeof(unsigned) * 2 * (size_t)nslots * (size_t)mask_rows;
    if(total <= ODPX_NOALLOC_SCRATCH_BYTES){ fits = 1; break; }
  }
  if(!fits){
    fprintf(stderr, "ODPX_Set_aspl_noalloc: a graph with %d nodes, degree %d and %d symmetries needs more than "
            "the %u bytes of fixed scratch memory\n", n, d, s, (unsigned)ODPX_NOALLOC_SCRATCH_BYTES);
    return ODPX_ERR_MEMORY;
  }

  NoallocDevice *nd = nullptr;
  int rc = noalloc_device(&nd);
  if(rc) return rc;
  unsigned char *base = nd->scratch;
  cudaStream_t st = cudaStreamPerThread;
  const int wc = 1 << wl;

  /* Host-side descriptors live on the stack. */
  gbx_expand_desc desc = {};
  desc.adj = (const int *)(base + off_adj);
  desc.ndeg = nullptr;
  desc.itable = nullptr;
  desc.nbr = (int *)(base + off_nbr);
  desc.n = n; desc.d = d; desc.dp = dp; desc.s = s;
  desc.first_vertex = 0;
  gbx_job jobs[NOALLOC_MAX_JOBS];
  const double level_bytes = (double)n * wc * 8.0 * (d + 2);
  const int vpr = wc / 2, g = vpr < 32 ? vpr : 32, rpp = 8 * (32 / g);
  int tile_rows = n;
  if(level_bytes > 96.0 * 1024.0){
    int tr = (int)(256.0 * 1024.0 / ((double)wc * 8.0 * (d + 2)));
    if(tr < rpp) tr = rpp;
    tile_rows = ((tr + rpp - 1) / rpp) * rpp;
    if(tile_rows > n) tile_rows = n;
  }
  for(int k = 0; k < njobs; k++){
    gbx_job &j = jobs[k];
    j = gbx_job();
    j.nbr = desc.nbr;
    j.n = n; j.dp = dp; j.d = d; j.wc_log2 = wl;
    j.src0 = k * wc * 64;
    j.nsrc = B - j.src0 < wc * 64 ? B - j.src0 : wc * 64;
    j.sym = s; j.graph = 0;
    j.tile_rows = tile_rows;
    j.ntiles = (n + tile_rows - 1) / tile_rows;
  }
  /* The array keeps whatever the previous call left in it: the engine state
   * is rewritten here in full; the neighbour table and the bitset buffers
   * are overwritten by the kernels before they are read. */
  /* aligned for the gbx_slot / gbx_ctrl / gbx_job_out views taken of it */
  alignas(64) unsigned char state[sizeof(gbx_slot) * 2 + sizeof(gbx_ctrl) + 64 + 64 +
                                  sizeof(gbx_job_out) * NOALLOC_MAX_JOBS];
  memset(state, 0, sizeof(state));
  gbx_slot *sl = (gbx_slot *)state;
  unsigned long long *bufs = (unsigned long long *)(base + off_buf);
  for(int k = 0; k < nslots; k++){
    sl[k].ticket = (unsigned long long)jobs[k].ntiles << 32;
    sl[k].job = k;
    sl[k].desc = jobs[k];
    sl[k].level = 1;
    sl[k].prev = (unsigned long long)jobs[k].nsrc;
    sl[k].sum = ((long long)n * jobs[k].nsrc - jobs[k].nsrc) * s;
    sl[k].buf0 = bufs + (size_t)k * 2 * ((size_t)n << wl);
    sl[k].buf1 = sl[k].buf0 + ((size_t)n << wl);
    sl[k].mask0 = (unsigned *)(base + off_mask) + (size_t)k * 2 * mask_rows;
    sl[k].mask1 = sl[k].mask0 + mask_rows;
  }
  ((gbx_ctrl *)(state + out_off))->next_job = (unsigned)nslots;

  if(cudaMemcpyAsync(base + off_adj, adjacency, sizeof(int) * (size_t)B * d, cudaMemcpyHostToDevice, st) ||
     cudaMemcpyAsync(base + off_desc, &desc, sizeof(desc), cudaMemcpyHostToDevice, st) ||
     cudaMemcpyAsync(base + off_jobs, jobs, sizeof(gbx_job) * (size_t)njobs, cudaMemcpyHostToDevice, st) ||
     cudaMemcpyAsync(base + off_state, state, state_bytes, cudaMemcpyHostToDevice, st))
    return ODPX_ERR_CUDA;
  unsigned int *d_err = (unsigned int *)(base + off_state + out_off + sizeof(gbx_ctrl));
  long long eblocks = ((long long)n + 255) / 256;
  if(eblocks > 65535LL * 8) eblocks = 65535LL * 8;
  expand_kernel<<<dim3((unsigned)eblocks, (unsigned)((desc.dp + EXPAND_GROUP - 1) / EXPAND_GROUP)), 256, 0, st>>>(
      (const gbx_expand_desc *)(base + off_desc), 1, n, d_err);
  engine_kernel<MODE_MIXED><<<nd->blocks, ENGINE_THREADS, STAGE_BYTES_PLAIN, st>>>(
      (const gbx_job *)(base + off_jobs), njobs, (gbx_slot *)(base + off_state), nslots,
      (gbx_ctrl *)(base + off_state + out_off), (gbx_graph_acc *)(base + off_state + acc_off),
      (gbx_job_out *)(base + off_state + levels_off), 60ull * 1000000000ull);
  if(cudaGetLastError() != cudaSuccess) return ODPX_ERR_CUDA;
  alignas(64) unsigned char out[sizeof(gbx_ctrl) + 64 + 64];
  if(cudaMemcpyAsync(out, base + off_state + out_off, sizeof(out), cudaMemcpyDeviceToHost, st) ||
     cudaStreamSynchronize(st))
    return ODPX_ERR_CUDA;
  const unsigned int err = ((const gbx_ctrl *)out)->error | *(const unsigned int *)(out + sizeof(gbx_ctrl));
  if(err & GBX_ERR_TIMEOUT) return ODPX_ERR_TIMEOUT;
  if(err & GBX_ERR_BAD_ADJ) return ODPX_ERR_ADJACENCY;
  const gbx_graph_acc *acc = (const gbx_graph_acc *)(out + sizeof(gbx_ctrl) + 64);
  if(acc->flags & 1){
    *diameter = INT_MAX;
    *sum = LONG_MAX;
    *ASPL = DBL_MAX;
    return 0;
  }
  long total_sum = (long)acc->sum;
  *diameter = acc->levels;
  *ASPL = total_sum / (((double)n - 1) * n);
  *sum = (long)(total_sum / 2.0);
  return 0;
}

/*
 * ref_bench.c -- times the reference ODP library through its own public API
 * (include/odp.h of the reference) on a list of graphs.  It is linked against
 * the reference's libodp_threads.a (CPU, OpenMP) or against its libodp_cuda.a
 * rebuilt for sm_103a (-DREF_CUDA), both compiled from the reference's
 * unmodified sources by baseline/Makefile.  Nothing of libodp_gb300 is linked.
 *
 * The graph list (SHAPES) is a text file, one graph per line:
 *     general N D S SEED
 *     grid    W H D LEN S SEED
 * and ADJ is the concatenation, in that order, of each graph's adjacency as
 * ODP_Set_aspl takes it: int32[n/s][d], row-major, little-endian.
 *
 * Commands:
 *   gen SHAPES OUT WORKERS
 *       ODP_Srand(SEED) then ODP_Generate_random_general_s / _grid_s and
 *       ODP_Conv_edge2adjacency_general_s / _grid_s for every graph, in
 *       WORKERS forked processes (the reference's rand() state is global);
 *       writes ADJ to OUT.
 *   cpu SHAPES ADJ STEPS WARMUP SETS        (threads build)
 *       For every step, every graph in a forked child of its own: Init,
 *       SETS x ODP_Set_aspl, Finalize.  A fresh process per graph is what the
 *       reference's static state needs: its Finalize leaves stale pointers and
 *       flags behind (aspl.c:290-297), so one process cannot Init graphs of
 *       mixed kinds in turn.  The OpenMP pool is started before the first Set.
 *       Only the last Set is timed (CLOCK_MONOTONIC), as ODP_PROFILE times
 *       ODP_Set_aspl alone (aspl.c:319-339); the first Set's time is reported
 *       beside it.
 *   gpu SHAPES ADJ REPS                      (CUDA build)
 *       One process: per graph Init, one untimed Set, REPS timed Sets,
 *       Finalize.  ODP_Set_aspl is synchronous (aspl_cuda.cu:242-263).  The
 *       reference's CUDA Finalize leaves _itable/_itable_dev and
 *       _enable_grid_s set (aspl_cuda.cu:226-240), so a general graph after a
 *       grid-symmetric one would read freed device memory: the list must hold
 *       every grid graph with symmetries > 1 after all other graphs, and
 *       graphs with num_degrees are not taken.  The driver refuses any other
 *       order.
 *
 * Output lines (stdout):
 *   step K WARM_NS FIRST_NS WALL_NS          (cpu, one per timed step)
 *   graph I DIAMETER SUM ASPL_HEX NS NS2     (cpu: last step; NS = last Set,
 *                                            NS2 = first Set; gpu: NS = mean,
 *                                            NS2 = minimum over REPS)
 */
#define _GNU_SOURCE
#include <errno.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/types.h>
#include <sys/wait.h>
#include <time.h>
#include <unistd.h>
#include <fcntl.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "odp.h"

typedef struct {
  int grid, n, w, h, d, len, s;
  unsigned seed;
  size_t off, ints;          /* position and length (int32s) of the adjacency in ADJ */
} shape_t;

typedef struct {
  int diameter;
  long sum;
  double aspl;
  long long ns_last, ns_first;
  int ok;
} result_t;

static long long now_ns(void)
{
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (long long)t.tv_sec * 1000000000LL + t.tv_nsec;
}

static shape_t *read_shapes(const char *path, int *count)
{
  FILE *f = fopen(path, "r");
  if(!f){ fprintf(stderr, "ref_bench: cannot open %s\n", path); exit(2); }
  int cap = 64, k = 0;
  shape_t *sh = malloc(sizeof(shape_t) * cap);
  char kind[16];
  size_t off = 0;
  while(fscanf(f, "%15s", kind) == 1){
    if(k == cap){ cap *= 2; sh = realloc(sh, sizeof(shape_t) * cap); }
    shape_t *g = &sh[k];
    memset(g, 0, sizeof(*g));
    if(strcmp(kind, "general") == 0){
      if(fscanf(f, "%d %d %d %u", &g->n, &g->d, &g->s, &g->seed) != 4) break;
    }
    else if(strcmp(kind, "grid") == 0){
      g->grid = 1;
      if(fscanf(f, "%d %d %d %d %d %u", &g->w, &g->h, &g->d, &g->len, &g->s, &g->seed) != 6) break;
      g->n = g->w * g->h;
    }
    else{ fprintf(stderr, "ref_bench: unknown graph kind %s\n", kind); exit(2); }
    if(g->n <= 0 || g->d <= 0 || g->s <= 0 || g->n % g->s != 0){ fprintf(stderr, "ref_bench: bad shape %d\n", k); exit(2); }
    g->off = off;
    g->ints = (size_t)(g->n / g->s) * g->d;
    off += g->ints;
    k++;
  }
  fclose(f);
  *count = k;
  return sh;
}

static int *read_adj(const char *path, const shape_t *sh, int count)
{
  size_t ints = count ? sh[count - 1].off + sh[count - 1].ints : 0;
  int *a = malloc(ints * sizeof(int) + 16);
  FILE *f = fopen(path, "rb");
  if(!f || fread(a, sizeof(int), ints, f) != ints){ fprintf(stderr, "ref_bench: short adjacency file %s\n", path); exit(2); }
  fclose(f);
  return a;
}

static void init_graph(const shape_t *g)
{
  if(g->grid){
    if(g->s == 1) ODP_Init_aspl_grid(g->w, g->h, g->d, NULL);
    else          ODP_Init_aspl_grid_s(g->w, g->h, g->d, NULL, g->s);
  }
  else{
    if(g->s == 1) ODP_Init_aspl_general(g->n, g->d, NULL);
    else          ODP_Init_aspl_general_s(g->n, g->d, NULL, g->s);
  }
}

/* ---- gen ---- */
static int cmd_gen(const char *shapes, const char *out, int workers)
{
  int count;
  shape_t *sh = read_shapes(shapes, &count);
  size_t ints = count ? sh[count - 1].off + sh[count - 1].ints : 0;
  int fd = open(out, O_RDWR | O_CREAT | O_TRUNC, 0644);
  if(fd < 0 || ftruncate(fd, (off_t)(ints * sizeof(int))) != 0){ fprintf(stderr, "ref_bench: cannot create %s\n", out); return 2; }
  int *next = mmap(NULL, sizeof(int), PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS, -1, 0);
  *next = 0;
  if(workers < 1) workers = 1;
  for(int w = 0; w < workers; w++){
    pid_t p = fork();
    if(p < 0){ perror("fork"); return 2; }
    if(p == 0){
      for(;;){
        int i = __atomic_fetch_add(next, 1, __ATOMIC_SEQ_CST);
        if(i >= count) break;
        const shape_t *g = &sh[i];
        int lines = (g->n * g->d) / 2;
        int (*edge)[2] = malloc(sizeof(int) * 2 * (size_t)lines);
        int *adj = malloc(sizeof(int) * g->ints);
        ODP_Srand(g->seed);
        if(g->grid){
          ODP_Generate_random_grid_s(g->w, g->h, g->d, g->len, g->s, edge);
          ODP_Conv_edge2adjacency_grid_s(g->w, g->h, lines, g->d, edge, g->s, (int (*)[g->d])adj);
        }
        else{
          ODP_Generate_random_general_s(g->n, g->d, g->s, edge);
          ODP_Conv_edge2adjacency_general_s(g->n, lines, g->d, edge, g->s, adj);
        }
        size_t bytes = g->ints * sizeof(int), done = 0;
        while(done < bytes){
          ssize_t r = pwrite(fd, (char *)adj + done, bytes - done, (off_t)(g->off * sizeof(int) + done));
          if(r <= 0){ perror("pwrite"); _exit(3); }
          done += (size_t)r;
        }
        free(edge);
        free(adj);
      }
      _exit(0);
    }
  }
  int bad = 0, st;
  while(wait(&st) > 0)
    if(!WIFEXITED(st) || WEXITSTATUS(st) != 0) bad = 1;
  close(fd);
  return bad ? 3 : 0;
}

/* ---- cpu ---- */
static int run_child(const shape_t *g, const int *adj, int sets, result_t *res)
{
  int fds[2];
  if(pipe(fds) != 0){ perror("pipe"); return -1; }
  pid_t p = fork();
  if(p < 0){ perror("fork"); return -1; }
  if(p == 0){
    close(fds[0]);
    result_t r;
    memset(&r, 0, sizeof(r));
    init_graph(g);
#ifdef _OPENMP
#pragma omp parallel
    { if(omp_get_thread_num() < 0) r.ok = -1; }
#endif
    for(int k = 0; k < sets; k++){
      long long t0 = now_ns();
      ODP_Set_aspl((void *)(adj + g->off), &r.diameter, &r.sum, &r.aspl);
      long long t1 = now_ns();
      if(k == 0) r.ns_first = t1 - t0;
      r.ns_last = t1 - t0;
    }
    ODP_Finalize_aspl();
    r.ok = 1;
    if(write(fds[1], &r, sizeof(r)) != (ssize_t)sizeof(r)) _exit(3);
    _exit(0);
  }
  close(fds[1]);
  ssize_t got = 0;
  while(got < (ssize_t)sizeof(*res)){
    ssize_t r = read(fds[0], (char *)res + got, sizeof(*res) - (size_t)got);
    if(r <= 0) break;
    got += r;
  }
  close(fds[0]);
  int st = 0;
  waitpid(p, &st, 0);
  if(got != (ssize_t)sizeof(*res) || !WIFEXITED(st) || WEXITSTATUS(st) != 0 || res->ok != 1) return -1;
  return 0;
}

static int cmd_cpu(const char *shapes, const char *adjpath, int steps, int warmup, int sets)
{
  int count;
  shape_t *sh = read_shapes(shapes, &count);
  int *adj = read_adj(adjpath, sh, count);
  result_t *res = calloc((size_t)count + 1, sizeof(result_t));
  if(sets < 1) sets = 1;
  for(int step = -warmup; step < steps; step++){
    long long warm = 0, first = 0, t0 = now_ns();
    for(int i = 0; i < count; i++){
      if(run_child(&sh[i], adj, sets, &res[i]) != 0){ fprintf(stderr, "ref_bench: graph %d failed\n", i); return 3; }
      warm += res[i].ns_last;
      first += res[i].ns_first;
    }
    if(step >= 0) printf("step %d %lld %lld %lld\n", step, warm, first, now_ns() - t0);
    fflush(stdout);
  }
  for(int i = 0; i < count; i++)
    printf("graph %d %d %ld %a %lld %lld\n", i, res[i].diameter, res[i].sum, res[i].aspl, res[i].ns_last,
           res[i].ns_first);
  return 0;
}

/* ---- gpu ---- */
static int cmd_gpu(const char *shapes, const char *adjpath, int reps)
{
  int count;
  shape_t *sh = read_shapes(shapes, &count);
  int seen_grid_s = 0;
  for(int i = 0; i < count; i++){
    int grid_s = sh[i].grid && sh[i].s > 1;
    if(seen_grid_s && !grid_s){
      fprintf(stderr, "ref_bench: graph %d comes after a grid graph with symmetries > 1; the reference's CUDA "
                      "Finalize leaves that graph's itable in use, so this order is refused\n", i);
      return 2;
    }
    seen_grid_s |= grid_s;
  }
  int *adj = read_adj(adjpath, sh, count);
  if(reps < 1) reps = 1;
  for(int i = 0; i < count; i++){
    const shape_t *g = &sh[i];
    result_t r;
    memset(&r, 0, sizeof(r));
    init_graph(g);
    ODP_Set_aspl((void *)(adj + g->off), &r.diameter, &r.sum, &r.aspl);
    long long total = 0, best = -1;
    for(int k = 0; k < reps; k++){
      long long t0 = now_ns();
      ODP_Set_aspl((void *)(adj + g->off), &r.diameter, &r.sum, &r.aspl);
      long long dt = now_ns() - t0;
      total += dt;
      if(best < 0 || dt < best) best = dt;
    }
    ODP_Finalize_aspl();
    printf("graph %d %d %ld %a %lld %lld\n", i, r.diameter, r.sum, r.aspl, total / reps, best);
    fflush(stdout);
  }
  return 0;
}

int main(int argc, char **argv)
{
  if(argc >= 5 && strcmp(argv[1], "gen") == 0) return cmd_gen(argv[2], argv[3], atoi(argv[4]));
#ifndef REF_CUDA
  if(argc >= 7 && strcmp(argv[1], "cpu") == 0)
    return cmd_cpu(argv[2], argv[3], atoi(argv[4]), atoi(argv[5]), atoi(argv[6]));
#else
  if(argc >= 5 && strcmp(argv[1], "gpu") == 0) return cmd_gpu(argv[2], argv[3], atoi(argv[4]));
#endif
  fprintf(stderr, "usage: ref_bench gen SHAPES OUT WORKERS | cpu SHAPES ADJ STEPS WARMUP SETS | gpu SHAPES ADJ REPS\n");
  return 2;
}

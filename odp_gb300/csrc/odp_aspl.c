/*
 * odp_aspl.c -- the drop-in ASPL entry points of odp.h on one GB300:
 * ODP_Init_aspl_general / _general_s / _grid / _grid_s, ODP_Set_aspl,
 * ODP_Finalize_aspl.  They replace the reference's CUDA driver
 * (aspl_cuda.cu:128-263) with the same arguments, results, environment
 * variables (ODP_ASPL, ODP_PROFILE) and error behaviour (message on stderr,
 * exit(1)).
 *
 * Differences that do not change results:
 *  - the column chunking is chosen for L2 residency whatever ODP_ASPL says;
 *    the kind only feeds the memory estimate and the profile report (the
 *    reference's kinds give identical results, as its own tests show);
 *  - CUDA errors are checked and reported (the reference ignores them);
 *  - re-initialising without ODP_Finalize_aspl releases the previous state,
 *    and Finalize resets every field, so Init/Finalize cycles of any variant
 *    may follow each other (the reference double-frees, aspl.c:290-297);
 *  - an adjacency entry outside [0, nodes) is reported instead of read out
 *    of bounds.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdarg.h>
#include <time.h>
#include <unistd.h>
#include <sys/time.h>
#include "odp_plan.h"
#include "odp_gb300.h"

#define KIND_MATRIX 1
#define KIND_SAVING 2
#define MEM_THRESHOLD_MB 2048.0      /* parameter.h:4 */
#define REF_BLOCKS 448               /* the reference's result buffer, counted in its estimate */
#define REF_CHUNK 64                 /* GPU_CHUNK, parameter.h:13 */

static struct {
  int initialized;
  int nodes, degree, symmetries, kind;
  double mem_usage, elapsed;
  unsigned int times;
  int profile;
  odp_plan *plan;
} S;

static void fail(const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vfprintf(stderr, fmt, ap);
  va_end(ap);
  exit(1);
}

static double now_seconds(void)       /* ODP_Get_time, utils.c:135-140 */
{
  struct timeval t;
  gettimeofday(&t, NULL);
  return t.tv_sec + 1.0e-6 * t.tv_usec;
}

/* ODP_Get_mem_usage for the GPU (utils.c:1206-1236, is_cpu = false, one process). */
static double mem_usage_mb(int kind, int nodes, int degree, int symmetries, const int *num_degrees, int grid_s)
{
  double ab;
  if(kind == KIND_MATRIX) ab = nodes * ((double)nodes / (4 * symmetries));
  else                    ab = (double)16 * nodes * REF_CHUNK;
  if(grid_s) ab += sizeof(int) * (double)nodes;
  double res = (double)sizeof(unsigned long long) * REF_BLOCKS;
  double adj = (double)sizeof(int) * (nodes / symmetries) * degree;
  double deg = num_degrees ? (double)sizeof(int) * nodes : 0;
  return (ab + res + adj + deg) / (1024.0 * 1024.0);
}

/* ODP_Get_kind for the GPU (utils.c:1238-1266). */
static int select_kind(int nodes, int degree, const int *num_degrees, int symmetries, int grid_s)
{
  const char *val = getenv("ODP_ASPL");
  if(!val)
    return mem_usage_mb(KIND_MATRIX, nodes, degree, symmetries, num_degrees, grid_s) <= MEM_THRESHOLD_MB
           ? KIND_MATRIX : KIND_SAVING;
  if(strcmp(val, "MATRIX") == 0) return KIND_MATRIX;
  if(strcmp(val, "MATRIX_SAVING") == 0) return KIND_SAVING;
  if(strcmp(val, "BFS") == 0) fail("BFS for CUDA is not implemented.\n");
  fail("Unknown ASPL value (%s)\n", val);
  return 0;
}

static int profile_requested(void)   /* ODP_Check_profile, utils.c:142-150 */
{
  const char *val = getenv("ODP_PROFILE");
  return val && atoi(val) == 1;
}

static void release_state(void)
{
  if(S.plan) odp_plan_destroy(S.plan);
  memset(&S, 0, sizeof(S));
}

static void init_common(const odp_shape *sh)
{
  if(S.initialized) release_state();
  int nodes = sh->grid ? sh->width * sh->height : sh->nodes;
  if(sh->symmetries <= 0 || nodes % sh->symmetries != 0)
    fail("nodes(%d) must be divisible by symmetries(%d)\n", nodes, sh->symmetries);
  int grid_s = sh->grid && sh->symmetries != 1;
  S.kind = select_kind(nodes, sh->degree, sh->num_degrees, sh->symmetries, grid_s);
  S.mem_usage = mem_usage_mb(S.kind, nodes, sh->degree, sh->symmetries, sh->num_degrees, grid_s);
  S.nodes = nodes;
  S.degree = sh->degree;
  S.symmetries = sh->symmetries;
  S.profile = profile_requested();
  odp_tuning t;
  odp_tuning_for(1, &t);
  int rc = odp_plan_create(sh, 1, &t, &S.plan);
  if(rc == ODPX_ERR_INVALID)
    fail("Invalid graph parameters (nodes=%d, degree=%d, symmetries=%d; the degree may be at most %d)\n", nodes,
         sh->degree, sh->symmetries, GBX_MAX_DEGREE);
  if(rc) fail("GPU initialisation failed (error %d)\n", rc);
  S.initialized = 1;
}

void ODP_Init_aspl_general(int nodes, int degree, int *num_degrees)
{
  odp_shape sh = { .grid = 0, .nodes = nodes, .degree = degree, .symmetries = 1, .num_degrees = num_degrees };
  init_common(&sh);
}

void ODP_Init_aspl_general_s(int nodes, int degree, int *num_degrees, int symmetries)
{
  odp_shape sh = { .grid = 0, .nodes = nodes, .degree = degree, .symmetries = symmetries,
                   .num_degrees = num_degrees };
  init_common(&sh);
}

void ODP_Init_aspl_grid(int width, int height, int degree, int *num_degrees)
{
  odp_shape sh = { .grid = 1, .width = width, .height = height, .degree = degree, .symmetries = 1,
                   .num_degrees = num_degrees };
  init_common(&sh);
}

void ODP_Init_aspl_grid_s(int width, int height, int degree, int *num_degrees, int symmetries)
{
  odp_shape sh = { .grid = 1, .width = width, .height = height, .degree = degree, .symmetries = symmetries,
                   .num_degrees = num_degrees };
  if(symmetries != 2 && symmetries != 4){
    /* The reference builds no rotation table for other values and runs the
     * general-symmetry rule (aspl_cuda.cu:190-198, utils_cuda.cu:133-151). */
    sh.grid = 0;
    sh.nodes = width * height;
  }
  init_common(&sh);
}

void ODP_Set_aspl(void *adjacency, int *diameter, long *sum, double *ASPL)
{
  if(!S.initialized) fail("ODP_Set_aspl called before ODP_Init_aspl_*\n");
  double t = now_seconds();
  const int *adj[1] = { (const int *)adjacency };
  odp_result r;
  int rc = odp_plan_run(S.plan, adj, &r);
  if(rc == ODPX_ERR_ADJACENCY) fail("adjacency holds a vertex outside [0, %d)\n", S.nodes);
  if(rc == ODPX_ERR_TIMEOUT) fail("GPU evaluation timed out\n");
  if(rc) fail("GPU evaluation failed (error %d)\n", rc);
  *diameter = r.diameter;
  *sum = r.sum;
  *ASPL = r.aspl;
  S.elapsed += now_seconds() - t;
  S.times++;
}

/* ODP_Profile, utils.c:1268-1294 */
static void print_profile(void)
{
  char host[256] = {0};
  gethostname(host, sizeof(host) - 1);
  time_t t = time(NULL);
  printf("------ Profile for SET_ASPL ------\n");
  printf("Date            = %s", ctime(&t));
  printf("Hostname        = %s\n", host);
  printf("Number of Times = %d\n", S.times);
  printf("Total Time      = %f sec.\n", S.elapsed);
  printf("Average Time    = %f sec.\n", S.elapsed / S.times);
  printf("Algorithm       = %s (%s)\n", S.kind == KIND_MATRIX ? "MATRIX" : "MATRIX_SAVING", "CUDA");
  printf("Symmetries      = %d\n", S.symmetries);
  printf("Memory Usage    = %.3f MB\n", S.mem_usage);
  printf("Num of Procs    = %d\n", 1);
  printf("Num of Threads  = %d\n", 1);
  printf("--------- End of Profile ---------\n");
}

void ODP_Finalize_aspl(void)
{
  if(!S.initialized) return;
  if(S.profile) print_profile();
  release_state();
}

ODPX_Batch *ODPX_Current_plan(void) { return S.initialized ? S.plan : NULL; }

const char *ODPX_Version(void) { return "odp_gb300 1.0 (sm_103a)"; }

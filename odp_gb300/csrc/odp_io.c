/*
 * odp_io.c -- the remaining odp.h utilities: edge-file I/O, degree and shape
 * queries, loop / multi-edge checks, printing, and the lower bounds that the
 * reference's sample programs print beside every result (the "Diameter Gap"
 * and "ASPL Gap" lines of sample/general.c and sample/grid.c).  Same
 * behaviour as the reference functions of the same names in utils.c; each
 * function cites the one it follows.
 */
#include <stdio.h>
#include <stdlib.h>
#include <stdbool.h>
#include <math.h>
#include <limits.h>
#include <float.h>
#include <string.h>
#include <pthread.h>
#include <unistd.h>
#include "odp.h"

#define FAIL(...) do{ fprintf(stderr, __VA_ARGS__); exit(1); }while(0)

static int max_i(int a, int b) { return a > b ? a : b; }
static int min_i(int a, int b) { return a < b ? a : b; }

/* ---------------------------------------------------------------------- */
/* Lower bounds printed as the "gap" lines of the sample programs.          */
/* ---------------------------------------------------------------------- */

/* Vertices that a graph of maximum degree d can hold within k hops of one
 * vertex (the Moore bound): 1 + d + d(d-1) + ... + d(d-1)^(k-1), clamped to
 * `cap`. */
static long long moore_ball(int degree, int k, long long cap)
{
  long long ball = 1, shell = degree;
  for(int r = 1; r <= k && ball < cap; r++){
    ball += shell;
    if(shell > cap) shell = cap;        /* no overflow; the ball is clamped anyway */
    else shell *= degree - 1;
  }
  return ball < cap ? ball : cap;
}

/* ODP_Set_lbounds_general (reference utils.c:1431-1459): the Moore bound for
 * `nodes` vertices of degree `degree`.  Distances from one vertex fill shells
 * r = 1, 2, ... of at most d(d-1)^(r-1) vertices each; the bound puts every
 * vertex in the nearest shell with room.  The ASPL bound is the mean distance
 * of that arrangement, the diameter bound its last shell.  The sum is an
 * integer, so one division gives the double the reference computes.  When
 * one hop already reaches every vertex (nodes <= degree + 1) the reference
 * reports diameter 0 and ASPL 0.0, and so does this function; a degree that
 * can never reach every vertex (d < 2 with more than d + 1 vertices) has no
 * finite bound: INT_MAX and DBL_MAX, where the reference does not return. */
void ODP_Set_lbounds_general(int nodes, int degree, int *low_diameter, double *low_ASPL)
{
  if(nodes <= degree + 1){
    *low_diameter = 0;
    *low_ASPL = 0.0;
    return;
  }
  long long placed = 1, distance_sum = 0, shell = degree;
  int r = 1;
  for(;;){
    const long long left = (long long)nodes - placed;
    if(shell >= left){
      distance_sum += (long long)r * left;
      break;
    }
    if(shell <= 0){
      *low_diameter = INT_MAX;
      *low_ASPL = DBL_MAX;
      return;
    }
    distance_sum += (long long)r * shell;
    placed += shell;
    shell *= degree - 1;
    r++;
  }
  *low_diameter = r;
  *low_ASPL = (double)distance_sum / (double)(nodes - 1);
}

/* Lattice points of an m x n grid within Manhattan distance D of (i, j):
 * for every row offset a, the rows at that offset (one or two) times the
 * columns within D - a. */
static long long lattice_ball(int m, int n, int i, int j, long long D)
{
  const int up = i, down = m - 1 - i, left = j, right = n - 1 - j;
  const long long amax = D < (up > down ? up : down) ? D : (up > down ? up : down);
  long long count = 0;
  for(long long a = 0; a <= amax; a++){
    const long long rows = a == 0 ? 1 : (a <= up) + (a <= down);
    const long long x = D - a;
    const long long cols = 1 + (x < left ? x : left) + (x < right ? x : right);
    count += rows * cols;
  }
  return count;
}

/* ODP_Set_lbounds_grid (reference utils.c:1461-1504, after the graph-golf
 * lattice bound): on an m x n grid whose edges span at most `length` lattice
 * steps, a vertex at Manhattan distance D from v is at least ceil(D / length)
 * hops away, and no more than the Moore ball of k hops is within k hops.  So
 * at most B_v(k) = min(#lattice points within k * length of v, Moore(k))
 * vertices lie within k hops of v, and the distances from v sum to at least
 * sum over k >= 0 of (mn - B_v(k)).  The ASPL bound averages that over all
 * ordered pairs; the diameter bound is the least k with B_v(k) = mn at a
 * corner vertex (a corner is farthest from everything, as in the
 * reference, which reads it from its last vertex, (m-1, n-1)).  Reflections
 * of the grid keep B_v, so one quadrant of vertices is enough; the integer
 * sum gives the reference's double after one division. */
void ODP_Set_lbounds_grid(int m, int n, int degree, int length, int *low_diameter, double *low_ASPL)
{
  const long long mn = (long long)m * n;
  if(degree < 2 && mn > degree + 1){           /* the Moore ball never covers the grid */
    *low_diameter = INT_MAX;
    *low_ASPL = DBL_MAX;
    return;
  }
  const long long span = (long long)(m - 1) + (n - 1);            /* largest Manhattan distance */
  int kmax = (int)((span + length - 1) / length);
  while(moore_ball(degree, kmax, mn) < mn) kmax++;                /* both parts of B reach mn by kmax */
  long long *moore = malloc(sizeof(long long) * (size_t)(kmax + 1));
  for(int k = 0; k <= kmax; k++) moore[k] = moore_ball(degree, k, mn);

  long long missing = 0;                       /* sum over v and k of (mn - B_v(k)) */
  for(int i = 0; i < (m + 1) / 2; i++){
    const int mult_i = (2 * i + 1 == m) ? 1 : 2;
    for(int j = 0; j < (n + 1) / 2; j++){
      const int mult_j = (2 * j + 1 == n) ? 1 : 2;
      long long v = 0;
      for(int k = 0; k < kmax; k++){
        long long b = lattice_ball(m, n, i, j, (long long)k * length);
        if(b > moore[k]) b = moore[k];
        if(b == mn) break;
        v += mn - b;
      }
      missing += v * mult_i * mult_j;
    }
  }
  int diam = 0;
  for(;; diam++){
    long long b = lattice_ball(m, n, m - 1, n - 1, (long long)diam * length);
    if((b < moore[diam] ? b : moore[diam]) == mn) break;
  }
  free(moore);
  *low_diameter = diam;
  *low_ASPL = (double)missing / ((double)mn * (double)(mn - 1));
}

/* ODP_Set_degrees, utils.c:1545-1555 */
void ODP_Set_degrees(int nodes, int lines, int (*edge)[2], int *num_degrees)
{
  for(int i = 0; i < nodes; i++) num_degrees[i] = 0;
  for(int i = 0; i < lines; i++){
    num_degrees[edge[i][0]]++;
    num_degrees[edge[i][1]]++;
  }
}

/* ODP_Get_lines, utils.c:1369-1384: number of newline characters (counted
 * a block at a time). */
int ODP_Get_lines(char *fname)
{
  FILE *fp = fopen(fname, "r");
  if(!fp) FAIL("File not found\n");
  enum { BLOCK = 1 << 20 };
  char *buf = malloc(BLOCK);
  long long lines = 0;
  size_t got;
  while((got = fread(buf, 1, BLOCK, fp)) > 0){
    const char *q = buf, *end = buf + got;
    while((q = memchr(q, '\n', (size_t)(end - q))) != NULL){ lines++; q++; }
  }
  free(buf);
  fclose(fp);
  return (int)lines;
}

/* ODP_Get_nodes, utils.c:1358-1367 */
int ODP_Get_nodes(int lines, int (*edge)[2])
{
  int hi = 0;
  for(int i = 0; i < lines; i++) hi = max_i(hi, max_i(edge[i][0], edge[i][1]));
  return hi + 1;
}

/* ODP_Get_degree, utils.c:1339-1356 */
int ODP_Get_degree(int nodes, int lines, int (*edge)[2])
{
  int *cnt = calloc((size_t)(nodes > 0 ? nodes : 1), sizeof(int));
  for(int i = 0; i < lines; i++){
    cnt[edge[i][0]]++;
    cnt[edge[i][1]]++;
  }
  int degree = cnt[0];
  for(int i = 1; i < nodes; i++) degree = max_i(degree, cnt[i]);
  free(cnt);
  return degree;
}

/* ODP_Get_length, utils.c:1316-1323: longest edge in lattice steps. */
int ODP_Get_length(int lines, int height, int (*edge)[2])
{
  int length = 0;
  for(int i = 0; i < lines; i++){
    int u = edge[i][0], v = edge[i][1];
    length = max_i(length, abs(u / height - v / height) + abs(u % height - v % height));
  }
  return length;
}

/* ODP_Check_general, utils.c:1325-1337: an edge file of "u v" lines (not "x,y x,y"). */
bool ODP_Check_general(char *fname)
{
  FILE *fp = fopen(fname, "r");
  if(!fp) FAIL("File not found\n");
  int a = 1, b = -1;
  if(fscanf(fp, "%d %d", &a, &b) < 0) b = -1;
  fclose(fp);
  return b != -1;
}

/* ODP_Check_multiple_edges, utils.c:1305-1314 */
bool ODP_Check_multiple_edges(int lines, int (*edge)[2])
{
  for(int i = 0; i < lines; i++)
    for(int j = i + 1; j < lines; j++){
      int a = edge[i][0], b = edge[i][1], c = edge[j][0], d = edge[j][1];
      if((a == c && b == d) || (a == d && b == c)){
        printf("Multiple edeges are found in lines %d %d\n", i + 1, j + 1);
        return true;
      }
    }
  return false;
}

/* ODP_Check_loop, utils.c:1296-1303 */
bool ODP_Check_loop(int lines, int (*edge)[2])
{
  for(int i = 0; i < lines; i++)
    if(edge[i][0] == edge[i][1]){
      printf("Loop is found in line %d\n", i + 1);
      return true;
    }
  return false;
}

/* ------------------------------------------------------------------------ */
/* Edge files.  The reference reads them with fscanf (utils.c:1386-1429), at  */
/* tens of MB/s; a graphgolf file of 10^6 vertices is hundreds of MB.  Here   */
/* the file is read whole and its integers are parsed by hand, in parallel    */
/* slices cut at newlines, with the conversion rules of %d (skip white space, */
/* optional sign, decimal digits).  On well-formed files the result is the    */
/* reference's; the reference loops until fscanf returns EOF, so an odd       */
/* integer at the end still makes one last edge whose second end is the      */
/* previous edge's, and so it is here.  A token that is not an integer ends   */
/* the read (where the reference would loop for ever).                        */
/* ------------------------------------------------------------------------ */

static char *read_whole(const char *fname, size_t *size)
{
  FILE *fp = fopen(fname, "rb");
  if(!fp) FAIL("File not found\n");
  if(fseek(fp, 0, SEEK_END) != 0) FAIL("Cannot read %s\n", fname);
  long len = ftell(fp);
  if(len < 0 || fseek(fp, 0, SEEK_SET) != 0) FAIL("Cannot read %s\n", fname);
  char *buf = malloc((size_t)len + 1);
  if(!buf) FAIL("Out of memory reading %s\n", fname);
  size_t got = fread(buf, 1, (size_t)len, fp);
  fclose(fp);
  buf[got] = '\0';
  *size = got;
  return buf;
}

static inline int is_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }

/* Next %d integer in [p, end): 1 and *v on success, 0 at the end, -1 on a
 * token that is not an integer.  *pp moves past what was read. */
static inline int scan_int(const char **pp, const char *end, int *v)
{
  const char *p = *pp;
  while(p < end && is_ws(*p)) p++;
  if(p == end){ *pp = p; return 0; }
  int neg = 0;
  if(*p == '+' || *p == '-'){ neg = *p == '-'; p++; }
  if(p == end || *p < '0' || *p > '9'){ *pp = p; return -1; }
  long long x = 0;
  while(p < end && *p >= '0' && *p <= '9'){ x = x * 10 + (*p - '0'); p++; }
  *v = (int)(neg ? -x : x);
  *pp = p;
  return 1;
}

typedef struct {
  const char *begin, *end;
  long long count;            /* integers before the slice's end or its first bad token */
  int bad;                    /* the slice holds a token that is not an integer */
  long long first;            /* global index of the slice's first integer (pass 2) */
  long long limit;            /* integers to store in total */
  int *out;
} int_slice;

static void *count_ints(void *arg)
{
  int_slice *s = arg;
  const char *p = s->begin;
  int v, r;
  s->count = 0;
  s->bad = 0;
  while((r = scan_int(&p, s->end, &v)) == 1) s->count++;
  if(r < 0) s->bad = 1;
  return NULL;
}

static void *store_ints(void *arg)
{
  int_slice *s = arg;
  const char *p = s->begin;
  long long g = s->first;
  int v;
  while(g < s->limit && scan_int(&p, s->end, &v) == 1) s->out[g++] = v;
  return NULL;
}

/* All integers of buf in order (up to the first bad token) into out (at most
 * `cap` of them, cap < 0: no limit); returns how many the file has. */
static long long parse_ints(const char *buf, size_t size, int *out, long long cap)
{
  long cpus = sysconf(_SC_NPROCESSORS_ONLN);
  int nt = size < (4u << 20) ? 1 : (int)(cpus < 16 ? (cpus < 1 ? 1 : cpus) : 16);
  int_slice sl[16];
  pthread_t th[16];
  const char *end = buf + size, *b = buf;
  for(int k = 0; k < nt; k++){
    const char *e = (k == nt - 1) ? end : buf + size / (size_t)nt * (size_t)(k + 1);
    if(e < b) e = b;
    while(e < end && *e != '\n') e++;            /* slices end after a newline: no token is cut */
    if(e < end) e++;
    sl[k].begin = b; sl[k].end = e;
    b = e;
  }
  for(int k = 1; k < nt; k++) if(pthread_create(&th[k], NULL, count_ints, &sl[k])) count_ints(&sl[k]), th[k] = 0;
  count_ints(&sl[0]);
  for(int k = 1; k < nt; k++) if(th[k]) pthread_join(th[k], NULL);
  long long total = 0;
  int last = nt - 1;
  for(int k = 0; k < nt; k++){
    sl[k].first = total;
    total += sl[k].count;
    if(sl[k].bad){ last = k; break; }
  }
  for(int k = 0; k <= last; k++){ sl[k].limit = (cap < 0 || total < cap) ? total : cap; sl[k].out = out; }
  for(int k = 1; k <= last; k++) if(pthread_create(&th[k], NULL, store_ints, &sl[k])) store_ints(&sl[k]), th[k] = 0;
  store_ints(&sl[0]);
  for(int k = 1; k <= last; k++) if(th[k]) pthread_join(th[k], NULL);
  return total;
}

/* ODP_Read_edge_general, utils.c:1386-1401 */
void ODP_Read_edge_general(char *fname, int (*edge)[2])
{
  size_t size;
  char *buf = read_whole(fname, &size);
  /* the integers go straight into edge, in file order, as the reference
   * stores them pair by pair (edge was sized by the caller) */
  int *flat = &edge[0][0];
  long long total = parse_ints(buf, size, flat, -1);
  if(total % 2) flat[total] = total >= 3 ? flat[total - 2] : 0;
  free(buf);
}

/* One "x,y x,y" record (the format "%d,%d %d,%d"): 1, 0 at the end, -1 on a
 * mismatch. */
static int scan_grid_record(const char **pp, const char *end, int c[4])
{
  const char *p = *pp;
  int r = scan_int(&p, end, &c[0]);
  if(r <= 0){ *pp = p; return r; }
  for(int k = 1; k < 4; k++){
    if(k != 2){                                  /* a literal ',' right after the integer */
      if(p == end || *p != ',') { *pp = p; return -1; }
      p++;
    }
    if(scan_int(&p, end, &c[k]) != 1){ *pp = p; return -1; }
  }
  *pp = p;
  return 1;
}

/* ODP_Read_edge_grid, utils.c:1403-1429: "x,y x,y" lines, vertex = x*height + y. */
void ODP_Read_edge_grid(char *fname, int *w, int *h, int (*edge)[2])
{
  size_t size;
  char *buf = read_whole(fname, &size);
  const char *p = buf, *end = buf + size;
  int c[4];
  long long rec = 0;
  int mw = 0, mh = 0;
  while(scan_grid_record(&p, end, c) == 1){
    if(c[0] > mw) mw = c[0];
    if(c[2] > mw) mw = c[2];
    if(c[1] > mh) mh = c[1];
    if(c[3] > mh) mh = c[3];
    rec++;
  }
  *w = mw + 1;
  *h = mh + 1;
  p = buf;
  for(long long i = 0; i < rec && scan_grid_record(&p, end, c) == 1; i++){
    edge[i][0] = c[0] * (*h) + c[1];
    edge[i][1] = c[2] * (*h) + c[3];
  }
  free(buf);
}

/* Writers: the same text as the reference's fprintf loops, formatted by hand
 * in parallel slices and written in order. */
static inline char *put_int(char *o, int v)
{
  char t[12];
  int n = 0;
  unsigned u = v < 0 ? 0u - (unsigned)v : (unsigned)v;
  do{ t[n++] = (char)('0' + u % 10); u /= 10; }while(u);
  if(v < 0) *o++ = '-';
  while(n) *o++ = t[--n];
  return o;
}

typedef struct {
  const int (*edge)[2];
  int first, last, height;      /* height > 0: grid text */
  char *text;
  size_t len;
} text_slice;

static void *format_edges(void *arg)
{
  text_slice *s = arg;
  char *o = s->text;
  for(int i = s->first; i < s->last; i++){
    if(s->height > 0){
      const int h = s->height;
      o = put_int(o, s->edge[i][0] / h); *o++ = ',';
      o = put_int(o, s->edge[i][0] % h); *o++ = ' ';
      o = put_int(o, s->edge[i][1] / h); *o++ = ',';
      o = put_int(o, s->edge[i][1] % h); *o++ = '\n';
    }
    else{
      o = put_int(o, s->edge[i][0]); *o++ = ' ';
      o = put_int(o, s->edge[i][1]); *o++ = '\n';
    }
  }
  s->len = (size_t)(o - s->text);
  return NULL;
}

static void write_edges(int lines, int height, int (*edge)[2], const char *fname)
{
  FILE *fp = fopen(fname, "w");
  if(!fp) FAIL("Cannot open %s\n", fname);
  long cpus = sysconf(_SC_NPROCESSORS_ONLN);
  int nt = lines < (1 << 18) ? 1 : (int)(cpus < 16 ? (cpus < 1 ? 1 : cpus) : 16);
  const size_t per_line = height > 0 ? 48 : 24;
  text_slice sl[16];
  pthread_t th[16];
  for(int k = 0; k < nt; k++){
    sl[k].edge = (const int (*)[2])edge;
    sl[k].first = (int)((long long)lines * k / nt);
    sl[k].last = (int)((long long)lines * (k + 1) / nt);
    sl[k].height = height;
    sl[k].text = malloc(per_line * (size_t)(sl[k].last - sl[k].first) + 1);
    if(!sl[k].text) FAIL("Out of memory writing %s\n", fname);
  }
  for(int k = 1; k < nt; k++) if(pthread_create(&th[k], NULL, format_edges, &sl[k])) format_edges(&sl[k]), th[k] = 0;
  format_edges(&sl[0]);
  for(int k = 1; k < nt; k++) if(th[k]) pthread_join(th[k], NULL);
  for(int k = 0; k < nt; k++){
    if(fwrite(sl[k].text, 1, sl[k].len, fp) != sl[k].len) FAIL("Cannot write %s\n", fname);
    free(sl[k].text);
  }
  fclose(fp);
}

/* ODP_Write_edge_general, utils.c:1153-1164: "%d %d\n" per edge */
void ODP_Write_edge_general(int lines, int (*edge)[2], char *fname)
{
  write_edges(lines, 0, edge, fname);
}

/* ODP_Write_edge_grid, utils.c:1166-1180: "%d,%d %d,%d\n" per edge */
void ODP_Write_edge_grid(int lines, int height, int (*edge)[2], char *fname)
{
  if(height <= 0) FAIL("height must be positive\n");
  write_edges(lines, height, edge, fname);
}

/* ODP_Print_adjacency, utils.c:25-38 */
void ODP_Print_adjacency(int nodes, int degree, int *num_degrees, void *adjacency)
{
  const int *adj = adjacency;
  for(int i = 0; i < nodes; i++){
    printf("%d ", i);
    int d = num_degrees ? num_degrees[i] : degree;
    for(int j = 0; j < d; j++)
      if(adj[(size_t)i * degree + j] != -1) printf("%3d", adj[(size_t)i * degree + j]);
    printf("\n");
  }
}

/* ODP_Print_edge_general, utils.c:40-44 */
void ODP_Print_edge_general(int lines, int (*edge)[2])
{
  for(int i = 0; i < lines; i++) printf("%d %d\n", edge[i][0], edge[i][1]);
}

/* ODP_Print_edge_grid, utils.c:46-53 */
void ODP_Print_edge_grid(int lines, int height, int (*edge)[2])
{
  for(int i = 0; i < lines; i++)
    printf("%d,%d %d,%d\n", edge[i][0] / height, edge[i][0] % height, edge[i][1] / height, edge[i][1] % height);
}

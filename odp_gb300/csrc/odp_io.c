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
#include "odp.h"

#define FAIL(...) do{ fprintf(stderr, __VA_ARGS__); exit(1); }while(0)

static int max_i(int a, int b) { return a > b ? a : b; }
static int min_i(int a, int b) { return a < b ? a : b; }

/* ODP_Set_lbounds_general, utils.c:1431-1459: the Moore bound. */
void ODP_Set_lbounds_general(int nodes, int degree, int *low_diameter, double *low_ASPL)
{
  int diam = -1, n = 1, r = 1;
  double aspl = 0.0;
  for(;;){
    int reach = n + degree * pow(degree - 1, r - 1);
    if(reach >= nodes) break;
    n = reach;
    aspl += r * degree * pow(degree - 1, r - 1);
    diam = r++;
  }
  diam++;
  aspl += diam * (nodes - n);
  aspl /= (nodes - 1);
  *low_diameter = diam;
  *low_ASPL = aspl;
}

/* ODP_Set_lbounds_grid, utils.c:1461-1504: per-vertex hop histogram capped
 * by the Moore bound, with edges of at most `length` lattice steps. */
void ODP_Set_lbounds_grid(int m, int n, int degree, int length, int *low_diameter, double *low_ASPL)
{
  int mn = m * n, current = degree, ii;
  int cap = mn + m + n + 8;
  int *moore = calloc((size_t)cap, sizeof(int));
  int *hist = calloc((size_t)cap, sizeof(int));
  int *mh = calloc((size_t)cap, sizeof(int));
  double sum = 0;
  moore[0] = 1;
  moore[1] = degree + 1;
  for(ii = 2;; ii++){
    current = current * (degree - 1);
    moore[ii] = moore[ii - 1] + current;
    if(moore[ii] >= mn){ moore[ii] = mn; break; }
  }
  int maxhop = max_i((m + n - 2 + (length - 1)) / length, ii);
  for(int i = ii + 1; i <= maxhop; i++) moore[i] = mn;
  for(int i = 0; i < m; i++){
    for(int j = 0; j < n; j++){
      for(int k = 0; k <= maxhop; k++) hist[k] = 0;
      for(int i2 = 0; i2 < m; i2++)
        for(int j2 = 0; j2 < n; j2++)
          hist[(abs(i - i2) + abs(j - j2) + length - 1) / length]++;
      for(int k = 1; k <= maxhop; k++) hist[k] += hist[k - 1];
      for(int k = 0; k <= maxhop; k++) mh[k] = min_i(hist[k], moore[k]);
      for(int k = 1; k <= maxhop; k++) sum += (double)(mh[k] - mh[k - 1]) * k;
    }
  }
  int dboth = 0;
  while(mh[dboth] != mn) dboth++;
  *low_diameter = dboth;
  *low_ASPL = sum / ((double)mn * (mn - 1));
  free(moore); free(hist); free(mh);
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

/* ODP_Get_lines, utils.c:1369-1384: number of newline characters. */
int ODP_Get_lines(char *fname)
{
  FILE *fp = fopen(fname, "r");
  if(!fp) FAIL("File not found\n");
  int lines = 0, c;
  while((c = fgetc(fp)) != EOF)
    if(c == '\n') lines++;
  fclose(fp);
  return lines;
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

/* ODP_Read_edge_general, utils.c:1386-1401 */
void ODP_Read_edge_general(char *fname, int (*edge)[2])
{
  FILE *fp = fopen(fname, "r");
  if(!fp) FAIL("File not found\n");
  int a, b, i = 0;
  while(fscanf(fp, "%d %d", &a, &b) == 2){
    edge[i][0] = a;
    edge[i][1] = b;
    i++;
  }
  fclose(fp);
}

/* ODP_Read_edge_grid, utils.c:1403-1429: "x,y x,y" lines, vertex = x*height + y. */
void ODP_Read_edge_grid(char *fname, int *w, int *h, int (*edge)[2])
{
  FILE *fp = fopen(fname, "r");
  if(!fp) FAIL("File not found\n");
  int c[4];
  *w = 0;
  *h = 0;
  while(fscanf(fp, "%d,%d %d,%d", &c[0], &c[1], &c[2], &c[3]) == 4){
    *w = max_i(*w, max_i(c[0], c[2]));
    *h = max_i(*h, max_i(c[1], c[3]));
  }
  *w += 1;
  *h += 1;
  rewind(fp);
  int i = 0;
  while(fscanf(fp, "%d,%d %d,%d", &c[0], &c[1], &c[2], &c[3]) == 4){
    edge[i][0] = c[0] * (*h) + c[1];
    edge[i][1] = c[2] * (*h) + c[3];
    i++;
  }
  fclose(fp);
}

/* ODP_Write_edge_general, utils.c:1153-1164 */
void ODP_Write_edge_general(int lines, int (*edge)[2], char *fname)
{
  FILE *fp = fopen(fname, "w");
  if(!fp) FAIL("Cannot open %s\n", fname);
  for(int i = 0; i < lines; i++) fprintf(fp, "%d %d\n", edge[i][0], edge[i][1]);
  fclose(fp);
}

/* ODP_Write_edge_grid, utils.c:1166-1180 */
void ODP_Write_edge_grid(int lines, int height, int (*edge)[2], char *fname)
{
  FILE *fp = fopen(fname, "w");
  if(!fp) FAIL("Cannot open %s\n", fname);
  for(int i = 0; i < lines; i++)
    fprintf(fp, "%d,%d %d,%d\n", edge[i][0] / height, edge[i][0] % height, edge[i][1] / height,
            edge[i][1] % height);
  fclose(fp);
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

/*
 * ref_driver.c -- command-line front end to the reference ODP CPU library
 * (libodp.a / libodp_threads.a), built from the reference's own sources by
 * oracle/Makefile into oracle/_ref/.  Test infrastructure only: it produces
 * golden vectors (seeded graphs, ASPL results, 2-opt mutation traces) that pin
 * the oracle restatement and the product's graph utilities.  Nothing in the
 * product links it.
 *
 * Every computation here is a call into the reference's public API
 * (include/odp.h); this file only moves bytes between files and those calls.
 *
 * Commands (all integers decimal; binary files are raw little-endian int32):
 *   gen general   N D S SEED OUT        ODP_Generate_random_general_s
 *   gen grid      W H D LEN S SEED OUT  ODP_Generate_random_grid_s
 *   conv general  N D S EDGES OUT       ODP_Conv_edge2adjacency_general_s
 *   conv grid     W H D S EDGES OUT     ODP_Conv_edge2adjacency_grid_s
 *   aspl general  N D S ADJ NUMDEG|-    Init_general(_s) / Set / Finalize
 *   aspl grid     W H D S ADJ NUMDEG|-  Init_grid(_s) / Set / Finalize
 *   mutate general N D S SEED ITERS ADJ OUT  ODP_Mutate_adjacency_general_s trace
 *   mutate grid   W H D LEN S SEED ITERS ADJ OUT  ODP_Mutate_adjacency_grid_s trace
 *   lines FILE                          ODP_Get_lines (edge text files)
 *   readedges general|grid FILE OUT     ODP_Read_edge_* -> raw pairs
 *   lbounds general N D                 ODP_Set_lbounds_general
 *   lbounds grid W H D LEN              ODP_Set_lbounds_grid
 *                                       ("<diameter> <ASPL as %a>")
 *
 * "aspl" prints one line: "<diameter> <sum> <ASPL as %a hex float> <ASPL %.10f>".
 * "mutate" writes, per iteration, the 8 ints of ODP_Restore followed by the
 * full adjacency after the last iteration.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "odp.h"

static void *read_file(const char *path, size_t *bytes)
{
  FILE *f = fopen(path, "rb");
  if(!f){ fprintf(stderr, "cannot open %s\n", path); exit(2); }
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  void *p = malloc(sz > 0 ? (size_t)sz : 1);
  if(sz > 0 && fread(p, 1, (size_t)sz, f) != (size_t)sz){ fprintf(stderr, "short read %s\n", path); exit(2); }
  fclose(f);
  *bytes = (size_t)sz;
  return p;
}

static void write_file(const char *path, const void *p, size_t bytes)
{
  FILE *f = fopen(path, "wb");
  if(!f){ fprintf(stderr, "cannot open %s\n", path); exit(2); }
  if(bytes && fwrite(p, 1, bytes, f) != bytes){ fprintf(stderr, "short write %s\n", path); exit(2); }
  fclose(f);
}

static void print_result(int diameter, long sum, double aspl)
{
  printf("%d %ld %a %.10f\n", diameter, sum, aspl, aspl);
}

int main(int argc, char **argv)
{
  if(argc < 3){ fprintf(stderr, "usage: see header\n"); return 2; }
  const char *cmd = argv[1], *kind = argv[2];
  int grid = strcmp(kind, "grid") == 0;

  if(strcmp(cmd, "gen") == 0){
    if(!grid){
      int n = atoi(argv[3]), d = atoi(argv[4]), s = atoi(argv[5]);
      unsigned seed = (unsigned)strtoul(argv[6], NULL, 10);
      int lines = (n * d) / 2;
      int (*edge)[2] = malloc(sizeof(int) * 2 * (size_t)lines);
      ODP_Srand(seed);
      ODP_Generate_random_general_s(n, d, s, edge);
      write_file(argv[7], edge, sizeof(int) * 2 * (size_t)lines);
    }
    else{
      int w = atoi(argv[3]), h = atoi(argv[4]), d = atoi(argv[5]), len = atoi(argv[6]), s = atoi(argv[7]);
      unsigned seed = (unsigned)strtoul(argv[8], NULL, 10);
      int lines = (w * h * d) / 2;
      int (*edge)[2] = malloc(sizeof(int) * 2 * (size_t)lines);
      ODP_Srand(seed);
      ODP_Generate_random_grid_s(w, h, d, len, s, edge);
      write_file(argv[9], edge, sizeof(int) * 2 * (size_t)lines);
    }
    return 0;
  }

  if(strcmp(cmd, "conv") == 0){
    size_t bytes;
    if(!grid){
      int n = atoi(argv[3]), d = atoi(argv[4]), s = atoi(argv[5]);
      int (*edge)[2] = read_file(argv[6], &bytes);
      int lines = (int)(bytes / 8);
      int *adj = malloc(sizeof(int) * (size_t)(n / s) * d);
      ODP_Conv_edge2adjacency_general_s(n, lines, d, edge, s, adj);
      write_file(argv[7], adj, sizeof(int) * (size_t)(n / s) * d);
    }
    else{
      int w = atoi(argv[3]), h = atoi(argv[4]), d = atoi(argv[5]), s = atoi(argv[6]);
      int (*edge)[2] = read_file(argv[7], &bytes);
      int lines = (int)(bytes / 8);
      int n = w * h;
      int (*adj)[d] = malloc(sizeof(int) * (size_t)(n / s) * d);
      ODP_Conv_edge2adjacency_grid_s(w, h, lines, d, edge, s, adj);
      write_file(argv[8], adj, sizeof(int) * (size_t)(n / s) * d);
    }
    return 0;
  }

  if(strcmp(cmd, "aspl") == 0){
    size_t bytes;
    int diameter; long sum; double aspl;
    if(!grid){
      int n = atoi(argv[3]), d = atoi(argv[4]), s = atoi(argv[5]);
      int *adj = read_file(argv[6], &bytes);
      int *numdeg = NULL;
      if(strcmp(argv[7], "-") != 0) numdeg = read_file(argv[7], &bytes);
      if(s == 1) ODP_Init_aspl_general(n, d, numdeg);
      else       ODP_Init_aspl_general_s(n, d, numdeg, s);
      ODP_Set_aspl(adj, &diameter, &sum, &aspl);
      ODP_Finalize_aspl();
    }
    else{
      int w = atoi(argv[3]), h = atoi(argv[4]), d = atoi(argv[5]), s = atoi(argv[6]);
      int *adj = read_file(argv[7], &bytes);
      int *numdeg = NULL;
      if(strcmp(argv[8], "-") != 0) numdeg = read_file(argv[8], &bytes);
      if(s == 1) ODP_Init_aspl_grid(w, h, d, numdeg);
      else       ODP_Init_aspl_grid_s(w, h, d, numdeg, s);
      ODP_Set_aspl(adj, &diameter, &sum, &aspl);
      ODP_Finalize_aspl();
    }
    print_result(diameter, sum, aspl);
    return 0;
  }

  if(strcmp(cmd, "mutate") == 0){
    size_t bytes;
    if(!grid){
      int n = atoi(argv[3]), d = atoi(argv[4]), s = atoi(argv[5]);
      unsigned seed = (unsigned)strtoul(argv[6], NULL, 10);
      int iters = atoi(argv[7]);
      int (*adj)[d] = read_file(argv[8], &bytes);
      size_t adj_bytes = sizeof(int) * (size_t)(n / s) * d;
      int *out = malloc(sizeof(int) * 8 * (size_t)iters + adj_bytes);
      ODP_Srand(seed);
      for(int i = 0; i < iters; i++){
        ODP_Restore r;
        ODP_Mutate_adjacency_general_s(n, d, NULL, s, &r, adj);
        memcpy(out + 8 * (size_t)i, &r, sizeof(int) * 8);
      }
      memcpy(out + 8 * (size_t)iters, adj, adj_bytes);
      write_file(argv[9], out, sizeof(int) * 8 * (size_t)iters + adj_bytes);
    }
    else{
      int w = atoi(argv[3]), h = atoi(argv[4]), d = atoi(argv[5]), len = atoi(argv[6]), s = atoi(argv[7]);
      unsigned seed = (unsigned)strtoul(argv[8], NULL, 10);
      int iters = atoi(argv[9]);
      int (*adj)[d] = read_file(argv[10], &bytes);
      int n = w * h;
      size_t adj_bytes = sizeof(int) * (size_t)(n / s) * d;
      int *out = malloc(sizeof(int) * 8 * (size_t)iters + adj_bytes);
      ODP_Srand(seed);
      for(int i = 0; i < iters; i++){
        ODP_Restore r;
        ODP_Mutate_adjacency_grid_s(w, h, d, NULL, len, s, &r, adj);
        memcpy(out + 8 * (size_t)i, &r, sizeof(int) * 8);
      }
      memcpy(out + 8 * (size_t)iters, adj, adj_bytes);
      write_file(argv[11], out, sizeof(int) * 8 * (size_t)iters + adj_bytes);
    }
    return 0;
  }

  if(strcmp(cmd, "readedges") == 0){
    int lines = ODP_Get_lines((char *)argv[3]);
    int (*edge)[2] = malloc(sizeof(int) * 2 * (size_t)lines);
    if(!grid){
      ODP_Read_edge_general((char *)argv[3], edge);
      printf("%d\n", lines);
    }
    else{
      int w, h;
      ODP_Read_edge_grid((char *)argv[3], &w, &h, edge);
      printf("%d %d %d\n", lines, w, h);
    }
    write_file(argv[4], edge, sizeof(int) * 2 * (size_t)lines);
    return 0;
  }

  if(strcmp(cmd, "lbounds") == 0){
    int low_diameter; double low_aspl;
    if(!grid) ODP_Set_lbounds_general(atoi(argv[3]), atoi(argv[4]), &low_diameter, &low_aspl);
    else      ODP_Set_lbounds_grid(atoi(argv[3]), atoi(argv[4]), atoi(argv[5]), atoi(argv[6]), &low_diameter, &low_aspl);
    printf("%d %a\n", low_diameter, low_aspl);
    return 0;
  }

  fprintf(stderr, "unknown command %s\n", cmd);
  return 2;
}

/*
 * replay.c -- a client of the drop-in odp.h API that prints the report of the
 * reference's sample programs (sample/general.c, sample/grid.c) for one edge
 * file, so that the output of a run against libodp_gb300 can be compared
 * with the reference's golden tables character for character.
 *
 *   replay general FILE.edges     |     replay grid FILE.edges
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "odp.h"

int main(int argc, char *argv[])
{
  if(argc != 3){ fprintf(stderr, "usage: replay general|grid FILE\n"); return 2; }
  int grid = strcmp(argv[1], "grid") == 0;
  char *file = argv[2];
  int diameter, low_diameter, width = 0, height = 0;
  long sum;
  double aspl, low_aspl;
  int lines = ODP_Get_lines(file);
  int (*edge)[2] = malloc(sizeof(int) * 2 * (size_t)lines);
  if(grid) ODP_Read_edge_grid(file, &width, &height, edge);
  else     ODP_Read_edge_general(file, edge);
  int nodes = ODP_Get_nodes(lines, edge);
  int degree = ODP_Get_degree(nodes, lines, edge);
  int *adjacency = malloc(sizeof(int) * (size_t)nodes * degree);
  if(grid){
    ODP_Conv_edge2adjacency_grid(width, height, lines, degree, edge, adjacency);
    ODP_Init_aspl_grid(width, height, degree, NULL);
  }
  else{
    ODP_Conv_edge2adjacency_general(nodes, lines, degree, edge, adjacency);
    ODP_Init_aspl_general(nodes, degree, NULL);
  }
  ODP_Set_aspl(adjacency, &diameter, &sum, &aspl);
  ODP_Finalize_aspl();
  if(grid){
    int length = ODP_Get_length(lines, height, edge);
    ODP_Set_lbounds_grid(width, height, degree, length, &low_diameter, &low_aspl);
    printf("Width = %d, Height = %d, Length = %d, Degrees = %d\n", width, height, length, degree);
  }
  else{
    ODP_Set_lbounds_general(nodes, degree, &low_diameter, &low_aspl);
    printf("Nodes = %d, Degrees = %d\n", nodes, degree);
  }
  printf("Diameter     = %d\n", diameter);
  printf("Diameter Gap = %d (%d - %d)\n", diameter - low_diameter, diameter, low_diameter);
  printf("ASPL         = %.10f (%ld/%.0f)\n", aspl, sum, (double)nodes * (nodes - 1) / 2);
  printf("ASPL Gap     = %.10f (%.10f - %.10f)\n", aspl - low_aspl, aspl, low_aspl);
  free(edge);
  free(adjacency);
  return 0;
}

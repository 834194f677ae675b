/*
 * odp.h -- drop-in public API of the GB300 ODP library (libodp_gb300).
 *
 * The declarations keep the reference's names, argument order and meaning
 * (reference include/odp.h:1-59) so that programs written against
 * libodp_cuda.a compile and link unchanged.  The ASPL entry points
 * (ODP_Init_aspl_*, ODP_Set_aspl, ODP_Finalize_aspl) run on one GB300 through
 * the CUDA layer in odp_gb300/csrc; the utilities run on the host.
 *
 * Entry point                 replaces (reference)
 *   ODP_Init_aspl_general       aspl_cuda.cu:159-162
 *   ODP_Init_aspl_general_s     aspl_cuda.cu:164-179
 *   ODP_Init_aspl_grid          aspl_cuda.cu:181-186
 *   ODP_Init_aspl_grid_s        aspl_cuda.cu:188-224
 *   ODP_Set_aspl                aspl_cuda.cu:242-263
 *   ODP_Finalize_aspl           aspl_cuda.cu:226-240
 *   utilities below             utils.c (same names)
 *
 * The MPI variants (reference odp.h:15-21) are not provided: this library
 * runs in one process on one GPU.
 */
#ifndef ODP_H_INCLUDED
#define ODP_H_INCLUDED
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int u[2], v[2], u_d[2], v_d[2];
} ODP_Restore;

/* ASPL evaluation (GPU). */
extern void ODP_Init_aspl_general(int nodes, int degree, int *num_degrees);
extern void ODP_Init_aspl_general_s(int nodes, int degree, int *num_degrees, int symmetries);
extern void ODP_Init_aspl_grid(int width, int height, int degree, int *num_degrees);
extern void ODP_Init_aspl_grid_s(int width, int height, int degree, int *num_degrees, int symmetries);
extern void ODP_Set_aspl(void *adjacency, int *diameter, long *sum, double *ASPL);
extern void ODP_Finalize_aspl(void);

/* Utilities (host). */
extern void ODP_Set_lbounds_general(int nodes, int degree, int *low_diameter, double *low_ASPL);
extern void ODP_Set_lbounds_grid(int m, int n, int degree, int length, int *low_diameter, double *low_ASPL);
extern void ODP_Set_degrees(int nodes, int lines, int (*edge)[2], int *num_degrees);
extern int  ODP_Get_lines(char *fname);
extern int  ODP_Get_nodes(int lines, int (*edge)[2]);
extern int  ODP_Get_degree(int nodes, int lines, int (*edge)[2]);
extern int  ODP_Get_length(int lines, int height, int (*edge)[2]);
extern bool ODP_Check_general(char *fname);
extern bool ODP_Check_multiple_edges(int lines, int (*edge)[2]);
extern bool ODP_Check_loop(int lines, int (*edge)[2]);
extern void ODP_Read_edge_general(char *fname, int (*edge)[2]);
extern void ODP_Read_edge_grid(char *fname, int *w, int *h, int (*edge)[2]);
extern void ODP_Write_edge_general(int lines, int (*edge)[2], char *fname);
extern void ODP_Write_edge_grid(int lines, int height, int (*edge)[2], char *fname);
extern void ODP_Conv_edge2adjacency_general(int nodes, int lines, int degree, int (*edge)[2], void *adjacency);
extern void ODP_Conv_edge2adjacency_grid(int width, int height, int lines, int degree, int (*edge)[2], void *adjacency);
extern void ODP_Conv_edge2adjacency_general_s(int nodes, int lines, int degree, int (*edge)[2], int symmetries, void *adjacency);
extern void ODP_Conv_edge2adjacency_grid_s(int width, int height, int lines, int degree, int (*edge)[2], int symmetries, void *adjacency);
extern void ODP_Conv_adjacency2edge_general(int nodes, int degree, int *num_degrees, void *adjacency, int (*edge)[2]);
extern void ODP_Conv_adjacency2edge_grid(int width, int height, int degree, int *num_degrees, void *adjacency, int (*edge)[2]);
extern void ODP_Conv_adjacency2edge_general_s(int nodes, int degree, int *num_degrees, void *adjacency, int symmetries, int (*edge)[2]);
extern void ODP_Conv_adjacency2edge_grid_s(int width, int height, int degree, int *num_degrees, void *adjacency, int symmetries, int (*edge)[2]);
extern void ODP_Srand(unsigned int seed);
extern void ODP_Generate_random_general(int nodes, int degree, int (*edge)[2]);
extern void ODP_Generate_random_general_s(int nodes, int degree, int symmetries, int (*edge)[2]);
extern void ODP_Generate_random_grid(int width, int height, int degree, int length, int (*edge)[2]);
extern void ODP_Generate_random_grid_s(int width, int height, int degree, int length, int symmetries, int (*edge)[2]);
extern void ODP_Print_adjacency(int nodes, int degree, int *num_degrees, void *adjacency);
extern void ODP_Print_edge_general(int lines, int (*edge)[2]);
extern void ODP_Print_edge_grid(int lines, int height, int (*edge)[2]);
#ifdef __cplusplus
extern void ODP_Mutate_adjacency_general(int nodes, int degree, int *num_degrees, ODP_Restore *r, void *adjacency);
extern void ODP_Mutate_adjacency_general_s(int nodes, int degree, int *num_degrees, int symmetries, ODP_Restore *r, void *adjacency);
extern void ODP_Mutate_adjacency_grid(int width, int height, int degree, int *num_degrees, int length, ODP_Restore *r, void *adjacency);
extern void ODP_Mutate_adjacency_grid_s(int width, int height, int degree, int *num_degrees, int length, int symmetries, ODP_Restore *r, void *adjacency);
#else
extern void ODP_Mutate_adjacency_general(int nodes, int degree, int *num_degrees, ODP_Restore *r, int (*adjacency)[degree]);
extern void ODP_Mutate_adjacency_general_s(int nodes, int degree, int *num_degrees, int symmetries, ODP_Restore *r, int (*adjacency)[degree]);
extern void ODP_Mutate_adjacency_grid(int width, int height, int degree, int *num_degrees, int length, ODP_Restore *r, int (*adjacency)[degree]);
extern void ODP_Mutate_adjacency_grid_s(int width, int height, int degree, int *num_degrees, int length, int symmetries, ODP_Restore *r, int (*adjacency)[degree]);
#endif
extern void ODP_Restore_adjacency_general(ODP_Restore r, void *adjacency);
extern void ODP_Restore_adjacency_grid(ODP_Restore r, void *adjacency);

#ifdef __cplusplus
}
#endif
#endif

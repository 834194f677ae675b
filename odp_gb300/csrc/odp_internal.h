/*
 * odp_internal.h -- declarations shared by the host-side C files of
 * libodp_gb300 (graph utilities, ASPL driver, batch and serving engines).
 * Not installed; the public surface is include/odp.h and include/odp_gb300.h.
 */
#ifndef ODP_INTERNAL_H
#define ODP_INTERNAL_H
#include <stddef.h>
#include "odp.h"
#include "odp_rng.h"

void odpx_generate_general(odp_rng *rng, int n, int d, int s, int (*edge)[2]);
void odpx_generate_grid(odp_rng *rng, int w, int h, int d, int len, int s, int (*edge)[2]);
void odpx_mutate_general(odp_rng *rng, int nodes, int degree, const int *num_degrees, int symmetries,
                         ODP_Restore *r, int *adjacency);
void odpx_mutate_grid(odp_rng *rng, int width, int height, int degree, const int *num_degrees, int length,
                      int symmetries, ODP_Restore *r, int *adjacency);
void odpx_restore_general(int nodes, int degree, int symmetries, ODP_Restore r, int *adjacency);
void odpx_restore_grid(int width, int height, int degree, int symmetries, ODP_Restore r, int *adjacency);

#endif

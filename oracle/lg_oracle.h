/*
 * lg_oracle.h -- CPU FP64 oracle of libgran's pair-force + integration path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU engine and the timed CPU baseline. The product
 * never includes this header. Parameter blocks are shared with the C ABI (libgran_gb300.h) so the
 * two sides are configured identically.
 */
#ifndef LG_ORACLE_H
#define LG_ORACLE_H

#include <stdint.h>
#include "../include/libgran_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lgo_system lgo_system;

/* threads: OpenMP threads used inside a force evaluation (1 = scalar). */
lgo_system *lgo_create(const lg_system_desc *d, const double *x0, const double *v0, const double *theta0,
                       const double *omega0, const lg_facet_desc *facets, const double *neck_strengths,
                       int64_t n_neck_strengths, int threads);
void lgo_destroy(lgo_system *s);
int lgo_step(lgo_system *s, double dt, int64_t nsteps, int64_t rebuild_every);
int lgo_update_neighbor_list(lgo_system *s);
int lgo_get(lgo_system *s, int field, double *out);
int lgo_set(lgo_system *s, int field, const double *in);
int lgo_get_pair_springs(lgo_system *s, int64_t i, int64_t j, double *out9);
int64_t lgo_count_bonds(lgo_system *s, int64_t *pairs, int64_t cap);
int64_t lgo_row_length(lgo_system *s, int64_t i);
int64_t lgo_row(lgo_system *s, int64_t i, int32_t *out, int64_t cap);
int lgo_observables(lgo_system *s, lg_observables *o);
int lgo_facet_update_positions(lgo_system *s, int32_t facet, double dt);
int lgo_facet_get_vertices(lgo_system *s, int32_t facet, double *out9);
int64_t lgo_step_index(lgo_system *s);
/* Step-handler hold mask (n bytes of LG_HOLD_* bits; NULL: none), body force, body-force centre. */
int lgo_set_hold_mask(lgo_system *s, const uint8_t *mask);
int lgo_set_body_force(lgo_system *s, const lg_body_force *f);
int lgo_set_body_centre(lgo_system *s, const double *centre);
int64_t lgo_get_connectors(lgo_system *s, double *out, int64_t cap);
int lgo_run_many(lgo_system **systems, const double *dts, const int64_t *nsteps, const int64_t *rebuild,
                 int count);
/* Seeded inputs of the benchmark workloads, bit-identical to lg_generate_rsa_aggregate and
 * lg_generate_velocities of the engine (0 = ok). */
int lgo_generate_rsa_aggregate(uint64_t seed, int64_t n, double r, double *x);
int lgo_generate_velocities(uint64_t seed, int64_t n, double vmax, double *v);

#ifdef __cplusplus
}
#endif

#endif

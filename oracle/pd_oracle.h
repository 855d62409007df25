/*
 * pd_oracle.h -- TEST INFRASTRUCTURE. CPU restatement of PeriDEM's explicit time step
 * (src/particle/timeloop.h:395-954 with particle2.h / contact.h), used only as the checker
 * by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs.
 * Nothing in the product links or calls it.
 *
 * Single-thread mode (threads == 1) reproduces the reference's per-rank serial path with
 * one MPI rank: the force Allreduce is the identity, every FP64 operation is evaluated in
 * the reference's order with contraction off (-ffp-contract=off). Multi-thread mode deals
 * particles and particle pairs round-robin to workers and sums their force vectors, like
 * the reference's MPI ranks (timeloop.h:544, 637, 658); it is used for timing only.
 */
#ifndef PD_ORACLE_H
#define PD_ORACLE_H
#include "peridem_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_sim or_sim;

/* ConfigVal's defaults (read_config.h:36-167), the same values pd_config_default gives. */
int or_config_default(pd_config *cfg);
or_sim *or_create(const pd_setup_arrays *setup, const pd_config *cfg);
void or_set_threads(or_sim *s, int threads);
/* Node-node and self-contact visit only the node pairs whose current positions lie in
 * neighbouring cells of edge just above the contact radius, in the reference's order: the
 * same sums, bit for bit, at a cost that follows the pairs in reach (large test cases). */
void or_set_cell_search(or_sim *s, int on);
/* Runs steps t = t0+1 .. t0+nsteps (t0 = steps already taken). */
int or_step(or_sim *s, uint32_t nsteps);
int or_get_state(or_sim *s, double *curpos, double *vel, double *acc, double *force);
int or_get_disp(or_sim *s, double *disp);
/* applied_force_density of every node (N*3; zero outside the prescribed-velocity particle and
 * before the constraint is first applied), timeloop.h:760-764. */
int or_get_afd(or_sim *s, double *afd);
int or_get_connectivity(or_sim *s, uint32_t particle, uint32_t *pairs, uint64_t cap,
                        uint64_t *n);
int or_get_wall(or_sim *s, double *wall_info, double *reaction);
int or_get_aabb(or_sim *s, double *lrtb);
/* counts[0] = pairwise computations of the last step, counts[1] = node contacts applied
 * in the last step, counts[2] = live directed bonds at the start of the last step,
 * counts[3] = step counter. */
int or_get_counts(or_sim *s, uint64_t *counts);
/* Stretch of every live bond of a particle from the last force evaluation, in NbdArr
 * order (row i ascending, neighbours ascending); returns the count. */
uint64_t or_get_stretch(or_sim *s, uint32_t particle, double *out, uint64_t cap);
int or_set_state(or_sim *s, const double *disp, const double *vel, const double *acc);
int or_set_connectivity(or_sim *s, uint32_t particle, const uint32_t *pairs, uint64_t n);
void or_destroy(or_sim *s);

#ifdef __cplusplus
}
#endif
#endif

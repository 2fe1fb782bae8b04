/* cube_gen.h -- the 3D P1 diffusion workload's hierarchy built on the oracle
 * side (cube_gen.c), so that the oracle and the CPU baseline need nothing
 * from the ug_gb300 library.  TEST INFRASTRUCTURE ONLY. */
#ifndef ORC_CUBE_GEN_H
#define ORC_CUBE_GEN_H
#include "lmgc_oracle.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_cube orc_cube;
/* unit cube, six Kuhn tetrahedra refined nref (0..8) times, k = exp(g) with
 * (seed, corr, var) (var = 0: k = 1), right-hand side from seed; the field is
 * evaluated on nthreads threads (the result does not depend on it) */
int orc_cube_create(int nref, unsigned long long seed, double corr, double var, int nthreads, orc_cube **out);
/* the same with the refinement rule: 0 = the Freudenthal triangulation
 * (orc_cube_create), 1 = UG's red rules with the shortest interior diagonal
 * (nref 0..7) */
int orc_cube_create_rule(int rule, int nref, unsigned long long seed, double corr, double var, int nthreads,
                         orc_cube **out);
/* level l (0..nref) as an orc_level (arrays owned by the generator) and its
 * node coordinates (3 per node) */
int orc_cube_level(const orc_cube *c, int l, orc_level *out, const double **xyz);
/* right-hand side of the finest level */
const double *orc_cube_rhs(const orc_cube *c, int *len);
void orc_cube_destroy(orc_cube *c);

#ifdef __cplusplus
}
#endif
#endif

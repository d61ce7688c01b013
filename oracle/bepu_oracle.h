// Oracle C API -- test infrastructure only.
//
// A single-threaded (and, for the CPU baseline, a multithreaded) C++
// restatement of the reference's velocity solver and integration step.  Only
// the tests, the smoke check and the CPU-baseline legs of bench.py load it;
// the product library never links it.
#pragma once
#include <stdint.h>
#include "../include/bepugpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_space oracle_space;

/* Order modes of the solver list. */
#define ORACLE_ORDER_PERMUTED 0  /* PermutationMapper order, Solver.cs:255-260 */
#define ORACLE_ORDER_IDENTITY 1  /* identity mapping over the list as given */

oracle_space* oracle_create(const bepugpu_settings* settings,
                            const bepugpu_body* bodies, int32_t body_count,
                            const bepugpu_manifold* manifolds, int32_t manifold_count,
                            const bepugpu_joint* joints, int32_t joint_count);
void oracle_destroy(oracle_space* s);
/* Puts the solver list (joints first, then manifolds, in array order) into the
 * given order: list[i] = updateable order[i]. */
int32_t oracle_set_list_order(oracle_space* s, const int32_t* order, int32_t count);
void oracle_set_order_mode(oracle_space* s, int32_t mode, int64_t permutation_index);
/* One Space step of the flagged stages (BEPUGPU_STEP_*), single-threaded. */
int32_t oracle_step(oracle_space* s, float dt, uint32_t flags, int32_t steps);
/* The same with Solver.UpdateMultithreaded and multithreaded force/position
 * stages on `threads` worker threads. */
int32_t oracle_step_multithreaded(oracle_space* s, float dt, uint32_t flags, int32_t steps,
                                  int32_t threads);
/* One shape per body, for manifolds flagged BEPUGPU_MANIFOLD_GENERATED. */
int32_t oracle_set_shapes(oracle_space* s, const bepugpu_shape* shapes, int32_t count);
/* Simulation islands as bepugpu_set_islands takes them; count 0 clears them. */
int32_t oracle_set_islands(oracle_space* s, const int32_t* island_of, const uint32_t* flags, int32_t count,
                           int32_t deactivation_index);
int32_t oracle_get_islands(oracle_space* s, uint32_t* flags, int32_t count, int32_t* deactivation_index);
void oracle_get_bodies(oracle_space* s, bepugpu_body* out);
void oracle_get_constraints(oracle_space* s, bepugpu_manifold* manifolds, bepugpu_joint* joints);
/* Counts of solves executed by the last step (manifold-children and joints). */
int64_t oracle_last_child_solves(oracle_space* s);

/* PermutationMapper (BEPUutilities/PermutationMapper.cs:27-44,113-127). */
int64_t oracle_permutation_map(int64_t permutation_index, int64_t index, int32_t set_size);
int32_t oracle_prime_count(void);
/* PermutationTestDemo's check: the first permutation index whose mapping is not
 * a permutation of [0, set_size), or -1; *distinct: different permutations seen. */
int64_t oracle_permutation_check(int64_t iterations, int32_t set_size, int64_t* distinct);

/* Restatement of the library's deterministic greedy colouring: returns the
 * colour count, or -1 on error. */
int32_t oracle_colour(const bepugpu_body* bodies, int32_t body_count,
                      const bepugpu_manifold* manifolds, int32_t manifold_count,
                      const bepugpu_joint* joints, int32_t joint_count,
                      int32_t* colour_out, int32_t* order_out);

#ifdef __cplusplus
}
#endif

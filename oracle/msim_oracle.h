/*
 * msim_oracle.h - CPU oracle for the movement-sim per-tick path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * GLSL (src/sim/shader/random_move.comp) used to check the CUDA path; it is
 * loaded only by the tests, by the smoke check and by the CPU-baseline leg of
 * bench.py.  The product never links or calls it.
 *
 * Parity pins (see tests/test_oracle.py):
 *  - xorshift128 reproduces the first outputs of Marsaglia's published xor128
 *    sequence (x,y,z,w = 123456789, 362436069, 521288629, 88675123);
 *  - PCG32 reproduces the published pcg32 demo sequence (seed 42, sequence 54);
 *  - the radius predicate matches the reference's own CPU quad tree
 *    (shader_validation/src/main.cpp, built by oracle/build_oracle.py into
 *    oracle/_ref) on random entity sets and on its known-answer test
 *    run_collision_detection_test_1 (main.cpp:1137-1199);
 *  - road choices on test_map.json are checked against hand-derived values.
 * The move step itself has no reference CPU code: its parity with the Vulkan
 * shader is unpinned (the shader cannot run without a graphics stack).
 */
#ifndef MSIM_ORACLE_H
#define MSIM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* xorshift128, random_move.comp:725-736; s = uvec4 (x, y, z, w). */
uint32_t oracle_xs128_next(uint32_t s[4]);
/* PCG-XSH-RR 64/32; s = {state_lo, state_hi, inc_lo, inc_hi}. */
uint32_t oracle_pcg32_next(uint32_t s[4]);
/* pcg32_srandom_r(initstate, initseq) */
void oracle_pcg32_seed(uint32_t s[4], uint64_t initstate, uint64_t initseq);
/* random_move.comp:738-741 next_float */
float oracle_next_float(uint32_t u);
/* random_move.comp:743-746 ranged next, on an already drawn u */
uint32_t oracle_ranged(uint32_t u, uint32_t lo, uint32_t hi);
/* n draws of generator `kind` (0 xorshift128, 1 pcg32); state updated. */
void oracle_rng_seq(uint32_t kind, uint32_t s[4], uint32_t n, uint32_t* out);

/* Counter-based draws used by every deterministic initializer. */
uint64_t oracle_splitmix64(uint64_t x);
uint64_t oracle_draw(uint64_t seed, uint64_t stream, uint64_t i);

/* Deterministic entity initializer (replaces Simulator.cpp:114-129 and
 * Entity.cpp:44-49).  placement 0: pos = road.start; 1: start + u*(end-start). */
void oracle_init_entities(uint32_t num_roads, const float* road_pos, uint32_t n, uint32_t rng_kind,
                          uint64_t seed, uint32_t placement, float speed_min, float speed_max,
                          float* pos, uint32_t* heading, uint32_t* rng, float* speed);

/* Synthetic L x L lattice road map of the workloads (see msim_oracle.c for the
 * rules); NULL on bad arguments or a lattice without edges. */
typedef struct oracle_lattice oracle_lattice;
oracle_lattice* oracle_lattice_new(uint32_t side, uint64_t seed, float spacing, float jitter, float keep_prob);
void oracle_lattice_info(const oracle_lattice* m, uint32_t* num_roads, uint32_t* num_conn, float* width,
                         float* height);
void oracle_lattice_copy(const oracle_lattice* m, float* road_pos, uint32_t* road_conn, uint32_t* conn);
void oracle_lattice_free(oracle_lattice* m);

/* `ticks` move ticks of random_move.comp:830-852 (+ new_target 778-828) over all
 * n entities.  factor may be NULL (1.0).  threads <= 0 -> 1. */
void oracle_step(uint32_t num_roads, const float* road_pos, const uint32_t* road_conn,
                 uint32_t num_conn, const uint32_t* conn, uint32_t n, uint32_t rng_kind, float dt,
                 const float* factor, uint32_t ticks, float* pos, uint32_t* heading, uint32_t* rng,
                 const float* speed, int threads);

/* Radius neighbour sets with the predicate of random_move.comp:551-562.
 * count[i] = all j != i in range; idx[i*cap ..] = the min(count, cap) smallest j
 * ascending, then 0xffffffff.  idx may be NULL.  Returns the pair count (j < i). */
uint64_t oracle_neighbours(uint32_t n, const float* pos, float radius, uint32_t cap,
                           uint32_t* count, uint32_t* idx, int threads);

/* Density calibration, FP64 reference of the loss and its gradient.  The FP32 move
 * step (as oracle_step, from pos0/head0/rng0) gives the event schedule (ticks at
 * which an entity snaps to its road end, and its road choices) and, unless
 * fp64_model, the trajectory p_t; with fp64_model the trajectory follows that
 * schedule in FP64 (p_t = p_{t-1} + (d/|d|) * speed*factor*dt, d = target -
 * p_{t-1}; p_t = target at an event), a smooth model for finite differences.
 * D = (1/ticks) sum_t splat(p_t) (bilinear, cell-centred, gw x gh cells over
 * [0,W) x [0,H); for the FP32 trajectory the cell coordinate u = x*gw/W - 1/2 is
 * formed in binary32 and truncated to fbits fraction bits, fbits the largest value
 * in 16..22 with |u| * 2^fbits < 2^30), loss = mean_g (D_g - target_g)^2, both in
 * FP64; the gradient is
 * the FP64 adjoint of the step about the trajectory with the events held fixed.
 * Writes density (may be NULL), grad_speed[n], grad_factor[num_roads] and, when
 * sched is not NULL, the event schedule (bit t-1 of word (t-1)/32 of entity i's
 * ceil(ticks/32) words set when i snaps at tick t); returns the loss. */
double oracle_density_adjoint(uint32_t num_roads, const float* road_pos, const uint32_t* road_conn,
                              uint32_t num_conn, const uint32_t* conn, uint32_t n, uint32_t rng_kind, float dt,
                              uint32_t ticks, const float* pos0, const uint32_t* head0, const uint32_t* rng0,
                              const float* speed, const float* factor, float world_w, float world_h, uint32_t gw,
                              uint32_t gh, const float* target, double* density, double* grad_speed,
                              double* grad_factor, int fp64_model, uint32_t* sched, int threads);

/* The single predicate, for tests. */
int oracle_in_range(float ax, float ay, float bx, float by, float radius);

#ifdef __cplusplus
}
#endif

#endif

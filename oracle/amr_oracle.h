/*
 * ORACLE — test infrastructure, not the product.
 *
 * A plain-C restatement of the gpu-amr reference algorithm for the hot path:
 * Morton ids, the ndtree refine/coarsen cycle with its incremental neighbour
 * bookkeeping, the face halo exchange, the Rusanov/forward-Euler update and the
 * CFL time step.  Every function cites the reference file:line it restates.
 * It is the checker for the CUDA path and the timed CPU baseline; only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 *
 * Parity pinned: the restatement is checked against golden dumps of the real
 * reference (oracle/ref_driver.cpp compiled from the reference's own headers,
 * fixtures in tests/golden/).
 */
#ifndef AMR_ORACLE_H
#define AMR_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_tree oracle_tree;

/* One neighbour entry per (leaf, direction); direction = 2*dim + positive,
 * dim 0 = slowest layout index (neighbor.hpp:103-255). kind: 0 none, 1 same,
 * 2 finer, 3 coarser (neighbor.hpp:22-100). */
typedef struct oracle_neighbor {
    uint8_t  kind;
    uint8_t  quadrant[3];
    uint32_t pad;
    uint64_t ids[4];
} oracle_neighbor;

/* rank 2|3, n cells per dim (even, >= 2*halo), halo width, Morton depth. */
oracle_tree* oracle_create(int rank, int n, int halo, int depth, size_t capacity);
/* The same with nvar fields per cell (the reference's SoA field tuple,
 * e.g. EulerCell2D = Rho, Rhou, Rhov, E2D); state layout per patch:
 * nvar padded patches, field-major. */
oracle_tree* oracle_create_fields(int rank, int n, int halo, int depth, size_t capacity, int nvar);
int          oracle_nvar(const oracle_tree* t);
void         oracle_destroy(oracle_tree* t);

size_t oracle_size(const oracle_tree* t);
size_t oracle_flat(const oracle_tree* t);
void   oracle_get_ids(const oracle_tree* t, uint64_t* out);
void   oracle_get_neighbors(const oracle_tree* t, oracle_neighbor* out);
void   oracle_get_state(const oracle_tree* t, double* out);        /* size*nvar*flat */
void   oracle_set_state(oracle_tree* t, const double* in);          /* size*nvar*flat */

/* Tree operations. reconstruct returns 0, or a negative code where the
 * reference would stop (e.g. coarsening into the root, ndtree.hpp:1106). */
int  oracle_reconstruct(oracle_tree* t, const int8_t* flags);
void oracle_refine_all(oracle_tree* t, int levels);
void oracle_halo_exchange(oracle_tree* t);

/* Criteria (write one int8 per leaf: 0 Stable, 1 Refine, 2 Coarsen). */
void oracle_flags_gradient(const oracle_tree* t, double rthr, double cthr,
                           int min_level, int max_level, int8_t* out);
void oracle_flags_max(const oracle_tree* t, double rthr, double cthr,
                      int min_level, int max_level, int8_t* out);
void oracle_flags_random(const oracle_tree* t, uint64_t seed, uint64_t pass,
                         double p_refine, double p_coarsen, int min_level,
                         int max_level, int8_t* out);

/* Initial data: sum of Gaussians (bumps: rank centre coords, sigma, amplitude
 * per bump) plus seeded uniform noise in [-noise, noise]. */
void oracle_init_state(oracle_tree* t, const double* bumps, int nbumps,
                       double noise, uint64_t noise_seed);
void oracle_random_state(oracle_tree* t, uint64_t seed);

/* CFL time step and forward-Euler advance (amr_solver.hpp:221-242, 355-413). */
double oracle_compute_dt(const oracle_tree* t, const double* velocity, double cfl);
double oracle_advance(oracle_tree* t, size_t steps, const double* velocity,
                      double cfl, double remaining, size_t* executed);
/* SSPRK2 / SSPRK3 steps of the FV advection operator (see amr_oracle.c). */
double oracle_ssprk_advance(oracle_tree* t, size_t steps, int order, const double* v, double cfl, double remaining,
                            size_t* executed);
/* Domain lengths per Morton axis (physics_system's Domain_Sizes; default 1). */
void oracle_set_lengths(oracle_tree* t, const double* lengths);

/* Euler physics (EulerPhysics<DIM>, nvar = rank + 2 fields): the CFL step
 * (compute_time_step_cpu x cfl), advance_batch_async (CPU branch; dts, if
 * not NULL, receives the executed step sizes) and the acoustic-pulse
 * initial state of the reference's Euler benchmark. */
double oracle_euler_dt(const oracle_tree* t, double gamma, double cfl);
double oracle_euler_advance(oracle_tree* t, size_t steps, double gamma, double cfl, double remaining,
                            size_t* executed, double* dts);
void   oracle_euler_init_pulse(oracle_tree* t, double gamma, double rho_bg, double p_bg, double amplitude,
                               double width_sq, const double* centre);

/* vtk_print::print of the current tree and state (legacy binary VTK, one
 * quad/voxel per interior cell); field = the scalar's name.  0 on success. */
int oracle_write_vtk(const oracle_tree* t, const char* path, const char* fields); /* names, comma-separated */

/* Gradient of <lam_T, u_T> w.r.t. the interior of u_0 for oracle_advance on
 * the current (frozen) mesh: transposed steps in reverse order (size*flat
 * padded buffers; ghost entries of lam_0 are zero).  Returns executed steps. */
size_t oracle_adjoint(oracle_tree* t, size_t steps, const double* velocity, double cfl, double remaining,
                      const double* lam_T, double* lam_0);

/* Hash shared by oracle, fixtures and product initialiser. */
double oracle_unit_hash(uint64_t a, uint64_t b, uint64_t c);

/* Morton helpers (morton_id.hpp:21-450). */
uint64_t oracle_encode(int rank, int depth, const uint32_t* coords, int level);
void     oracle_decode(int rank, uint64_t id, uint32_t* coords, int* level);
uint64_t oracle_child_of(int rank, int depth, uint64_t id, int offset);
uint64_t oracle_parent_of(int rank, int depth, uint64_t id);

void oracle_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif

/*
 * gb300-amr — C ABI of the GB300-native (sm_103a) hot path of gpu-amr:
 * the per-leaf-patch finite-volume update over the Morton-ordered ndtree, the
 * face halo exchange with coarse-fine prolongation/restriction, and the
 * refine/coarsen cycle (flagging, 2:1 balance, Morton order, compaction).
 *
 * All functions return an amr_status (0 = success).  Pointers named `device_*`
 * are CUDA device pointers; `host_*` are host pointers.  `stream` is a
 * cudaStream_t passed as void* (NULL = legacy default stream).  No torch or
 * C++ types cross this boundary.
 *
 * Layout contract (identical to the reference's patch<double, padded_layout>):
 * one leaf = one padded patch of (n + 2*halo)^rank cells, row-major, layout
 * dimension 0 slowest, physical x on the last (fastest) index; patches are
 * contiguous, patch-major, in Morton order.
 */
#ifndef AMR_GB300_H
#define AMR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum amr_status {
    AMR_OK                = 0,
    AMR_ERR_INVALID       = 1, /* bad argument or size */
    AMR_ERR_CUDA          = 2, /* a CUDA call failed; see amr_last_error() */
    AMR_ERR_CAPACITY      = 3, /* a re-mesh would exceed the tree capacity */
    AMR_ERR_UNBALANCED    = 4, /* neighbour rebuild met a non-2:1 configuration */
    AMR_ERR_UNSUPPORTED   = 5, /* rank/size combination not built */
    AMR_ERR_NO_DEVICE     = 6,
    AMR_ERR_TIMEOUT       = 7  /* a bounded device-side wait gave up; results are invalid */
} amr_status;

typedef enum amr_dtype { AMR_F64 = 0, AMR_F32 = 1 } amr_dtype;

/* Neighbour relation per (leaf, direction); direction = 2*dim + positive with
 * dim 0 the slowest layout index.  Same memory layout as the reference's
 * amr::cuda::halo_direction_metadata (include/cuda/halo_exchange.hpp:19-26):
 * relation 0 none, 1 same, 2 finer, 3 coarser. */
typedef struct amr_halo_meta {
    int32_t neighbor;
    int32_t finer_ids[4];
    int32_t quadrant[3];
    int8_t  relation;
    int8_t  padding[3];
} amr_halo_meta;

/* Reference-compatible launch configuration for the free-function entry
 * points (include/cuda/halo_exchange.hpp:28-40, intergrid_transfer.hpp:17-26,
 * fvm_time_step.hpp:9-27), reduced to what the kernels need. */
typedef struct amr_patch_geometry {
    int32_t rank;      /* 2 or 3 */
    int32_t n;         /* interior cells per dimension (even, >= 2*halo) */
    int32_t halo;      /* ghost layers */
    int32_t depth;     /* Morton depth of the patch index (morton_id<Depth,Rank>) */
    double  lengths[3];/* physical domain lengths per Morton axis x, y, z */
} amr_patch_geometry;

/* Reference intergrid_transfer_task_metadata (intergrid_transfer.hpp:11-15). */
typedef struct amr_transfer_task {
    int32_t source_patch;
    int32_t destination_patch;
} amr_transfer_task;

/* ------------------------------------------------------------------ info */
const char* amr_last_error(void);
int         amr_version(void);

/* ---------------------------------------------- free-function drop-ins
 * Each replaces one amr::cuda:: launcher of the reference; they operate on
 * caller-owned device buffers with the reference layout. */

/* Replaces amr::cuda::halo_exchange_scalar_patches_inplace
 * (include/cuda/halo_exchange.hpp:42-47; src/cuda/halo_exchange.cu:351-403):
 * fills every face ghost cell of `num_patches` patches from `meta`
 * (num_patches * 2*rank records).  Corners are left untouched. */
amr_status amr_halo_exchange_f64(double* device_patches, const amr_halo_meta* device_meta,
                                 size_t meta_count, size_t num_patches,
                                 const amr_patch_geometry* geom, void* stream);
amr_status amr_halo_exchange_f32(float* device_patches, const amr_halo_meta* device_meta,
                                 size_t meta_count, size_t num_patches,
                                 const amr_patch_geometry* geom, void* stream);

/* Replace interpolate_scalar_patches_inplace / restrict_scalar_patches_inplace
 * (include/cuda/intergrid_transfer.hpp:28-42): for each task, copy the parent
 * at source_patch into the 2^rank children starting at destination_patch
 * (piecewise constant), or average the 2^rank children starting at
 * source_patch into the parent at destination_patch. */
amr_status amr_interpolate_patches_f64(double* device_patches, const amr_transfer_task* device_tasks,
                                       size_t task_count, const amr_patch_geometry* geom, void* stream);
amr_status amr_restrict_patches_f64(double* device_patches, const amr_transfer_task* device_tasks,
                                    size_t task_count, const amr_patch_geometry* geom, void* stream);

/* Replaces permute_patches_inplace_batch's gather (include/cuda/permutation.hpp:10-17):
 * dst[i] = src[sources[i]] for whole patches of patch_bytes bytes (out of place). */
amr_status amr_gather_patches(void* device_dst, const void* device_src, size_t patch_bytes,
                              const int32_t* device_sources, size_t count, void* stream);

/* Replaces launch_compute_dt_kernel_device + launch_finalize_step_dt
 * (include/cuda/fvm_time_step.hpp:39-58) for linear advection: raw dt =
 * min over leaves and axes of dx/|v|, step dt = cfl*raw clamped to the
 * remaining time; accumulates into *device_dt_accumulator and counts the
 * step in *device_step_count when the step dt is positive. */
amr_status amr_compute_step_dt(const int32_t* device_levels, size_t num_patches,
                               const amr_patch_geometry* geom, const double* velocity3, double cfl,
                               double* device_dt, double* device_dt_accumulator,
                               double* device_remaining_time, uint32_t* device_step_count,
                               void* stream);

/* Replaces launch_time_step_kernel_with_device_dt<AdvectionPhysics,DIM>
 * (include/cuda/fvm_time_step.hpp:30-37): one forward-Euler Rusanov step of
 * linear advection with velocity `velocity3`, reading the face ghosts the
 * caller filled, writing the interior of device_out. */
amr_status amr_time_step_f64(const double* device_in, double* device_out,
                             const int32_t* device_levels, size_t num_patches,
                             const amr_patch_geometry* geom, const double* velocity3,
                             const double* device_dt, void* stream);

/* Replaces compute_scalar_patch_amr_decisions_from_device
 * (include/cuda/fvm_refinement_criterion.hpp:20-27): per patch, Refine (1) if
 * the maximum exceeds refine_threshold and level < max_level, Coarsen (2) if
 * it is below coarsen_threshold and level > min_level, else Stable (0).  The
 * maximum runs over interior and face-ghost cells. */
amr_status amr_flags_max_f64(const double* device_patches, const int32_t* device_levels,
                             size_t num_patches, const amr_patch_geometry* geom,
                             double refine_threshold, double coarsen_threshold, int min_level,
                             int max_level, int8_t* device_flags, void* stream);

/* ------------------------------------------------- device-resident tree
 * The GB300-native core behind the ndtree / amr_solver API: state, Morton
 * ids, levels and neighbour tables live in HBM; the whole refine/coarsen
 * cycle runs on the device. */
typedef struct amr_tree amr_tree;

typedef struct amr_tree_desc {
    amr_patch_geometry geom;
    size_t             capacity;  /* maximum number of leaves (all instances) */
    int32_t            dtype;     /* amr_dtype of the cell state */
    void*              stream;    /* cudaStream_t for every call on this tree */
    int32_t            instances; /* independent trees held together (a forest);
                                     0 or 1 = one tree */
    int32_t            fields;    /* state fields per cell (the cell type's SoA
                                     tuple; Euler: rank + 2; DG: 16); 0 or 1 =
                                     one, at most 16 */
} amr_tree_desc;

/* ndtree(capacity) (include/ndtree/ndtree.hpp:320-425): one root leaf with
 * periodic self-neighbours.  With instances = K > 1 the object holds K
 * independent trees (a forest): instance i starts as its own root, every
 * Morton id carries i above its interleaved coordinate bits
 * (id = i << (6 + rank*depth) | morton id within the instance), so the leaves
 * of all instances form one Morton-ordered array, instance by instance, and
 * each instance has its own periodic domain, neighbour tables, 2:1 balance,
 * CFL step and level bounds.  Every call below acts on all instances. */
amr_status amr_tree_create(const amr_tree_desc* desc, amr_tree** out);
amr_status amr_tree_destroy(amr_tree* t);
/* ndtree::size() */
amr_status amr_tree_size(const amr_tree* t, size_t* out);
/* Change the capacity (the maximum number of leaves) keeping the leaves,
 * their state, ids, levels, neighbour tables and flags; new_capacity must
 * hold the current leaves.  Device buffers move, so pointers from
 * amr_tree_device_state taken before the call are invalid after it. */
amr_status amr_tree_reserve(amr_tree* t, size_t new_capacity);
amr_status amr_tree_capacity(const amr_tree* t, size_t* out);
/* Flat cell count of one padded patch. */
amr_status amr_tree_patch_cells(const amr_tree* t, size_t* out);

/* State transfer, the reference's sync_current_{to,from}_device
 * (ndtree.hpp:583-613); host layout = size() padded patches in Morton order,
 * elements of the tree's dtype; with several fields, field by field (the
 * reference's SoA buffers: fields x size() x padded patch). */
amr_status amr_tree_upload_state(amr_tree* t, const void* host_state, size_t num_patches);
amr_status amr_tree_download_state(amr_tree* t, void* host_state, size_t num_patches);
/* Device-to-device state load and copy-out (same layout as upload_state). */
amr_status amr_tree_load_state_device(amr_tree* t, const void* device_state, size_t num_patches);
amr_status amr_tree_download_state_device(amr_tree* t, void* device_dst, size_t num_patches);
/* Back to the freshly constructed tree: one root leaf, periodic
 * self-neighbours, zero state (ndtree::ndtree, ndtree.hpp:320-425),
 * without reallocating. */
amr_status amr_tree_reset(amr_tree* t);
/* Device pointers of the current/next state buffers (get_device_buffer). */
amr_status amr_tree_device_state(amr_tree* t, void** current, void** next);

/* Topology readback: Morton ids (get_node_index_at), levels, neighbour tables. */
amr_status amr_tree_get_ids(const amr_tree* t, uint64_t* host_ids, size_t num_patches);
amr_status amr_tree_get_levels(const amr_tree* t, int32_t* host_levels, size_t num_patches);
amr_status amr_tree_get_neighbors(const amr_tree* t, amr_halo_meta* host_meta, size_t num_patches);

/* ndtree::halo_exchange_update (ndtree.hpp:1862-1877). */
amr_status amr_tree_halo_exchange(amr_tree* t);

/* Refinement flags: ndtree::update_refine_flags (ndtree.hpp:886-902). */
amr_status amr_tree_flags_gradient(amr_tree* t, double refine_threshold, double coarsen_threshold,
                                   int min_level, int max_level);
amr_status amr_tree_flags_max(amr_tree* t, double refine_threshold, double coarsen_threshold,
                              int min_level, int max_level);
amr_status amr_tree_set_flags(amr_tree* t, const int8_t* host_flags, size_t num_patches);
amr_status amr_tree_get_flags(const amr_tree* t, int8_t* host_flags, size_t num_patches);

/* ndtree::reconstruct_tree after the flags are set (ndtree.hpp:1249-1271):
 * 2:1 balance, refinement (prolongation), coarsening (restriction), Morton
 * order and neighbour tables, all on the device.  *changed (optional) tells
 * whether the topology changed. */
amr_status amr_tree_remesh(amr_tree* t, int* changed);
/* Uniform refinement, `levels` times (reconstruct_tree with refine-all). */
amr_status amr_tree_refine_uniform(amr_tree* t, int levels);

/* amr_solver::advance_batch_async / finish_advance_batch
 * (include/solver/amr_solver.hpp:155-262) for linear advection with constant
 * velocity: `steps` forward-Euler Rusanov steps, each with dt = cfl * min(dx/|v|)
 * clamped to the remaining time.  Face ghosts are produced on the fly from
 * neighbour patches, so no halo pass runs between steps; call
 * amr_tree_halo_exchange before reading ghost cells. */
amr_status amr_tree_advance(amr_tree* t, size_t steps, const double* velocity3, double cfl,
                            double remaining_time);
amr_status amr_tree_finish_advance(amr_tree* t, double* sum_dt, size_t* executed_steps);

/* The reference benchmark loop (benchmark/bench_fvm_solver_integration_
 * active_amr.b.cpp:220-250) as one call: repeat { advance
 * min(remesh_interval, steps left) steps with remaining time
 * remaining_time - (time advanced so far); flag with the criterion; re-mesh }
 * until `steps` steps ran or the time is used up.  criterion: 0 none (no
 * re-mesh), 1 gradient (amr_tree_flags_gradient), 2 max value
 * (amr_tree_flags_max).  While the tree has few leaves the whole loop runs as
 * one persistent kernel on a thread-block cluster with no host round trip.
 * Larger trees and forests run interval by interval: the interval (step
 * coefficients, the update steps, flags, 2:1 balance, re-mesh, neighbour
 * rebuild) is one CUDA graph whose kernels read the leaf count and the
 * buffer selection from device memory, captured once and replayed with no
 * host round trip between intervals (AMR_RUN_NO_GRAPH: host-driven launches
 * with a readback per re-mesh).  On FP32 forests of 16x16 patches whose every
 * instance is uniform at a level >= 2, an interval of 10 steps with the
 * gradient criterion (or none) runs its steps and flags in one kernel over
 * 4x4-patch blocks (AMR_RUN_NO_FUSED: multi-step passes and a separate flag
 * kernel instead; AMR_RUN_FUSED: the fused kernel even where the
 * environment turns it off).  Results are identical on every path. */
typedef struct amr_cycle_params {
    uint64_t steps;
    uint64_t remesh_interval;
    double   velocity[3];
    double   cfl;
    double   remaining_time;
    int32_t  criterion;
    int32_t  min_level;
    int32_t  max_level;
    int32_t  options;        /* AMR_RUN_PER_LAUNCH: never use the cluster kernel;
                                AMR_RUN_INSTANCE_PARAMS: per-instance velocities
                                and bounds (amr_tree_set_instance_params);
                                AMR_RUN_NO_GRAPH: host-driven intervals instead
                                of the captured interval graph;
                                AMR_RUN_NO_FUSED / AMR_RUN_FUSED: without / with
                                the fused interval kernel;
                                bits 8-15: cluster size (CTAs) to use, 0 = largest that fits */
    double   refine_threshold;
    double   coarsen_threshold;
} amr_cycle_params;

#define AMR_RUN_PER_LAUNCH 1
#define AMR_RUN_INSTANCE_PARAMS 2
#define AMR_RUN_NO_GRAPH 4
#define AMR_RUN_NO_FUSED 8
#define AMR_RUN_FUSED 16

typedef struct amr_cycle_stats {
    uint64_t executed_steps;   /* steps with dt > 0 */
    double   sum_dt;
    uint64_t cell_updates;     /* sum over intervals of executed x leaves x n^rank */
    uint64_t remeshes;
    uint64_t intervals;
    uint64_t leaves_min;       /* leaf counts at interval starts */
    uint64_t leaves_max;
    double   leaves_mean;
    uint64_t persistent_intervals; /* intervals run inside the cluster kernel */
    uint64_t graph_intervals;      /* intervals run as graph replays */
    uint64_t remeshes_changed;     /* re-meshes that changed the tree */
} amr_cycle_stats;

amr_status amr_tree_run(amr_tree* t, const amr_cycle_params* params, amr_cycle_stats* stats);

/* Strong-stability-preserving Runge-Kutta steps of linear advection: the
 * reference's SSPRK2 / SSPRK3 integrators (include/dg_helpers/
 * time_integration/time.hpp:83-272, driven with a halo exchange before every
 * stage as include/dg_helpers/solver.hpp:162-244 does) on the FV residual
 * -sum_d (F_R - F_L) / dx_d with the Rusanov flux of AdvectionPhysics.  The
 * step size is amr_tree_advance's (CFL from the finest level, clamped to the
 * remaining time); a one-field FP64 tree; velocity3 NULL = the per-instance
 * velocities.  As in the reference, every stage combines whole padded
 * patches and no halo exchange follows the last stage, so a criterion
 * evaluated after the advance reads the combined ghost cells.  States are
 * bit-identical to the reference's CPU path.  Use amr_tree_finish_advance
 * for the simulated time and executed steps. */
amr_status amr_tree_advance_ssprk(amr_tree* t, size_t steps, int order, const double* velocity3, double cfl,
                                  double remaining_time);

/* ------------------------------------------------------------- DG
 * Nodal discontinuous-Galerkin steps of the reference's DG patch solver
 * (include/dg_helpers: DGSolver::advance_patches, solver.hpp:162-244, with
 * RHSEvaluator::evaluate, rhs.hpp:117-255, and SSPRK2, time.hpp:134-168) in
 * its generated configuration (include/config/generated_config.hpp): order
 * 2, 2D, 4 x 4 cells per patch with one ghost cell, four advected variables
 * per node, velocity 1, Courant number 0.5.  The tree holds the 16 nodal
 * values of a cell as 16 FP64 fields (field = node * 4 + variable, node =
 * x-node * 2 + y-node); create it with rank 2, n 4, halo 1, 16 fields
 * (depth 6 is the reference's MaxDepth).  Each step: halo exchange (same-
 * level copies; across coarse-fine faces the DG restriction or
 * interpolation of amr_tree_dg_remesh's policy), the first stage,
 * halo exchange, the second stage; no halo exchange follows the last stage
 * (the ghost cells hold the stage combination, as the reference's tree
 * does).  *dt: on entry the step size of the first step (the reference's
 * initial_dt for a new run), on return the next one; each step then takes
 * dt = min(dt, 0.1 x finest cell edge), the reference's CFL rule for this
 * order (1 / (order^dim + 1) x Courant x edge / |v|).  *time (optional)
 * then grows by that updated step size, as in the reference's loop
 * (dt = min(dt, dt_min); time += dt: after k steps it has grown by the
 * sizes of steps 2..k+1).  Interior states are bit-identical to
 * the reference's CPU path. */
amr_status amr_tree_dg_advance(amr_tree* t, size_t steps, double* dt, double* time);

/* DGSolver::apply_amr (solver.hpp:249-310) on such a tree:
 * GradientAMRIndicator::compute_patch_decisions (include/dg_helpers/
 * globals/amr_indicators.hpp:86-225: per cell the largest nodal range of
 * variables 0..1 over |mean of variable 2| + 1e-10; refine if a cell exceeds
 * refine_threshold, coarsen if every cell is below coarsen_threshold), then
 * the re-mesh of amr_tree_remesh with the tree's DG policy
 * (tree_builder.hpp:59-289): refined cells interpolate the parent cell's
 * polynomial at their nodes, coarsened cells take the polynomial of the
 * child holding each node.  The halo of amr_tree_dg_advance applies the same
 * operators across coarse-fine faces.  *changed (optional) = 1 if the tree
 * changed. */
amr_status amr_tree_dg_remesh(amr_tree* t, double refine_threshold, double coarsen_threshold, int* changed);

/* DGSolver::run (solver.hpp:109-151) without its VTK output: from time 0,
 * step size initial_dt for the first step, steps while time < end_time,
 * after step k >= next (next = 0 at the start) a re-mesh and next = k +
 * amr_interval (0: a re-mesh after every step, as in the reference).
 * stats: steps, re-meshes, the reference's
 * processed-cell count (leaves x 16 per step), final time and next step
 * size, largest leaf count. */
typedef struct amr_dg_stats {
    uint64_t steps, remeshes, cells, leaves_max;
    double   time, next_dt;
} amr_dg_stats;
amr_status amr_tree_dg_run(amr_tree* t, double initial_dt, double end_time, int amr_interval,
                           double refine_threshold, double coarsen_threshold, amr_dg_stats* stats);

/* The equation of the DG tree, the reference's compile-time
 * GlobalConfigPolicy::equation (include/config/generated_config.hpp,
 * include/dg_helpers/equations/): AMR_DG_ADVECTION (the default; linear
 * advection, velocity 1 in both directions, the 4 variables independent) or
 * AMR_DG_EULER (include/dg_helpers/equations/euler.hpp: variables
 * [rho u, rho v, rho, E] per node, gamma 1.4).  With Euler the Rusanov speed
 * of a face is the patch's running maximum, in the reference's loop order,
 * of max(eigenvalue of the cell, of the neighbour) (|u_n| + sqrt(gamma p /
 * rho) at the cell's first node), and each step's CFL step comes from every
 * patch's final speed (0.1 x edge / lambda, solver.hpp:227-234), computed on
 * the device: amr_tree_dg_advance reads the step size back once per call.
 * amr_tree_dg_advance, amr_tree_dg_remesh and amr_tree_dg_run apply the
 * setting; states are bit-identical to the reference's CPU path. */
/* The reference's DG printer (ndt::print::dg_tree_printer_2d::print,
 * include/ndtree/print_dg_tree_v2.hpp:145-370) for the tree's current
 * leaves and DG state, written to `path` (the reference builds the name
 * vtk_output/DG_<equation>_ord2_<integrator><suffix> itself): a legacy
 * binary big-endian unstructured grid with one VTK Lagrange quadrilateral
 * (type 70) per interior cell, its 9 points at xi, eta in {0, 1/2, 1} and
 * four POINT_DATA arrays dof_component_0..3, the cell's polynomial evaluated
 * there.  Built on the device in chunks; the file is byte-identical to the
 * reference's. */
amr_status amr_tree_dg_write_vtk(amr_tree* t, const char* path);

#define AMR_DG_ADVECTION 0
#define AMR_DG_EULER     1
amr_status amr_tree_dg_set_equation(amr_tree* t, int equation);

/* ------------------------------------------------------------- Euler
 * EulerPhysics<DIM> (include/solver/EulerPhysics.hpp:17-170) through
 * amr_solver (amr_solver.hpp:155-413) on a tree created with fields =
 * rank + 2 (rho, rho u_d, E; FP64): each step takes the CFL step from the
 * current state (min over cells and axes of dx / (|u_d| + a), times cfl,
 * clamped to the remaining time) and applies the Rusanov update with face
 * ghosts from the neighbours by the halo rules, every field.  The arithmetic
 * is the reference's, operation for operation (no contraction), so states
 * are bit-identical to its CPU path.  Use amr_tree_finish_advance for the
 * simulated time and executed steps. */
amr_status amr_tree_euler_advance(amr_tree* t, size_t steps, double gamma, double cfl, double remaining_time);

/* The reference's Euler benchmark loop (benchmark/bench_fvm_solver_
 * integration.b.cpp:208-250): repeat { advance min(remesh_interval, steps
 * left) steps with the remaining time end_time - t; flags from the maximum
 * of rho over interior and face-ghost cells (Refine above refine_threshold
 * below max_level, Coarsen under coarsen_threshold above min_level);
 * re-mesh } until `steps` steps ran or t reaches end_time. */
typedef struct amr_euler_params {
    uint64_t steps;
    uint64_t remesh_interval;
    double   gamma;
    double   cfl;
    double   end_time;
    double   refine_threshold;
    double   coarsen_threshold;
    int32_t  min_level;
    int32_t  max_level;
} amr_euler_params;
amr_status amr_tree_euler_run(amr_tree* t, const amr_euler_params* params, amr_cycle_stats* stats);

/* ----------------------------------------------------------- forests
 * Per-instance parameters (instances > 1): velocity (3 per instance, Morton
 * axis order x, y, z) and level bounds (min_level, max_level per instance).
 * Either array may be NULL to leave that part unchanged; level_bounds NULL
 * also keeps (or, on the first call, leaves off) the per-instance bounds.
 * amr_tree_advance with velocity3 == NULL and amr_tree_run with
 * AMR_RUN_INSTANCE_PARAMS use these velocities; the flag calls and
 * amr_tree_run use these bounds in place of min_level/max_level once set. */
amr_status amr_tree_set_instance_params(amr_tree* t, const double* velocity, const int32_t* level_bounds,
                                        size_t instances);
/* Refine every leaf of instance i until it reaches target_levels[i]
 * (one reconstruct_tree per level, with 2:1 balance). */
amr_status amr_tree_refine_to_levels(amr_tree* t, const int32_t* target_levels, size_t instances);
/* offsets[i] = index of the first leaf of instance i, offsets[instances] =
 * size(); instances + 1 entries. */
amr_status amr_tree_instance_offsets(amr_tree* t, uint64_t* offsets, size_t instances_plus_one);
/* Simulated time and executed steps per instance since the last
 * amr_tree_advance/amr_tree_run started. */
amr_status amr_tree_instance_time(amr_tree* t, double* sum_dt, uint32_t* executed_steps, size_t instances);

/* ------------------------------------------------------------ adjoint
 * Discrete adjoint of amr_tree_advance on a frozen mesh (no counterpart in
 * the reference; it differentiates the reference's flux update
 * (amr_solver.hpp:265-353), halo fill (patch_utils.hpp:162-441) and forward
 * Euler integrator).  The map from the interior of u_0 to the interior of
 * u_T is linear; amr_adjoint_backward applies its transpose, step by step in
 * reverse order: the transposed flux update (upwind -> downwind) and the
 * transposed halo rules (copy, restriction mean, injection), with the step
 * sizes of the forward run.
 *
 * amr_adjoint_forward runs the steps from the tree's current state (the
 * kernels of amr_tree_advance, velocity and CFL of create, or the
 * per-instance velocities when velocity3 is NULL) and stores a checkpoint
 * every checkpoint_every steps: the state and the step sizes of the segment.
 * The reverse sweep walks the segments from the last to the first and
 * rebuilds each segment's step coefficients from its checkpoint; the
 * transposed update of linear advection reads no forward state, so the
 * checkpointed states are not recomputed step by step (they remain
 * available through amr_adjoint_checkpoint).  Memory: (steps /
 * checkpoint_every + 1) states.  Any re-mesh of the tree after create makes
 * forward/backward fail with AMR_ERR_INVALID. */
typedef struct amr_adjoint amr_adjoint;
amr_status amr_adjoint_create(amr_tree* t, size_t steps, const double* velocity3, double cfl,
                              double remaining_time, size_t checkpoint_every, amr_adjoint** out);
amr_status amr_adjoint_destroy(amr_adjoint* a);
amr_status amr_adjoint_forward(amr_adjoint* a);
/* lambda_T, lambda_0: device buffers of size() padded patches of the tree's
 * dtype.  lambda_0 = d<lambda_T, u_T>/d u_0 on interior cells (the ghost
 * entries of lambda_T are ignored; those of lambda_0 are zero). */
amr_status amr_adjoint_backward(amr_adjoint* a, const void* device_lambda_T, void* device_lambda_0);
/* The same with host buffers (copied through the adjoint's own device
 * buffers). */
amr_status amr_adjoint_backward_host(amr_adjoint* a, const void* host_lambda_T, void* host_lambda_0);
/* State at step index * checkpoint_every (index 0 = u_0; the last index
 * holds u_T), copied to a device buffer. */
amr_status amr_adjoint_checkpoint(amr_adjoint* a, size_t index, void* device_dst);
amr_status amr_adjoint_checkpoint_count(const amr_adjoint* a, size_t* count);

/* Per-launch timing of the fused update kernel (advection or Euler) with CUDA
 * events on the tree's stream (the counterpart of the reference's profiler ranges,
 * include/cuda/profiler.hpp:7-30).  get_timing synchronizes, returns the
 * summed kernel time, launch count and cell updates since the last call, and
 * clears them. */
amr_status amr_tree_set_timing(amr_tree* t, int enabled);
amr_status amr_tree_get_timing(amr_tree* t, double* step_kernel_ms, uint64_t* step_launches,
                               uint64_t* cell_updates);

/* vtk_print::print (include/ndtree/vtk_print.hpp:53-257) of the current
 * leaves and state: legacy binary VTK (big-endian), one quad (2D) or voxel
 * (3D) per interior cell, CELL_DATA cell_index, is_halo and the field named
 * field_name (an FP32 tree writes its values as "float"; with several fields,
 * field_name lists their names separated by commas and each gets its own
 * SCALARS block).  Every section is built on the device; byte-identical to
 * the reference writer for FP64 trees. */
amr_status amr_tree_write_vtk(amr_tree* t, const char* path, const char* field_name);

/* Launch shape of the 2D update kernel used by the tree's last advance or
 * run: warps per block, copy stages per warp, blocks (0 = full residency).
 * The autotuner picks it on first use per device, dtype, patch shape and
 * leaf-count octave (AMR_GB300_AUTOTUNE=0 keeps the default 8, 2, 0;
 * AMR_GB300_STEP_CONFIG="warps,stages,blocks_per_sm" fixes it, with
 * blocks_per_sm 0 for full residency, warps and stages one of the tuned
 * pairs). */
amr_status amr_tree_step_config(const amr_tree* t, int32_t* warps, int32_t* stages, int32_t* blocks);

/* Block until all work queued on the tree's stream has finished. */
amr_status amr_tree_synchronize(amr_tree* t);

/* ------------------------------------------------ allocation-free re-mesh
 * No counterpart in the reference: an addition for callers that cannot
 * allocate device memory, e.g. code running inside a memory pool or arena
 * they do not own, or a host process whose allocator is locked down.  It runs
 * the re-mesh of amr_tree_remesh for a finite-volume tree of ONE FP64 field
 * (the padded state layout; piecewise-constant prolongation and FP64-mean
 * restriction), on caller-owned buffers, and calls no cudaMalloc, cudaFree or
 * other allocating routine.  Multi-field trees (Euler) and DG trees, whose
 * re-mesh remaps several fields or interpolates polynomials, are not served
 * by it.  Its working storage is one static
 * device array of AMR_NOALLOC_SCRATCH_BYTES per GPU that loads the library,
 * held until the process exits; that bounds the input to
 * AMR_NOALLOC_MAX_LEAVES leaves, and larger inputs (or out_capacity) are
 * rejected with AMR_ERR_INVALID.
 *
 * Inputs: num_leaves leaves in Morton order (ids, neighbour tables as
 * produced by amr_tree_get_neighbors, refine/coarsen flags, FP64 padded
 * state).  Outputs (room for out_capacity leaves): the new ids, levels,
 * neighbour tables and state, and the new leaf count in *device_out_count
 * and, if host_out_count is not NULL, in *host_out_count.  The call
 * synchronizes `stream` before it returns.  AMR_ERR_CAPACITY means the new
 * tree would not fit in out_capacity; the outputs are then undefined.
 *
 * The first call on each device looks up the scratch array's device address
 * with that device current; make that first call before capturing a stream.
 * All calls share the one array, so calls that overlap on the GPU (other
 * streams, other host threads) race and corrupt each other's results. */
#define AMR_NOALLOC_MAX_LEAVES 65536
#define AMR_NOALLOC_SCRATCH_BYTES (17 * AMR_NOALLOC_MAX_LEAVES + 4096)
amr_status amr_remesh_noalloc(const amr_patch_geometry* geom, size_t num_leaves,
                              const uint64_t* device_ids_in, const amr_halo_meta* device_meta_in,
                              const int8_t* device_flags, const double* device_state_in,
                              size_t out_capacity, uint64_t* device_ids_out, int32_t* device_levels_out,
                              amr_halo_meta* device_meta_out, double* device_state_out,
                              uint32_t* device_out_count, size_t* host_out_count, void* stream);

/* Self-test of the bounded waits: one warp waits on an mbarrier whose
 * transaction never arrives, gives up after `polls` polls and records
 * AMR_ERR_TIMEOUT, which the host reads; then a second kernel runs to show
 * the context is still usable.  *observed = the status the kernel recorded.
 * Returns AMR_OK when the wait timed out as designed. */
amr_status amr_selftest_wait_timeout(int32_t polls, amr_status* observed);

/* Kernel launches issued by this library since load (for launch accounting). */
uint64_t amr_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* AMR_GB300_H */

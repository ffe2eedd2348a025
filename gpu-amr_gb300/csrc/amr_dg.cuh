// Interface of the nodal DG stage kernel (amr_dg.cu, compiled without
// multiply-add contraction).
#pragma once

#include <string>

#include "amr_device.cuh"
#include "amr_gb300.h"

namespace amr_gb300 {

// The reference's DG patch solver configuration (include/config/
// generated_config.hpp): order 2 (2 x 2 Gauss-Legendre nodes per cell), 2D,
// 4 variables per node, 4 x 4 cells per patch with one ghost cell, linear
// advection with velocity 1.  On the tree a cell's 16 nodal values are 16
// fields (field = node * 4 + variable, node = x-node * 2 + y-node).
constexpr int kDgOrder = 2, kDgVars = 4, kDgFields = 16, kDgPatch = 4;

// Basis tables: face kernels k[s][i] = L_i(s) (s = 0, 1) and the derivative
// tensor d[i][j] = L_i'(x_j) of the 1D Lagrange basis at the Gauss-Legendre
// points on [0, 1].
struct DgTables {
    double k[2][2];
    double d[2][2];
};
DgTables dg_tables();

// One SSPRK2 stage over every cell of P padded patches.  mode 0: out = in +
// dt R(in); mode 1: out = ((un + in) + dt R(in)) * 0.5.  Ghost cells take a
// zero residual (the reference combines whole patch containers).  out may
// alias un.
struct DgStage {
    const double*   in;
    const double*   un;
    double*         out;
    const uint64_t* keys;
    int             P;
    Geo             g;
    size_t          fstride;
    double          dt;
    int             mode;
    cudaStream_t    stream;
};
cudaError_t dg_stage(const DgStage& s);

// The DG Euler equations (include/dg_helpers/equations/euler.hpp, variables
// [rho u, rho v, rho, E], gamma 1.4) with the same residual structure; the
// Rusanov speed is the patch's running maximum of max(eig(cell),
// eig(neighbour)) over its faces in the reference's loop order (cells row-
// major, faces y-, y+, x-, x+), eig from the cell's first node.
//   prims: per padded cell and node, p, u, v (fields 0-11, fstride apart),
//   then the cell's eigenvalues in x and y (fields 12, 13), formed after
//   each halo exchange by dg_euler_prims (corner ghosts left unset).
//   dt: the step in use (device, [0]); in the last stage (mode 1) each patch
//   folds 0.1 x edge / lambda into dt_min (ordered bit pattern of a positive
//   double), and dg_euler_next takes dt = min(dt, min(dt, dt_min)), adds
//   that updated step to time (the reference's loop order) and resets
//   dt_min.
struct DgEulerStage {
    const double*       in;
    const double*       un;
    double*             out;
    const double*       prims;
    const uint64_t*     keys;
    int                 P;
    Geo                 g;
    size_t              fstride;
    const double*       dt;
    unsigned long long* dt_min;
    int                 mode;
    cudaStream_t        stream;
};
cudaError_t dg_euler_prims(const double* in, double* prims, int P, const Geo& g, size_t fstride, cudaStream_t s);
cudaError_t dg_euler_stage(const DgEulerStage& s);
cudaError_t dg_euler_next(double* dt, double* time, unsigned long long* dt_min, cudaStream_t s);

// The reference's DG printer (dg_tree_printer_2d) for the tree's leaves and
// DG state, written to `path`; `launches` counts the kernels run.
amr_status dg_write_vtk(const uint64_t* keys, const double* state, size_t size, const Geo& g, size_t fstride,
                        cudaStream_t s, const char* path, std::string& err, uint64_t& launches);

// Halo exchange of a DG state (16 fields fstride apart): same-level faces
// copy, coarse-fine faces restrict or interpolate the DG polynomials.
cudaError_t dg_halo(double* buf, const amr_halo_meta* meta, int P, const Geo& g, size_t fstride, cudaStream_t s);

// Re-mesh of a DG state from the re-mesh source table (src, skind as for
// the FV remap): copies, polynomial interpolation, polynomial restriction.
cudaError_t dg_remap(const double* old_state, double* new_state, const int32_t* src, const int8_t* skind, int P,
                     const Geo& g, size_t fstride, cudaStream_t s);

// Refine / coarsen / stable per leaf by the reference's DG gradient
// indicator with thresholds rthr / cthr.
cudaError_t dg_flags(const double* in, int P, const Geo& g, size_t fstride, double rthr, double cthr, int8_t* flags,
                     cudaStream_t s);

} // namespace amr_gb300

// Interface of the device-resident VTK writer (amr_vtk.cu) for the tree.
#pragma once

#include <string>

#include "amr_device.cuh"

namespace amr_gb300 {

struct VtkDomain {
    double lengths[3]; // physical domain lengths per Morton axis
};

struct VtkTree {
    Geo             g;
    VtkDomain       dom;
    const uint64_t* keys;  // device, Morton order
    const void*     state; // device, padded patches
    size_t          size;  // leaves
    size_t          esize; // bytes per state value
    int             nvar;    // fields, one SCALARS block each
    size_t          fstride; // elements between fields
    cudaStream_t    stream;
};

// `fields`: the field names, separated by commas, one per field.
amr_status vtk_write(const VtkTree& v, const char* path, const char* fields, std::string& err);

} // namespace amr_gb300

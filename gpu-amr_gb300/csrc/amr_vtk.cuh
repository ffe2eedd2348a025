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
    cudaStream_t    stream;
};

amr_status vtk_write(const VtkTree& v, const char* path, const char* field, std::string& err);

} // namespace amr_gb300

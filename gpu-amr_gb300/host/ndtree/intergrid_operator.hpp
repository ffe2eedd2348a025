// The inter-grid operator of gpu-amr (include/ndtree/intergrid_operator.hpp):
// piecewise-constant prolongation and mean restriction.  The arithmetic runs
// in the CUDA kernels; this type selects it as the tree's template argument.
#pragma once

namespace amr::ndt::intergrid_operator
{

template <typename Patch_Layout>
struct linear_interpolator
{
    using patch_layout_t = Patch_Layout;
};

} // namespace amr::ndt::intergrid_operator

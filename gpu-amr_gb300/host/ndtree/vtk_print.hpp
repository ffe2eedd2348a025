// vtk_print (include/ndtree/vtk_print.hpp:17-282 of the reference) over the
// device-resident writer: print(tree, extension) writes
// vtk_output/<base><extension>, byte-identical to the reference's file, with
// every section built on the GPU (amr_tree_write_vtk).
#pragma once

#include <filesystem>
#include <iostream>
#include <stdexcept>
#include <string>
#include <string_view>
#include <type_traits>

#include "amr_gb300.h"
#include "ndtree/ndtree.hpp"

namespace amr::ndt::print
{

template <typename Physics_System>
struct vtk_print
{
    using physics_system_t = Physics_System;

    explicit vtk_print(std::string_view base_filename) : m_base_filename{ base_filename }
    {
        std::filesystem::path output_path = "vtk_output";
        std::filesystem::create_directory(output_path);
        std::cout << "VTK files will be saved to: " << std::filesystem::absolute(output_path) << std::endl;
    }

    auto print(auto const& tree, std::string filename_extension) const -> void
    {
        using tree_t                   = std::remove_cvref_t<decltype(tree)>;
        const std::string full_filename = "vtk_output/" + m_base_filename + filename_extension;
        const std::string field = tree_t::field_names(); // one SCALARS block per field
        auto&             t = const_cast<tree_t&>(tree);
        const amr_status  s = amr_tree_write_vtk(t.handle(), full_filename.c_str(), field.c_str());
        if (s != AMR_OK) throw std::runtime_error("Cannot write file: " + full_filename + ": " + amr_last_error());
    }

private:
    std::string m_base_filename;
};

} // namespace amr::ndt::print

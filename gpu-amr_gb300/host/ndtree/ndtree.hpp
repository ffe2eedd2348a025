// gpu-amr's amr::ndt::tree::ndtree (include/ndtree/ndtree.hpp:94-2157) backed
// by the GB300 device-resident tree of libamr_gb300 (include/amr_gb300.h).
//
// The leaf set, Morton ids, neighbour tables and cell state live in HBM and
// every tree operation runs on the GPU.  get_patch() returns a host mirror of
// the current buffer, downloaded when the device holds newer data; writes
// through it reach the device before the next device operation (or on
// sync_current_to_device(), as in the reference's CUDA path).  Errors from the
// C ABI become std::runtime_error, the reference's convention
// (src/cuda/device_buffer.cu:17-27).
//
// Supported: cells of FP64 fields (the advection cell, the Euler cells), one
// device array per field; cubic patches, halo >= 1, rank 2 or 3.  Edge and
// corner ghosts, which the face halo exchange never writes, read as -1000
// through get_patch, the value the reference's checking build leaves in them
// (swap_buffers, ndtree.hpp:1558-1579).
#pragma once

#include "amr_gb300.h"
#include "morton/morton_id.hpp"
#include "ndtree/intergrid_operator.hpp"
#include "ndtree/patch.hpp"
#include "ndtree/patch_layout.hpp"

#include <algorithm>
#include <array>
#include <cstdint>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

namespace amr::gb300
{
inline void check(amr_status s)
{
    if (s != AMR_OK) throw std::runtime_error(std::string("gb300-amr: ") + amr_last_error());
}
} // namespace amr::gb300

namespace amr::ndt::tree
{

template <typename T, typename Patch_Index, typename Patch_Layout, typename Intergrid_Operator>
class ndtree
{
public:
    using map_type             = T;
    using size_type            = std::size_t;
    using patch_index_t        = Patch_Index;
    using patch_layout_t       = Patch_Layout;
    using intergrid_operator_t = Intergrid_Operator;
    using linear_index_t       = size_type;
    using deconstructed_raw_map_types_t = typename T::deconstructed_types_map_t;
    template <typename Map_Type>
    using patch_t = patches::patch<typename Map_Type::type, patch_layout_t>;

    static constexpr std::size_t n_fields = std::tuple_size_v<deconstructed_raw_map_types_t>;
    using field_t = std::tuple_element_t<0, deconstructed_raw_map_types_t>;
    static_assert([]<std::size_t... I>(std::index_sequence<I...>) {
        return (std::is_same_v<typename std::tuple_element_t<I, deconstructed_raw_map_types_t>::type, double> && ...);
    }(std::make_index_sequence<n_fields>{}), "FP64 fields");

    // position of a field tag in the cell's tuple (its device array)
    template <typename Map_Type>
    static constexpr auto field_index() noexcept -> std::size_t
    {
        return []<std::size_t... I>(std::index_sequence<I...>) {
            std::size_t r = n_fields;
            ((std::is_same_v<Map_Type, std::tuple_element_t<I, deconstructed_raw_map_types_t>> ? (r = I) : 0), ...);
            return r;
        }(std::make_index_sequence<n_fields>{});
    }

    // the field names in tuple order, separated by commas (the VTK writer)
    static auto field_names() -> std::string
    {
        std::string out;
        [&]<std::size_t... I>(std::index_sequence<I...>) {
            ((out += (I ? "," : ""), out += std::tuple_element_t<I, deconstructed_raw_map_types_t>::name()), ...);
        }(std::make_index_sequence<n_fields>{});
        return out;
    }

    enum struct RefinementStatus : std::int8_t { Stable = 0, Refine = 1, Coarsen = 2 };
    using refine_status_t = RefinementStatus;

    struct current_buffer_t {};
    struct next_buffer_t {};
    static constexpr current_buffer_t current_buffer{};
    static constexpr next_buffer_t    next_buffer{};

    static constexpr auto rank() noexcept { return patch_layout_t::rank(); }
    static constexpr auto nd_fanout() noexcept { return patch_index_t::nd_fanout(); }

    // ndtree(size) (ndtree.hpp:320-425): one root leaf with periodic
    // self-neighbours, fixed capacity.
    explicit ndtree(size_type capacity, void* stream = nullptr) : ndtree(capacity, { 1.0, 1.0, 1.0 }, stream) {}

    // The physical domain lengths per Morton axis come from the geometry
    // (physics_system's Domain_Sizes); amr_solver passes them.
    ndtree(size_type capacity, std::array<double, 3> const& lengths, void* stream = nullptr)
    {
        static_assert(patch_layout_t::rank() == patch_index_t::rank());
        amr_tree_desc d{};
        d.geom.rank  = static_cast<int32_t>(rank());
        d.geom.n     = static_cast<int32_t>(patch_layout_t::data_layout_t::sizes()[0]);
        d.geom.halo  = static_cast<int32_t>(patch_layout_t::halo_width());
        d.geom.depth = static_cast<int32_t>(patch_index_t::max_depth());
        for (int a = 0; a < 3; ++a) d.geom.lengths[a] = lengths[a];
        d.capacity = capacity;
        d.dtype    = AMR_F64;
        d.stream   = stream;
        d.fields   = static_cast<int32_t>(n_fields);
        amr::gb300::check(amr_tree_create(&d, &m_tree));
        m_capacity = capacity;
        m_host.resize(n_fields);
        std::memset(static_cast<void*>(m_host.data()), 0, n_fields * sizeof(patch_t<field_t>));
        m_host_valid = true;
    }

    ~ndtree()
    {
        if (m_tree) amr_tree_destroy(m_tree);
    }
    ndtree(ndtree const&)                    = delete;
    auto operator=(ndtree const&) -> ndtree& = delete;

    [[nodiscard]] auto size() const -> size_type
    {
        size_type n = 0;
        amr::gb300::check(amr_tree_size(m_tree, &n));
        return n;
    }

    [[nodiscard]] auto get_node_index_at(linear_index_t i) const -> patch_index_t
    {
        load_ids();
        return patch_index_t(m_ids.at(i));
    }

    [[nodiscard]] auto get_linear_index_at(patch_index_t id) const -> linear_index_t
    {
        load_ids();
        auto it = std::lower_bound(m_ids.begin(), m_ids.end(), id.id());
        if (it == m_ids.end() || *it != id.id()) throw std::out_of_range("patch index not in the tree");
        return static_cast<linear_index_t>(it - m_ids.begin());
    }

    template <typename Map_Type>
    [[nodiscard]] auto get_patch(linear_index_t i) -> patch_t<Map_Type>&
    {
        static_assert(field_index<Map_Type>() < n_fields, "not a field of this cell");
        return get_field_patch(field_index<Map_Type>(), i);
    }
    template <typename Map_Type>
    [[nodiscard]] auto get_patch(linear_index_t i) const -> patch_t<Map_Type> const&
    {
        static_assert(field_index<Map_Type>() < n_fields, "not a field of this cell");
        load_host();
        return m_host.at(field_index<Map_Type>() * host_patches() + i);
    }
    // patch i of field f (tuple position), for code that loops over fields
    [[nodiscard]] auto get_field_patch(std::size_t f, linear_index_t i) -> patch_t<field_t>&
    {
        load_host();
        m_host_dirty = true;
        return m_host.at(f * host_patches() + i);
    }
    template <typename Map_Type>
    [[nodiscard]] auto get_patch(patch_index_t id) -> patch_t<Map_Type>&
    {
        return get_patch<Map_Type>(get_linear_index_at(id));
    }
    template <typename Map_Type>
    [[nodiscard]] auto get_patch(patch_index_t id) const -> patch_t<Map_Type> const&
    {
        return get_patch<Map_Type>(get_linear_index_at(id));
    }

    // get_device_buffer<Map, Buffer>() (ndtree.hpp:562-581)
    template <typename Map_Type, auto Buffer = current_buffer>
    [[nodiscard]] auto get_device_buffer() -> patch_t<Map_Type>*
    {
        push_host();
        void *cur = nullptr, *nxt = nullptr;
        amr::gb300::check(amr_tree_device_state(m_tree, &cur, &nxt));
        const std::size_t off = field_index<Map_Type>() * m_capacity; // field arrays, capacity patches apart
        if constexpr (std::is_same_v<std::remove_cvref_t<decltype(Buffer)>, next_buffer_t>)
            return static_cast<patch_t<Map_Type>*>(nxt) + off;
        else
            return static_cast<patch_t<Map_Type>*>(cur) + off;
    }

    void sync_current_to_device()
    {
        m_host_dirty = true;
        push_host();
    }
    void sync_current_from_device()
    {
        m_host_valid = false;
        load_host();
    }
    void sync_all_to_device() { sync_current_to_device(); }
    void sync_all_from_device() { sync_current_from_device(); }
    // levels are kept on the device by every re-mesh
    void build_patch_levels_on_device() {}

    // halo_exchange_update (ndtree.hpp:1862-1877)
    void halo_exchange_update()
    {
        push_host();
        amr::gb300::check(amr_tree_halo_exchange(m_tree));
        m_host_valid = false;
    }

    // Buffers are swapped inside the device step; kept for the interface.
    constexpr void swap_buffers() noexcept {}

    // reconstruct_tree(fn) (ndtree.hpp:1249-1271).  fn is a per-patch
    // functor fn(patch_index_t) -> refine_status_t evaluated on the host over
    // the current state (halos exchanged first), or an object with
    // fill_refine_flags(tree&) that sets the flags on the device.
    template <typename Fn>
    void reconstruct_tree(Fn&& fn)
    {
        push_host();
        if constexpr (requires(std::remove_reference_t<Fn> const& c, ndtree& t) { c.fill_refine_flags(t); }) {
            std::as_const(fn).fill_refine_flags(*this);
        } else {
            halo_exchange_update();
            load_host();
            const size_type           n = size();
            std::vector<std::int8_t>  f(n);
            for (size_type i = 0; i != n; ++i) f[i] = static_cast<std::int8_t>(fn(get_node_index_at(i)));
            amr::gb300::check(amr_tree_set_flags(m_tree, f.data(), n));
            // the criterion reads the patches; it does not change the state
            m_host_dirty = false;
        }
        int changed = 0;
        amr::gb300::check(amr_tree_remesh(m_tree, &changed));
        m_ids_valid  = false;
        m_host_valid = false;
        m_host_dirty = false;
    }

    [[nodiscard]] auto get_refine_status(linear_index_t i) const -> refine_status_t
    {
        std::vector<std::int8_t> f(size());
        amr::gb300::check(amr_tree_get_flags(m_tree, f.data(), f.size()));
        return static_cast<refine_status_t>(f.at(i));
    }

    // ------------------------------------------------ GB300 device criteria
    void flag_gradient(double rthr, double cthr, int min_level, int max_level)
    {
        push_host();
        amr::gb300::check(amr_tree_flags_gradient(m_tree, rthr, cthr, min_level, max_level));
    }
    void flag_max_value(double rthr, double cthr, int min_level, int max_level)
    {
        push_host();
        amr::gb300::check(amr_tree_flags_max(m_tree, rthr, cthr, min_level, max_level));
    }

    [[nodiscard]] auto handle() -> amr_tree*
    {
        push_host();
        m_host_valid = false;
        m_ids_valid  = false;
        return m_tree;
    }

private:
    void load_ids() const
    {
        if (m_ids_valid) return;
        m_ids.resize(size());
        amr::gb300::check(amr_tree_get_ids(m_tree, m_ids.data(), m_ids.size()));
        m_ids_valid = true;
    }
    auto host_patches() const -> std::size_t { return m_host.size() / n_fields; }
    void load_host() const
    {
        if (m_host_valid) return;
        const std::size_t n = size();
        m_host.resize(n_fields * n);
        amr::gb300::check(amr_tree_download_state(m_tree, m_host.data(), n));
        // edge and corner ghosts: never written by the face halo exchange
        for (auto& patch : m_host)
            for (std::size_t li = 0; li != patch_layout_t::flat_size(); ++li)
                if (edge_or_corner(li)) patch[static_cast<typename patch_layout_t::index_t>(li)] = -1000;
        m_host_valid = true;
        m_host_dirty = false;
    }
    static auto edge_or_corner(std::size_t li) -> bool
    {
        constexpr std::size_t P1 = patch_layout_t::data_layout_t::sizes()[0] + 2 * patch_layout_t::halo_width();
        constexpr std::size_t h  = patch_layout_t::halo_width();
        int                   outside = 0;
        for (std::size_t k = 0; k < rank(); ++k, li /= P1) outside += (li % P1 < h || li % P1 >= P1 - h) ? 1 : 0;
        return outside > 1;
    }
    void push_host()
    {
        if (!m_host_dirty) return;
        amr::gb300::check(amr_tree_upload_state(m_tree, m_host.data(), host_patches()));
        m_host_dirty = false;
    }

    amr_tree*                                 m_tree = nullptr;
    std::size_t                               m_capacity = 0;
    mutable std::vector<patch_t<field_t>>     m_host;
    mutable std::vector<std::uint64_t>        m_ids;
    mutable bool                              m_host_valid = false;
    mutable bool                              m_host_dirty = false;
    mutable bool                              m_ids_valid  = false;
};

} // namespace amr::ndt::tree

namespace amr::gb300
{

// Device criteria usable with ndtree::reconstruct_tree: the gradient rule
// max|grad u|*h (refine above refine_threshold below max_level, coarsen below
// coarsen_threshold above min_level, any/all patch rule) and the max-value
// rule of the reference's examples.
struct gradient_criterion
{
    double refine_threshold  = 0.05;
    double coarsen_threshold = 0.01;
    int    min_level         = 1;
    int    max_level         = 5;
    template <typename Tree>
    void fill_refine_flags(Tree& t) const
    {
        t.flag_gradient(refine_threshold, coarsen_threshold, min_level, max_level);
    }
};

struct max_value_criterion
{
    double refine_threshold  = 0.1;
    double coarsen_threshold = 0.05;
    int    min_level         = 1;
    int    max_level         = 5;
    template <typename Tree>
    void fill_refine_flags(Tree& t) const
    {
        t.flag_max_value(refine_threshold, coarsen_threshold, min_level, max_level);
    }
};

} // namespace amr::gb300

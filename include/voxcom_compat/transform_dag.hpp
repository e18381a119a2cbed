// voxcom_compat/transform_dag.hpp — header-only C++ shim that gives the reference's C++ callers
// (voxelizer, svdag_encoding, transform_subset_comparison) the signatures they already call, with
// the work done by libtdag.so on the GPU.
//
// Reference interfaces mirrored here (tools/lib/include/voxcom/voxel/transform_dag.h):
//   TransformDAGConfig ......................................... :157-160
//   constructTransformDAG<Structure>(inDag, config) ............ :161-162
//   constructTransformDAGHierarchical<Structure>(inDag, config)  :168-169
//   findDuplicatesAmongFlattenedItems_cpp2<Level>(...) ......... :307-308 (dense-grid form)
// EditStructure's member layout follows tools/lib/include/voxcom/voxel/structure.h:159-211.
//
// Errors: the reference throws std::runtime_error from assert_always (error_handling.h:34-44); this
// shim throws tdag_compat::Error (derived from std::runtime_error) with the library's message.
#pragma once
#include <array>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../tdag.h"

namespace tdag_compat {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m)
        : std::runtime_error(m)
        , code(c)
    {
    }
};

inline void check(int rc)
{
    if (rc != TDAG_OK)
        throw Error(rc, tdag_last_error_message());
}

// TransformDAGConfig (transform_dag.h:157-160): same members, same defaults, same 8-byte layout.
struct TransformDAGConfig {
    bool symmetry = true, axisPermutation = true, translation = true;
    uint32_t maxTranslationLevel = 4;
};
static_assert(sizeof(TransformDAGConfig) == 8, "TransformDAGConfig must keep the reference's 8-byte layout");

enum class StructureType : uint32_t { Tree = 0, DAG = 1 };

template <typename Child>
struct EditNode {
    std::array<Child, 8> children;
};
struct EditSubGrid {
    uint64_t bitmask = 0;
};

// EditStructure<void, Child> with the reference's members (structure.h:159-171).
template <typename Child>
struct EditStructure {
    std::vector<std::vector<EditNode<Child>>> nodesPerLevel;
    std::vector<EditSubGrid> subGrids;
    static constexpr uint32_t subGridLevel = 2;
    unsigned resolution = 0;
    uint32_t rootLevel = 0;
    StructureType structureType = StructureType::Tree;
};

using TransformPointerBits = uint64_t; // TransformPointer's 64-bit compact layout (transform_dag.h:19-33)

// One library context per thread (a context owns one CUDA stream).
inline tdag_ctx* threadContext(int device = 0)
{
    struct Holder {
        tdag_ctx* ctx = nullptr;
        ~Holder()
        {
            if (ctx)
                tdag_ctx_destroy(ctx);
        }
    };
    thread_local Holder h;
    if (!h.ctx)
        check(tdag_ctx_create(device, nullptr, &h.ctx));
    return h.ctx;
}

namespace detail {
    inline tdag_config toC(const TransformDAGConfig& c)
    {
        return tdag_config { c.symmetry ? 1 : 0, c.axisPermutation ? 1 : 0, c.translation ? 1 : 0, c.maxTranslationLevel };
    }
    inline tdag_svdag_view viewOf(const EditStructure<uint32_t>& s)
    {
        tdag_svdag_view v;
        std::memset(&v, 0, sizeof(v));
        v.resolution = s.resolution;
        v.root_level = s.rootLevel;
        v.structure_type = (uint32_t)s.structureType;
        for (uint32_t l = 3; l <= s.rootLevel && l < TDAG_MAX_LEVELS; ++l) {
            v.nodes[l] = reinterpret_cast<const uint32_t*>(s.nodesPerLevel[l].data());
            v.node_counts[l] = s.nodesPerLevel[l].size();
        }
        v.leaves = reinterpret_cast<const uint64_t*>(s.subGrids.data());
        v.leaf_count = s.subGrids.size();
        return v;
    }
    inline EditStructure<TransformPointerBits> takeResult(tdag_result* r)
    {
        std::unique_ptr<tdag_result, int (*)(tdag_result*)> guard(r, tdag_result_free);
        EditStructure<TransformPointerBits> out;
        out.resolution = r->resolution;
        out.rootLevel = r->root_level;
        out.structureType = (StructureType)r->structure_type;
        out.nodesPerLevel.resize(r->root_level + 1);
        for (uint32_t l = 3; l <= r->root_level; ++l) {
            auto& lvl = out.nodesPerLevel[l];
            lvl.resize(r->node_counts[l]);
            if (!lvl.empty())
                std::memcpy(lvl.data(), r->nodes[l], lvl.size() * sizeof(EditNode<TransformPointerBits>));
        }
        out.subGrids.resize(r->leaf_count);
        if (!out.subGrids.empty())
            std::memcpy(out.subGrids.data(), r->leaves, out.subGrids.size() * sizeof(EditSubGrid));
        return out;
    }
}

// constructTransformDAG (transform_dag.h:161-162).
inline EditStructure<TransformPointerBits> constructTransformDAG(const EditStructure<uint32_t>& inDag, const TransformDAGConfig& config)
{
    const tdag_svdag_view v = detail::viewOf(inDag);
    const tdag_config c = detail::toC(config);
    tdag_result* r = nullptr;
    check(tdag_build(threadContext(), &v, &c, &r));
    return detail::takeResult(r);
}

// constructTransformDAGHierarchical (transform_dag.h:168-169).
inline EditStructure<TransformPointerBits> constructTransformDAGHierarchical(const EditStructure<uint32_t>& inDag, const TransformDAGConfig& config)
{
    const tdag_svdag_view v = detail::viewOf(inDag);
    const tdag_config c = detail::toC(config);
    tdag_result* r = nullptr;
    check(tdag_build_hierarchical(threadContext(), &v, &c, &r));
    return detail::takeResult(r);
}

// findDuplicatesAmongFlattenedItems_cpp2<Level> on dense grids (transform_dag.h:307-308).
// grids: n * (R^3 / 64) words, R = 1 << Level. Returns the kept item positions; outMapping gets one
// TransformPointer per item.
template <uint32_t Level>
inline std::vector<uint32_t> findDuplicatesAmongFlattenedItems(const std::vector<uint64_t>& grids, std::vector<TransformPointerBits>& outMapping,
    const TransformDAGConfig& config)
{
    constexpr size_t W = ((size_t)1 << (3 * Level)) / 64;
    const uint32_t n = (uint32_t)(grids.size() / W);
    outMapping.resize(n);
    std::vector<uint32_t> unique(n);
    uint32_t nu = 0;
    const tdag_config c = detail::toC(config);
    check(tdag_find_duplicates_level(threadContext(), Level, grids.data(), n, &c, outMapping.data(), unique.data(), &nu, nullptr));
    unique.resize(nu);
    return unique;
}

} // namespace tdag_compat

// Test driver for include/voxcom_compat/transform_dag.hpp: reads an .svo (EditStructure<void,uint32_t>,
// magic 72198382, version 2), calls tdag_compat::constructTransformDAG exactly as the reference's
// voxelizer does (tools/voxelizer/src/main.cpp:145-150) and writes the .tdag (structure + config).
// Exit code: 0 ok, 2 bad input, otherwise the library's error code + 10.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <iterator>
#include <vector>

#include "voxcom_compat/transform_dag.hpp"

using namespace tdag_compat;

template <typename T>
static bool readPod(std::istream& in, T& v) { return (bool)in.read(reinterpret_cast<char*>(&v), sizeof(T)); }
template <typename T>
static void writePod(std::ostream& out, const T& v) { out.write(reinterpret_cast<const char*>(&v), sizeof(T)); }

int main(int argc, char** argv)
{
    if (argc < 3)
        return 2;
    std::ifstream in(argv[1], std::ios::binary);
    uint32_t magic = 0, version = 0;
    if (!readPod(in, magic) || !readPod(in, version) || magic != 72198382u || version != 2u)
        return 2;
    EditStructure<uint32_t> dag;
    uint64_t nl = 0;
    readPod(in, nl);
    dag.nodesPerLevel.resize(nl);
    for (auto& lvl : dag.nodesPerLevel) {
        uint64_t c = 0;
        readPod(in, c);
        lvl.resize(c);
        in.read(reinterpret_cast<char*>(lvl.data()), (std::streamsize)(c * sizeof(EditNode<uint32_t>)));
    }
    uint64_t ns = 0;
    readPod(in, ns);
    dag.subGrids.resize(ns);
    in.read(reinterpret_cast<char*>(dag.subGrids.data()), (std::streamsize)(ns * 8));
    uint32_t st = 0;
    readPod(in, dag.resolution);
    readPod(in, dag.rootLevel);
    readPod(in, st);
    dag.structureType = (StructureType)st;
    if (!in)
        return 2;
    TransformDAGConfig config; // reference defaults: all transforms, maxTranslationLevel 4
    try {
        const auto tdag = constructTransformDAG(dag, config);
        std::ofstream out(argv[2], std::ios::binary);
        writePod(out, (uint64_t)tdag.nodesPerLevel.size());
        for (const auto& lvl : tdag.nodesPerLevel) {
            writePod(out, (uint64_t)lvl.size());
            out.write(reinterpret_cast<const char*>(lvl.data()), (std::streamsize)(lvl.size() * sizeof(lvl[0])));
        }
        writePod(out, (uint64_t)tdag.subGrids.size());
        out.write(reinterpret_cast<const char*>(tdag.subGrids.data()), (std::streamsize)(tdag.subGrids.size() * 8));
        writePod(out, tdag.resolution);
        writePod(out, tdag.rootLevel);
        writePod(out, (uint32_t)tdag.structureType);
        writePod(out, config); // raw 8-byte TransformDAGConfig; padding byte is zero-initialised below
    } catch (const Error& e) {
        std::cerr << e.what() << "\n";
        return 10 + e.code;
    }
    return 0;
}

// C entry points over the reference's own Transform-DAG sources (test infrastructure only).
//
// oracle/ref.mk compiles the reference's files where they lie (find_translation.cpp,
// transform_dag.cpp, transform_dag_hierarchical.cpp, transform_dag_encoding.cpp, huffman.cpp and
// the headers they include) together with this file into oracle/_ref/libtdag_ref.so. Only the
// test-suite and the golden-fixture script load it, to pin the CPU restatement (tdag_oracle.cpp,
// tdag16_oracle.cpp) against the reference itself. It exists only where the reference's sources
// are present; nothing in the product links it.
//
// Each entry point takes and returns the reference's own byte formats and does what the
// reference's command-line tools do with them:
//  * ref_svo_from_dense: EditStructure(VoxelGrid) (structure.h:423-429), written as an .svo
//    (export_import_structure.cpp:16-24: magic, version, EditStructure::writeTo);
//  * ref_to_dag: EditStructure::toDAG (structure.h:703-763);
//  * ref_construct_tdag: constructTransformDAG (transform_dag.cpp:138-240), written as the
//    voxelizer writes a .tdag (voxelizer/src/main.cpp:144-151);
//  * ref_hierarchical: constructTransformDAGHierarchical with no mid level
//    (transform_dag_hierarchical.cpp:524-529), structure only;
//  * ref_encode_tdag16: a .tdag read and encoded as svdag_encoding does
//    (svdag_encoding/src/main.cpp:88-96, 126-132);
//  * ref_to_static / ref_construct_static_tdag: StaticStructure(EditStructure) (structure.h:765-798)
//    and constructStaticTransformDAG (transform_dag.cpp:242-390), StaticStructure::writeTo bytes;
//  * ref_encode_static_tdag16: constructTransformDAG16 of a StaticStructure<void, TransformPointer>
//    (transform_dag_encoding.cpp:519-697), written like ref_encode_tdag16.
#include "transform_dag_encoding.h"
#include <voxcom/utility/binary_reader.h>
#include <voxcom/utility/binary_writer.h>
#include <voxcom/voxel/structure.h>
#include <voxcom/voxel/transform_dag.h>
#include <voxcom/voxel/voxel_grid.h>

#include <cstdlib>
#include <cstring>
#include <exception>
#include <limits>
#include <sstream>
#include <string>

using namespace voxcom;

namespace {

thread_local std::string g_error;

constexpr uint32_t kSvoMagic = 72198382; // export_import_structure.cpp:13
constexpr uint32_t kSvoVersion = 2; // export_import_structure.cpp:14

int fail(const std::exception& e)
{
    g_error = e.what();
    return 1;
}

void check(bool ok, const char* what)
{
    if (!ok)
        throw std::runtime_error(what);
}

std::istringstream inStream(const uint8_t* data, uint64_t len)
{
    return std::istringstream(std::string(reinterpret_cast<const char*>(data), size_t(len)), std::ios::binary);
}

int emit(const std::ostringstream& os, uint8_t** out, uint64_t* outLen)
{
    const std::string s = os.str();
    auto* buf = static_cast<uint8_t*>(std::malloc(s.size() ? s.size() : 1));
    if (!buf)
        throw std::bad_alloc();
    std::memcpy(buf, s.data(), s.size());
    *out = buf;
    *outLen = s.size();
    return 0;
}

EditStructure<void, uint32_t> readSvo(const uint8_t* svo, uint64_t len)
{
    auto is = inStream(svo, len);
    BinaryReader reader { is };
    check(reader.read<uint32_t>() == kSvoMagic, "not an .svo (magic)");
    check(reader.read<uint32_t>() == kSvoVersion, "unsupported .svo version");
    EditStructure<void, uint32_t> s;
    s.readFrom(reader);
    return s;
}

int writeSvo(const EditStructure<void, uint32_t>& s, uint8_t** out, uint64_t* outLen)
{
    std::ostringstream os(std::ios::binary);
    BinaryWriter writer { os };
    writer.write(kSvoMagic);
    writer.write(kSvoVersion);
    s.writeTo(writer);
    return emit(os, out, outLen);
}

TransformDAGConfig makeConfig(int sym, int axis, int trans, uint32_t level)
{
    // The struct holds three bools and a uint32_t; byte 3 is padding that the reference never
    // initialises. Zero it so that the written bytes are defined.
    TransformDAGConfig cfg;
    std::memset(static_cast<void*>(&cfg), 0, sizeof(cfg));
    cfg.symmetry = sym != 0;
    cfg.axisPermutation = axis != 0;
    cfg.translation = trans != 0;
    cfg.maxTranslationLevel = level;
    return cfg;
}

}

extern "C" {

const char* ref_last_error() { return g_error.c_str(); }

void ref_free(void* p) { std::free(p); }

// dense[z][y][x], one byte per voxel (non-zero = solid), res a power of two.
int ref_svo_from_dense(const uint8_t* dense, uint32_t res, uint8_t** out, uint64_t* outLen)
{
    try {
        VoxelGrid<void> grid { res };
        for (uint32_t z = 0; z < res; ++z)
            for (uint32_t y = 0; y < res; ++y)
                for (uint32_t x = 0; x < res; ++x)
                    if (dense[(size_t(z) * res + y) * res + x])
                        grid.set(glm::ivec3(int(x), int(y), int(z)));
        const EditStructure<void, uint32_t> s { grid };
        return writeSvo(s, out, outLen);
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int ref_to_dag(const uint8_t* svo, uint64_t len, uint8_t** out, uint64_t* outLen)
{
    try {
        auto s = readSvo(svo, len);
        s.toDAG();
        return writeSvo(s, out, outLen);
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int ref_construct_tdag(const uint8_t* svo, uint64_t len, int sym, int axis, int trans, uint32_t level,
    uint8_t** out, uint64_t* outLen)
{
    try {
        const auto in = readSvo(svo, len);
        const auto cfg = makeConfig(sym, axis, trans, level);
        const auto tdag = constructTransformDAG(in, cfg);
        std::ostringstream os(std::ios::binary);
        BinaryWriter writer { os };
        writer.write(tdag);
        writer.write(cfg);
        return emit(os, out, outLen);
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int ref_hierarchical(const uint8_t* svo, uint64_t len, int sym, int axis, uint8_t** out, uint64_t* outLen)
{
    try {
        const auto in = readSvo(svo, len);
        const auto cfg = makeConfig(sym, axis, 0, 0);
        std::vector<uint32_t> unused;
        const auto h = constructTransformDAGHierarchical(in, std::numeric_limits<uint32_t>::max(), unused, cfg);
        std::ostringstream os(std::ios::binary);
        BinaryWriter writer { os };
        h.writeTo(writer);
        return emit(os, out, outLen);
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int ref_encode_tdag16(const uint8_t* tdag, uint64_t len, int pointerTables, int huffman, uint8_t** out,
    uint64_t* outLen)
{
    try {
        auto is = inStream(tdag, len);
        BinaryReader reader { is };
        EditStructure<void, TransformPointer> transformDAG;
        reader.read(transformDAG);
        TransformDAGConfig dagConfig;
        std::memset(static_cast<void*>(&dagConfig), 0, sizeof(dagConfig));
        reader.read(dagConfig);
        TransformEncodingConfig encodingConfig;
        encodingConfig.pointerTables = pointerTables != 0;
        encodingConfig.huffmanCode = huffman != 0;
        DAGEncodingStats stats;
        const TransformDAG16 encoded = constructTransformDAG16(std::move(transformDAG), dagConfig, encodingConfig, stats);
        std::ostringstream os(std::ios::binary);
        BinaryWriter writer { os };
        writer.write(encoded);
        return emit(os, out, outLen);
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int ref_encode_static_tdag16(const uint8_t* st, uint64_t len, int sym, int axis, int trans, uint32_t level, int pointerTables,
    int huffman, uint8_t** out, uint64_t* outLen)
{
    try {
        auto is = inStream(st, len);
        BinaryReader reader { is };
        StaticStructure<void, TransformPointer> in;
        in.readFrom(reader);
        const auto cfg = makeConfig(sym, axis, trans, level);
        TransformEncodingConfig encodingConfig;
        encodingConfig.pointerTables = pointerTables != 0;
        encodingConfig.huffmanCode = huffman != 0;
        DAGEncodingStats stats;
        const TransformDAG16 encoded = constructTransformDAG16(std::move(in), cfg, encodingConfig, stats);
        std::ostringstream os(std::ios::binary);
        BinaryWriter writer { os };
        writer.write(encoded);
        return emit(os, out, outLen);
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int ref_to_static(const uint8_t* svo, uint64_t len, uint8_t** out, uint64_t* outLen)
{
    try {
        const auto in = readSvo(svo, len);
        const StaticStructure<void, uint32_t> st { in };
        std::ostringstream os(std::ios::binary);
        BinaryWriter writer { os };
        st.writeTo(writer);
        return emit(os, out, outLen);
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int ref_construct_static_tdag(const uint8_t* st, uint64_t len, int sym, int axis, int trans, uint32_t level,
    uint8_t** out, uint64_t* outLen)
{
    try {
        auto is = inStream(st, len);
        BinaryReader reader { is };
        StaticStructure<void, uint32_t> in;
        in.readFrom(reader);
        const auto cfg = makeConfig(sym, axis, trans, level);
        const auto tdag = constructStaticTransformDAG(std::move(in), cfg);
        std::ostringstream os(std::ios::binary);
        BinaryWriter writer { os };
        tdag.writeTo(writer);
        return emit(os, out, outLen);
    } catch (const std::exception& e) {
        return fail(e);
    }
}

}

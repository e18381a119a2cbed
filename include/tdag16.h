/* tdag16.h — C ABI of the .tdag16 encoder in libtdag.so.
 *
 * Replaces constructTransformDAG16(EditStructure<void, TransformPointer>, const TransformDAGConfig&,
 * const TransformEncodingConfig&, DAGEncodingStats&)
 * (tools/svdag_encoding/src/transform_dag_encoding.h:232; transform_dag_encoding.cpp:240-497) followed
 * by BinaryWriter::write(TransformDAG16) (transform_dag_encoding.cpp:1023-1030), as the svdag_encoding
 * tool does for a .tdag16 output (tools/svdag_encoding/src/main.cpp:87-134).
 *
 * The result is the .tdag16 file image. Two steps of the reference order items with equal reference
 * counts by whatever std::sort and std::unordered_map iteration give (pointer_encoding.h:49;
 * transform_dag_encoding.cpp:276-295), so the file bytes depend on the standard library. By default
 * (TDAG16_TIES_REFERENCE) the encoder runs exactly those two steps on the host with libstdc++'s
 * std::sort and std::unordered_map, the reference's hash of a TransformPointer and the reference's
 * insertion sequence, and its bytes equal the reference's as built with GCC (serial parallel-algorithm
 * backend); struct padding that the reference leaves uninitialised is written as zero.
 * TDAG16_TIES_CANONICAL orders ties by ascending item index and pointer value with stable radix sorts
 * on the device: the same voxels, Huffman tables and sizes, no host step, different bytes.
 */
#ifndef TDAG16_H_
#define TDAG16_H_

#include "tdag.h"

#ifdef __cplusplus
extern "C" {
#endif

/* TransformEncodingConfig (transform_dag_encoding.h:180-182). The svdag_encoding tool's defaults are
 * both off (main.cpp:34); the renderer's format sets both. */
typedef struct tdag_encoding_config {
    int32_t pointer_tables; /* frequent pointers through a per-level table (--pointertables) */
    int32_t huffman_code; /* Huffman-coded pointer types (--huffman) */
    int32_t tie_order; /* TDAG16_TIES_REFERENCE (0, the reference's bytes) or TDAG16_TIES_CANONICAL (1) */
} tdag_encoding_config;

#define TDAG16_TIES_REFERENCE 0
#define TDAG16_TIES_CANONICAL 1

/* DAGEncodingStats::LevelStats (transform_dag_encoding.h:187-203), index = tree level. */
typedef struct tdag16_level_stats {
    uint64_t num_nodes; /* nodes (level 2: leaves) after pruning */
    uint64_t memory_in_bytes; /* bytes of the level's u16 node stream (level 2: the leaves) */
    uint64_t table_size; /* entries of the pointer table into this level's children */
    uint64_t unique_pointers; /* distinct child pointers of this level */
    uint64_t table_pointers[3]; /* children stored as table references of 16 / 32 / 48 bits */
    uint64_t direct_pointers[3]; /* children stored inline in 16 / 32 / 48 bits */
} tdag16_level_stats;

typedef struct tdag16_result {
    uint8_t* bytes; /* the .tdag16 file (TransformDAG16::writeTo), host memory owned by the library */
    uint64_t size;
    uint32_t root_level;
    uint32_t reserved;
    tdag16_level_stats levels[TDAG_MAX_LEVELS];
    float encode_ms; /* device timeline of the encoder, from the first copy to the last kernel */
    float wall_ms; /* host wall time of the whole call, including the file assembly */
    uint64_t kernel_launches;
} tdag16_result;

/* Encode a transform DAG (tdag_build / tdag_build_device result; host or device arrays) with the
 * construction config it was built with. Release the result with tdag16_result_free. Returns
 * TDAG_ERR_ARG for a root level below 3, a pointer wider than 48 bits without pointer tables (the
 * reference asserts), or a level beyond 2^32 u16 words; TDAG_ERR_CORRUPT for dangling child pointers. */
int tdag_encode16(tdag_ctx* ctx, const tdag_result* dag, const tdag_config* config, const tdag_encoding_config* encoding,
    tdag16_result** out);
int tdag16_result_free(tdag16_result* result);

/* ------------------------------------------------------------------------------------------------
 * Queries on an encoded .tdag16 resident in device memory.
 * ------------------------------------------------------------------------------------------------ */
typedef struct tdag16_device tdag16_device; /* device copy of a .tdag16 file, library-owned */

/* Parse .tdag16 bytes (host memory) into device arrays and Huffman decode tables. Every index
 * later read from them is bounds-checked on the device (TDAG_ERR_CORRUPT). Free the handle with
 * tdag16_device_free before destroying the context. Root levels 3..23. */
int tdag16_upload(tdag_ctx* ctx, const uint8_t* bytes, uint64_t size, tdag16_device** out);
int tdag16_device_free(tdag16_device* dev);

/* TranslateTransformBaseDAG<TransformDAG16>::get (transform_dag_encoding.cpp:699-745) for n voxels:
 * d_xyz = n x (x, y, z) uint32 and d_out = n uint8 (1 = solid), both device memory. Coordinates
 * outside the grid answer 0. */
int tdag16_get(tdag_ctx* ctx, const tdag16_device* dev, const uint32_t* d_xyz, uint64_t n, uint8_t* d_out);

/* First solid voxel along rays (the CUDA part of the renderer's transform-DAG traversal,
 * renderer/src/dags/transform_dag/transform_dag.cu:5-41, as a batch query). Rays are in voxel units of
 * the grid [0, resolution)^3; d_rays and d_hits are device arrays of n entries. hit.t is the ray
 * parameter where the ray enters the hit voxel (t = tmax and hit = 0 for a miss); steps counts the
 * empty boxes crossed. Empty space is skipped in aligned boxes above the translation levels and
 * voxel by voxel inside translated boxes. Computed in double precision. */
typedef struct tdag16_ray {
    float origin[3];
    float direction[3];
    float tmin, tmax;
} tdag16_ray;
typedef struct tdag16_hit {
    float t;
    uint32_t voxel[3];
    uint32_t hit;
    uint32_t steps;
} tdag16_hit;
int tdag16_raycast(tdag_ctx* ctx, const tdag16_device* dev, const tdag16_ray* d_rays, uint64_t n, tdag16_hit* d_hits);

/* Lossless check of a .tdag16 against the SVDAG it encodes (device view, e.g. tdag_svdag_get_view):
 * the role of verifyComplexTransformDAG (transform_dag_encoding.h:81-117). Above box_level the two
 * structures are walked together and every child present on one side only counts as an existence
 * mismatch; at box_level (the highest level whose incoming pointers may carry a translation, else
 * the leaf level) every voxel of each reached box is compared. Empty regions are covered as well.
 * The encoding is lossless when both mismatch counts are 0. */
typedef struct tdag16_verify_stats {
    uint64_t existence_mismatches;
    uint64_t voxel_mismatches;
    uint64_t boxes_compared;
    uint64_t pairs_walked; /* (source node, .tdag16 node) pairs walked above box_level */
    uint32_t box_level;
    uint32_t reserved;
} tdag16_verify_stats;
int tdag16_verify(tdag_ctx* ctx, const tdag16_device* dev, const tdag_svdag_view* source_device, tdag16_verify_stats* out);

/* createLengthLimitedHuffmanCodeTable(frequencies, max_code_length) and, if lsb_first,
 * convertHuffmanToLSB (tools/svdag_encoding/src/huffman.h:22-25; huffman.cpp:165-182): the code of
 * every symbol (bit-reversed when lsb_first) and its length. The encoder uses it with the level's
 * pointer-type histogram and max_code_length 16. Host computation; needs no device. */
int tdag16_huffman_code_table(const uint64_t* frequencies, uint32_t n, uint32_t max_code_length, int lsb_first,
    uint64_t* out_codes, uint32_t* out_bits);

#ifdef __cplusplus
}
#endif

#endif /* TDAG16_H_ */

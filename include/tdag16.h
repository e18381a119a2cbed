/* tdag16.h — C ABI of the .tdag16 encoder in libtdag.so.
 *
 * Replaces constructTransformDAG16(EditStructure<void, TransformPointer>, const TransformDAGConfig&,
 * const TransformEncodingConfig&, DAGEncodingStats&)
 * (tools/svdag_encoding/src/transform_dag_encoding.h:232; transform_dag_encoding.cpp:240-497) followed
 * by BinaryWriter::write(TransformDAG16) (transform_dag_encoding.cpp:1023-1030), as the svdag_encoding
 * tool does for a .tdag16 output (tools/svdag_encoding/src/main.cpp:87-134).
 *
 * The result is the .tdag16 file image. It decodes to the same voxels as the reference's encoding of
 * the same transform DAG and uses the same Huffman tables; equal reference counts are ordered by
 * ascending item index and ascending pointer value, where the reference leaves the order to std::sort
 * and std::unordered_map iteration (so its bytes depend on the standard-library build).
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
} tdag_encoding_config;

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

#ifdef __cplusplus
}
#endif

#endif /* TDAG16_H_ */

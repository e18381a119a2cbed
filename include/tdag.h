/* tdag.h — C ABI of libtdag.so, the GB300 (sm_103a) Transform-Aware SVDAG construction library.
 *
 * Plain C: fixed-width integers, plain pointers and sizes; no C++ or torch types.
 * Every entry point returns an int status (TDAG_OK = 0). The message of the last failure on the
 * calling thread is returned by tdag_last_error_message().
 *
 * The layouts mirror the reference's in-memory structures, so a caller can hand its vectors over
 * without conversion:
 *   EditNode<uint32_t>           = 8 x uint32_t, empty child 0xFFFFFFFF
 *                                  (tools/lib/include/voxcom/voxel/structure.h:44-69)
 *   EditSubGrid<void>            = uint64_t Morton-order 4x4x4 occupancy mask (structure.h:116-125)
 *   EditNode<TransformPointer>   = 8 x uint64_t TransformPointer (transform_dag.h:19-33)
 *   TransformDAGConfig           = {bool symmetry, axisPermutation, translation; uint32_t maxTranslationLevel}
 *                                  (tools/lib/include/voxcom/voxel/transform_dag.h:157-160)
 */
#ifndef TDAG_H_
#define TDAG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TDAG_OK 0
#define TDAG_ERR_ARG 1 /* invalid argument / unsupported configuration */
#define TDAG_ERR_OOM 2 /* device or host allocation failed */
#define TDAG_ERR_TABLE_FULL 3 /* a bounded hash-table probe sequence ran out (never spins) */
#define TDAG_ERR_ALLOC 4 /* a bounded device sub-allocation failed */
#define TDAG_ERR_CUDA 5 /* a CUDA runtime call failed */
#define TDAG_ERR_CORRUPT 6 /* malformed input structure (dangling child pointer, bad sizes) */
#define TDAG_ERR_NO_DEVICE 7 /* no CUDA device / kernels not loadable for this GPU */
#define TDAG_ERR_INTERRUPTED 8 /* a build stopped where the caller asked; its checkpoint is on disk */

#define TDAG_MAX_LEVELS 32

typedef struct tdag_ctx tdag_ctx;

/* TransformDAGConfig (transform_dag.h:157-160). */
typedef struct tdag_config {
    int32_t symmetry; /* search mirror transforms */
    int32_t axis_permutation; /* search axis permutations */
    int32_t translation; /* run the translation matcher on levels 2..max_translation_level */
    uint32_t max_translation_level; /* 2..4 when translation != 0 (reference default 4) */
} tdag_config;

/* Read-only view of an EditStructure<void, uint32_t> (structure.h:159-211). Pointers are host
 * memory for tdag_build() and device memory for tdag_build_device(). nodes[l] holds node_counts[l]
 * EditNode<uint32_t> (8 x u32 each) for l in [3, root_level]; leaves holds the level-2 subgrids. */
typedef struct tdag_svdag_view {
    uint32_t resolution;
    uint32_t root_level;
    uint32_t structure_type; /* 0 = Tree, 1 = DAG (constructTransformDAG requires DAG) */
    uint32_t reserved;
    const uint32_t* nodes[TDAG_MAX_LEVELS];
    uint64_t node_counts[TDAG_MAX_LEVELS];
    const uint64_t* leaves;
    uint64_t leaf_count;
} tdag_svdag_view;

/* Per-level statistics of one build. Index = tree level (2 = leaves). */
typedef struct tdag_level_stats {
    uint64_t items; /* items entering the stage at this level */
    uint64_t unique; /* items kept */
    uint64_t probes; /* non-empty directional hash values looked up (translation levels) */
    uint64_t filter_pass; /* lookups that passed the membership filter */
    uint64_t hits; /* lookups that found a corner-hash range */
    uint64_t candidates; /* candidate (target, corner) pairs examined */
    uint64_t verifications; /* exact grid comparisons */
    uint64_t verified; /* comparisons that matched */
    uint64_t table_entries; /* corner views in the table (translation levels) */
    float search_ms; /* device time of the search kernels (probe and lookup) */
    float probe_ms; /* device time of the probe kernel alone */
} tdag_level_stats;

typedef struct tdag_stats {
    tdag_level_stats hierarchical[TDAG_MAX_LEVELS];
    tdag_level_stats translation[TDAG_MAX_LEVELS];
    float total_ms; /* device time of the whole construction (tdag_build*: without host copies) */
    float hierarchical_ms;
    float translation_ms;
    uint32_t table_regrows; /* class tables doubled after TDAG_ERR_TABLE_FULL (see tdag_tuning) */
    uint64_t kernel_launches; /* kernels this library launched for the construction */
} tdag_stats;

/* EditStructure<void, TransformPointer> result. Arrays are owned by the library: host memory from
 * tdag_build() (page-locked blocks the device writes directly; tdag_result_free keeps up to 2 GiB
 * of them for reuse by later calls), device memory from tdag_build_device(). Release with
 * tdag_result_free(), never with free(). */
typedef struct tdag_result {
    uint32_t resolution;
    uint32_t root_level;
    uint32_t structure_type; /* 0 (the reference's output EditStructure is default-constructed) */
    uint32_t on_device;
    uint64_t* nodes[TDAG_MAX_LEVELS]; /* node_counts[l] x 8 TransformPointer (u64) */
    uint64_t node_counts[TDAG_MAX_LEVELS];
    uint64_t* leaves;
    uint64_t leaf_count;
    tdag_stats stats;
} tdag_result;

/* Tuning knobs (0 = library default). */
typedef struct tdag_tuning {
    uint32_t filter_bits_per_key; /* membership filter size (power of two rounded) */
    uint32_t table_load_percent; /* corner-hash table load factor in percent (50..85) */
    uint32_t search_ctas_per_sm; /* persistent search CTAs per SM */
    uint32_t class_table_load_percent; /* initial load of the class tables of the hierarchical pass and
                                        * toDAG (default 50). A table whose bounded probes run out
                                        * (TDAG_ERR_TABLE_FULL on the device) is doubled and the pass
                                        * rerun; above 100 the first table is certain to be too small. */
    uint32_t table_regrow_limit; /* doublings allowed per table (default 4); past them the call
                                  * returns TDAG_ERR_TABLE_FULL */
    uint32_t slab_pool_slabs; /* initial spare slabs of each global slab hash table of the streamed
                               * scene build (0: one per bucket); a pool that runs out
                               * (TDAG_ERR_ALLOC on the device) is doubled and the insertion resumed */
    uint64_t device_memory_limit; /* bytes of device memory the context's calls may hold at once
                                   * (0 = no limit); an allocation past it fails with TDAG_ERR_OOM */
    uint32_t probe_bulk_copy; /* level-4 probe: 1 stages the source grids by a bulk copy (TMA) one
                               * source ahead; 0 (default) or 2 load them cooperatively */
    uint32_t verify_lanes; /* threads per exact subgrid verification in the lookup: 1, 4, 8 or 32
                            * (0 = 32, the whole warp); smaller groups verify 32 / lanes candidates
                            * side by side */
    uint32_t lookup_tile; /* probe records a lookup warp claims at a time when the records are
                           * balanced dynamically (fewer than 2^20): a multiple of 32 in 32..1024
                           * (0 = 32) */
    uint32_t reserved3;
} tdag_tuning;

/* Library/version information. */
const char* tdag_version(void);
const char* tdag_last_error_message(void);

/* Context = one CUDA device + one stream + a stream-ordered memory pool. Calls on one context are
 * serialised by the caller; separate contexts may be used from separate threads. */
int tdag_ctx_create(int device, const tdag_tuning* tuning, tdag_ctx** out_ctx);
int tdag_ctx_destroy(tdag_ctx* ctx);
/* Underlying cudaStream_t (as void*) for callers that want to order their own work with the library's. */
int tdag_ctx_stream(tdag_ctx* ctx, void** out_stream);

/* constructTransformDAG<Structure>(inDag, config)
 * (tools/lib/include/voxcom/voxel/transform_dag.h:161-162; tools/lib/src/voxel/transform_dag.cpp:138-240).
 * Input in host memory; result in host memory. Host<->device copies are part of the call. */
int tdag_build(tdag_ctx* ctx, const tdag_svdag_view* in_host, const tdag_config* config, tdag_result** out);

/* Same as tdag_build with the input already resident in device memory and the result left there. */
int tdag_build_device(tdag_ctx* ctx, const tdag_svdag_view* in_device, const tdag_config* config, tdag_result** out);

int tdag_result_free(tdag_result* result);

/* Host copy of a device-resident result (release both with tdag_result_free). */
int tdag_result_to_host(tdag_ctx* ctx, const tdag_result* device_result, tdag_result** host_out);

/* Batched constructTransformDAG (no reference counterpart: the reference builds one structure per
 * call). Builds `count` independent SVDAGs of any sizes together — every stage runs one set of
 * launches for the whole batch — and out[i] equals tdag_build of in[i] bit for bit. out must hold
 * `count` pointers, each released with tdag_result_free. batch_stats (may be NULL) receives the
 * statistics of the whole batch. Host in / host out, or device in / device out. */
int tdag_build_batched(tdag_ctx* ctx, const tdag_svdag_view* in_host, uint32_t count, const tdag_config* config,
    tdag_result** out, tdag_stats* batch_stats);
int tdag_build_batched_device(tdag_ctx* ctx, const tdag_svdag_view* in_device, uint32_t count, const tdag_config* config,
    tdag_result** out, tdag_stats* batch_stats);

/* Batched build captured in one CUDA graph (no reference counterpart; the host-side batching it
 * replaces is find_translation.cpp:661-664, 771). tdag_batch_graph_create builds the device-resident
 * batch once as tdag_build_batched_device does, recording every value the build reads back to steer
 * itself (compaction counts, scan totals, probe record counts, live table entries, status words),
 * and then captures the same build -- every stage of every level, for the whole batch -- into one
 * CUDA graph whose sizes and launch shapes are those values. The views' device arrays must stay
 * allocated while the graph lives; the graph snapshots their contents.
 * tdag_batch_graph_launch replays the graph: one cudaGraphLaunch, no host round trip inside the
 * build. It first compares the views' arrays with the snapshot on the device and returns
 * TDAG_ERR_ARG, without launching, if any word changed (a changed batch needs a new graph). Every
 * read the replay would have made is checked on the device against the recorded value; a
 * difference returns TDAG_ERR_CUDA. out[i] (device-resident, released with tdag_result_free) equals
 * tdag_build_batched_device's out[i] bit for bit. stats (may be NULL) receives total_ms (the
 * graph's device time) and kernel_launches (the graph's kernel nodes). Calls are synchronous on the
 * context's stream; launches need the context alive, tdag_batch_graph_free does not. Learned-proposal
 * hooks cannot be captured. */
typedef struct tdag_batch_graph tdag_batch_graph;
int tdag_batch_graph_create(tdag_ctx* ctx, const tdag_svdag_view* in_device, uint32_t count, const tdag_config* config,
    tdag_batch_graph** out);
int tdag_batch_graph_launch(tdag_batch_graph* graph, tdag_result** out, tdag_stats* stats);
int tdag_batch_graph_free(tdag_batch_graph* graph);

/* findDuplicatesAmongFlattenedItems_cpp2<Level>(items, grids, outPrevLevelMapping, config)
 * (transform_dag.h:307-308; tools/lib/src/voxel/find_translation.cpp:616-1000), on dense grids:
 * grids = n x (R^3 / 64) uint64 words, R = 1 << level, bit index x + R*y + R*R*z
 * (LargeSubGrid, tools/lib/include/voxcom/voxel/large_sub_grid.h:80-97). Host pointers.
 * out_mapping[n]: TransformPointer of every item into the unique list; out_unique[n]: positions of
 * the kept items (ascending); *n_unique: their count. stats may be NULL. */
int tdag_find_duplicates_level(tdag_ctx* ctx, uint32_t level, const uint64_t* grids, uint32_t n,
    const tdag_config* config, uint64_t* out_mapping, uint32_t* out_unique, uint32_t* n_unique,
    tdag_level_stats* stats);

/* No counterpart in the reference: tdag_find_duplicates_level for callers that cannot allocate
 * device memory (code inside a host application that owns all device memory, such as an engine's
 * fixed arena, or a memory-capped service where an allocation could fail or stall). Same result as
 * tdag_find_duplicates_level, but grids and outputs are DEVICE pointers and every temporary lives in
 * one 4 MiB array compiled into libtdag.so; the call makes no cudaMalloc/cudaFree. At most 4096
 * items per call (levels 2..4; larger calls return TDAG_ERR_ARG). The array is shared by all calls
 * on all contexts of a device: calls that overlap on the GPU race and must be serialised by the
 * caller. tdag_ctx_create resolves the array's address and loads this path's kernels, so the driver's
 * lazy loading places them at context creation, not inside a call. The call is synchronous on the
 * context's stream (it reads the device status word before returning). *d_n_unique is written on
 * the device. */
int tdag_find_duplicates_level_noalloc(tdag_ctx* ctx, uint32_t level, const uint64_t* d_grids, uint32_t n,
    const tdag_config* config, uint64_t* d_out_mapping, uint32_t* d_out_unique, uint32_t* d_n_unique);

/* No counterpart in the reference: tdag_find_duplicates_level on DEVICE grids and outputs, with an
 * optional subset of searching sources. d_sources == NULL: the exhaustive search (every item a
 * source). Otherwise only the num_sources listed item indices (distinct, < n) probe; every item is
 * still a target and every match is verified exactly, so the mapping is a valid one whose unique
 * set can only be larger than the exhaustive search's. *n_unique is written on the host. */
int tdag_find_duplicates_level_device(tdag_ctx* ctx, uint32_t level, const uint64_t* d_grids, uint32_t n,
    const tdag_config* config, const uint32_t* d_sources, uint32_t num_sources, uint64_t* d_out_mapping,
    uint32_t* d_out_unique, uint32_t* n_unique, tdag_level_stats* stats);

/* Learned-proposal extension (no counterpart in the reference). At every translation level the build
 * calls fn with the level's n flattened items (d_grids: device, R^3/64 words each, bit x + R*y + R^2*z)
 * before matching. fn writes up to n item indices into d_sources (device) -- the items allowed to
 * search as sources -- sets *num_sources and returns 0; any other return value aborts the build with
 * TDAG_ERR_ARG. fn must have finished its device writes when it returns. Only the listed items probe,
 * every match is verified exactly, and the result is a valid TDAG with possibly more nodes than the
 * exhaustive build. Single-grid builds only. */
typedef int (*tdag_proposal_fn)(void* user, uint32_t level, const uint64_t* d_grids, uint32_t n, uint32_t* d_sources,
    uint32_t* num_sources);
int tdag_build_device_proposed(tdag_ctx* ctx, const tdag_svdag_view* in_device, const tdag_config* config,
    tdag_proposal_fn fn, void* user, tdag_result** out);
/* Device-to-device copy of `bytes` on the context's stream, complete on return: lets proposal
 * functions written without CUDA bindings (ctypes) read d_grids and fill d_sources. */
int tdag_device_copy(tdag_ctx* ctx, void* d_dst, const void* d_src, uint64_t bytes);

/* constructTransformDAGHierarchical(inDag, config) (transform_dag.h:168-169;
 * tools/lib/src/voxel/transform_dag_hierarchical.cpp:304-529): symmetry + permutation only.
 * Host in, host out. */
int tdag_build_hierarchical(tdag_ctx* ctx, const tdag_svdag_view* in_host, const tdag_config* config, tdag_result** out);

/* StaticStructure (tools/lib/include/voxcom/voxel/structure.h:298-320, 765-798): the memory-lean
 * packed layout. Per level a word stream; every node is a header word (child mask, bit i = child i)
 * followed by one word per present child in child order, each the word offset of the child in the
 * level below (level 3: the leaf index). Input words are uint32_t (StaticStructure<void, uint32_t>),
 * output words uint64_t (StaticStructure<void, TransformPointer>: headers and TransformPointers). */
typedef struct tdag_static_view {
    uint32_t resolution;
    uint32_t root_level;
    uint32_t structure_type;
    uint32_t reserved;
    const uint32_t* words[TDAG_MAX_LEVELS]; /* host memory, levels 3..root_level */
    uint64_t word_counts[TDAG_MAX_LEVELS];
    const uint64_t* leaves;
    uint64_t leaf_count;
} tdag_static_view;

typedef struct tdag_static_result {
    uint32_t resolution;
    uint32_t root_level;
    uint32_t structure_type;
    uint32_t reserved;
    uint64_t* words[TDAG_MAX_LEVELS]; /* host memory owned by the library */
    uint64_t word_counts[TDAG_MAX_LEVELS];
    uint64_t* leaves;
    uint64_t leaf_count;
    tdag_stats stats;
} tdag_static_result;

/* constructStaticTransformDAG(StaticStructure<void, uint32_t>&&, config)
 * (tools/lib/include/voxcom/voxel/transform_dag.h:163; tools/lib/src/voxel/transform_dag.cpp:242-390).
 * The same construction as tdag_build, except that its hierarchical pass groups nodes by a hash of
 * their children's word offsets (transform_dag_hierarchical.cpp:531-743), which orders the levels
 * above the translation levels differently. Every node of a packed level must be referenced by the
 * level above (true of SVDAGs); a level holding unreferenced words is rejected (TDAG_ERR_CORRUPT).
 * Release the result with tdag_static_result_free. */
int tdag_build_static(tdag_ctx* ctx, const tdag_static_view* in_host, const tdag_config* config, tdag_static_result** out);
int tdag_static_result_free(tdag_static_result* result);

/* ------------------------------------------------------------------------------------------------
 * Input side of the path: procedural scenes, SVO construction and toDAG on the device.
 * (EditStructure(VoxelGrid), structure.h:423-429, 658-701; EditStructure::toDAG, structure.h:703-763.)
 * These have no C-ABI counterpart in the reference (it builds SVOs on the host); they produce the
 * same structures in device memory so the Transform-DAG build can start from HBM.
 * ------------------------------------------------------------------------------------------------ */
#define TDAG_SCENE_TERRAIN 0 /* solid fBm terrain: solid where fbm(v) - z/res > 0 */
#define TDAG_SCENE_PRIMITIVES 1 /* union of boxes, spheres and terrain blocks with transformed copies */

typedef struct tdag_scene {
    uint32_t kind; /* TDAG_SCENE_* */
    uint32_t resolution; /* power of two, 16 .. 16384 */
    uint32_t seed;
    uint32_t num_primitives; /* TDAG_SCENE_PRIMITIVES */
    uint32_t copy_percent; /* percent of primitives placed as mirrored / permuted / translated copies */
    uint32_t shell; /* 1: keep only the 1-voxel surface shell (6-neighbourhood) */
    uint32_t chunk_resolution; /* 0: automatic (streamed in 2048^3 chunks above 4096^3). Otherwise the
                                  grid is generated and deduplicated chunk by chunk (power of two in
                                  64..2048); the resulting SVDAG is the same. */
    uint32_t reserved;
} tdag_scene;

/* One primitive of a TDAG_SCENE_PRIMITIVES scene. A world voxel v is inside when
 * w = v - offset lies in [0, size[perm[k]]) per axis k, then mirrored axes map w_k -> E_k - 1 - w_k,
 * and the local voxel u (u[perm[k]] = w_k) is inside the shape:
 * box: always; sphere: |u - radius|^2 <= radius^2; terrain: fbm(u, seed) * size > u.z * 31 * 65535. */
typedef struct tdag_primitive {
    uint32_t type; /* 0 box, 1 sphere, 2 terrain block */
    uint32_t xform; /* permutation id (0..5, order 012 021 102 120 201 210) | mirror bits << 3 */
    int32_t size[3]; /* local extent per local axis */
    int32_t radius; /* sphere radius */
    int32_t offset[3]; /* world position of the transformed box's minimum corner */
    uint32_t seed; /* terrain noise seed */
    uint32_t source; /* primitive this one is a copy of (itself for originals) */
    uint32_t reserved;
} tdag_primitive;

typedef struct tdag_svdag tdag_svdag; /* device-resident EditStructure<void, uint32_t>, library-owned */

/* Primitive list of a scene (host computation, deterministic in scene->seed). */
int tdag_scene_primitives(const tdag_scene* scene, tdag_primitive* out, uint32_t capacity, uint32_t* count);
/* Generate the scene on the device, build its SVO and, if to_dag, deduplicate it (toDAG). */
int tdag_scene_svdag(tdag_ctx* ctx, const tdag_scene* scene, int to_dag, tdag_svdag** out);
/* tdag_scene_svdag (to_dag = 1) of a streamed scene (chunk_resolution set, or above 4096^3) with
 * checkpoints, for builds long enough to be interrupted (no counterpart in the reference, whose stage
 * files are its only checkpoints). After every `every_chunks` finished chunks (0: never) the build
 * writes its state -- the global levels' unique items, every finished chunk's root, the voxel count
 * and the next chunk -- to checkpoint_path (through a temporary file and a rename). If
 * checkpoint_path holds a checkpoint of the same scene, the build resumes from it; one of another
 * scene or a damaged one returns TDAG_ERR_CORRUPT. stop_after_chunks > 0 stops the call after that
 * many chunks, checkpoint written, with TDAG_ERR_INTERRUPTED. A resumed build's result is identical
 * to an uninterrupted build's. The caller removes the file when done. */
int tdag_scene_svdag_checkpointed(tdag_ctx* ctx, const tdag_scene* scene, const char* checkpoint_path, uint32_t every_chunks,
    uint32_t stop_after_chunks, tdag_svdag** out);
/* Same from a host dense grid: dense[x + res*y + res*res*z] != 0 means solid. */
int tdag_svdag_from_dense(tdag_ctx* ctx, const uint8_t* dense, uint32_t resolution, int to_dag, tdag_svdag** out);
/* Device-pointer view (valid until tdag_svdag_free), the number of solid voxels of the grid, and
 * host copies of one level (level 2 = leaves: leaf_count x 8 bytes; level >= 3: node_counts x 32 bytes). */
int tdag_svdag_get_view(const tdag_svdag* svdag, tdag_svdag_view* out_device_view);
int tdag_svdag_voxel_count(const tdag_svdag* svdag, uint64_t* out);
int tdag_svdag_copy_level(tdag_ctx* ctx, const tdag_svdag* svdag, uint32_t level, void* host_dst, uint64_t dst_bytes);
int tdag_svdag_free(tdag_svdag* svdag);

#ifdef __cplusplus
}
#endif

#endif /* TDAG_H_ */

// A plain C++ caller of the batch graph through the C ABI only (no CUDA headers): device scenes from
// tdag_scene_svdag, one graph over them, two launches, each result compared word for word with
// tdag_build_batched_device's. Exit code 0 when equal; 10 + a status code when a call fails; 2 on a
// mismatch.
#include <cstdio>
#include <cstring>
#include <vector>

#include "tdag.h"

static int check(int rc, const char* what)
{
    if (rc != TDAG_OK)
        std::fprintf(stderr, "%s: %s\n", what, tdag_last_error_message());
    return rc;
}

static bool same(const tdag_result* a, const tdag_result* b)
{
    if (a->root_level != b->root_level || a->leaf_count != b->leaf_count || std::memcmp(a->leaves, b->leaves, a->leaf_count * 8) != 0)
        return false;
    for (uint32_t l = 3; l <= a->root_level; ++l)
        if (a->node_counts[l] != b->node_counts[l] || std::memcmp(a->nodes[l], b->nodes[l], a->node_counts[l] * 64) != 0)
            return false;
    return true;
}

int main()
{
    tdag_ctx* ctx = nullptr;
    if (int rc = check(tdag_ctx_create(0, nullptr, &ctx), "tdag_ctx_create"))
        return 10 + rc;
    const uint32_t res[3] = { 64, 128, 64 };
    std::vector<tdag_svdag*> scenes(3, nullptr);
    std::vector<tdag_svdag_view> views(3);
    for (uint32_t g = 0; g < 3; ++g) {
        tdag_scene sc {};
        sc.kind = TDAG_SCENE_PRIMITIVES;
        sc.resolution = res[g];
        sc.seed = 40 + g;
        sc.num_primitives = 20 + 30 * g;
        sc.copy_percent = 30;
        sc.shell = 1;
        if (int rc = check(tdag_scene_svdag(ctx, &sc, 1, &scenes[g]), "tdag_scene_svdag"))
            return 10 + rc;
        tdag_svdag_get_view(scenes[g], &views[g]);
    }
    const tdag_config cfg { 1, 1, 1, 4 };
    std::vector<tdag_result*> eager(3, nullptr), host(3, nullptr);
    if (int rc = check(tdag_build_batched_device(ctx, views.data(), 3, &cfg, eager.data(), nullptr), "tdag_build_batched_device"))
        return 10 + rc;
    for (uint32_t g = 0; g < 3; ++g)
        if (int rc = check(tdag_result_to_host(ctx, eager[g], &host[g]), "tdag_result_to_host"))
            return 10 + rc;
    tdag_batch_graph* graph = nullptr;
    if (int rc = check(tdag_batch_graph_create(ctx, views.data(), 3, &cfg, &graph), "tdag_batch_graph_create"))
        return 10 + rc;
    int status = 0;
    for (int launch = 0; launch < 2 && status == 0; ++launch) {
        std::vector<tdag_result*> out(3, nullptr);
        tdag_stats st;
        if (int rc = check(tdag_batch_graph_launch(graph, out.data(), &st), "tdag_batch_graph_launch"))
            return 10 + rc;
        for (uint32_t g = 0; g < 3; ++g) {
            tdag_result* h = nullptr;
            if (int rc = check(tdag_result_to_host(ctx, out[g], &h), "tdag_result_to_host"))
                return 10 + rc;
            if (!same(h, host[g])) {
                std::fprintf(stderr, "launch %d, grid %u differs from the eager batch\n", launch, g);
                status = 2;
            }
            tdag_result_free(h);
            tdag_result_free(out[g]);
        }
    }
    tdag_batch_graph_free(graph);
    for (uint32_t g = 0; g < 3; ++g) {
        tdag_result_free(eager[g]);
        tdag_result_free(host[g]);
        tdag_svdag_free(scenes[g]);
    }
    tdag_ctx_destroy(ctx);
    return status;
}

/* tdag_nn.h — kernels of the learned source proposal (an approximate build mode with no counterpart
 * in the reference; every match it proposes is verified exactly by the matcher, see tdag.h's
 * tdag_build_device_proposed and tdag_find_duplicates_level_device).
 *
 * Two encoders share the kernels. The block encoder is an MLP 64 -> 256 -> 256 -> 32 over the 64-bit
 * occupancy masks of an item's 4^3 blocks, mean-pooled over the item's non-empty blocks and
 * L2-normalised. The hierarchical encoder embeds a 4^3 item by the same leaf MLP, and an 8^3 or 16^3
 * item by an MLP 256 -> 256 -> 256 -> 32 of its level over its eight children's vectors placed in a
 * canonical octant order (tdag_nn_canon_gather). Both are trained with a
 * symmetric InfoNCE loss and AdamW on FP32 master weights. Its dense layers, the InfoNCE logits and
 * the candidate-scoring dot products run as bf16 GEMMs on the tcgen05 tensor cores (operands staged
 * in shared memory, FP32 accumulators in tensor memory); everything else is plain CUDA.
 *
 * All pointers are device pointers; every call is enqueued on the context's stream (tdag_ctx_stream)
 * and returns without synchronising, except where noted. bf16 values are passed as uint16_t bit
 * patterns. Error codes are those of tdag.h; TDAG_ERR_CUDA also reports a tensor-core wait that did
 * not complete within its bound (the kernel then frees its tensor memory and returns).
 */
#ifndef TDAG_NN_H
#define TDAG_NN_H

#include <stddef.h>
#include <stdint.h>

#include "tdag.h"

#ifdef __cplusplus
extern "C" {
#endif

/* How a GEMM operand with R rows (M for A, N for B) and K columns is stored. */
enum {
    TDAG_NN_KMAJOR = 0,  /* bf16, element (r, k) at ptr[r * ld + k]; ptr 16-byte aligned, ld % 8 == 0 */
    TDAG_NN_MNMAJOR = 1, /* bf16, element (r, k) at ptr[k * ld + r] */
    TDAG_NN_BITS = 2,    /* uint64 masks, element (r, k) = bit k of ptr[r] as 1.0 or 0.0; K == 64 */
    TDAG_NN_BITS_T = 3   /* uint64 masks, element (r, k) = bit r of ptr[k]; R <= 64 */
};

typedef struct tdag_nn_operand {
    const void* ptr;
    uint32_t mode; /* TDAG_NN_* */
    uint32_t ld;   /* leading dimension in elements (ignored for the bit modes) */
} tdag_nn_operand;

/* C[m][n] = epilogue(alpha * sum_k A(m, k) * B(n, k)), FP32 accumulation, for m < M, n < N:
 *   + bias[n] (if bias), then max(., 0) (if relu), then 0 where gate[m * ld_gate + n] (bf16) is not
 *   > 0 (if gate: the ReLU derivative of a stored activation). C is FP32 (c_bf16 == 0) or bf16
 *   (round to nearest even), element (m, n) at c[m * ldc + n].
 * K must be a positive multiple of 16; M, N >= 1. */
int tdag_nn_gemm(tdag_ctx* ctx, const tdag_nn_operand* a, const tdag_nn_operand* b, uint32_t m, uint32_t n, uint32_t k, float alpha,
    const float* bias, int relu, const uint16_t* gate, uint32_t ld_gate, void* c, uint32_t ldc, int c_bf16);

/* The 64-bit occupancy mask of every 4^3 block of n items of a translation level (R = 2^level,
 * level 2..4; item words bit x + R y + R^2 z): masks[i * B + b], B = (R/4)^3 blocks, block
 * b = bx + (R/4) by + (R/4)^2 bz, mask bit dx + 4 dy + 16 dz. */
int tdag_nn_block_masks(tdag_ctx* ctx, const uint64_t* words, uint32_t n, uint32_t level, uint64_t* masks);

/* Mean over each item's non-empty blocks (mask != 0) of the 32-wide block outputs, row r = i * B + b
 * of z (or row row_of[i * B + b] when row_of is given: the MLP then ran once per distinct mask), then
 * L2 normalisation: u[i * 32 + d] (FP32) and u_bf16 (optional), norm[i] (the pre-normalisation
 * length, floored at 1e-12) and count[i] (non-empty blocks, floored at 1). */
int tdag_nn_pool_forward(tdag_ctx* ctx, const float* z, const uint32_t* row_of, const uint64_t* masks, uint32_t n, uint32_t blocks, float* u,
    uint16_t* u_bf16, float* norm, float* count);

/* Gradient of pool_forward: from du (FP32, n x 32) to dz (bf16, (n * B) x 32); zero for empty blocks. */
int tdag_nn_pool_backward(tdag_ctx* ctx, const float* du, const float* u, const float* norm, const float* count, const uint64_t* masks,
    uint32_t n, uint32_t blocks, uint16_t* dz);

/* Symmetric InfoNCE with in-batch negatives over logits[i * b + j] = <t_i, p_j> / tau (FP32, b x b):
 * loss = (CE over rows + CE over columns) / 2, labels on the diagonal. Writes *loss_dev (FP32, one
 * value) and the gradient with respect to the logits, dlogits (bf16, b x b). */
int tdag_nn_info_nce(tdag_ctx* ctx, const float* logits, uint32_t b, float* loss_dev, uint16_t* dlogits);

/* out[n] = sum over m < M of x[m * ldx + n] (bf16 x; FP32 out, overwritten). */
int tdag_nn_column_sums(tdag_ctx* ctx, const uint16_t* x, uint32_t m, uint32_t n, uint32_t ldx, float* out);

/* One AdamW step (decoupled weight decay) of `count` FP32 master weights with FP32 gradients and
 * moments; `step` counts from 1. Writes the updated weights' bf16 copy to w_bf16 (optional). */
int tdag_nn_adamw(tdag_ctx* ctx, float* w, const float* grad, float* m1, float* m2, uint64_t count, float lr, float beta1, float beta2,
    float eps, float weight_decay, uint32_t step, uint16_t* w_bf16);

/* Candidate scoring: for every row i < n of emb (bf16, n x 32, items in source order), the k rows
 * j < i with the largest <emb_i, emb_j> (tensor-core dot products, FP32 accumulation). Writes
 * idx[i * k + s] (j, or -1 where fewer than k exist) and score[i * k + s] (optional), in no
 * particular order; k is 8, 16 or 32. */
int tdag_nn_topk(tdag_ctx* ctx, const uint16_t* emb, uint32_t n, uint32_t k, int32_t* idx, float* score);

/* The upper levels' encoder input: each item's eight children pooled under a canonical axis order.
 * Item i has children o = ox + 2 oy + 4 oz (its octants); child o's 32-wide vector is row
 * child_row[i * 8 + o] of child (FP32, child_rows rows; -1: an empty child, a zero vector). With b
 * the item's child occupancy byte (bit o set for a non-empty child) and t the first of the 48
 * transforms (ID sym | perm << 3) whose image of b is the smallest, child o goes to slot pos_t(o),
 * its octant under t: x[i * 256 + 32 * slot + d] (bf16) = child[row * 32 + d], zeros for empty
 * children; slot_of[i * 8 + o] receives each child's slot. A row >= child_rows is recorded as
 * TDAG_ERR_ARG (reported by tdag_nn_sync) and read as an empty child. */
int tdag_nn_canon_gather(tdag_ctx* ctx, const float* child, uint32_t child_rows, const int32_t* child_row, uint32_t n, uint16_t* x,
    uint8_t* slot_of);

/* Gradient of tdag_nn_canon_gather: dchild[row * 32 + d] += dx[i * 256 + 32 * slot_of[i * 8 + o] + d]
 * for every non-empty child o of every item i (FP32 atomics, so rows may be shared); dx is FP32, or
 * bf16 when dx_bf16 != 0. dchild (child_rows rows) is accumulated into, not overwritten. */
int tdag_nn_canon_scatter(tdag_ctx* ctx, const void* dx, int dx_bf16, const int32_t* child_row, const uint8_t* slot_of, uint32_t n,
    float* dchild, uint32_t child_rows);

/* Synchronises the context's stream and returns the first error a kernel of this header recorded
 * (a tensor-core wait past its bound: TDAG_ERR_CUDA), clearing it. */
int tdag_nn_sync(tdag_ctx* ctx);

/* Convert n FP32 values to bf16 (round to nearest even). */
int tdag_nn_to_bf16(tdag_ctx* ctx, const float* x, uint64_t n, uint16_t* out);

#ifdef __cplusplus
}
#endif

#endif

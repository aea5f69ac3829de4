/* Compiles and links as plain C11 against include/stntt.h and libstntt: the
 * calls a C host makes for single transforms, uneven batches, device-side
 * parameters, TMA-staged passes and the allocation-free entry point. Not run
 * by the tests (it would need a GPU); linking checks every symbol. */
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#include "stntt.h"

int run(void *d_a, void *d_b, uint64_t *d_params, stntt_stream stream) {
    stntt_ctx *ctx = NULL;
    if (stntt_init(&ctx, 0) != STNTT_OK)
        return 1;
    uint32_t p = 0, root = 0;
    int rc = stntt_params_u32(12, &p, &root);
    if (rc == STNTT_OK)
        rc = stntt_find_params_device(1u << 12, 11, d_params, stream);
    if (rc == STNTT_OK)
        rc = stntt_ntt_gl64(ctx, (uint64_t *)d_a, 18, 1, STNTT_FORWARD, stream);
    stntt_job jobs[2] = {
        {STNTT_FIELD_GL64, 18, STNTT_FORWARD, 0, 0, 0, d_a},
        {STNTT_FIELD_U32, 12, STNTT_INVERSE, p, root, 0, d_b},
    };
    stntt_batch *b = NULL;
    if (rc == STNTT_OK)
        rc = stntt_batch_create(ctx, jobs, 2, &b);
    if (rc == STNTT_OK)
        rc = stntt_batch_launch(b, stream);
    if (rc == STNTT_OK)
        rc = stntt_batch_status(b);
    if (b)
        stntt_batch_destroy(b);
    const uint32_t logs[2] = {7, 11};
    if (rc == STNTT_OK)
        rc = stntt_set_plan_batched(ctx, STNTT_FIELD_GL64, 18, 2, logs);
    if (rc == STNTT_OK)
        rc = stntt_set_tma(ctx, 1);
    if (rc == STNTT_OK)
        rc = stntt_device_status(ctx);
    if (rc == STNTT_OK)
        rc = stntt_ntt_gl64_noalloc((const uint64_t *)d_a, (uint64_t *)d_b, 16, 1, STNTT_INVERSE, stream);
    if (rc != STNTT_OK)
        fprintf(stderr, "%s: %s\n", stntt_status_string(rc), stntt_last_error(ctx));
    stntt_destroy(ctx);
    return rc;
}

int main(void) { return 0; }

// qew_rk_resident.cu -- form selection for rk_block.
#include "qew_rk_internal.cuh"

qew_status qew_rk_block_dispatch(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                                 const qew_params *p, const qew_rk_params *rp,
                                 qew_rk_result *res) {
    return qew_rk_block_plain(ctx, field, d_h, n, p, rp, res);
}

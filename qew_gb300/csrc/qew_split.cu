// qew_split.cu -- FP32 split-index gather (placeholder until implemented).
#include "qew_internal.cuh"
#include "qew_model_kernels.cuh"

qew_status qew_gradient_split_enqueue(qew_ctx *ctx, const qew_field *field, const double *d_h,
                                      int n, const qew_params *p, double *d_grad) {
    (void)field; (void)d_h; (void)n; (void)p; (void)d_grad;
    return qew_fail(ctx, QEW_ERR_UNSUPPORTED, "FP32 split gather not built yet");
}

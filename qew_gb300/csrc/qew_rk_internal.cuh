// qew_rk_internal.cuh -- Rosso-Krauth entry points shared between forms.
#pragma once

#include "qew_internal.cuh"

qew_status qew_rk_validate(qew_ctx *ctx, int n, const qew_params *p, const qew_rk_params *rp);
// precision: QEW_PREC_FP64 or QEW_PREC_FP64_REFERENCE (the reference's
// arithmetic bit for bit).
qew_status qew_rk_block_plain(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                              const qew_params *p, const qew_rk_params *rp, qew_rk_result *res,
                              int precision);
// Chooses the persistent form when available, else the host-driven one.
qew_status qew_rk_block_dispatch(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                                 const qew_params *p, const qew_rk_params *rp,
                                 qew_rk_result *res);
// Persistent cooperative form; precision QEW_PREC_FP64, QEW_PREC_FP64_REFERENCE
// or QEW_PREC_FP32_SPLIT (velocities from the FP32 coefficients, heights and
// the update in FP64).
qew_status qew_rk_block_resident(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                                 const qew_params *p, const qew_rk_params *rp, int precision,
                                 qew_rk_result *res);

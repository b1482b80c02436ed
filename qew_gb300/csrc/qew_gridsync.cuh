// qew_gridsync.cuh -- bounded grid barrier for cooperative persistent kernels.
//
// Thread 0 of each CTA arrives on a counter; the last arrival resets it and
// bumps a generation word; the others poll the generation with a bounded
// number of polls. A wait that gives up sets `err` (every other CTA then
// stops waiting too) and the barrier returns false, so a kernel can leave
// its loop and the host can report QEW_ERR_TIMEOUT instead of hanging. Only
// use it in kernels launched with cudaLaunchCooperativeKernel, which
// guarantees that every CTA is resident.
#pragma once

#include "qew_internal.cuh"

constexpr long long kGridBarrierPolls = 1LL << 26;  // ~4 s of 64 ns polls

struct GridSync {
    unsigned int count;   // arrivals in the current generation
    unsigned int gen;     // barrier generation
    int err;              // set when a wait gave up
    int skip_block;       // a CTA that never arrives (a test's injected fault), -1: none
    long long max_polls;  // polls before a wait gives up
};

// Fresh barrier state for one launch, with the context's limits.
static __global__ void k_gridsync_init(GridSync *s, long long max_polls, int skip_block) {
    s->count = 0;
    s->gen = 0;
    s->err = 0;
    s->skip_block = skip_block;
    s->max_polls = max_polls;
}
static inline qew_status qew_gridsync_init(qew_ctx *ctx, GridSync *s) {
    k_gridsync_init<<<1, 1, 0, ctx->stream>>>(s, ctx->barrier_polls, ctx->barrier_skip);
    return qew_launch_check(ctx, "gridsync_init");
}

__device__ __forceinline__ bool grid_sync_bounded(GridSync *s, unsigned int nblocks) {
    __syncthreads();
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        volatile unsigned int *vgen = &s->gen;
        volatile int *verr = &s->err;
        if ((int)blockIdx.x == s->skip_block) {
            s_ok = 0;  // leaves without arriving: the other CTAs' waits run out
        } else {
            const long long limit = s->max_polls;
            const unsigned int g = *vgen;
            __threadfence();
            if (atomicAdd(&s->count, 1u) == nblocks - 1) {
                s->count = 0;
                __threadfence();
                atomicAdd(&s->gen, 1u);
            } else {
                long long polls = 0;
                while (*vgen == g && !*verr) {
                    if (++polls > limit) {
                        atomicExch(&s->err, 1);
                        break;
                    }
                    __nanosleep(64);
                }
            }
            __threadfence();
            s_ok = *verr ? 0 : 1;
        }
    }
    __syncthreads();
    return s_ok != 0;
}

// qew_nvtx.cuh -- NVTX ranges around the library's compute entry points: the
// counterpart of the reference's Kokkos kernel labels (qew_model.h:62, 164,
// 178), which reach a profiler through Kokkos Tools. Here Nsight Systems, or
// Nsight Compute's --nvtx filters, see each entry-point call as a range named
// for the function. NVTX is header-only: with no tool attached a range costs a
// load and a branch. -DQEW_NO_NVTX compiles the ranges out.
#pragma once

#ifndef QEW_NO_NVTX
#include <nvtx3/nvToolsExt.h>

struct QewRange {
    explicit QewRange(const char *name) { nvtxRangePushA(name); }
    ~QewRange() { nvtxRangePop(); }
    QewRange(const QewRange &) = delete;
    QewRange &operator=(const QewRange &) = delete;
};
#define QEW_RANGE() QewRange qew_range_(__func__)
#else
#define QEW_RANGE() ((void)0)
#endif

// qew_serve_lane.cuh -- the server's device-resident loop for static lines
// (qew_ensemble.cu): a persistent grid takes jobs from a ring in mapped host
// memory while the host keeps publishing them.
#pragma once

#include "qew_internal.cuh"

constexpr int kLaneRing = 1024;  // jobs in flight at most (published, not yet collected)

struct StaticLane;
// nmax: longest line; lp: the L-BFGS parameters of every job (FP64 phase);
// ftol32 > 0: an FP32 phase to that tolerance first; ctas: persistent CTAs.
qew_status qew_lane_create(int device, int nmax, const qew_lbfgs_params *lp, double ftol32,
                           int ctas, StaticLane **out);
// Makes job k = the number of jobs published before it readable to the
// grid; the field and line must already be on the device.
qew_status qew_lane_publish(StaticLane *L, const qew_field *f, double *d_h, int n,
                            const qew_params *p, double shift, unsigned int *k);
// (Re)launches the grid when it has left with published jobs unclaimed.
qew_status qew_lane_pump(StaticLane *L, cudaStream_t aux);
// True (and the result) once job k is finished.
bool qew_lane_done(StaticLane *L, unsigned int k, qew_lbfgs_result *r);
uint64_t qew_lane_launches(const StaticLane *L);
// Lets the grid leave, waits for it and frees everything.
void qew_lane_destroy(StaticLane *L);

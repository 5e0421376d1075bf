// What the request server (gnc_serve.cu) needs from the plan (gnc_api.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "../../include/guanaco_gb300.h"

namespace gnc {

// GNC_OK, or the status gnc_fbp_plan_create would return for d (and its message).
int desc_check(const gnc_fbp_desc *d);
// Device bytes of a plan for d plus one request's input and output buffers.
size_t plan_bytes(const gnc_fbp_desc *d);
// Requests with equal keys share a plan and its captured launches.
std::string plan_key(const gnc_fbp_desc *d);
// Size of the per-request parameter block of a plan.
size_t plan_param_bytes(const gnc_fbp_plan *p);
// Fills host_block (page-locked) for request d and enqueues its copy on s.
int plan_set_request(gnc_fbp_plan *p, const gnc_fbp_desc *d, unsigned char *host_block,
                     cudaStream_t s);
// The plan's device error word (bounded waits that gave up).
int *plan_error_word(gnc_fbp_plan *p);
// gnc_fbp_plan_create with the plan's device memory allocated from `pool`,
// ordered on stream `alloc` (cudaMallocFromPoolAsync; freed with
// cudaFreeAsync on the same stream when the plan is destroyed, so neither
// synchronises the device).  Its buffers may be used on another stream once
// `alloc` has been synchronised (or waited on with an event).
int plan_create_pooled(const gnc_fbp_desc *d, cudaMemPool_t pool, cudaStream_t alloc,
                       gnc_fbp_plan **out);

}  // namespace gnc

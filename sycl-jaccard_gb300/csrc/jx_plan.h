// Launch plan of the fused operator, shared by the operator, the batch runtime and the
// server: grid sizes and class-stream capacities.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/jx.h"

namespace jx {

struct Plan {
  int b2_ctas;      // CTAs of the B2 kernel (one class-stream region per warp)
  int hub_clusters; // 8-CTA clusters of the hub kernel (one bitmap slot each)
  int cap_b2, cap_hub;
  int b1_ctas;      // CTAs of the warp-per-row kernel
  int b0_ctas;      // CTAs of the lane-per-task kernel
};

Plan default_plan();
// Workspace bytes of one call under plan P.
size_t plan_workspace(int32_t n, int32_t e, bool weighted_vc, const Plan &P);
// The fused operator under plan P (arguments as jx_jaccard_ws; workspace >= plan_workspace).
jx_status run_plan(const jx_csr &g, const float *vertex_w, float *out, jx_algo algo, void *workspace,
                   const Plan &P, cudaStream_t s);

} // namespace jx

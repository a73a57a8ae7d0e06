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
  int hub_clusters; // clusters of the hub kernel (one bitmap slot each)
  int cap_b2, cap_hub;
  int b1_ctas;      // CTAs of the warp-per-row kernel (0: as many as fit on the GPU at once)
  int b0_ctas;      // CTAs of the lane-per-task kernel
  // cap_b2 holds every match of any CTA-bin task (8 * cap_b2 >= the largest CTA-bin row degree
  // the graph can have): the CTA kernel then skips the overflow bookkeeping
  bool b2_exact = false;
  // degree bins: lane rows d <= b0_max (<= 32), warp rows d <= b1_max (<= 512), CTA rows
  // d <= b2_max (<= 24576), hub rows above; hub rows split into work units of hub_unit tasks
  // (R-MAT 24 weighted, 4-CTA clusters, units of 8192 / 32768 / 65536 / 131072 tasks: hub kernel
  // 172 / 153 / 149 / 152 ms), a hub warp takes at most hub_batch tasks per fetch (8-CTA
  // clusters with 32 / 8 / 4 / 2 / 1: 293 / 214 / 198 / 188 / 186 ms; 4-CTA clusters with
  // 4 / 2 / 1: 155 / 152 / 152 ms)
  int32_t b0_max = 32, b1_max = 512, b2_max = 24576;
  int32_t hub_unit = 65536, hub_batch = 2;
  // one persistent launch over the CTA, warp and lane rows on b2_ctas CTAs, instead of one
  // kernel per bin
  bool persistent = false;
  // the hub kernel runs on a second stream beside the row kernels (they read the same inputs and
  // write disjoint outputs, so CTA rows fill the SMs the hub clusters leave free); class streams
  // then need separate regions.  Off: the kernels run one after the other on the call's stream.
  bool hub_beside = false;
  // CTAs per hub cluster (4 or 8): smaller clusters fit more SMs at once (on GB300 only 15
  // clusters of 8 fit, leaving 32 of the 152 SMs idle), each adds a bitmap
  int hub_cluster = 8;
  // the row kernels work on vertex ids relabelled by plan position (hubs first, each bin by
  // descending log2 degree), the lists staying in place; costs a copy of col in the workspace.
  // Off by default: R-MAT 24 weighted 660 ms with it against 615 ms without (its own ids are
  // already degree-ordered), relabelled R-MAT 24 689 against 744 ms.
  bool relabel = false;
};

Plan default_plan();
// Clusters of `cluster_size` (4 or 8) hub CTAs that can be resident at once on this device.
int hub_cluster_count(int cluster_size);
// P with its class-stream capacities cut to what a graph of e edges and the given maximum
// degree can use.  max_degree must be an upper bound of the graph's largest degree (-1:
// unknown); results do not depend on the capacities as long as it is.
Plan fit_plan(Plan P, int64_t e, int64_t max_degree);
// P with the fields a schedule sets (zero fields keep P's), then fitted to the graph.
Plan apply_schedule(Plan P, const jx_schedule *sch, int64_t e, int64_t max_degree);
// Workspace bytes of one call under plan P.
size_t plan_workspace(int32_t n, int32_t e, bool weighted_vc, const Plan &P);
// The fused operator under plan P (arguments as jx_jaccard_ws; workspace >= plan_workspace).
// row_sums (weighted vertex-centric only): per-vertex sums of the neighbours' weights computed
// earlier (jx_rowsum) and kept on the device; the call then skips its row-sum kernel.
jx_status run_plan(const jx_csr &g, const float *vertex_w, float *out, jx_algo algo, void *workspace,
                   const Plan &P, cudaStream_t s, const float *row_sums = nullptr);

// Turn graph-local row offsets / column ids packed back to back into super-CSR ones: rows of
// graph g get +ebase[g], columns +vbase[g] (device arrays of ngraphs + 1 bases).
jx_status shift_to_super(int64_t nv, int64_t ne, int32_t ngraphs, const int64_t *vbase, const int64_t *ebase,
                         int32_t *row_ptr, int32_t *col, cudaStream_t s);

} // namespace jx

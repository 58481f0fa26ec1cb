// What the batch (batch.cpp) needs of an instance beyond the C ABI: its step graph,
// to become one child of the batch's step graph, and the host side of the steps the
// batch graph ran (context.cu).
#pragma once
#include <cuda_runtime.h>

#include "../../include/cuibm.h"

extern "C" {
// The instance's step graph, or null when its steps need host work between them (no
// step graph, per-phase profiling, or a hierarchy rebuilt as an embedded body moves).
cudaGraph_t cuibm_batch_member_graph(cuibm_ctx *h);
// The instance's stream (its work outside the batch graph runs there).
cudaStream_t cuibm_batch_member_stream(cuibm_ctx *h);
// Account for n steps the batch graph ran for the instance.
void cuibm_batch_member_advance(cuibm_ctx *h, int n);
}

// Internal interface between the EDT entry point (edt.cu) and the 2-D/3-D
// unit-spacing fast path (edt_compact.cu).
#pragma once

#include "tm_common.cuh"

namespace tmc {

bool edt_compact_eligible(const Geometry &g, bool unit);
size_t edt_compact_workspace(const Geometry &g);
int edt_compact_run(const void *input, int in_dtype, const Geometry &g, float *dist, int32_t *indices,
                    int32_t *sqdist, unsigned char *ws, cudaStream_t stream);

}  // namespace tmc

// Binary morphology of 1-D / 2-D items on bit-packed tiles (bitmorph.cu),
// used by the uniform (morphology.cu) and ragged (ragged.cu) binary
// operators.  kind: 0 erosion, 1 dilation, 2 opening, 3 closing (one
// iteration each).  *done = false, with nothing launched, when the
// structure is beyond the kernel's limits; the caller then uses its own path.
#pragma once

#include "tm_common.cuh"

namespace tmc {

int bitmorph_uniform(int kind, const uint8_t *in, uint8_t *out, int64_t batch, int ndim, const int64_t *shape,
                     const uint8_t *structure, const int64_t *sshape, const int64_t *origin, int border,
                     cudaStream_t s, bool *done);
int bitmorph_ragged(int kind, const uint8_t *in, uint8_t *out, const void *plan, const uint8_t *structure,
                    const int64_t *sshape, const int64_t *origin, int border, cudaStream_t s, bool *done);

}  // namespace tmc

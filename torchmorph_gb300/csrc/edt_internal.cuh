// Internal interface between the EDT / chamfer entry points (edt.cu,
// cdt.cu) and the 2-D/3-D unit-spacing fast paths (edt_compact.cu).
#pragma once

#include "tm_common.cuh"

namespace tmc {

bool edt_compact_eligible(const Geometry &g, bool unit);
size_t edt_compact_workspace(const Geometry &g);
int edt_compact_run(const void *input, int in_dtype, const Geometry &g, float *dist, int32_t *indices,
                    int32_t *sqdist, unsigned char *ws, cudaStream_t stream);

// Chamfer distances without indices for 3-D items (bitmap shell search);
// items it cannot finish are marked in *todo_out (device int per item) for
// the raster passes.  ws: cdt_shell_workspace(g) bytes.
bool cdt_shell_eligible(const Geometry &g, const float *dist, const int32_t *indices);
size_t cdt_shell_workspace(const Geometry &g);
int cdt_shell_run(const void *input, int in_dtype, const Geometry &g, int metric, float *dist, unsigned char *ws,
                  int **todo_out, cudaStream_t stream);

}  // namespace tmc

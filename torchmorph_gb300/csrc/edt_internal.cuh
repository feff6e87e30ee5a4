// Internal interface between the EDT / chamfer entry points (edt.cu,
// cdt.cu) and the 2-D/3-D unit-spacing fast paths (edt_compact.cu).
#pragma once

#include "tm_tma.cuh"

namespace tmc {

// One item of a ragged EDT batch, as tm_ragged_edt_plan writes it.
struct ReItem {
    int64_t off;            // first voxel of the item in the packed buffers
    int shape[3];           // (D, H, W) or (H, W, 1)
    int plane_begin;        // 3-D items: the item's first axis-0 plane in the batch
    int64_t line_begin[3];  // first line of the item along each axis
};
static_assert(sizeof(ReItem) == 48, "descriptor layout");

// Ragged batches of 3-D items whose axes are all at most ragged_edt3_max_line():
// one cooperative launch (pass 0 over every column, then passes 1 + 2 fused per
// plane on chip, the uniform fused path's plane code).  cols = total voxel
// columns along axis 0 (sum of H * W), c1 = `total` int16 of workspace.
int ragged_edt3_max_line();
int ragged_edt3_run(const void *input, int in_f32, const ReItem *items, int nitems, int64_t cols, int64_t total,
                    int max_line, int16_t *c1, float *dist, int32_t *indices, int32_t *sqdist, GridControl *ctl,
                    cudaStream_t stream);

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
                  int **todo_out, cudaStream_t stream, bool block_kernel);

}  // namespace tmc

/*
 * CPU oracle for the torchmorph hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain C restatements of the algorithms that torchmorph's CUDA operators
 * (and scipy.ndimage, which the reference's own test-suite uses as its
 * oracle) compute.  Only the tests, the smoke check and the CPU-baseline
 * leg of the benchmark may call into this library; the product path
 * (torchmorph_gb300 and libtmcore) never links or loads it.
 *
 * Layout conventions shared by every entry point:
 *   - `batch` independent items (the reference's B*C), each a C-contiguous
 *     N-D array of `ndim` spatial dimensions `shape[0..ndim)`;
 *   - index outputs are int32 planes laid out (ndim, batch, *shape), the
 *     layout of the reference's `indices` tensors;
 *   - every function returns 0 on success and a negative value on a bad
 *     argument.
 */
#ifndef TM_ORACLE_H
#define TM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Grey erosion (dilation = 0) / dilation (dilation = 1).
 * Follows torchmorph/csrc/grey_kernel.cu:101-170 (tap loop),
 * :63-97 (border modes) and :247-292 (tap-offset table). */
int tmo_grey(int dilation, const float *in, float *out, int64_t batch, int ndim,
             const int64_t *shape, const float *structure, const uint8_t *footprint,
             const int64_t *sshape, const int64_t *origin, int mode, float cval,
             int nthreads);

/* Binary erosion / dilation, torchmorph/csrc/binary_kernel.cu:56-127. */
int tmo_binary(int dilation, const uint8_t *in, uint8_t *out, int64_t batch, int ndim,
               const int64_t *shape, const uint8_t *structure, const int64_t *sshape,
               const int64_t *origin, int border_value, int nthreads);

/* Exact Euclidean distance transform (scipy.ndimage.distance_transform_edt
 * semantics, which the reference's tests pin it to).
 * sampling == NULL means unit spacing; sqdist is only written in that case.
 * Any output may be NULL. */
int tmo_edt(const uint8_t *fg, int64_t batch, int ndim, const int64_t *shape,
            const double *sampling, int64_t *sqdist, double *dist, int32_t *indices,
            int nthreads);

/* Chamfer distance transform as two raster passes (scipy's
 * distance_transform_cdt).  metric: 0 chessboard, 1 taxicab,
 * 2 weighted 3-4-5 chamfer (ndim <= 3).  dist is the integer path cost,
 * -1 where no background exists. */
int tmo_cdt(const uint8_t *fg, int64_t batch, int ndim, const int64_t *shape, int metric,
            int32_t *dist, int32_t *indices, int nthreads);

/* Brute-force distance transform (scipy.ndimage.distance_transform_bf).
 * metric: 0 euclidean, 1 taxicab, 2 chessboard. */
int tmo_bfdt(const uint8_t *fg, int64_t batch, int ndim, const int64_t *shape, int metric,
             const double *sampling, int return_indices, double *dist, int32_t *indices,
             int nthreads);

/* Sinkhorn iterations in float64 (torchmorph/optimal_transport.py:71-125):
 * a (n, d1), b (n, d2) row-normalised marginals sharing cost C (d1, d2).
 * log_space selects _log_iterations over _scaling_iterations.
 * Returns the number of iterations run. */
int64_t tmo_sinkhorn(const double *a, const double *b, const double *cost, int64_t n,
                     int64_t d1, int64_t d2, double eps, int64_t max_iter, double threshold,
                     int log_space, double *log_u, double *log_v, int nthreads);

/* Transport cost <P, C> and marginals of P = exp(log_u - C/eps + log_v),
 * torchmorph/optimal_transport.py:139-140.  row/col marginals may be NULL. */
void tmo_sinkhorn_cost(const double *cost, const double *log_u, const double *log_v,
                       int64_t n, int64_t d1, int64_t d2, double eps, double *dist,
                       double *row_marg, double *col_marg, int nthreads);

#ifdef __cplusplus
}
#endif

#endif

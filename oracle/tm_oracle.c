/*
 * CPU oracle for the torchmorph hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Each function restates, in plain C, the algorithm of the reference file
 * cited beside it.  The tests compare the CUDA product path against these
 * functions; the benchmark times them as the CPU baseline.  Nothing in the
 * shipped library calls into this file.
 *
 * Where the reference's operator and its test oracle (scipy.ndimage)
 * disagree on ties, this file follows scipy.ndimage; the rules are pinned
 * against scipy outputs committed under tests/golden/:
 *   - EDT feature index: the nearest background voxel, ties broken by the
 *     smallest coordinate along the LAST axis, then the previous axis, ...
 *     (the result of separable passes in axis order 0..n-1 where every pass
 *     keeps the lowest position on a tie).
 *   - CDT: two raster chamfer passes over the causal half of the 3^n
 *     neighbourhood, offsets in raster order, strict '<' (first offset wins).
 *   - Brute-force DT: the LAST background voxel in raster order among the
 *     nearest ones.
 */
#include "tm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TMO_MAX_NDIM 8

static int64_t prod64(const int64_t *s, int n) {
    int64_t p = 1;
    for (int i = 0; i < n; i++) p *= s[i];
    return p;
}

static void strides_of(const int64_t *shape, int ndim, int64_t *stride) {
    stride[ndim - 1] = 1;
    for (int d = ndim - 2; d >= 0; d--) stride[d] = stride[d + 1] * shape[d + 1];
}

static void set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

/* ------------------------------------------------------------------------
 * Border handling: torchmorph/csrc/grey_kernel.cu:63-97 (scipy modes).
 * Returns -1 when the constant value must be used.
 * ---------------------------------------------------------------------- */
static int64_t map_coord(int64_t c, int64_t n, int mode) {
    if (c >= 0 && c < n) return c;
    switch (mode) {
    case 0: /* constant */
        return -1;
    case 2: /* nearest */
        return c < 0 ? 0 : n - 1;
    case 1: { /* reflect: period 2n, [b a | a b c d | d c] */
        int64_t period = 2 * n;
        int64_t r = ((c % period) + period) % period;
        return r >= n ? period - 1 - r : r;
    }
    case 3: { /* mirror: period 2(n-1), [c b | a b c d | c b] */
        int64_t period = 2 * (n - 1);
        if (period <= 0) return 0;
        int64_t r = ((c % period) + period) % period;
        return r >= n ? period - r : r;
    }
    case 4: /* wrap */
        return ((c % n) + n) % n;
    default:
        return -1;
    }
}

/* Active taps of a structuring element: per-dimension offsets applied to
 * the output coordinate (torchmorph/csrc/grey_kernel.cu:271-291):
 * delta = k - (size//2 + origin); erosion reads x + delta, dilation x - delta. */
static int build_taps(int dilation, int ndim, const int64_t *sshape, const int64_t *origin,
                      const uint8_t *active, int64_t *taps, int64_t *tap_index) {
    int64_t sstride[TMO_MAX_NDIM];
    strides_of(sshape, ndim, sstride);
    int64_t total = prod64(sshape, ndim);
    int n = 0;
    for (int64_t i = 0; i < total; i++) {
        if (active && !active[i]) continue;
        int64_t rem = i;
        for (int d = 0; d < ndim; d++) {
            int64_t k = rem / sstride[d];
            rem %= sstride[d];
            int64_t delta = k - (sshape[d] / 2 + origin[d]);
            taps[(int64_t)n * ndim + d] = dilation ? -delta : delta;
        }
        if (tap_index) tap_index[n] = i;
        n++;
    }
    return n;
}

int tmo_grey(int dilation, const float *in, float *out, int64_t batch, int ndim,
             const int64_t *shape, const float *structure, const uint8_t *footprint,
             const int64_t *sshape, const int64_t *origin, int mode, float cval,
             int nthreads) {
    if (ndim < 1 || ndim > TMO_MAX_NDIM) return -1;
    int64_t stotal = prod64(sshape, ndim);
    int64_t *taps = (int64_t *)malloc(sizeof(int64_t) * (size_t)(stotal * ndim + 1));
    int64_t *tidx = (int64_t *)malloc(sizeof(int64_t) * (size_t)(stotal + 1));
    int ntaps = build_taps(dilation, ndim, sshape, origin, footprint, taps, tidx);
    if (ntaps == 0) {
        free(taps);
        free(tidx);
        return -2;
    }
    int64_t stride[TMO_MAX_NDIM];
    strides_of(shape, ndim, stride);
    int64_t n = prod64(shape, ndim);
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int64_t idx = 0; idx < batch * n; idx++) {
        int64_t b = idx / n, sp = idx % n;
        const float *img = in + b * n;
        int64_t coord[TMO_MAX_NDIM];
        int64_t rem = sp;
        for (int d = 0; d < ndim; d++) {
            coord[d] = rem / stride[d];
            rem %= stride[d];
        }
        float acc = dilation ? -INFINITY : INFINITY;
        for (int t = 0; t < ntaps; t++) {
            int64_t flat = 0;
            int use_cval = 0;
            for (int d = 0; d < ndim; d++) {
                int64_t m = map_coord(coord[d] + taps[(int64_t)t * ndim + d], shape[d], mode);
                if (m < 0) {
                    use_cval = 1;
                    break;
                }
                flat += m * stride[d];
            }
            float v = use_cval ? cval : img[flat];
            float s = structure[tidx[t]];
            /* grey_kernel.cu:39 / :55 */
            acc = dilation ? fmaxf(acc, v + s) : fminf(acc, v - s);
        }
        out[idx] = acc;
    }
    free(taps);
    free(tidx);
    return 0;
}

int tmo_binary(int dilation, const uint8_t *in, uint8_t *out, int64_t batch, int ndim,
               const int64_t *shape, const uint8_t *structure, const int64_t *sshape,
               const int64_t *origin, int border_value, int nthreads) {
    if (ndim < 1 || ndim > TMO_MAX_NDIM) return -1;
    int64_t stotal = prod64(sshape, ndim);
    int64_t *taps = (int64_t *)malloc(sizeof(int64_t) * (size_t)(stotal * ndim + 1));
    int ntaps = build_taps(dilation, ndim, sshape, origin, structure, taps, NULL);
    if (ntaps == 0) {
        free(taps);
        return -2;
    }
    int64_t stride[TMO_MAX_NDIM];
    strides_of(shape, ndim, stride);
    int64_t n = prod64(shape, ndim);
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int64_t idx = 0; idx < batch * n; idx++) {
        int64_t b = idx / n, sp = idx % n;
        const uint8_t *img = in + b * n;
        int64_t coord[TMO_MAX_NDIM];
        int64_t rem = sp;
        for (int d = 0; d < ndim; d++) {
            coord[d] = rem / stride[d];
            rem %= stride[d];
        }
        /* erosion = AND over taps, dilation = OR; out-of-bounds taps read
         * border_value (binary_kernel.cu:104-121). */
        int acc = dilation ? 0 : 1;
        for (int t = 0; t < ntaps; t++) {
            int64_t flat = 0;
            int inb = 1;
            for (int d = 0; d < ndim; d++) {
                int64_t c = coord[d] + taps[(int64_t)t * ndim + d];
                if (c < 0 || c >= shape[d]) {
                    inb = 0;
                    break;
                }
                flat += c * stride[d];
            }
            int v = inb ? (img[flat] != 0) : (border_value != 0);
            if (dilation ? v : !v) {
                acc = dilation ? 1 : 0;
                break;
            }
        }
        out[idx] = (uint8_t)acc;
    }
    free(taps);
    return 0;
}

/* ------------------------------------------------------------------------
 * EDT: separable lower-envelope passes (Felzenszwalb & Huttenlocher) in
 * axis order 0..n-1; each pass keeps the lowest position on a tie.  The
 * unit-spacing variant is exact in int64; the sampled variant works in
 * double like scipy.  Distances are recomputed from the final feature, as
 * scipy does, so the sampled result is sqrt(sum((x_d - f_d) * s_d)^2).
 * ---------------------------------------------------------------------- */
#define EDT_INF ((int64_t)1 << 60)

/* One exact pass over a line; g/f are read and written in place. */
static void edt_line_exact(int64_t *g, int64_t *f, int64_t L, int64_t *v, int64_t *tg,
                           int64_t *tf) {
    int64_t k = -1;
    for (int64_t q = 0; q < L; q++) {
        tg[q] = g[q];
        tf[q] = f[q];
        if (g[q] >= EDT_INF) continue;
        int64_t Gq = g[q] + q * q;
        while (k >= 1) {
            int64_t r = v[k], p = v[k - 1];
            int64_t Gr = tg[r] + r * r, Gp = tg[p] + p * p;
            /* pop r when s(q,r) <= s(r,p), cross-multiplied (denominators > 0) */
            __int128 lhs = (__int128)(Gq - Gr) * (r - p);
            __int128 rhs = (__int128)(Gr - Gp) * (q - r);
            if (lhs <= rhs)
                k--;
            else
                break;
        }
        v[++k] = q;
    }
    if (k < 0) {
        for (int64_t q = 0; q < L; q++) {
            g[q] = EDT_INF;
            f[q] = -1;
        }
        return;
    }
    int64_t j = 0;
    for (int64_t q = 0; q < L; q++) {
        while (j < k) {
            int64_t a = v[j], b = v[j + 1];
            int64_t fa = (q - a) * (q - a) + tg[a];
            int64_t fb = (q - b) * (q - b) + tg[b];
            if (fb < fa)
                j++;
            else
                break;
        }
        int64_t p = v[j];
        g[q] = (q - p) * (q - p) + tg[p];
        f[q] = tf[p];
    }
}

static void edt_line_sampled(double *g, int64_t *f, int64_t L, double s, int64_t *v,
                             double *tg, int64_t *tf) {
    int64_t k = -1;
    for (int64_t q = 0; q < L; q++) {
        tg[q] = g[q];
        tf[q] = f[q];
        if (isinf(g[q])) continue;
        double Pq = (double)q * s;
        double Gq = g[q] + Pq * Pq;
        while (k >= 1) {
            int64_t r = v[k], p = v[k - 1];
            double Pr = (double)r * s, Pp = (double)p * s;
            double Gr = tg[r] + Pr * Pr, Gp = tg[p] + Pp * Pp;
            if ((Gq - Gr) * (Pr - Pp) <= (Gr - Gp) * (Pq - Pr))
                k--;
            else
                break;
        }
        v[++k] = q;
    }
    if (k < 0) {
        for (int64_t q = 0; q < L; q++) {
            g[q] = INFINITY;
            f[q] = -1;
        }
        return;
    }
    int64_t j = 0;
    for (int64_t q = 0; q < L; q++) {
        double Q = (double)q * s;
        while (j < k) {
            double a = (double)v[j] * s, b = (double)v[j + 1] * s;
            double fa = (Q - a) * (Q - a) + tg[v[j]];
            double fb = (Q - b) * (Q - b) + tg[v[j + 1]];
            if (fb < fa)
                j++;
            else
                break;
        }
        int64_t p = v[j];
        double P = (double)p * s;
        g[q] = (Q - P) * (Q - P) + tg[p];
        f[q] = tf[p];
    }
}

/* The passes are parallel over every line of every item (an item's lines
 * along one axis are independent), so all host threads work on a batch of
 * any size; the per-voxel set-up and the outputs are parallel over voxels. */
int tmo_edt(const uint8_t *fg, int64_t batch, int ndim, const int64_t *shape,
            const double *sampling, int64_t *sqdist, double *dist, int32_t *indices,
            int nthreads) {
    if (ndim < 1 || ndim > TMO_MAX_NDIM) return -1;
    int64_t stride[TMO_MAX_NDIM];
    strides_of(shape, ndim, stride);
    const int64_t n = prod64(shape, ndim);
    const int64_t total = n * batch;
    int64_t maxL = 1;
    for (int d = 0; d < ndim; d++)
        if (shape[d] > maxL) maxL = shape[d];
    set_threads(nthreads);
    int64_t *feat = (int64_t *)malloc(sizeof(int64_t) * (size_t)(total ? total : 1));
    int64_t *gi = sampling ? NULL : (int64_t *)malloc(sizeof(int64_t) * (size_t)(total ? total : 1));
    double *gd = sampling ? (double *)malloc(sizeof(double) * (size_t)(total ? total : 1)) : NULL;
    uint8_t *any_bg = (uint8_t *)calloc((size_t)(batch ? batch : 1), 1);
    if (!feat || (!gi && !gd) || !any_bg) {
        free(feat);
        free(gi);
        free(gd);
        free(any_bg);
        return -2;
    }
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < total; t++) {
        const int bg = fg[t] == 0;
        feat[t] = bg ? t % n : -1;
        if (sampling)
            gd[t] = bg ? 0.0 : INFINITY;
        else
            gi[t] = bg ? 0 : EDT_INF;
        if (bg && !any_bg[t / n]) any_bg[t / n] = 1; /* benign race: only ever set to 1 */
    }
    for (int a = 0; a < ndim; a++) {
        const int64_t L = shape[a], st = stride[a];
        const int64_t lines_per_item = n / L;
        const int64_t lines = lines_per_item * batch;
#pragma omp parallel
        {
            int64_t *lf = (int64_t *)malloc(sizeof(int64_t) * (size_t)maxL);
            int64_t *v = (int64_t *)malloc(sizeof(int64_t) * (size_t)maxL);
            int64_t *tf = (int64_t *)malloc(sizeof(int64_t) * (size_t)maxL);
            int64_t *lgi = (int64_t *)malloc(sizeof(int64_t) * (size_t)maxL);
            int64_t *tgi = (int64_t *)malloc(sizeof(int64_t) * (size_t)maxL);
            double *lgd = (double *)malloc(sizeof(double) * (size_t)maxL);
            double *tgd = (double *)malloc(sizeof(double) * (size_t)maxL);
#pragma omp for schedule(static)
            for (int64_t line = 0; line < lines; line++) {
                const int64_t b = line / lines_per_item;
                if (!any_bg[b]) continue;
                const int64_t r = line % lines_per_item;
                const int64_t o = r / st, in = r % st;
                const int64_t base = b * n + o * L * st + in;
                for (int64_t q = 0; q < L; q++) {
                    lf[q] = feat[base + q * st];
                    if (sampling)
                        lgd[q] = gd[base + q * st];
                    else
                        lgi[q] = gi[base + q * st];
                }
                if (sampling)
                    edt_line_sampled(lgd, lf, L, sampling[a], v, tgd, tf);
                else
                    edt_line_exact(lgi, lf, L, v, tgi, tf);
                for (int64_t q = 0; q < L; q++) {
                    feat[base + q * st] = lf[q];
                    if (sampling)
                        gd[base + q * st] = lgd[q];
                    else
                        gi[base + q * st] = lgi[q];
                }
            }
            free(lf);
            free(v);
            free(tf);
            free(lgi);
            free(tgi);
            free(lgd);
            free(tgd);
        }
    }
    /* Outputs from the final feature.  With no background at all the
     * feature is the virtual site (-1, 0, ..., 0) (scipy behaviour,
     * reference edt_kernel.cu:415-437). */
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < total; t++) {
        const int64_t b = t / n, i = t % n;
        int64_t fc[TMO_MAX_NDIM], xc[TMO_MAX_NDIM];
        int64_t rem = i;
        for (int d = 0; d < ndim; d++) {
            xc[d] = rem / stride[d];
            rem %= stride[d];
        }
        if (any_bg[b]) {
            int64_t fr = feat[t];
            for (int d = 0; d < ndim; d++) {
                fc[d] = fr / stride[d];
                fr %= stride[d];
            }
        } else {
            for (int d = 0; d < ndim; d++) fc[d] = d == 0 ? -1 : 0;
        }
        if (indices)
            for (int d = 0; d < ndim; d++) indices[(int64_t)d * total + t] = (int32_t)fc[d];
        int64_t s2 = 0;
        double ds = 0.0;
        for (int d = 0; d < ndim; d++) {
            int64_t delta = xc[d] - fc[d];
            s2 += delta * delta;
            double dd = (double)delta * (sampling ? sampling[d] : 1.0);
            ds += dd * dd;
        }
        if (sqdist && !sampling) sqdist[t] = s2;
        if (dist) dist[t] = sqrt(ds);
    }
    free(feat);
    free(gi);
    free(gd);
    free(any_bg);
    return 0;
}

/* ------------------------------------------------------------------------
 * Chamfer DT: two raster passes with the causal half of the 3^n
 * neighbourhood (scipy.ndimage.distance_transform_cdt: forward pass, flip,
 * same pass, flip back).  The reference's own CDT (cdt_kernel.cu) is an
 * approximation of this for the chessboard metric; the values here are
 * exact.
 * ---------------------------------------------------------------------- */
int tmo_cdt(const uint8_t *fg, int64_t batch, int ndim, const int64_t *shape, int metric,
            int32_t *dist, int32_t *indices, int nthreads) {
    if (ndim < 1 || ndim > TMO_MAX_NDIM) return -1;
    if (metric == 2 && ndim > 3) return -1;
    int64_t stride[TMO_MAX_NDIM];
    strides_of(shape, ndim, stride);
    int64_t n = prod64(shape, ndim);
    /* causal offsets: structure elements before the centre, raster order */
    int total = 1;
    for (int d = 0; d < ndim; d++) total *= 3;
    int noff = 0;
    int offs[3280][TMO_MAX_NDIM];
    int wts[3280];
    for (int j = 0; j < total / 2; j++) {
        int rem = j, nz = 0, o[TMO_MAX_NDIM];
        for (int d = ndim - 1; d >= 0; d--) {
            o[d] = rem % 3 - 1;
            rem /= 3;
            nz += o[d] != 0;
        }
        if (metric == 1 && nz != 1) continue;
        for (int d = 0; d < ndim; d++) offs[noff][d] = o[d];
        wts[noff] = metric == 2 ? (nz == 1 ? 3 : nz == 2 ? 4 : 5) : 1;
        noff++;
    }
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t b = 0; b < batch; b++) {
        const uint8_t *img = fg + b * n;
        int32_t *dt = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
        int64_t *ft = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
        for (int64_t i = 0; i < n; i++) {
            dt[i] = img[i] ? -1 : 0;
            ft[i] = i;
        }
        for (int pass = 0; pass < 2; pass++) {
            int sgn = pass == 0 ? 1 : -1;
            for (int64_t t = 0; t < n; t++) {
                int64_t i = pass == 0 ? t : n - 1 - t;
                if (dt[i] == 0) continue;
                int64_t xc[TMO_MAX_NDIM], rem = i;
                for (int d = 0; d < ndim; d++) {
                    xc[d] = rem / stride[d];
                    rem %= stride[d];
                }
                int32_t best = dt[i];
                int64_t bf = ft[i];
                for (int k = 0; k < noff; k++) {
                    int64_t flat = 0;
                    int inb = 1;
                    for (int d = 0; d < ndim; d++) {
                        int64_t c = xc[d] + sgn * offs[k][d];
                        if (c < 0 || c >= shape[d]) {
                            inb = 0;
                            break;
                        }
                        flat += c * stride[d];
                    }
                    if (!inb) continue;
                    int32_t tv = dt[flat];
                    if (tv < 0) continue;
                    int32_t cand = tv + wts[k];
                    if (best < 0 || cand < best) {
                        best = cand;
                        bf = ft[flat];
                    }
                }
                dt[i] = best;
                ft[i] = bf;
            }
        }
        for (int64_t i = 0; i < n; i++) {
            if (dist) dist[b * n + i] = dt[i];
            if (indices) {
                int64_t fr = ft[i];
                for (int d = 0; d < ndim; d++) {
                    indices[(int64_t)d * batch * n + b * n + i] = (int32_t)(fr / stride[d]);
                    fr %= stride[d];
                }
            }
        }
        free(dt);
        free(ft);
    }
    return 0;
}

/* ------------------------------------------------------------------------
 * Brute-force DT (scipy.ndimage.distance_transform_bf): every foreground
 * voxel scans every background voxel; the last nearest one in raster
 * order wins.  Items without background get +inf (euclidean) or
 * 2^32-1 (others) with zero indices, as in reference bfdt_kernel.cu:208-221.
 * ---------------------------------------------------------------------- */
int tmo_bfdt(const uint8_t *fg, int64_t batch, int ndim, const int64_t *shape, int metric,
             const double *sampling, int return_indices, double *dist, int32_t *indices,
             int nthreads) {
    if (ndim < 1 || ndim > TMO_MAX_NDIM) return -1;
    int64_t stride[TMO_MAX_NDIM];
    strides_of(shape, ndim, stride);
    int64_t n = prod64(shape, ndim);
    set_threads(nthreads);
    for (int64_t b = 0; b < batch; b++) {
        const uint8_t *img = fg + b * n;
        int64_t nbg = 0, nfg = 0;
        for (int64_t i = 0; i < n; i++) {
            if (img[i])
                nfg++;
            else
                nbg++;
        }
        int64_t *bg = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nbg + 1));
        int64_t k = 0;
        for (int64_t i = 0; i < n; i++)
            if (!img[i]) bg[k++] = i;
        if (nfg == 0 && !return_indices) {
            if (dist)
                for (int64_t i = 0; i < n; i++) dist[b * n + i] = 0.0;
            free(bg);
            continue;
        }
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t i = 0; i < n; i++) {
            int64_t xc[TMO_MAX_NDIM], rem = i;
            for (int d = 0; d < ndim; d++) {
                xc[d] = rem / stride[d];
                rem %= stride[d];
            }
            double bestd;
            int64_t best = -1;
            if (!img[i]) {
                bestd = 0.0;
                best = i;
            } else if (nbg == 0) {
                bestd = metric == 0 ? INFINITY : 4294967295.0;
                best = -2;
            } else {
                bestd = INFINITY;
                for (int64_t j = 0; j < nbg; j++) {
                    int64_t r = bg[j];
                    double acc = 0.0;
                    for (int d = 0; d < ndim; d++) {
                        int64_t c = r / stride[d];
                        r %= stride[d];
                        double delta = (double)(xc[d] - c) * (sampling ? sampling[d] : 1.0);
                        if (metric == 0)
                            acc += delta * delta;
                        else if (metric == 1)
                            acc += fabs(delta);
                        else
                            acc = fmax(acc, fabs(delta));
                    }
                    if (acc <= bestd) {
                        bestd = acc;
                        best = bg[j];
                    }
                }
                if (metric == 0) bestd = sqrt(bestd);
            }
            if (dist) dist[b * n + i] = bestd;
            if (indices && return_indices) {
                int64_t fr = best;
                for (int d = 0; d < ndim; d++) {
                    int32_t v = 0;
                    if (best >= 0) {
                        v = (int32_t)(fr / stride[d]);
                        fr %= stride[d];
                    }
                    indices[(int64_t)d * batch * n + b * n + i] = v;
                }
            }
        }
        free(bg);
    }
    return 0;
}

/* ------------------------------------------------------------------------
 * Sinkhorn in float64: torchmorph/optimal_transport.py:71-93 (scaling form)
 * and :96-125 (log form), including the every-10-iterations stopping test
 * on the change of u (or log u).
 * ---------------------------------------------------------------------- */
static double lse_row(const double *x, int64_t m, int64_t stride) {
    double mx = -INFINITY;
    for (int64_t j = 0; j < m; j++)
        if (x[j * stride] > mx) mx = x[j * stride];
    if (mx == -INFINITY) return -INFINITY;
    double s = 0.0;
    for (int64_t j = 0; j < m; j++) s += exp(x[j * stride] - mx);
    return mx + log(s);
}

int64_t tmo_sinkhorn(const double *a, const double *b, const double *cost, int64_t n,
                     int64_t d1, int64_t d2, double eps, int64_t max_iter, double threshold,
                     int log_space, double *log_u, double *log_v, int nthreads) {
    set_threads(nthreads);
    int64_t it_run = 0;
    double *prev = (double *)malloc(sizeof(double) * (size_t)(n * d1));
    if (log_space) {
        double *logK = (double *)malloc(sizeof(double) * (size_t)(d1 * d2));
        for (int64_t i = 0; i < d1 * d2; i++) logK[i] = -cost[i] / eps;
        for (int64_t i = 0; i < n * d1; i++) log_u[i] = 0.0;
        for (int64_t i = 0; i < n * d2; i++) log_v[i] = 0.0;
        for (int64_t it = 0; it < max_iter; it++) {
            memcpy(prev, log_u, sizeof(double) * (size_t)(n * d1));
#pragma omp parallel for collapse(2) schedule(static)
            for (int64_t r = 0; r < n; r++)
                for (int64_t i = 0; i < d1; i++) {
                    double tmp_max = -INFINITY;
                    const double *kr = logK + i * d2;
                    const double *lv = log_v + r * d2;
                    for (int64_t j = 0; j < d2; j++) {
                        double z = kr[j] + lv[j];
                        if (z > tmp_max) tmp_max = z;
                    }
                    double s = 0.0;
                    if (tmp_max != -INFINITY)
                        for (int64_t j = 0; j < d2; j++) s += exp(kr[j] + lv[j] - tmp_max);
                    double lse = tmp_max == -INFINITY ? -INFINITY : tmp_max + log(s);
                    log_u[r * d1 + i] = log(a[r * d1 + i]) - lse;
                }
#pragma omp parallel for collapse(2) schedule(static)
            for (int64_t r = 0; r < n; r++)
                for (int64_t j = 0; j < d2; j++) {
                    double tmp_max = -INFINITY;
                    const double *lu = log_u + r * d1;
                    for (int64_t i = 0; i < d1; i++) {
                        double z = logK[i * d2 + j] + lu[i];
                        if (z > tmp_max) tmp_max = z;
                    }
                    double s = 0.0;
                    if (tmp_max != -INFINITY)
                        for (int64_t i = 0; i < d1; i++)
                            s += exp(logK[i * d2 + j] + lu[i] - tmp_max);
                    double lse = tmp_max == -INFINITY ? -INFINITY : tmp_max + log(s);
                    log_v[r * d2 + j] = log(b[r * d2 + j]) - lse;
                }
            it_run = it + 1;
            if (threshold > 0 && it % 10 == 0) {
                double worst = 0.0;
                for (int64_t r = 0; r < n; r++) {
                    double acc = 0.0;
                    for (int64_t i = 0; i < d1; i++) acc += fabs(log_u[r * d1 + i] - prev[r * d1 + i]);
                    if (acc > worst) worst = acc;
                }
                if (worst <= threshold) break;
            }
        }
        free(logK);
    } else {
        double *K = (double *)malloc(sizeof(double) * (size_t)(d1 * d2));
        double *u = (double *)malloc(sizeof(double) * (size_t)(n * d1));
        double *v = (double *)malloc(sizeof(double) * (size_t)(n * d2));
        for (int64_t i = 0; i < d1 * d2; i++) K[i] = exp(-cost[i] / eps);
        for (int64_t i = 0; i < n * d1; i++) u[i] = 1.0;
        for (int64_t i = 0; i < n * d2; i++) v[i] = 1.0;
        for (int64_t it = 0; it < max_iter; it++) {
            memcpy(prev, u, sizeof(double) * (size_t)(n * d1));
#pragma omp parallel for collapse(2) schedule(static)
            for (int64_t r = 0; r < n; r++)
                for (int64_t i = 0; i < d1; i++) {
                    double s = 0.0;
                    for (int64_t j = 0; j < d2; j++) s += K[i * d2 + j] * v[r * d2 + j];
                    u[r * d1 + i] = a[r * d1 + i] / (s + 1e-12);
                }
#pragma omp parallel for collapse(2) schedule(static)
            for (int64_t r = 0; r < n; r++)
                for (int64_t j = 0; j < d2; j++) {
                    double s = 0.0;
                    for (int64_t i = 0; i < d1; i++) s += K[i * d2 + j] * u[r * d1 + i];
                    v[r * d2 + j] = b[r * d2 + j] / (s + 1e-12);
                }
            it_run = it + 1;
            if (threshold > 0 && it % 10 == 0) {
                double worst = 0.0;
                for (int64_t r = 0; r < n; r++) {
                    double acc = 0.0;
                    for (int64_t i = 0; i < d1; i++) acc += fabs(u[r * d1 + i] - prev[r * d1 + i]);
                    if (acc > worst) worst = acc;
                }
                if (worst <= threshold) break;
            }
        }
        for (int64_t i = 0; i < n * d1; i++) log_u[i] = log(u[i]);
        for (int64_t i = 0; i < n * d2; i++) log_v[i] = log(v[i]);
        free(K);
        free(u);
        free(v);
    }
    free(prev);
    (void)lse_row;
    return it_run;
}

void tmo_sinkhorn_cost(const double *cost, const double *log_u, const double *log_v,
                       int64_t n, int64_t d1, int64_t d2, double eps, double *dist,
                       double *row_marg, double *col_marg, int nthreads) {
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < n; r++) {
        double acc = 0.0;
        if (col_marg)
            for (int64_t j = 0; j < d2; j++) col_marg[r * d2 + j] = 0.0;
        for (int64_t i = 0; i < d1; i++) {
            double rs = 0.0;
            for (int64_t j = 0; j < d2; j++) {
                double c = cost[i * d2 + j];
                double p = exp(log_u[r * d1 + i] - c / eps + log_v[r * d2 + j]);
                acc += p * c;
                rs += p;
                if (col_marg) col_marg[r * d2 + j] += p;
            }
            if (row_marg) row_marg[r * d1 + i] = rs;
        }
        dist[r] = acc;
    }
}

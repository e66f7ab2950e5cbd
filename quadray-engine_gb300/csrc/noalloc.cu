/*
 * noalloc.cu: path-tracer entry point whose running sums live in a fixed
 * device array of the library (qr_render_pt_noalloc, include/qr_gpu.h).
 *
 * The sums of QR_NOALLOC_MAX_PX pixels (3 floats each) are a file-scope
 * __device__ array, loaded with the library.  Its address is looked up once
 * per device with cudaGetSymbolAddress, with that device current, on the
 * first call for the device; the call makes no allocation (no cudaMalloc,
 * no cudaFree, no allocating library call).  Nothing in the array has to
 * start at zero: a call with pts_c == 0 writes the sums without reading
 * them.  One array per device serves every context and scene of the
 * process, so calls that overlap (other threads, or launches on streams
 * that run concurrently) race on it.
 */
#include <cuda_runtime.h>
#include <stdio.h>

#include "qr_gpu.h"
#include "tracer.cuh"

#define QR_NOALLOC_MAX_DEVICES  64

int qr_internal_scene(qr_ctx *ctx, int scene_id, const qr_dscene **sc, int *device);
int qr_internal_check_fp(const qr_frame_params *fp);
int qr_internal_fail(qr_ctx *ctx, int code, const char *what, cudaError_t e);
void qr_internal_message(qr_ctx *ctx, const char *msg);

static __device__ __align__(256) float g_pt_sums[3 * (size_t)QR_NOALLOC_MAX_PX];

/* per device: the array's address, and the frame size (pixels) whose sums a
 * call with pts_c == 0 started (0: none) */
static float *g_sums_addr[QR_NOALLOC_MAX_DEVICES];
static size_t g_sums_px[QR_NOALLOC_MAX_DEVICES];

extern "C" int qr_render_pt_noalloc(qr_ctx *ctx, int scene_id, const qr_frame_params *fp,
                                    uint32_t *dev_frame, void *stream)
{
    if (ctx == NULL) return QR_ERR_ARG;
    const qr_dscene *sc = NULL;
    int dev = -1;
    int rc = qr_internal_scene(ctx, scene_id, &sc, &dev);
    if (rc != QR_OK) return rc;
    rc = qr_internal_check_fp(fp);
    if (rc != QR_OK) return rc;
    if (fp->pt_on <= 0 || dev_frame == NULL) return QR_ERR_ARG;
    if (dev < 0 || dev >= QR_NOALLOC_MAX_DEVICES) return QR_ERR_LIMIT;
    const size_t px = (size_t)fp->x_row * (size_t)fp->y_res;
    if (px > (size_t)QR_NOALLOC_MAX_PX)
    {
        char msg[160];
        snprintf(msg, sizeof(msg), "qr_render_pt_noalloc: a frame of %zu pixels "
                 "(x_row * y_res) exceeds its fixed sums of %d pixels", px,
                 QR_NOALLOC_MAX_PX);
        qr_internal_message(ctx, msg);
        return QR_ERR_LIMIT;
    }
    if (fp->pts_c > 0.0f && g_sums_px[dev] != px)
    {
        qr_internal_message(ctx, "qr_render_pt_noalloc: no sums were started for "
                            "this frame size (the first call needs pts_c == 0)");
        return QR_ERR_STATE;
    }
    cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) return qr_internal_fail(ctx, QR_ERR_CUDA, "cudaSetDevice", e);
    if (g_sums_addr[dev] == NULL)
    {
        void *p = NULL;
        e = cudaGetSymbolAddress(&p, g_pt_sums);
        if (e != cudaSuccess)
            return qr_internal_fail(ctx, QR_ERR_CUDA, "cudaGetSymbolAddress", e);
        g_sums_addr[dev] = (float *)p;
    }
    e = qr_launch_pt(*sc, *fp, g_sums_addr[dev], dev_frame, (cudaStream_t)stream);
    if (e != cudaSuccess) return qr_internal_fail(ctx, QR_ERR_CUDA, "path-tracer launch", e);
    if (fp->pts_c == 0.0f) g_sums_px[dev] = px;
    return QR_OK;
}

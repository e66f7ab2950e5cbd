/*
 * noalloc.cu: path-tracer entry point whose running sums live in a fixed
 * device array of the library (qr_render_pt_noalloc, include/qr_gpu.h).
 *
 * Who needs it: callers that may not allocate device memory once their
 * render loop runs (a frame server that keeps every allocation out of its
 * steady state, an embedding host that owns the device heap), but still want
 * the path tracer's running sums, which qr_render_pt asks the caller to
 * allocate.
 *
 * The sums of QR_NOALLOC_MAX_PX pixels (3 floats each) are a file-scope
 * __device__ array, loaded with the library.  Host code cannot use the
 * array's name as a device address, so its address is looked up once per
 * device with cudaGetSymbolAddress, with that device current, on the first
 * call for the device; the caller's current device is restored before the
 * call returns.  The call makes no allocation (no cudaMalloc, no cudaFree,
 * no allocating library call).  Nothing in the array has to start at zero:
 * a call with pts_c == 0 writes the sums without reading them.  One array
 * per device serves every context and scene of the process, so calls that
 * overlap on the GPU (other threads, or launches on streams that run
 * concurrently) race on it.  The host-side bookkeeping below is guarded by
 * a mutex, so concurrent host calls are well defined.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include <mutex>

#include "qr_gpu.h"
#include "tracer.cuh"

#define QR_NOALLOC_MAX_DEVICES  64

int qr_internal_scene(qr_ctx *ctx, int scene_id, const qr_dscene **sc, int *device);
int qr_internal_check_fp(const qr_frame_params *fp);
int qr_internal_fail(qr_ctx *ctx, int code, const char *what, cudaError_t e);
void qr_internal_message(qr_ctx *ctx, const char *msg);

static __device__ __align__(256) float g_pt_sums[3 * (size_t)QR_NOALLOC_MAX_PX];

/* per device: the array's address, and who started the sums it holds (a
 * call with pts_c == 0): context, scene and frame shape; later calls must
 * name the same ones */
struct NoallocSums
{
    float        *addr;
    const qr_ctx *ctx;
    int           scene_id;
    int           x_row, y_res;
    int           started;
};
static NoallocSums g_sums[QR_NOALLOC_MAX_DEVICES];
static std::mutex g_sums_lock;

/* sets `dev` current for the lifetime of the object and puts the caller's
 * device back afterwards */
struct DeviceScope
{
    int prev;
    cudaError_t err;
    explicit DeviceScope(int dev) : prev(-1)
    {
        err = cudaGetDevice(&prev);
        if (err == cudaSuccess && prev != dev) err = cudaSetDevice(dev);
    }
    ~DeviceScope()
    {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev)
            cudaSetDevice(prev);
    }
};

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
    std::lock_guard<std::mutex> guard(g_sums_lock);
    NoallocSums &g = g_sums[dev];
    if (fp->pts_c > 0.0f && !(g.started && g.ctx == ctx && g.scene_id == scene_id &&
                              g.x_row == fp->x_row && g.y_res == fp->y_res))
    {
        qr_internal_message(ctx, "qr_render_pt_noalloc: no sums were started for "
                            "this context, scene and frame shape (the first call "
                            "needs pts_c == 0)");
        return QR_ERR_STATE;
    }
    DeviceScope scope(dev);
    if (scope.err != cudaSuccess)
        return qr_internal_fail(ctx, QR_ERR_CUDA, "cudaSetDevice", scope.err);
    if (g.addr == NULL)
    {
        void *p = NULL;
        cudaError_t e = cudaGetSymbolAddress(&p, g_pt_sums);
        if (e != cudaSuccess)
            return qr_internal_fail(ctx, QR_ERR_CUDA, "cudaGetSymbolAddress", e);
        g.addr = (float *)p;
    }
    cudaError_t e = qr_launch_pt(*sc, *fp, g.addr, dev_frame, (cudaStream_t)stream);
    if (e != cudaSuccess) return qr_internal_fail(ctx, QR_ERR_CUDA, "path-tracer launch", e);
    if (fp->pts_c == 0.0f)
    {
        g.ctx = ctx;
        g.scene_id = scene_id;
        g.x_row = fp->x_row;
        g.y_res = fp->y_res;
        g.started = 1;
    }
    return QR_OK;
}

/*
 * batch.cu: batched persistent rendering of many frame requests (qr_batch_*
 * of include/qr_gpu.h).
 *
 * A batch holds up to max_requests requests on resident scenes of one
 * context, Whitted or path-traced, of any size.  The Whitted requests are
 * cut into warp tiles and one persistent kernel walks the tiles of all of
 * them (tracer.cu batch_kernel).  The path-traced requests run, one after
 * the other on a second stream, as frames of the wavefront path tracer
 * (wavefront.cu) over the batch's own scratch, so the two classes overlap
 * in each other's tail.  The counter reset and all the launches are
 * captured once into a CUDA graph and replayed by every launch until the
 * requests or the tile configuration change.  The tile shape and the tiles
 * a warp claims at once come from qr_batch_tune, which times each
 * configuration on the batch itself and keeps the fastest.
 *
 * Completion per request: the warp that finishes a request's last tile sets
 * the request's flag in host memory mapped into the device
 * (qr_batch_done), so a caller can take each frame as soon as it is ready
 * instead of when the whole batch is.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>
#include <algorithm>
#include <new>
#include <vector>

#include "qr_gpu.h"
#include "tracer.cuh"
#include "wavefront.h"

/* side streams of the path-traced requests: their frames run side by side,
 * so one frame's stage tails overlap another's work */
#ifndef QR_BATCH_PT_STREAMS
#define QR_BATCH_PT_STREAMS 2
#endif

int qr_internal_scene(qr_ctx *ctx, int scene_id, const qr_dscene **sc, int *device);
int qr_internal_check_fp(const qr_frame_params *fp);
int qr_internal_device(qr_ctx *ctx);
int qr_internal_fail(qr_ctx *ctx, int code, const char *what, cudaError_t e);
void qr_internal_message(qr_ctx *ctx, const char *msg);

struct qr_batch
{
    qr_ctx      *ctx;
    int          device;
    int          max;
    qr_job      *djobs;         /* Whitted jobs, then path-tracer jobs */
    int         *dcount;        /* claim counters of the two kernels */
    int         *dtiles;        /* finished tiles per job */
    uint32_t    *hdone;         /* per request: 1 once its frame is done
                                   (mapped host memory) */
    uint32_t    *ddone;         /* its device address */
    std::vector<qr_request> reqs;
    int          nw, np;        /* jobs per mode */
    int          tiles[2];      /* tiles per mode */
    int          tw, th, grab;
    int          once;          /* Whitted kernel: a block for every 4 runs
                                   of tiles (qr_batch_persistent(b, 0)) */
    int          blocks[2];
    cudaStream_t main, side[QR_BATCH_PT_STREAMS];
    cudaEvent_t  fork, join[QR_BATCH_PT_STREAMS], done;
    cudaGraphExec_t exec;
    int          graph_ok;
    int          launched;
    int          sms;
    int          graph_kernels;  /* kernel nodes of the captured graph */
    /* path-traced requests: wavefront capacities of each PT job, the side
     * stream each runs on, and a scratch per side stream that fits the
     * largest */
    std::vector<qr_wf_caps> pt_caps;
    std::vector<int> pt_stream;
    void        *wf[QR_BATCH_PT_STREAMS];
    size_t       wf_bytes;
    int          nwf;            /* scratch blocks allocated */
    std::vector<qr_job> pt_jobs;    /* host copies of the path-traced jobs */
};

/* wavefront chunks of the batch's path-traced requests (as a context's) */
#define QR_BATCH_WF_PATHS (4ll << 20)

static int bfail(qr_batch *b, int code, const char *what, cudaError_t e)
{
    return qr_internal_fail(b->ctx, code, what, e);
}

extern "C" int qr_batch_create(qr_ctx *ctx, int max_requests, qr_batch **out)
{
    if (ctx == NULL || out == NULL || max_requests <= 0 || max_requests > (1 << 20))
        return QR_ERR_ARG;
    *out = NULL;
    qr_batch *b = new (std::nothrow) qr_batch();
    if (b == NULL) return QR_ERR_OOM;
    b->ctx = ctx;
    b->max = max_requests;
    b->tw = 8;
    b->th = 4;
    b->grab = 1;
    b->device = qr_internal_device(ctx);
    cudaError_t e = cudaSetDevice(b->device);
    if (e == cudaSuccess) e = cudaMalloc(&b->djobs, sizeof(qr_job) * (size_t)max_requests);
    if (e == cudaSuccess) e = cudaMalloc(&b->dcount, 2 * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&b->dtiles, sizeof(int) * (size_t)max_requests);
    if (e == cudaSuccess)
        e = cudaHostAlloc((void **)&b->hdone, sizeof(uint32_t) * (size_t)max_requests,
                          cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&b->ddone, b->hdone, 0);
    if (e == cudaSuccess) memset(b->hdone, 0, sizeof(uint32_t) * (size_t)max_requests);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking);
    for (int k = 0; k < QR_BATCH_PT_STREAMS && e == cudaSuccess; k++)
    {
        e = cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    if (e != cudaSuccess)
    {
        int rc = qr_internal_fail(ctx, QR_ERR_CUDA, "batch create", e);
        qr_batch_destroy(b);
        return rc;
    }
    for (int m = 0; m < 2; m++)
    {
        int per = qr_batch_blocks_per_sm(m);
        b->blocks[m] = sms * (per > 0 ? per : 1);
    }
    b->sms = sms;
    qr_wf_prepare();
    *out = b;
    return QR_OK;
}

extern "C" int qr_batch_destroy(qr_batch *b)
{
    if (b == NULL) return QR_ERR_ARG;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->djobs) cudaFree(b->djobs);
    if (b->dcount) cudaFree(b->dcount);
    if (b->dtiles) cudaFree(b->dtiles);
    if (b->hdone) cudaFreeHost(b->hdone);
    if (b->main) cudaStreamDestroy(b->main);
    for (int k = 0; k < QR_BATCH_PT_STREAMS; k++)
    {
        if (b->side[k]) cudaStreamDestroy(b->side[k]);
        if (b->join[k]) cudaEventDestroy(b->join[k]);
        if (b->wf[k]) cudaFree(b->wf[k]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->done) cudaEventDestroy(b->done);
    delete b;
    return QR_OK;
}

/* job table of the current requests and tile configuration */
static int upload_jobs(qr_batch *b)
{
    std::vector<qr_job> jobs;
    jobs.reserve(b->reqs.size());
    for (int pass = 0; pass < 2; pass++)
    {
        int tile = 0;
        for (size_t i = 0; i < b->reqs.size(); i++)
        {
            const qr_request &r = b->reqs[i];
            const int pt = r.fp.pt_on > 0;
            if (pt != pass) continue;
            const qr_dscene *sc = NULL;
            int dev = 0;
            if (qr_internal_scene(b->ctx, r.scene_id, &sc, &dev) != QR_OK) return QR_ERR_NOSCENE;
            qr_job j;
            memset(&j, 0, sizeof(j));
            j.S = *sc;
            j.P = r.fp;
            j.frame = r.dev_frame;
            j.acc = r.dev_acc;
            /* 4x AA Whitted requests: tiles of 4 x 2 pixels, a thread per
             * sub-sample; otherwise tiles of tw x th pixels */
            const int aa = !pt && r.fp.fsaa == 2;
            const int tw = aa ? 4 : b->tw, th = aa ? 2 : b->th;
            j.tiles_x = (r.fp.x_res + tw - 1) / tw;
            const int ty = (r.fp.y_res + th - 1) / th;
            j.tile0 = tile;
            j.ntiles = j.tiles_x * ty;
            j.req = (int)i;
            tile += j.ntiles;
            jobs.push_back(j);
        }
        b->tiles[pass] = tile;
        if (pass == 0) b->nw = (int)jobs.size();
        else b->np = (int)jobs.size() - b->nw;
    }
    if (!jobs.empty())
    {
        cudaError_t e = cudaMemcpy(b->djobs, jobs.data(), sizeof(qr_job) * jobs.size(),
                                   cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return bfail(b, QR_ERR_CUDA, "batch job upload", e);
    }
    /* the path-traced jobs' wavefront capacities, their side streams (each
     * job to the stream with the least work so far, by pixels x samples,
     * largest jobs first) and a scratch per stream used for the largest */
    b->pt_caps.clear();
    b->pt_stream.assign(b->np, 0);
    size_t need = 0;
    for (int j = b->nw; j < b->nw + b->np; j++)
    {
        const qr_wf_caps c = qr_wf_caps_for(jobs[j].P, QR_BATCH_WF_PATHS, 2, 8);
        b->pt_caps.push_back(c);
        need = std::max(need, qr_wf_bytes(c));
    }
    {
        std::vector<int> ord(b->np);
        for (int j = 0; j < b->np; j++) ord[j] = j;
        auto work = [&](int j) {
            const qr_frame_params &P = jobs[b->nw + j].P;
            return (double)P.x_res * P.y_res * P.pt_on;
        };
        std::stable_sort(ord.begin(), ord.end(), [&](int u, int v) { return work(u) > work(v); });
        double load[QR_BATCH_PT_STREAMS] = {0.0};
        for (int j : ord)
        {
            int k = 0;
            for (int q = 1; q < QR_BATCH_PT_STREAMS; q++)
                if (load[q] < load[k]) k = q;
            b->pt_stream[j] = k;
            load[k] += work(j);
        }
    }
    const int nwf = std::min(b->np, QR_BATCH_PT_STREAMS);
    if (need > b->wf_bytes || nwf > b->nwf)
    {
        for (int k = 0; k < QR_BATCH_PT_STREAMS; k++)
        {
            if (b->wf[k]) cudaFree(b->wf[k]);
            b->wf[k] = NULL;
        }
        b->wf_bytes = 0;
        b->nwf = 0;
        for (int k = 0; k < nwf; k++)
        {
            cudaError_t e = cudaMalloc(&b->wf[k], need);
            if (e != cudaSuccess) return bfail(b, QR_ERR_OOM, "batch wavefront scratch", e);
        }
        b->wf_bytes = need;
        b->nwf = nwf;
    }
    b->pt_jobs.assign(jobs.begin() + b->nw, jobs.end());
    if (b->exec)
    {
        cudaGraphExecDestroy(b->exec);
        b->exec = NULL;
    }
    b->graph_ok = 0;
    return QR_OK;
}

extern "C" int qr_batch_set(qr_batch *b, const qr_request *reqs, int n)
{
    if (b == NULL || (n > 0 && reqs == NULL) || n < 0) return QR_ERR_ARG;
    if (n > b->max) return QR_ERR_LIMIT;
    for (int i = 0; i < n; i++)
    {
        const qr_dscene *sc;
        int dev;
        int rc = qr_internal_scene(b->ctx, reqs[i].scene_id, &sc, &dev);
        if (rc != QR_OK) return rc;
        rc = qr_internal_check_fp(&reqs[i].fp);
        if (rc != QR_OK) return rc;
        if (reqs[i].dev_frame == NULL) return QR_ERR_ARG;
        if (reqs[i].fp.pt_on > 0 && reqs[i].dev_acc == NULL) return QR_ERR_ARG;
    }
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return bfail(b, QR_ERR_CUDA, "cudaSetDevice", e);
    b->reqs.assign(reqs, reqs + n);
    return upload_jobs(b);
}

extern "C" int qr_batch_config(qr_batch *b, int tile_w, int grab)
{
    if (b == NULL) return QR_ERR_ARG;
    if (tile_w != 4 && tile_w != 8 && tile_w != 16 && tile_w != 32) return QR_ERR_ARG;
    if (grab < 1 || grab > 64) return QR_ERR_ARG;
    b->tw = tile_w;
    b->th = 32 / tile_w;
    b->grab = grab;
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return bfail(b, QR_ERR_CUDA, "cudaSetDevice", e);
    return upload_jobs(b);
}

extern "C" int qr_batch_persistent(qr_batch *b, int on)
{
    if (b == NULL) return QR_ERR_ARG;
    b->once = on ? 0 : 1;
    if (b->exec)
    {
        cudaGraphExecDestroy(b->exec);
        b->exec = NULL;
    }
    b->graph_ok = 0;
    return QR_OK;
}

/* the Whitted launch on b->main, the path-traced frames on the side
 * streams */
static cudaError_t enqueue(qr_batch *b)
{
    cudaError_t e = cudaMemsetAsync(b->dcount, 0, 2 * sizeof(int), b->main);
    if (e == cudaSuccess && b->nw + b->np > 0)
        e = cudaMemsetAsync(b->dtiles, 0, sizeof(int) * (size_t)(b->nw + b->np), b->main);
    if (e == cudaSuccess) e = cudaEventRecord(b->fork, b->main);
    for (int k = 0; k < QR_BATCH_PT_STREAMS && e == cudaSuccess; k++)
        e = cudaStreamWaitEvent(b->side[k], b->fork, 0);
    if (e == cudaSuccess)
        e = qr_launch_batch(0, b->djobs, b->nw, b->tiles[0], b->dcount, b->tw, b->th,
                            b->grab, b->blocks[0], b->once, b->dtiles, b->ddone, b->main);
    /* the path-traced requests one after the other on each side stream,
     * each marked done as soon as its frame is in device memory */
    for (int j = 0; j < b->np && e == cudaSuccess; j++)
    {
        const qr_job &J = b->pt_jobs[j];
        const int k = b->pt_stream[j];
        e = qr_wf_launch_pt(J.S, J.P, J.acc, J.frame, b->wf[k], b->pt_caps[j], b->sms,
                            b->side[k]);
        if (e == cudaSuccess) e = qr_wf_mark_done(b->ddone, J.req, b->side[k]);
    }
    for (int k = 0; k < QR_BATCH_PT_STREAMS && e == cudaSuccess; k++)
    {
        e = cudaEventRecord(b->join[k], b->side[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->main, b->join[k], 0);
    }
    return e;
}

extern "C" int qr_batch_launch(qr_batch *b, void *stream)
{
    if (b == NULL) return QR_ERR_ARG;
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return bfail(b, QR_ERR_CUDA, "cudaSetDevice", e);
    if (!b->graph_ok)
    {
        cudaGraph_t g = NULL;
        e = cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess)
        {
            cudaError_t e2 = enqueue(b);
            e = cudaStreamEndCapture(b->main, &g);
            if (e2 != cudaSuccess) e = e2;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, g, 0);
        b->graph_kernels = 0;
        size_t nn = 0;
        if (e == cudaSuccess) e = cudaGraphGetNodes(g, NULL, &nn);
        if (e == cudaSuccess && nn > 0)
        {
            std::vector<cudaGraphNode_t> nodes(nn);
            e = cudaGraphGetNodes(g, nodes.data(), &nn);
            for (size_t i = 0; i < nn && e == cudaSuccess; i++)
            {
                cudaGraphNodeType t;
                e = cudaGraphNodeGetType(nodes[i], &t);
                if (e == cudaSuccess && t == cudaGraphNodeTypeKernel) b->graph_kernels++;
            }
        }
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) return bfail(b, QR_ERR_CUDA, "batch graph capture", e);
        b->graph_ok = 1;
    }
    /* the previous launch has finished (the caller polled or waited): clear
     * the completion flags before the graph can set them */
    memset(b->hdone, 0, sizeof(uint32_t) * b->reqs.size());
    e = cudaGraphLaunch(b->exec, (cudaStream_t)stream);
    if (e == cudaSuccess) qr_note_launches((cudaStream_t)stream, b->graph_kernels);
    if (e == cudaSuccess) e = cudaEventRecord(b->done, (cudaStream_t)stream);
    if (e != cudaSuccess) return bfail(b, QR_ERR_CUDA, "batch graph launch", e);
    b->launched = 1;
    return QR_OK;
}

extern "C" int qr_batch_poll(qr_batch *b)
{
    if (b == NULL) return QR_ERR_ARG;
    if (!b->launched) return QR_OK;
    cudaError_t e = cudaEventQuery(b->done);
    if (e == cudaSuccess) return QR_OK;
    if (e == cudaErrorNotReady) return QR_ERR_BUSY;
    return bfail(b, QR_ERR_CUDA, "batch poll", e);
}

extern "C" int qr_batch_done(qr_batch *b, const volatile uint32_t **flags)
{
    if (b == NULL || flags == NULL) return QR_ERR_ARG;
    *flags = b->hdone;
    return QR_OK;
}

extern "C" int qr_batch_wait(qr_batch *b)
{
    if (b == NULL) return QR_ERR_ARG;
    if (!b->launched) return QR_OK;
    cudaError_t e = cudaEventSynchronize(b->done);
    if (e != cudaSuccess) return bfail(b, QR_ERR_CUDA, "batch wait", e);
    return QR_OK;
}

extern "C" int qr_batch_tune(qr_batch *b, int *tile_w, int *grab, float *ms)
{
    if (b == NULL) return QR_ERR_ARG;
    static const int tws[4] = {8, 16, 32, 4};
    static const int grabs[2] = {1, 4};
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return bfail(b, QR_ERR_CUDA, "cudaSetDevice", e);
    cudaEvent_t t0, t1;
    e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    if (e != cudaSuccess) return bfail(b, QR_ERR_CUDA, "tune events", e);
    float best = -1.0f;
    int bw = 8, bg = 1;
    for (int i = 0; i < 4 && e == cudaSuccess; i++)
    {
        for (int j = 0; j < 2 && e == cudaSuccess; j++)
        {
            int rc = qr_batch_config(b, tws[i], grabs[j]);
            if (rc != QR_OK) { cudaEventDestroy(t0); cudaEventDestroy(t1); return rc; }
            e = enqueue(b);                         /* warm-up */
            if (e == cudaSuccess) e = cudaEventRecord(t0, b->main);
            if (e == cudaSuccess) e = enqueue(b);
            if (e == cudaSuccess) e = cudaEventRecord(t1, b->main);
            if (e == cudaSuccess) e = cudaEventSynchronize(t1);
            float t = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t, t0, t1);
            if (e == cudaSuccess && (best < 0.0f || t < best))
            {
                best = t;
                bw = tws[i];
                bg = grabs[j];
            }
        }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (e != cudaSuccess) return bfail(b, QR_ERR_CUDA, "batch tune", e);
    int rc = qr_batch_config(b, bw, bg);
    if (rc != QR_OK) return rc;
    if (tile_w) *tile_w = bw;
    if (grab) *grab = bg;
    if (ms) *ms = best;
    return QR_OK;
}

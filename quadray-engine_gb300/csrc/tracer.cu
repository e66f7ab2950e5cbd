/*
 * tracer.cu: sm_103a kernels of the GB300 QuadRay tracer: one thread a pixel
 * (whitted_kernel, pt_kernel) or a 4x AA sub-sample (whitted_aa_kernel),
 * and the batched persistent kernel (batch_kernel), over the device code of
 * tracer_dev.cuh; their launch functions.
 *
 * Work counters.  This file is compiled twice: as namespace qr_dev (the
 * timed kernels, no counter code at all) and, from tracer_stats.cu with
 * QR_STATS defined, as namespace qr_dev_stats, where every counted event
 * increments a per-thread counter that is warp-reduced into the global
 * totals once at the end of the kernel.
 */
#include "tracer_dev.cuh"

namespace QR_NS
{

__global__ void __launch_bounds__(128, QR_MIN_BLOCKS)
whitted_kernel(const qr_dscene S, const qr_frame_params P, uint32_t *frame,
               qr_dstats *gst)
{
    const int x = tile_x(), y = tile_y();
    if (x >= P.x_res || y >= P.y_res) return;
#ifdef QR_STATS
    TCnt cnt;
    #pragma unroll
    for (int k = 0; k < QR_STAT_COUNT; k++) cnt.c[k] = 0;
    StP st = &cnt;
#else
    StP st = NULL;
    (void)gst;
#endif
    whitted_pixel(S, P, x, y, frame, st);
#ifdef QR_STATS
    const unsigned am = __activemask();
    const int leader = __ffs(am) - 1;
    #pragma unroll
    for (int k = 0; k < QR_STAT_COUNT; k++)
    {
        const unsigned v = __reduce_add_sync(am, cnt.c[k]);
        if ((int)(threadIdx.x & 31) == leader && v != 0)
            atomicAdd(&gst->c[k], (unsigned long long)v);
    }
#endif
}


/*
 * 4x AA frames with one thread per sub-sample.  The four sub-samples of a
 * pixel are neighbouring lanes (lane = 4 * pixel + sub-sample), a warp
 * covers 4 x 2 pixels and a block of 32 x 4 threads 8 x 4 pixels, so the
 * lanes of a warp trace rays a fraction of a pixel apart and mostly take
 * the same branches and nodes.  The AA average is formed with shuffles in
 * the reference's pairing: p01 = c0 / 2 + c1 / 2 between lanes 0 and 1,
 * p23 likewise, then p01 / 2 + p23 / 2 (the two operands of each sum are the
 * same in both lanes and the sum commutes, so every lane holds the same
 * bits).
 */
__device__ __forceinline__ void aa_subsample(const qr_dscene &S, const qr_frame_params &P,
                                             int x, int y, int sub, uint32_t *frame, StP st)
{
    const int inside = x < P.x_res && y < P.y_res;
    float c[3] = {0.0f, 0.0f, 0.0f};
    if (inside)
    {
        primary(S, P, x, y, (float)x + c_aa4_h[sub], (float)y + c_aa4_v[sub], c, st);
        #pragma unroll
        for (int k = 0; k < 3; k++) c[k] = clamp1(c[k]);
    }
    float col[3];
    #pragma unroll
    for (int k = 0; k < 3; k++)
    {
        const float h = c[k] * 0.5f;
        const float pr = h + __shfl_xor_sync(0xFFFFFFFFu, h, 1);
        const float q = pr * 0.5f;
        col[k] = q + __shfl_xor_sync(0xFFFFFFFFu, q, 2);
    }
    if (inside && sub == 0) frame[(size_t)y * P.x_row + x] = pack(P, col);
}

__global__ void __launch_bounds__(128, QR_MIN_BLOCKS)
whitted_aa_kernel(const qr_dscene S, const qr_frame_params P, uint32_t *frame,
                  qr_dstats *gst)
{
    const int lane = threadIdx.x;
    const int sub = lane & 3, pix = lane >> 2;
    const int x = blockIdx.x * 8 + (threadIdx.y & 1) * 4 + (pix & 3);
    const int y = blockIdx.y * 4 + (threadIdx.y >> 1) * 2 + (pix >> 2);
#ifdef QR_STATS
    TCnt cnt;
    #pragma unroll
    for (int k = 0; k < QR_STAT_COUNT; k++) cnt.c[k] = 0;
    StP st = &cnt;
#else
    StP st = NULL;
    (void)gst;
#endif
    aa_subsample(S, P, x, y, sub, frame, st);
#ifdef QR_STATS
    #pragma unroll
    for (int k = 0; k < QR_STAT_COUNT; k++)
    {
        const unsigned v = __reduce_add_sync(0xFFFFFFFFu, cnt.c[k]);
        if (lane == 0 && v != 0) atomicAdd(&gst->c[k], (unsigned long long)v);
    }
#endif
}


template <int FLAT>
__global__ void __launch_bounds__(128, QR_PT_MIN_BLOCKS)
pt_kernel(const qr_dscene S, const qr_frame_params P, float *acc, uint32_t *frame,
          qr_dstats *gst)
{
    const int x = tile_x(), y = tile_y();
    if (x >= P.x_res || y >= P.y_res) return;
#ifdef QR_STATS
    TCnt cnt;
    #pragma unroll
    for (int k = 0; k < QR_STAT_COUNT; k++) cnt.c[k] = 0;
    StP st = &cnt;
#else
    StP st = NULL;
    (void)gst;
#endif
    if (FLAT) pt_pixel_flat(S, P, x, y, acc, frame, st);
    else pt_pixel_seq(S, P, x, y, acc, frame, st);
#ifdef QR_STATS
    const unsigned am = __activemask();
    const int leader = __ffs(am) - 1;
    #pragma unroll
    for (int k = 0; k < QR_STAT_COUNT; k++)
    {
        const unsigned v = __reduce_add_sync(am, cnt.c[k]);
        if ((int)(threadIdx.x & 31) == leader && v != 0)
            atomicAdd(&gst->c[k], (unsigned long long)v);
    }
#endif
}


#ifndef QR_STATS
/*
 * Batched persistent launch: every request of a batch is cut into warp
 * tiles of tw x th pixels (tw * th = 32), numbered request after request;
 * each warp claims `grab` tiles at a time from a global counter until none
 * are left, staging the request's scene and frame parameters in shared
 * memory when it moves to another request.  One kernel per mode (Whitted or
 * path tracer), so each keeps only its own code.
 */
template <int MODE>
__global__ void __launch_bounds__(128, MODE == 0 ? QR_MIN_BLOCKS : QR_PT_MIN_BLOCKS)
batch_kernel(const qr_job *__restrict__ jobs, int njobs, int total, int *counter,
             int tw, int th, int grab, int once, int *tiles_done, uint32_t *done)
{
    __shared__ qr_dscene sS[4];
    __shared__ qr_frame_params sP[4];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.y;
    int cur = -1;
    /* once: a warp takes one run of tiles and its block retires when its
     * warps are done, so kernels of higher-priority streams get SMs as
     * blocks finish; else warps claim runs until none are left */
    #pragma unroll 1
    for (int claim = 0; !once || claim == 0; claim++)
    {
        int t0 = 0;
        if (lane == 0) t0 = atomicAdd(counter, grab);
        t0 = __shfl_sync(0xFFFFFFFFu, t0, 0);
        if (t0 >= total) break;
        const int t1 = min(t0 + grab, total);
        #pragma unroll 1
        for (int t = t0; t < t1; t++)
        {
            /* request of tile t: the last job whose first tile is <= t */
            int lo = 0, hi = njobs - 1;
            while (lo < hi)
            {
                const int mid = (lo + hi + 1) >> 1;
                if (__ldg(&jobs[mid].tile0) <= t) lo = mid; else hi = mid - 1;
            }
            if (lo != cur)
            {
                __syncwarp();
                const uint32_t *src = (const uint32_t *)&jobs[lo].S;
                uint32_t *dst = (uint32_t *)&sS[wid];
                for (int i = lane; i < (int)(sizeof(qr_dscene) / 4); i += 32) dst[i] = __ldg(&src[i]);
                src = (const uint32_t *)&jobs[lo].P;
                dst = (uint32_t *)&sP[wid];
                for (int i = lane; i < (int)(sizeof(qr_frame_params) / 4); i += 32) dst[i] = __ldg(&src[i]);
                __syncwarp();
                cur = lo;
            }
            const qr_job *__restrict__ J = &jobs[lo];
            const int local = t - __ldg(&J->tile0);
            const int tx = __ldg(&J->tiles_x);
            /* 4x AA requests: a tile is 4 x 2 pixels and a thread a
             * sub-sample (the whole warp takes part in the shuffle
             * average); otherwise a tile is tw x th pixels, a thread a
             * pixel.  One camera-ray call site serves both. */
            const int aa = MODE == 0 && sP[wid].fsaa == 2;
            const int pix = lane >> 2, sub = lane & 3;
            const int x = aa ? (local % tx) * 4 + (pix & 3) : (local % tx) * tw + lane % tw;
            const int y = aa ? (local / tx) * 2 + (pix >> 2) : (local / tx) * th + lane / tw;
            const int inside = x < sP[wid].x_res && y < sP[wid].y_res;
            if (MODE == 0)
            {
                /* a thread's samples: one, or its pixel's two of 2x AA */
                const int n2 = (!aa && sP[wid].fsaa == 1) ? 2 : 1;
                float c[3] = {0.0f, 0.0f, 0.0f}, h0[3];
                #pragma unroll 1
                for (int s = 0; s < n2 && inside; s++)
                {
                    float hs = (float)x, vs = (float)y;
                    if (aa) { hs = hs + c_aa4_h[sub]; vs = vs + c_aa4_v[sub]; }
                    if (n2 == 2) { hs = hs + c_aa2_h[x & 1][s]; vs = vs + c_aa2_v[x & 1][s]; }
                    float cc[3];
                    primary(sS[wid], sP[wid], x, y, hs, vs, cc, NULL);
                    #pragma unroll
                    for (int k = 0; k < 3; k++)
                    {
                        cc[k] = clamp1(cc[k]);
                        if (n2 == 1)     c[k] = cc[k];
                        else if (s == 0) h0[k] = cc[k] * 0.5f;
                        else             c[k] = h0[k] + cc[k] * 0.5f;
                    }
                }
                if (aa)
                {
                    float col[3];
                    #pragma unroll
                    for (int k = 0; k < 3; k++)
                    {
                        const float h = c[k] * 0.5f;
                        const float pr = h + __shfl_xor_sync(0xFFFFFFFFu, h, 1);
                        const float q = pr * 0.5f;
                        col[k] = q + __shfl_xor_sync(0xFFFFFFFFu, q, 2);
                    }
                    if (inside && sub == 0)
                        J->frame[(size_t)y * sP[wid].x_row + x] = pack(sP[wid], col);
                }
                else if (inside)
                {
                    J->frame[(size_t)y * sP[wid].x_row + x] = pack(sP[wid], c);
                }
            }
            else if (inside)
            {
                pt_pixel_seq(sS[wid], sP[wid], x, y, J->acc, J->frame, NULL);
            }
            /* the tile's pixels are written (the warp barrier orders the
             * lanes' stores before lane 0's fence): count the tile; the
             * warp with the request's last tile publishes its completion */
            __syncwarp();
            if (lane == 0)
            {
                __threadfence();
                const int d = atomicAdd(&tiles_done[lo], 1) + 1;
                if (d == __ldg(&J->ntiles))
                {
                    __threadfence_system();
                    *(volatile uint32_t *)&done[__ldg(&J->req)] = 1u;
                }
            }
        }
    }
}
#endif

} /* namespace QR_NS */

#ifndef QR_STATS
cudaError_t qr_launch_batch(int mode, const qr_job *jobs, int njobs, int total_tiles,
                            int *counter, int tw, int th, int grab, int blocks, int once,
                            int *tiles_done, uint32_t *done, cudaStream_t stream)
{
    if (njobs <= 0 || total_tiles <= 0) return cudaSuccess;
    const dim3 block(32, 4);
    /* one run of grab tiles a warp: as many blocks as runs / 4 */
    if (once) blocks = (int)(((long long)total_tiles + 4ll * grab - 1) / (4ll * grab));
    if (mode == 0)
        QR_NS::batch_kernel<0><<<blocks, block, 0, stream>>>(jobs, njobs, total_tiles,
                                                            counter, tw, th, grab, once,
                                                            tiles_done, done);
    else
        QR_NS::batch_kernel<1><<<blocks, block, 0, stream>>>(jobs, njobs, total_tiles,
                                                            counter, tw, th, grab, once,
                                                            tiles_done, done);
    qr_note_launches(stream, 1);
    return cudaGetLastError();
}

int qr_batch_blocks_per_sm(int mode)
{
    int n = 0;
    cudaError_t e = mode == 0
        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, QR_NS::batch_kernel<0>, 128, 0)
        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, QR_NS::batch_kernel<1>, 128, 0);
    return e == cudaSuccess ? n : 0;
}
#endif

#ifdef QR_STATS
cudaError_t qr_launch_pt_stats(const qr_dscene &sc, const qr_frame_params &fp, float *acc,
                               uint32_t *dev_frame, qr_dstats *dstats,
                               cudaStream_t stream)
#else
cudaError_t qr_launch_pt(const qr_dscene &sc, const qr_frame_params &fp, float *acc,
                         uint32_t *dev_frame, cudaStream_t stream)
#endif
{
    const dim3 block(32, 4);
    const dim3 grid((fp.x_res + 2 * QR_TILE_W - 1) / (2 * QR_TILE_W),
                    (fp.y_res + 2 * QR_TILE_H - 1) / (2 * QR_TILE_H));
#ifdef QR_STATS
    qr_dstats *ds = dstats;
#else
    qr_dstats *ds = NULL;
#endif
    if (fp.pt_on >= QR_PT_FLAT_SPP)
        QR_NS::pt_kernel<1><<<grid, block, 0, stream>>>(sc, fp, acc, dev_frame, ds);
    else
        QR_NS::pt_kernel<0><<<grid, block, 0, stream>>>(sc, fp, acc, dev_frame, ds);
    qr_note_launches(stream, 1);
    return cudaGetLastError();
}

#ifdef QR_STATS
cudaError_t qr_launch_whitted_stats(const qr_dscene &sc, const qr_frame_params &fp,
                                    uint32_t *dev_frame, qr_dstats *dstats,
                                    cudaStream_t stream)
#else
cudaError_t qr_launch_whitted(const qr_dscene &sc, const qr_frame_params &fp,
                              uint32_t *dev_frame, cudaStream_t stream)
#endif
{
    const dim3 block(32, 4);
#ifndef QR_STATS
    qr_dstats *dstats = NULL;
#endif
    if (fp.fsaa == 2 && !(fp.flags & QR_FP_PIXEL_THREADS))
    {
        const dim3 grid((fp.x_res + 7) / 8, (fp.y_res + 3) / 4);
        QR_NS::whitted_aa_kernel<<<grid, block, 0, stream>>>(sc, fp, dev_frame, dstats);
        qr_note_launches(stream, 1);
        return cudaGetLastError();
    }
    const dim3 grid((fp.x_res + 2 * QR_TILE_W - 1) / (2 * QR_TILE_W),
                    (fp.y_res + 2 * QR_TILE_H - 1) / (2 * QR_TILE_H));
    QR_NS::whitted_kernel<<<grid, block, 0, stream>>>(sc, fp, dev_frame, dstats);
    qr_note_launches(stream, 1);
    return cudaGetLastError();
}


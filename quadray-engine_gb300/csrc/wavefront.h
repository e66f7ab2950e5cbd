/*
 * wavefront.h: host side of the wavefront path tracer (wavefront.cu).
 */
#ifndef QR_WAVEFRONT_H
#define QR_WAVEFRONT_H

#include <cuda_runtime.h>
#include <stddef.h>
#include "tracer.cuh"

/* capacities of a frame's scratch: paths of a chunk, rays of a level's
 * queue, nodes of a chunk's pool, pixels of the frame */
struct qr_wf_caps
{
    long long cap_paths, cap_q, cap_pool, cap_px;
};

/* the capacities for a frame: chunks of at most max_paths paths, queues
 * of q_per_path rays and a pool of pool_per_path nodes a path of a chunk
 * (at least one each) */
qr_wf_caps qr_wf_caps_for(const qr_frame_params &fp, long long max_paths, int q_per_path,
                          int pool_per_path);
/* device bytes of a scratch block with these capacities */
size_t qr_wf_bytes(const qr_wf_caps &caps);
/* a second chunk in flight: its scratch (qr_wf_bytes(caps) bytes), the
 * stream it runs on and three events of the caller's (disable-timing) */
struct qr_wf_second
{
    void        *scratch;
    cudaStream_t stream;
    cudaEvent_t  ev[3];
};

/* path-trace fp.pt_on samples a pixel into acc / frame (as qr_launch_pt)
 * with the wavefront stages, using `scratch` (qr_wf_bytes(caps) bytes, 256
 * aligned, not shared with work in flight); `sms` = the device's SMs.
 * With `second`, chunks alternate between the two scratch blocks and
 * streams, so one chunk's stage tails overlap the next chunk's stages;
 * each chunk's samples still join the sums after the chunk before it */
cudaError_t qr_wf_launch_pt(const qr_dscene &sc, const qr_frame_params &fp, float *acc,
                            uint32_t *frame, void *scratch, const qr_wf_caps &caps,
                            int sms, cudaStream_t stream,
                            const qr_wf_second *second = NULL);
/* resident blocks a SM of the stages' tracing kernel (queried once; call it
 * before a stream capture that holds wavefront launches) */
int qr_wf_prepare(void);
/* set done[req] to 1 on `stream` once the work before it has run (done may
 * be host memory mapped into the device) */
cudaError_t qr_wf_mark_done(uint32_t *done, int req, cudaStream_t stream);
/* whether the last frame rendered with this scratch overflowed its queues
 * (and was rendered by the per-pixel kernel instead); synchronises stream */
int qr_wf_overflowed(const void *scratch, cudaStream_t stream, int *out);

#endif /* QR_WAVEFRONT_H */

/*
 * whitted_wf.h: host side of the wavefront Whitted tracer (whitted_wf.cu).
 */
#ifndef QR_WHITTED_WF_H
#define QR_WHITTED_WF_H

#include <cuda_runtime.h>
#include <stddef.h>
#include "tracer.cuh"

/* capacities of a frame's scratch: samples of a chunk, rays of a level's
 * queue, shadow rays of a level, nodes of a chunk's pool; ok = 0 when the
 * scene's light lists are too long for the stages (the per-pixel kernel
 * renders such scenes) */
struct qr_wh_caps
{
    long long cap_samples, cap_q, cap_s, cap_pool;
    int ok;
};

/* capacities for a frame of a scene whose light lists hold at most
 * max_lights lights: chunks of at most max_samples camera rays (fewer when
 * many lights make the shadow queue long) */
qr_wh_caps qr_wh_caps_for(const qr_frame_params &fp, int max_lights, long long max_samples);
size_t qr_wh_bytes(const qr_wh_caps &caps);
/* render a Whitted frame (as qr_launch_whitted) with the wavefront stages,
 * using `scratch` (qr_wh_bytes(caps) bytes, not shared with work in flight) */
cudaError_t qr_wh_launch(const qr_dscene &sc, const qr_frame_params &fp, uint32_t *frame,
                         void *scratch, const qr_wh_caps &caps, int sms, cudaStream_t stream);

#endif /* QR_WHITTED_WF_H */

/*
 * qr_oracle.h: CPU restatement of the QuadRay Whitted render path.
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline).
 */
#ifndef QR_ORACLE_H
#define QR_ORACLE_H

#include <stdint.h>
#include "qr_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* render rows [y0, y1) of the frame into frame[y * x_row + x] (XRGB);
 * nrays (optional) receives the number of traced segments */
int qr_oracle_render(const qr_scene_desc *d, const qr_frame_params *fp,
                     uint32_t *frame, int y0, int y1, uint64_t *nrays);

/* the hit-ID exclusion mask of rows [y0, y1): mask[y * x_res + x] = 1 where
 * a camera ray of the pixel (every AA sub-sample) meets, no farther than
 * its hit, a solver or clipper decision within 1e-5 relative of its
 * boundary (a tangent, a clip boundary, two surfaces at the same distance):
 * there float rounding may pick either surface */
int qr_oracle_boundary(const qr_scene_desc *d, const qr_frame_params *fp, uint8_t *mask,
                       int y0, int y1);

/* path tracer: add fp->pt_on samples per pixel of rows [y0, y1) to the
 * running sums acc[3 * (y * x_row + x)] (reset first when fp->pts_c == 0;
 * the element type is the build's precision: float, or double with
 * QR_ORACLE_FP64) and, when frame is not NULL, write the mean over
 * pts_c + pt_on samples as XRGB */
int qr_oracle_pt(const qr_scene_desc *d, const qr_frame_params *fp, void *acc,
                 uint32_t *frame, int y0, int y1, uint64_t *nrays);

#ifdef __cplusplus
}
#endif

#endif /* QR_ORACLE_H */

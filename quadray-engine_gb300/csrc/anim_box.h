/*
 * anim_box.h: the box stage of the device-side update (anim.cu stage 3) as
 * host-and-device functions, so that host tests run the same float steps:
 * a record's world-from-local frame, a term's world box (accel.cpp
 * world_box / affine_image in float) and a surface's box at one level (the
 * meet of its terms, padded as accel.cpp pad does).
 */
#ifndef QR_ANIM_BOX_H
#define QR_ANIM_BOX_H

#include <math.h>
#include "qr_gpu.h"
#include "accel.h"
#include "xform.h"

namespace qr
{

/* world-from-local matrix of a record's frame (accel.cpp
 * qr_accel_record_frame, in float): the inverse of the transform rows as the
 * tracer applies them (diagonal only when amap[3] == 1, "scaling only");
 * f[9] = 1 when singular */
QR_HD void record_frame(const qr_srf &t, float *f)
{
    float m[3][3];
    const float *row[3] = {t.tci, t.tcj, t.tck};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            m[i][j] = (t.amap[3] == 1 && i != j) ? 0.0f : row[i][j];
    const float c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
    const float c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
    const float c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
    const float det = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
    if (!(fabsf(det) > 1e-30f))
    {
        f[9] = 1.0f;
        return;
    }
    const float id = 1.0f / det;
    f[0] = c00 * id;
    f[1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
    f[2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
    f[3] = c01 * id;
    f[4] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
    f[5] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
    f[6] = c02 * id;
    f[7] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
    f[8] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
    f[9] = 0.0f;
}

/* world box of one term at level l (accel.h, QR_TERM_*) from the records
 * srf and their frames (10 floats each); false when the frame is singular */
QR_HD bool term_box(const qr_srf *srf, const float *frame, const qr_anim_term &t, int l,
                    float lo[3], float hi[3])
{
    const qr_srf &s = srf[t.srf];
    const bool node = t.mode == QR_TERM_NODE || t.mode == QR_TERM_NODE_SHIFT;
    const int fr = node ? t.xf : t.srf;
    const qr_srf &F = srf[fr];
    float u[6];
    for (int k = 0; k < 6; k++) u[k] = t.u[l][k];
    if (node)
    {
        for (int k = 0; k < 3; k++)
        {
            u[k] += s.pos[k];
            u[3 + k] += s.pos[k];
        }
    }
    if (t.mode == QR_TERM_NODE_SHIFT || t.mode == QR_TERM_OWN_SHIFT)
    {
        for (int k = 0; k < 3; k++)
        {
            lo[k] = u[k] + F.pos[k];
            hi[k] = u[3 + k] + F.pos[k];
        }
        return true;
    }
    const float *a = frame + 10 * (size_t)fr;
    if (a[9] != 0.0f) return false;
    /* interval image of u under h = a u + o (accel.cpp affine_image) */
    for (int i = 0; i < 3; i++)
    {
        float l0 = F.pos[i], h0 = F.pos[i];
        for (int j = 0; j < 3; j++)
        {
            const float c = a[3 * i + j];
            if (c == 0.0f) continue;
            const float p = c * u[j], q = c * u[3 + j];
            if (p != p || q != q) { l0 = -HUGE_VALF; h0 = HUGE_VALF; break; }
            l0 += fminf(p, q);
            h0 += fmaxf(p, q);
        }
        lo[i] = l0;
        hi[i] = h0;
    }
    return true;
}

/* a target surface's box at level l (< QR_BVH_LEVELS): the meet of its
 * terms, padded (accel.cpp pad); false when a frame is singular or the box
 * is empty or unbounded */
QR_HD bool target_box(const qr_srf *srf, const float *frame, const qr_anim_term *terms,
                      const qr_anim_target &tg, int l, float b[6])
{
    float lo[3] = {-HUGE_VALF, -HUGE_VALF, -HUGE_VALF};
    float hi[3] = {HUGE_VALF, HUGE_VALF, HUGE_VALF};
    bool ok = true;
    for (int j = 0; j < tg.tn && ok; j++)
    {
        float tl[3], th[3];
        ok = term_box(srf, frame, terms[tg.t0 + j], l, tl, th);
        for (int k = 0; k < 3 && ok; k++)
        {
            lo[k] = fmaxf(lo[k], tl[k]);
            hi[k] = fminf(hi[k], th[k]);
        }
    }
    for (int k = 0; k < 3 && ok; k++)
        ok = lo[k] <= hi[k] && lo[k] > -HUGE_VALF && hi[k] < HUGE_VALF;
    if (!ok) return false;
    for (int k = 0; k < 3; k++)
    {
        const float m = 1e-3f + 1e-4f * (fabsf(lo[k]) + fabsf(hi[k]));
        b[k] = lo[k] - m;
        b[3 + k] = hi[k] + m;
    }
    return true;
}

} /* namespace qr */

#endif /* QR_ANIM_BOX_H */

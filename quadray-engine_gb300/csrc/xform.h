/*
 * xform.h: the 4x4 matrix steps of the update phases (core/engine/rtgeom.cpp
 * 59-228), shared by the host flattening (flatten.cpp) and the device-side
 * update of animated surfaces (anim.cu), so both form the same bits: float
 * arithmetic in the reference's operation order, no fused multiply-add
 * (host -ffp-contract=off, device -fmad=false) and IEEE division.
 * Matrices are column-major: m[column][row], the translation in m[3].
 */
#ifndef QR_XFORM_H
#define QR_XFORM_H

#ifdef __CUDACC__
#define QR_HD __host__ __device__ inline
#else
#define QR_HD inline
#endif

namespace qr
{

QR_HD void mat_mul_vec(float vp[4], const float (*m1)[4], const float v1[4])
{
    for (int i = 0; i < 4; i++)
    {
        vp[i] = m1[0][i] * v1[0] +
                m1[1][i] * v1[1] +
                m1[2][i] * v1[2] +
                m1[3][i] * v1[3];
    }
}

QR_HD void mat_mul_mat(float (*mp)[4], const float (*m1)[4], const float (*m2)[4])
{
    for (int i = 0; i < 4; i++)
    {
        mat_mul_vec(mp[i], m1, m2[i]);
    }
}

/* T * Rz * Ry * Rx * S (rtgeom.cpp:102-164) from the sines and cosines of
 * the three rotation angles, the translation and the scale */
QR_HD void mat_from_sc(float (*mp)[4], const float s3[3], const float c3[3],
                       const float pos[3], const float scl[3])
{
    float mt[4][4];
    const float sc[4][4] = {{scl[0], 0, 0, 0}, {0, scl[1], 0, 0}, {0, 0, scl[2], 0},
                            {0, 0, 0, 1}};
    float s = s3[0], c = c3[0];
    const float rx[4][4] = {{1, 0, 0, 0}, {0, +c, +s, 0}, {0, -s, +c, 0}, {0, 0, 0, 1}};
    s = s3[1]; c = c3[1];
    const float ry[4][4] = {{+c, 0, -s, 0}, {0, 1, 0, 0}, {+s, 0, +c, 0}, {0, 0, 0, 1}};
    s = s3[2]; c = c3[2];
    const float rz[4][4] = {{+c, +s, 0, 0}, {-s, +c, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    const float ps[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0},
                            {pos[0], pos[1], pos[2], 1}};

    mat_mul_mat(mt, rx, sc);
    mat_mul_mat(mp, ry, mt);
    mat_mul_mat(mt, rz, mp);
    mat_mul_mat(mp, ps, mt);
}

/* 3x3 inverse by cofactors (rtgeom.cpp:167-195) */
QR_HD void mat_inverse(float (*mp)[4], const float (*m1)[4])
{
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) mp[i][j] = 0.0f;

    float a = m1[1][1] * m1[2][2] - m1[2][1] * m1[1][2];
    float b = m1[2][1] * m1[0][2] - m1[0][1] * m1[2][2];
    float c = m1[0][1] * m1[1][2] - m1[1][1] * m1[0][2];

    float d = m1[2][0] * m1[1][2] - m1[1][0] * m1[2][2];
    float e = m1[0][0] * m1[2][2] - m1[2][0] * m1[0][2];
    float f = m1[0][2] * m1[1][0] - m1[0][0] * m1[1][2];

    float g = m1[1][0] * m1[2][1] - m1[2][0] * m1[1][1];
    float h = m1[2][0] * m1[0][1] - m1[0][0] * m1[2][1];
    float l = m1[0][0] * m1[1][1] - m1[1][0] * m1[0][1];

    float q = 1.0f / (m1[0][0] * a + m1[1][0] * b + m1[2][0] * c);

    mp[0][0] = a * q; mp[0][1] = b * q; mp[0][2] = c * q;
    mp[1][0] = d * q; mp[1][1] = e * q; mp[1][2] = f * q;
    mp[2][0] = g * q; mp[2][1] = h * q; mp[2][2] = l * q;
}

} /* namespace qr */

#endif /* QR_XFORM_H */

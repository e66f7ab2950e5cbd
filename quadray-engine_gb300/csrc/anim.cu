/*
 * anim.cu: device-side update phases of animated scenes, one block per
 * scene and one launch for all the scenes of a batch (a scene's work is a
 * few hundred matrices and boxes; one block keeps the ordering between its
 * stages to block barriers, and the blocks of different scenes run side by
 * side).
 *
 * Stage 1  transform chain, generation by generation: the matrices of
 *          rt_Object::update_matrix (core/engine/object.cpp:221-389) with
 *          the shared matrix steps of xform.h, so the records equal those
 *          of the host update bit for bit (no FMA contraction, IEEE
 *          division: the library's device flags).
 * Stage 2  records: inverse matrix rows tci/tcj/tck and position
 *          (rt_Node::update_fields, object.cpp:826-857), light positions
 *          (the light's pos in rt_Light::update_fields, object.cpp:649-667).
 * Stage 3  world boxes of the surfaces that move, as accel.cpp forms them
 *          (world_box, affine_image, pad) but in float: the pad (1e-3 +
 *          1e-4 of the coordinates) is far above float rounding, and the
 *          local boxes are rounded outwards; and the check that every
 *          moved record and surface stays inside the motion bound the
 *          boxes' rounding allowance was sized for.
 * Stage 4  hierarchy node boxes bottom-up by depth band; when the check
 *          failed, every node box is opened instead, so every ray walks
 *          every surface and the frame stays exact.
 */
#include <float.h>
#include <math.h>
#include "anim.cuh"
#include "tracer.cuh"
#include "anim_box.h"
#include "xform.h"

namespace
{

__device__ void load16(float (*m)[4], const float *p)
{
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) m[i][j] = p[4 * i + j];
}

__device__ void store16(float *p, const float (*m)[4])
{
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) p[4 * i + j] = m[i][j];
}

__device__ bool inside(const float ext[6], const float lo[3], const float hi[3])
{
    for (int k = 0; k < 3; k++)
        if (!(lo[k] >= ext[k] && hi[k] <= ext[3 + k])) return false;
    return true;
}

__global__ void __launch_bounds__(512) anim_kernel(const qr_anim_dev *devs)
{
    __shared__ int fail;
    __shared__ qr_anim_dev A;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (tid == 0)
    {
        fail = 0;
        A = devs[blockIdx.x];
    }
    __syncthreads();

    /* stage 1: matrices, parents before children */
    for (int g = 0; g < A.ngen; g++)
    {
        for (int i = A.gen_off[g] + tid; i < A.gen_off[g + 1]; i += nt)
        {
            const int e = A.order[i];
            const qr_anim_node &N = A.nodes[e];
            float P[4][4], R[4][4], M[4][4], T[4][4], tmp[4][4];
            load16(P, N.p);
            if (N.kind != QR_ANIM_NODE)
            {
                if (N.param >= 0)
                {
                    const qr_anim_param &q = A.params[N.param];
                    const float one[3] = {1.0f, 1.0f, 1.0f};
                    qr::mat_from_sc(R, q.sin, q.cos, q.pos, one);
                }
                else
                {
                    load16(R, N.r);
                }
            }
            if (N.kind != QR_ANIM_OWN) load16(T, A.mtx + 16 * (size_t)N.parent);
            if (N.kind == QR_ANIM_OWN)
            {
                qr::mat_mul_mat(M, P, R);
            }
            else if (N.kind == QR_ANIM_UNDER)
            {
                qr::mat_mul_mat(tmp, T, P);
                qr::mat_mul_mat(M, tmp, R);
            }
            else
            {
                qr::mat_mul_mat(M, T, P);
            }
            store16(A.mtx + 16 * (size_t)e, M);
        }
        __syncthreads();
    }

    /* stage 2: records and lights */
    for (int e = tid; e < A.n; e += nt)
    {
        const qr_anim_node &N = A.nodes[e];
        float M[4][4];
        load16(M, A.mtx + 16 * (size_t)e);
        if (N.rec >= 0)
        {
            float inv[4][4];
            qr::mat_inverse(inv, M);
            qr_srf &s = A.srf[N.rec];
            for (int k = 0; k < 3; k++)
            {
                s.tci[k] = inv[k][0];
                s.tcj[k] = inv[k][1];
                s.tck[k] = inv[k][2];
                s.pos[k] = M[3][k];
            }
            qr::record_frame(s, A.frame + 10 * (size_t)N.rec);
            /* record positions bound the local coordinates the walk forms
             * (light positions take no part, as in the host build) */
            const float p[3] = {M[3][0], M[3][1], M[3][2]};
            if (!inside(A.ext, p, p)) fail = 1;
        }
        if (N.light >= 0)
        {
            for (int k = 0; k < 3; k++) A.lgt[N.light].pos[k] = M[3][k];
        }
    }
    __syncthreads();

    /* stage 3: world boxes of the moved surfaces per level, and the extent
     * check on their boxes without rounding allowance */
    const int L = QR_BVH_LEVELS;
    for (int w = tid; w < A.ntargets * (L + 1); w += nt)
    {
        const qr_anim_target tg = A.targets[w / (L + 1)];
        const int l = w % (L + 1);
        if (l < L && ((tg.levels >> l) & 1) == 0) continue;
        if (l == L)
        {
            /* the extent holds the finite ones of these boxes (a quadric
             * that only its clippers bound has none), as in the host build */
            float lo[3], hi[3];
            const bool ok = qr::term_box(A.srf, A.frame, A.terms[tg.t0], L, lo, hi);
            bool fin = ok;
            for (int k = 0; k < 3; k++)
                fin = fin && lo[k] > -HUGE_VALF && hi[k] < HUGE_VALF && lo[k] <= hi[k];
            if (!ok || (fin && !inside(A.ext, lo, hi))) fail = 1;
            continue;
        }
        if (!qr::target_box(A.srf, A.frame, A.terms, tg, l,
                            A.lboxes + ((size_t)l * A.nsrf + tg.srf) * 6))
            fail = 1;
    }
    __syncthreads();

    /* stage 4: node boxes */
    if (fail)
    {
        for (int i = tid; i < A.nbvh; i += nt)
        {
            qr_bnode &nd = A.bvh[i];
            for (int k = 0; k < 3; k++) { nd.lo[k] = -1e30f; nd.hi[k] = 1e30f; }
        }
    }
    else
    {
        for (int band = 0; band < A.nbands; band++)
        {
            for (int i = A.depth_off[band] + tid; i < A.depth_off[band + 1]; i += nt)
            {
                const int ni = A.rorder[i];
                qr_bnode &nd = A.bvh[ni];
                float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
                float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
                if (nd.count > 0)
                {
                    int l = 0;
                    while (l < L - 1 && ni >= A.lvl_end[l]) l++;
                    for (int j = nd.a; j < nd.a + nd.count; j++)
                    {
                        const float *b = A.lboxes + ((size_t)l * A.nsrf + A.items[j].srf) * 6;
                        for (int k = 0; k < 3; k++)
                        {
                            lo[k] = fminf(lo[k], b[k]);
                            hi[k] = fmaxf(hi[k], b[3 + k]);
                        }
                    }
                }
                else
                {
                    const qr_bnode &ca = A.bvh[nd.a], &cb = A.bvh[nd.b];
                    for (int k = 0; k < 3; k++)
                    {
                        lo[k] = fminf(ca.lo[k], cb.lo[k]);
                        hi[k] = fmaxf(ca.hi[k], cb.hi[k]);
                    }
                }
                for (int k = 0; k < 3; k++) { nd.lo[k] = lo[k]; nd.hi[k] = hi[k]; }
            }
            __syncthreads();
        }
    }
    __syncthreads();

    /* stage 5: the walk's records take the nodes' new boxes (the codes,
     * which follow the topology, stay) */
    for (int w = tid; w < 4 * A.nquads; w += nt)
    {
        const int sn = A.quad_src[w];
        if (sn < 0) continue;
        const qr_bnode &c = A.bvh[sn];
        qr_bquad &q = A.quads[w >> 2];
        const int k = w & 3;
        q.lo_x[k] = c.lo[0]; q.lo_y[k] = c.lo[1]; q.lo_z[k] = c.lo[2];
        q.hi_x[k] = c.hi[0]; q.hi_y[k] = c.hi[1]; q.hi_z[k] = c.hi[2];
    }
    for (int i = tid; i < A.nbvh; i += nt)
    {
        const qr_bnode &nd = A.bvh[i];
        if (nd.count > 0) continue;
        const qr_bnode &ca = A.bvh[nd.a], &cb = A.bvh[nd.b];
        qr_bpair &pr = A.pairs[i];
        for (int k = 0; k < 3; k++)
        {
            pr.lo_a[k] = ca.lo[k];
            pr.hi_a[k] = ca.hi[k];
            pr.lo_b[k] = cb.lo[k];
            pr.hi_b[k] = cb.hi[k];
        }
    }
    if (tid == 0)
    {
        A.status[0] += 1;
        if (fail) A.status[1] += 1;
    }
}

} /* namespace */

cudaError_t qr_launch_anim(const qr_anim_dev *devs, int n, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    anim_kernel<<<n, 512, 0, stream>>>(devs);
    qr_note_launches(stream, 1);
    return cudaGetLastError();
}

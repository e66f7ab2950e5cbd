/*
 * tracer_dev.cuh: device code of the GB300 QuadRay tracer shared by its
 * kernels (tracer.cu: one thread a pixel or AA sub-sample, the batched
 * persistent kernel; wavefront.cu: the wavefront path tracer).
 *
 * Ray generation, list walk with plane / quadric / two-plane solvers,
 * clipping (axis boxes, custom clippers, boolean accumulators, conic apex
 * adjustment), shading with hard shadows to every light, refraction and
 * reflection with Fresnel, the 8-bit pack, and the path tracer's node
 * shading.  The arithmetic restates the reference's fp32 SIMD tracer
 * (VectorChief/QuadRay-engine core/tracer/tracer.cpp render0, 2086-7622)
 * operation by operation so the frames are bit-identical to the reference's
 * CPU render; it is compiled with -fmad=false -prec-div=true
 * -prec-sqrt=true -ftz=false, and divisions and square roots use the IEEE
 * round-to-nearest intrinsics.
 *
 * Per-lane view of the reference's SIMD masks: the reference shades every
 * surface that is nearest so far; per lane that is the nearest hit in walk
 * order (a later hit wins only if strictly nearer), which is what these
 * functions keep and shade once.
 *
 * Every translation unit that includes this file gets its own copy (device
 * code is compiled per unit); constant tables are static.
 */
#ifndef QR_TRACER_DEV_CUH
#define QR_TRACER_DEV_CUH

#include <cuda_runtime.h>
#include <stdint.h>
#include <float.h>

#include "tracer.cuh"

#define FLAG_PASS   2
#define FLAG_SHAD   4
#define SIDE_OUTER  0
#define SIDE_INNER  1
#define D_EPS       0.00000000001f  /* root-sorting threshold, object.h:41 */
#define T_EPS       0.0000001f      /* root-split threshold, object.h:42 */
#define SIGN_BIT    0x80000000u
#define QR_CODE_NONE ((int)0x80000000)  /* no code (qr_bpair codes are above it) */

/*
 * Work counters: with QR_STATS defined (tracer_stats.cu) the code lives in
 * namespace qr_dev_stats and every counted event increments a per-thread
 * counter; otherwise (the timed kernels) in namespace qr_dev, with no
 * counter code at all.
 */
#ifdef QR_STATS
#define QR_NS qr_dev_stats
#else
#define QR_NS qr_dev
#endif

namespace QR_NS
{

#ifdef QR_STATS
struct TCnt { uint32_t c[QR_STAT_COUNT]; };
typedef TCnt *StP;
#define CNT(k) (st->c[k]++)
#else
typedef void *StP;
#define CNT(k) ((void)0)
#endif

struct Ray
{
    float org[3];
    float dir[3];
    float t_min, t_max;
    int   from;         /* originating surface, -1 for camera rays */
    int   flags;        /* side | pass | shadow */
    float phit[3];      /* originating surface's local hit */
    int   depth;        /* remaining secondary-ray depth */
};

struct Hit
{
    int   srf;
    int   side;
    float hit[3];
    float loc[3];
};

struct Walk
{
    int   shadow;
    int   occluded;
    float tbuf;
    int   bestp;        /* list position of the nearest hit (-1: none) */
    Hit   best;
    int   fault;        /* QR_FAULT_STACK when the walk gave up */
};

__device__ __forceinline__ uint32_t f2u(float f) { return __float_as_uint(f); }
__device__ __forceinline__ float u2f(uint32_t u) { return __uint_as_float(u); }
__device__ __forceinline__ float fxor(float a, uint32_t m) { return u2f(f2u(a) ^ m); }
__device__ __forceinline__ uint32_t sgnbit(float a) { return f2u(a) & SIGN_BIT; }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }
/* 128-bit read-only loads of the 16-byte groups of the records (qr_srf,
 * qr_elem, qr_bitem, qr_bnode are laid out in such groups) */
__device__ __forceinline__ float4 ldf4(const float *p)
{
    return __ldg(reinterpret_cast<const float4 *>(p));
}
__device__ __forceinline__ int4 ldi4(const int32_t *p)
{
    return __ldg(reinterpret_cast<const int4 *>(p));
}
/* full-precision rsqrt of the reference's compat mode: 1 / sqrt(x) */
__device__ __forceinline__ float rsq(float x) { return __fdiv_rn(1.0f, __fsqrt_rn(x)); }

/* transform-node matrix times vector, diagonal first (tracer.cpp:2537-2568) */
__device__ __forceinline__ void xform(const qr_srf *__restrict__ t,
                                      const float v[3], float o[3])
{
    const int am = __ldg(&t->amap[3]);
    const float4 a = ldf4(t->tci), b = ldf4(t->tcj), c = ldf4(t->tck);
    float x = a.x * v[0];
    float y = b.y * v[1];
    float z = c.z * v[2];
    if (am != 1)
    {
        x = x + a.y * v[1];
        x = x + a.z * v[2];
        y = y + b.x * v[0];
        y = y + b.z * v[2];
        z = z + c.x * v[0];
        z = z + c.y * v[1];
    }
    o[0] = x; o[1] = y; o[2] = z;
}

/* clipping subroutine for one root (tracer.cpp:2686-3249) */
static __device__ int clip_root(const qr_dscene &S, const Ray &r, int si, float t,
                         const Walk &w, int p, const float ldff[3], const float lray[3],
                         int side, int dmask, uint32_t amask, float hit[3],
                         float loc[3], StP st)
{
    CNT(QR_STAT_CLIP_ROOT);
    const qr_srf *__restrict__ s = &S.srf[si];
    /* depth test (2688-2699); an equal distance wins only from a surface
     * earlier in the list, which is what the in-order walk keeps */
    int valid = ((w.tbuf > t) || (w.tbuf == t && p < w.bestp)) && (r.t_min < t);

    #pragma unroll
    for (int k = 0; k < 3; k++) hit[k] = r.dir[k] * t + r.org[k];

    const int am3 = __ldg(&s->amap[3]);
    if (am3 != 0)
    {
        #pragma unroll
        for (int k = 0; k < 3; k++) loc[k] = lray[k] * t + ldff[k];
    }
    else
    {
        const float4 ps = ldf4(s->pos);
        const float pp[3] = {ps.x, ps.y, ps.z};
        #pragma unroll
        for (int k = 0; k < 3; k++) loc[k] = hit[k] - pp[k];
    }

    const int conic = __ldg(&s->conic);
    if (conic != 0 && dmask)
    {
        /* conic singularity adjustment near the apex (2795-2945) */
        const int mi = __ldg(&s->amap[0]), mj = __ldg(&s->amap[1]),
                  mk = __ldg(&s->amap[2]);
        float r2 = loc[mi] * loc[mi];
        if (conic != 2) r2 = r2 + loc[mj] * loc[mj];
        r2 = r2 + loc[mk] * loc[mk];
        if (r2 < T_EPS)
        {
            float li, lj = 0.0f, lk, lr, sk;
            li = fxor(1.0f, sgnbit(ldff[mi]));
            sk = __ldg(&s->sci[mi]);
            lr = 1.0f;
            if (conic != 2)
            {
                lj = fxor(1.0f, sgnbit(ldff[mj]));
                sk = sk + __ldg(&s->sci[mj]);
                lr = lr + 1.0f;
            }
            sk = fdiv(sk, __ldg(&s->sci[mk]));
            sk = fxor(sk, SIGN_BIT);
            lk = fsqrt(sk);
            float inv = rsq(sk + lr);
            inv = inv * T_EPS;
            li = li * inv;
            lj = lj * inv;
            lk = lk * inv;
            const uint32_t tside = side ? SIGN_BIT : 0u;
            lk = fxor(lk, sgnbit(ldff[mk]));
            lk = fxor(lk, amask & ~tside);
            li = fxor(li, tside & ~amask);
            lj = fxor(lj, tside & ~amask);
            loc[mi] = li;
            if (conic != 2) loc[mj] = lj;
            loc[mk] = lk;
        }
    }

    /* axis clippers (2963-3014) */
    const float4 bn = ldf4(s->bmin), bx = ldf4(s->bmax);
    const int mint = __float_as_int(bn.w), maxt = __float_as_int(bx.w);
    const float bl[3] = {bn.x, bn.y, bn.z}, bh[3] = {bx.x, bx.y, bx.z};
    #pragma unroll
    for (int k = 0; k < 3; k++)
    {
        if ((mint >> k) & 1) valid = valid && (bl[k] <= loc[k]);
        if ((maxt >> k) & 1) valid = valid && (bh[k] >= loc[k]);
    }

    /* custom clippers with boolean accumulator segments (3020-3240) */
    const int cnum = __ldg(&s->clip_num);
    if (cnum > 0)
    {
        const int coff = __ldg(&s->clip_off);
        int mask = valid, saved = 0, cache_last = -1;
        float nx[3] = {0.0f, 0.0f, 0.0f};
        for (int e = 0; e < cnum; e++)
        {
            const int ei = coff + e;
            const qr_elem *__restrict__ el = &S.elems[ei];
            const int kind = __ldg(&el->kind);
            if (kind == QR_ELM_ACC_ENTER) { saved = mask; mask = 1; continue; }
            if (kind == QR_ELM_ACC_LEAVE) { mask = !mask && saved; continue; }
            const int ref = __ldg(&el->ref);
            const qr_srf *__restrict__ c = &S.srf[ref];
            float p[3], v;
            if (kind == QR_ELM_TRNODE)
            {
                if (__ldg(&s->trnode) == ref)
                {
                    #pragma unroll
                    for (int k = 0; k < 3; k++) nx[k] = loc[k] + __ldg(&s->pos[k]);
                }
                else
                {
                    #pragma unroll
                    for (int k = 0; k < 3; k++) p[k] = hit[k] - __ldg(&c->pos[k]);
                    if (__ldg(&c->amap[3]) != 0) xform(c, p, nx);
                    else { nx[0] = p[0]; nx[1] = p[1]; nx[2] = p[2]; }
                }
                cache_last = __ldg(&el->last);
                continue;
            }
            if (cache_last >= 0)
            {
                #pragma unroll
                for (int k = 0; k < 3; k++) p[k] = nx[k] - __ldg(&c->pos[k]);
                if (ei == cache_last) cache_last = -1;
            }
            else
            {
                float d[3];
                #pragma unroll
                for (int k = 0; k < 3; k++) d[k] = hit[k] - __ldg(&c->pos[k]);
                if (__ldg(&c->amap[3]) != 0) xform(c, d, p);
                else { p[0] = d[0]; p[1] = d[1]; p[2] = d[2]; }
            }
            CNT(QR_STAT_CLIP_CUSTOM);
            const int clpk = __ldg(&c->clpk);
            if (clpk == 1)
            {
                v = fxor(p[__ldg(&c->amap[2])], __ldg(&c->asgn[2]) ? SIGN_BIT : 0u);
            }
            else
            {
                float d2[3];
                #pragma unroll
                for (int k = 0; k < 3; k++)
                {
                    d2[k] = p[k] * p[k] * __ldg(&c->sci[k]);
                    if (clpk == 2)
                    {
                        const float sj = __ldg(&c->scj[k]);
                        d2[k] = p[k] * p[k] * __ldg(&c->sci[k]) - (sj + sj) * p[k];
                    }
                }
                v = ((d2[0] - __ldg(&c->sci[3])) + d2[1]) + d2[2];
            }
            if (__ldg(&el->rel) < 0) mask = mask && (v >= 0.0f);
            else                    mask = mask && (v <= 0.0f);
        }
        valid = mask;
    }
    return valid;
}

__device__ __forceinline__ void accept_root(const qr_dscene &S, Walk &w, int si,
                                            int p, int side, float t,
                                            const float hit[3],
                                            const float loc[3])
{
    if (w.shadow)
    {
        /* light sources and transparent non-refractive surfaces do not
         * occlude (CHECK_SHAD, 576-616) */
        const int props = __ldg(&S.srf[si].props[side]);
        if (props & QR_PROP_LIGHT) return;
        if ((props & QR_PROP_TRANSP) && !(props & QR_PROP_REFRACT)) return;
        w.occluded = 1;
        return;
    }
    w.tbuf = t;
    w.bestp = p;
    w.best.srf = si;
    w.best.side = side;
    #pragma unroll
    for (int k = 0; k < 3; k++) { w.best.hit[k] = hit[k]; w.best.loc[k] = loc[k]; }
}

/* CHECK_SIDE (558-567) */
__device__ __forceinline__ int side_blocked(const Ray &r, int si, int side)
{
    if (r.from != si) return 0;
    const int f = r.flags & 3;
    return f == 1 - side || f == 2 + side;
}

/* quadric roots with root sorting and splitting (5785-6206) */
static __device__ void root_pair(const qr_dscene &S, const Ray &r, Walk &w, int si, int p,
                          const float ldff[3], const float lray[3],
                          float a, float b, float c, float d, StP st)
{
    if (!(0.0f <= d)) return;
    const float nb = fxor(b, SIGN_BIT);
    const int dmask = d < D_EPS;

    float sd = fsqrt(d);
    sd = fxor(sd, sgnbit(nb));
    const float q = nb + sd;
    const int m_neg = 0.0f > sd;
    float t1n, t1d, t2n, t2d;
    if (m_neg) { t1n = q; t1d = a; t2n = c; t2d = q; }
    else       { t1n = c; t1d = q; t2n = q; t2d = a; }
    const uint32_t amask = sgnbit(a);

    float t1, t2;
    int t1m, t2m;
    if (dmask)
    {
        if (t1n == 0.0f) t1d = 1.0f;
        if (t2n == 0.0f) t2d = 1.0f;
        t1 = fdiv(t1n, t1d);
        t2 = fdiv(t2n, t2d);
        t1m = t1d != 0.0f;
        t2m = t2d != 0.0f;
        float tdff = t1 - t2;
        tdff = fxor(tdff, amask);
        const int fmask = 0.0f <= tdff;
        tdff = fmask ? tdff : 0.0f;
        float teps = fmask ? T_EPS : 0.0f;
        teps = teps * t1;
        teps = fabsf(teps);
        tdff = tdff * -0.5f;
        tdff = tdff - teps;
        tdff = fxor(tdff, amask);
        if (!(t1m && t2m)) tdff = 0.0f;
        t1 = t1 + tdff;
        t2 = t2 - tdff;
    }
    else
    {
        t1 = fdiv(t1n, t1d);
        t2 = fdiv(t2n, t2d);
        t1m = t1d != 0.0f;
        t2m = t2d != 0.0f;
    }

    const int first = (0.0f > a) ? SIDE_INNER : SIDE_OUTER;
    float hit[3], loc[3];
    #pragma unroll 1
    for (int k = 0; k < 2; k++)
    {
        const int side = k == 0 ? first : 1 - first;
        const float t = side == SIDE_OUTER ? t1 : t2;
        const int tm = side == SIDE_OUTER ? t1m : t2m;
        if (side_blocked(r, si, side) || !tm) continue;
        if (clip_root(S, r, si, t, w, p, ldff, lray, side, dmask, amask, hit, loc, st))
        {
            accept_root(S, w, si, p, side, t, hit, loc);
            if (w.shadow && w.occluded) return;
        }
    }
}

/* plane / quadric / two-plane solvers for one surface (5522-6497) on the
 * ray in the surface's local coordinates; p is the surface's list position */
__device__ __forceinline__ void solve_surface(const qr_dscene &S, const Ray &r, Walk &w,
                                              int si, int p, const float ldff[3],
                                              const float lray[3], StP st)
{
    const qr_srf *__restrict__ s = &S.srf[si];
    const int solver = __ldg(&s->solver);
    if (solver == 1)
    {
        /* plane (5545-5634) */
        if (r.from == si) return;
        const int mk = __ldg(&s->amap[2]);
        const uint32_t sg = __ldg(&s->asgn[2]) ? SIGN_BIT : 0u;
        float dk = fxor(ldff[mk], sg);
        const float rk = fxor(lray[mk], sg);
        dk = fxor(dk, SIGN_BIT);
        if (!(rk != 0.0f)) return;
        const float t = fdiv(dk, rk);
        float hit[3], loc[3];
        CNT(QR_STAT_TEST_PLANE);
        if (!clip_root(S, r, si, t, w, p, ldff, lray, 0, 0, 0u, hit, loc, st)) return;
        accept_root(S, w, si, p, rk < 0.0f ? SIDE_OUTER : SIDE_INNER, t, hit, loc);
    }
    else if (solver == 2)
    {
        /* quadric coefficients (5722-5783) */
        const float4 ci = ldf4(s->sci), cj = ldf4(s->scj);
        const float sciv[3] = {ci.x, ci.y, ci.z}, scjv[3] = {cj.x, cj.y, cj.z};
        float a = 0.0f, b = 0.0f, c = 0.0f;
        #pragma unroll
        for (int k = 0; k < 3; k++)
        {
            const float sci = sciv[k], scj = scjv[k];
            const float sri = sci * lray[k];
            float sdi = sci * ldff[k];
            sdi = sdi - scj;
            const float ax = lray[k] * sri;
            const float bx = lray[k] * sdi;
            sdi = sdi - scj;
            const float cx = ldff[k] * sdi;
            if (k == 0) { a = ax; b = bx; c = cx; }
            else { a = a + ax; b = b + bx; c = c + cx; }
        }
        c = c - ci.w;
        const float d = b * b - c * a;
        CNT(QR_STAT_TEST_QUADRIC);
        root_pair(S, r, w, si, p, ldff, lray, a, b, c, d, st);
    }
    else
    {
        /* two-plane (6349-6402) */
        const int mi = __ldg(&s->amap[0]), mk = __ldg(&s->amap[2]);
        const float ri = lray[mi], di = ldff[mi], rk = lray[mk], dk = ldff[mk];
        const float si_ = __ldg(&s->sci[mi]), sk = __ldg(&s->sci[mk]);
        float dd = di * rk - dk * ri;
        dd = dd * dd;
        dd = dd * si_;
        dd = dd * sk;
        dd = fabsf(dd);
        const float bb = si_ * di * ri + sk * dk * rk;
        const float cc = di * di * si_ + dk * dk * sk;
        const float aa = ri * ri * si_ + rk * rk * sk;
        CNT(QR_STAT_TEST_TWOPLANE);
        root_pair(S, r, w, si, p, ldff, lray, aa, bb, cc, dd, st);
    }
}

/* the surface's local ray outside a transform node's group: through the
 * surface's own transform or a translation (2518-2645) */
__device__ __forceinline__ void local_ray(const qr_dscene &S, const Ray &r, int si,
                                          float ldff[3], float lray[3], StP st)
{
    const qr_srf *__restrict__ s = &S.srf[si];
    const int am3 = __ldg(&s->amap[3]);
    if (r.from == si)
    {
        #pragma unroll
        for (int k = 0; k < 3; k++) ldff[k] = r.phit[k];
        if (am3 != 0) xform(s, r.dir, lray);
        else
        {
            #pragma unroll
            for (int k = 0; k < 3; k++) lray[k] = r.dir[k];
        }
        return;
    }
    float d[3];
    const float4 ps = ldf4(s->pos);
    d[0] = r.org[0] - ps.x;
    d[1] = r.org[1] - ps.y;
    d[2] = r.org[2] - ps.z;
    if (am3 != 0) { CNT(QR_STAT_XFORM); xform(s, d, ldff); xform(s, r.dir, lray); }
    else
    {
        #pragma unroll
        for (int k = 0; k < 3; k++) { ldff[k] = d[k]; lray[k] = r.dir[k]; }
    }
}

/* ray / box slab test against the node's box, for t in (t_min, tmax]; the
 * slab distances are (lo - org) / dir formed as lo * inv - org * inv with a
 * fused multiply-add (oinv = org * inv per ray).  The test only prunes
 * nodes and every box carries a margin far above this rounding, so which
 * surfaces are tested, and the frame, do not depend on it. */
__device__ __forceinline__ int box_hit4(const float4 l4, const float4 h4, const Ray &r,
                                        const float inv[3], const float oinv[3], float tmax,
                                        float &tn, StP st)
{
    CNT(QR_STAT_BOX_TEST);
    float t0 = -FLT_MAX, t1 = FLT_MAX;
    const float los[3] = {l4.x, l4.y, l4.z}, his[3] = {h4.x, h4.y, h4.z};
    #pragma unroll
    for (int k = 0; k < 3; k++)
    {
        const float lo = los[k], hi = his[k];
        if (r.dir[k] == 0.0f)
        {
            if (r.org[k] < lo || r.org[k] > hi) return 0;
            continue;
        }
        const float a = __fmaf_rn(lo, inv[k], -oinv[k]);
        const float b = __fmaf_rn(hi, inv[k], -oinv[k]);
        t0 = fmaxf(t0, fminf(a, b));
        t1 = fminf(t1, fmaxf(a, b));
    }
    tn = t0;
    return t0 <= t1 && t1 >= r.t_min && t0 <= tmax;
}

__device__ __forceinline__ int box_hit(const qr_bnode *__restrict__ n, const Ray &r,
                                       const float inv[3], const float oinv[3], float tmax,
                                       float &tn, StP st)
{
    return box_hit4(ldf4(n->lo), ldf4(n->hi), r, inv, oinv, tmax, tn, st);
}

/*
 * One surface list, nearest hit or any occluder.  The surfaces come either
 * from the list in order (2413-2680, with the per-node transform cache) or,
 * for the scene's full camera / shadow list and a ray that starts near the
 * scene (where the boxes allow for the solvers' rounding), from the
 * bounding-volume hierarchy: unbounded surfaces first, then the tree, near
 * child first, skipping boxes that start beyond the nearest hit so far.
 * Hits are accepted by (distance, list position), so both give the in-order
 * walk's result.  There is one solver site for both sources.
 */
template <int QUADS>
static __device__ void walk_t(const qr_dscene &S, const qr_frame_params &P, const Ray &r,
                              int off, int num, Walk &w, StP st)
{
    const float dx = r.org[0] - S.ray_c[0], dy = r.org[1] - S.ray_c[1],
                dz = r.org[2] - S.ray_c[2];
    const int full = (off == S.cam_off && num == S.cam_num) ||
                     (off == S.shd_off && num == S.shd_num);
    /* the smallest hierarchy level that covers the ray's origin */
    const float d2 = dx * dx + dy * dy + dz * dz;
    int lvl = -1;
    #pragma unroll
    for (int l = QR_BVH_LEVELS - 1; l >= 0; l--)
        if (d2 <= S.lvl_r2[l]) lvl = l;
    const int use_bvh = S.nnodes >= 0 && !(P.flags & QR_FP_LINEAR_WALK) && lvl >= 0 && full;
    if (S.nnodes >= 0 && full && lvl < 0) CNT(QR_STAT_FAR_WALK);
    /* list source (cache_last) and hierarchy source (cxf): the transform
     * node whose transformed ray cdff / cray holds */
    int e = 0, cache_last = -1, cxf = -1;
    float cdff[3] = {0.0f, 0.0f, 0.0f}, cray[3] = {0.0f, 0.0f, 0.0f};
    /* hierarchy source */
    int ai = 0, ia = 0, ib = 0, sp = 0;
    int2 stk[QR_BVH_STACK];         /* code, entry distance (float bits) */
    int cur = QR_CODE_NONE;         /* code (qr_bpair) to take next without a pop */
    float inv[3], oinv[3];
    int aend = 0;
    if (use_bvh)
    {
        #pragma unroll
        for (int k = 0; k < 3; k++)
        {
            inv[k] = r.dir[k] != 0.0f ? fdiv(1.0f, r.dir[k]) : 0.0f;
            oinv[k] = r.org[k] * inv[k];
        }
        ai = S.lvl_aoff[lvl];
        aend = ai + S.lvl_anum[lvl];
        const int root = S.lvl_root[lvl];
        float tn;
        if (box_hit(&S.nodes[root], r, inv, oinv, w.tbuf, tn, st))
        {
            (void)tn;
            cur = QUADS ? S.lvl_quad[lvl] : qr_bnode_code(S.nodes[root], root);
        }
    }

    #pragma unroll 1
    for (;;)
    {
        int si, p, xf = -1, cached = 0;
        if (!use_bvh)
        {
            int found = 0;
            #pragma unroll 1
            while (e < num)
            {
                const int ei = off + e;
                const int4 el = ldi4(&S.elems[ei].kind);   /* kind, ref, last, rel */
                const int kind = el.x;
                const int ref = el.y;
                e++;
                if (kind == QR_ELM_TRNODE)
                {
                    const qr_srf *__restrict__ t = &S.srf[ref];
                    if (__ldg(&t->amap[3]) == 0) continue;
                    const float4 tp = ldf4(t->pos);
                    const float d[3] = {r.org[0] - tp.x, r.org[1] - tp.y, r.org[2] - tp.z};
                    CNT(QR_STAT_XFORM);
                    xform(t, d, cdff);
                    xform(t, r.dir, cray);
                    cache_last = el.z;
                    continue;
                }
                si = ref;
                p = e - 1;
                if (cache_last >= 0)
                {
                    cached = 1;
                    if (ei == cache_last) cache_last = -1;
                }
                found = 1;
                break;
            }
            if (!found) break;
        }
        else
        {
            const qr_bitem *__restrict__ it;
            if (ai < aend)
            {
                it = &S.always[ai++];
            }
            else
            {
                /* near child first: it is visited at once, the far one
                 * pushed with its entry distance and skipped on the pop
                 * if a hit nearer than that has been found meanwhile */
                /* an inner node's record holds both children's boxes and
                 * codes: one fetch a visit; a leaf is taken from its code */
                #pragma unroll 1
                while (ia >= ib)
                {
                    int code = cur;
                    if (code != QR_CODE_NONE)
                    {
                        cur = QR_CODE_NONE;
                    }
                    else
                    {
                        if (sp <= 0) break;
                        const int2 e = stk[--sp];
                        if (__int_as_float(e.y) > w.tbuf) continue;
                        code = e.x;
                    }
                    if (code < 0)
                    {
                        const int lc = ~code;
                        ia = lc >> 4;
                        ib = ia + (lc & 15);
                        continue;
                    }
                    if (QUADS)
                    {
                    /* a 4-wide record: the hit slots' codes, the nearest
                     * taken next and the others pushed farthest first (so
                     * the nearer pop first) */
                    const qr_bquad *__restrict__ qd = &S.quads[code];
                    const float4 lx = ldf4(qd->lo_x), ly = ldf4(qd->lo_y), lz = ldf4(qd->lo_z);
                    const float4 hx = ldf4(qd->hi_x), hy = ldf4(qd->hi_y), hz = ldf4(qd->hi_z);
                    const int4 cd = ldi4(qd->code);
                    const float lxs[4] = {lx.x, lx.y, lx.z, lx.w}, lys[4] = {ly.x, ly.y, ly.z, ly.w};
                    const float lzs[4] = {lz.x, lz.y, lz.z, lz.w}, hxs[4] = {hx.x, hx.y, hx.z, hx.w};
                    const float hys[4] = {hy.x, hy.y, hy.z, hy.w}, hzs[4] = {hz.x, hz.y, hz.z, hz.w};
                    const int cds[4] = {cd.x, cd.y, cd.z, cd.w};
                    float td[4];
                    int tc[4], nh = 0;
                    #pragma unroll
                    for (int k = 0; k < 4; k++)
                    {
                        float t;
                        const int h = cds[k] != QR_BQUAD_EMPTY &&
                                      box_hit4(make_float4(lxs[k], lys[k], lzs[k], 0.0f),
                                               make_float4(hxs[k], hys[k], hzs[k], 0.0f),
                                               r, inv, oinv, w.tbuf, t, st);
                        td[k] = h ? t : __int_as_float(0x7f800000);   /* misses last */
                        tc[k] = cds[k];
                        nh += h;
                    }
                    if (nh == 0) continue;
                    /* ascending distance: a sorting network of 4 */
#define QR_CSWAP(a, b)                                                            \
                    if (td[b] < td[a])                                            \
                    {                                                             \
                        const float tt = td[a]; td[a] = td[b]; td[b] = tt;        \
                        const int cc = tc[a]; tc[a] = tc[b]; tc[b] = cc;          \
                    }
                    QR_CSWAP(0, 1) QR_CSWAP(2, 3) QR_CSWAP(0, 2) QR_CSWAP(1, 3) QR_CSWAP(1, 2)
#undef QR_CSWAP
                    if (sp + nh - 1 > QR_BVH_STACK) { w.fault = QR_FAULT_STACK; return; }
                    #pragma unroll
                    for (int m = 3; m > 0; m--)
                        if (m < nh) stk[sp++] = make_int2(tc[m], __float_as_int(td[m]));
                    cur = tc[0];
                    continue;
                    }
                    const qr_bpair *__restrict__ pr = &S.pairs[code];
                    const float4 la = ldf4(pr->lo_a), ha4 = ldf4(pr->hi_a);
                    const float4 lb = ldf4(pr->lo_b), hb4 = ldf4(pr->hi_b);
                    float ta, tb;
                    const int ha = box_hit4(la, ha4, r, inv, oinv, w.tbuf, ta, st);
                    const int hb = box_hit4(lb, hb4, r, inv, oinv, w.tbuf, tb, st);
                    const int ca = __float_as_int(la.w), cb = __float_as_int(lb.w);
                    if (ha && hb)
                    {
                        if (sp >= QR_BVH_STACK) { w.fault = QR_FAULT_STACK; return; }
                        const int near_a = ta <= tb;
                        stk[sp++] = make_int2(near_a ? cb : ca, __float_as_int(near_a ? tb : ta));
                        cur = near_a ? ca : cb;
                    }
                    else if (ha) cur = ca;
                    else if (hb) cur = cb;
                }
                if (ia >= ib) break;
                it = &S.items[ia++];
            }
            const int4 iv = ldi4(&it->pos);              /* pos, srf, xf, pad */
            si = iv.y;
            p = iv.x;
            xf = iv.z;
            if (xf >= 0)
            {
                if (xf != cxf)
                {
                    const qr_srf *__restrict__ t = &S.srf[xf];
                    const float4 tp = ldf4(t->pos);
                    const float d[3] = {r.org[0] - tp.x, r.org[1] - tp.y, r.org[2] - tp.z};
                    CNT(QR_STAT_XFORM);
                    xform(t, d, cdff);
                    xform(t, r.dir, cray);
                    cxf = xf;
                }
                cached = 1;
            }
        }

        float ldff[3], lray[3];
        if (cached)
        {
            const float4 ps = ldf4(S.srf[si].pos);
            const float pp[3] = {ps.x, ps.y, ps.z};
            #pragma unroll
            for (int k = 0; k < 3; k++)
            {
                ldff[k] = r.from == si ? r.phit[k] : cdff[k] - pp[k];
                lray[k] = cray[k];
            }
        }
        else
        {
            local_ray(S, r, si, ldff, lray, st);
        }
        solve_surface(S, r, w, si, p, ldff, lray, st);
        if (w.shadow && w.occluded) return;
    }
}

/* the walk over the binary tree's child records (qr_bpair): the Whitted
 * kernels' form.  Over the 4-wide records (qr_bquad) the animated 1080p
 * frame took 22.9 against 20.1 ms and the plain frame 0.111 against
 * 0.103 ms (the Whitted kernels' registers spill around the sort; at 6 and
 * 5 resident blocks 22.9 and 21.4 ms), the 256-quadric frame 57.5 against
 * 60.4 ms; the path tracer's tracing stage,
 * with 80 registers and incoherent rays, gains from them (wf_trace) */
static __device__ __forceinline__ void walk(const qr_dscene &S, const qr_frame_params &P,
                                            const Ray &r, int off, int num, Walk &w, StP st)
{
    walk_t<0>(S, P, r, off, num, w, st);
}

/* shading state of one hit, kept while its shadow rays are traced */
struct Shade
{
    int   srf, side, props;
    float hit[3], loc[3];
    float nrm[3], tex[3];
    float c[3];             /* colour so far: ambient, then lights */
    float dir[3];           /* direction of the shaded ray */
    int   depth;            /* its remaining secondary depth */
    int   loff, lnum;       /* light list of the hit side */
};

/* side-oriented normal in world axes (PL 5669-5687, QD 6237-6283,
 * TP 6415-6457, node transform 3273-3352) and texel colour (3380-3416,
 * PAINT_COLX 970-979) of a hit */
__device__ __forceinline__ void hit_surface(const qr_dscene &S, const Hit &h,
                                            float nrm[3], float tex[3])
{
    const qr_srf *__restrict__ s = &S.srf[h.srf];
    const int side = h.side;
    const int props = __ldg(&s->props[side]);
    const qr_mat *__restrict__ m = &S.mat[__ldg(&s->mat[side])];
    const uint32_t tside = side ? SIGN_BIT : 0u;
    float tu = 0.0f, tv = 0.0f;
    const int nrmk = __ldg(&s->nrmk);

    if (nrmk == 1)
    {
        const int mk = __ldg(&s->amap[2]);
        nrm[0] = nrm[1] = nrm[2] = 0.0f;
        nrm[mk] = fxor(fxor(1.0f, tside), __ldg(&s->asgn[2]) ? SIGN_BIT : 0u);
        if (props & QR_PROP_TEXTURE)
        {
            tu = fxor(h.loc[__ldg(&s->amap[0])], __ldg(&s->asgn[0]) ? SIGN_BIT : 0u);
            tv = fxor(h.loc[__ldg(&s->amap[1])], __ldg(&s->asgn[1]) ? SIGN_BIT : 0u);
        }
    }
    else
    {
        float x = h.loc[0] * __ldg(&s->sci[0]);
        float y = h.loc[1] * __ldg(&s->sci[1]);
        float z = h.loc[2] * __ldg(&s->sci[2]);
        if (nrmk == 2)
        {
            x = x - __ldg(&s->scj[0]);
            y = y - __ldg(&s->scj[1]);
            z = z - __ldg(&s->scj[2]);
        }
        float l2 = x * x + y * y;
        l2 = l2 + z * z;
        const float inv = fxor(rsq(l2), tside);
        nrm[0] = x * inv; nrm[1] = y * inv; nrm[2] = z * inv;
    }

    if (__ldg(&s->amap[3]) != 0)
    {
        /* transposed inverse of the transform node (3273-3352) */
        const int tn = __ldg(&s->trnode);
        const qr_srf *__restrict__ t = &S.srf[tn >= 0 ? tn : h.srf];
        const float n1 = nrm[0], n2 = nrm[1], n3 = nrm[2];
        float x = __ldg(&t->tci[0]) * n1;
        float y = __ldg(&t->tcj[1]) * n2;
        float z = __ldg(&t->tck[2]) * n3;
        const int tam = __ldg(&t->amap[3]);
        int renorm = 1;
        if (tam != 1)
        {
            x = x + __ldg(&t->tcj[0]) * n2;
            x = x + __ldg(&t->tck[0]) * n3;
            y = y + __ldg(&t->tci[1]) * n1;
            y = y + __ldg(&t->tck[1]) * n3;
            z = z + __ldg(&t->tci[2]) * n1;
            z = z + __ldg(&t->tcj[2]) * n2;
            if (tam == 2) renorm = 0;
        }
        if (renorm)
        {
            float l2 = x * x + y * y;
            l2 = l2 + z * z;
            const float inv = rsq(l2);
            x = x * inv; y = y * inv; z = z * inv;
        }
        nrm[0] = x; nrm[1] = y; nrm[2] = z;
    }

    /* texel (3380-3416, PAINT_COLX 970-979) */
    {
        int32_t idx = 0;
        if (props & QR_PROP_TEXTURE)
        {
            const float uv[2] = {tu, tv};
            float tx = uv[__ldg(&m->tmap[0])], ty = uv[__ldg(&m->tmap[1])];
            tx = tx - __ldg(&m->xoffs);
            ty = ty - __ldg(&m->yoffs);
            tx = tx * __ldg(&m->xscal);
            ty = ty * __ldg(&m->yscal);
            idx = (__float2int_rd(tx) & __ldg(&m->xmask)) +
                  ((__float2int_rd(ty) & __ldg(&m->ymask)) << __ldg(&m->yshft));
        }
        const uint32_t texel = __ldg(&S.texels[__ldg(&m->tex_off) + idx]);
        tex[0] = fdiv((float)(int32_t)((texel >> 16) & 0xFF), 255.0f);
        tex[1] = fdiv((float)(int32_t)((texel >> 8) & 0xFF), 255.0f);
        tex[2] = fdiv((float)(int32_t)(texel & 0xFF), 255.0f);
        if (props & QR_PROP_GAMMA)
        {
            #pragma unroll
            for (int k = 0; k < 3; k++) tex[k] = tex[k] * tex[k];
        }
    }

}

/* normal, texel and ambient of a hit (3255-3416, 3945-3987) */
static __device__ void shade_begin(const qr_dscene &S, const qr_frame_params &P, const Ray &r,
                            const Hit &h, Shade &sh)
{
    const qr_srf *__restrict__ s = &S.srf[h.srf];
    const int side = h.side;
    const int props = __ldg(&s->props[side]);
    const qr_mat *__restrict__ m = &S.mat[__ldg(&s->mat[side])];
    float nrm[3], tex[3];

    sh.srf = h.srf;
    sh.side = side;
    sh.props = props;
    #pragma unroll
    for (int k = 0; k < 3; k++)
    {
        sh.hit[k] = h.hit[k];
        sh.loc[k] = h.loc[k];
        sh.dir[k] = r.dir[k];
    }
    sh.depth = r.depth;

    hit_surface(S, h, nrm, tex);

    #pragma unroll
    for (int k = 0; k < 3; k++)
    {
        sh.nrm[k] = nrm[k];
        sh.tex[k] = tex[k];
        sh.c[k] = tex[k];
    }
    sh.loff = 0;
    sh.lnum = 0;
    if (!(props & QR_PROP_LIGHT))
    {
        /* ambient (3945-3987) */
        const float m_trn = __ldg(&m->c_trn), m_rfl = __ldg(&m->c_rfl);
        #pragma unroll
        for (int k = 0; k < 3; k++) sh.c[k] = sh.c[k] * P.amb[k];
        float f = 1.0f - m_trn;
        f = f - m_rfl;
        f = (0.0f <= f) ? f : 0.0f;
        #pragma unroll
        for (int k = 0; k < 3; k++) sh.c[k] = sh.c[k] * f;
        sh.loff = __ldg(&s->lgt_off[side]);
        sh.lnum = __ldg(&s->lgt_num[side]);
    }
}

/* light vector and its dot with the normal (4008-4050) */
__device__ __forceinline__ float light_dot(const qr_dscene &S, const Shade &sh, int li,
                                           float lv[3])
{
    const qr_lelem *__restrict__ le = &S.lelems[sh.loff + li];
    const qr_light *__restrict__ L = &S.lgt[__ldg(&le->light)];
    #pragma unroll
    for (int k = 0; k < 3; k++) lv[k] = __ldg(&L->pos[k]) - sh.hit[k];
    float dot = lv[0] * sh.nrm[0] + lv[1] * sh.nrm[1];
    dot = dot + lv[2] * sh.nrm[2];
    return dot;
}

/* the next light at or after li that faces the surface (lnum if none) */
__device__ __forceinline__ int next_light(const qr_dscene &S, const Shade &sh, int li)
{
    #pragma unroll 1
    for (; li < sh.lnum; li++)
    {
        float lv[3];
        if (0.0f < light_dot(S, sh, li, lv)) break;
    }
    return li;
}

/* shadow ray of light li: origin at the hit, direction L, t in (0, 1) */
__device__ __forceinline__ void shadow_ray(const qr_dscene &S, const Shade &sh, int li,
                                           Ray &sr, int &off, int &num)
{
    const qr_lelem *__restrict__ le = &S.lelems[sh.loff + li];
    const qr_light *__restrict__ L = &S.lgt[__ldg(&le->light)];
    #pragma unroll
    for (int k = 0; k < 3; k++)
    {
        sr.org[k] = sh.hit[k];
        sr.dir[k] = __ldg(&L->pos[k]) - sh.hit[k];
        sr.phit[k] = sh.loc[k];
    }
    sr.t_min = 0.0f;
    sr.t_max = __ldg(&L->t_max);
    sr.from = sh.srf;
    sr.flags = sh.side | FLAG_SHAD;
    sr.depth = sh.depth - 1;
    off = __ldg(&le->shd_off);
    num = __ldg(&le->shd_num);
}

/* diffuse, attenuation and specular of an unshadowed light (4100-4391) */
static __device__ void light_add(const qr_dscene &S, Shade &sh, int li)
{
    const qr_srf *__restrict__ s = &S.srf[sh.srf];
    const qr_mat *__restrict__ m = &S.mat[__ldg(&s->mat[sh.side])];
    const int props = sh.props;
    const qr_lelem *__restrict__ le = &S.lelems[sh.loff + li];
    const qr_light *__restrict__ L = &S.lgt[__ldg(&le->light)];
    float lv[3];
    const float dot = light_dot(S, sh, li, lv);
    const float l_dff = __ldg(&m->l_dff), l_spc = __ldg(&m->l_spc);
    const uint32_t l_pow = (uint32_t)__ldg(&m->l_pow);

    float r2 = lv[0] * lv[0] + lv[1] * lv[1];
    r2 = r2 + lv[2] * lv[2];

    float diff, sdot = dot;
    if (props & QR_PROP_DIFFUSE)
    {
        const float inv_r = rsq(r2);
        float r1 = inv_r * r2;
        float att = r2 * __ldg(&L->a_qdr);
        r1 = r1 * __ldg(&L->a_lnr);
        att = att + __ldg(&L->a_cnt);
        att = att + r1;
        const float inv_a = rsq(att);
        diff = dot * inv_a;
        diff = diff * inv_r;
        diff = diff * l_dff;
    }
    else
    {
        diff = 0.0f;
    }

    int spec_on = 0;
    float spec = 0.0f;
    if (props & QR_PROP_SPECULAR)
    {
        float pn, rx, ry, rz;
        pn = sdot * sh.nrm[0]; rx = lv[0] - pn; rx = rx - pn;
        pn = sdot * sh.nrm[1]; ry = lv[1] - pn; ry = ry - pn;
        pn = sdot * sh.nrm[2]; rz = lv[2] - pn; rz = rz - pn;
        rx = rx * sh.dir[0];
        ry = ry * sh.dir[1];
        rz = rz * sh.dir[2];
        float ray2 = sh.dir[2] * sh.dir[2];
        ray2 = ray2 + sh.dir[0] * sh.dir[0];
        ray2 = ray2 + sh.dir[1] * sh.dir[1];
        float sv = rx + ry;
        sv = sv + rz;
        if (0.0f < sv)
        {
            /* power in 28.4 fixed point (4225-4285) */
            sv = sv * rsq(ray2);
            sv = sv * rsq(r2);
            float p1 = 1.0f, p2 = sv;
            uint32_t fr = l_pow & 0xF, in = l_pow >> 4;
            if (fr != 0)
            {
                float s4 = sv;
                do
                {
                    s4 = fsqrt(s4);
                    if (fr & 0x8) p1 = p1 * s4;
                    fr = (fr << 1) & 0xF;
                } while (fr != 0);
            }
            if (in != 0)
            {
                const float p3 = p1;
                p1 = 1.0f;
                do
                {
                    if (in & 1) p1 = p1 * p2;
                    p2 = p2 * p2;
                    in >>= 1;
                } while (in != 0);
                p1 = p1 * p3;
            }
            spec = p1 * l_spc;
            spec_on = 1;
        }
    }

    float lc[3];
    if (spec_on && !(props & QR_PROP_METAL))
    {
        /* plain: highlight in the light's colour (4323-4355) */
        #pragma unroll
        for (int k = 0; k < 3; k++)
        {
            const float lk = __ldg(&L->col[k]);
            float t1 = sh.tex[k] * diff;
            t1 = t1 * lk;
            lc[k] = t1 + lk * spec;
        }
    }
    else
    {
        /* metal: highlight tinted by the surface (4287-4317) */
        if (spec_on) diff = diff + spec;
        #pragma unroll
        for (int k = 0; k < 3; k++)
        {
            lc[k] = sh.tex[k] * __ldg(&L->col[k]);
            lc[k] = lc[k] * diff;
        }
    }
    #pragma unroll
    for (int k = 0; k < 3; k++) sh.c[k] = lc[k] + sh.c[k];
}

/* what a shaded hit asks of its children: a refracted ray (weight c_trn)
 * and a reflected ray (weight c_rfl), traced in that order (4820-4883,
 * 5235-5298) */
struct Sec
{
    int   trn, rfl;             /* child wanted (before the depth check) */
    int   split;                /* Fresnel weights were computed (no TIR) */
    float c_trn, c_rfl;
    float nw[3], rw[3];         /* refracted / reflected directions */
};

/* transparency (4442-4936) and reflection (4942-5359): weights and
 * directions of the children */
static __device__ void shade_end(const qr_dscene &S, const Shade &sh, Sec &o, StP st)
{
    const qr_srf *__restrict__ s = &S.srf[sh.srf];
    const qr_mat *__restrict__ m = &S.mat[__ldg(&s->mat[sh.side])];
    const int props = sh.props;
    const float *nrm = sh.nrm;
    const float *dir = sh.dir;
    const float m_trn = __ldg(&m->c_trn), m_rfl = __ldg(&m->c_rfl);

    float c_trn = m_trn, c_rfl = m_rfl;
    o.trn = 0;
    o.split = 0;
    if (!(props & QR_PROP_OPAQUE))
    {
        const int fres = (props & QR_PROP_FRESNEL) != 0;
        const int refr = (props & QR_PROP_REFRACT) != 0;
        const float c_rfr = __ldg(&m->c_rfr), rfr_2 = __ldg(&m->rfr_2);
        float nw[3];
        int do_trn = 0, m_ok = 1;
        if (refr || fres)
        {
            CNT(QR_STAT_REFRACT);
            float l2 = dir[0] * dir[0];
            l2 = l2 + dir[1] * dir[1];
            l2 = l2 + dir[2] * dir[2];
            const float inv = rsq(l2);
            float dn[3];
            #pragma unroll
            for (int k = 0; k < 3; k++) dn[k] = dir[k] * inv;
            float cosi = dn[0] * nrm[0];
            cosi = cosi + dn[1] * nrm[1];
            cosi = cosi + dn[2] * nrm[2];
            float nci = cosi * c_rfr;
            float kk = nci * nci;
            kk = kk + 1.0f;
            kk = kk - rfr_2;
            if (fres) m_ok = 0.0f <= kk;
            if (fres && !m_ok)
            {
                c_trn = 0.0f;
                c_rfl = m_rfl + m_trn;
            }
            else
            {
                const float sq = fsqrt(kk);
                nci = nci + sq;
                if (refr)
                {
                    #pragma unroll
                    for (int k = 0; k < 3; k++)
                    {
                        const float a1 = nrm[k] * nci;
                        const float a2 = dn[k] * c_rfr;
                        nw[k] = a2 - a1;
                    }
                }
                else
                {
                    #pragma unroll
                    for (int k = 0; k < 3; k++) nw[k] = dir[k];
                }
                if (fres)
                {
                    float x1 = cosi, x2, x3;
                    x2 = x1 * c_rfr;
                    x2 = x2 - sq;
                    const float sqn = sq * c_rfr;
                    x3 = x1;
                    x1 = x1 + sqn;
                    x3 = x3 - sqn;
                    float f0 = fdiv(nci, x2);
                    float f1 = fdiv(x1, x3);
                    f0 = f0 * f0;
                    f1 = f1 * f1;
                    float fr = f0 + f1;
                    fr = fabsf(fr * -0.5f);
                    fr = fr * m_trn;
                    c_trn = m_trn - fr;
                    c_rfl = m_rfl + fr;
                    o.split = 1;
                }
                do_trn = 1;
            }
        }
        else
        {
            #pragma unroll
            for (int k = 0; k < 3; k++) nw[k] = dir[k];
            do_trn = 1;
        }
        o.trn = do_trn && m_ok;
        #pragma unroll
        for (int k = 0; k < 3; k++) o.nw[k] = nw[k];
    }

    /* reflection (4942-5359) */
    {
        const int refl = (props & QR_PROP_REFLECT) != 0;
        const int do_rfl = refl || (!(props & QR_PROP_OPAQUE) && (props & QR_PROP_FRESNEL));
        o.rfl = do_rfl;
        if (do_rfl)
        {
            CNT(QR_STAT_REFLECT);
            float l2 = dir[0] * dir[0];
            l2 = l2 + dir[1] * dir[1];
            l2 = l2 + dir[2] * dir[2];
            const float inv = rsq(l2);
            float dn[3];
            #pragma unroll
            for (int k = 0; k < 3; k++) dn[k] = dir[k] * inv;
            float cosi = dn[0] * nrm[0];
            cosi = cosi + dn[1] * nrm[1];
            cosi = cosi + dn[2] * nrm[2];
            #pragma unroll
            for (int k = 0; k < 3; k++)
            {
                const float p = nrm[k] * cosi;
                float rw = dn[k] - p;
                o.rw[k] = rw - p;
            }
            if ((props & QR_PROP_FRESNEL) && (props & QR_PROP_OPAQUE))
            {
                float fr;
                if (props & QR_PROP_METAL)
                {
                    /* fast complex-IOR Fresnel (5067-5089) */
                    float r6 = __ldg(&m->c_rcp);
                    float x4 = cosi * r6;
                    x4 = x4 + x4;
                    float x0 = cosi * cosi;
                    r6 = r6 * r6;
                    r6 = r6 + __ldg(&m->ext_2);
                    float x1 = x0 * r6;
                    x0 = x0 + r6;
                    x1 = x1 + 1.0f;
                    float x2 = x0, x3 = x1;
                    x0 = x0 + x4;
                    x1 = x1 + x4;
                    x2 = x2 - x4;
                    x3 = x3 - x4;
                    x0 = fdiv(x0, x2);
                    x1 = fdiv(x1, x3);
                    x0 = x0 + x1;
                    fr = fabsf(x0 * -0.5f);
                }
                else
                {
                    /* dielectric Fresnel for opaque surfaces (5108-5134) */
                    const float n = __ldg(&m->c_rfr);
                    float x0 = cosi * n;
                    float x7 = x0 * x0;
                    x7 = x7 + 1.0f;
                    x7 = x7 - __ldg(&m->rfr_2);
                    x7 = fsqrt(x7);
                    x0 = x0 + x7;
                    float x1 = cosi;
                    float x2 = x1 * n;
                    x2 = x2 - x7;
                    x7 = x7 * n;
                    float x3 = x1;
                    x1 = x1 + x7;
                    x3 = x3 - x7;
                    x0 = fdiv(x0, x2);
                    float f1 = fdiv(x1, x3);
                    x0 = x0 * x0;
                    f1 = f1 * f1;
                    x0 = x0 + f1;
                    fr = fabsf(x0 * -0.5f);
                }
                fr = fr - 1.0f;
                fr = fr * m_rfl;
                c_rfl = m_rfl + fr;
            }
        }
    }
    o.c_trn = c_trn;
    o.c_rfl = c_rfl;
}

/* a shaded hit waiting for the colour of its refracted child (stage 0) or
 * reflected child (stage 1) */
struct Pend
{
    float c[3];
    float c_trn, c_rfl;
    float hit[3], loc[3], rw[3];
    int   srf, side, depth, stage, rfl;
};

__device__ __forceinline__ void child_ray(Ray &cr, const float hit[3], const float dir[3],
                                          const float loc[3], int srf, int flags,
                                          int depth)
{
    #pragma unroll
    for (int k = 0; k < 3; k++)
    {
        cr.org[k] = hit[k];
        cr.dir[k] = dir[k];
        cr.phit[k] = loc[k];
    }
    cr.t_min = 0.0f;
    cr.t_max = FLT_MAX;
    cr.from = srf;
    cr.flags = flags;
    cr.depth = depth;
}

/* record a pixel that ran past a loop bound in the context's fault word */
static __device__ __noinline__ void note_fault(const qr_dscene &S, int bit, int x, int y)
{
    if (S.fault == NULL) return;
    if (atomicOr(&S.fault[0], (uint32_t)bit) == 0u)
    {
        S.fault[1] = (uint32_t)x;
        S.fault[2] = (uint32_t)y;
    }
    atomicAdd(&S.fault[3], 1u);
}

/*
 * The Whitted ray tree of one camera ray as one loop with a single list walk.
 * Each turn of the loop traces one segment: a camera or secondary ray
 * (nearest hit), or one shadow ray of the hit being shaded (any occluder).
 * The reference recurses through its context stack (tracer.cpp:4820-4860,
 * 5235-5275) and loops over lights inside the shading (4008-4096); here a
 * shaded hit that spawns a child is parked on a small per-thread stack and
 * combined when the child's colour is known, in the reference's order:
 * colour = rc * c_rfl + (tc * c_trn + local).
 * The tree holds at most 2^(depth+1) - 1 rays, each with one shadow ray a
 * light; a pixel that traces more segments (or whose walk gives up) is
 * recorded in the fault word and rendered black.
 */
static __device__ void trace_tree(const qr_dscene &S, const qr_frame_params &P, Ray r,
                           int x, int y, float col[3], StP st)
{
    Pend stk[QR_MAX_DEPTH];
    int sp = 0, off = S.cam_off, num = S.cam_num;
    float ret[3];
    Shade sh;
    int shadow = 0, li = 0;
    const int seg_lim = ((2 << P.depth) - 1) * (1 + S.nlgt);
    int seg = 0;
    #pragma unroll 1
    for (;;)
    {
        if (++seg > seg_lim)
        {
            note_fault(S, QR_FAULT_TREE, x, y);
            col[0] = col[1] = col[2] = 0.0f;
            return;
        }
        Walk w;
        w.fault = 0;
        w.shadow = shadow;
        w.occluded = 0;
        w.tbuf = r.t_max;
        w.bestp = -1;
        w.best.srf = -1;
        walk(S, P, r, off, num, w, st);
        if (w.fault)
        {
            note_fault(S, w.fault, x, y);
            col[0] = col[1] = col[2] = 0.0f;
            return;
        }

        int finish = 0;         /* the shading of sh is complete */
        if (shadow)
        {
            if (!w.occluded)
            {
                CNT(QR_STAT_LIGHT);
                light_add(S, sh, li);
            }
            li = next_light(S, sh, li + 1);
            if (li < sh.lnum)
            {
                CNT(QR_STAT_RAY_SHADOW);
                shadow_ray(S, sh, li, r, off, num);
                continue;
            }
            shadow = 0;
            finish = 1;
        }
        else if (w.best.srf < 0)
        {
            ret[0] = ret[1] = ret[2] = 0.0f;
        }
        else
        {
            CNT(QR_STAT_SHADE);
            shade_begin(S, P, r, w.best, sh);
            li = next_light(S, sh, 0);
            if (li < sh.lnum)
            {
                CNT(QR_STAT_RAY_SHADOW);
                shadow = 1;
                shadow_ray(S, sh, li, r, off, num);
                continue;
            }
            finish = 1;
        }

        if (finish)
        {
            Sec o;
            shade_end(S, sh, o, st);
            const qr_srf *__restrict__ s = &S.srf[sh.srf];
            const int side = sh.side;
            float c[3] = {sh.c[0], sh.c[1], sh.c[2]};
            int spawned = 0;
            if (o.trn)
            {
                if (sh.depth != 0)
                {
                    Pend &p = stk[sp++];
                    #pragma unroll
                    for (int k = 0; k < 3; k++)
                    {
                        p.c[k] = c[k];
                        p.hit[k] = sh.hit[k];
                        p.loc[k] = sh.loc[k];
                        p.rw[k] = o.rw[k];
                    }
                    p.c_trn = o.c_trn;
                    p.c_rfl = o.c_rfl;
                    p.srf = sh.srf;
                    p.side = side;
                    p.depth = sh.depth;
                    p.stage = 0;
                    p.rfl = o.rfl;
                    CNT(QR_STAT_RAY_SECONDARY);
                    child_ray(r, sh.hit, o.nw, sh.loc, sh.srf, side | FLAG_PASS,
                              sh.depth - 1);
                    off = __ldg(&s->sec_off[1 - side]);
                    num = __ldg(&s->sec_num[1 - side]);
                    spawned = 1;
                }
                else
                {
                    #pragma unroll
                    for (int k = 0; k < 3; k++) c[k] = 0.0f + c[k];
                }
            }
            if (!spawned && o.rfl)
            {
                if (sh.depth != 0)
                {
                    Pend &p = stk[sp++];
                    #pragma unroll
                    for (int k = 0; k < 3; k++) p.c[k] = c[k];
                    p.c_rfl = o.c_rfl;
                    p.stage = 1;
                    CNT(QR_STAT_RAY_SECONDARY);
                    child_ray(r, sh.hit, o.rw, sh.loc, sh.srf, side, sh.depth - 1);
                    off = __ldg(&s->sec_off[side]);
                    num = __ldg(&s->sec_num[side]);
                    spawned = 1;
                }
                else
                {
                    #pragma unroll
                    for (int k = 0; k < 3; k++) c[k] = 0.0f + c[k];
                }
            }
            if (spawned) continue;
            #pragma unroll
            for (int k = 0; k < 3; k++) ret[k] = c[k];
        }

        /* fold finished children into their parents */
        int more = 0;
        #pragma unroll 1
        while (sp > 0)
        {
            Pend &p = stk[sp - 1];
            if (p.stage == 0)
            {
                #pragma unroll
                for (int k = 0; k < 3; k++)
                {
                    const float tc = ret[k] * p.c_trn;
                    p.c[k] = tc + p.c[k];
                }
                if (p.rfl)
                {
                    const qr_srf *__restrict__ s = &S.srf[p.srf];
                    p.stage = 1;
                    CNT(QR_STAT_RAY_SECONDARY);
                    child_ray(r, p.hit, p.rw, p.loc, p.srf, p.side, p.depth - 1);
                    off = __ldg(&s->sec_off[p.side]);
                    num = __ldg(&s->sec_num[p.side]);
                    more = 1;
                    break;
                }
            }
            else
            {
                #pragma unroll
                for (int k = 0; k < 3; k++)
                {
                    const float rc = ret[k] * p.c_rfl;
                    p.c[k] = rc + p.c[k];
                }
            }
            #pragma unroll
            for (int k = 0; k < 3; k++) ret[k] = p.c[k];
            sp--;
        }
        if (!more) break;
    }
    #pragma unroll
    for (int k = 0; k < 3; k++) col[k] = ret[k];
}

/* sub-sample offsets of the 4x rotated grid (engine.cpp:3572-3606) */
static __constant__ float c_aa4_h[4] = {-0.08f - 0.25f, -0.08f + 0.25f,
                                 +0.08f - 0.25f, +0.08f + 0.25f};
static __constant__ float c_aa4_v[4] = {+0.08f - 0.25f, -0.08f - 0.25f,
                                 +0.08f + 0.25f, -0.08f + 0.25f};
/* 2x alternating (engine.cpp:3536-3570): the pair of offsets depends on the
 * parity of the pixel's column */
static __constant__ float c_aa2_h[2][2] = {{-0.08f + 0.25f, +0.08f - 0.25f},
                                    {+0.08f - 0.25f, -0.08f + 0.25f}};
static __constant__ float c_aa2_v[2][2] = {{+0.08f + 0.25f, -0.08f - 0.25f},
                                    {+0.08f + 0.25f, -0.08f - 0.25f}};

/* camera ray through image position (hs, vs): dir = hor * hs + ver * vs +
 * dir, from the camera position (engine.cpp:3530-3610) */
__device__ __forceinline__ void camera_ray(const qr_frame_params &P, float hs, float vs,
                                           Ray &r)
{
    #pragma unroll
    for (int k = 0; k < 3; k++)
    {
        float hx = P.hor[k] * hs;
        const float vx = P.ver[k] * vs;
        hx = hx + vx;
        r.dir[k] = hx + P.dir[k];
        r.org[k] = P.org[k];
        r.phit[k] = 0.0f;
    }
    r.t_min = P.t_min;
    r.t_max = P.t_max;
    r.from = -1;
    r.flags = 0;
    r.depth = P.depth;
}

/* the colour of the camera ray through (hs, vs) of pixel (x, y) */
__device__ __forceinline__ void primary(const qr_dscene &S, const qr_frame_params &P,
                                        int x, int y, float hs, float vs, float col[3],
                                        StP st)
{
    Ray r;
    camera_ray(P, hs, vs, r);
    CNT(QR_STAT_RAY_PRIMARY);
    trace_tree(S, P, r, x, y, col, st);
}

__device__ __forceinline__ float clamp1(float v) { return v < 1.0f ? v : 1.0f; }

/* clamp, gamma, x255, round to nearest, pack XRGB (7028-7145, 1922-1940) */
__device__ __forceinline__ uint32_t pack(const qr_frame_params &P, const float col[3])
{
    uint32_t px = 0;
    #pragma unroll
    for (int k = 0; k < 3; k++)
    {
        float v = col[k];
        if (P.ctx_props & QR_PROP_GAMMA) v = fsqrt(v);
        v = v * 255.0f;
        /* x86 cvtps2dq gives 0x80000000 for NaN / out of range */
        const int32_t iv = (v != v || v >= 2147483648.0f || v < -2147483648.0f)
                           ? (int32_t)0x80000000 : __float2int_rn(v);
        px |= ((uint32_t)iv & 0xFFu) << (16 - 8 * k);
    }
    return px;
}

/* pixels of a frame kernel's thread: each warp of a 32x4 block covers a
 * tile of QR_TILE_W x (32 / QR_TILE_W) pixels, the block's four warps 2 x 2
 * tiles, so neighbouring lanes trace neighbouring rays */
#ifndef QR_TILE_W
#define QR_TILE_W 16
#endif
#define QR_TILE_H (32 / QR_TILE_W)

__device__ __forceinline__ int tile_x()
{
    return blockIdx.x * (2 * QR_TILE_W) + (threadIdx.y & 1) * QR_TILE_W +
           threadIdx.x % QR_TILE_W;
}

__device__ __forceinline__ int tile_y()
{
    return blockIdx.y * (2 * QR_TILE_H) + (threadIdx.y >> 1) * QR_TILE_H +
           threadIdx.x / QR_TILE_W;
}

/* blocks of 32x4 threads; QR_MIN_BLOCKS resident blocks per SM bound the
 * registers per thread (65536 / (128 * QR_MIN_BLOCKS)).  Measured on the
 * 1920x1080 4x AA animated frame with a thread a pixel: 1 (152 registers)
 * 55.0 ms, unbounded (128) 48.0 ms, 5 (96) 44.8 ms, 6 (80) 44.0 ms, 8 (64)
 * 46.5 ms; with a thread a sub-sample (whitted_aa_kernel): 6 (80) 21.07 ms,
 * 7 (72) 20.67 ms, and with 256 quadrics 65.0 against 61.8 ms (the
 * 800x480 plain frame 0.105 ms both) */
#ifndef QR_MIN_BLOCKS
#define QR_MIN_BLOCKS 7
#endif
/* the path tracer's own bound: 6 (80 registers) 66.5 ms, 8 (64) 67.9 ms
 * on the 1280x720 16-spp frame with 64-byte pending-node records */
/* samples per launch from which the path tracer runs its samples inside one
 * segment loop (pt_pixel_flat) */
#define QR_PT_FLAT_SPP 32
#ifndef QR_PT_MIN_BLOCKS
#define QR_PT_MIN_BLOCKS 6
#endif

/* one pixel of a Whitted frame: the camera ray, or the 4 sub-samples of
 * 4x AA combined in the reference's tree order, then clamp and pack */
__device__ __forceinline__ void whitted_pixel(const qr_dscene &S, const qr_frame_params &P,
                                              int x, int y, uint32_t *frame, StP st)
{
    /* one camera-ray call site for all forms (1 ray, 2x alternating, 4x
     * rotated grid); the AA average keeps the reference's pairing, every
     * term halved before it is added (7047-7135) */
    const int ns = P.fsaa == 2 ? 4 : P.fsaa == 1 ? 2 : 1;
    float col[3], half[3], p01[3];
    #pragma unroll 1
    for (int s = 0; s < ns; s++)
    {
        float hs = (float)x, vs = (float)y;
        if (ns == 4) { hs = hs + c_aa4_h[s]; vs = vs + c_aa4_v[s]; }
        if (ns == 2) { hs = hs + c_aa2_h[x & 1][s]; vs = vs + c_aa2_v[x & 1][s]; }
        float c[3];
        primary(S, P, x, y, hs, vs, c, st);
        #pragma unroll
        for (int k = 0; k < 3; k++)
        {
            c[k] = clamp1(c[k]);
            if (ns == 1) { col[k] = c[k]; continue; }
            const float hv = c[k] * 0.5f;
            if (s & 1)
            {
                const float pv = half[k] + hv;
                if (ns == 2)     col[k] = pv;
                else if (s == 1) p01[k] = pv;
                else             col[k] = p01[k] * 0.5f + pv * 0.5f;
            }
            else
            {
                half[k] = hv;
            }
        }
    }
    frame[(size_t)y * P.x_row + x] = pack(P, col);
}

/* ==== path tracer (the reference's RT_FEAT_PT estimator) ====================
 *
 * Per sample: a camera ray with a tent-filter jitter of +-0.5 pixel
 * (2267-2342); at each hit the material's emission (the light colour x 100
 * of a LIGHT material, object.cpp:1346-1375) plus, for a diffuse material
 * with depth left, l_dff * tex * the colour of one cosine-weighted bounce
 * (3470-3930; power-series sin/cos, 1979-2007) under Russian roulette at
 * probability max(tex) once the depth left is at most RT_STACK_DEPTH - 5
 * (3484-3528); then the refracted and reflected children of the Whitted path,
 * where a dielectric, once the depth left is at most RT_STACK_DEPTH - 2,
 * follows only one: reflection with probability P = 0.25 + 0.5 Re (weight
 * c_rfl / P) or refraction (weight c_trn / (1 - P)) (4685-4723).  Both
 * thresholds use the reference's compile-time stack depth (10, tracer.h:51,
 * QR_MAX_DEPTH here), not the scene's depth.  No point lights, no
 * ambient.  colour = rc c_rfl + (tc c_trn + (bounce l_dff tex + emission)).
 * Random numbers are counter-based: each draw is a hash (the SplitMix64
 * finaliser, Steele, Lea, Flood 2014, chained over the key) of (seed, frame
 * index, pixel, sample, the drawing node's code in the sample's ray tree,
 * the draw's purpose), so every order of evaluation draws the same numbers.
 * Node codes: the camera ray 0; the diffuse, refracted and reflected
 * children of node c are 3c + 1, 3c + 2, 3c + 3.
 */

__device__ __forceinline__ unsigned long long mix64(unsigned long long z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

#define PT_GOLDEN   0x9E3779B97F4A7C15ull
#define PT_CODEMUL  0xD6E8FEB86659FD93ull
/* draws of a node: roulette, bounce (two), dielectric split, camera jitter
 * (two, node 0) */
#define PT_DRAW_RR      0
#define PT_DRAW_BOUNCE  1
#define PT_DRAW_SPLIT   3
#define PT_DRAW_JITTER  4

/* the key of sample n of a pixel */
__device__ __forceinline__ unsigned long long pt_sample_key(unsigned long long seed,
                                                            int frame,
                                                            unsigned long long pixel, int n)
{
    const unsigned long long kp =
        mix64(seed ^ mix64(((unsigned long long)(uint32_t)frame << 40) ^ pixel));
    return mix64(kp + (unsigned long long)(uint32_t)n * PT_GOLDEN);
}

/* the key of the node with tree code `code` in a sample */
__device__ __forceinline__ unsigned long long pt_node_key(unsigned long long ks,
                                                          uint32_t code)
{
    return mix64(ks ^ ((unsigned long long)code * PT_CODEMUL));
}

/* draw d of a node: uniform in [0, 1), 24 bits */
__device__ __forceinline__ float pt_draw(unsigned long long kn, int d)
{
    const uint32_t u = (uint32_t)(mix64(kn + (unsigned long long)(d + 1) * PT_GOLDEN) >> 40);
    return (float)(int32_t)u * (1.0f / 16777216.0f);
}

/* Taylor series of sin and cos on [-pi, pi] with fused multiply-adds, as the
 * reference's sinps / cosps (terms to x^9 and x^8) */
__device__ __forceinline__ float pt_sin(float x)
{
    const float t = x * x;
    float s = x, p = x * t;
    s = __fmaf_rn(p, (float)(-1.0 / 6.0), s);
    p = p * t;
    s = __fmaf_rn(p, (float)(1.0 / 120.0), s);
    p = p * t;
    s = __fmaf_rn(p, (float)(-1.0 / 5040.0), s);
    p = p * t;
    s = __fmaf_rn(p, (float)(1.0 / 362880.0), s);
    return s;
}

__device__ __forceinline__ float pt_cos(float x)
{
    const float t = x * x;
    float c = 1.0f, p = t;
    c = __fmaf_rn(p, -0.5f, c);
    p = p * t;
    c = __fmaf_rn(p, (float)(1.0 / 24.0), c);
    p = p * t;
    c = __fmaf_rn(p, (float)(-1.0 / 720.0), c);
    p = p * t;
    c = __fmaf_rn(p, (float)(1.0 / 40320.0), c);
    return c;
}

/* cosine-weighted direction about the unit normal w */
__device__ __forceinline__ void pt_bounce(const float w[3], float u1, float u2, float d[3])
{
    float a[3] = {0.0f, 0.0f, 0.0f}, u[3], v[3];
    if (fabsf(w[0]) > 0.1f) a[1] = 1.0f; else a[0] = 1.0f;
    u[0] = a[1] * w[2] - a[2] * w[1];
    u[1] = a[2] * w[0] - a[0] * w[2];
    u[2] = a[0] * w[1] - a[1] * w[0];
    float l = u[0] * u[0] + u[1] * u[1];
    l = l + u[2] * u[2];
    const float inv = rsq(l);
    #pragma unroll
    for (int k = 0; k < 3; k++) u[k] = u[k] * inv;
    v[0] = w[1] * u[2] - w[2] * u[1];
    v[1] = w[2] * u[0] - w[0] * u[2];
    v[2] = w[0] * u[1] - w[1] * u[0];
    const float s1 = fsqrt(u1);
    const float s0 = fsqrt(1.0f - u1);
    float ph = u2 + u2;
    ph = ph * 3.14159265358979323846f;
    ph = ph - 3.14159265358979323846f;
    const float cp = pt_cos(ph) * s1;
    const float sp = pt_sin(ph) * s1;
    #pragma unroll
    for (int k = 0; k < 3; k++)
    {
        float x = w[k] * s0;
        x = x + u[k] * cp;
        d[k] = x + v[k] * sp;
    }
}

/* tent filter on [-1, 1] from one uniform number, halved */
__device__ __forceinline__ float pt_tent(float u)
{
    const float r = u + u;
    const float d = r < 1.0f ? fsqrt(r) - 1.0f : 1.0f - fsqrt(2.0f - r);
    return d * 0.5f;
}

/* a shaded path-tracer hit with its children: 0 awaits the bounce, 1 may
 * spawn the refracted child, 2 awaits it, 3 may spawn the reflected child,
 * 4 awaits it */
/* a shaded node of a path-tracer ray tree waiting for its children, in
 * 16-byte fields that are written only when a later stage reads them:
 *   a   stage 0: tex, l_dff (the diffuse child's weight); from stage 1 on:
 *       the node's colour so far
 *   b   emission (stage 0 only), c_trn
 *   h   hit point, c_rfl            (a refracted or reflected child to come)
 *   l   local hit point, bits       (always: stage, flags, side, depth,
 *                                    the node's tree code from bit 12)
 *   n   refracted direction, record (a refracted child to come)
 *   m   reflected direction, record (a reflected child to come) */
struct PtPend
{
    float4 a, b, h, l, n, m;
};

#define PT_TRN   8
#define PT_RFL   16
#define PT_SIDE  32

__device__ __forceinline__ int pt_bits(const PtPend &p) { return __float_as_int(p.l.w); }
__device__ __forceinline__ uint32_t pt_code(const PtPend &p)
{
    return (uint32_t)pt_bits(p) >> 12;
}
__device__ __forceinline__ void pt_set_stage(PtPend &p, int stage)
{
    p.l.w = __int_as_float((pt_bits(p) & ~7) | stage);
}

/* shade a hit: normal, texel, the random draws (roulette, bounce, split)
 * and the children's weights; returns whether the bounce is taken (its
 * direction in ddir) */
static __device__ int pt_begin(const qr_dscene &S, const qr_frame_params &P, const Ray &r,
                        const Hit &h, PtPend &p, unsigned long long ks, uint32_t code,
                        float ddir[3], StP st)
{
    const unsigned long long kn = pt_node_key(ks, code);
    const qr_srf *__restrict__ s = &S.srf[h.srf];
    const int side = h.side;
    const int props = __ldg(&s->props[side]);
    const qr_mat *__restrict__ m = &S.mat[__ldg(&s->mat[side])];
    float nrm[3], tex[3];
    hit_surface(S, h, nrm, tex);

    int dif = (props & QR_PROP_DIFFUSE) && r.depth != 0;
    if (dif && r.depth <= QR_MAX_DEPTH - 5)
    {
        float pr = tex[0] > tex[1] ? tex[0] : tex[1];
        pr = pr > tex[2] ? pr : tex[2];
        const float u = pt_draw(kn, PT_DRAW_RR);
        if (!(u < pr)) dif = 0;
        else
        {
            const float rc = fdiv(1.0f, pr);
            #pragma unroll
            for (int k = 0; k < 3; k++) tex[k] = tex[k] * rc;
        }
    }
    if (dif)
    {
        const float u1 = pt_draw(kn, PT_DRAW_BOUNCE);
        const float u2 = pt_draw(kn, PT_DRAW_BOUNCE + 1);
        pt_bounce(nrm, u1, u2, ddir);
    }

    Shade sh;
    sh.srf = h.srf;
    sh.side = side;
    sh.props = props;
    #pragma unroll
    for (int k = 0; k < 3; k++) { sh.nrm[k] = nrm[k]; sh.dir[k] = r.dir[k]; }
    Sec o;
    shade_end(S, sh, o, st);
    if (o.split && o.trn && o.rfl && r.depth != 0 && r.depth <= QR_MAX_DEPTH - 2)
    {
        const float u = pt_draw(kn, PT_DRAW_SPLIT);
        const float re = fdiv(o.c_rfl, o.c_trn + o.c_rfl);
        float pr = re * 0.5f;
        pr = pr + 0.25f;
        if (u < pr)
        {
            o.trn = 0;
            o.c_rfl = fdiv(o.c_rfl, pr);
        }
        else
        {
            o.rfl = 0;
            o.c_trn = fdiv(o.c_trn, 1.0f - pr);
        }
    }

    /* stage 0 waits for the diffuse child; without one the node starts
     * with its emission and stage 1 folds nothing */
    const float4 emit = make_float4(__ldg(&m->emit[0]), __ldg(&m->emit[1]),
                                    __ldg(&m->emit[2]), o.c_trn);
    if (dif)
        p.a = make_float4(tex[0], tex[1], tex[2], __ldg(&m->l_dff));
    else
        p.a = make_float4(0.0f + emit.x, 0.0f + emit.y, 0.0f + emit.z, 0.0f);
    if (dif || o.trn) p.b = emit;
    const int spawn = (o.trn || o.rfl) && r.depth != 0;
    if (spawn || o.rfl) p.h = make_float4(h.hit[0], h.hit[1], h.hit[2], o.c_rfl);
    p.l = make_float4(h.loc[0], h.loc[1], h.loc[2],
                      __int_as_float((dif ? 0 : 1) | (o.trn ? PT_TRN : 0) |
                                     (o.rfl ? PT_RFL : 0) | (side ? PT_SIDE : 0) |
                                     (r.depth << 8) | (int)(code << 12)));
    if (spawn && o.trn) p.n = make_float4(o.nw[0], o.nw[1], o.nw[2], __int_as_float(h.srf));
    if (spawn && o.rfl) p.m = make_float4(o.rw[0], o.rw[1], o.rw[2], __int_as_float(h.srf));
    return dif;
}

/* fold the finished child's colour ret into p and spawn its next child
 * into (r, off, num); returns 1 when a child was spawned, else 0 with the
 * node's colour in ret */
static __device__ int pt_advance(const qr_dscene &S, PtPend &p, float ret[3], Ray &r,
                          int &off, int &num, uint32_t &rcode, StP st)
{
    const int bits = pt_bits(p);
    int stage = bits & 7;
    const int side = (bits & PT_SIDE) ? 1 : 0, depth = (bits >> 8) & 15;
    float4 c = p.a;
    if (stage == 0)
    {
        const float4 e = p.b;
        float t;
        t = ret[0] * c.w; c.x = t * c.x; c.x = c.x + e.x;
        t = ret[1] * c.w; c.y = t * c.y; c.y = c.y + e.y;
        t = ret[2] * c.w; c.z = t * c.z; c.z = c.z + e.z;
        stage = 1;
    }
    if (stage == 1)
    {
        if (bits & PT_TRN)
        {
            if (depth != 0)
            {
                const float4 hh = p.h, n = p.n;
                const int srf = __float_as_int(n.w);
                const qr_srf *__restrict__ s = &S.srf[srf];
                const float hit[3] = {hh.x, hh.y, hh.z}, dir[3] = {n.x, n.y, n.z};
                const float4 l = p.l;
                const float loc[3] = {l.x, l.y, l.z};
                CNT(QR_STAT_RAY_SECONDARY);
                child_ray(r, hit, dir, loc, srf, side | FLAG_PASS, depth - 1);
                off = __ldg(&s->sec_off[1 - side]);
                num = __ldg(&s->sec_num[1 - side]);
                rcode = 3u * pt_code(p) + 2u;
                c.w = 0.0f;
                p.a = c;
                pt_set_stage(p, 2);
                return 1;
            }
            c.x = 0.0f + c.x; c.y = 0.0f + c.y; c.z = 0.0f + c.z;
        }
        stage = 3;
    }
    else if (stage == 2)
    {
        const float ct = p.b.w;
        float t;
        t = ret[0] * ct; c.x = t + c.x;
        t = ret[1] * ct; c.y = t + c.y;
        t = ret[2] * ct; c.z = t + c.z;
        stage = 3;
    }
    if (stage == 3)
    {
        if (bits & PT_RFL)
        {
            if (depth != 0)
            {
                const float4 hh = p.h, m = p.m;
                const int srf = __float_as_int(m.w);
                const qr_srf *__restrict__ s = &S.srf[srf];
                const float hit[3] = {hh.x, hh.y, hh.z}, dir[3] = {m.x, m.y, m.z};
                const float4 l = p.l;
                const float loc[3] = {l.x, l.y, l.z};
                CNT(QR_STAT_RAY_SECONDARY);
                child_ray(r, hit, dir, loc, srf, side, depth - 1);
                off = __ldg(&s->sec_off[side]);
                num = __ldg(&s->sec_num[side]);
                rcode = 3u * pt_code(p) + 3u;
                c.w = 0.0f;
                p.a = c;
                pt_set_stage(p, 4);
                return 1;
            }
            c.x = 0.0f + c.x; c.y = 0.0f + c.y; c.z = 0.0f + c.z;
        }
        ret[0] = c.x; ret[1] = c.y; ret[2] = c.z;
        return 0;
    }
    /* stage 4: the reflected child's colour */
    const float cr = p.h.w;
    float t;
    t = ret[0] * cr; ret[0] = t + c.x;
    t = ret[1] * cr; ret[1] = t + c.y;
    t = ret[2] * cr; ret[2] = t + c.z;
    return 0;
}

/* the camera ray of a path-tracer sample: tent-jittered position in the
 * pixel (the two jitter draws of node 0) */
__device__ __forceinline__ void pt_camera_ray(const qr_frame_params &P, int x, int y,
                                              unsigned long long ks, Ray &r, StP st)
{
    const unsigned long long k0 = pt_node_key(ks, 0u);
    float hs = pt_tent(pt_draw(k0, PT_DRAW_JITTER));
    float vs = pt_tent(pt_draw(k0, PT_DRAW_JITTER + 1));
    hs = (float)x + hs;
    vs = (float)y + vs;
    camera_ray(P, hs, vs, r);
    CNT(QR_STAT_RAY_PRIMARY);
}

/* one path-tracer sample: the ray tree as one loop over traced segments.
 * Every node has at most three children (diffuse, transmitted, reflected),
 * so the tree holds at most (3^(depth+1) - 1) / 2 rays; a pixel that traces
 * more (or whose walk gives up) is recorded in the fault word and the
 * sample is black */
static __device__ void trace_pt(const qr_dscene &S, const qr_frame_params &P, Ray r,
                         int x, int y, int seg_lim, unsigned long long ks, float col[3],
                         StP st)
{
    PtPend stk[QR_MAX_DEPTH + 1];
    int sp = 0, off = S.cam_off, num = S.cam_num;
    uint32_t rcode = 0u;                /* tree code of the ray r */
    float ret[3];
    int seg = 0;
    #pragma unroll 1
    for (;;)
    {
        if (++seg > seg_lim)
        {
            note_fault(S, QR_FAULT_TREE, x, y);
            col[0] = col[1] = col[2] = 0.0f;
            return;
        }
        Walk w;
        w.fault = 0;
        w.shadow = 0;
        w.occluded = 0;
        w.tbuf = r.t_max;
        w.bestp = -1;
        w.best.srf = -1;
        walk(S, P, r, off, num, w, st);
        if (w.fault)
        {
            note_fault(S, w.fault, x, y);
            col[0] = col[1] = col[2] = 0.0f;
            return;
        }
        if (w.best.srf >= 0 && sp > QR_MAX_DEPTH)
        {
            /* a node below the deepest level a tree of QR_MAX_DEPTH has */
            note_fault(S, QR_FAULT_TREE, x, y);
            col[0] = col[1] = col[2] = 0.0f;
            return;
        }
        if (w.best.srf < 0)
        {
            ret[0] = ret[1] = ret[2] = 0.0f;
        }
        else
        {
            CNT(QR_STAT_SHADE);
            PtPend &p = stk[sp++];
            float ddir[3];
            const Hit hb = w.best;
            if (pt_begin(S, P, r, hb, p, ks, rcode, ddir, st))
            {
                const qr_srf *__restrict__ s = &S.srf[hb.srf];
                CNT(QR_STAT_RAY_SECONDARY);
                child_ray(r, hb.hit, ddir, hb.loc, hb.srf, hb.side, r.depth - 1);
                off = __ldg(&s->sec_off[hb.side]);
                num = __ldg(&s->sec_num[hb.side]);
                rcode = 3u * rcode + 1u;
                continue;
            }
        }

        int spawned = 0;
        #pragma unroll 1
        while (sp > 0)
        {
            if (pt_advance(S, stk[sp - 1], ret, r, off, num, rcode, st)) { spawned = 1; break; }
            sp--;
        }
        if (!spawned) break;
    }
    #pragma unroll
    for (int k = 0; k < 3; k++) col[k] = ret[k];
}

/* one pixel of a path-traced frame, one sample after the other: pt_on
 * samples added to the running sums, the mean clamped and packed */
__device__ __forceinline__ void pt_pixel_seq(const qr_dscene &S, const qr_frame_params &P,
                                         int x, int y, float *acc, uint32_t *frame, StP st)
{
    const unsigned long long pixel = (unsigned long long)y * P.x_res + x;
    const int spp = P.pt_on;
    const int n0 = (int)P.pts_c;
    int seg_lim = 1;
    #pragma unroll 1
    for (int d = 0; d <= P.depth; d++) seg_lim *= 3;
    seg_lim = (seg_lim - 1) / 2;
    float sum[3] = {0.0f, 0.0f, 0.0f};
    #pragma unroll 1
    for (int n = 0; n < spp; n++)
    {
        Ray r;
        const unsigned long long ks = pt_sample_key(P.seed, P.frame_idx, pixel, n0 + n);
        pt_camera_ray(P, x, y, ks, r, st);
        float col[3];
        trace_pt(S, P, r, x, y, seg_lim, ks, col, st);
        #pragma unroll
        for (int k = 0; k < 3; k++) sum[k] = sum[k] + col[k];
    }
    float *a = acc + 3 * ((size_t)y * P.x_row + x);
    float mean[3];
    #pragma unroll
    for (int k = 0; k < 3; k++)
    {
        a[k] = (n0 == 0 ? 0.0f : a[k]) + sum[k];
        mean[k] = fdiv(a[k], (float)(n0 + spp));
        mean[k] = clamp1(mean[k]);
    }
    frame[(size_t)y * P.x_row + x] = pack(P, mean);
}

/*
 * The same with the samples inside one loop over traced segments.
 *
 * Each sample's ray tree is walked as a loop over traced segments.  Every
 * node has at most three children (diffuse, transmitted, reflected), so
 * the tree holds at most (3^(depth+1) - 1) / 2 rays; a sample that traces
 * more (or whose walk gives up) is recorded in the fault word and is black.
 * The samples follow one another inside the same loop: a lane whose sample
 * tree ends starts its next sample at once instead of waiting for the
 * largest tree of its warp, so the lanes of a warp stay in the walk
 * together; each pixel draws its stream and sums its samples in the same
 * order as one sample after the other, so the frame is the same.  It pays
 * from about 32 samples a launch on (fewer samples leave too short a run to
 * even out, and the longer loop costs instructions): qr_launch_pt picks it
 * from QR_PT_FLAT_SPP samples on.
 */
__device__ __forceinline__ void pt_pixel_flat(const qr_dscene &S, const qr_frame_params &P,
                                         int x, int y, float *acc, uint32_t *frame, StP st)
{
    const unsigned long long pixel = (unsigned long long)y * P.x_res + x;
    const int spp = P.pt_on;
    const int n0 = (int)P.pts_c;
    int seg_lim = 1;
    #pragma unroll 1
    for (int d = 0; d <= P.depth; d++) seg_lim *= 3;
    seg_lim = (seg_lim - 1) / 2;
    float sum[3] = {0.0f, 0.0f, 0.0f};

    PtPend stk[QR_MAX_DEPTH + 1];
    int n = 0, sp = 0, seg = 0, off = S.cam_off, num = S.cam_num;
    uint32_t rcode = 0u;                /* tree code of the ray r */
    float ret[3];
    Ray r;
    unsigned long long ks = pt_sample_key(P.seed, P.frame_idx, pixel, n0);
    if (spp > 0) pt_camera_ray(P, x, y, ks, r, st);
    #pragma unroll 1
    while (n < spp)
    {
        int done = 0;
        if (++seg > seg_lim)
        {
            note_fault(S, QR_FAULT_TREE, x, y);
            ret[0] = ret[1] = ret[2] = 0.0f;
            done = 1;
        }
        else
        {
            Walk w;
            w.fault = 0;
            w.shadow = 0;
            w.occluded = 0;
            w.tbuf = r.t_max;
            w.bestp = -1;
            w.best.srf = -1;
            walk(S, P, r, off, num, w, st);
            if (w.fault)
            {
                note_fault(S, w.fault, x, y);
                ret[0] = ret[1] = ret[2] = 0.0f;
                done = 1;
            }
            else
            {
                int spawned = 0;
                if (w.best.srf >= 0 && sp > QR_MAX_DEPTH)
                {
                    /* a node below the deepest level a tree can have: the
                     * sample is black */
                    note_fault(S, QR_FAULT_TREE, x, y);
                    ret[0] = ret[1] = ret[2] = 0.0f;
                    sp = 0;
                }
                else if (w.best.srf < 0)
                {
                    ret[0] = ret[1] = ret[2] = 0.0f;
                }
                else
                {
                    CNT(QR_STAT_SHADE);
                    PtPend &p = stk[sp++];
                    float ddir[3];
                    const Hit hb = w.best;
                    if (pt_begin(S, P, r, hb, p, ks, rcode, ddir, st))
                    {
                        const qr_srf *__restrict__ s = &S.srf[hb.srf];
                        CNT(QR_STAT_RAY_SECONDARY);
                        child_ray(r, hb.hit, ddir, hb.loc, hb.srf, hb.side, r.depth - 1);
                        off = __ldg(&s->sec_off[hb.side]);
                        num = __ldg(&s->sec_num[hb.side]);
                        rcode = 3u * rcode + 1u;
                        spawned = 1;
                    }
                }
                #pragma unroll 1
                while (!spawned && sp > 0)
                {
                    if (pt_advance(S, stk[sp - 1], ret, r, off, num, rcode, st)) spawned = 1;
                    else sp--;
                }
                done = !spawned;
            }
        }
        if (done)
        {
            /* the sample's colour; the next sample starts in this lane */
            #pragma unroll
            for (int k = 0; k < 3; k++) sum[k] = sum[k] + ret[k];
            n++;
            sp = 0;
            seg = 0;
            off = S.cam_off;
            num = S.cam_num;
            rcode = 0u;
            if (n < spp)
            {
                ks = pt_sample_key(P.seed, P.frame_idx, pixel, n0 + n);
                pt_camera_ray(P, x, y, ks, r, st);
            }
        }
    }
    float *a = acc + 3 * ((size_t)y * P.x_row + x);
    float mean[3];
    #pragma unroll
    for (int k = 0; k < 3; k++)
    {
        a[k] = (n0 == 0 ? 0.0f : a[k]) + sum[k];
        mean[k] = fdiv(a[k], (float)(n0 + spp));
        mean[k] = clamp1(mean[k]);
    }
    frame[(size_t)y * P.x_row + x] = pack(P, mean);
}

} /* namespace QR_NS */

#endif /* QR_TRACER_DEV_CUH */

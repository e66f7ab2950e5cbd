/*
 * whitted_wf.cu: the Whitted tracer as wavefront stages over ray queues in
 * HBM.
 *
 * The reference traces one SIMD group of rays through its whole ray tree:
 * the surface list walk, the lights loop with a shadow ray to each light
 * (core/tracer/tracer.cpp:4008-4096), then the refracted and reflected
 * children through its context stack (4820-4860, 5235-5275).  Here each
 * level of the frame's ray trees is a set of stages over a compacted queue,
 * so that every kernel runs one kind of ray and keeps only that ray's state:
 *
 *   wh_gen     camera rays (and AA sub-samples) of a chunk of samples;
 *   wh_step    level d: walk to the nearest hit, shade the hit (normal,
 *              texel, ambient: tracer.cpp:3255-3416, 3945-3987) into a node
 *              record, append a shadow ray for each light facing the hit and
 *              the refracted and reflected children (4442-5359), warp by
 *              warp with a scan and one atomic (no dead lanes); the shadow
 *              rays are appended light by light across the warp, so runs of
 *              neighbouring hits aim at the same light;
 *   wh_shadow  level d's shadow rays: any occluder (CHECK_SHAD, 576-616),
 *              recorded as a bit of the node's light mask;
 *   wh_light   level d's nodes: the diffuse and specular terms of every
 *              facing light that is not occluded, in light-list order
 *              (4100-4391), as the reference adds them;
 *   wh_fold    levels from the deepest up: colour = rc c_rfl + (tc c_trn +
 *              local), handed to the parent's record or the sample's slot;
 *   wh_pack    clamp, AA average in the reference's pairing, gamma, pack
 *              (7028-7145, 1922-1940).
 *
 * Every step is the arithmetic of tracer_dev.cuh in the same order, so the
 * frame is the per-pixel kernel's (whitted_kernel / whitted_aa_kernel) bit
 * for bit.  Capacities are fixed per chunk; a queue or the node pool that
 * would overflow sets the overflow word, every later stage does nothing and
 * wh_fallback renders the frame with the per-pixel code instead.
 */
#include <atomic>
#include "wf_common.cuh"
#include "whitted_wf.h"

namespace qr_dev
{

/* a shaded hit (or a miss) of a Whitted ray tree, 144 bytes */
struct HNode
{
    float4 h;       /* hit point, surface (int) */
    float4 l;       /* local hit point, material props (int) */
    float4 n;       /* normal, light list offset (int) */
    float4 x;       /* texel colour, light list length (int) */
    float4 r;       /* direction of the shaded ray, depth | side << 8 | HN_* << 9 */
    float4 c;       /* colour: ambient, then with the lights; owner (int) */
    float4 w;       /* c_trn, c_rfl, occluded lights 0-31, 32-63 (bits) */
    float4 ct;      /* the refracted child's colour */
    float4 cr;      /* the reflected child's colour */
};

#define HN_HIT      1
#define HN_TRN      2
#define HN_RFL      4
#define HN_SPAWN    8

/* lights a light list may hold for the wavefront (two mask words) */
#define QR_WH_MAX_LIGHTS 64

struct WhCtl
{
    int cnt[QR_MAX_DEPTH + 2];      /* rays of each level */
    int off[QR_MAX_DEPTH + 2];      /* first pool node of each level */
    int next[QR_MAX_DEPTH + 2];     /* rays of each level handed to warps */
    int scnt[QR_MAX_DEPTH + 2];     /* shadow rays of each level */
    int snext[QR_MAX_DEPTH + 2];    /* shadow rays handed to warps */
    int overflow;
    int pad[3];
};

#ifndef QR_WH_MIN_BLOCKS
#define QR_WH_MIN_BLOCKS 6
#endif

/* level 0: the camera rays of samples [c0, c1); sample q is sub-sample
 * q % ns of pixel place q / ns in the tile order */
__global__ void __launch_bounds__(128)
wh_gen(const qr_frame_params P, long long c0, long long c1, int ns, int tx, WRay *q0,
       WhCtl *ctl)
{
    if (ctl->overflow) return;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q00 = c0 + (((long long)blockIdx.x * blockDim.x + threadIdx.x) & ~31ll);
         q00 < c1; q00 += stride)
    {
        const long long q = q00 + (threadIdx.x & 31);
        int x = 0, y = 0, ok = 0, sub = 0;
        if (q < c1)
        {
            const int t = (int)(q / ns);
            sub = (int)(q - (long long)t * ns);
            tile_pixel(t, tx, x, y);
            ok = x < P.x_res && y < P.y_res;
        }
        int tot;
        const int ex = warp_excl_scan(ok, &tot);
        const int base = warp_reserve(&ctl->cnt[0], tot);
        if (!ok) continue;
        float hs = (float)x, vs = (float)y;
        if (ns == 4) { hs = hs + c_aa4_h[sub]; vs = vs + c_aa4_v[sub]; }
        if (ns == 2) { hs = hs + c_aa2_h[x & 1][sub]; vs = vs + c_aa2_v[x & 1][sub]; }
        Ray r;
        camera_ray(P, hs, vs, r);
        put_ray(q0, base + ex, r.org, r.t_min, r.dir, r.t_max, r.phit, r.from, r.flags,
                r.depth, (int)(q - c0), 0u, -1, 0, 0ull, 0);
    }
}

/* level d: nearest hit, shading, shadow rays and children */
__global__ void __launch_bounds__(128, QR_WH_MIN_BLOCKS)
wh_step(const qr_dscene S, const qr_frame_params P, int d, const WRay *__restrict__ qin,
        WRay *qout, WRay *sq, HNode *pool, WhCtl *ctl, int cap_q, int cap_s, int cap_pool)
{
    if (ctl->overflow) return;
    const int n = ctl->cnt[d];
    const int base = d == 0 ? 0 : ctl->off[d];
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->off[d + 1] = base + n;
    const int lane = threadIdx.x & 31;
    #pragma unroll 1
    for (;;)
    {
        int i0 = 0;
        if (lane == 0) i0 = atomicAdd(&ctl->next[d], 32);
        i0 = __shfl_sync(0xFFFFFFFFu, i0, 0);
        if (i0 >= n) break;
        const int i = i0 + lane;
        const int node = base + i;
        Shade sh;
        Sec o;
        int lnum = 0, trn = 0, rfl = 0;
        sh.srf = -1;
        if (i < n)
        {
            Ray r;
            int off, num;
            const int owner = get_ray(qin[i], S, r, off, num);
            Walk w;
            walk_init(w, r, 0);
            walk(S, P, r, off, num, w, NULL);
            HNode &N = pool[node];
            if (w.fault)
            {
                note_fault(S, w.fault, 0, 0);
                w.best.srf = -1;
            }
            if (w.best.srf < 0)
            {
                N.c = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(owner));
                N.r = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(0));
            }
            else
            {
                shade_begin(S, P, r, w.best, sh);
                shade_end(S, sh, o, NULL);
                const int spawn = sh.depth != 0;
                trn = o.trn && spawn;
                rfl = o.rfl && spawn;
                lnum = sh.lnum;
                N.h = make_float4(sh.hit[0], sh.hit[1], sh.hit[2], __int_as_float(sh.srf));
                N.l = make_float4(sh.loc[0], sh.loc[1], sh.loc[2], __int_as_float(sh.props));
                N.n = make_float4(sh.nrm[0], sh.nrm[1], sh.nrm[2], __int_as_float(sh.loff));
                N.x = make_float4(sh.tex[0], sh.tex[1], sh.tex[2], __int_as_float(sh.lnum));
                N.r = make_float4(sh.dir[0], sh.dir[1], sh.dir[2],
                                  __int_as_float(sh.depth | (sh.side << 8) |
                                                 ((HN_HIT | (o.trn ? HN_TRN : 0) |
                                                   (o.rfl ? HN_RFL : 0) |
                                                   (spawn ? HN_SPAWN : 0)) << 9)));
                N.c = make_float4(sh.c[0], sh.c[1], sh.c[2], __int_as_float(owner));
                N.w = make_float4(o.c_trn, o.c_rfl, __int_as_float(0), __int_as_float(0));
            }
        }
        /* a shadow ray to every facing light, light by light over the warp */
        const int maxl = __reduce_max_sync(0xFFFFFFFFu, lnum);
        #pragma unroll 1
        for (int li = 0; li < maxl; li++)
        {
            int f = 0;
            if (li < lnum)
            {
                float lv[3];
                f = 0.0f < light_dot(S, sh, li, lv);
            }
            int tot;
            const int ex = warp_excl_scan(f, &tot);
            const int sb = warp_reserve(&ctl->scnt[d], tot);
            if (sb + tot > cap_s)
            {
                if (lane == 0 && tot > 0) atomicExch(&ctl->overflow, 1);
                continue;
            }
            if (f)
            {
                Ray sr;
                int soff, snum;
                shadow_ray(S, sh, li, sr, soff, snum);
                put_ray(sq, sb + ex, sr.org, sr.t_min, sr.dir, sr.t_max, sr.phit, sr.from,
                        sr.flags, sr.depth, node, (uint32_t)li, soff, snum, 0ull, 0);
            }
        }
        /* the children, refracted first (4820-4860, 5235-5298) */
        const int nch = trn + rfl;
        int tot;
        const int ex = warp_excl_scan(nch, &tot);
        const int qb = warp_reserve(&ctl->cnt[d + 1], tot);
        if (qb + tot > cap_q || base + n + qb + tot > cap_pool)
        {
            if (lane == 0 && tot > 0) atomicExch(&ctl->overflow, 1);
            continue;
        }
        if (nch == 0) continue;
        const qr_srf *__restrict__ s = &S.srf[sh.srf];
        const int side = sh.side;
        int at = qb + ex;
        if (trn)
            put_ray(qout, at++, sh.hit, 0.0f, o.nw, FLT_MAX, sh.loc, sh.srf, side | FLAG_PASS,
                    sh.depth - 1, owner_of(node, 1), 0u, __ldg(&s->sec_off[1 - side]),
                    __ldg(&s->sec_num[1 - side]), 0ull, 0);
        if (rfl)
            put_ray(qout, at++, sh.hit, 0.0f, o.rw, FLT_MAX, sh.loc, sh.srf, side,
                    sh.depth - 1, owner_of(node, 2), 0u, __ldg(&s->sec_off[side]),
                    __ldg(&s->sec_num[side]), 0ull, 0);
    }
}

/* level d's shadow rays: any occluder marks the light in its node's mask */
__global__ void __launch_bounds__(128)
wh_shadow(const qr_dscene S, const qr_frame_params P, int d, const WRay *__restrict__ sq,
          HNode *pool, WhCtl *ctl)
{
    if (ctl->overflow) return;
    const int n = ctl->scnt[d];
    const int lane = threadIdx.x & 31;
    #pragma unroll 1
    for (;;)
    {
        int j0 = 0;
        if (lane == 0) j0 = atomicAdd(&ctl->snext[d], 32);
        j0 = __shfl_sync(0xFFFFFFFFu, j0, 0);
        if (j0 >= n) break;
        const int j = j0 + lane;
        if (j >= n) continue;
        const WRay q = sq[j];
        Ray r;
        int off, num;
        const int node = get_ray(q, S, r, off, num);
        const int li = q.m.z;
        Walk w;
        walk_init(w, r, 1);
        walk(S, P, r, off, num, w, NULL);
        if (w.fault) note_fault(S, w.fault, 0, 0);
        if (w.occluded || w.fault)
        {
            unsigned int *mask = reinterpret_cast<unsigned int *>(&pool[node].w.z);
            atomicOr(&mask[li >> 5], 1u << (li & 31));
        }
    }
}

/* level d's nodes: the unoccluded facing lights, in list order */
__global__ void __launch_bounds__(128)
wh_light(const qr_dscene S, int d, HNode *pool, const WhCtl *ctl)
{
    if (ctl->overflow) return;
    const int n = ctl->cnt[d];
    const int base = d == 0 ? 0 : ctl->off[d];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        HNode &N = pool[base + i];
        const float4 xv = N.x;
        const int lnum = __float_as_int(xv.w);
        const float4 rv = N.r;
        const int bits = __float_as_int(rv.w);
        if (!((bits >> 9) & HN_HIT) || lnum <= 0) continue;
        Shade sh;
        const float4 hv = N.h, lv4 = N.l, nv = N.n, cv = N.c, wv = N.w;
        sh.srf = __float_as_int(hv.w);
        sh.side = (bits >> 8) & 1;
        sh.props = __float_as_int(lv4.w);
        sh.hit[0] = hv.x; sh.hit[1] = hv.y; sh.hit[2] = hv.z;
        sh.loc[0] = lv4.x; sh.loc[1] = lv4.y; sh.loc[2] = lv4.z;
        sh.nrm[0] = nv.x; sh.nrm[1] = nv.y; sh.nrm[2] = nv.z;
        sh.tex[0] = xv.x; sh.tex[1] = xv.y; sh.tex[2] = xv.z;
        sh.c[0] = cv.x; sh.c[1] = cv.y; sh.c[2] = cv.z;
        sh.dir[0] = rv.x; sh.dir[1] = rv.y; sh.dir[2] = rv.z;
        sh.depth = bits & 255;
        sh.loff = __float_as_int(nv.w);
        sh.lnum = lnum;
        const unsigned int m0 = __float_as_uint(wv.z), m1 = __float_as_uint(wv.w);
        #pragma unroll 1
        for (int li = 0; li < lnum; li++)
        {
            float l3[3];
            if (!(0.0f < light_dot(S, sh, li, l3))) continue;
            const unsigned int m = li < 32 ? m0 : m1;
            if ((m >> (li & 31)) & 1u) continue;
            light_add(S, sh, li);
        }
        N.c = make_float4(sh.c[0], sh.c[1], sh.c[2], cv.w);
    }
}

/* level d, deepest first: the node's colour to its owner */
__global__ void __launch_bounds__(128)
wh_fold(int d, HNode *pool, float4 *samples, const WhCtl *ctl)
{
    if (ctl->overflow) return;
    const int n = ctl->cnt[d];
    const int base = d == 0 ? 0 : ctl->off[d];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const HNode &N = pool[base + i];
        const int bits = __float_as_int(N.r.w) >> 9;
        const float4 cv = N.c;
        const int owner = __float_as_int(cv.w);
        float c[3] = {0.0f, 0.0f, 0.0f};
        if (bits & HN_HIT)
        {
            const float4 wv = N.w;
            c[0] = cv.x; c[1] = cv.y; c[2] = cv.z;
            if (bits & HN_TRN)
            {
                float tc[3] = {0.0f, 0.0f, 0.0f};
                if (bits & HN_SPAWN)
                {
                    const float4 t = N.ct;
                    tc[0] = t.x * wv.x; tc[1] = t.y * wv.x; tc[2] = t.z * wv.x;
                }
                c[0] = tc[0] + c[0]; c[1] = tc[1] + c[1]; c[2] = tc[2] + c[2];
            }
            if (bits & HN_RFL)
            {
                float rc[3] = {0.0f, 0.0f, 0.0f};
                if (bits & HN_SPAWN)
                {
                    const float4 t = N.cr;
                    rc[0] = t.x * wv.y; rc[1] = t.y * wv.y; rc[2] = t.z * wv.y;
                }
                c[0] = rc[0] + c[0]; c[1] = rc[1] + c[1]; c[2] = rc[2] + c[2];
            }
        }
        const float4 out = make_float4(c[0], c[1], c[2], 0.0f);
        if (d == 0)
            samples[owner] = out;
        else if ((owner & 3) == 1)
            pool[owner >> 2].ct = out;
        else
            pool[owner >> 2].cr = out;
    }
}

/* the pixels of samples [c0, c1): clamp, AA average, pack */
__global__ void __launch_bounds__(128)
wh_pack(const qr_frame_params P, long long c0, long long c1, int ns, int tx,
        const float4 *__restrict__ samples, uint32_t *frame, const WhCtl *ctl)
{
    if (ctl->overflow) return;
    const long long t0 = c0 / ns, t1 = c1 / ns;
    for (long long t = t0 + blockIdx.x * blockDim.x + threadIdx.x; t < t1;
         t += (long long)gridDim.x * blockDim.x)
    {
        int x, y;
        tile_pixel((int)t, tx, x, y);
        if (x >= P.x_res || y >= P.y_res) continue;
        const float4 *sp = samples + (t * ns - c0);
        float col[3];
        if (ns == 1)
        {
            const float4 v = sp[0];
            col[0] = clamp1(v.x); col[1] = clamp1(v.y); col[2] = clamp1(v.z);
        }
        else if (ns == 2)
        {
            const float4 a = sp[0], b = sp[1];
            const float av[3] = {a.x, a.y, a.z}, bv[3] = {b.x, b.y, b.z};
            #pragma unroll
            for (int k = 0; k < 3; k++)
            {
                const float h0 = clamp1(av[k]) * 0.5f;
                col[k] = h0 + clamp1(bv[k]) * 0.5f;
            }
        }
        else
        {
            const float4 a = sp[0], b = sp[1], c = sp[2], e = sp[3];
            const float v0[3] = {a.x, a.y, a.z}, v1[3] = {b.x, b.y, b.z};
            const float v2[3] = {c.x, c.y, c.z}, v3[3] = {e.x, e.y, e.z};
            #pragma unroll
            for (int k = 0; k < 3; k++)
            {
                const float p01 = clamp1(v0[k]) * 0.5f + clamp1(v1[k]) * 0.5f;
                const float p23 = clamp1(v2[k]) * 0.5f + clamp1(v3[k]) * 0.5f;
                col[k] = p01 * 0.5f + p23 * 0.5f;
            }
        }
        frame[(size_t)y * P.x_row + x] = pack(P, col);
    }
}

/* the whole frame by the per-pixel code, when a queue overflowed */
__global__ void __launch_bounds__(128, QR_MIN_BLOCKS)
wh_fallback(const qr_dscene S, const qr_frame_params P, uint32_t *frame, const WhCtl *ctl)
{
    if (!ctl->overflow) return;
    const int x = tile_x(), y = tile_y();
    if (x >= P.x_res || y >= P.y_res) return;
    whitted_pixel(S, P, x, y, frame, NULL);
}

} /* namespace qr_dev */

using namespace qr_dev;

static inline size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

qr_wh_caps qr_wh_caps_for(const qr_frame_params &fp, int max_lights, long long max_samples)
{
    qr_wh_caps c;
    const int ns = fp.fsaa == 2 ? 4 : fp.fsaa == 1 ? 2 : 1;
    const int tx = (fp.x_res + 7) / 8, ty = (fp.y_res + 3) / 4;
    const long long total = (long long)tx * ty * 32 * ns;
    const int nl = max_lights < 1 ? 1 : max_lights;
    long long cap = max_samples;
    /* the shadow queue holds up to a ray per light of every hit of a level */
    if (cap * nl > 8 * max_samples) cap = 8 * max_samples / nl;
    cap = (cap / 128) * 128;
    if (cap < 128) cap = 128;
    if (cap > total) cap = ((total + 127) / 128) * 128;
    c.cap_samples = cap;
    c.cap_q = 2 * cap;
    c.cap_s = (long long)nl * cap;
    c.cap_pool = 4 * cap;
    c.ok = max_lights <= QR_WH_MAX_LIGHTS;
    return c;
}

size_t qr_wh_bytes(const qr_wh_caps &c)
{
    return al256(sizeof(WhCtl)) + 2 * al256((size_t)c.cap_q * sizeof(WRay)) +
           al256((size_t)c.cap_s * sizeof(WRay)) + al256((size_t)c.cap_pool * sizeof(HNode)) +
           al256((size_t)c.cap_samples * sizeof(float4));
}

cudaError_t qr_wh_launch(const qr_dscene &sc, const qr_frame_params &fp, uint32_t *frame,
                         void *scratch, const qr_wh_caps &caps, int sms, cudaStream_t stream)
{
    unsigned char *b = (unsigned char *)scratch;
    WhCtl *ctl = (WhCtl *)b;
    b += al256(sizeof(WhCtl));
    WRay *qa = (WRay *)b;
    b += al256((size_t)caps.cap_q * sizeof(WRay));
    WRay *qb = (WRay *)b;
    b += al256((size_t)caps.cap_q * sizeof(WRay));
    WRay *sq = (WRay *)b;
    b += al256((size_t)caps.cap_s * sizeof(WRay));
    HNode *pool = (HNode *)b;
    b += al256((size_t)caps.cap_pool * sizeof(HNode));
    float4 *samples = (float4 *)b;

    const int ns = fp.fsaa == 2 ? 4 : fp.fsaa == 1 ? 2 : 1;
    const int tx = (fp.x_res + 7) / 8, ty = (fp.y_res + 3) / 4;
    const long long total = (long long)tx * ty * 32 * ns;
    const int levels = fp.depth + 1;
    /* resident blocks a SM of the stepping and shadow stages (queried once;
     * the values are the same whichever thread stores them) */
    static std::atomic<int> g_step(0), g_shadow(0);
    if (g_step.load(std::memory_order_acquire) == 0)
    {
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, wh_step, 128, 0) != cudaSuccess ||
            nb <= 0)
            nb = QR_WH_MIN_BLOCKS;
        int ns2 = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ns2, wh_shadow, 128, 0) != cudaSuccess ||
            ns2 <= 0)
            ns2 = 8;
        g_shadow.store(ns2, std::memory_order_relaxed);
        g_step.store(nb, std::memory_order_release);
    }
    const int step_per_sm = g_step.load(std::memory_order_acquire);
    const int shadow_per_sm = g_shadow.load(std::memory_order_relaxed);
    const int blocks = sms * 8;
    cudaError_t e = cudaMemsetAsync(ctl, 0, sizeof(WhCtl), stream);
    for (long long c0 = 0; c0 < total && e == cudaSuccess; c0 += caps.cap_samples)
    {
        const long long c1 = c0 + caps.cap_samples < total ? c0 + caps.cap_samples : total;
        e = cudaMemsetAsync(ctl, 0, offsetof(WhCtl, overflow), stream);
        if (e != cudaSuccess) break;
        wh_gen<<<blocks, 128, 0, stream>>>(fp, c0, c1, ns, tx, qa, ctl);
        for (int d = 0; d < levels; d++)
        {
            WRay *qi = (d & 1) ? qb : qa, *qo = (d & 1) ? qa : qb;
            wh_step<<<sms * step_per_sm, 128, 0, stream>>>(sc, fp, d, qi, qo, sq, pool, ctl,
                                                          (int)caps.cap_q, (int)caps.cap_s,
                                                          (int)caps.cap_pool);
            wh_shadow<<<sms * shadow_per_sm, 128, 0, stream>>>(sc, fp, d, sq, pool, ctl);
            wh_light<<<blocks, 128, 0, stream>>>(sc, d, pool, ctl);
        }
        for (int d = levels - 1; d >= 0; d--)
            wh_fold<<<blocks, 128, 0, stream>>>(d, pool, samples, ctl);
        wh_pack<<<blocks, 128, 0, stream>>>(fp, c0, c1, ns, tx, samples, frame, ctl);
        qr_note_launches(stream, 2 + 4 * levels);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
    {
        const dim3 block(32, 4);
        const dim3 grid((fp.x_res + 2 * QR_TILE_W - 1) / (2 * QR_TILE_W),
                        (fp.y_res + 2 * QR_TILE_H - 1) / (2 * QR_TILE_H));
        wh_fallback<<<grid, block, 0, stream>>>(sc, fp, frame, ctl);
        qr_note_launches(stream, 1);
        e = cudaGetLastError();
    }
    return e;
}

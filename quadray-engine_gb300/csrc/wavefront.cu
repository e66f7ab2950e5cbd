/*
 * wavefront.cu: the path tracer as wavefront stages over ray queues in HBM.
 *
 * The reference bins its path-tracer rays per surface, side and depth in
 * SIMD buffers and shades a buffer once a full SIMD group waits in it, which
 * keeps its lanes busy while paths end at different depths
 * (core/tracer/tracer.cpp:783-1100 SLICE_FRAG / STORE_BUFF / SLICE_SPTR,
 * 6686-6915, end-of-frame flush 7239-7375).  Here every level of the
 * samples' ray trees is one stage over a compacted queue:
 *
 *   wf_gen    camera rays of a chunk of samples, pixel tiles of 8 x 4 in a
 *             warp, appended to level 0's queue;
 *   wf_trace  level d: each ray walks the scene to its nearest hit, which
 *             is stored for the next stage (32 bytes a ray);
 *   wf_step   level d: each ray's hit is
 *             shaded (the node's random draws, emission, roulette,
 *             cosine-weighted bounce, the dielectric split) into a node
 *             record, and the node's children are appended to level d+1's
 *             queue: the lanes of a warp count their children, a warp scan
 *             gives each lane its offset and one atomic reserves the warp's
 *             run (warp-vote compaction: level d+1 holds no dead lanes);
 *   wf_fold   levels from the deepest up: a node's colour from its
 *             children's colours (written into its record by their fold),
 *             in the reference's order colour = rc c_rfl + (tc c_trn +
 *             (bounce l_dff tex + emission)), handed to its parent's record
 *             or, at level 0, to the sample's slot;
 *   wf_accum  each pixel adds its samples of the chunk in sample order;
 *   wf_final  running sums, mean, clamp and pack (as pt_kernel).
 *
 * Random draws are counter-based (tracer_dev.cuh pt_node_key / pt_draw), so
 * breadth-first evaluation draws what the depth-first oracle draws and the
 * frame is the per-pixel kernel's (pt_kernel) bit for bit.
 *
 * Chunks.  A frame's samples are numbered sample-major (path q = s * Ppad +
 * t, t the pixel's place in the tile order over Ppad padded pixels) and cut
 * into chunks of at most cap_paths paths, rendered one after the other or,
 * with a second scratch block, two at a time on two streams; either way a
 * chunk's samples join the sums after the previous chunk's, so a pixel's
 * samples are summed in ascending s whatever the chunking.  Queues
 * and the node pool have fixed capacities: a level whose children would not
 * fit sets the overflow word; every later stage of the frame then does
 * nothing and wf_fallback renders the whole frame with the per-pixel kernel
 * (the same frame).  No host synchronisation is needed: every kernel reads
 * its level's count from device memory and strides over it.
 */
#include <atomic>
#include "wf_common.cuh"
#include "wavefront.h"

namespace qr_dev
{

/* a shaded node (or a miss), 96 bytes; its children write cl / ct / cr */
struct WNode
{
    float4 t;       /* tex scaled by roulette, l_dff (diffuse child) */
    float4 e;       /* emission, c_trn */
    float4 f;       /* c_rfl, bits (int), owner (int), - */
    float4 cl;      /* the diffuse child's colour */
    float4 ct;      /* the refracted child's colour */
    float4 cr;      /* the reflected child's colour */
};

#define WN_HIT      1
#define WN_DIF      2
#define WN_TRN      4
#define WN_RFL      8
#define WN_SPAWN    16

#ifndef QR_WF_MIN_BLOCKS
#define QR_WF_MIN_BLOCKS 6
#endif
#ifndef QR_WF_TRACE_MIN_BLOCKS
#define QR_WF_TRACE_MIN_BLOCKS 7
#endif

/* a ray's nearest hit from the tracing stage, 32 bytes: hit point and
 * surface (-1: none), local hit point and side | walk fault << 8 */
struct WHit
{
    float4 h;
    float4 l;
};

/* level d's nearest hits: warps take runs of 32 rays as they come free.
 * The walk in a kernel of its own, ahead of the shading: each kernel is
 * smaller (the shading's registers no longer spill around the walk), and
 * the 1280x720 64-spp frame takes 175.0 against 181.9 ms with the walk
 * inside the shading stage (at 8 resident blocks for the shading 177.0,
 * and for both 178.6 ms) */
__global__ void __launch_bounds__(128, QR_WF_TRACE_MIN_BLOCKS)
wf_trace(const qr_dscene S, const qr_frame_params P, int d, const WRay *__restrict__ qin,
         WHit *hits, WCtl *ctl)
{
    if (ctl->overflow) return;
    const int n = ctl->cnt[d];
    const int lane = threadIdx.x & 31;
    #pragma unroll 1
    for (;;)
    {
        int i0 = 0;
        if (lane == 0) i0 = atomicAdd(&ctl->tnext[d], 32);
        i0 = __shfl_sync(0xFFFFFFFFu, i0, 0);
        if (i0 >= n) break;
        const int i = i0 + lane;
        if (i >= n) continue;
        Ray r;
        int off, num;
        get_ray(qin[i], S, r, off, num);
        Walk w;
        walk_init(w, r, 0);
        /* over the 4-wide records: the 720p 64-spp frame 169.2 against
         * 175.1 ms over the binary tree's child records (and 170.0 ms with
         * the binary records for the camera rays only); 5, 7 and 8
         * resident blocks instead of 6: 174.0, 174.1, 182.3 ms.  With the
         * room's walls out of the tree: 121.6 ms (binary records 125.0),
         * at 7 resident blocks 120.0 ms */
        walk_t<1>(S, P, r, off, num, w, NULL);
        /* a ray without a hit has no side (the field is not set) */
        const int side = w.best.srf >= 0 ? (w.best.side & 1) : 0;
        WHit hh;
        hh.h = make_float4(w.best.hit[0], w.best.hit[1], w.best.hit[2],
                           __int_as_float(w.best.srf));
        hh.l = make_float4(w.best.loc[0], w.best.loc[1], w.best.loc[2],
                           __int_as_float(side | (w.fault << 8)));
        hits[i] = hh;
    }
}

/* level 0: camera rays of paths [c0, c1) */
__global__ void __launch_bounds__(128)
wf_gen(const qr_frame_params P, long long c0, long long c1, int ppad, int tx,
       WRay *q0, WCtl *ctl)
{
    if (ctl->overflow) return;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q00 = c0 + (((long long)blockIdx.x * blockDim.x + threadIdx.x) & ~31ll);
         q00 < c1; q00 += stride)
    {
        const long long q = q00 + (threadIdx.x & 31);
        int x = 0, y = 0, ok = 0, s = 0, t = 0;
        if (q < c1)
        {
            s = (int)(q / ppad);
            t = (int)(q - (long long)s * ppad);
            tile_pixel(t, tx, x, y);
            ok = x < P.x_res && y < P.y_res;
        }
        int tot;
        const int ex = warp_excl_scan(ok, &tot);
        const int base = warp_reserve(&ctl->cnt[0], tot);
        if (!ok) continue;
        const unsigned long long pixel = (unsigned long long)y * P.x_res + x;
        const unsigned long long ks = pt_sample_key(P.seed, P.frame_idx, pixel,
                                                    (int)P.pts_c + s);
        Ray r;
        pt_camera_ray(P, x, y, ks, r, NULL);
        put_ray(q0, base + ex, r.org, r.t_min, r.dir, r.t_max, r.phit, r.from, r.flags,
                r.depth, (int)(q - c0), 0u, -1, 0, ks, t);
    }
}

/* level d: take the tracing stage's hit, shade, append the children to
 * level d + 1 */
__global__ void __launch_bounds__(128, QR_WF_MIN_BLOCKS)
wf_step(const qr_dscene S, const qr_frame_params P, int d, const WRay *__restrict__ qin,
        const WHit *__restrict__ hits, WRay *qout, WNode *pool, WCtl *ctl, int cap_q,
        int cap_pool)
{
    if (ctl->overflow) return;
    const int n = ctl->cnt[d];
    const int base = d == 0 ? 0 : ctl->off[d];
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->off[d + 1] = base + n;
    const int lane = threadIdx.x & 31;
    /* warps take runs of 32 rays as they come free (rays differ widely in
     * cost) */
    #pragma unroll 1
    for (;;)
    {
        int i0 = 0;
        if (lane == 0) i0 = atomicAdd(&ctl->next[d], 32);
        i0 = __shfl_sync(0xFFFFFFFFu, i0, 0);
        if (i0 >= n) break;
        const int i = i0 + lane;
        int nch = 0, dif = 0, trn = 0, rfl = 0, side = 0, srf = -1, depth = 0;
        float hit[3], loc[3], ddir[3], nw[3], rw[3];
        uint32_t code = 0u;
        unsigned long long ks = 0ull;
        int tp = 0;
        if (i < n)
        {
            const WRay q = qin[i];
            Ray r;
            r.org[0] = q.o.x; r.org[1] = q.o.y; r.org[2] = q.o.z; r.t_min = q.o.w;
            r.dir[0] = q.d.x; r.dir[1] = q.d.y; r.dir[2] = q.d.z; r.t_max = q.d.w;
            r.phit[0] = q.p.x; r.phit[1] = q.p.y; r.phit[2] = q.p.z;
            r.from = __float_as_int(q.p.w);
            r.flags = q.m.x & 255;
            r.depth = q.m.x >> 8;
            const int owner = q.m.y;
            code = (uint32_t)q.m.z;
            const int off = q.m.w >= 0 ? q.m.w : S.cam_off;
            const int num = q.m.w >= 0 ? q.k.z : S.cam_num;
            ks = (unsigned long long)(uint32_t)q.k.x |
                 ((unsigned long long)(uint32_t)q.k.y << 32);
            tp = q.k.w;
            Walk w;
            w.fault = 0;
            w.shadow = 0;
            w.occluded = 0;
            w.tbuf = r.t_max;
            w.bestp = -1;
            w.best.srf = -1;
            {
                const WHit hh = hits[i];
                const int bits = __float_as_int(hh.l.w);
                w.best.srf = __float_as_int(hh.h.w);
                w.best.side = bits & 1;
                w.fault = (int)((unsigned)bits >> 8);
                w.best.hit[0] = hh.h.x; w.best.hit[1] = hh.h.y; w.best.hit[2] = hh.h.z;
                w.best.loc[0] = hh.l.x; w.best.loc[1] = hh.l.y; w.best.loc[2] = hh.l.z;
            }
            WNode &N = pool[base + i];
            if (w.fault)
            {
                int x, y;
                tile_pixel(tp, (P.x_res + 7) / 8, x, y);
                note_fault(S, w.fault, x, y);
                w.best.srf = -1;
            }
            if (w.best.srf < 0)
            {
                N.f = make_float4(0.0f, __int_as_float(0), __int_as_float(owner), 0.0f);
            }
            else
            {
                const Hit h = w.best;
                PtPend pp;
                dif = pt_begin(S, P, r, h, pp, ks, code, ddir, NULL);
                const int bits = pt_bits(pp);
                trn = (bits & PT_TRN) != 0;
                rfl = (bits & PT_RFL) != 0;
                const int spawn = r.depth != 0;
                side = h.side;
                srf = h.srf;
                depth = r.depth;
                #pragma unroll
                for (int k = 0; k < 3; k++) { hit[k] = h.hit[k]; loc[k] = h.loc[k]; }
                if (spawn && trn) { nw[0] = pp.n.x; nw[1] = pp.n.y; nw[2] = pp.n.z; }
                if (spawn && rfl) { rw[0] = pp.m.x; rw[1] = pp.m.y; rw[2] = pp.m.z; }
                /* the node: pt_begin's fields, repacked */
                if (dif) N.t = pp.a;
                N.e = make_float4(dif ? pp.b.x : pp.a.x, dif ? pp.b.y : pp.a.y,
                                  dif ? pp.b.z : pp.a.z, (dif || trn) ? pp.b.w : 0.0f);
                N.f = make_float4(rfl ? pp.h.w : 0.0f,
                                  __int_as_float(WN_HIT | (dif ? WN_DIF : 0) |
                                                 (trn ? WN_TRN : 0) | (rfl ? WN_RFL : 0) |
                                                 (spawn ? WN_SPAWN : 0)),
                                  __int_as_float(owner), 0.0f);
                nch = dif + (spawn && trn) + (spawn && rfl);
                trn = spawn && trn;
                rfl = spawn && rfl;
            }
        }
        int tot;
        const int ex = warp_excl_scan(nch, &tot);
        int qb = warp_reserve(&ctl->cnt[d + 1], tot);
        /* the children of level d + 1 take pool nodes base + n + [0, cnt) */
        if (qb + tot > cap_q || base + n + qb + tot > cap_pool)
        {
            if (lane == 0 && tot > 0) atomicExch(&ctl->overflow, 1);
            continue;
        }
        if (nch == 0) continue;
        const qr_srf *__restrict__ s = &S.srf[srf];
        int at = qb + ex;
        const int node = base + i;
        const float fmax = FLT_MAX;
        if (dif)
        {
            put_ray(qout, at++, hit, 0.0f, ddir, fmax, loc, srf, side, depth - 1,
                    owner_of(node, 0), 3u * code + 1u, __ldg(&s->sec_off[side]),
                    __ldg(&s->sec_num[side]), ks, tp);
        }
        if (trn)
        {
            put_ray(qout, at++, hit, 0.0f, nw, fmax, loc, srf, side | FLAG_PASS, depth - 1,
                    owner_of(node, 1), 3u * code + 2u, __ldg(&s->sec_off[1 - side]),
                    __ldg(&s->sec_num[1 - side]), ks, tp);
        }
        if (rfl)
        {
            put_ray(qout, at++, hit, 0.0f, rw, fmax, loc, srf, side, depth - 1,
                    owner_of(node, 2), 3u * code + 3u, __ldg(&s->sec_off[side]),
                    __ldg(&s->sec_num[side]), ks, tp);
        }
    }
}

/* level d, deepest first: the node's colour to its owner */
__global__ void __launch_bounds__(128)
wf_fold(int d, WNode *pool, float4 *samples, const WCtl *ctl)
{
    if (ctl->overflow) return;
    const int n = ctl->cnt[d];
    const int base = d == 0 ? 0 : ctl->off[d];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const WNode &N = pool[base + i];
        const float4 f = N.f;
        const int bits = __float_as_int(f.y), owner = __float_as_int(f.z);
        float c[3] = {0.0f, 0.0f, 0.0f};
        if (bits & WN_HIT)
        {
            const float4 e = N.e;
            if (bits & WN_DIF)
            {
                const float4 t = N.t, cl = N.cl;
                float v;
                v = cl.x * t.w; c[0] = v * t.x;
                v = cl.y * t.w; c[1] = v * t.y;
                v = cl.z * t.w; c[2] = v * t.z;
            }
            c[0] = c[0] + e.x;
            c[1] = c[1] + e.y;
            c[2] = c[2] + e.z;
            if (bits & WN_TRN)
            {
                float tc[3] = {0.0f, 0.0f, 0.0f};
                if (bits & WN_SPAWN)
                {
                    const float4 ct = N.ct;
                    tc[0] = ct.x * e.w; tc[1] = ct.y * e.w; tc[2] = ct.z * e.w;
                }
                c[0] = tc[0] + c[0]; c[1] = tc[1] + c[1]; c[2] = tc[2] + c[2];
            }
            if (bits & WN_RFL)
            {
                float rc[3] = {0.0f, 0.0f, 0.0f};
                if (bits & WN_SPAWN)
                {
                    const float4 cr = N.cr;
                    rc[0] = cr.x * f.x; rc[1] = cr.y * f.x; rc[2] = cr.z * f.x;
                }
                c[0] = rc[0] + c[0]; c[1] = rc[1] + c[1]; c[2] = rc[2] + c[2];
            }
        }
        const float4 cv = make_float4(c[0], c[1], c[2], 0.0f);
        if (d == 0)
        {
            samples[owner] = cv;
        }
        else
        {
            WNode &Pn = pool[owner >> 2];
            const int slot = owner & 3;
            if (slot == 0) Pn.cl = cv;
            else if (slot == 1) Pn.ct = cv;
            else Pn.cr = cv;
        }
    }
}

/* each pixel adds its samples of paths [c0, c1) in sample order */
__global__ void __launch_bounds__(128)
wf_accum(const qr_frame_params P, long long c0, long long c1, int ppad, int tx,
         const float4 *__restrict__ samples, float4 *sums, const WCtl *ctl)
{
    if (ctl->overflow) return;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ppad; t += gridDim.x * blockDim.x)
    {
        int x, y;
        tile_pixel(t, tx, x, y);
        if (x >= P.x_res || y >= P.y_res) continue;
        /* samples s with c0 <= s * ppad + t < c1 */
        long long s0 = c0 - t <= 0 ? 0 : (c0 - t + ppad - 1) / ppad;
        const size_t px = (size_t)y * P.x_res + x;
        float4 a = sums[px];
        int any = 0;
        for (long long s = s0; s * ppad + t < c1; s++)
        {
            const float4 v = samples[s * ppad + t - c0];
            a.x = a.x + v.x;
            a.y = a.y + v.y;
            a.z = a.z + v.z;
            any = 1;
        }
        if (any) sums[px] = a;
    }
}

/* the running sums and the frame (pt_pixel_seq's end) */
__global__ void __launch_bounds__(128)
wf_final(const qr_frame_params P, const float4 *__restrict__ sums, float *acc,
         uint32_t *frame, const WCtl *ctl)
{
    if (ctl->overflow) return;
    const int npx = P.x_res * P.y_res;
    const int n0 = (int)P.pts_c, spp = P.pt_on;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npx; i += gridDim.x * blockDim.x)
    {
        const int y = i / P.x_res, x = i - y * P.x_res;
        const float4 sv = sums[i];
        const float sum[3] = {sv.x, sv.y, sv.z};
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
}

/* the whole frame by the per-pixel kernel's path, when a queue overflowed */
__global__ void __launch_bounds__(128, QR_PT_MIN_BLOCKS)
wf_fallback(const qr_dscene S, const qr_frame_params P, float *acc, uint32_t *frame,
            const WCtl *ctl)
{
    if (!ctl->overflow) return;
    const int x = tile_x(), y = tile_y();
    if (x >= P.x_res || y >= P.y_res) return;
    pt_pixel_seq(S, P, x, y, acc, frame, NULL);
}

} /* namespace qr_dev */

using namespace qr_dev;

/* resident blocks a SM of the shading and tracing stages (queried once;
 * the value is the same whichever thread stores it) */
static std::atomic<int> g_step_per_sm(0), g_trace_per_sm(0);

int qr_wf_prepare(void)
{
    if (g_step_per_sm.load(std::memory_order_acquire) == 0)
    {
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, wf_step, 128, 0) != cudaSuccess ||
            nb <= 0)
            nb = QR_WF_MIN_BLOCKS;
        int nt = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nt, wf_trace, 128, 0) != cudaSuccess ||
            nt <= 0)
            nt = QR_WF_TRACE_MIN_BLOCKS;
        g_trace_per_sm.store(nt, std::memory_order_relaxed);
        g_step_per_sm.store(nb, std::memory_order_release);
    }
    return g_step_per_sm.load(std::memory_order_acquire);
}

/* a batched request's completion word, once the frame before it on the
 * stream is in device memory */
__global__ void wf_mark_done(uint32_t *done, int req)
{
    __threadfence_system();
    *(volatile uint32_t *)&done[req] = 1u;
}

cudaError_t qr_wf_mark_done(uint32_t *done, int req, cudaStream_t stream)
{
    wf_mark_done<<<1, 1, 0, stream>>>(done, req);
    qr_note_launches(stream, 1);
    return cudaGetLastError();
}

size_t qr_wf_bytes(const qr_wf_caps &c)
{
    return sizeof(WCtl) + 2 * (size_t)c.cap_q * sizeof(WRay) +
           (size_t)c.cap_q * sizeof(WHit) + 256 +
           (size_t)c.cap_pool * sizeof(WNode) + (size_t)c.cap_paths * sizeof(float4) +
           (size_t)c.cap_px * sizeof(float4) + 5 * 256;
}

qr_wf_caps qr_wf_caps_for(const qr_frame_params &fp, long long max_paths, int q_per_path,
                          int pool_per_path)
{
    qr_wf_caps c;
    const int tx = (fp.x_res + 7) / 8, ty = (fp.y_res + 3) / 4;
    const long long ppad = (long long)tx * ty * 32;
    long long paths = ppad * (long long)fp.pt_on;
    if (paths > max_paths) paths = max_paths;
    if (paths < 32) paths = 32;
    c.cap_paths = paths;
    c.cap_q = (long long)q_per_path * paths;
    c.cap_pool = (long long)pool_per_path * paths;
    if (c.cap_q < paths) c.cap_q = paths;
    if (c.cap_pool < paths) c.cap_pool = paths;
    c.cap_px = (long long)fp.x_res * fp.y_res;
    return c;
}

static inline size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

/* the stages' arrays in a scratch block */
struct WPipe
{
    WCtl   *ctl;
    WRay   *qa, *qb;
    WHit   *hits;
    WNode  *pool;
    float4 *samples, *sums;
};

static WPipe carve(void *scratch, const qr_wf_caps &caps)
{
    WPipe p;
    unsigned char *b = (unsigned char *)scratch;
    p.ctl = (WCtl *)b;
    b += al256(sizeof(WCtl));
    p.qa = (WRay *)b;
    b += al256((size_t)caps.cap_q * sizeof(WRay));
    p.qb = (WRay *)b;
    b += al256((size_t)caps.cap_q * sizeof(WRay));
    p.hits = (WHit *)b;
    b += al256((size_t)caps.cap_q * sizeof(WHit));
    p.pool = (WNode *)b;
    b += al256((size_t)caps.cap_pool * sizeof(WNode));
    p.samples = (float4 *)b;
    b += al256((size_t)caps.cap_paths * sizeof(float4));
    p.sums = (float4 *)b;
    return p;
}

/* the second pipeline's overflow word into the first's */
__global__ void wf_merge(WCtl *a, const WCtl *b)
{
    if (b->overflow) a->overflow = 1;
}

cudaError_t qr_wf_launch_pt(const qr_dscene &sc, const qr_frame_params &fp, float *acc,
                            uint32_t *frame, void *scratch, const qr_wf_caps &caps,
                            int sms, cudaStream_t stream, const qr_wf_second *second)
{
    const int tx = (fp.x_res + 7) / 8, ty = (fp.y_res + 3) / 4;
    const int ppad = tx * ty * 32;
    const long long total = (long long)ppad * fp.pt_on;
    const long long nchunks = (total + caps.cap_paths - 1) / caps.cap_paths;
    const int levels = fp.depth + 1;
    /* two pipelines only when there are two chunks to overlap */
    const int np = second != NULL && nchunks >= 2 ? 2 : 1;
    WPipe P[2];
    P[0] = carve(scratch, caps);
    P[1] = np == 2 ? carve(second->scratch, caps) : P[0];
    cudaStream_t st[2] = {stream, np == 2 ? second->stream : stream};
    float4 *sums = P[0].sums;
    /* every kernel strides over its level: as many blocks as are resident */
    const int step_per_sm = qr_wf_prepare();
    const int blocks = sms * 8;             /* memory-bound stages: 8 blocks of 128 a SM */
    const int sblocks = sms * step_per_sm;
    /* the tracing stage fills its own resident slots (7 blocks a SM against
     * the shading stage's 6): the 720p 64-spp frame 118.1 against 121.8 ms
     * with the shading stage's grid */
    const int tblocks = sms * g_trace_per_sm.load(std::memory_order_relaxed);
    cudaError_t e = cudaMemsetAsync(P[0].ctl, 0, sizeof(WCtl), stream);
    if (e == cudaSuccess && np == 2) e = cudaMemsetAsync(P[1].ctl, 0, sizeof(WCtl), stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(sums, 0, (size_t)fp.x_res * fp.y_res * sizeof(float4), stream);
    if (e == cudaSuccess && np == 2) e = cudaEventRecord(second->ev[0], stream);
    if (e == cudaSuccess && np == 2) e = cudaStreamWaitEvent(st[1], second->ev[0], 0);
    long long c = 0;
    for (long long c0 = 0; c0 < total && e == cudaSuccess; c0 += caps.cap_paths, c++)
    {
        const int p = (int)(c % np);
        const WPipe &W = P[p];
        cudaStream_t s = st[p];
        const long long c1 = c0 + caps.cap_paths < total ? c0 + caps.cap_paths : total;
        /* counts of this chunk (the overflow word stays) */
        e = cudaMemsetAsync(W.ctl, 0, offsetof(WCtl, overflow), s);   /* cnt, off, next */
        if (e != cudaSuccess) break;
        wf_gen<<<blocks, 128, 0, s>>>(fp, c0, c1, ppad, tx, W.qa, W.ctl);
        for (int d = 0; d < levels; d++)
        {
            WRay *qi = (d & 1) ? W.qb : W.qa, *qo = (d & 1) ? W.qa : W.qb;
            wf_trace<<<tblocks, 128, 0, s>>>(sc, fp, d, qi, W.hits, W.ctl);
            wf_step<<<sblocks, 128, 0, s>>>(sc, fp, d, qi, W.hits, qo, W.pool, W.ctl,
                                            (int)caps.cap_q, (int)caps.cap_pool);
        }
        for (int d = levels - 1; d >= 0; d--)
            wf_fold<<<blocks, 128, 0, s>>>(d, W.pool, W.samples, W.ctl);
        /* the chunk's samples join the sums after the chunk before it's */
        if (np == 2 && c >= 1) e = cudaStreamWaitEvent(s, second->ev[1 + (1 - p)], 0);
        if (e != cudaSuccess) break;
        wf_accum<<<blocks, 128, 0, s>>>(fp, c0, c1, ppad, tx, W.samples, sums, W.ctl);
        if (np == 2) e = cudaEventRecord(second->ev[1 + p], s);
        qr_note_launches(s, 2 + 3 * levels);
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    if (e == cudaSuccess && np == 2)
    {
        /* the second stream's last chunk, then its overflow word */
        e = cudaStreamWaitEvent(stream, second->ev[2], 0);
        if (e == cudaSuccess)
        {
            wf_merge<<<1, 1, 0, stream>>>(P[0].ctl, P[1].ctl);
            qr_note_launches(stream, 1);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess)
    {
        WCtl *ctl = P[0].ctl;
        wf_final<<<blocks, 128, 0, stream>>>(fp, sums, acc, frame, ctl);
        const dim3 block(32, 4);
        const dim3 grid((fp.x_res + 2 * QR_TILE_W - 1) / (2 * QR_TILE_W),
                        (fp.y_res + 2 * QR_TILE_H - 1) / (2 * QR_TILE_H));
        wf_fallback<<<grid, block, 0, stream>>>(sc, fp, acc, frame, ctl);
        qr_note_launches(stream, 2);
        e = cudaGetLastError();
    }
    return e;
}

int qr_wf_overflowed(const void *scratch, cudaStream_t stream, int *out)
{
    const WCtl *ctl = (const WCtl *)scratch;
    cudaError_t e = cudaMemcpyAsync(out, &ctl->overflow, sizeof(int), cudaMemcpyDeviceToHost,
                                    stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    return e == cudaSuccess ? 0 : -1;
}

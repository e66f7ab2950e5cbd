/*
 * wf_common.cuh: queues of the wavefront stages (wavefront.cu, the path
 * tracer; whitted_wf.cu, the Whitted tracer): the queued ray record, the
 * per-frame control block, warp-scan compaction of appends and the pixel
 * tile order.
 */
#ifndef QR_WF_COMMON_CUH
#define QR_WF_COMMON_CUH

#include "tracer_dev.cuh"

namespace qr_dev
{

/* a queued ray, 80 bytes */
struct WRay
{
    float4 o;       /* origin, t_min */
    float4 d;       /* direction, t_max */
    float4 p;       /* originating surface's local hit, surface (int bits) */
    int4   m;       /* flags | depth << 8, owner, tree code, list offset */
    int4   k;       /* sample key (low, high), list length, pixel tile place */
};

/* owners: level-0 rays own a sample slot of the chunk; deeper rays own a
 * child slot of a node in the pool (path tracer: 0 diffuse, 1 refracted,
 * 2 reflected; Whitted: 1 refracted, 2 reflected) */
__device__ __forceinline__ int owner_of(int node, int slot) { return (node << 2) | slot; }

/* the device-side control block of a frame */
struct WCtl
{
    int cnt[QR_MAX_DEPTH + 2];      /* rays of each level in this chunk */
    int off[QR_MAX_DEPTH + 2];      /* first pool node of each level */
    int next[QR_MAX_DEPTH + 2];     /* rays of each level handed to warps */
    int tnext[QR_MAX_DEPTH + 2];    /* the same for the tracing stage */
    int overflow;                   /* a queue or the pool ran full */
    int pad[3];
};

/* exclusive warp scan of small counts; returns the warp's total in *tot */
__device__ __forceinline__ int warp_excl_scan(int v, int *tot)
{
    const int lane = threadIdx.x & 31;
    int x = v;
    #pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    *tot = __shfl_sync(0xFFFFFFFFu, x, 31);
    return x - v;
}

/* reserve the warp's run of `total` entries in a queue counter */
__device__ __forceinline__ int warp_reserve(int *counter, int total)
{
    int base = 0;
    if ((threadIdx.x & 31) == 0 && total > 0) base = atomicAdd(counter, total);
    return __shfl_sync(0xFFFFFFFFu, base, 0);
}

__device__ __forceinline__ void put_ray(WRay *q, int i, const float org[3], float t_min,
                                        const float dir[3], float t_max, const float phit[3],
                                        int from, int flags, int depth, int owner,
                                        uint32_t code, int off, int num,
                                        unsigned long long ks, int tp)
{
    WRay r;
    r.o = make_float4(org[0], org[1], org[2], t_min);
    r.d = make_float4(dir[0], dir[1], dir[2], t_max);
    r.p = make_float4(phit[0], phit[1], phit[2], __int_as_float(from));
    r.m = make_int4(flags | (depth << 8), owner, (int)code, off);
    r.k = make_int4((int)(uint32_t)ks, (int)(uint32_t)(ks >> 32), num, tp);
    q[i] = r;
}

/* pixel of tile place t: tiles of 8 x 4 pixels, tile rows of tx tiles */
__device__ __forceinline__ void tile_pixel(int t, int tx, int &x, int &y)
{
    const int tile = t >> 5, in = t & 31;
    x = (tile % tx) * 8 + (in & 7);
    y = (tile / tx) * 4 + (in >> 3);
}

/* the queued ray as the walk takes it; returns its owner */
__device__ __forceinline__ int get_ray(const WRay &q, const qr_dscene &S, Ray &r, int &off,
                                       int &num)
{
    r.org[0] = q.o.x; r.org[1] = q.o.y; r.org[2] = q.o.z; r.t_min = q.o.w;
    r.dir[0] = q.d.x; r.dir[1] = q.d.y; r.dir[2] = q.d.z; r.t_max = q.d.w;
    r.phit[0] = q.p.x; r.phit[1] = q.p.y; r.phit[2] = q.p.z;
    r.from = __float_as_int(q.p.w);
    r.flags = q.m.x & 255;
    r.depth = q.m.x >> 8;
    off = q.m.w >= 0 ? q.m.w : S.cam_off;
    num = q.m.w >= 0 ? q.k.z : S.cam_num;
    return q.m.y;
}

/* a fresh walk state: nearest hit, or any occluder */
__device__ __forceinline__ void walk_init(Walk &w, const Ray &r, int shadow)
{
    w.fault = 0;
    w.shadow = shadow;
    w.occluded = 0;
    w.tbuf = r.t_max;
    w.bestp = -1;
    w.best.srf = -1;
}

} /* namespace qr_dev */

#endif /* QR_WF_COMMON_CUH */

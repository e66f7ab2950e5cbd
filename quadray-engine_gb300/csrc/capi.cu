/*
 * capi.cu: C ABI of the GB300 render backend (include/qr_gpu.h).
 *
 * A context owns device-resident scenes (flattened records copied once and
 * replaced in place on update) and a device frame buffer for host renders.
 * Every entry point returns a status code and never throws; CUDA errors are
 * kept in the context's message buffer.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <atomic>
#include <mutex>
#include <new>
#include <vector>

#include "qr_gpu.h"
#include "tracer.cuh"
#include "accel.h"
#include "anim.cuh"
#include "wavefront.h"
#include "whitted_wf.h"


/* device update of an animated scene (qr_scene_anim_*) */
#define QR_ANIM_RING 4          /* parameter / launch sets in turn */
struct qr_anim_state
{
    int          ok;        /* prepared for the scene's current upload */
    void        *block;     /* device: table, matrices, terms, boxes, order */
    size_t       bytes;
    qr_anim_param *ring;    /* mapped host memory: QR_ANIM_RING param sets */
    size_t       ring_n;    /* params a set holds */
    cudaEvent_t  ev[QR_ANIM_RING];  /* the update that last read each set */
    int          next;
    int          nparams;
    qr_anim_dev  dev;
};

struct qr_scene_slot
{
    int          used;
    void        *block;     /* one device allocation for all arrays */
    size_t       bytes;
    qr_dscene    d;
    qr_scene_desc shape;    /* sizes of the uploaded arrays */
    qr_anim_state *anim;    /* NULL until qr_scene_anim_init */
    int          max_lnum;  /* longest per-side light list */
};

static void anim_free(qr_anim_state *a)
{
    if (a == NULL) return;
    if (a->block) cudaFree(a->block);
    if (a->ring) cudaFreeHost(a->ring);
    for (int k = 0; k < QR_ANIM_RING; k++)
        if (a->ev[k]) cudaEventDestroy(a->ev[k]);
    delete a;
}

struct qr_ctx
{
    int          device;
    char         err[256];
    /* scene table: slots live on the heap (their addresses stay valid),
     * the table and the error text are guarded by mu so that scenes can be
     * uploaded and updated from several host threads */
    std::vector<qr_scene_slot *> scenes;
    std::mutex   mu;
    uint32_t    *dframe;    /* frame buffer for qr_render_host */
    size_t       dframe_px;
    float       *dacc;      /* path-tracer running sums (3 floats a pixel) */
    size_t       dacc_px;
    uint32_t    *dfault;    /* fault word of the context's scenes (qr_fault) */
    cudaStream_t stream;
    /* scene updates (qr_scene_anim_update_many): per launch a set of
     * qr_anim_dev in mapped host memory, QR_ANIM_RING sets in turn, each
     * reused once the launch that read it has run */
    std::mutex   amu;
    qr_anim_dev *adevs;
    size_t       adevs_n;
    cudaEvent_t  aev[4];
    int          anext;
    /* scratch of the wavefront path tracer (queues, node pool, sample and
     * pixel sums), grown as frames need; one frame at a time uses it: a
     * frame on another stream waits for the last one (wf_ev) */
    std::mutex   wfmu;
    void        *wf;
    size_t       wf_bytes;
    cudaEvent_t  wf_ev;
    cudaStream_t wf_last;
    /* the path tracer's second chunk in flight: its scratch, stream and
     * events (without the scratch, chunks run one at a time) */
    void        *wf2;
    size_t       wf2_bytes;
    cudaStream_t wf_side;
    cudaEvent_t  wf_sev[3];
    int          sms;
    long long    wf_paths;      /* paths of a chunk at most */
    int          wf_q, wf_pool; /* queue rays, pool nodes a path */
    long long    wh_samples;    /* Whitted: camera rays of a chunk at most */
};

/* the wavefront's chunks: 2^22 paths, queues of 2 rays and a pool of 8
 * nodes a path: about 1.2 KB a path, 4.9 GB.  Fewer, larger chunks leave
 * fewer stage tails: the 1280x720 64-spp frame takes 183.9 / 169.6 / 162.9
 * / 161.9 ms at 2^20 / 2^21 / 2^22 / 2^23 paths.  QR_WF_CAPS="paths,q,pool"
 * in the environment of the process (read when a context is created) sets
 * other capacities (tests use small ones to exercise chunks and the
 * overflow path) */
#define QR_WF_MAX_PATHS (4ll << 20)
/* Whitted chunks: 2^21 camera rays (about 1.3 KB a ray with four lights,
 * 2.7 GB); QR_WH_SAMPLES in the environment sets another number */
#define QR_WH_MAX_SAMPLES (2ll << 20)
#define QR_WF_Q_PER_PATH 2
#define QR_WF_POOL_PER_PATH 8

/* kernels the library has launched (graph launches count their kernels) */
static std::atomic<unsigned long long> g_launches(0);

void qr_note_launches(cudaStream_t stream, int n)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
        return;
    g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed);
}

extern "C" unsigned long long qr_kernel_launches(void)
{
    return g_launches.load(std::memory_order_relaxed);
}

static int fail(qr_ctx *ctx, int code, const char *what, cudaError_t e)
{
    if (ctx != NULL)
    {
        std::lock_guard<std::mutex> lock(ctx->mu);
        snprintf(ctx->err, sizeof(ctx->err), "%s: %s", what,
                 e == cudaSuccess ? "error" : cudaGetErrorString(e));
    }
    return code;
}

extern "C" int qr_ctx_create(int device, qr_ctx **out)
{
    if (out == NULL) return QR_ERR_ARG;
    *out = NULL;
    qr_ctx *ctx = new (std::nothrow) qr_ctx();
    if (ctx == NULL) return QR_ERR_OOM;
    ctx->device = device;
    ctx->err[0] = 0;
    ctx->dframe = NULL;
    ctx->dframe_px = 0;
    ctx->dacc = NULL;
    ctx->dacc_px = 0;
    ctx->dfault = NULL;
    ctx->stream = 0;
    ctx->adevs = NULL;
    ctx->adevs_n = 0;
    ctx->anext = 0;
    for (int k = 0; k < 4; k++) ctx->aev[k] = NULL;
    ctx->wf = NULL;
    ctx->wf_bytes = 0;
    ctx->wf_ev = NULL;
    ctx->wf_last = 0;
    ctx->wf2 = NULL;
    ctx->wf2_bytes = 0;
    ctx->wf_side = NULL;
    for (int k = 0; k < 3; k++) ctx->wf_sev[k] = NULL;
    ctx->sms = 0;
    ctx->wf_paths = QR_WF_MAX_PATHS;
    ctx->wf_q = QR_WF_Q_PER_PATH;
    ctx->wf_pool = QR_WF_POOL_PER_PATH;
    ctx->wh_samples = QR_WH_MAX_SAMPLES;
    {
        const char *ev = getenv("QR_WH_SAMPLES");
        long long a = ev != NULL ? atoll(ev) : 0;
        if (a >= 128 && a <= (1ll << 24)) ctx->wh_samples = a;
    }
    {
        const char *ev = getenv("QR_WF_CAPS");
        long long a = 0;
        int b = 0, c = 0;
        if (ev != NULL && sscanf(ev, "%lld,%d,%d", &a, &b, &c) == 3 && a >= 32 &&
            a <= (1ll << 24) && b >= 1 && b <= 16 && c >= 1 && c <= 64 &&
            a * c <= (1ll << 28))         /* pool nodes << 2 stay in an int */
        {
            ctx->wf_paths = a;
            ctx->wf_q = b;
            ctx->wf_pool = c;
        }
    }
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount,
                                                     device);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->wf_ev, cudaEventDisableTiming);
    for (int k = 0; k < 3 && e == cudaSuccess; k++)
        e = cudaEventCreateWithFlags(&ctx->wf_sev[k], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->wf_side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->dfault, 4 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->dfault, 0, 4 * sizeof(uint32_t), ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess)
    {
        fprintf(stderr, "qr_ctx_create: %s\n", cudaGetErrorString(e));
        if (ctx->dfault) cudaFree(ctx->dfault);
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        if (ctx->wf_side) cudaStreamDestroy(ctx->wf_side);
        if (ctx->wf_ev) cudaEventDestroy(ctx->wf_ev);
        for (int k = 0; k < 3; k++)
            if (ctx->wf_sev[k]) cudaEventDestroy(ctx->wf_sev[k]);
        delete ctx;
        return QR_ERR_CUDA;
    }
    *out = ctx;
    return QR_OK;
}

extern "C" int qr_ctx_destroy(qr_ctx *ctx)
{
    if (ctx == NULL) return QR_ERR_ARG;
    cudaSetDevice(ctx->device);
    for (size_t i = 0; i < ctx->scenes.size(); i++)
    {
        if (ctx->scenes[i] != NULL)
        {
            cudaFree(ctx->scenes[i]->block);
            anim_free(ctx->scenes[i]->anim);
            delete ctx->scenes[i];
        }
    }
    if (ctx->dframe) cudaFree(ctx->dframe);
    if (ctx->dacc) cudaFree(ctx->dacc);
    if (ctx->dfault) cudaFree(ctx->dfault);
    if (ctx->adevs) cudaFreeHost(ctx->adevs);
    for (int k = 0; k < 4; k++)
        if (ctx->aev[k]) cudaEventDestroy(ctx->aev[k]);
    if (ctx->wf) cudaFree(ctx->wf);
    if (ctx->wf2) cudaFree(ctx->wf2);
    if (ctx->wf_ev) cudaEventDestroy(ctx->wf_ev);
    for (int k = 0; k < 3; k++)
        if (ctx->wf_sev[k]) cudaEventDestroy(ctx->wf_sev[k]);
    if (ctx->wf_side) cudaStreamDestroy(ctx->wf_side);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return QR_OK;
}

extern "C" const char *qr_last_error(qr_ctx *ctx)
{
    return ctx == NULL ? "null context" : ctx->err;
}

static size_t al16(size_t n) { return (n + 255) & ~(size_t)255; }

static int check_desc(const qr_scene_desc *d)
{
    if (d == NULL) return QR_ERR_ARG;
    if (d->nsrf < 0 || d->nmat < 0 || d->nlgt < 0 || d->nelem < 0 ||
        d->nlelem < 0 || d->ntex < 0) return QR_ERR_ARG;
    if ((d->nsrf && !d->srf) || (d->nmat && !d->mat) || (d->nlgt && !d->lgt) ||
        (d->nelem && !d->elems) || (d->nlelem && !d->lelems) ||
        (d->ntex && !d->texels)) return QR_ERR_ARG;
    if (d->cam_off < 0 || d->cam_num < 0 || d->cam_off + d->cam_num > d->nelem)
        return QR_ERR_ARG;
    /* every index the kernel follows must stay in bounds */
    for (int i = 0; i < d->nelem; i++)
    {
        const qr_elem &e = d->elems[i];
        if (e.kind == QR_ELM_SURFACE || e.kind == QR_ELM_TRNODE)
        {
            if (e.ref < 0 || e.ref >= d->nsrf) return QR_ERR_ARG;
        }
        else if (e.kind != QR_ELM_ACC_ENTER && e.kind != QR_ELM_ACC_LEAVE)
        {
            return QR_ERR_ARG;
        }
    }
    for (int i = 0; i < d->nsrf; i++)
    {
        const qr_srf &s = d->srf[i];
        if (s.is_node) continue;
        for (int k = 0; k < 2; k++)
        {
            if (s.mat[k] < 0 || s.mat[k] >= d->nmat) return QR_ERR_ARG;
            if (s.lgt_off[k] < 0 || s.lgt_off[k] + s.lgt_num[k] > d->nlelem) return QR_ERR_ARG;
            if (s.sec_off[k] < 0 || s.sec_off[k] + s.sec_num[k] > d->nelem) return QR_ERR_ARG;
        }
        if (s.clip_off < 0 || s.clip_off + s.clip_num > d->nelem) return QR_ERR_ARG;
        if (s.trnode >= d->nsrf) return QR_ERR_ARG;
        for (int k = 0; k < 3; k++)
            if (s.amap[k] < 0 || s.amap[k] > 2) return QR_ERR_ARG;
    }
    for (int i = 0; i < d->nlelem; i++)
    {
        const qr_lelem &l = d->lelems[i];
        if (l.light < 0 || l.light >= d->nlgt) return QR_ERR_ARG;
        if (l.shd_off < 0 || l.shd_off + l.shd_num > d->nelem) return QR_ERR_ARG;
    }
    for (int i = 0; i < d->nmat; i++)
    {
        const qr_mat &m = d->mat[i];
        if (m.tex_off < 0 || m.tex_off >= d->ntex) return QR_ERR_ARG;
        if (m.props & QR_PROP_TEXTURE)
        {
            /* the texel index is (x & xmask) + ((y & ymask) << yshft) */
            if (m.xmask < 0 || m.ymask < 0 || m.yshft < 0 || m.yshft > 30) return QR_ERR_ARG;
            if (m.tmap[0] < 0 || m.tmap[0] > 1 || m.tmap[1] < 0 || m.tmap[1] > 1)
                return QR_ERR_ARG;
            const long long top = (long long)m.xmask + ((long long)m.ymask << m.yshft);
            if ((long long)m.tex_off + top >= (long long)d->ntex) return QR_ERR_ARG;
        }
    }
    return QR_OK;
}

/* the shadow list that every light shares, if it holds the camera list's
 * surfaces in the camera list's order (then the hierarchy serves it) */
static void shadow_list(const qr_scene_desc *d, int *off, int *num)
{
    *off = -1;
    *num = -1;
    if (d->nlelem == 0) return;
    const int so = d->lelems[0].shd_off, sn = d->lelems[0].shd_num;
    for (int i = 1; i < d->nlelem; i++)
        if (d->lelems[i].shd_off != so || d->lelems[i].shd_num != sn) return;
    if (sn != d->cam_num) return;
    for (int e = 0; e < sn; e++)
    {
        const qr_elem &a = d->elems[so + e], &b = d->elems[d->cam_off + e];
        if (a.kind != b.kind || a.ref != b.ref) return;
        if (a.kind == QR_ELM_TRNODE && a.last - so != b.last - d->cam_off) return;
    }
    *off = so;
    *num = sn;
}

/* copy a scene's arrays, and the hierarchy built over them (for the motion
 * bound `bound`, NULL: none), into one device block (or into an existing
 * one); the hierarchy is left in *accp when given */
static int upload(qr_ctx *ctx, qr_scene_slot &sl, const qr_scene_desc *d, bool fresh,
                  const float *bound = NULL, qr_accel_host *accp = NULL)
{
    qr_accel_host acc_local;
    qr_accel_host &acc = accp != NULL ? *accp : acc_local;
    int lvl_root[QR_BVH_LEVELS], lvl_aoff[QR_BVH_LEVELS], lvl_anum[QR_BVH_LEVELS];
    float lvl_r2[QR_BVH_LEVELS];
    qr_accel_build_levels(d, &acc, lvl_root, lvl_aoff, lvl_anum, lvl_r2, bound);
    if (sl.anim != NULL) sl.anim->ok = 0;
    const bool use_bvh = !acc.nodes.empty();
    size_t o_srf = 0;
    size_t o_mat = o_srf + al16(sizeof(qr_srf) * d->nsrf);
    size_t o_lgt = o_mat + al16(sizeof(qr_mat) * d->nmat);
    size_t o_elm = o_lgt + al16(sizeof(qr_light) * d->nlgt);
    size_t o_lel = o_elm + al16(sizeof(qr_elem) * d->nelem);
    size_t o_tex = o_lel + al16(sizeof(qr_lelem) * d->nlelem);
    size_t o_nod = o_tex + al16(sizeof(uint32_t) * d->ntex);
    std::vector<qr_bpair> pairs;
    qr_accel_pairs(acc.nodes, pairs);
    std::vector<qr_bquad> quads;
    std::vector<int32_t> quad_src;
    int32_t lvl_quad[QR_BVH_LEVELS], stack_need[QR_BVH_LEVELS];
    qr_accel_quads(acc.nodes, lvl_root, QR_BVH_LEVELS, quads, quad_src, lvl_quad, stack_need);
    for (int l = 0; l < QR_BVH_LEVELS; l++)
        if (stack_need[l] > QR_BVH_STACK) lvl_r2[l] = -1.0f;   /* that level walks the list */
    size_t o_par = o_nod + al16(sizeof(qr_bnode) * acc.nodes.size());
    size_t o_qud = o_par + al16(sizeof(qr_bpair) * acc.nodes.size());
    size_t o_qsr = o_qud + al16(sizeof(qr_bquad) * quads.size());
    size_t o_itm = o_qsr + al16(sizeof(int32_t) * quad_src.size());
    size_t o_alw = o_itm + al16(sizeof(qr_bitem) * acc.items.size());
    size_t total = o_alw + al16(sizeof(qr_bitem) * acc.always.size());

    std::vector<unsigned char> h(total, 0);
    memcpy(&h[o_srf], d->srf, sizeof(qr_srf) * d->nsrf);
    memcpy(&h[o_mat], d->mat, sizeof(qr_mat) * d->nmat);
    memcpy(&h[o_lgt], d->lgt, sizeof(qr_light) * d->nlgt);
    memcpy(&h[o_elm], d->elems, sizeof(qr_elem) * d->nelem);
    memcpy(&h[o_lel], d->lelems, sizeof(qr_lelem) * d->nlelem);
    memcpy(&h[o_tex], d->texels, sizeof(uint32_t) * d->ntex);
    if (!acc.nodes.empty())
    {
        memcpy(&h[o_nod], acc.nodes.data(), sizeof(qr_bnode) * acc.nodes.size());
        memcpy(&h[o_par], pairs.data(), sizeof(qr_bpair) * pairs.size());
    }
    if (!quads.empty())
    {
        memcpy(&h[o_qud], quads.data(), sizeof(qr_bquad) * quads.size());
        memcpy(&h[o_qsr], quad_src.data(), sizeof(int32_t) * quad_src.size());
    }
    if (!acc.items.empty())
        memcpy(&h[o_itm], acc.items.data(), sizeof(qr_bitem) * acc.items.size());
    if (!acc.always.empty())
        memcpy(&h[o_alw], acc.always.data(), sizeof(qr_bitem) * acc.always.size());

    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "cudaSetDevice", e);
    if (fresh || sl.bytes < total)
    {
        /* a quarter of headroom: the hierarchy of an animated scene changes
         * size from frame to frame, and replacing the block (cudaFree waits
         * for all work on the device) would stall in-place updates */
        const size_t cap = (total + total / 4 + 65535) & ~(size_t)65535;
        if (!fresh && sl.block) cudaFree(sl.block);
        sl.block = NULL;
        e = cudaMalloc(&sl.block, cap);
        if (e != cudaSuccess) return fail(ctx, QR_ERR_OOM, "cudaMalloc scene", e);
        sl.bytes = cap;
    }
    e = cudaMemcpyAsync(sl.block, h.data(), total, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "scene copy", e);

    unsigned char *b = (unsigned char *)sl.block;
    sl.d.srf = (const qr_srf *)(b + o_srf);
    sl.d.mat = (const qr_mat *)(b + o_mat);
    sl.d.lgt = (const qr_light *)(b + o_lgt);
    sl.d.elems = (const qr_elem *)(b + o_elm);
    sl.d.lelems = (const qr_lelem *)(b + o_lel);
    sl.d.texels = (const uint32_t *)(b + o_tex);
    sl.d.nsrf = d->nsrf; sl.d.nmat = d->nmat; sl.d.nlgt = d->nlgt;
    sl.d.nelem = d->nelem; sl.d.nlelem = d->nlelem; sl.d.ntex = d->ntex;
    sl.d.cam_off = d->cam_off;
    sl.d.cam_num = d->cam_num;
    sl.d.nodes = (const qr_bnode *)(b + o_nod);
    sl.d.pairs = (const qr_bpair *)(b + o_par);
    sl.d.quads = (const qr_bquad *)(b + o_qud);
    sl.d.quad_src = (const int32_t *)(b + o_qsr);
    sl.d.nquads = (int32_t)quads.size();
    sl.d.items = (const qr_bitem *)(b + o_itm);
    sl.d.always = (const qr_bitem *)(b + o_alw);
    sl.d.nnodes = use_bvh ? (int32_t)acc.nodes.size() : -1;
    sl.d.nitems = (int32_t)acc.items.size();
    sl.d.nalways = (int32_t)acc.always.size();
    shadow_list(d, &sl.d.shd_off, &sl.d.shd_num);
    for (int k = 0; k < 3; k++) sl.d.ray_c[k] = acc.ray_c[k];
    for (int l = 0; l < QR_BVH_LEVELS; l++)
    {
        sl.d.lvl_root[l] = lvl_root[l];
        sl.d.lvl_quad[l] = lvl_quad[l];
        sl.d.lvl_aoff[l] = lvl_aoff[l];
        sl.d.lvl_anum[l] = lvl_anum[l];
        sl.d.lvl_r2[l] = lvl_r2[l];
    }
    sl.d.fault = ctx->dfault;
    sl.shape = *d;
    sl.max_lnum = 0;
    for (int i = 0; i < d->nsrf; i++)
        for (int k = 0; k < 2; k++)
            sl.max_lnum = std::max(sl.max_lnum, (int)d->srf[i].lgt_num[k]);
    return QR_OK;
}

/* ---- device update of animated scenes ----------------------------------- */

static qr_scene_slot *slot(qr_ctx *ctx, int id);
static int add_slot(qr_ctx *ctx, qr_scene_slot *sl, int *scene_id);

static int check_anim_table(const qr_scene_desc *d, const qr_anim_node *nodes, int n,
                            int *nparams)
{
    if (n < 0 || (n > 0 && nodes == NULL)) return QR_ERR_ARG;
    std::vector<char> rec(d->nsrf, 0), lgt(d->nlgt, 0);
    int np = 0;
    for (int i = 0; i < n; i++)
    {
        const qr_anim_node &N = nodes[i];
        if (N.kind < QR_ANIM_OWN || N.kind > QR_ANIM_NODE) return QR_ERR_ARG;
        if (N.kind == QR_ANIM_OWN ? N.parent != -1 : (N.parent < 0 || N.parent >= i))
            return QR_ERR_ARG;
        /* only records are transform nodes */
        if (N.parent >= 0 && nodes[N.parent].rec < 0) return QR_ERR_ARG;
        if (N.param < -1 || (N.kind == QR_ANIM_NODE && N.param != -1)) return QR_ERR_ARG;
        if (N.rec < -1 || N.rec >= d->nsrf || N.light < -1 || N.light >= d->nlgt)
            return QR_ERR_ARG;
        if (N.rec >= 0)
        {
            if (rec[N.rec]) return QR_ERR_ARG;
            rec[N.rec] = 1;
        }
        if (N.light >= 0)
        {
            if (lgt[N.light]) return QR_ERR_ARG;
            lgt[N.light] = 1;
        }
        if (N.param + 1 > np) np = N.param + 1;
    }
    *nparams = np;
    return QR_OK;
}

static int anim_prepare(qr_ctx *ctx, qr_scene_slot *sl, const qr_scene_desc *desc,
                        const qr_anim_node *nodes, int n, const float *bound);

extern "C" int qr_scene_anim_init(qr_ctx *ctx, int scene_id, const qr_scene_desc *desc,
                                  const qr_anim_node *nodes, int n, const float *bound)
{
    qr_scene_slot *sl = slot(ctx, scene_id);
    if (sl == NULL) return QR_ERR_NOSCENE;
    return anim_prepare(ctx, sl, desc, nodes, n, bound);
}

extern "C" int qr_scene_anim_upload(qr_ctx *ctx, const qr_scene_desc *desc,
                                    const qr_anim_node *nodes, int n, const float *bound,
                                    int *scene_id)
{
    if (ctx == NULL || scene_id == NULL) return QR_ERR_ARG;
    qr_scene_slot *sl = new (std::nothrow) qr_scene_slot();
    if (sl == NULL) return QR_ERR_OOM;
    memset(sl, 0, sizeof(*sl));
    int rc = anim_prepare(ctx, sl, desc, nodes, n, bound);
    if (rc != QR_OK)
    {
        if (sl->block) cudaFree(sl->block);
        anim_free(sl->anim);
        delete sl;
        return rc;
    }
    return add_slot(ctx, sl, scene_id);
}

static int anim_prepare(qr_ctx *ctx, qr_scene_slot *sl, const qr_scene_desc *desc,
                        const qr_anim_node *nodes, int n, const float *bound)
{
    if (ctx == NULL) return QR_ERR_ARG;
    int rc = check_desc(desc);
    if (rc != QR_OK) return rc;
    int nparams = 0;
    rc = check_anim_table(desc, nodes, n, &nparams);
    if (rc != QR_OK) return rc;

    /* the motion bound: given, or where rotations about fixed origins can
     * take the moving records and surfaces */
    float b[6];
    if (bound != NULL)
    {
        for (int k = 0; k < 3; k++)
            if (!(bound[k] <= bound[3 + k]) || !isfinite(bound[k]) || !isfinite(bound[3 + k]))
                return QR_ERR_ARG;
        memcpy(b, bound, sizeof(b));
    }
    else
    {
        qr_accel_rotation_bound(desc, nodes, n, b);
    }

    /* updates of this scene still in flight write its block: they finish
     * before the block is replaced, and no update starts meanwhile */
    std::lock_guard<std::mutex> lock(ctx->amu);
    if (sl->anim != NULL)
    {
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < QR_ANIM_RING && e == cudaSuccess; k++)
            e = cudaEventSynchronize(sl->anim->ev[k]);
        if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "anim wait", e);
    }
    qr_accel_host acc;
    rc = upload(ctx, *sl, desc, false, b, &acc);
    if (rc != QR_OK) return rc;

    /* entries by generation */
    std::vector<int> gen(n, 0);
    int ngen = n > 0 ? 1 : 0;
    for (int i = 0; i < n; i++)
    {
        if (nodes[i].parent >= 0) gen[i] = gen[nodes[i].parent] + 1;
        ngen = std::max(ngen, gen[i] + 1);
    }
    std::vector<int32_t> order, gen_off(ngen + 1, 0);
    for (int g = 0; g < ngen; g++)
    {
        gen_off[g] = (int)order.size();
        for (int i = 0; i < n; i++)
            if (gen[i] == g) order.push_back(i);
    }
    gen_off[ngen] = (int)order.size();

    /* surface boxes that move */
    std::vector<char> dyn(desc->nsrf, 0);
    for (int i = 0; i < n; i++)
        if (nodes[i].rec >= 0) dyn[nodes[i].rec] = 1;
    std::vector<qr_anim_term> terms;
    std::vector<qr_anim_target> targets;
    qr_accel_anim_terms(desc, &acc, b, dyn, terms, targets);

    /* hierarchy nodes by depth, deepest first (nodes are stored parent
     * before children within a level) */
    const int nbvh = sl->d.nnodes > 0 ? sl->d.nnodes : 0;
    std::vector<int> depth(nbvh, 0);
    int maxd = 0;
    for (int i = 0; i < nbvh; i++)
    {
        const qr_bnode &nd = acc.nodes[i];
        if (nd.count == 0)
        {
            depth[nd.a] = depth[i] + 1;
            depth[nd.b] = depth[i] + 1;
            maxd = std::max(maxd, depth[i] + 1);
        }
    }
    std::vector<int32_t> rorder, depth_off;
    for (int dd = nbvh > 0 ? maxd : -1; dd >= 0; dd--)
    {
        depth_off.push_back((int)rorder.size());
        for (int i = 0; i < nbvh; i++)
            if (depth[i] == dd) rorder.push_back(i);
    }
    depth_off.push_back((int)rorder.size());
    /* world-from-local frames of the records (moving ones are redone by
     * every update) */
    std::vector<float> frames((size_t)desc->nsrf * 10, 0.0f);
    for (int i = 0; i < desc->nsrf; i++)
        if (!qr_accel_record_frame(desc->srf[i], &frames[10 * (size_t)i]))
            frames[10 * (size_t)i + 9] = 1.0f;
    std::vector<float> lboxes((size_t)QR_BVH_LEVELS * desc->nsrf * 6, 0.0f);
    for (int l = 0; l < QR_BVH_LEVELS; l++)
        if (acc.lboxes[l].size() == (size_t)desc->nsrf * 6)
            memcpy(&lboxes[(size_t)l * desc->nsrf * 6], acc.lboxes[l].data(),
                   sizeof(float) * 6 * desc->nsrf);

    /* one device block */
    size_t o_nod = 0;
    size_t o_ord = o_nod + al16(sizeof(qr_anim_node) * n);
    size_t o_gof = o_ord + al16(sizeof(int32_t) * order.size());
    size_t o_mtx = o_gof + al16(sizeof(int32_t) * gen_off.size());
    size_t o_trm = o_mtx + al16(sizeof(float) * 16 * n);
    size_t o_tgt = o_trm + al16(sizeof(qr_anim_term) * terms.size());
    size_t o_lbx = o_tgt + al16(sizeof(qr_anim_target) * targets.size());
    size_t o_ror = o_lbx + al16(sizeof(float) * lboxes.size());
    size_t o_dof = o_ror + al16(sizeof(int32_t) * rorder.size());
    size_t o_frm = o_dof + al16(sizeof(int32_t) * depth_off.size());
    size_t o_sta = o_frm + al16(sizeof(float) * frames.size());
    size_t total = o_sta + al16(sizeof(uint32_t) * 2);
    std::vector<unsigned char> h(total, 0);
    if (n) memcpy(&h[o_nod], nodes, sizeof(qr_anim_node) * n);
    if (!order.empty()) memcpy(&h[o_ord], order.data(), sizeof(int32_t) * order.size());
    memcpy(&h[o_gof], gen_off.data(), sizeof(int32_t) * gen_off.size());
    if (!terms.empty()) memcpy(&h[o_trm], terms.data(), sizeof(qr_anim_term) * terms.size());
    if (!targets.empty())
        memcpy(&h[o_tgt], targets.data(), sizeof(qr_anim_target) * targets.size());
    if (!lboxes.empty()) memcpy(&h[o_lbx], lboxes.data(), sizeof(float) * lboxes.size());
    if (!rorder.empty()) memcpy(&h[o_ror], rorder.data(), sizeof(int32_t) * rorder.size());
    memcpy(&h[o_dof], depth_off.data(), sizeof(int32_t) * depth_off.size());
    if (!frames.empty()) memcpy(&h[o_frm], frames.data(), sizeof(float) * frames.size());

    qr_anim_state *a = sl->anim;
    if (a == NULL)
    {
        a = new (std::nothrow) qr_anim_state();
        if (a == NULL) return QR_ERR_OOM;
        memset(a, 0, sizeof(*a));
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < QR_ANIM_RING && e == cudaSuccess; k++)
            e = cudaEventCreateWithFlags(&a->ev[k], cudaEventDisableTiming);
        if (e != cudaSuccess)
        {
            anim_free(a);
            return fail(ctx, QR_ERR_CUDA, "cudaEventCreate", e);
        }
        sl->anim = a;
    }
    a->ok = 0;
    cudaError_t e = cudaSuccess;
    if (a->bytes < total)
    {
        if (a->block) cudaFree(a->block);
        a->block = NULL;
        a->bytes = 0;
        e = cudaMalloc(&a->block, total);
        if (e != cudaSuccess) return fail(ctx, QR_ERR_OOM, "cudaMalloc anim", e);
        a->bytes = total;
    }
    const size_t ring_n = nparams > 0 ? (size_t)nparams : 1;
    if (a->ring_n < ring_n)
    {
        if (a->ring) cudaFreeHost(a->ring);
        a->ring = NULL;
        a->ring_n = 0;
        e = cudaHostAlloc((void **)&a->ring, sizeof(qr_anim_param) * ring_n * QR_ANIM_RING,
                          cudaHostAllocMapped);
        if (e != cudaSuccess) return fail(ctx, QR_ERR_OOM, "cudaHostAlloc anim params", e);
        a->ring_n = ring_n;
    }
    e = cudaMemcpyAsync(a->block, h.data(), total, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "anim copy", e);

    unsigned char *blk = (unsigned char *)a->block;
    qr_anim_dev &D = a->dev;
    D.nodes = (const qr_anim_node *)(blk + o_nod);
    D.order = (const int32_t *)(blk + o_ord);
    D.gen_off = (const int32_t *)(blk + o_gof);
    D.n = n;
    D.ngen = ngen;
    D.params = NULL;
    D.mtx = (float *)(blk + o_mtx);
    D.srf = const_cast<qr_srf *>(sl->d.srf);
    D.lgt = const_cast<qr_light *>(sl->d.lgt);
    D.terms = (const qr_anim_term *)(blk + o_trm);
    D.targets = (const qr_anim_target *)(blk + o_tgt);
    D.ntargets = (int32_t)targets.size();
    D.nsrf = desc->nsrf;
    D.lboxes = (float *)(blk + o_lbx);
    D.bvh = const_cast<qr_bnode *>(sl->d.nodes);
    D.pairs = const_cast<qr_bpair *>(sl->d.pairs);
    D.quads = const_cast<qr_bquad *>(sl->d.quads);
    D.quad_src = sl->d.quad_src;
    D.nquads = sl->d.nquads;
    D.items = sl->d.items;
    D.rorder = (const int32_t *)(blk + o_ror);
    D.depth_off = (const int32_t *)(blk + o_dof);
    D.nbvh = nbvh;
    D.nbands = (int32_t)depth_off.size() - 1;
    for (int l = 0; l < QR_BVH_LEVELS; l++)
        D.lvl_end[l] = l + 1 < QR_BVH_LEVELS ? sl->d.lvl_root[l + 1] : nbvh;
    D.frame = (float *)(blk + o_frm);
    for (int k = 0; k < 3; k++)
    {
        /* rounded inwards: a float box inside it is inside the double one */
        float lo = (float)acc.ext[k], hi = (float)acc.ext[3 + k];
        if ((double)lo < acc.ext[k]) lo = nextafterf(lo, HUGE_VALF);
        if ((double)hi > acc.ext[3 + k]) hi = nextafterf(hi, -HUGE_VALF);
        D.ext[k] = lo;
        D.ext[3 + k] = hi;
    }
    D.status = (uint32_t *)(blk + o_sta);
    a->nparams = nparams;
    a->next = 0;
    a->ok = 1;
    return QR_OK;
}

extern "C" int qr_scene_anim_update_many(qr_ctx *ctx, const qr_anim_request *reqs, int n,
                                         void *stream)
{
    if (ctx == NULL || n < 0 || (n > 0 && reqs == NULL)) return QR_ERR_ARG;
    if (n == 0) return QR_OK;
    std::lock_guard<std::mutex> lock(ctx->amu);
    std::vector<qr_scene_slot *> sls(n);
    for (int i = 0; i < n; i++)
    {
        qr_scene_slot *sl = slot(ctx, reqs[i].scene_id);
        if (sl == NULL) return QR_ERR_NOSCENE;
        const qr_anim_state *a = sl->anim;
        if (a == NULL || !a->ok) return QR_ERR_STATE;
        if (reqs[i].nparams != a->nparams || (a->nparams > 0 && reqs[i].params == NULL))
            return QR_ERR_ARG;
        sls[i] = sl;
    }
    {
        /* two blocks must not update one scene */
        std::vector<qr_scene_slot *> u(sls);
        std::sort(u.begin(), u.end());
        if (std::adjacent_find(u.begin(), u.end()) != u.end()) return QR_ERR_ARG;
    }
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "cudaSetDevice", e);
    for (int k = 0; k < QR_ANIM_RING && e == cudaSuccess; k++)
        if (ctx->aev[k] == NULL) e = cudaEventCreateWithFlags(&ctx->aev[k], cudaEventDisableTiming);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "cudaEventCreate", e);
    if (ctx->adevs_n < (size_t)n)
    {
        for (int k = 0; k < QR_ANIM_RING && e == cudaSuccess; k++) e = cudaEventSynchronize(ctx->aev[k]);
        if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "anim wait", e);
        if (ctx->adevs) cudaFreeHost(ctx->adevs);
        ctx->adevs = NULL;
        ctx->adevs_n = 0;
        const size_t cap = std::max((size_t)n, (size_t)64);
        e = cudaHostAlloc((void **)&ctx->adevs, sizeof(qr_anim_dev) * cap * QR_ANIM_RING,
                          cudaHostAllocMapped);
        if (e != cudaSuccess) return fail(ctx, QR_ERR_OOM, "cudaHostAlloc anim launch", e);
        ctx->adevs_n = cap;
    }
    /* the next launch set, once the launch that last read it has run */
    const int k = ctx->anext;
    ctx->anext = (k + 1) % QR_ANIM_RING;
    e = cudaEventSynchronize(ctx->aev[k]);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "anim ring wait", e);
    qr_anim_dev *set = ctx->adevs + (size_t)k * ctx->adevs_n;
    std::vector<int> used(n);
    for (int i = 0; i < n; i++)
    {
        /* each scene's next parameter set, likewise */
        qr_anim_state *a = sls[i]->anim;
        const int kk = a->next;
        a->next = (kk + 1) % QR_ANIM_RING;
        used[i] = kk;
        e = cudaEventSynchronize(a->ev[kk]);
        if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "anim ring wait", e);
        qr_anim_param *ps = a->ring + (size_t)kk * a->ring_n;
        if (a->nparams > 0) memcpy(ps, reqs[i].params, sizeof(qr_anim_param) * a->nparams);
        qr_anim_param *dps = NULL;
        e = cudaHostGetDevicePointer((void **)&dps, ps, 0);
        if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "cudaHostGetDevicePointer", e);
        set[i] = a->dev;
        set[i].params = dps;
    }
    qr_anim_dev *dset = NULL;
    e = cudaHostGetDevicePointer((void **)&dset, set, 0);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "cudaHostGetDevicePointer", e);
    cudaStream_t st = stream != NULL ? (cudaStream_t)stream : ctx->stream;
    e = qr_launch_anim(dset, n, st);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->aev[k], st);
    for (int i = 0; i < n && e == cudaSuccess; i++)
        e = cudaEventRecord(sls[i]->anim->ev[used[i]], st);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "anim launch", e);
    return QR_OK;
}

extern "C" int qr_scene_anim_update(qr_ctx *ctx, int scene_id, const qr_anim_param *params,
                                    int nparams, void *stream)
{
    qr_anim_request r;
    r.scene_id = scene_id;
    r.nparams = nparams;
    r.params = params;
    return qr_scene_anim_update_many(ctx, &r, 1, stream);
}

extern "C" int qr_scene_anim_status(qr_ctx *ctx, int scene_id, int32_t out[2])
{
    qr_scene_slot *sl = slot(ctx, scene_id);
    if (sl == NULL) return QR_ERR_NOSCENE;
    if (out == NULL) return QR_ERR_ARG;
    qr_anim_state *a = sl->anim;
    if (a == NULL || !a->ok) return QR_ERR_STATE;
    uint32_t st[2];
    cudaError_t e = cudaSetDevice(ctx->device);
    for (int k = 0; k < QR_ANIM_RING && e == cudaSuccess; k++) e = cudaEventSynchronize(a->ev[k]);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(st, a->dev.status, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "anim status", e);
    out[0] = (int32_t)st[0];
    out[1] = (int32_t)st[1];
    return QR_OK;
}

/* enter a filled slot into the context's table */
static int add_slot(qr_ctx *ctx, qr_scene_slot *sl, int *scene_id)
{
    sl->used = 1;
    std::lock_guard<std::mutex> lock(ctx->mu);
    for (size_t i = 0; i < ctx->scenes.size(); i++)
    {
        if (ctx->scenes[i] == NULL)
        {
            ctx->scenes[i] = sl;
            *scene_id = (int)i;
            return QR_OK;
        }
    }
    ctx->scenes.push_back(sl);
    *scene_id = (int)ctx->scenes.size() - 1;
    return QR_OK;
}

extern "C" int qr_scene_upload(qr_ctx *ctx, const qr_scene_desc *desc, int *scene_id)
{
    if (ctx == NULL || scene_id == NULL) return QR_ERR_ARG;
    int rc = check_desc(desc);
    if (rc != QR_OK) return rc;
    qr_scene_slot *sl = new (std::nothrow) qr_scene_slot();
    if (sl == NULL) return QR_ERR_OOM;
    memset(sl, 0, sizeof(*sl));
    rc = upload(ctx, *sl, desc, true);
    if (rc != QR_OK)
    {
        if (sl->block) cudaFree(sl->block);
        delete sl;
        return rc;
    }
    return add_slot(ctx, sl, scene_id);
}

static qr_scene_slot *slot(qr_ctx *ctx, int id)
{
    if (ctx == NULL) return NULL;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (id < 0 || id >= (int)ctx->scenes.size()) return NULL;
    return ctx->scenes[id];
}

extern "C" int qr_scene_update(qr_ctx *ctx, int scene_id, const qr_scene_desc *desc)
{
    qr_scene_slot *sl = slot(ctx, scene_id);
    if (sl == NULL) return QR_ERR_NOSCENE;
    int rc = check_desc(desc);
    if (rc != QR_OK) return rc;
    return upload(ctx, *sl, desc, false);
}

extern "C" int qr_scene_release(qr_ctx *ctx, int scene_id)
{
    if (ctx == NULL) return QR_ERR_ARG;
    qr_scene_slot *sl = NULL;
    {
        std::lock_guard<std::mutex> lock(ctx->mu);
        if (scene_id < 0 || scene_id >= (int)ctx->scenes.size()) return QR_ERR_NOSCENE;
        sl = ctx->scenes[scene_id];
        ctx->scenes[scene_id] = NULL;
    }
    if (sl == NULL) return QR_ERR_NOSCENE;
    cudaSetDevice(ctx->device);
    cudaFree(sl->block);
    anim_free(sl->anim);
    delete sl;
    return QR_OK;
}

static int check_fp(const qr_frame_params *fp)
{
    if (fp == NULL) return QR_ERR_ARG;
    if (fp->x_res <= 0 || fp->y_res <= 0 || fp->x_row < fp->x_res) return QR_ERR_ARG;
    if (fp->x_res > 16384 || fp->y_res > 16384) return QR_ERR_LIMIT;
    if (fp->fsaa < 0 || fp->fsaa > 2) return QR_ERR_ARG;   /* none, 2x, 4x */
    if (fp->depth < 0 || fp->depth > QR_MAX_DEPTH) return QR_ERR_LIMIT;
    if (fp->pt_on < 0 || fp->pt_on > QR_MAX_PT_SAMPLES) return QR_ERR_LIMIT;
    if (!(fp->pts_c >= 0.0f) || fp->pts_c > 16777216.0f) return QR_ERR_ARG;
    return QR_OK;
}

/* the context's path-tracer sums, kept across renders of one frame size */
static int ensure_acc(qr_ctx *ctx, size_t px)
{
    if (ctx->dacc_px >= px) return QR_OK;
    if (ctx->dacc) cudaFree(ctx->dacc);
    ctx->dacc = NULL;
    ctx->dacc_px = 0;
    cudaError_t e = cudaMalloc(&ctx->dacc, px * 3 * sizeof(float));
    if (e != cudaSuccess) return fail(ctx, QR_ERR_OOM, "cudaMalloc path-tracer sums", e);
    ctx->dacc_px = px;
    return QR_OK;
}

/* the context's wavefront scratch, at least `need` bytes (ctx->wfmu held);
 * false when it cannot be had */
static bool wf_scratch(qr_ctx *ctx, size_t need)
{
    if (ctx->wf_bytes >= need) return true;
    /* cudaFree waits for the device: no frame still uses the old block */
    if (ctx->wf) cudaFree(ctx->wf);
    ctx->wf = NULL;
    ctx->wf_bytes = 0;
    if (cudaMalloc(&ctx->wf, need) != cudaSuccess)
    {
        ctx->wf = NULL;
        cudaGetLastError();             /* clear the allocation error */
        return false;
    }
    ctx->wf_bytes = need;
    return true;
}

/* the second chunk's scratch, at least `need` bytes (ctx->wfmu held);
 * false when it cannot be had (chunks then run one at a time) */
static bool wf_scratch2(qr_ctx *ctx, size_t need)
{
    if (ctx->wf2_bytes >= need) return true;
    if (ctx->wf2) cudaFree(ctx->wf2);
    ctx->wf2 = NULL;
    ctx->wf2_bytes = 0;
    if (cudaMalloc(&ctx->wf2, need) != cudaSuccess)
    {
        ctx->wf2 = NULL;
        cudaGetLastError();
        return false;
    }
    ctx->wf2_bytes = need;
    return true;
}

/* a frame on `stream` may use the scratch once the last frame that used it
 * (perhaps on another stream) is done; returns the wait's status */
static cudaError_t wf_begin(qr_ctx *ctx, cudaStream_t stream)
{
    return ctx->wf_last != stream ? cudaStreamWaitEvent(stream, ctx->wf_ev, 0) : cudaSuccess;
}

static cudaError_t wf_end(qr_ctx *ctx, cudaStream_t stream, cudaError_t e)
{
    if (e == cudaSuccess) e = cudaEventRecord(ctx->wf_ev, stream);
    ctx->wf_last = stream;
    return e;
}

/* path-tracer samples: the wavefront stages over the context's scratch, or
 * the per-pixel kernel (QR_FP_PIXEL_PT, or when the scratch cannot be had);
 * both give the same frame */
static cudaError_t launch_pt(qr_ctx *ctx, const qr_scene_slot *sl, const qr_frame_params *fp,
                             float *acc, uint32_t *dev_frame, cudaStream_t stream)
{
    if (fp->flags & QR_FP_PIXEL_PT) return qr_launch_pt(sl->d, *fp, acc, dev_frame, stream);
    std::lock_guard<std::mutex> lock(ctx->wfmu);
    const qr_wf_caps caps = qr_wf_caps_for(*fp, ctx->wf_paths, ctx->wf_q, ctx->wf_pool);
    if (!wf_scratch(ctx, qr_wf_bytes(caps)))
        return qr_launch_pt(sl->d, *fp, acc, dev_frame, stream);
    /* a frame of two chunks or more keeps two in flight */
    const int tx = (fp->x_res + 7) / 8, ty = (fp->y_res + 3) / 4;
    const long long paths = (long long)tx * ty * 32 * fp->pt_on;
    qr_wf_second sec;
    const qr_wf_second *second = NULL;
    if (paths > caps.cap_paths && wf_scratch2(ctx, qr_wf_bytes(caps)))
    {
        sec.scratch = ctx->wf2;
        sec.stream = ctx->wf_side;
        for (int k = 0; k < 3; k++) sec.ev[k] = ctx->wf_sev[k];
        second = &sec;
    }
    cudaError_t e = wf_begin(ctx, stream);
    if (e == cudaSuccess)
        e = qr_wf_launch_pt(sl->d, *fp, acc, dev_frame, ctx->wf, caps, ctx->sms, stream,
                            second);
    return wf_end(ctx, stream, e);
}

/* a Whitted frame: the per-pixel kernels, or with QR_FP_WAVEFRONT the
 * wavefront stages over the context's scratch (unless the light lists are
 * longer than the stages take, or there is no scratch); the frame is the
 * same.  The per-pixel kernels are the default: on the animated 1080p 4x
 * AA frame they take 21.0 ms against 31.9 ms for the stages, whose shadow
 * rays lose the coherence a thread's own sub-samples give them */
static cudaError_t launch_whitted(qr_ctx *ctx, const qr_scene_slot *sl,
                                  const qr_frame_params *fp, uint32_t *dev_frame,
                                  cudaStream_t stream)
{
    if (!(fp->flags & QR_FP_WAVEFRONT)) return qr_launch_whitted(sl->d, *fp, dev_frame, stream);
    const qr_wh_caps caps = qr_wh_caps_for(*fp, sl->max_lnum, ctx->wh_samples);
    if (!caps.ok) return qr_launch_whitted(sl->d, *fp, dev_frame, stream);
    std::lock_guard<std::mutex> lock(ctx->wfmu);
    if (!wf_scratch(ctx, qr_wh_bytes(caps)))
        return qr_launch_whitted(sl->d, *fp, dev_frame, stream);
    cudaError_t e = wf_begin(ctx, stream);
    if (e == cudaSuccess)
        e = qr_wh_launch(sl->d, *fp, dev_frame, ctx->wf, caps, ctx->sms, stream);
    return wf_end(ctx, stream, e);
}

/* Whitted frame, or path-tracer samples when fp->pt_on > 0 */
static cudaError_t launch(qr_ctx *ctx, const qr_scene_slot *sl, const qr_frame_params *fp,
                          float *acc, uint32_t *dev_frame, cudaStream_t stream)
{
    if (fp->pt_on > 0) return launch_pt(ctx, sl, fp, acc, dev_frame, stream);
    return launch_whitted(ctx, sl, fp, dev_frame, stream);
}

extern "C" int qr_render_device(qr_ctx *ctx, int scene_id, const qr_frame_params *fp,
                                uint32_t *dev_frame, void *stream)
{
    qr_scene_slot *sl = slot(ctx, scene_id);
    if (sl == NULL) return QR_ERR_NOSCENE;
    int rc = check_fp(fp);
    if (rc != QR_OK) return rc;
    if (dev_frame == NULL) return QR_ERR_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "cudaSetDevice", e);
    if (fp->pt_on > 0)
    {
        rc = ensure_acc(ctx, (size_t)fp->x_row * fp->y_res);
        if (rc != QR_OK) return rc;
    }
    e = launch(ctx, sl, fp, ctx->dacc, dev_frame, (cudaStream_t)stream);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "render launch", e);
    return QR_OK;
}

extern "C" int qr_render_pt(qr_ctx *ctx, int scene_id, const qr_frame_params *fp,
                            float *dev_acc, uint32_t *dev_frame, void *stream)
{
    qr_scene_slot *sl = slot(ctx, scene_id);
    if (sl == NULL) return QR_ERR_NOSCENE;
    int rc = check_fp(fp);
    if (rc != QR_OK) return rc;
    if (fp->pt_on <= 0 || dev_acc == NULL || dev_frame == NULL) return QR_ERR_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess)
        e = launch_pt(ctx, sl, fp, dev_acc, dev_frame, (cudaStream_t)stream);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "path-tracer launch", e);
    return QR_OK;
}

extern "C" int qr_render_host(qr_ctx *ctx, int scene_id, const qr_frame_params *fp,
                              uint32_t *host_frame)
{
    qr_scene_slot *sl = slot(ctx, scene_id);
    if (sl == NULL) return QR_ERR_NOSCENE;
    int rc = check_fp(fp);
    if (rc != QR_OK) return rc;
    if (host_frame == NULL) return QR_ERR_ARG;
    size_t px = (size_t)fp->x_row * fp->y_res;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess && ctx->dframe_px < px)
    {
        if (ctx->dframe) cudaFree(ctx->dframe);
        ctx->dframe = NULL;
        e = cudaMalloc(&ctx->dframe, px * sizeof(uint32_t));
        if (e != cudaSuccess) return fail(ctx, QR_ERR_OOM, "cudaMalloc frame", e);
        ctx->dframe_px = px;
    }
    if (e == cudaSuccess && fp->pt_on > 0)
    {
        rc = ensure_acc(ctx, px);
        if (rc != QR_OK) return rc;
    }
    if (e == cudaSuccess) e = launch(ctx, sl, fp, ctx->dacc, ctx->dframe, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host_frame, ctx->dframe, px * sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "render host", e);
    int32_t f[4];
    return qr_fault(ctx, f);
}

extern "C" int qr_render_stats(qr_ctx *ctx, int scene_id, const qr_frame_params *fp,
                               uint32_t *host_frame, uint64_t *counts)
{
    qr_scene_slot *sl = slot(ctx, scene_id);
    if (sl == NULL) return QR_ERR_NOSCENE;
    int rc = check_fp(fp);
    if (rc != QR_OK) return rc;
    if (host_frame == NULL || counts == NULL) return QR_ERR_ARG;
    size_t px = (size_t)fp->x_row * fp->y_res;
    uint32_t *dframe = NULL;
    qr_dstats *dst = NULL;
    qr_dstats hst;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaMalloc(&dframe, px * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&dst, sizeof(qr_dstats));
    float *dacc = NULL;
    if (e == cudaSuccess && fp->pt_on > 0)
        e = cudaMalloc(&dacc, px * 3 * sizeof(float));
    if (e == cudaSuccess && dacc != NULL)
        e = cudaMemsetAsync(dacc, 0, px * 3 * sizeof(float), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(dst, 0, sizeof(qr_dstats), ctx->stream);
    if (e == cudaSuccess)
    {
        if (fp->pt_on > 0) e = qr_launch_pt_stats(sl->d, *fp, dacc, dframe, dst, ctx->stream);
        else e = qr_launch_whitted_stats(sl->d, *fp, dframe, dst, ctx->stream);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host_frame, dframe, px * sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&hst, dst, sizeof(qr_dstats), cudaMemcpyDeviceToHost,
                            ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (dframe) cudaFree(dframe);
    if (dacc) cudaFree(dacc);
    if (dst) cudaFree(dst);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "render stats", e);
    for (int k = 0; k < QR_STAT_COUNT; k++) counts[k] = hst.c[k];
    return QR_OK;
}

extern "C" int qr_fault(qr_ctx *ctx, int32_t out[4])
{
    if (ctx == NULL || out == NULL) return QR_ERR_ARG;
    uint32_t h[4];
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h, ctx->dfault, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "fault word", e);
    for (int k = 0; k < 4; k++) out[k] = (int32_t)h[k];
    if (h[0] == 0) return QR_OK;
    e = cudaMemsetAsync(ctx->dfault, 0, sizeof(h), ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "fault word", e);
    {
        std::lock_guard<std::mutex> lock(ctx->mu);
        snprintf(ctx->err, sizeof(ctx->err),
                 "%u pixel(s) ran past a loop bound (faults 0x%x, first at %u, %u)",
                 h[3], h[0], h[1], h[2]);
    }
    return QR_ERR_TRACE;
}

extern "C" int qr_sync(qr_ctx *ctx, void *stream)
{
    if (ctx == NULL) return QR_ERR_ARG;
    cudaError_t e = cudaStreamSynchronize(stream ? (cudaStream_t)stream : ctx->stream);
    if (e != cudaSuccess) return fail(ctx, QR_ERR_CUDA, "sync", e);
    return QR_OK;
}

/* ---- internal accessors for other translation units of the library ---- */

int qr_internal_scene(qr_ctx *ctx, int scene_id, const qr_dscene **sc, int *device)
{
    qr_scene_slot *sl = slot(ctx, scene_id);
    if (sl == NULL) return QR_ERR_NOSCENE;
    *sc = &sl->d;
    *device = ctx->device;
    return QR_OK;
}

int qr_internal_device(qr_ctx *ctx)
{
    return ctx->device;
}

int qr_internal_check_fp(const qr_frame_params *fp)
{
    return check_fp(fp);
}

int qr_internal_fail(qr_ctx *ctx, int code, const char *what, cudaError_t e)
{
    return fail(ctx, code, what, e);
}

void qr_internal_message(qr_ctx *ctx, const char *msg)
{
    if (ctx == NULL) return;
    std::lock_guard<std::mutex> lock(ctx->mu);
    snprintf(ctx->err, sizeof(ctx->err), "%s", msg);
}

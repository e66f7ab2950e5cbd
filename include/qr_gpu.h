/*
 * qr_gpu.h: C ABI of the GB300 QuadRay render backend.
 *
 * This is the boundary between the host engine (rt_Platform / rt_Scene, which
 * keeps the reference API of VectorChief/QuadRay-engine core/engine/engine.h
 * and flattens the object tree) and the sm_103a CUDA tracer.  It replaces the
 * reference's backend entry points, which take pre-broadcast SIMD structs:
 *
 *   rt_Platform::render0(rt_SIMD_INFOX*)   core/tracer/tracer.cpp:8454
 *                                          (declared core/engine/engine.h:129)
 *   rt_Platform::update0(rt_SIMD_SURFACE*) core/tracer/tracer.cpp:8115
 *                                          (declared core/engine/engine.h:128)
 *   rt_Platform::switch0(...)              core/tracer/tracer.cpp:8180
 *
 * Everything here is plain C: fixed-layout structs, integers, pointers and
 * sizes.  Every entry point returns a status (QR_OK = 0); nothing throws.
 *
 * Flattened scene ("qr_scene_desc"): one record per surface or transform
 * node (qr_srf, the fields the reference keeps in rt_SIMD_SURFACE,
 * core/tracer/tracer.h:1024-1183), one per material (rt_SIMD_MATERIAL,
 * tracer.h:1193-1292) and light (rt_SIMD_LIGHT, tracer.h:968-1014), and flat
 * element arrays for the linked lists the reference walks (rt_ELEM,
 * tracer.h:132-146): the camera's surface list, per-surface clipper lists,
 * per-side light lists with their shadow lists, and per-side lists for
 * reflected/refracted rays.
 */
#ifndef QR_GPU_H
#define QR_GPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define QR_OK               0
#define QR_ERR_ARG          1   /* invalid argument / size */
#define QR_ERR_OOM          2   /* device or host allocation failed */
#define QR_ERR_CUDA         3   /* CUDA runtime error (message in last_error) */
#define QR_ERR_TIMEOUT      4   /* bounded device wait expired */
#define QR_ERR_STATE        5   /* call out of order (e.g. render w/o scene) */
#define QR_ERR_NOSCENE      6   /* unknown scene id */
#define QR_ERR_LIMIT        7   /* request exceeds a compiled-in limit */
#define QR_ERR_BUSY         8   /* launched work still running (poll) */
#define QR_ERR_TRACE        9   /* a pixel's ray tree or hierarchy walk ran
                                   past its bound (corrupt scene data); see
                                   qr_fault */

/* bounds of the per-pixel loops; a pixel that runs past one is rendered
 * black and recorded in the context's fault word (qr_fault):
 *   QR_FAULT_TREE   more traced segments than a ray tree of the frame's
 *                   depth can hold (Whitted: (2^(depth+1) - 1) * (1 + lights)
 *                   per camera ray; path tracer: (3^(depth+1) - 1) / 2 per
 *                   sample)
 *   QR_FAULT_STACK  the hierarchy walk's node stack (48 entries) is full */
#define QR_FAULT_TREE       1
#define QR_FAULT_STACK      2

/* ---- material / context property bits (tracer.h:66-77) ----------------- */
#define QR_PROP_LIGHT       0x00000010
#define QR_PROP_METAL       0x00000020
#define QR_PROP_GAMMA       0x00000040
#define QR_PROP_FRESNEL     0x00000080
#define QR_PROP_NORMAL      0x00000100
#define QR_PROP_OPAQUE      0x00000200
#define QR_PROP_TRANSP      0x00000400
#define QR_PROP_TEXTURE     0x00000800
#define QR_PROP_REFLECT     0x00001000
#define QR_PROP_REFRACT     0x00002000
#define QR_PROP_DIFFUSE     0x00004000
#define QR_PROP_SPECULAR    0x00008000

/* ---- element kinds in flattened lists ------------------------------------ */
#define QR_ELM_SURFACE      0   /* ref = surface index */
#define QR_ELM_TRNODE       1   /* ref = node index, last = index (in the same
                                   list) of the node's last surface element */
#define QR_ELM_ACC_ENTER    2   /* clip lists: boolean accumulator enter */
#define QR_ELM_ACC_LEAVE    3   /* clip lists: boolean accumulator leave */

typedef struct qr_elem
{
    int32_t kind;       /* QR_ELM_* */
    int32_t ref;        /* surface / node index */
    int32_t last;       /* trnode: list index of its last element */
    int32_t rel;        /* clip lists: -1 minus inner, +1 minus outer */
} qr_elem;

/* light list element: a light and the surfaces that can shadow it */
typedef struct qr_lelem
{
    int32_t light;      /* light index */
    int32_t shd_off;    /* shadow list: offset into qr_scene_desc.elems */
    int32_t shd_num;    /* shadow list length */
    int32_t pad;
} qr_lelem;

/*
 * Surface or transform-node record, 256 bytes, 16-byte aligned.
 * Axis mapping: local axis I/J/K of the surface is stored in world (or
 * transform-node) axis amap[0..2] with sign asgn[0..2] (1 = negated);
 * amap[3] is the transform class (0 none, 1 scaling only, 2 rotation,
 * 3 rotation + scaling) and asgn[3] is 1 when the surface's coordinates come
 * from a transform node (the IJK fields of the reference context).
 */
typedef struct qr_srf
{
    float   pos[3];     int32_t tag;        /* RT_TAG_* of format.h */
    float   tci[3];     int32_t solver;     /* 1 plane 2 quadric 3 two-plane */
    float   tcj[3];     int32_t nrmk;       /* normal kind (update0 srf_t[1]) */
    float   tck[3];     int32_t clpk;       /* clipper kind (srf_t[2]) */
    float   sci[4];                         /* x,y,z,w quadric coefficients */
    float   scj[3];     int32_t conic;      /* apex adjust: 0 no, 1 cone, 2 hc */
    float   bmin[3];    int32_t mint;       /* axis clip min, bit k = active */
    float   bmax[3];    int32_t maxt;       /* axis clip max, bit k = active */
    int32_t amap[4];
    int32_t asgn[4];
    int32_t mat[2];                         /* outer/inner material index */
    int32_t props[2];                       /* outer/inner material props */
    int32_t trnode;                         /* transform node index or -1 */
    int32_t clip_off, clip_num;             /* clipper list in elems */
    int32_t is_node;                        /* 1 for transform-node records */
    int32_t lgt_off[2], lgt_num[2];         /* per-side light lists, lelems */
    int32_t sec_off[2], sec_num[2];         /* per-side lists for secondary
                                               rays, in elems */
    int32_t id;                             /* generation index (hit IDs) */
    int32_t pad[7];
} qr_srf;

typedef struct qr_mat
{
    float   l_dff, l_spc;   int32_t l_pow;  int32_t props;
    float   c_rfl, c_trn, c_rfr, rfr_2;
    float   c_rcp, ext_2;   float col_e[2];         /* col_e: reserved */
    float   xscal, yscal, xoffs, yoffs;             /* texture transform */
    int32_t xmask, ymask, yshft, tex_off;           /* texel offset in texels */
    int32_t tmap[2];    int32_t pad0[2];            /* UV -> XY mapping */
    float   emit[4];                                /* PT emission r,g,b,src */
} qr_mat;

typedef struct qr_light
{
    float   pos[3];     float t_max;
    float   col[3];     float l_src;
    float   a_qdr, a_lnr, a_cnt, a_rng;
} qr_light;

/* flattened scene (host memory, copied to the device by qr_scene_upload) */
typedef struct qr_scene_desc
{
    int32_t         nsrf;       const qr_srf   *srf;
    int32_t         nmat;       const qr_mat   *mat;
    int32_t         nlgt;       const qr_light *lgt;
    int32_t         nelem;      const qr_elem  *elems;
    int32_t         nlelem;     const qr_lelem *lelems;
    int32_t         ntex;       const uint32_t *texels;
    int32_t         cam_off, cam_num;   /* camera's surface list in elems */
} qr_scene_desc;

/* per-frame camera and mode parameters (rt_SIMD_CAMERA, tracer.h:869-958,
 * and the per-thread setup of rt_Scene::render_slice, engine.cpp:3514) */
typedef struct qr_frame_params
{
    float   org[3];     float t_min;        /* camera position, near clip */
    float   dir[3];     float t_max;        /* ray to pixel (0,0) centre */
    float   hor[3];     int32_t flags;      /* per-pixel horizontal step;
                                               QR_FP_* bits */
    float   ver[3];     float pad1;         /* per-pixel vertical step */
    float   amb[3];     float l_amb;        /* accumulated ambient colour */
    int32_t x_res, y_res, x_row;            /* frame size, row stride (px) */
    int32_t fsaa;                           /* 0 none, 1 2x, 2 4x */
    int32_t depth;                          /* secondary-ray depth */
    int32_t ctx_props;                      /* QR_PROP_GAMMA when gamma on */
    int32_t pt_on;                          /* path-tracer samples (0 off) */
    int32_t frame_idx;                      /* PT frame counter */
    uint64_t seed;                          /* PT seed */
    float   pts_c;  float pad2;             /* PT samples so far */
} qr_frame_params;

/* most path-tracer samples per pixel in one render call */
#define QR_MAX_PT_SAMPLES   65536

/* qr_frame_params.flags */
#define QR_FP_LINEAR_WALK   1   /* walk every surface list in order instead of
                                   the scene's bounding-volume hierarchy (the
                                   frame is the same; for tests) */
#define QR_FP_PIXEL_THREADS 2   /* 4x AA: one thread traces all four
                                   sub-samples of its pixel instead of one
                                   thread a sub-sample (the frame is the
                                   same; for tests; single-frame renders
                                   only, batches ignore it) */
#define QR_FP_WAVEFRONT     8   /* Whitted: wavefront stages (queues of
                                   camera, shadow and secondary rays)
                                   instead of a thread a pixel or 4x AA
                                   sub-sample tracing its whole ray tree
                                   (the frame is the same; slower on the
                                   benchmarked frames) */
#define QR_FP_PIXEL_PT      4   /* path tracer: one thread a pixel with its
                                   samples in turn (the per-pixel kernel)
                                   instead of the wavefront stages (the
                                   frame is the same; for tests and
                                   comparisons) */

typedef struct qr_ctx qr_ctx;

/* library / device context */
int qr_ctx_create(int device, qr_ctx **out);
int qr_ctx_destroy(qr_ctx *ctx);
const char *qr_last_error(qr_ctx *ctx);

/* scenes are kept resident on the device; returns a scene id */
int qr_scene_upload(qr_ctx *ctx, const qr_scene_desc *desc, int *scene_id);
/* replace the scene's records in place (same list structure, new fields) */
int qr_scene_update(qr_ctx *ctx, int scene_id, const qr_scene_desc *desc);
int qr_scene_release(qr_ctx *ctx, int scene_id);

/*
 * Device-side update phases for animated scenes.  The reference runs the
 * update phases on the host for every frame (rt_Scene::render,
 * core/engine/engine.cpp:3350-3501: animators and transforms in
 * rt_Object::update_status / update_matrix, object.cpp:175-389; inverse
 * matrices in rt_Node::update_fields, object.cpp:826-857).  Here the host
 * runs only the animators and hands over each animated transform's sines,
 * cosines and position; one kernel launch per frame then forms the
 * transform chain, the inverse matrices and positions of the records that
 * move, the world boxes of the surfaces that move and the hierarchy's node
 * boxes, and the frame equals the frame of a full host update.
 *
 * The table (qr_anim_node, one entry per record or light whose transform
 * changes when animators run, parents before children) says how each
 * entry's matrix M follows from its parent entry's matrix T and fixed
 * matrices P, R (rt_Object::update_matrix, object.cpp:221-389):
 *   QR_ANIM_OWN     M = P R            (own rotation, no transform node)
 *   QR_ANIM_UNDER   M = (T P) R        (own rotation under a transform node)
 *   QR_ANIM_NODE    M = T P            (becomes a transform node)
 * where R is the entry's own rotation: T(pos) Rz Ry Rx from animated
 * transform `param`, or the fixed matrix r when param < 0.
 */
#define QR_ANIM_OWN     0
#define QR_ANIM_UNDER   1
#define QR_ANIM_NODE    2

typedef struct qr_anim_node
{
    int32_t kind;       /* QR_ANIM_* */
    int32_t parent;     /* entry of T (QR_ANIM_UNDER, QR_ANIM_NODE), else -1 */
    int32_t param;      /* animated transform forming R, -1: R = r */
    int32_t rec;        /* record whose tci/tcj/tck/pos M gives, -1: none */
    int32_t light;      /* light whose pos M gives, -1: none */
    int32_t pad[3];
    float   p[16];      /* P, column-major (m[column][row]) */
    float   r[16];      /* R when param < 0 */
} qr_anim_node;

/* one animated transform for a frame: sines and cosines of its rotation
 * about x, y, z in degrees as the reference computes them (RT_SINA /
 * RT_COSA, core/config/rtbase.h:858-875) and its position */
typedef struct qr_anim_param
{
    float   sin[3];
    float   cos[3];
    float   pos[3];
    float   pad[3];
} qr_anim_param;

/* The update calls may come from several host threads: a preparation waits
 * for the scene's updates still in flight, and no update starts while a
 * scene is prepared.  As with qr_scene_update, renders of a scene must not
 * overlap its updates: order them on one stream.
 *
 * Upload `desc` into scene `scene_id` in place (as qr_scene_update) with
 * the hierarchy sized for the motion bound (lo[3], hi[3]; NULL: where
 * rotations of the animated transforms about their origins can take the
 * moving records and surfaces, joined with the scene's extent) and prepare the
 * device update of the n entries of `nodes` (records and lights in range,
 * parents earlier).  A later qr_scene_update drops the preparation. */
int qr_scene_anim_init(qr_ctx *ctx, int scene_id, const qr_scene_desc *desc,
                       const qr_anim_node *nodes, int n, const float *bound);
/* the same into a new resident scene (qr_scene_upload then
 * qr_scene_anim_init, with one upload); returns its id */
int qr_scene_anim_upload(qr_ctx *ctx, const qr_scene_desc *desc,
                         const qr_anim_node *nodes, int n, const float *bound,
                         int *scene_id);
/* one frame's update on `stream` (asynchronous; NULL: the context's own
 * stream, which qr_render_host and the uploads use; `params` is copied
 * before the call returns): params[i] for every animated transform i named
 * by the table.  When a moved record or surface leaves the motion bound the
 * hierarchy's boxes are opened to the whole space for that frame (the frame
 * stays exact, rays walk every surface) and the miss is counted */
int qr_scene_anim_update(qr_ctx *ctx, int scene_id, const qr_anim_param *params,
                         int nparams, void *stream);
/* the updates of n scenes (distinct, each prepared by qr_scene_anim_init)
 * in one launch on `stream` (NULL: the context's stream), one block a
 * scene: for a batch of frames of animated scenes, ahead of the batched
 * render on the same stream */
typedef struct qr_anim_request
{
    int32_t              scene_id;
    int32_t              nparams;
    const qr_anim_param *params;
} qr_anim_request;
int qr_scene_anim_update_many(qr_ctx *ctx, const qr_anim_request *reqs, int n,
                              void *stream);
/* out[0] = frames updated on the device, out[1] = frames whose update left
 * the motion bound (opened boxes); updates on other streams must have
 * finished */
int qr_scene_anim_status(qr_ctx *ctx, int scene_id, int32_t out[2]);

/* render one frame into a device frame buffer (uint32 XRGB, x_row stride),
 * asynchronously on `stream` (a cudaStream_t, 0 = default stream).
 * With fp->pt_on > 0 the frame is path traced: pt_on samples per pixel are
 * added to the context's running sums (reset when fp->pts_c == 0, which
 * counts the samples already summed) and the frame shows the mean over
 * pts_c + pt_on samples; every random draw is a counter-based hash of
 * (fp->seed, fp->frame_idx, pixel, sample number pts_c + i, the drawing
 * node's place in the sample's ray tree, the draw's purpose), so the frame
 * does not depend on the order the GPU evaluates paths in.  This replaces
 * the reference's
 * path-tracer accumulation planes (rt_Scene::render with set_pton,
 * core/engine/engine.cpp:2914-2919, 3674; tracer.cpp:2115-2139) */
int qr_render_device(qr_ctx *ctx, int scene_id, const qr_frame_params *fp,
                     uint32_t *dev_frame, void *stream);

/* path tracer with caller-owned running sums: dev_acc holds 3 floats per
 * pixel (x_row stride) and is overwritten when fp->pts_c == 0 */
int qr_render_pt(qr_ctx *ctx, int scene_id, const qr_frame_params *fp,
                 float *dev_acc, uint32_t *dev_frame, void *stream);
/* path tracer without any device allocation.  This entry point has no
 * counterpart in the reference.  It serves callers that may not allocate
 * device memory inside their render loop (a server that keeps allocations
 * out of its steady state, a host application that owns the device heap):
 * it is qr_render_pt with its running sums in a fixed array inside the
 * library (QR_NOALLOC_MAX_PX pixels of 3 floats, 12 MiB a device, held
 * until the process exits; x_row * y_res may not exceed it: QR_ERR_LIMIT).
 * The first call on a device looks the array up (cudaGetSymbolAddress) with
 * that device current and should come before any stream capture; the
 * caller's current device is restored before the call returns.  A call with
 * pts_c == 0 starts the sums for its context, scene and frame shape (x_row,
 * y_res); later calls add to them and must name the same context, scene and
 * shape (else QR_ERR_STATE); nothing has to be cleared first.  The array is
 * shared by every context and scene on a device: calls that overlap on the
 * GPU race on it. */
#define QR_NOALLOC_MAX_PX   (1 << 20)
int qr_render_pt_noalloc(qr_ctx *ctx, int scene_id, const qr_frame_params *fp,
                         uint32_t *dev_frame, void *stream);

/* render one frame into host memory: copies in, renders, copies out, syncs */
int qr_render_host(qr_ctx *ctx, int scene_id, const qr_frame_params *fp,
                   uint32_t *host_frame);
int qr_sync(qr_ctx *ctx, void *stream);

/* read and clear the context's fault word: out[0] = QR_FAULT_* bits seen
 * since the last call (0: none), out[1], out[2] = x, y of the first pixel
 * that recorded one, out[3] = how many pixels did.  Renders on a caller's
 * stream must have finished (qr_sync) before the call.  Returns QR_OK, or
 * QR_ERR_TRACE when a bit was set.  qr_render_host checks the word itself
 * and returns QR_ERR_TRACE */
int qr_fault(qr_ctx *ctx, int32_t out[4]);

/* instrumented render: counts the work of one frame (traced segments by
 * kind, solver tests, clip evaluations, shaded hits, light evaluations) into
 * counts[QR_STAT_*]; the frame is rendered into host_frame as usual.  Used to
 * derive rays/s and the algorithmic FLOPs of the roofline; the counters are
 * never compiled into timed launches */
#define QR_STAT_RAY_PRIMARY     0
#define QR_STAT_RAY_SHADOW      1
#define QR_STAT_RAY_SECONDARY   2
#define QR_STAT_TEST_PLANE      3
#define QR_STAT_TEST_QUADRIC    4
#define QR_STAT_TEST_TWOPLANE   5
#define QR_STAT_XFORM           6
#define QR_STAT_CLIP_ROOT       7
#define QR_STAT_CLIP_CUSTOM     8
#define QR_STAT_SHADE           9
#define QR_STAT_LIGHT           10
#define QR_STAT_REFRACT         11
#define QR_STAT_REFLECT         12
#define QR_STAT_BOX_TEST        13      /* bounding-volume box tests */
#define QR_STAT_FAR_WALK        14      /* full-list walks of rays starting
                                           beyond the hierarchy's radius */
#define QR_STAT_COUNT           15
int qr_render_stats(qr_ctx *ctx, int scene_id, const qr_frame_params *fp,
                    uint32_t *host_frame, uint64_t *counts);

/*
 * Batched rendering: many frame requests on resident scenes of one context,
 * Whitted or path-traced (fp.pt_on > 0), of any sizes, rendered by one
 * persistent launch per mode over all their pixel tiles, captured in a CUDA
 * graph.  The reference renders one frame per rt_Scene::render call
 * (core/engine/engine.cpp:3014) with a CPU thread pool; it has no batch.
 * Each frame is the same as the frame of qr_render_device / qr_render_pt for
 * the same request.
 */
typedef struct qr_request
{
    int32_t         scene_id;
    int32_t         pad;
    qr_frame_params fp;             /* frame size, camera, depth, pt_on ... */
    uint32_t       *dev_frame;      /* output, x_row stride */
    float          *dev_acc;        /* path tracer: running sums (3 floats a
                                       pixel), NULL for Whitted frames */
} qr_request;

typedef struct qr_batch qr_batch;

int qr_batch_create(qr_ctx *ctx, int max_requests, qr_batch **out);
int qr_batch_destroy(qr_batch *b);
/* replace the batch's requests (validated; scenes must stay resident) */
int qr_batch_set(qr_batch *b, const qr_request *reqs, int n);
/* tile width (4, 8, 16 or 32; tiles are 32 pixels) and tiles a warp claims
 * at once (1-64) */
int qr_batch_config(qr_batch *b, int tile_w, int grab);
/* on (the default): the Whitted requests' kernel is persistent, a block
 * for each resident slot, its warps claiming runs of tiles until none are
 * left; off: a block for every 4 runs of tiles, each warp taking one run,
 * so that blocks retire as they finish and kernels on streams of higher
 * priority take the SMs between them (a server's urgent requests) */
int qr_batch_persistent(qr_batch *b, int on);
/* time every tile configuration on the batch and keep the fastest;
 * tile_w, grab and ms (optional) receive the choice and its time */
int qr_batch_tune(qr_batch *b, int *tile_w, int *grab, float *ms);
/* render every request on `stream` (asynchronous) */
int qr_batch_launch(qr_batch *b, void *stream);
/* QR_OK once the last launch finished, QR_ERR_BUSY while it runs */
int qr_batch_poll(qr_batch *b);
int qr_batch_wait(qr_batch *b);
/* per-request completion of the last launch: *flags points at one word per
 * request (in qr_batch_set order) in host memory that the device writes;
 * a word turns 1 once that request's frame is complete in device memory,
 * while the rest of the batch may still run.  qr_batch_launch clears the
 * words, so when they are read, launch again only after the previous launch
 * finished (qr_batch_poll / qr_batch_wait); read them as volatile.  No
 * counterpart in the reference (it renders one frame per call) */
int qr_batch_done(qr_batch *b, const volatile uint32_t **flags);

/* measured FP32 issue rate of `device` in TFLOP/s (*tflops): plain FP32
 * additions (fma == 0, one operation a lane and instruction, the rate of
 * this tracer's arithmetic, which issues no fused multiply-add) or fused
 * multiply-adds (fma != 0, counted as two operations), every SM filled,
 * timed with CUDA events at the clock the device runs.  The roofline
 * denominator of the render kernels; no counterpart in the reference */
int qr_fp32_peak(int device, int fma, double *tflops);

/* Kernels the library has launched in this process, all contexts together:
 * renders, path-tracer stages, device updates, batches (a batch counts the
 * kernels of its graph at each launch).  No counterpart in the reference. */
unsigned long long qr_kernel_launches(void);

#ifdef __cplusplus
}
#endif

#endif /* QR_GPU_H */

/*
 * tracer.cuh: device-side data of the GB300 QuadRay tracer.
 */
#ifndef QR_TRACER_CUH
#define QR_TRACER_CUH

#include <stdint.h>
#include "qr_gpu.h"
#include "accel.h"

/* secondary-ray depth limit: the reference's context stack depth
 * (RT_STACK_DEPTH, core/tracer/tracer.h:51); the tracer keeps one pending
 * shaded hit per level */
#define QR_MAX_DEPTH        10

/* device copy of a flattened scene (qr_scene_desc with device pointers) */
struct qr_dscene
{
    const qr_srf   *srf;
    const qr_mat   *mat;
    const qr_light *lgt;
    const qr_elem  *elems;
    const qr_lelem *lelems;
    const uint32_t *texels;
    int32_t nsrf, nmat, nlgt, nelem, nlelem, ntex;
    int32_t cam_off, cam_num;
    /* bounding-volume hierarchy over the camera list (accel.h); nnodes < 0
     * when the scene has none.  The shadow list [shd_off, shd_off + shd_num)
     * holds the same surfaces, so shadow rays use it too */
    const qr_bnode *nodes;          /* all levels, concatenated */
    const qr_bpair *pairs;          /* the walk's child records, one a node */
    const qr_bquad *quads;          /* the walk's 4-wide records */
    const int32_t  *quad_src;       /* each quad slot's node (-1: empty) */
    int32_t nquads;
    const qr_bitem *items;
    const qr_bitem *always;
    int32_t nnodes, nitems, nalways;
    int32_t shd_off, shd_num;
    /* level l: root node, unbounded surfaces always[aoff, aoff + anum),
     * and the rays it serves: origin within sqrt(r2) of ray_c (r2 < 0: the
     * level is missing) */
    int32_t lvl_root[QR_BVH_LEVELS], lvl_aoff[QR_BVH_LEVELS], lvl_anum[QR_BVH_LEVELS];
    int32_t lvl_quad[QR_BVH_LEVELS];    /* code of level l's root in the 4-wide view */
    float   lvl_r2[QR_BVH_LEVELS];
    float   ray_c[3];
    /* the owning context's fault word: QR_FAULT_* bits, x, y of the first
     * pixel that set one, count of such pixels (NULL: not recorded) */
    uint32_t *fault;
};

/* count n kernel launches on `stream` in the library's total
 * (qr_kernel_launches); launches into a stream capture are not counted
 * there: a graph's kernels count when the graph is launched */
void qr_note_launches(cudaStream_t stream, int n);

/* per-launch counters (instrumented runs only) */
struct qr_dstats
{
    unsigned long long c[QR_STAT_COUNT];   /* QR_STAT_* counters */
};

/* launch the per-pixel Whitted kernel for one frame */
cudaError_t qr_launch_whitted(const qr_dscene &sc, const qr_frame_params &fp,
                              uint32_t *dev_frame, cudaStream_t stream);

/* the same kernel built with work counters (tracer_stats.cu); dstats must
 * hold zeros before the launch */
cudaError_t qr_launch_whitted_stats(const qr_dscene &sc, const qr_frame_params &fp,
                                    uint32_t *dev_frame, qr_dstats *dstats,
                                    cudaStream_t stream);

/* path tracer: add fp.pt_on samples per pixel to the running sums acc
 * (3 floats per pixel, x_row stride; reset when fp.pts_c == 0) and write the
 * mean over pts_c + pt_on samples into dev_frame */
cudaError_t qr_launch_pt(const qr_dscene &sc, const qr_frame_params &fp, float *acc,
                         uint32_t *dev_frame, cudaStream_t stream);
cudaError_t qr_launch_pt_stats(const qr_dscene &sc, const qr_frame_params &fp, float *acc,
                               uint32_t *dev_frame, qr_dstats *dstats,
                               cudaStream_t stream);

/* one request of a batched launch: its scene, frame parameters, output
 * frame (and path-tracer sums) and its first tile in the batch's numbering */
struct qr_job
{
    qr_dscene       S;
    qr_frame_params P;
    uint32_t       *frame;
    float          *acc;
    int32_t         tile0, tiles_x;
    int32_t         ntiles;         /* tiles of the request */
    int32_t         req;            /* its index in the batch */
};

/* launch over the tiles of njobs requests of one mode (0 Whitted, 1 path
 * tracer): `blocks` persistent blocks, or with `once` a block for every 4
 * runs of grab tiles; *counter and tiles_done[0, njobs) must hold 0.
 * The warp that finishes a request's last tile sets done[req] to 1 (done
 * may be host memory mapped into the device) */
cudaError_t qr_launch_batch(int mode, const qr_job *jobs, int njobs, int total_tiles,
                            int *counter, int tw, int th, int grab, int blocks, int once,
                            int *tiles_done, uint32_t *done, cudaStream_t stream);
/* resident blocks of 128 threads per SM of the batch kernel of a mode */
int qr_batch_blocks_per_sm(int mode);

#endif /* QR_TRACER_CUH */

/*
 * anim.cuh: device-side update of an animated scene's records, surface
 * boxes and hierarchy (qr_scene_anim_update in include/qr_gpu.h).
 */
#ifndef QR_ANIM_CUH
#define QR_ANIM_CUH

#include <cuda_runtime.h>
#include "qr_gpu.h"
#include "accel.h"

/* everything one update launch reads and writes, in device memory (params
 * in mapped host memory) */
struct qr_anim_dev
{
    const qr_anim_node  *nodes;     /* the table */
    const int32_t       *order;     /* entries by generation (parents first) */
    const int32_t       *gen_off;   /* generation g: order[gen_off[g], gen_off[g+1]) */
    int32_t              n, ngen;
    const qr_anim_param *params;
    float               *mtx;       /* per entry: M, 16 floats */
    qr_srf              *srf;
    qr_light            *lgt;
    const qr_anim_term  *terms;
    const qr_anim_target *targets;
    int32_t              ntargets, nsrf;
    float               *lboxes;    /* [QR_BVH_LEVELS][nsrf][6] surface boxes */
    qr_bnode            *bvh;       /* hierarchy nodes, all levels */
    qr_bpair            *pairs;     /* the walk's child records of the nodes */
    qr_bquad            *quads;     /* the walk's 4-wide records */
    const int32_t       *quad_src;  /* each slot's node (-1: empty) */
    int32_t              nquads;
    const qr_bitem      *items;
    const int32_t       *rorder;    /* nodes by depth, deepest first */
    const int32_t       *depth_off; /* depth band b: rorder[depth_off[b], depth_off[b+1]) */
    int32_t              nbvh, nbands;
    int32_t              lvl_end[QR_BVH_LEVELS];   /* level l: nodes below lvl_end[l] */
    float               *frame;     /* per record: world-from-local 3x3
                                       (row-major) and a singular flag, 10
                                       floats (qr_accel_record_frame) */
    float                ext[6];    /* motion bound the boxes allow for */
    uint32_t            *status;    /* [0] frames updated, [1] frames out of bound */
};

/* updates of n scenes on `stream`, one block each; devs (n entries, in
 * mapped host memory) must stay unchanged until the launch has run */
cudaError_t qr_launch_anim(const qr_anim_dev *devs, int n, cudaStream_t stream);

#endif /* QR_ANIM_CUH */

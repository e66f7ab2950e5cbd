/*
 * accel.h: bounding-volume hierarchy over a flattened scene's surface list.
 *
 * The reference tests every surface of a (per-tile, culled) list for every
 * ray (core/tracer/tracer.cpp:2413-2680).  The GB300 tracer replaces the
 * walk of the full camera / shadow / secondary list with a traversal of a
 * BVH built over conservative world-space boxes of the list's surfaces;
 * surfaces without a finite box are tested by every ray.  A hit is accepted
 * by (t, list position): among equal distances the surface earlier in the
 * list wins, which is exactly what the in-order walk with its strict depth
 * test keeps, so frames are bit-identical to the walk.
 *
 * Boxes are derived from the records the tracer itself uses (qr_srf): the
 * surface's local coordinates as the walk forms them (transform node, own
 * transform or translation only), bounded by the quadric's sublevel set
 * {f <= 0}, the active axis clippers and the clippers that keep only the
 * inside of a surface (RT_REL_MINUS_OUTER outside accumulator segments), and
 * mapped back to world space in double precision with a safety margin.
 */
#ifndef QR_ACCEL_H
#define QR_ACCEL_H

#include <stdint.h>
#include <vector>
#include "qr_gpu.h"

/* hierarchy levels built per scene; levels past the first only for lists of
 * at least QR_BVH_OUTER_MIN elements */
#define QR_BVH_LEVELS 3
#define QR_BVH_OUTER_MIN 64

/* BVH node: inner nodes have count == 0 and children a, b; leaves hold
 * items [a, a + count) */
struct qr_bnode
{
    float   lo[3];
    int32_t a;
    float   hi[3];
    int32_t count;
    int32_t b;
    int32_t pad[3];
};

/* leaves hold at most QR_BVH_LEAF_MAX items, and a level at most
 * QR_BVH_MAX_ITEMS items: a leaf is then coded in one int (qr_bpair) */
#define QR_BVH_LEAF_MAX 15
#define QR_BVH_MAX_ITEMS (1 << 26)

/* the two children of an inner node as the walk reads them, 64 bytes:
 * each child's box, and in the fourth word of its lo group the child's
 * code: an inner node's index, or for a leaf ~(first item << 4 | count).
 * One record a node (a leaf's is unused); the device update rewrites the
 * boxes from the nodes' after each refit */
struct qr_bpair
{
    float   lo_a[3];
    int32_t code_a;
    float   hi_a[3];
    int32_t pad_a;
    float   lo_b[3];
    int32_t code_b;
    float   hi_b[3];
    int32_t pad_b;
};

/* the walk's 4-wide view of the tree, 128 bytes a record: up to four
 * children's boxes (structure of arrays, one 16-byte group per bound and
 * axis) and codes (qr_bpair's, QR_BQUAD_EMPTY for an unused slot, whose
 * box is empty).  A record collapses a node of the binary tree with its
 * children (and theirs) until it holds four, the largest boxes opened
 * first; each slot's box is the box of a node of the binary tree (its
 * source), which the device update copies after each refit */
#define QR_BQUAD_EMPTY ((int32_t)0x80000000)
struct qr_bquad
{
    float   lo_x[4], lo_y[4], lo_z[4];
    float   hi_x[4], hi_y[4], hi_z[4];
    int32_t code[4];
    int32_t pad[4];
};

/* the walk's code of node i (see qr_bpair) */
#if defined(__CUDACC__)
__host__ __device__
#endif
static inline int32_t qr_bnode_code(const qr_bnode &n, int32_t i)
{
    return n.count > 0 ? (int32_t)~(((uint32_t)n.a << 4) | (uint32_t)n.count) : i;
}

/* one surface of the list: its position in the list (tie order), record
 * index, and the transform node whose cached transform the walk applies
 * (-1: the surface's own transform or translation) */
struct qr_bitem
{
    int32_t pos;
    int32_t srf;
    int32_t xf;
    int32_t pad;
};

struct qr_accel_host
{
    std::vector<qr_bnode> nodes;        /* nodes[0] is the root */
    std::vector<qr_bitem> items;        /* leaf items (BVH order) */
    std::vector<qr_bitem> always;       /* unbounded surfaces (list order) */
    std::vector<float>    boxes;        /* per record: lo[3], hi[3] (level 0) */
    std::vector<int32_t>  bounded;      /* per record (level 0) */
    /* the same per level (qr_accel_build_levels; empty for levels not built) */
    std::vector<float>    lboxes[QR_BVH_LEVELS];
    std::vector<int32_t>  lbounded[QR_BVH_LEVELS];
    int depth;
    /* rays whose origin lies within sqrt(ray_r2) of ray_c may use the
     * hierarchy (the boxes allow for their rounding); others walk the list */
    float ray_c[3], ray_r2;
    /* the extent the levels' radii and rounding allowances follow from
     * (lo[3], hi[3]), and the largest gain from world distances to local
     * coordinates */
    double ext[6], gain;
};

/* build the hierarchy of one level over the camera list of `d` (which the
 * flattening also uses, in the same order, for shadow and secondary rays):
 * level l serves rays starting within 8^l times the base radius of the
 * scene's centre, its boxes allowing for their rounding; returns 0 */
int qr_accel_build(const qr_scene_desc *d, qr_accel_host *out, int level);

/* the walk's child records of `nodes` (one a node) */
void qr_accel_pairs(const std::vector<qr_bnode> &nodes, std::vector<qr_bpair> &pairs);

/* the 4-wide records of the trees rooted at root[l] (l < nlev; roots past
 * the node array are skipped): quads, each slot's source node (src, 4 a
 * record, -1 for an empty slot), and per level the code of its root
 * (quad_root) and the deepest stack its walk can need (stack_need: 3 a
 * record on the way down) */
void qr_accel_quads(const std::vector<qr_bnode> &nodes, const int *root, int nlev,
                    std::vector<qr_bquad> &quads, std::vector<int32_t> &src,
                    int32_t *quad_root, int32_t *stack_need);

/* all levels concatenated into `out` (node indices and item ranges shifted
 * by the preceding levels); per level its root node, its unbounded surfaces
 * always[aoff, aoff + anum) and the squared radius it serves (-1: none) */
void qr_accel_build_levels(const qr_scene_desc *d, qr_accel_host *out,
                           int root[QR_BVH_LEVELS], int aoff[QR_BVH_LEVELS],
                           int anum[QR_BVH_LEVELS], float r2[QR_BVH_LEVELS],
                           const float *bound);

/* the extent of the scene's surfaces and records (lo[3], hi[3]) that the
 * levels' radii follow from when there is no motion bound */
void qr_accel_extent(const qr_scene_desc *d, double ext[6]);

/* one term of a surface's world box: record srf's local box u[l] at level l
 * (u[QR_BVH_LEVELS]: the surface's box without rounding allowance, for the
 * extent check) mapped to world space by the frame `mode`:
 *   QR_TERM_NODE        h = M_T^-1 (u + srf.pos) + T.pos, T = record xf
 *   QR_TERM_NODE_SHIFT  h = u + srf.pos + T.pos
 *   QR_TERM_OWN         h = M_s^-1 u + srf.pos
 *   QR_TERM_OWN_SHIFT   h = u + srf.pos
 * (world_box in accel.cpp) */
#define QR_TERM_NODE        0
#define QR_TERM_NODE_SHIFT  1
#define QR_TERM_OWN         2
#define QR_TERM_OWN_SHIFT   3

struct qr_anim_term
{
    int32_t srf, xf, mode, pad;
    float   u[QR_BVH_LEVELS + 1][6];    /* rounded outwards from double */
};

/* a surface whose box is the meet of terms [t0, t0 + tn), the first its
 * own; bit l of levels: the surface is bounded at level l */
struct qr_anim_target
{
    int32_t srf, t0, tn, levels;
};

/* world-from-local matrix of a record's frame as the box terms use it: the
 * inverse of the record's transform rows (record_matrix), row-major, in
 * float; false when singular */
bool qr_accel_record_frame(const qr_srf &t, float a[9]);
bool qr_accel_record_frame_d(const qr_srf &t, double a[9]);     /* the same in double */

/* the terms of every bounded surface whose box depends on a record marked
 * in dyn (its own, its transform node's, a bounding clipper's or that
 * clipper's node); acc is the hierarchy built with the same bound */
int qr_accel_anim_terms(const qr_scene_desc *d, const qr_accel_host *acc,
                        const float *bound, const std::vector<char> &dyn,
                        std::vector<qr_anim_term> &terms,
                        std::vector<qr_anim_target> &targets);

/* where rotations of the table's animated transforms about their origins
 * can take the moving records and surfaces, joined with the scene's extent
 * (lo[3], hi[3]): the default motion bound of qr_scene_anim_init */
void qr_accel_rotation_bound(const qr_scene_desc *d, const qr_anim_node *nodes, int n,
                             float out[6]);

/* deepest traversal stack the tracer supports */
#define QR_BVH_STACK 48

#endif /* QR_ACCEL_H */

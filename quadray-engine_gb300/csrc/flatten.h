/*
 * flatten.h: host-side object tree and its flattening into qr_scene_desc.
 *
 * Restates the reference engine's per-frame update phases
 * (core/engine/object.cpp and core/engine/engine.cpp) for the render path:
 *   phase 0.5  hierarchical transforms and transform-node selection
 *              (rt_Object::update_matrix, object.cpp:221-389;
 *               rt_Array::update_object, object.cpp:1753-1781)
 *   phase 1    per-object backend fields: inverse transforms, axis mapping,
 *              quadric coefficients, lights, camera
 *              (object.cpp:826-857, 1786-1850, 2497-2528, 2920-3936, 649-667)
 *   phase 2    custom clipper lists and clip boxes
 *              (engine.cpp:1850-1979 sclip; object.cpp:2533-2870 minmax)
 *   lists      camera surface list, light/shadow lists, secondary-ray lists
 *              (engine.cpp:1145-2782), brute force: no culling, same order
 *   phase 3    solver/normal/clipper kinds (rt_Platform::update0,
 *              core/tracer/tracer.cpp:8115-8149)
 *   camera     ray basis and ambient (rt_Scene::render, engine.cpp:3078-3318;
 *              render_slice, engine.cpp:3514-3672)
 * All float arithmetic is written in the reference's operation order and must
 * be compiled with -ffp-contract=off so results are bit-identical on x86-64
 * and AArch64.
 */
#ifndef QR_FLATTEN_H
#define QR_FLATTEN_H

#include <deque>
#include <string>
#include <vector>
#include "format.h"
#include "qr_gpu.h"

#ifndef RT_CAMERA_CROUCH
/* camera actions (codes of core/engine/object.h:47-63) */
#define RT_CAMERA_CROUCH            0
#define RT_CAMERA_JUMP              1
#define RT_CAMERA_MOVE_DOWN         2
#define RT_CAMERA_MOVE_UP           3
#define RT_CAMERA_MOVE_LEFT         4
#define RT_CAMERA_MOVE_RIGHT        5
#define RT_CAMERA_MOVE_BACK         6
#define RT_CAMERA_MOVE_FORWARD      7
#define RT_CAMERA_LEAN_LEFT         8
#define RT_CAMERA_LEAN_RIGHT        9
#define RT_CAMERA_ROTATE_DOWN       10
#define RT_CAMERA_ROTATE_UP         11
#define RT_CAMERA_ROTATE_LEFT       12
#define RT_CAMERA_ROTATE_RIGHT      13
#endif

namespace qr
{

/* sine / cosine of an angle in degrees, exact at multiples of 90 degrees
 * (RT_SINA / RT_COSA, core/config/rtbase.h:858-875) */
float sina(float deg);
float cosa(float deg);

struct Node;

/* material as seen by the backend (rt_Material, object.cpp:4038-4180) */
struct Material
{
    rt_MATERIAL *mat;
    rt_SIDE     *sd;
    int          props;
    int          map[2];
    float        scl[2];
    qr_mat       m;         /* backend record */
    rt_ui32     *texels;    /* resolved texel pointer */
    int          x_dim, y_dim;
};

struct Node
{
    int          kind;      /* 0 array, 1 surface, 2 camera, 3 light */
    int          tag;
    rt_OBJECT   *obj;
    rt_TRANSFORM3D *trm;
    Node        *parent;
    Node        *trnode;
    float        mtx[4][4];
    float        inv[4][4];
    float        scm[4][4];     /* arrays: scalers for sub-objects */
    float      (*pmtx)[4];      /* matrix handed down by the parent */
    int          map[4];
    int          sgn[4];
    float        scl[4];
    int          obj_changed, obj_has_trm, mtx_has_trm;
    int          in_flags;      /* update flags handed down by the parent */
    std::vector<Node*> children;

    /* surfaces */
    rt_SURFACE  *srf;
    int          outer, inner;  /* material indices */
    float        sci[4], scj[4];/* shape (before the 0.5 scj scale) */
    float        bmin[4], bmax[4], cmin[4], cmax[4];
    /* relations template: (data, object or NULL for accum markers) in the
     * order the backend evaluates them */
    struct Rel { int data; Node *obj; };
    std::vector<Rel> rel;
    int          index;         /* flat record index */
    int          gen;           /* creation order among surfaces */

    /* lights */
    float        lcol[3];       /* colour * source intensity */
    float        hdr[4];        /* light / camera colour */
    /* arrays: accumulated light colour for emitters */
    float        acc[4];

    /* camera */
    float        pov;

    qr_srf       rec;           /* backend record */

    Node() : kind(0), tag(0), obj(0), trm(0), parent(0), trnode(0), pmtx(0),
             obj_changed(0), obj_has_trm(0), mtx_has_trm(0), in_flags(0), srf(0),
             outer(-1), inner(-1), index(-1), gen(-1), pov(1.0f) {}
};

/*
 * Scene tree built once from the scene structs; update(time) recomputes all
 * backend fields for a frame and refreshes the flat arrays.
 */
class Flat
{
public:
    Flat(rt_SCENE *scn, int opts, int x_res, int y_res, int fsaa);
    ~Flat();

    /* run the update phases for `time` and rebuild the flat arrays */
    void update(rt_time time);
    /* camera movement from user input before the next update
     * (rt_Camera::update_action, object.cpp:495-573) */
    void camera_action(rt_time time, int action);
    /* the next camera of the reference's list (rt_Scene::next_cam,
     * engine.cpp:3836-3850); returns its index in that list */
    int next_cam();
    /* ambient/camera parameters for the current camera */
    void frame_params(qr_frame_params *fp) const;
    /* descriptor pointing into this object's arrays */
    void desc(qr_scene_desc *d) const;
    /* the device update table (qr_anim_node, include/qr_gpu.h) of the
     * records and lights that move when animators run, from the state of
     * the last update(); nonzero (and the reason in *why) when the scene
     * cannot be updated on the device: an animated object without a free
     * rotation (all angles multiples of 90 degrees) or a camera under one */
    int anim_table(std::vector<qr_anim_node> &out, std::string *why);
    /* run the animators for `time` (as update() does, without the update
     * phases), refresh the cameras (their transforms after camera actions;
     * no camera moves with an animated object) and give each animated
     * transform of the table; nonzero when one lost its free rotation (1)
     * or changed its scale (2): the frame then needs update() and a new
     * table */
    int anim_params(rt_time time, std::vector<qr_anim_param> &out);

    int  opts;
    int  x_res, y_res, fsaa;
    int  depth;
    int  cam_idx;               /* current camera in `cameras`; the
                                   reference's list runs the other way */
    float factor, aspect;
    float hor_sin, hor_cos;     /* current camera's heading as of the last
                                   update (object.cpp:485-486) */

    std::vector<Node*>  nodes;      /* all nodes, creation order */
    std::vector<Node*>  surfaces;   /* creation order */
    std::vector<Node*>  arrays;     /* creation order */
    std::vector<Node*>  lights;     /* creation order */
    std::vector<Node*>  cameras;    /* creation order */
    std::vector<Material> mats;
    /* textures loaded from files, by name (rt_Texture registry,
     * object.cpp:3990-4011) */
    std::deque<std::vector<rt_ui32> > file_tex;
    std::vector<std::string> file_tex_name;
    std::vector<int> file_tex_dim;

    std::vector<qr_srf>   srf;
    std::vector<qr_mat>   mat;
    std::vector<qr_light> lgt;
    std::vector<qr_elem>  elems;
    std::vector<qr_lelem> lelems;
    std::vector<rt_ui32>  texels;
    int cam_off, cam_num;

    Node *root;
    rt_OBJECT rootobj;
    /* animated transforms of the update table and their scales */
    std::vector<Node*> anim_nodes;
    std::vector<std::vector<float> > anim_scl;

private:
    Node *build(Node *parent, rt_OBJECT *obj);
    int   material(rt_SIDE *sd, rt_MATERIAL *mt);
    void  relations(Node *arr);
    void  add_relation(Node *n, const std::vector<Node::Rel> &lst);

    void  update_object(Node *n, rt_time time, int flags, Node *trnode,
                        float (*mtx)[4]);
    void  update_status(Node *n, rt_time time, int flags, Node *trnode);
    void  update_matrix(Node *n, float (*mtx)[4]);
    void  fields_node(Node *n);
    void  fields_surface(Node *n);
    void  fields_array(Node *n);
    void  bounds(Node *n);
    void  recalc_minmax(Node *n, float *smin, float *smax, float *bmin,
                        float *bmax, float *cmin, float *cmax);
    void  adjust_minmax(Node *n, const float *smin, const float *smax,
                        float *bmin, float *bmax, float *cmin, float *cmax);
    void  invert_minmax(Node *n, const float *smin, const float *smax,
                        float *dmin, float *dmax);
    void  direct_minmax(Node *n, const float *smin, const float *smax,
                        float *dmin, float *dmax);
    void  emit_records();
    void  emit_lists();
    int   emit_surface_list(const std::vector<Node*> &order);
};

} /* namespace qr */

#endif /* QR_FLATTEN_H */

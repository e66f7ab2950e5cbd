/*
 * engine.h: host API of the GB300 QuadRay engine.
 *
 * Keeps the construction / update / render interface of the reference
 * engine (VectorChief/QuadRay-engine core/engine/engine.h:71-369) so an
 * application written against rt_Platform / rt_Scene switches by relinking.
 * Scenes are the static structs of format.h.  Rendering runs on the GPU
 * through the C ABI of qr_gpu.h; the CPU thread-pool callbacks are accepted
 * for signature compatibility and drive nothing (there is no CPU render).
 * Errors are reported as rt_Exception, as in the reference.
 */
#ifndef QR_ENGINE_H
#define QR_ENGINE_H

#include <vector>
#include "format.h"
#include "rt_exception.h"
#include "qr_gpu.h"
#include "flatten.h"

#define RT_FSAA_NO              0
#define RT_FSAA_2X              1
#define RT_FSAA_4X              2
#define RT_FSAA_8X              3

#define RT_TILE_W               8
#define RT_TILE_H               8

class rt_Platform;
class rt_Scene;
namespace qr { class Flat; }

typedef rt_pntr (*rt_FUNC_ALLOC)(rt_size size);
typedef rt_void (*rt_FUNC_FREE)(rt_pntr ptr, rt_size size);
typedef rt_pntr (*rt_FUNC_INIT)(rt_si32 thnum, rt_Platform *pfm);
typedef rt_void (*rt_FUNC_TERM)(rt_pntr tdata, rt_si32 thnum);
typedef rt_void (*rt_FUNC_UPDATE)(rt_pntr tdata, rt_si32 thnum, rt_si32 phase);
typedef rt_void (*rt_FUNC_RENDER)(rt_pntr tdata, rt_si32 thnum, rt_si32 phase);
typedef rt_void (*rt_FUNC_PRINT_LOG)(rt_pstr format, ...);
typedef rt_void (*rt_FUNC_PRINT_ERR)(rt_pstr format, ...);

/*
 * Platform: allocator callbacks, antialiasing mode and the GPU context
 * (the reference's platform owns the thread pool and the SIMD target).
 */
class rt_Platform
{
public:
    rt_Platform(rt_FUNC_ALLOC f_alloc, rt_FUNC_FREE f_free, rt_si32 thnum = 0,
                rt_FUNC_INIT f_init = RT_NULL, rt_FUNC_TERM f_term = RT_NULL,
                rt_FUNC_UPDATE f_update = RT_NULL,
                rt_FUNC_RENDER f_render = RT_NULL,
                rt_FUNC_PRINT_LOG f_print_log = RT_NULL,
                rt_FUNC_PRINT_ERR f_print_err = RT_NULL);
    virtual ~rt_Platform();

    rt_si32     get_thnum();
    rt_si32     set_thnum(rt_si32 thnum);
    /* the SIMD target of the reference; the GPU build has one target and
     * returns its code (sm_103a) for any request */
    rt_si32     set_simd(rt_si32 simd);
    rt_si32     set_fsaa(rt_si32 fsaa);
    rt_si32     get_fsaa_max();
    rt_si32     get_fsaa();
    rt_si32     get_tile_w();

    rt_Scene*   get_cur_scene();
    rt_Scene*   set_cur_scene(rt_Scene *scn);
    rt_void     next_scene();

    rt_pntr     alloc(rt_size size);
    rt_void     free(rt_pntr ptr, rt_size size);

    /* GPU context used by all scenes of this platform */
    qr_ctx     *get_ctx();

private:
    rt_FUNC_ALLOC   f_alloc;
    rt_FUNC_FREE    f_free;
    rt_si32         thnum;
    rt_si32         fsaa;
    qr_ctx         *ctx;
    rt_Scene       *head;
    rt_Scene       *cur;

    friend class rt_Scene;
};

/*
 * Scene: the engine instance for one rt_SCENE.  render() runs the update
 * phases on the host, refreshes the device-resident scene and renders the
 * frame on the GPU into the frame buffer given at construction (or an
 * internal one).
 */
class rt_Scene
{
public:
    rt_pntr operator new(size_t size, rt_Platform *pfm);
    rt_void operator delete(rt_pntr ptr);

    rt_Scene(rt_SCENE *scn, rt_si32 x_res, rt_si32 y_res, rt_si32 x_row,
             rt_ui32 *frame, rt_Platform *pfm);
    virtual ~rt_Scene();

    rt_void     update(rt_time time, rt_si32 action);
    rt_void     render(rt_time time);

    rt_si32     get_x_row();
    rt_void     print_state();
    rt_si32     get_opts();
    rt_si32     set_opts(rt_si32 opts);
    rt_si32     get_pton();
    rt_si32     set_pton(rt_si32 pton);
    rt_si32     get_cam_idx();
    rt_si32     next_cam();
    rt_ui32*    get_frame();
    rt_void     save_frame(rt_si32 index);
    rt_Platform*get_platform();

    /* GB300 extensions: render into a device buffer on a stream without
     * host copies, and access to the flattened scene */
    rt_void     render_device(rt_time time, rt_ui32 *dev_frame, rt_pntr stream);
    const qr::Flat *flat() const { return fl; }
    rt_si32     get_depth();
    rt_si32     set_depth(rt_si32 depth);
    /* update animated scenes on the device (qr_scene_anim_*, on by
     * default): each render runs only the animators on the host, and a
     * scene without animated objects is uploaded once; the frames are those
     * of the host update phases */
    rt_si32     set_device_update(rt_si32 on);
    rt_si32     get_device_update();

private:
    rt_Platform *pfm;
    rt_SCENE    *scn;
    rt_si32      x_res, y_res, x_row;
    rt_ui32     *frame;
    rt_ui32     *own_frame;
    rt_si32      opts;
    rt_si32      pt_on;
    rt_si32      pts_c;         /* path-tracer samples accumulated */
    rt_si32      pt_frame;      /* path-tracer launches (stream index) */
    std::vector<unsigned char> pt_key;  /* scene records of the last frame */
    rt_si32      depth;
    qr::Flat    *fl;
    int          scene_id;
    int          print;
    rt_Scene    *next;
    /* device-side updates: 1 prepared, 0 to be tried at the next host
     * update, -1 the scene does not allow them; host updates come back every
     * QR_ENGINE_REBUILD device updates (the hierarchy's tree is the first
     * frame's, refitted) */
    int          dev_update;
    int          anim_state;
    int          since_host;
    std::vector<qr_anim_node>  table;
    std::vector<qr_anim_param> params;

    rt_void     prepare(rt_time time, rt_pntr stream);
    rt_void     frame_setup(qr_frame_params *fp);
    friend class rt_Platform;
};

#endif /* QR_ENGINE_H */

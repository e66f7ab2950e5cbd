/*
 * engine.cpp: host API of the GB300 QuadRay engine (engine.h).
 *
 * rt_Scene::render follows the reference's frame (core/engine/engine.cpp
 * rt_Scene::render, 3014-3384): update phases on the host (qr::Flat), then
 * the render, which here is one GPU launch through the C ABI instead of the
 * per-thread render0 calls.
 */
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <new>

#include <string>
#include "engine.h"
#include "flatten.h"

static rt_pntr default_alloc(rt_size size) { return malloc((size_t)size); }
static rt_void default_free(rt_pntr ptr, rt_size size) { (void)size; free(ptr); }

/* ---- platform ------------------------------------------------------------ */

rt_Platform::rt_Platform(rt_FUNC_ALLOC f_alloc_, rt_FUNC_FREE f_free_,
                         rt_si32 thnum_, rt_FUNC_INIT f_init,
                         rt_FUNC_TERM f_term, rt_FUNC_UPDATE f_update,
                         rt_FUNC_RENDER f_render, rt_FUNC_PRINT_LOG f_print_log,
                         rt_FUNC_PRINT_ERR f_print_err)
    : f_alloc(f_alloc_ ? f_alloc_ : default_alloc),
      f_free(f_free_ ? f_free_ : default_free),
      thnum(thnum_ > 0 ? thnum_ : 1), fsaa(RT_FSAA_NO), ctx(RT_NULL),
      head(RT_NULL), cur(RT_NULL)
{
    (void)f_init; (void)f_term; (void)f_update; (void)f_render;
    (void)f_print_log; (void)f_print_err;
    const char *dev = getenv("QR_DEVICE");
    int rc = qr_ctx_create(dev ? atoi(dev) : 0, &ctx);
    if (rc != QR_OK)
    {
        throw rt_Exception("GPU context creation failed");
    }
}

rt_Platform::~rt_Platform()
{
    if (ctx != RT_NULL) qr_ctx_destroy(ctx);
}

rt_si32 rt_Platform::get_thnum() { return thnum; }
rt_si32 rt_Platform::set_thnum(rt_si32 n) { thnum = n > 0 ? n : 1; return thnum; }
rt_si32 rt_Platform::set_simd(rt_si32 simd) { (void)simd; return 103; }
rt_si32 rt_Platform::set_fsaa(rt_si32 f)
{
    /* none, 2x alternating, 4x rotated grid; as the reference, modes above
     * the maximum fall back to it (engine.cpp:662-672) */
    fsaa = f > RT_FSAA_4X ? RT_FSAA_4X : (f < RT_FSAA_NO ? RT_FSAA_NO : f);
    return fsaa;
}
rt_si32 rt_Platform::get_fsaa_max() { return RT_FSAA_4X; }
rt_si32 rt_Platform::get_fsaa() { return fsaa; }
rt_si32 rt_Platform::get_tile_w() { return RT_TILE_W; }
rt_Scene *rt_Platform::get_cur_scene() { return cur; }
rt_Scene *rt_Platform::set_cur_scene(rt_Scene *s) { cur = s; return cur; }
rt_void rt_Platform::next_scene()
{
    if (cur != RT_NULL) cur = cur->next != RT_NULL ? cur->next : head;
}
rt_pntr rt_Platform::alloc(rt_size size)
{
    rt_pntr p = f_alloc(size);
    if (p == RT_NULL) throw rt_Exception("alloc failed with NULL address");
    return p;
}
rt_void rt_Platform::free(rt_pntr ptr, rt_size size) { f_free(ptr, size); }
qr_ctx *rt_Platform::get_ctx() { return ctx; }

/* ---- scene --------------------------------------------------------------- */

struct scene_hdr { rt_Platform *pfm; size_t size; };

rt_pntr rt_Scene::operator new(size_t size, rt_Platform *pfm)
{
    scene_hdr *h = (scene_hdr *)pfm->alloc((rt_size)(size + sizeof(scene_hdr) + 15));
    h->pfm = pfm;
    h->size = size + sizeof(scene_hdr) + 15;
    return (rt_pntr)((char *)h + sizeof(scene_hdr));
}

rt_void rt_Scene::operator delete(rt_pntr ptr)
{
    scene_hdr *h = (scene_hdr *)((char *)ptr - sizeof(scene_hdr));
    h->pfm->free(h, (rt_size)h->size);
}

rt_Scene::rt_Scene(rt_SCENE *scn_, rt_si32 x_res_, rt_si32 y_res_,
                   rt_si32 x_row_, rt_ui32 *frame_, rt_Platform *pfm_)
    : pfm(pfm_), scn(scn_), x_res(x_res_), y_res(y_res_), x_row(x_row_),
      frame(frame_), own_frame(RT_NULL), opts(0), pt_on(0), pts_c(0), pt_frame(0),
      depth(10),
      fl(RT_NULL), scene_id(-1), print(0), next(RT_NULL), dev_update(1), anim_state(0),
      since_host(0)
{
    if (scn == RT_NULL) throw rt_Exception("null-pointer in scene");
    if (scn->lock != RT_NULL)
    {
        throw rt_Exception("scene data is locked by another instance");
    }
    if (x_res <= 0 || y_res <= 0 || x_row < x_res)
    {
        /* negative strides (bottom-up frames) are not supported */
        throw rt_Exception("frambuffer's dimensions are not valid");
    }
    if (frame == RT_NULL)
    {
        own_frame = (rt_ui32 *)pfm->alloc((rt_size)x_row * y_res * sizeof(rt_ui32));
        frame = own_frame;
    }
    memset(frame, 0, (size_t)x_row * y_res * sizeof(rt_ui32));

    /* default runtime options minus the scene's opt-outs (object.h:164,
     * engine.cpp:2904) */
    opts = (rt_si32)(RT_OPTS_FULL & ~scn->opts);
    fl = new qr::Flat(scn, opts, x_res, y_res, pfm->fsaa);
    fl->depth = depth;
    scn->lock = this;

    next = pfm->head;
    pfm->head = this;
    if (pfm->cur == RT_NULL) pfm->cur = this;
}

rt_Scene::~rt_Scene()
{
    if (scene_id >= 0) qr_scene_release(pfm->get_ctx(), scene_id);
    delete fl;
    scn->lock = RT_NULL;
    if (own_frame != RT_NULL)
    {
        pfm->free(own_frame, (rt_size)x_row * y_res * sizeof(rt_ui32));
    }
    rt_Scene **p = &pfm->head;
    while (*p != RT_NULL && *p != this) p = &(*p)->next;
    if (*p == this) *p = next;
    if (pfm->cur == this) pfm->cur = pfm->head;
}

rt_void rt_Scene::update(rt_time time, rt_si32 action)
{
    /* camera movement from user input (rt_Scene::update, engine.cpp:3006) */
    fl->camera_action(time, action);
}

#define QR_ENGINE_REBUILD 32

/* the scene at `time` on the device: the animators and one device update
 * (on `stream`, NULL: the context's stream) when the scene allows it, else
 * the host update phases and an upload */
rt_void rt_Scene::prepare(rt_time time, rt_pntr stream)
{
    if (fl->fsaa != pfm->fsaa)
    {
        fl->fsaa = pfm->fsaa;
    }
    fl->depth = depth;
    qr_ctx *ctx = pfm->get_ctx();
    int rc;
    /* a scene without animated objects (an empty table) changes only by
     * its cameras, which anim_params refreshes: its records stay as
     * uploaded and need no rebuild */
    if (dev_update && anim_state == 1 && scene_id >= 0 &&
        (table.empty() || since_host < QR_ENGINE_REBUILD))
    {
        if (fl->anim_params(time, params) == 0)
        {
            rc = table.empty() ? QR_OK
                               : qr_scene_anim_update(ctx, scene_id, params.data(),
                                                      (int)params.size(), stream);
            if (rc != QR_OK)
            {
                fprintf(stderr, "qr scene update: %d %s\n", rc, qr_last_error(ctx));
                throw rt_Exception("scene update on the GPU failed");
            }
            since_host++;
            return;
        }
        anim_state = 0;     /* the table no longer fits: a new one below */
    }
    fl->update(time);
    qr_scene_desc d;
    fl->desc(&d);
    if (dev_update && anim_state == 0)
    {
        std::string why;
        anim_state = fl->anim_table(table, &why) == 0 ? 1 : -1;
        if (table.empty()) params.clear();
    }
    if (dev_update && anim_state == 1 && !table.empty())
    {
        fl->anim_params(time, params);      /* the transforms of this frame */
        rc = scene_id < 0 ? qr_scene_anim_upload(ctx, &d, table.data(), (int)table.size(),
                                                 RT_NULL, &scene_id)
                          : qr_scene_anim_init(ctx, scene_id, &d, table.data(),
                                               (int)table.size(), RT_NULL);
        since_host = 0;
    }
    else
    {
        rc = scene_id < 0 ? qr_scene_upload(ctx, &d, &scene_id)
                          : qr_scene_update(ctx, scene_id, &d);
    }
    if (rc != QR_OK)
    {
        fprintf(stderr, "qr scene upload: %d %s\n", rc, qr_last_error(ctx));
        throw rt_Exception("scene upload to the GPU failed");
    }
}

rt_si32 rt_Scene::set_device_update(rt_si32 on)
{
    dev_update = on ? 1 : 0;
    since_host = QR_ENGINE_REBUILD;     /* the next render updates on the host */
    return dev_update;
}

rt_si32 rt_Scene::get_device_update() { return dev_update; }

/* frame parameters of this render; in path-tracer mode the samples
 * accumulate over frames until the scene changes (rt_Scene::render,
 * core/engine/engine.cpp:3054), each render adding pt_on per pixel */
rt_void rt_Scene::frame_setup(qr_frame_params *fp)
{
    fl->frame_params(fp);
    fp->x_row = x_row;
    if (pt_on <= 0) return;
    qr_scene_desc d;
    fl->desc(&d);
    std::vector<unsigned char> key;
    key.insert(key.end(), (const unsigned char *)d.srf,
               (const unsigned char *)(d.srf + d.nsrf));
    key.insert(key.end(), (const unsigned char *)d.mat,
               (const unsigned char *)(d.mat + d.nmat));
    key.insert(key.end(), (const unsigned char *)fp,
               (const unsigned char *)fp + offsetof(qr_frame_params, x_res));
    key.push_back((unsigned char)fl->fsaa);
    /* a device-updated frame differs from the last host update by the
     * animated transforms */
    if (anim_state == 1)
        key.insert(key.end(), (const unsigned char *)params.data(),
                   (const unsigned char *)(params.data() + params.size()));
    if (key != pt_key)
    {
        pts_c = 0;
        pt_key.swap(key);
    }
    fp->pt_on = pt_on;
    fp->pts_c = (float)pts_c;
    fp->frame_idx = pt_frame++;
    fp->seed = 0x5A17F00Dull;
    pts_c += pt_on;
}

rt_void rt_Scene::render(rt_time time)
{
    prepare(time, RT_NULL);
    qr_frame_params fp;
    frame_setup(&fp);
    int rc = qr_render_host(pfm->get_ctx(), scene_id, &fp, frame);
    if (rc != QR_OK)
    {
        fprintf(stderr, "qr render: %d %s\n", rc, qr_last_error(pfm->get_ctx()));
        throw rt_Exception("GPU render failed");
    }
}

rt_void rt_Scene::render_device(rt_time time, rt_ui32 *dev_frame, rt_pntr stream)
{
    prepare(time, stream);
    /* the legacy default stream does not wait for the context's stream */
    if (stream == RT_NULL) qr_sync(pfm->get_ctx(), RT_NULL);
    qr_frame_params fp;
    frame_setup(&fp);
    int rc = qr_render_device(pfm->get_ctx(), scene_id, &fp, dev_frame, stream);
    if (rc != QR_OK) throw rt_Exception("GPU render failed");
}

rt_si32 rt_Scene::get_x_row() { return x_row; }
rt_void rt_Scene::print_state() { print = 1; }
rt_si32 rt_Scene::get_opts() { return opts; }
rt_si32 rt_Scene::set_opts(rt_si32 o)
{
    opts = o & ~(rt_si32)scn->opts;
    int keep_cam = fl->cam_idx;
    delete fl;
    fl = new qr::Flat(scn, opts, x_res, y_res, pfm->fsaa);
    fl->cam_idx = keep_cam < (int)fl->cameras.size() ? keep_cam
                                                      : (int)fl->cameras.size() - 1;
    if (scene_id >= 0)
    {
        qr_scene_release(pfm->get_ctx(), scene_id);
        scene_id = -1;
    }
    anim_state = 0;
    return opts;
}
rt_si32 rt_Scene::get_pton() { return pt_on; }
/* path-tracer samples per render (0 off); refused while the options
 * prohibit the path tracer (RT_OPTS_PT, rt_Scene::set_pton,
 * core/engine/engine.cpp:3807-3822) */
rt_si32 rt_Scene::set_pton(rt_si32 pton)
{
    if ((opts & RT_OPTS_PT) == 0)
    {
        rt_si32 was = pt_on;
        pt_on = pton > 0 ? pton : 0;
        if (pt_on && !was) pts_c = 0;
    }
    return pt_on;
}
/* the index in the reference's camera list: the camera created last is 0
 * (engine.cpp:3828-3850) */
rt_si32 rt_Scene::get_cam_idx() { return (rt_si32)fl->cameras.size() - 1 - fl->cam_idx; }
rt_si32 rt_Scene::next_cam()
{
    return fl->next_cam();
}
rt_ui32 *rt_Scene::get_frame() { return frame; }
rt_Platform *rt_Scene::get_platform() { return pfm; }
rt_si32 rt_Scene::get_depth() { return depth; }
rt_si32 rt_Scene::set_depth(rt_si32 d)
{
    depth = d < 0 ? 0 : d > 10 ? 10 : d;
    return depth;
}

/* 24-bit BMP of the frame into the current directory as frameNNN.bmp
 * (rt_Scene::save_frame, engine.cpp:3863-3899) */
rt_void rt_Scene::save_frame(rt_si32 index)
{
    char name[64];
    snprintf(name, sizeof(name), "frame%03d.bmp", index % 1000);
    FILE *f = fopen(name, "wb");
    if (f == NULL) return;
    int row = (x_res * 3 + 3) & ~3;
    unsigned int size = 54 + row * y_res;
    unsigned char h[54];
    memset(h, 0, sizeof(h));
    h[0] = 'B'; h[1] = 'M';
    memcpy(h + 2, &size, 4);
    unsigned int off = 54, dib = 40, img = row * y_res;
    memcpy(h + 10, &off, 4);
    memcpy(h + 14, &dib, 4);
    memcpy(h + 18, &x_res, 4);
    memcpy(h + 22, &y_res, 4);
    h[26] = 1; h[28] = 24;
    memcpy(h + 34, &img, 4);
    fwrite(h, 1, 54, f);
    unsigned char *line = (unsigned char *)calloc(row, 1);
    for (int y = y_res - 1; y >= 0; y--)
    {
        for (int x = 0; x < x_res; x++)
        {
            rt_ui32 p = frame[(size_t)y * x_row + x];
            line[x * 3 + 0] = p & 0xFF;
            line[x * 3 + 1] = (p >> 8) & 0xFF;
            line[x * 3 + 2] = (p >> 16) & 0xFF;
        }
        fwrite(line, 1, row, f);
    }
    ::free(line);
    fclose(f);
}

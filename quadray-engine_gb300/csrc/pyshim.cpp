/*
 * pyshim.cpp: C entry points used by the Python side of the package
 * (tests, bench, the graft entry) on top of the C++ host and the C ABI.
 *
 *   qrpy_gen_*     seeded synthetic scenes (scenegen.hpp)
 *   qrpy_flat_*    host flattening without a GPU: the descriptor and frame
 *                  parameters the C ABI consumes (and the CPU oracle checks)
 *   qrpy_scene_*   the rt_Platform / rt_Scene API (GPU render)
 */
#include <stdio.h>
#include <string.h>

#include "scenegen.hpp"
#include "flatten.h"
#include "engine.h"

extern "C"
{

void *qrpy_gen_new(int kind, unsigned long long seed, int nq, int flags)
{
    try { return qr_gen::build(kind, seed, nq, flags); }
    catch (...) { return NULL; }
}

void qrpy_gen_free(void *g)
{
    delete (qr_gen::Scene *)g;
}

int qrpy_gen_nsurf(void *g)
{
    return ((qr_gen::Scene *)g)->nsurf;
}

int qrpy_gen_write_textures(unsigned long long seed, const char *dir)
{
    return qr_gen::write_texture_files(seed, dir);
}

void *qrpy_flat_new(void *g, int opts, int x_res, int y_res, int fsaa)
{
    qr_gen::Scene *sc = (qr_gen::Scene *)g;
    try
    {
        /* the scene's opt-outs always apply (rt_Scene::set_opts,
         * core/engine/engine.cpp:3786) */
        int o = (int)((opts < 0 ? RT_OPTS_FULL : opts) & ~sc->scn.opts);
        return new qr::Flat(&sc->scn, o, x_res, y_res, fsaa);
    }
    catch (rt_Exception &e)
    {
        fprintf(stderr, "qrpy_flat_new: %s\n", e.err);
        return NULL;
    }
}

int qrpy_flat_update(void *f, long long time, int depth)
{
    qr::Flat *fl = (qr::Flat *)f;
    try
    {
        fl->depth = depth;
        fl->update((rt_time)time);
    }
    catch (rt_Exception &e)
    {
        fprintf(stderr, "qrpy_flat_update: %s\n", e.err);
        return QR_ERR_ARG;
    }
    return QR_OK;
}

int qrpy_flat_next_cam(void *f)
{
    return ((qr::Flat *)f)->next_cam();
}

void qrpy_flat_action(void *f, long long time, int action)
{
    ((qr::Flat *)f)->camera_action((rt_time)time, action);
}

int qrpy_flat_desc(void *f, qr_scene_desc *d, qr_frame_params *fp)
{
    qr::Flat *fl = (qr::Flat *)f;
    fl->desc(d);
    fl->frame_params(fp);
    return QR_OK;
}

void qrpy_flat_free(void *f)
{
    delete (qr::Flat *)f;
}

/* ---- engine API --------------------------------------------------------- */

struct qrpy_engine
{
    rt_Platform *pfm;
    rt_Scene    *scn;
};

void *qrpy_scene_new(void *g, int x_res, int y_res, int fsaa, int opts, int depth,
                     unsigned int *frame)
{
    qr_gen::Scene *sc = (qr_gen::Scene *)g;
    qrpy_engine *e = new qrpy_engine();
    e->pfm = NULL;
    e->scn = NULL;
    try
    {
        e->pfm = new rt_Platform(NULL, NULL);
        e->pfm->set_fsaa(fsaa);
        /* frame: caller-owned x_res x y_res buffer, or NULL for the scene's
         * own (rt_Scene's frame argument) */
        e->scn = new(e->pfm) rt_Scene(&sc->scn, x_res, y_res, x_res, (rt_ui32 *)frame,
                                      e->pfm);
        if (opts >= 0) e->scn->set_opts(opts);
        e->scn->set_depth(depth);
    }
    catch (rt_Exception &ex)
    {
        fprintf(stderr, "qrpy_scene_new: %s\n", ex.err);
        if (e->scn) delete e->scn;
        if (e->pfm) delete e->pfm;
        delete e;
        return NULL;
    }
    return e;
}

int qrpy_scene_render(void *h, long long time, unsigned int *out)
{
    qrpy_engine *e = (qrpy_engine *)h;
    try
    {
        e->scn->render((rt_time)time);
    }
    catch (rt_Exception &ex)
    {
        fprintf(stderr, "qrpy_scene_render: %s\n", ex.err);
        return QR_ERR_CUDA;
    }
    if (out != NULL)
    {
        const qr::Flat *fl = e->scn->flat();
        memcpy(out, e->scn->get_frame(),
               (size_t)e->scn->get_x_row() * fl->y_res * sizeof(unsigned int));
    }
    return QR_OK;
}

int qrpy_scene_render_device(void *h, long long time, unsigned int *dev_frame,
                             void *stream)
{
    qrpy_engine *e = (qrpy_engine *)h;
    try
    {
        e->scn->render_device((rt_time)time, dev_frame, stream);
    }
    catch (rt_Exception &ex)
    {
        fprintf(stderr, "qrpy_scene_render_device: %s\n", ex.err);
        return QR_ERR_CUDA;
    }
    return QR_OK;
}

int qrpy_scene_next_cam(void *h)
{
    return ((qrpy_engine *)h)->scn->next_cam();
}

void qrpy_scene_update(void *h, long long time, int action)
{
    ((qrpy_engine *)h)->scn->update((rt_time)time, action);
}

void *qrpy_scene_ctx(void *h)
{
    return ((qrpy_engine *)h)->pfm->get_ctx();
}

int qrpy_scene_set_pton(void *h, int pton)
{
    return ((qrpy_engine *)h)->scn->set_pton(pton);
}

void qrpy_scene_free(void *h)
{
    qrpy_engine *e = (qrpy_engine *)h;
    if (e == NULL) return;
    delete e->scn;
    delete e->pfm;
    delete e;
}

} /* extern "C" */

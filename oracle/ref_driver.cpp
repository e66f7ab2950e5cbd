/*
 * ref_driver.cpp: headless driver for the reference engine (test oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  This program is linked against the reference
 * engine's own sources (VectorChief/QuadRay-engine core/engine, core/system,
 * core/tracer), compiled from where they lie by oracle/Makefile into
 * oracle/_ref/.  It renders the seeded synthetic scenes of
 * quadray-engine_gb300/csrc/scenegen.hpp with the reference's fp32 CPU
 * renderer (rt_Scene::render, core/engine/engine.cpp:3014) and writes the
 * frames, so that golden fixtures can be produced and the CPU restatement in
 * oracle/qr_oracle.c can be pinned.  It follows the structure of the
 * reference's own test harness (test/core_test.cpp:976-1094): build scene,
 * set options, render, read the frame.
 *
 * usage: ref_driver KIND SEED NQ W H FSAA FRAMES FLAGS OPTS OUT [THREADS]
 *                   [DEPTH] [DUMP]
 *   KIND    1 plain Whitted, 2 animated, 3 path tracer; 101-118 the
 *           reference's own test scene 1-18 (test/scenes/scn_testNN.h, as
 *           test/core_test.cpp:193-475 builds them; SEED, NQ and FLAGS are
 *           ignored), 201-218 the same scene path traced (one sample a
 *           frame, FRAMES frames accumulated: the last frame is the mean)
 *   FSAA    0 none, 2 4x
 *   FRAMES  frames rendered at t = i*16 ms; all are written (PT: accumulated)
 *   FLAGS   scenegen flags (1 = hit-ID materials)
 *   OPTS    "full", "none" or a number: runtime options (rt_Scene::set_opts)
 *   OUT     output file: FRAMES x H x W little-endian uint32 XRGB
 *   THREADS worker threads (pthread pool), default 1
 *   DEPTH   secondary-ray depth, default 10 (the compiled-in RT_STACK_DEPTH,
 *           core/tracer/tracer.h:51); the engine copies its member "depth"
 *           into every slice's s_inf per frame (core/engine/engine.cpp:2903,
 *           3667), so a smaller value is set on that member after
 *           construction (the context stack keeps its 1 + 10 levels)
 *   DUMP    if "dump", print the engine's per-surface backend fields
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <sys/time.h>

#define private public
#define protected public
#include "engine.h"
#undef private
#undef protected

#include "../quadray-engine_gb300/csrc/scenegen.hpp"

/* the reference's test scenes (test/scenes, found on the include path) */
#include "scn_test01.h"
#include "scn_test02.h"
#include "scn_test03.h"
#include "scn_test04.h"
#include "scn_test05.h"
#include "scn_test06.h"
#include "scn_test07.h"
#include "scn_test08.h"
#include "scn_test09.h"
#include "scn_test10.h"
#include "scn_test11.h"
#include "scn_test12.h"
#include "scn_test13.h"
#include "scn_test14.h"
#include "scn_test15.h"
#include "scn_test16.h"
#include "scn_test17.h"
#include "scn_test18.h"

static rt_SCENE *test_scene(int n)
{
    static rt_SCENE *const all[18] = {
        &scn_test01::sc_root, &scn_test02::sc_root, &scn_test03::sc_root,
        &scn_test04::sc_root, &scn_test05::sc_root, &scn_test06::sc_root,
        &scn_test07::sc_root, &scn_test08::sc_root, &scn_test09::sc_root,
        &scn_test10::sc_root, &scn_test11::sc_root, &scn_test12::sc_root,
        &scn_test13::sc_root, &scn_test14::sc_root, &scn_test15::sc_root,
        &scn_test16::sc_root, &scn_test17::sc_root, &scn_test18::sc_root};
    return n >= 1 && n <= 18 ? all[n - 1] : NULL;
}

static rt_pntr sys_alloc(rt_size size)
{
    rt_pntr p = malloc(size);
    if (p == NULL) throw rt_Exception("alloc failed");
    return p;
}

static rt_void sys_free(rt_pntr ptr, rt_size size)
{
    (void)size;
    free(ptr);
}

/* ---- pthread pool following the callback pattern of the reference demo
 *      (root/RooT_linux.cpp:581-760): one worker per thread index, the main
 *      thread waits for all workers of a phase ------------------------------ */

struct Pool
{
    rt_Platform *pfm;
    rt_si32 thnum;
    pthread_t *th;
    pthread_barrier_t b0, b1;
    volatile rt_si32 cmd;      /* 0 exit, 1 update, 2 render */
    volatile rt_si32 phase;
    rt_Scene *volatile scn;
    struct Arg { Pool *pool; rt_si32 index; } *args;
};

static void *pool_worker(void *p)
{
    Pool::Arg *a = (Pool::Arg *)p;
    Pool *pl = a->pool;
    for (;;)
    {
        pthread_barrier_wait(&pl->b0);
        if (pl->cmd == 0) break;
        if (pl->cmd == 1) pl->scn->update_slice(a->index, pl->phase);
        else              pl->scn->render_slice(a->index, pl->phase);
        pthread_barrier_wait(&pl->b1);
    }
    return NULL;
}

static Pool *g_pool = NULL;

static rt_pntr f_init(rt_si32 thnum, rt_Platform *pfm)
{
    Pool *pl = new Pool;
    pl->pfm = pfm;
    pl->thnum = thnum;
    pl->th = new pthread_t[thnum];
    pl->args = new Pool::Arg[thnum];
    pthread_barrier_init(&pl->b0, NULL, thnum + 1);
    pthread_barrier_init(&pl->b1, NULL, thnum + 1);
    pl->cmd = 1;
    for (rt_si32 i = 0; i < thnum; i++)
    {
        pl->args[i].pool = pl;
        pl->args[i].index = i;
        pthread_create(&pl->th[i], NULL, pool_worker, &pl->args[i]);
    }
    g_pool = pl;
    return pl;
}

static rt_void f_term(rt_pntr tdata, rt_si32 thnum)
{
    Pool *pl = (Pool *)tdata;
    pl->cmd = 0;
    pthread_barrier_wait(&pl->b0);
    for (rt_si32 i = 0; i < thnum; i++) pthread_join(pl->th[i], NULL);
    pthread_barrier_destroy(&pl->b0);
    pthread_barrier_destroy(&pl->b1);
    delete[] pl->th;
    delete[] pl->args;
    delete pl;
}

static rt_Scene *g_cur = NULL;

static rt_void f_update(rt_pntr tdata, rt_si32 thnum, rt_si32 phase)
{
    Pool *pl = (Pool *)tdata;
    (void)thnum;
    pl->scn = g_cur; pl->cmd = 1; pl->phase = phase;
    pthread_barrier_wait(&pl->b0);
    pthread_barrier_wait(&pl->b1);
}

static rt_void f_render(rt_pntr tdata, rt_si32 thnum, rt_si32 phase)
{
    Pool *pl = (Pool *)tdata;
    (void)thnum;
    pl->scn = g_cur; pl->cmd = 2; pl->phase = phase;
    pthread_barrier_wait(&pl->b0);
    pthread_barrier_wait(&pl->b1);
}

static double now_ms()
{
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return tv.tv_sec * 1000.0 + tv.tv_usec / 1000.0;
}

/* print the backend fields of one surface as hex floats (for field-by-field
 * comparison with the GB300 host flattening) */
static void dump_srf(rt_SIMD_SURFACE *s, rt_si32 idx)
{
    #define QF_(x) ((double)(x)[0])
    printf("srf %d tag %d t %d %d %d msc1 %ld amap %d %d %d %d asgn %d %d %d %d\n",
           idx, (int)s->srf_t[3], (int)s->srf_t[0], (int)s->srf_t[1],
           (int)s->srf_t[2], (long)(rt_word)s->msc_p[1],
           s->a_map[0], s->a_map[1], s->a_map[2], s->a_map[3],
           s->a_sgn[0], s->a_sgn[1], s->a_sgn[2], s->a_sgn[3]);
    printf("  pos %a %a %a\n", QF_(s->pos_x), QF_(s->pos_y), QF_(s->pos_z));
    printf("  min %a %a %a  max %a %a %a  mint %d %d %d maxt %d %d %d\n",
           QF_(s->min_x), QF_(s->min_y), QF_(s->min_z),
           QF_(s->max_x), QF_(s->max_y), QF_(s->max_z),
           s->min_t[0], s->min_t[1], s->min_t[2],
           s->max_t[0], s->max_t[1], s->max_t[2]);
    printf("  tci %a %a %a tcj %a %a %a tck %a %a %a\n",
           QF_(s->tci_x), QF_(s->tci_y), QF_(s->tci_z),
           QF_(s->tcj_x), QF_(s->tcj_y), QF_(s->tcj_z),
           QF_(s->tck_x), QF_(s->tck_y), QF_(s->tck_z));
    printf("  sci %a %a %a %a scj %a %a %a\n",
           QF_(s->sci_x), QF_(s->sci_y), QF_(s->sci_z), QF_(s->sci_w),
           QF_(s->scj_x), QF_(s->scj_y), QF_(s->scj_z));
    for (int side = 0; side < 2; side++)
    {
        rt_SIMD_MATERIAL *m = (rt_SIMD_MATERIAL *)s->mat_p[side * 2];
        printf("  mat%d props %lx ldff %a lspc %a lpow %u crfl %a ctrn %a "
               "crfr %a rfr2 %a crcp %a ext2 %a\n", side,
               (unsigned long)(rt_word)s->mat_p[side * 2 + 1],
               QF_(m->l_dff), QF_(m->l_spc), m->l_pow[0], QF_(m->c_rfl), QF_(m->c_trn),
               QF_(m->c_rfr), QF_(m->rfr_2), QF_(m->c_rcp), QF_(m->ext_2));
    }
    #undef QF_
}

static void dump_list(const char *name, rt_ELEM *e, int depth)
{
    for (; e != NULL; e = e->next)
    {
        rt_SIMD_SURFACE *s = (rt_SIMD_SURFACE *)e->simd;
        printf("%s %*s elm data %lx srf %p tag %d\n", name, depth * 2, "",
               (unsigned long)e->data, (void *)s,
               s != NULL ? (int)s->srf_t[3] : -99);
    }
}

int main(int argc, char **argv)
{
    if (argc < 11)
    {
        fprintf(stderr, "usage: %s KIND SEED NQ W H FSAA FRAMES FLAGS OPTS OUT "
                        "[THREADS] [DEPTH] [DUMP]\n", argv[0]);
        return 2;
    }
    int kind = atoi(argv[1]);
    unsigned long long seed = strtoull(argv[2], NULL, 10);
    int nq = atoi(argv[3]);
    int w = atoi(argv[4]), h = atoi(argv[5]);
    int fsaa = atoi(argv[6]);
    int frames = atoi(argv[7]);
    int flags = atoi(argv[8]);
    const char *opts = argv[9];
    const char *out = argv[10];
    int thnum = argc > 11 ? atoi(argv[11]) : 1;
    int depth = argc > 12 ? atoi(argv[12]) : 10;
    int dump = argc > 13 && strcmp(argv[13], "dump") == 0;
    if (depth < 0 || depth > 10)
    {
        fprintf(stderr, "DEPTH must be in [0, 10]\n");
        return 2;
    }

    /* file-named textures: written where the reference's load_image looks
     * (RT_PATH "data/textures/", RT_PATH = "../" in this build) */
    if (flags & QR_GEN_TEXFILE)
    {
        if (qr_gen::write_texture_files(seed, "../data/textures") != 0)
        {
            fprintf(stderr, "cannot write ../data/textures/qr_tex*.bmp\n");
            return 1;
        }
    }
    const int ref_scene = kind > 200 ? kind - 200 : kind > 100 ? kind - 100 : 0;
    const int ref_pt = kind > 200;
    qr_gen::Scene *sc = ref_scene ? NULL : qr_gen::build(kind, seed, nq, flags);
    rt_SCENE *scn = ref_scene ? test_scene(ref_scene) : &sc->scn;
    if (scn == NULL)
    {
        fprintf(stderr, "unknown scene kind %d\n", kind);
        return 2;
    }

    rt_Platform *pfm;
    if (thnum > 1)
        pfm = new rt_Platform(sys_alloc, sys_free, thnum, f_init, f_term,
                              f_update, f_render);
    else
        pfm = new rt_Platform(sys_alloc, sys_free);

    pfm->set_fsaa(fsaa == 2 ? RT_FSAA_4X : fsaa == 1 ? RT_FSAA_2X : RT_FSAA_NO);

    FILE *fo = fopen(out, "wb");
    if (fo == NULL) { perror(out); return 1; }

    double tsum = 0.0;
    try
    {
        rt_Scene *scene = new(pfm) rt_Scene(scn, w, h, w, RT_NULL, pfm);
        g_cur = scene;
        if (strcmp(opts, "none") == 0) scene->set_opts(RT_OPTS_NONE);
        else if (strcmp(opts, "full") == 0) scene->set_opts(RT_OPTS_FULL);
        else scene->set_opts((rt_si32)strtoul(opts, NULL, 0));
        if (kind == QR_SCN_PT || ref_pt) scene->set_pton(1);
        scene->depth = depth;

        /* QR_ACTIONS="a,b,...": camera action a_k (object.h:47-62) through
         * rt_Scene::update before frame k + 1, at that frame's time */
        std::vector<int> actions;
        if (getenv("QR_ACTIONS") != NULL)
        {
            const char *p = getenv("QR_ACTIONS");
            while (*p)
            {
                actions.push_back(atoi(p));
                while (*p && *p != ',') p++;
                if (*p == ',') p++;
            }
        }
        /* QR_NEXTCAM="k,...": rt_Scene::next_cam before frame k */
        std::vector<int> nextcam;
        if (getenv("QR_NEXTCAM") != NULL)
        {
            const char *p = getenv("QR_NEXTCAM");
            while (*p)
            {
                nextcam.push_back(atoi(p));
                while (*p && *p != ',') p++;
                if (*p == ',') p++;
            }
        }
        for (int f = 0; f < frames; f++)
        {
            for (size_t c = 0; c < nextcam.size(); c++)
                if (nextcam[c] == f) scene->next_cam();
            if (f > 0 && !actions.empty())
                scene->update((rt_time)f * 16, actions[(f - 1) % actions.size()]);
            double t0 = now_ms();
            scene->render((rt_time)f * 16);
            tsum += now_ms() - t0;
            rt_ui32 *fr = scene->get_frame();
            rt_si32 xr = scene->get_x_row();
            for (int y = 0; y < h; y++)
                fwrite(fr + (size_t)y * xr, sizeof(rt_ui32), w, fo);
        }

        if (dump)
        {
            printf("opts %x fsaa %d simd %d\n", scene->opts, pfm->fsaa,
                   pfm->simd_width);
            int i = 0;
            for (rt_Surface *s = scene->srf_head; s != NULL; s = s->next, i++)
                dump_srf(s->s_srf, i);
            dump_list("clist", scene->clist, 0);
            dump_list("slist", scene->slist, 0);
            for (rt_Surface *s = scene->srf_head; s != NULL; s = s->next)
            {
                printf("lgt-outer of %p\n", (void *)s->s_srf);
                dump_list("  lo", (rt_ELEM *)s->s_srf->lst_p[0], 0);
                printf("lgt-inner of %p\n", (void *)s->s_srf);
                dump_list("  li", (rt_ELEM *)s->s_srf->lst_p[2], 0);
            }
        }
        delete scene;
    }
    catch (rt_Exception &e)
    {
        fprintf(stderr, "rt_Exception: %s\n", e.err);
        return 1;
    }
    fclose(fo);
    fprintf(stderr, "ms_per_frame %.3f threads %d\n", tsum / frames, thnum);
    delete pfm;
    if (sc != NULL) delete sc;
    return 0;
}

/*
 * scene_fixture.cpp: flattens the reference's own test scenes with this
 * repository's host engine (TEST INFRASTRUCTURE ONLY).
 *
 * The reference's regression scenes (test/scenes/scn_test01.h ...
 * scn_test18.h, with their material and object libraries data/materials,
 * data/objects) are included unchanged from the reference checkout, by
 * include path, against this repository's format.h: that they compile is
 * the drop-in claim for static scene data.  Each scene is then flattened by
 * the same host code rt_Scene uses (csrc/flatten.cpp: update phases,
 * records, lists) and the flattened scene and frame parameters are written
 * to a file, which tests/golden/make_golden.py stores beside the
 * reference's own frames of the scene.  The GPU and oracle tests render
 * these records without the reference being present.
 *
 * usage: scene_fixture N W H FSAA OPTS DEPTH OUT
 *   N      test scene 1-18
 *   OPTS   "none" (RT_OPTS_NONE) or "full" (RT_OPTS_FULL), minus the
 *          scene's own opt-outs, as rt_Scene::set_opts applies them
 *   OUT    QRSF file: "QRSF", version 1, the eight counts and offsets of
 *          qr_scene_desc (nsrf nmat nlgt nelem nlelem ntex cam_off cam_num,
 *          int32), the six record arrays in that order, qr_frame_params
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "format.h"
#include "flatten.h"
#include "rt_exception.h"

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

static int put(FILE *f, const void *p, size_t n)
{
    return n == 0 || fwrite(p, 1, n, f) == n ? 0 : -1;
}

int main(int argc, char **argv)
{
    if (argc != 8)
    {
        fprintf(stderr, "usage: %s N W H FSAA OPTS DEPTH OUT\n", argv[0]);
        return 2;
    }
    rt_SCENE *scn = test_scene(atoi(argv[1]));
    const int w = atoi(argv[2]), h = atoi(argv[3]), fsaa = atoi(argv[4]);
    const int depth = atoi(argv[6]);
    if (scn == NULL || w <= 0 || h <= 0 || depth < 0 || depth > 10)
    {
        fprintf(stderr, "bad arguments\n");
        return 2;
    }
    const unsigned opts = strcmp(argv[5], "none") == 0 ? (unsigned)RT_OPTS_NONE
                                                       : (unsigned)RT_OPTS_FULL;
    try
    {
        qr::Flat fl(scn, (int)(opts & ~scn->opts), w, h, fsaa);
        fl.depth = depth;
        fl.update(0);
        qr_scene_desc d;
        qr_frame_params fp;
        fl.desc(&d);
        fl.frame_params(&fp);
        FILE *f = fopen(argv[7], "wb");
        if (f == NULL)
        {
            perror(argv[7]);
            return 1;
        }
        const int32_t hdr[10] = {0x46535251 /* "QRSF" */, 1, d.nsrf, d.nmat, d.nlgt,
                                 d.nelem, d.nlelem, d.ntex, d.cam_off, d.cam_num};
        int rc = put(f, hdr, sizeof(hdr));
        rc |= put(f, d.srf, sizeof(qr_srf) * d.nsrf);
        rc |= put(f, d.mat, sizeof(qr_mat) * d.nmat);
        rc |= put(f, d.lgt, sizeof(qr_light) * d.nlgt);
        rc |= put(f, d.elems, sizeof(qr_elem) * d.nelem);
        rc |= put(f, d.lelems, sizeof(qr_lelem) * d.nlelem);
        rc |= put(f, d.texels, sizeof(uint32_t) * d.ntex);
        rc |= put(f, &fp, sizeof(fp));
        fclose(f);
        if (rc != 0)
        {
            fprintf(stderr, "write failed\n");
            return 1;
        }
    }
    catch (rt_Exception &e)
    {
        fprintf(stderr, "rt_Exception: %s\n", e.err);
        return 1;
    }
    return 0;
}

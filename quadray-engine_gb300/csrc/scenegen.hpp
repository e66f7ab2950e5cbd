/*
 * scenegen.hpp: seeded synthetic scenes in the QuadRay scene-struct format.
 *
 * The reference publishes no scene set for its render benchmarks, so the
 * workloads are generated from a seed: random quadrics, planes, clippers,
 * lights and materials written into the scene structs of format.h.  The
 * generator only uses the struct API, so the same source builds against the
 * reference's core/engine/format.h (to render golden frames with the
 * reference engine) and against this package's format.h (to render the same
 * scene on the GPU).  Random numbers come from SplitMix64 and are turned into
 * floats with plain double arithmetic, so a seed gives bit-identical scenes
 * on x86-64 and AArch64 when built with -ffp-contract=off.
 *
 * Workloads (sizes are the caller's choice):
 *   QR_SCN_PLAIN   one ground plane z=0 plus N quadrics (sphere, cylinder,
 *                  cone, paraboloid, 1-sheet hyperboloid), each with its own
 *                  random rotation, 2 point lights, plain materials, shadows
 *   QR_SCN_ANIM    N quadrics under a 3-level array hierarchy with animated
 *                  rotations, 1-2 plane clippers per quadric, boolean-minus
 *                  pairs, 4 lights, 25% transparent (refractive) materials,
 *                  mirror/metal materials, Fresnel on
 *   QR_SCN_PT      a closed box of 5 planes with N quadrics inside, 60%
 *                  Lambertian / 25% mirror / 15% dielectric, a LIGHT-material
 *                  emitter with a light cluster, for the path tracer
 * Flag QR_GEN_SPIN makes the quadrics of QR_SCN_PLAIN spin (the animated
 * scenes of the serving workload).
 * Flag QR_GEN_IDS replaces every material with a LIGHT material whose colour
 * encodes (surface index, side), so the rendered frame is a hit-ID buffer.
 * Flag QR_GEN_TEX binds XRGB texel arrays (power-of-two sizes, as
 * RT_TEX_BIND does) to the ground of QR_SCN_PLAIN and adds three textured
 * finite planes (scaled and rotated, some by non-right angles), with
 * per-side texture scales (either sign), rotations and offsets.  Only planes
 * are textured: the reference computes texture coordinates for planes alone
 * (tracer.cpp:5647-5667) and reads stale context fields for quadrics.  Flag
 * QR_GEN_GAMMA turns the reference's gamma mode on (scene opts).  Flag
 * QR_GEN_SHAPES adds the quadric kinds the plain mix leaves out: a
 * paracylinder, a hypercylinder, a hypercylinder of zero hyp (two planes,
 * the two-plane solver), a hyperboloid of zero hyp (a double cone, the
 * apex adjustment) and a hyperbolic paraboloid, each cut to a finite
 * extent, at right-angle or other rotations.  Flag QR_GEN_ATTN gives the
 * lights an ambient share and constant, linear and quadratic attenuation.
 * Flag QR_GEN_CAMERAS adds a second camera (created last, so the
 * reference starts with it) to QR_SCN_PLAIN; rt_Scene::next_cam switches.
 * Flag QR_GEN_TEXFILE (with QR_GEN_TEX) names the textures as files
 * (qr_tex0-2.bmp, written by write_texture_files) instead of binding arrays,
 * so the renderer loads them the way the reference's load_image does.
 * These flags draw from their own random stream, so the rest of the scene
 * is unchanged.
 */
#ifndef QR_SCENEGEN_HPP
#define QR_SCENEGEN_HPP

#include <stdint.h>
#include <stdio.h>
#include <math.h>
#include <string.h>
#include <vector>
#include <deque>

/* the reference's format.h defines RT_FORMAT_H; use it when already seen */
#if !defined(RT_FORMAT_H) && !defined(QR_FORMAT_H)
#include "format.h"
#endif

#define QR_SCN_PLAIN    1
#define QR_SCN_ANIM     2
#define QR_SCN_PT       3

#define QR_GEN_IDS      (1 << 0)   /* hit-ID materials */
#define QR_GEN_NOSPEC   (1 << 1)   /* debug: no specular */
#define QR_GEN_ONELIGHT (1 << 2)   /* debug: a single light */
#define QR_GEN_TARRAY   (1 << 3)   /* QR_SCN_ANIM: keep RT_OPTS_TARRAY on */
#define QR_GEN_SPIN     (1 << 4)   /* QR_SCN_PLAIN, QR_SCN_PT: the quadrics spin
                                      (anim_spin) */
#define QR_GEN_TEX      (1 << 5)   /* QR_SCN_PLAIN: textured ground and quadrics */
#define QR_GEN_GAMMA    (1 << 6)   /* opt out of RT_OPTS_GAMMA: gamma on */
#define QR_GEN_SHAPES   (1 << 7)   /* QR_SCN_PLAIN: the other quadric kinds too */
#define QR_GEN_ATTN     (1 << 8)   /* QR_SCN_PLAIN: light ambient and attenuation */
#define QR_GEN_NOFRESNEL (1 << 9)  /* QR_SCN_ANIM: keep the default, Fresnel off */
#define QR_GEN_TEXFILE  (1 << 10)  /* with QR_GEN_TEX: textures named as BMP files */
#define QR_GEN_CAMERAS  (1 << 11)  /* QR_SCN_PLAIN: a second camera */
#define QR_GEN_RISE     (1 << 12)  /* QR_SCN_PLAIN: the quadrics turn and rise
                                      (anim_rise: their transforms move) */
#define QR_GEN_SETTLE   (1 << 13)  /* QR_SCN_PLAIN: the quadrics turn, grow
                                      from 1 s and rest at right angles from
                                      2 s (anim_settle) */

namespace qr_gen
{

/* SplitMix64 (Steele, Lea, Flood 2014) */
struct Rng
{
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    float uf(double lo, double hi) { double t = u01(); return (float)(lo + (hi - lo) * t); }
    int ui(int lo, int hi) /* inclusive */
    {
        return lo + (int)(next() % (uint64_t)(hi - lo + 1));
    }
};

static inline rt_ui32 pack_rgb(float r, float g, float b)
{
    rt_ui32 cr = (rt_ui32)(r * 255.0f + 0.5f), cg = (rt_ui32)(g * 255.0f + 0.5f),
            cb = (rt_ui32)(b * 255.0f + 0.5f);
    if (cr > 255) cr = 255;
    if (cg > 255) cg = 255;
    if (cb > 255) cb = 255;
    return (cr << 16) | (cg << 8) | cb;
}

/* a random colour, channels drawn in the order r, g, b (separate statements:
 * the evaluation order of function arguments differs between compilers and
 * targets, so no call below takes two draws as arguments) */
static inline rt_ui32 rand_rgb(Rng &r, double lo, double hi)
{
    float cr = r.uf(lo, hi);
    float cg = r.uf(lo, hi);
    float cb = r.uf(lo, hi);
    return pack_rgb(cr, cg, cb);
}

/* a random position in a box, drawn x, y, z */
static inline void rand_pos(Rng &r, float p[3], double x0, double x1, double y0,
                            double y1, double z0, double z1)
{
    p[0] = r.uf(x0, x1);
    p[1] = r.uf(y0, y1);
    p[2] = r.uf(z0, z1);
}

/*
 * Animator of QR_SCN_ANIM (rt_FUNC_ANIM3D, the reference's f_anim hook): the
 * object spins about its three axes at a constant rate.  The rotation is a
 * pure function of the frame time and of the object's position, which the
 * animator never changes: a SplitMix64 stream seeded by the position bits
 * gives the base angles U(-180,180) and the rates U[0,2] deg per frame
 * (frames are 16 ms apart).  Being stateless, it gives the same angles in
 * every engine instance that holds a copy of the scene.
 */
static inline uint64_t pos_hash(const rt_TRANSFORM3D *trm)
{
    uint64_t h = 0x51A7u;
    for (int k = 0; k < 3; k++)
    {
        uint32_t b;
        memcpy(&b, &trm->pos[k], 4);
        h = h * 0x100000001B3ull ^ b;
    }
    return h;
}

static inline float spin_angle(uint64_t h, int k, rt_time time)
{
    Rng r(h + (uint64_t)k);
    double base = -180.0 + 360.0 * r.u01();
    double rate = 2.0 * r.u01();
    double a = base + rate * ((double)time / 16.0);
    a = fmod(a + 180.0, 360.0);
    if (a < 0.0) a += 360.0;
    return (float)(a - 180.0);
}

static void anim_spin(rt_time time, rt_time last_time, rt_TRANSFORM3D *trm,
                      rt_pntr pobj)
{
    (void)last_time; (void)pobj;
    uint64_t h = pos_hash(trm);
    for (int k = 0; k < 3; k++)
        trm->rot[k] = spin_angle(h, k, time);
}

/*
 * Animator of QR_GEN_RISE: the object turns about its three axes at rates
 * that depend on the time alone (so they never stop at a multiple of 90
 * degrees at a frame time), and rises by 2 units a second of animation time
 * since the last call, a move relative to its previous position.
 */
static void anim_rise(rt_time time, rt_time last_time, rt_TRANSFORM3D *trm,
                      rt_pntr pobj)
{
    (void)pobj;
    const float t = (float)time;
    trm->rot[RT_X] = 17.0f + 0.0371f * t;
    trm->rot[RT_Y] = -23.0f + 0.0293f * t;
    trm->rot[RT_Z] = 41.0f + 0.0137f * t;
    while (trm->rot[RT_X] > 180.0f) trm->rot[RT_X] -= 360.0f;
    while (trm->rot[RT_Y] > 180.0f) trm->rot[RT_Y] -= 360.0f;
    while (trm->rot[RT_Z] > 180.0f) trm->rot[RT_Z] -= 360.0f;
    trm->pos[RT_Z] += 0.002f * (float)(time - last_time);
}

/*
 * Animator of QR_GEN_SETTLE: the object turns (as anim_rise), from 1000 ms
 * on it is scaled by 1.5, and from 2000 ms on it rests at right angles (the
 * update phases then give it no rotation of its own).
 */
static void anim_settle(rt_time time, rt_time last_time, rt_TRANSFORM3D *trm,
                        rt_pntr pobj)
{
    (void)pobj;
    const float t = (float)time;
    if (time < 2000)
    {
        trm->rot[RT_X] = 17.0f + 0.0371f * t;
        trm->rot[RT_Y] = -23.0f + 0.0293f * t;
        trm->rot[RT_Z] = 41.0f + 0.0137f * t;
    }
    else
    {
        trm->rot[RT_X] = 90.0f;
        trm->rot[RT_Y] = 0.0f;
        trm->rot[RT_Z] = -90.0f;
    }
    const float sc = time >= 1000 ? 1.5f : 1.0f;
    trm->scl[RT_X] = trm->scl[RT_Y] = trm->scl[RT_Z] = sc;
    (void)last_time;
}

/*
 * Scene storage: every struct lives in a deque so pointers stay valid while
 * the scene is built.  The scene is usable as long as the holder lives.
 */
struct Scene
{
    rt_SCENE scn;
    std::deque<rt_OBJECT>   objs;       /* individual objects (copied) */
    std::deque<std::vector<rt_OBJECT> > arrays;
    std::deque<std::vector<rt_RELATION> > rels;
    std::deque<rt_MATERIAL> mats;
    std::deque<std::vector<rt_ui32> > texs;
    std::deque<rt_CAMERA>   cams;
    std::deque<rt_LIGHT>    lgts;
    std::deque<rt_PLANE>    planes;
    std::deque<rt_CYLINDER> cyls;
    std::deque<rt_SPHERE>   sphs;
    std::deque<rt_CONE>     cones;
    std::deque<rt_PARABOLOID> pars;
    std::deque<rt_HYPERBOLOID> hyps;
    std::deque<rt_PARACYLINDER> pcyls;
    std::deque<rt_HYPERCYLINDER> hcyls;
    std::deque<rt_HYPERPARABOLOID> hpars;
    int nsurf;          /* surfaces generated, in generation order */
    int flags;

    Scene() : nsurf(0), flags(0) { memset(&scn, 0, sizeof(scn)); }

    rt_MATERIAL *material(int tag, rt_ui32 col, float dff, float spc, float pw,
                          float rfl, float trn, float rfr, float ext)
    {
        rt_MATERIAL m;
        memset(&m, 0, sizeof(m));
        m.tag = tag;
        m.tex.tag = RT_TEX_PCOLOR;
        m.tex.col.val = col;
        m.lgt[0] = dff; m.lgt[1] = spc; m.lgt[2] = pw; m.lgt[3] = 0.0f;
        m.prp[0] = rfl; m.prp[1] = trn; m.prp[2] = rfr; m.prp[3] = ext;
        mats.push_back(m);
        return &mats.back();
    }

    /* material m with an XRGB texel array of xd x yd (powers of two) bound
     * in place of its plain colour */
    rt_MATERIAL *textured(const rt_MATERIAL *m, const rt_ui32 *tx, int xd, int yd)
    {
        rt_MATERIAL t = *m;
        t.tex.col.val = 0;
        t.tex.ptex = (rt_void *)tx;
        t.tex.x_dim = xd;
        t.tex.y_dim = yd;
        mats.push_back(t);
        return &mats.back();
    }

    /* material m with a texture named as a file (RT_TEX with a name in
     * ptex and no dimensions: the engine loads it) */
    rt_MATERIAL *textured_file(const rt_MATERIAL *m, const char *name)
    {
        rt_MATERIAL t = *m;
        t.tex.col.val = 0;
        t.tex.ptex = (rt_void *)name;
        t.tex.x_dim = 0;
        t.tex.y_dim = 0;
        mats.push_back(t);
        return &mats.back();
    }

    /* hit-ID material: colour = (surface index + 1) * 2 + side */
    rt_MATERIAL *id_material(int sidx, int side)
    {
        rt_ui32 id = (rt_ui32)((sidx + 1) * 2 + side) & 0xFFFFFF;
        return material(RT_MAT_LIGHT, id, 1.0f, 0.0f, 1.0f, 0.0f, 0.0f, 1.0f, 0.0f);
    }

    void side(rt_SIDE *sd, rt_MATERIAL *m)
    {
        sd->scl[0] = 1.0f; sd->scl[1] = 1.0f; sd->rot = 0.0f;
        sd->pos[0] = 0.0f; sd->pos[1] = 0.0f; sd->pmat = m;
    }

    void srf_init(rt_SURFACE *s, rt_MATERIAL *mo, rt_MATERIAL *mi)
    {
        for (int k = 0; k < 3; k++) { s->min[k] = -RT_INF; s->max[k] = +RT_INF; }
        if (flags & QR_GEN_IDS)
        {
            mo = id_material(nsurf, 0);
            mi = id_material(nsurf, 1);
        }
        side(&s->side_outer, mo);
        side(&s->side_inner, mi);
        nsurf++;
    }

    static void trm_set(rt_TRANSFORM3D *t, float sx, float sy, float sz,
                        float rx, float ry, float rz, float px, float py, float pz)
    {
        t->scl[0] = sx; t->scl[1] = sy; t->scl[2] = sz;
        t->rot[0] = rx; t->rot[1] = ry; t->rot[2] = rz;
        t->pos[0] = px; t->pos[1] = py; t->pos[2] = pz;
    }

    static rt_OBJECT obj(int tag, void *p, int num)
    {
        rt_OBJECT o;
        memset(&o, 0, sizeof(o));
        trm_set(&o.trm, 1, 1, 1, 0, 0, 0, 0, 0, 0);
        o.obj.tag = tag;
        o.obj.pobj = p;
        o.obj.obj_num = num;
        return o;
    }

    rt_OBJECT camera(float px, float py, float pz, float rx, float ry, float rz,
                     float pov, rt_ui32 amb_col, float amb_lum)
    {
        rt_CAMERA c;
        memset(&c, 0, sizeof(c));
        c.tag = RT_CAM_PLAIN;
        c.col.val = amb_col;
        c.lum[0] = amb_lum;
        c.vpt[0] = pov;
        /* movement and rotation steps per unit of time (50 ms) for the
         * camera actions of rt_Scene::update */
        c.dps[0] = 0.6f; c.dps[1] = 0.8f; c.dps[2] = 0.4f;
        c.drt[0] = 3.0f; c.drt[1] = 2.0f; c.drt[2] = 0.0f;
        cams.push_back(c);
        rt_OBJECT o = obj(RT_TAG_CAMERA, &cams.back(), 1);
        trm_set(&o.trm, 1, 1, 1, rx, ry, rz, px, py, pz);
        return o;
    }

    rt_OBJECT light(float px, float py, float pz, rt_ui32 col, float lamb,
                    float lsrc, float a_cnt, float a_lnr, float a_qdr)
    {
        rt_LIGHT l;
        memset(&l, 0, sizeof(l));
        l.tag = RT_LGT_PLAIN;
        l.col.val = col;
        l.lum[0] = lamb; l.lum[1] = lsrc;
        l.atn[0] = 0.0f; l.atn[1] = a_cnt; l.atn[2] = a_lnr; l.atn[3] = a_qdr;
        lgts.push_back(l);
        rt_OBJECT o = obj(RT_TAG_LIGHT, &lgts.back(), 1);
        o.trm.pos[0] = px; o.trm.pos[1] = py; o.trm.pos[2] = pz;
        return o;
    }

    rt_OBJECT array(const std::vector<rt_OBJECT> &v,
                    const std::vector<rt_RELATION> *rel = RT_NULL)
    {
        arrays.push_back(v);
        rt_OBJECT o = obj(RT_TAG_ARRAY, arrays.back().data(), (int)v.size());
        if (rel != RT_NULL && !rel->empty())
        {
            rels.push_back(*rel);
            o.obj.prel = rels.back().data();
            o.obj.rel_num = (int)rel->size();
        }
        return o;
    }

    rt_OBJECT plane(rt_MATERIAL *mo, rt_MATERIAL *mi)
    {
        rt_PLANE p; memset(&p, 0, sizeof(p));
        srf_init(&p.srf, mo, mi);
        planes.push_back(p);
        return obj(RT_TAG_PLANE, &planes.back(), 1);
    }

    /* quadric of a given tag with shape parameters a, b and K-extent */
    rt_OBJECT quadric(int tag, float a, float b, float kmin, float kmax,
                      rt_MATERIAL *mo, rt_MATERIAL *mi)
    {
        rt_SURFACE *s = RT_NULL;
        void *p = RT_NULL;
        switch (tag)
        {
        case RT_TAG_CYLINDER:
        { rt_CYLINDER q; memset(&q, 0, sizeof(q)); q.rad = a; cyls.push_back(q);
          s = &cyls.back().srf; p = &cyls.back(); } break;
        case RT_TAG_SPHERE:
        { rt_SPHERE q; memset(&q, 0, sizeof(q)); q.rad = a; sphs.push_back(q);
          s = &sphs.back().srf; p = &sphs.back(); } break;
        case RT_TAG_CONE:
        { rt_CONE q; memset(&q, 0, sizeof(q)); q.rat = a; cones.push_back(q);
          s = &cones.back().srf; p = &cones.back(); } break;
        case RT_TAG_PARABOLOID:
        { rt_PARABOLOID q; memset(&q, 0, sizeof(q)); q.par = a; pars.push_back(q);
          s = &pars.back().srf; p = &pars.back(); } break;
        case RT_TAG_HYPERBOLOID:
        { rt_HYPERBOLOID q; memset(&q, 0, sizeof(q)); q.rat = a; q.hyp = b;
          hyps.push_back(q); s = &hyps.back().srf; p = &hyps.back(); } break;
        case RT_TAG_PARACYLINDER:
        { rt_PARACYLINDER q; memset(&q, 0, sizeof(q)); q.par = a;
          pcyls.push_back(q); s = &pcyls.back().srf; p = &pcyls.back(); } break;
        case RT_TAG_HYPERCYLINDER:
        { rt_HYPERCYLINDER q; memset(&q, 0, sizeof(q)); q.rat = a; q.hyp = b;
          hcyls.push_back(q); s = &hcyls.back().srf; p = &hcyls.back(); } break;
        case RT_TAG_HYPERPARABOLOID:
        { rt_HYPERPARABOLOID q; memset(&q, 0, sizeof(q)); q.pr1 = a; q.pr2 = b;
          hpars.push_back(q); s = &hpars.back().srf; p = &hpars.back(); } break;
        default: return obj(RT_TAG_ARRAY, RT_NULL, 0);
        }
        srf_init(s, mo, mi);
        s->min[RT_K] = kmin;
        s->max[RT_K] = kmax;
        return obj(tag, p, 1);
    }
};

static const int plain_tags[5] =
{
    RT_TAG_SPHERE, RT_TAG_CYLINDER, RT_TAG_CONE, RT_TAG_PARABOLOID,
    RT_TAG_HYPERBOLOID
};

/* random quadric of one of the five plain kinds, radii/scales U[0.5,2] */
static rt_OBJECT random_quadric(Scene &sc, Rng &r, rt_MATERIAL *mo,
                                rt_MATERIAL *mi, int *ptag)
{
    int tag = plain_tags[r.ui(0, 4)];
    float a = r.uf(0.5, 2.0), b = 0.0f, kmin = -RT_INF, kmax = +RT_INF;
    switch (tag)
    {
    case RT_TAG_SPHERE: break;
    case RT_TAG_CYLINDER:
        kmax = r.uf(0.5, 2.0); kmin = -kmax; break;
    case RT_TAG_CONE:
        a = r.uf(0.3, 1.0); kmax = r.uf(0.5, 2.0); kmin = -kmax; break;
    case RT_TAG_PARABOLOID:
        kmax = r.uf(0.5, 2.0); break;
    case RT_TAG_HYPERBOLOID:
        a = r.uf(0.3, 1.0); b = r.uf(0.25, 1.5);
        kmax = r.uf(0.5, 2.0); kmin = -kmax; break;
    }
    *ptag = tag;
    return sc.quadric(tag, a, b, kmin, kmax, mo, mi);
}

static rt_MATERIAL *random_plain(Scene &sc, Rng &r)
{
    rt_ui32 col = rand_rgb(r, 0.2, 1.0);
    float dff = r.uf(0.2, 0.9);
    float spc = r.uf(0.1, 0.6);
    float pw  = (float)r.ui(8, 64);
    if (sc.flags & QR_GEN_NOSPEC) spc = 0.0f;
    return sc.material(RT_MAT_PLAIN, col, dff, spc, pw, 0.0f, 0.0f, 1.0f, 0.0f);
}

/* camera at (0,-25,8) looking at the origin: rotation about X only,
 * hor = +X, nrm = direction to the origin */
static rt_OBJECT look_camera(Scene &sc, float px, float py, float pz,
                             float fov_deg)
{
    double dy = -py, dz = -pz;
    double ang = atan2(-dy, dz) * 180.0 / RT_PI;  /* nrm = (0,-sin,cos) */
    float pov = (float)(0.5 / tan(0.5 * fov_deg * RT_PI / 180.0));
    return sc.camera(px, py, pz, (float)ang, 0.0f, 0.0f, pov, 0xFFFFFF, 0.1f);
}

/* texture set of QR_GEN_TEX: a checker of two colours with a distinct low
 * nibble per texel, so a wrong texel index changes the colour */
static void make_textures(Scene &sc, Rng &r)
{
    static const int dims[3][2] = {{16, 16}, {32, 8}, {8, 64}};
    for (int k = 0; k < 3; k++)
    {
        const rt_ui32 a = rand_rgb(r, 0.2, 1.0), b = rand_rgb(r, 0.2, 1.0);
        std::vector<rt_ui32> t((size_t)dims[k][0] * dims[k][1]);
        for (int y = 0; y < dims[k][1]; y++)
            for (int x = 0; x < dims[k][0]; x++)
            {
                const rt_ui32 n = (rt_ui32)((x * 7 + y * 13) & 0x0F);
                t[(size_t)y * dims[k][0] + x] = (((x ^ y) & 1) ? a : b) ^ (n * 0x010101u);
            }
        sc.texs.push_back(t);
    }
}

static float r_half(Rng &r) { return r.uf(1.5, 3.0); }

/* the texture set of a seed as 24-bit BMP files qr_tex0-2.bmp in dir (rows
 * in array order, so loading them gives the arrays back): returns 0, or -1
 * when a file cannot be written */
static int write_texture_files(uint64_t seed, const char *dir)
{
    static const int dims[3][2] = {{16, 16}, {32, 8}, {8, 64}};
    Scene sc;
    Rng rt(seed ^ 0x7E57C0DE5EEDull);
    make_textures(sc, rt);
    for (int k = 0; k < 3; k++)
    {
        char path[4096];
        snprintf(path, sizeof(path), "%s/qr_tex%d.bmp", dir, k);
        FILE *f = fopen(path, "wb");
        if (f == NULL) return -1;
        const int w = dims[k][0], h = dims[k][1], row = (w * 3 + 3) & ~3;
        const unsigned size = 54u + (unsigned)(row * h), img = (unsigned)(row * h);
        unsigned char hd[54];
        memset(hd, 0, sizeof(hd));
        const unsigned v[6] = {size, 0u, 54u, 40u, (unsigned)w, (unsigned)h};
        const int at[6] = {2, 6, 10, 14, 18, 22};
        hd[0] = 'B'; hd[1] = 'M';
        for (int i = 0; i < 6; i++)
            for (int b = 0; b < 4; b++) hd[at[i] + b] = (unsigned char)(v[i] >> (8 * b));
        hd[26] = 1; hd[28] = 24;
        for (int b = 0; b < 4; b++) hd[34 + b] = (unsigned char)(img >> (8 * b));
        fwrite(hd, 1, 54, f);
        std::vector<unsigned char> line((size_t)row, 0);
        for (int y = 0; y < h; y++)
        {
            for (int x = 0; x < w; x++)
            {
                const rt_ui32 p = sc.texs[k][(size_t)y * w + x];
                line[x * 3 + 0] = (unsigned char)(p & 0xFF);
                line[x * 3 + 1] = (unsigned char)((p >> 8) & 0xFF);
                line[x * 3 + 2] = (unsigned char)((p >> 16) & 0xFF);
            }
            fwrite(line.data(), 1, line.size(), f);
        }
        if (fclose(f) != 0) return -1;
    }
    return 0;
}

/* bind texture k of the set to both sides of surface s with side
 * transforms drawn from r (scale, right-angle or other rotation, offset) */
static void texture_sides(Scene &sc, Rng &r, rt_SURFACE *s, int k)
{
    static const int dims[3][2] = {{16, 16}, {32, 8}, {8, 64}};
    static const float rots[5] = {0.0f, 90.0f, -90.0f, 180.0f, 30.0f};
    const rt_ui32 *tx = sc.texs[k].data();
    rt_SIDE *sd[2] = {&s->side_outer, &s->side_inner};
    for (int i = 0; i < 2; i++)
    {
        float v[5];
        v[0] = r.uf(0.5, 2.0);
        v[0] = r.ui(0, 3) == 0 ? -v[0] : v[0];
        v[1] = r.uf(0.5, 2.0);
        v[1] = r.ui(0, 3) == 0 ? -v[1] : v[1];
        v[2] = rots[r.ui(0, 4)];
        v[3] = r.uf(-1.0, 1.0);
        v[4] = r.uf(-1.0, 1.0);
        /* hit-ID scenes keep their ID materials (same draws, same scene) */
        if (sc.flags & QR_GEN_IDS) continue;
        static const char *const files[3] = {"qr_tex0.bmp", "qr_tex1.bmp", "qr_tex2.bmp"};
        sd[i]->pmat = (sc.flags & QR_GEN_TEXFILE) ? sc.textured_file(sd[i]->pmat, files[k])
                                                  : sc.textured(sd[i]->pmat, tx, dims[k][0],
                                                                dims[k][1]);
        sd[i]->scl[0] = v[0];
        sd[i]->scl[1] = v[1];
        sd[i]->rot = v[2];
        sd[i]->pos[0] = v[3];
        sd[i]->pos[1] = v[4];
    }
}

/* QR_SCN_PLAIN: ground plane + nq quadrics + 2 lights */
static void build_plain(Scene &sc, uint64_t seed, int nq, int nl)
{
    Rng rt(seed ^ 0x7E57C0DE5EEDull);
    if (sc.flags & QR_GEN_TEX) make_textures(sc, rt);
    Rng ra(seed ^ 0xA77E0A7E0ull);
    Rng r(seed);
    std::vector<rt_OBJECT> root;
    root.push_back(look_camera(sc, 0.0f, -25.0f, 8.0f, 60.0f));
    for (int i = 0; i < nl; i++)
    {
        float px = r.uf(-15, 15), py = r.uf(-15, 15), pz = r.uf(8, 15);
        rt_ui32 col = rand_rgb(r, 0.3, 1.0);
        if ((sc.flags & QR_GEN_ONELIGHT) && i > 0) continue;
        float lamb = 0.0f, lsrc = 1.0f, ac = 0.0f, al = 0.0f, aq = 0.0f;
        if (sc.flags & QR_GEN_ATTN)
        {
            lamb = ra.uf(0.0, 0.3);
            lsrc = ra.uf(2.0, 6.0);
            ac = ra.uf(0.5, 1.5);
            al = ra.uf(0.0, 0.1);
            aq = ra.uf(0.0, 0.02);
        }
        root.push_back(sc.light(px, py, pz, col, lamb, lsrc, ac, al, aq));
    }
    rt_MATERIAL *gm = sc.material(RT_MAT_PLAIN, 0xB0B0A8, 0.8f,
                                  (sc.flags & QR_GEN_NOSPEC) ? 0.0f : 0.2f, 16.0f,
                                  0.0f, 0.0f, 1.0f, 0.0f);
    root.push_back(sc.plane(gm, gm));
    if (sc.flags & QR_GEN_TEX)
        texture_sides(sc, rt, &((rt_PLANE *)root.back().obj.pobj)->srf, 0);
    for (int i = 0; i < nq; i++)
    {
        rt_MATERIAL *m = random_plain(sc, r);
        int tag;
        rt_OBJECT q = random_quadric(sc, r, m, m, &tag);
        float px = r.uf(-10, 10), py = r.uf(-10, 10), pz = r.uf(0.5, 5);
        float rx = r.uf(-180, 180), ry = r.uf(-180, 180), rz = r.uf(-180, 180);
        Scene::trm_set(&q.trm, 1, 1, 1, rx, ry, rz, px, py, pz);
        if (sc.flags & QR_GEN_SPIN) q.f_anim = anim_spin;
        if (sc.flags & QR_GEN_RISE) q.f_anim = anim_rise;
        if (sc.flags & QR_GEN_SETTLE) q.f_anim = anim_settle;
        root.push_back(q);
    }
    if (sc.flags & QR_GEN_SHAPES)
    {
        Rng rs(seed ^ 0x5A4E5EC0DE11ull);
        static const int tags[5] = {RT_TAG_PARACYLINDER, RT_TAG_HYPERCYLINDER,
                                    RT_TAG_HYPERCYLINDER, RT_TAG_HYPERBOLOID,
                                    RT_TAG_HYPERPARABOLOID};
        for (int k = 0; k < 5; k++)
        {
            rt_MATERIAL *m = random_plain(sc, rs);
            float a = rs.uf(0.4, 1.2), b = 0.0f;
            if (k == 1) b = rs.uf(0.25, 1.0);           /* hypercylinder */
            if (k == 4) b = rs.uf(0.5, 2.0);            /* saddle: pr2 */
            const float ke = rs.uf(0.8, 2.0);
            rt_OBJECT q = sc.quadric(tags[k], a, b, k == 4 ? -RT_INF : -ke,
                                     k == 4 ? +RT_INF : +ke, m, m);
            rt_SURFACE *sf = (rt_SURFACE *)q.obj.pobj;
            if (k == 0 || k == 4)
            {
                /* open in I (paracylinder) or I and J (saddle): cut */
                const float ie = rs.uf(1.0, 2.5), je = rs.uf(1.0, 2.5);
                sf->min[RT_I] = -ie; sf->max[RT_I] = +ie;
                if (k == 4) { sf->min[RT_J] = -je; sf->max[RT_J] = +je; }
            }
            const int right = rs.ui(0, 1);
            float rx = right ? 90.0f * (float)rs.ui(-2, 2) : rs.uf(-180, 180);
            float ry = right ? 90.0f * (float)rs.ui(-2, 2) : rs.uf(-180, 180);
            float rz = right ? 90.0f * (float)rs.ui(-2, 2) : rs.uf(-180, 180);
            const float px = rs.uf(-8, 8), py = rs.uf(-4, 8), pz = rs.uf(1.0, 4.0);
            Scene::trm_set(&q.trm, 1, 1, 1, rx, ry, rz, px, py, pz);
            root.push_back(q);
        }
    }
    if (sc.flags & QR_GEN_TEX)
    {
        /* three textured walls: finite planes, scaled, turned about two
         * axes (right angles or not), facing the camera's side */
        static const float turns[4] = {90.0f, -90.0f, 60.0f, 105.0f};
        for (int k = 0; k < 3; k++)
        {
            rt_MATERIAL *m = random_plain(sc, rt);
            rt_OBJECT w = sc.plane(m, m);
            rt_PLANE *pl = (rt_PLANE *)w.obj.pobj;
            pl->srf.min[RT_I] = -r_half(rt); pl->srf.max[RT_I] = +r_half(rt);
            pl->srf.min[RT_J] = -r_half(rt); pl->srf.max[RT_J] = +r_half(rt);
            const float sx = rt.uf(0.6, 1.6), sy = rt.uf(0.6, 1.6);
            const float rx = turns[rt.ui(0, 3)], rz = rt.uf(-40, 40);
            const float px = rt.uf(-8, 8), py = rt.uf(-4, 8), pz = rt.uf(1.5, 4);
            Scene::trm_set(&w.trm, sx, sy, 1, rx, 0, rz, px, py, pz);
            texture_sides(sc, rt, &pl->srf, k);
            root.push_back(w);
        }
    }
    if (sc.flags & QR_GEN_CAMERAS)
        root.push_back(sc.camera(14.0f, -18.0f, 6.0f, -72.0f, 0.0f, 38.0f, 0.7f,
                                 0xE0E8FF, 0.15f));
    rt_OBJECT ro = sc.array(root);
    sc.scn.root = ro.obj;
    sc.scn.opts = (sc.flags & QR_GEN_GAMMA) ? RT_OPTS_GAMMA : 0;
    sc.scn.lock = RT_NULL;
}

/* material of QR_SCN_ANIM objects: 25% transparent dielectric (relative
 * index 1/n outside, n inside, n = U[1.3,1.6]), 15% metal, 15% reflective
 * plain, the rest plain; *inner receives the inner side's material */
static rt_MATERIAL *random_anim_material(Scene &sc, Rng &r, rt_MATERIAL **inner)
{
    double u = r.u01();
    rt_ui32 col = rand_rgb(r, 0.2, 1.0);
    float dff = r.uf(0.2, 0.9);
    float spc = r.uf(0.1, 0.6);
    float pw  = (float)r.ui(8, 64);
    if (sc.flags & QR_GEN_NOSPEC) spc = 0.0f;
    if (u < 0.25)
    {
        float n = r.uf(1.3, 1.6), trn = r.uf(0.6, 0.9);
        rt_MATERIAL *mo = sc.material(RT_MAT_PLAIN, col, dff, spc, pw,
                                      0.0f, trn, 1.0f / n, 0.0f);
        *inner = sc.material(RT_MAT_PLAIN, col, dff, spc, pw, 0.0f, trn, n, 0.0f);
        return mo;
    }
    if (u < 0.40)
    {
        float rfl = r.uf(0.3, 0.7), ext = r.uf(2.0, 9.0);
        rt_MATERIAL *mo = sc.material(RT_MAT_METAL, col, 1.0f, spc, pw,
                                      rfl, 0.0f, 1.0f, ext);
        *inner = sc.material(RT_MAT_PLAIN, 0x808080, dff, 0.0f, 1.0f,
                             0.0f, 0.0f, 1.0f, 0.0f);
        return mo;
    }
    float rfl = u < 0.55 ? r.uf(0.2, 0.5) : 0.0f;
    rt_MATERIAL *mo = sc.material(RT_MAT_PLAIN, col, dff, spc, pw, rfl, 0.0f, 1.0f, 0.0f);
    *inner = mo;
    return mo;
}

/* a transform that is "trivial" in the reference's sense (multiples of 90
 * degrees and a translation) placing a plane across local axis a (0 I, 1 J,
 * 2 K) at offset d, facing +a or -a */
static void axis_plane_trm(rt_TRANSFORM3D *t, int a, int flip, float d)
{
    float rx = 0.0f, ry = 0.0f;
    if (a == 0) ry = flip ? -90.0f : 90.0f;
    else if (a == 1) rx = flip ? 90.0f : -90.0f;
    else rx = flip ? 180.0f : 0.0f;
    Scene::trm_set(t, 1, 1, 1, rx, ry, 0, a == 0 ? d : 0.0f, a == 1 ? d : 0.0f,
                   a == 2 ? d : 0.0f);
}

/* QR_SCN_ANIM: ground plane, 4 lights, and a 3-level hierarchy of spinning
 * arrays (4 clusters x 4 groups x nq/16 items); each item is a quadric cut
 * by 1-2 axis planes (RT_REL_MINUS_INNER/OUTER) whose caps are clipped back
 * to the quadric's inside (RT_REL_MINUS_OUTER), and each cluster holds 2
 * boolean-minus pairs (a sphere drilled by a cylinder) */
static void build_anim(Scene &sc, uint64_t seed, int nq)
{
    Rng r(seed);
    std::vector<rt_OBJECT> root;
    root.push_back(look_camera(sc, 0.0f, -25.0f, 8.0f, 60.0f));
    for (int i = 0; i < 4; i++)
    {
        float px = r.uf(-15, 15), py = r.uf(-15, 15), pz = r.uf(8, 15);
        rt_ui32 col = rand_rgb(r, 0.3, 1.0);
        if ((sc.flags & QR_GEN_ONELIGHT) && i > 0) continue;
        root.push_back(sc.light(px, py, pz, col, 0.0f, 0.6f, 0.0f, 0.0f, 0.0f));
    }
    rt_MATERIAL *gm = sc.material(RT_MAT_PLAIN, 0xB0B0A8, 0.8f,
                                  (sc.flags & QR_GEN_NOSPEC) ? 0.0f : 0.2f, 16.0f,
                                  0.25f, 0.0f, 1.0f, 0.0f);
    root.push_back(sc.plane(gm, gm));

    int per_group = nq / 16 > 0 ? nq / 16 : 1;
    for (int c = 0; c < 4; c++)
    {
        std::vector<rt_OBJECT> cluster;
        for (int g = 0; g < 4; g++)
        {
            std::vector<rt_OBJECT> group;
            for (int i = 0; i < per_group; i++)
            {
                std::vector<rt_OBJECT> item;
                std::vector<rt_RELATION> rel;
                rt_MATERIAL *mi, *mo = random_anim_material(sc, r, &mi);
                int tag;
                item.push_back(random_quadric(sc, r, mo, mi, &tag));
                int np = r.ui(1, 2);
                for (int j = 0; j < np; j++)
                {
                    rt_MATERIAL *pi, *po = random_anim_material(sc, r, &pi);
                    rt_OBJECT p = sc.plane(po, pi);
                    int a = r.ui(0, 2), flip = r.ui(0, 1);
                    axis_plane_trm(&p.trm, a, flip, r.uf(-0.6, 0.6));
                    rt_PLANE *pl = (rt_PLANE *)p.obj.pobj;
                    pl->srf.min[RT_I] = -2.5f; pl->srf.max[RT_I] = +2.5f;
                    pl->srf.min[RT_J] = -2.5f; pl->srf.max[RT_J] = +2.5f;
                    item.push_back(p);
                    rt_RELATION cut = {0, r.ui(0, 1) ? RT_REL_MINUS_INNER
                                                     : RT_REL_MINUS_OUTER, j + 1};
                    rt_RELATION cap = {j + 1, RT_REL_MINUS_OUTER, 0};
                    rel.push_back(cut);
                    rel.push_back(cap);
                }
                rt_OBJECT it = sc.array(item, &rel);
                float ip[3];
                rand_pos(r, ip, -1.5, 1.5, -1.5, 1.5, -1.0, 1.0);
                Scene::trm_set(&it.trm, 1, 1, 1, 0, 0, 0, ip[0], ip[1], ip[2]);
                it.f_anim = anim_spin;
                group.push_back(it);
            }
            rt_OBJECT go = sc.array(group);
            float gp[3];
            rand_pos(r, gp, -3.0, 3.0, -3.0, 3.0, -0.5, 0.5);
            Scene::trm_set(&go.trm, 1, 1, 1, 0, 0, 0, gp[0], gp[1], gp[2]);
            go.f_anim = anim_spin;
            cluster.push_back(go);
        }
        for (int b = 0; b < 2; b++)
        {
            std::vector<rt_OBJECT> pair;
            std::vector<rt_RELATION> rel;
            rt_MATERIAL *ai, *ao = random_anim_material(sc, r, &ai);
            rt_MATERIAL *bi, *bo = random_anim_material(sc, r, &bi);
            float ra = r.uf(0.8, 1.5);
            pair.push_back(sc.quadric(RT_TAG_SPHERE, ra, 0.0f, -RT_INF, +RT_INF, ao, ai));
            rt_OBJECT cyl = sc.quadric(RT_TAG_CYLINDER, ra * r.uf(0.3, 0.6), 0.0f,
                                       -RT_INF, +RT_INF, bo, bi);
            axis_plane_trm(&cyl.trm, r.ui(0, 2), 0, 0.0f);
            pair.push_back(cyl);
            rt_RELATION drill = {0, RT_REL_MINUS_INNER, 1};
            rt_RELATION wall = {1, RT_REL_MINUS_OUTER, 0};
            rel.push_back(drill);
            rel.push_back(wall);
            rt_OBJECT po = sc.array(pair, &rel);
            float pp[3];
            rand_pos(r, pp, -3.0, 3.0, -3.0, 3.0, 0.5, 1.5);
            Scene::trm_set(&po.trm, 1, 1, 1, 0, 0, 0, pp[0], pp[1], pp[2]);
            po.f_anim = anim_spin;
            cluster.push_back(po);
        }
        rt_OBJECT co = sc.array(cluster);
        float cp[3];
        rand_pos(r, cp, -9.0, 9.0, -9.0, 9.0, 2.5, 4.0);
        Scene::trm_set(&co.trm, 1, 1, 1, 0, 0, 0, cp[0], cp[1], cp[2]);
        co.f_anim = anim_spin;
        root.push_back(co);
    }
    rt_OBJECT ro = sc.array(root);
    sc.scn.root = ro.obj;
    /* opt-outs of the reference's default options (rt_SCENE.opts): Fresnel
     * on, and no array-level transform nodes (RT_OPTS_TARRAY), under which
     * the reference's per-surface shadow and secondary-ray lists of this
     * spinning hierarchy lose occluders and candidates (its frame then
     * departs from its own unculled render); QR_GEN_TARRAY keeps it on,
     * QR_GEN_NOFRESNEL the reference's default (no Fresnel terms) */
    sc.scn.opts = (sc.flags & QR_GEN_NOFRESNEL) ? 0 : RT_OPTS_FRESNEL;
    if ((sc.flags & QR_GEN_TARRAY) == 0) sc.scn.opts |= RT_OPTS_TARRAY;
    sc.scn.lock = RT_NULL;
}

/* camera at p looking at t, both in one x = const plane (rotation about X
 * only, as look_camera) */
static rt_OBJECT camera_at(Scene &sc, float px, float py, float pz, float ty,
                           float tz, float fov_deg, float amb_lum)
{
    double dy = ty - py, dz = tz - pz;
    double ang = atan2(-dy, dz) * 180.0 / RT_PI;
    float pov = (float)(0.5 / tan(0.5 * fov_deg * RT_PI / 180.0));
    return sc.camera(px, py, pz, (float)ang, 0.0f, 0.0f, pov, 0xFFFFFF, amb_lum);
}

/* a box wall: plane through p with rotation r (multiples of 90 degrees, so
 * the surface maps to the axes), clipped to [-a, a] x [-b, b] in its I, J */
static rt_OBJECT wall(Scene &sc, rt_MATERIAL *m, float rx, float ry, float px,
                      float py, float pz, float a, float b)
{
    rt_OBJECT o = sc.plane(m, m);
    rt_PLANE *pl = (rt_PLANE *)o.obj.pobj;
    pl->srf.min[RT_I] = -a; pl->srf.max[RT_I] = +a;
    pl->srf.min[RT_J] = -b; pl->srf.max[RT_J] = +b;
    Scene::trm_set(&o.trm, 1, 1, 1, rx, ry, 0, px, py, pz);
    return o;
}

/* QR_SCN_PT: path-tracer scene.  A closed box of 5 planes (x = +-10,
 * y = 20, z = 0, z = 12; the front y = 0 is where the camera looks in) with
 * red / green side walls, nq quadrics inside (60% Lambertian, 25% mirror,
 * 15% dielectric of index 1.5) and a light cluster: one array holding 16
 * point lights and a LIGHT-material sphere, whose emission is the cluster's
 * accumulated light colour x 100 (core/engine/object.cpp:1346-1375) */
static void build_pt(Scene &sc, uint64_t seed, int nq)
{
    Rng r(seed);
    const float bw = 10.0f, bd = 20.0f, bh = 12.0f;
    std::vector<rt_OBJECT> root;
    root.push_back(camera_at(sc, 0.0f, -14.0f, 6.0f, 10.0f, 6.0f, 60.0f, 0.05f));

    rt_MATERIAL *white = sc.material(RT_MAT_PLAIN, 0xC8C8C8, 0.9f, 0.0f, 1.0f,
                                     0.0f, 0.0f, 1.0f, 0.0f);
    rt_MATERIAL *red = sc.material(RT_MAT_PLAIN, 0xC03028, 0.9f, 0.0f, 1.0f,
                                   0.0f, 0.0f, 1.0f, 0.0f);
    rt_MATERIAL *green = sc.material(RT_MAT_PLAIN, 0x30B040, 0.9f, 0.0f, 1.0f,
                                     0.0f, 0.0f, 1.0f, 0.0f);
    root.push_back(wall(sc, white, 0.0f, 0.0f, 0.0f, 0.5f * bd, 0.0f, bw, 0.5f * bd));
    root.push_back(wall(sc, white, 180.0f, 0.0f, 0.0f, 0.5f * bd, bh, bw, 0.5f * bd));
    root.push_back(wall(sc, red, 0.0f, 90.0f, -bw, 0.5f * bd, 0.5f * bh, 0.5f * bh, 0.5f * bd));
    root.push_back(wall(sc, green, 0.0f, -90.0f, bw, 0.5f * bd, 0.5f * bh, 0.5f * bh, 0.5f * bd));
    root.push_back(wall(sc, white, 90.0f, 0.0f, 0.0f, bd, 0.5f * bh, bw, 0.5f * bh));

    /* light cluster */
    std::vector<rt_OBJECT> cluster;
    for (int i = 0; i < 16; i++)
    {
        float lx = -0.6f + 0.4f * (float)(i & 3);
        float ly = -0.6f + 0.4f * (float)(i >> 2);
        if ((sc.flags & QR_GEN_ONELIGHT) && i > 0) continue;
        cluster.push_back(sc.light(lx, ly, 0.0f, 0xFFF4E8, 0.0f, 0.025f,
                                   0.0f, 0.0f, 0.0f));
    }
    rt_MATERIAL *lm = sc.material(RT_MAT_LIGHT, 0xFFFFFF, 1.0f, 0.0f, 1.0f,
                                  0.0f, 0.0f, 1.0f, 0.0f);
    cluster.push_back(sc.quadric(RT_TAG_SPHERE, 1.2f, 0.0f, -RT_INF, +RT_INF, lm, lm));
    rt_OBJECT co = sc.array(cluster);
    Scene::trm_set(&co.trm, 1, 1, 1, 0, 0, 0, 0.0f, 0.55f * bd, bh - 1.6f);
    root.push_back(co);

    for (int i = 0; i < nq; i++)
    {
        double u = r.u01();
        rt_ui32 col = rand_rgb(r, 0.3, 1.0);
        rt_MATERIAL *mo, *mi;
        if (u < 0.60)
        {
            mo = mi = sc.material(RT_MAT_PLAIN, col, 1.0f, 0.0f, 1.0f,
                                  0.0f, 0.0f, 1.0f, 0.0f);
        }
        else if (u < 0.85)
        {
            mo = sc.material(RT_MAT_METAL, col, 0.0f, 0.0f, 1.0f,
                             1.0f, 0.0f, 1.0f, 9.0f);
            mi = sc.material(RT_MAT_PLAIN, 0x808080, 1.0f, 0.0f, 1.0f,
                             0.0f, 0.0f, 1.0f, 0.0f);
        }
        else
        {
            mo = sc.material(RT_MAT_PLAIN, 0xF0F8FF, 0.0f, 0.0f, 1.0f,
                             0.0f, 1.0f, 1.0f / 1.5f, 0.0f);
            mi = sc.material(RT_MAT_PLAIN, 0xF0F8FF, 0.0f, 0.0f, 1.0f,
                             0.0f, 1.0f, 1.5f, 0.0f);
        }
        int tag;
        rt_OBJECT q = random_quadric(sc, r, mo, mi, &tag);
        float p[3];
        rand_pos(r, p, -bw + 2.5, bw - 2.5, 3.0, bd - 2.5, 1.5, bh - 4.0);
        float rx = r.uf(-180, 180);
        float ry = r.uf(-180, 180);
        float rz = r.uf(-180, 180);
        Scene::trm_set(&q.trm, 1, 1, 1, rx, ry, rz, p[0], p[1], p[2]);
        if (sc.flags & QR_GEN_SPIN) q.f_anim = anim_spin;
        root.push_back(q);
    }
    rt_OBJECT ro = sc.array(root);
    sc.scn.root = ro.obj;
    /* opt-outs of the default options: Fresnel on, and the path tracer
     * allowed (RT_OPTS_PT prohibits it, core/engine/format.h:64) */
    sc.scn.opts = RT_OPTS_FRESNEL | RT_OPTS_PT;
    sc.scn.lock = RT_NULL;
}

static Scene *build(int kind, uint64_t seed, int nq, int flags)
{
    Scene *sc = new Scene();
    sc->flags = flags;
    switch (kind)
    {
    case QR_SCN_ANIM:
        build_anim(*sc, seed, nq > 0 ? nq : 64);
        break;
    case QR_SCN_PT:
        build_pt(*sc, seed, nq > 0 ? nq : 32);
        break;
    case QR_SCN_PLAIN:
    default:
        build_plain(*sc, seed, nq > 0 ? nq : 16, 2);
        break;
    }
    return sc;
}

} /* namespace qr_gen */

#endif /* QR_SCENEGEN_HPP */

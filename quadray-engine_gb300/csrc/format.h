/*
 * format.h: scene-description structs of the QuadRay scene API.
 *
 * Scenes are static (or runtime-filled) C structs that point at each other to
 * form the object hierarchy.  The struct layouts, tag values, relation codes,
 * material tags and runtime option bits are the same as the reference
 * engine's core/engine/format.h (tags 112-137, relations 162-177, transforms
 * 183-195, colour/texture 201-301, material 307-330, object 336-387, camera
 * 393-420, light 426-450, surfaces 456-753, scene 759-764, options 40-110),
 * so scene data authored for the reference builds against this header and
 * renders through the GB300 engine unchanged.  All surfaces are defined in
 * their local IJK space where K is the axis of symmetry (the plane normal).
 */
#ifndef QR_FORMAT_H
#define QR_FORMAT_H

#include "rt_types.h"

/* runtime option bits; a set bit in rt_SCENE.opts turns the option off for
 * that scene.  GAMMA and FRESNEL are inverted: when the bit is present in
 * the active options the effect is OFF (gamma/Fresnel are on only for scenes
 * that opt out of the bit). */
#define RT_OPTS_THREAD          (1 << 0)
#define RT_OPTS_TILING          (1 << 1)
#define RT_OPTS_TILING_EXT1     (1 << 2)
#define RT_OPTS_FSCALE          (1 << 3)
#define RT_OPTS_TARRAY          (1 << 4)
#define RT_OPTS_VARRAY          (1 << 5)
#define RT_OPTS_ADJUST          (1 << 7)
#define RT_OPTS_UPDATE          (1 << 8)
#define RT_OPTS_RENDER          (1 << 9)
#define RT_OPTS_SHADOW          (1 << 10)
#define RT_OPTS_SHADOW_EXT1     (1 << 11)
#define RT_OPTS_SHADOW_EXT2     (1 << 12)
#define RT_OPTS_2SIDED          (1 << 13)
#define RT_OPTS_2SIDED_EXT1     (1 << 14)
#define RT_OPTS_2SIDED_EXT2     (1 << 15)
#define RT_OPTS_INSERT          (0 << 16)
#define RT_OPTS_INSERT_EXT1     (0 << 17)
#define RT_OPTS_INSERT_EXT2     (0 << 18)
#define RT_OPTS_REMOVE          (0 << 19)
#define RT_OPTS_GAMMA           (1 << 20)
#define RT_OPTS_FRESNEL         (1 << 21)
#define RT_OPTS_BUFFERS         (0 << 24)
#define RT_OPTS_PT              (1 << 25)
#define RT_OPTS_UPDATE_EXT0     (1 << 26)
#define RT_OPTS_UPDATE_EXT1     (1 << 27)
#define RT_OPTS_UPDATE_EXT2     (1 << 28)
#define RT_OPTS_UPDATE_EXT3     (1 << 29)
#define RT_OPTS_RENDER_EXT0     (1 << 30)
#define RT_OPTS_RENDER_EXT1     (1u << 31)

#define RT_OPTS_NONE  (RT_OPTS_GAMMA | RT_OPTS_FRESNEL | RT_OPTS_BUFFERS |     \
                       RT_OPTS_PT)

#define RT_OPTS_FULL  (RT_OPTS_THREAD | RT_OPTS_TILING | RT_OPTS_TILING_EXT1 | \
                       RT_OPTS_FSCALE | RT_OPTS_TARRAY | RT_OPTS_VARRAY |      \
                       RT_OPTS_ADJUST | RT_OPTS_UPDATE | RT_OPTS_RENDER |      \
                       RT_OPTS_SHADOW | RT_OPTS_SHADOW_EXT1 |                 \
                       RT_OPTS_SHADOW_EXT2 | RT_OPTS_2SIDED |                 \
                       RT_OPTS_2SIDED_EXT1 | RT_OPTS_2SIDED_EXT2 |            \
                       RT_OPTS_INSERT | RT_OPTS_INSERT_EXT1 |                 \
                       RT_OPTS_INSERT_EXT2 | RT_OPTS_REMOVE | RT_OPTS_GAMMA |  \
                       RT_OPTS_FRESNEL | RT_OPTS_BUFFERS | RT_OPTS_PT)

/* object tags */
#define RT_TAG_ARRAY                       -1
#define RT_TAG_PLANE                        0
#define RT_TAG_CYLINDER                     1
#define RT_TAG_SPHERE                       2
#define RT_TAG_CONE                         3
#define RT_TAG_PARABOLOID                   4
#define RT_TAG_HYPERBOLOID                  5
#define RT_TAG_PARACYLINDER                 6
#define RT_TAG_HYPERCYLINDER                7
#define RT_TAG_HYPERPARABOLOID              8
#define RT_TAG_SURFACE_MAX                  9
#define RT_TAG_CAMERA                       100
#define RT_TAG_LIGHT                        101
#define RT_TAG_MAX                          102

#define RT_IS_CAMERA(o)     ((o)->tag == RT_TAG_CAMERA)
#define RT_IS_LIGHT(o)      ((o)->tag == RT_TAG_LIGHT)
#define RT_IS_ARRAY(o)      ((o)->tag == RT_TAG_ARRAY)
#define RT_IS_SURFACE(o)    ((o)->tag  > RT_TAG_ARRAY &&                      \
                             (o)->tag  < RT_TAG_SURFACE_MAX)
#define RT_IS_PLANE(o)      ((o)->tag == RT_TAG_PLANE)

/* relations between objects of an array (obj1 rel obj2) */
#define RT_REL_MINUS_INNER                 -1 /* subtract srf inner subspace */
#define RT_REL_MINUS_OUTER                 +1 /* subtract srf outer subspace */
#define RT_REL_MINUS_ACCUM                  2 /* subtract accum subspace */
#define RT_REL_INDEX_ARRAY                  3 /* next index in sub-array */
#define RT_REL_BOUND_ARRAY                  4 /* array has bounding volume */
#define RT_REL_UNTIE_ARRAY                  5 /* array has no bounding volume */
#define RT_REL_BOUND_INDEX                  6 /* add index to bounding volume */
#define RT_REL_UNTIE_INDEX                  7 /* remove index from bnd volume */

struct rt_RELATION
{
    rt_si32             obj1;
    rt_si32             rel;
    rt_si32             obj2;
};

struct rt_TRANSFORM2D
{
    rt_vec2             scl;
    rt_real             rot;
    rt_vec2             pos;
};

struct rt_TRANSFORM3D
{
    rt_vec3             scl;
    rt_vec3             rot;    /* Euler angles in degrees, applied X, Y, Z */
    rt_vec3             pos;
};

struct rt_COL
{
    rt_ui32             val;    /* packed XRGB, 0 selects hdr */
    rt_vec4             hdr;
};

#define RT_COL(val)                 { val, {0.0f} }
#define RT_COL_HDR(r, g, b, a)      { 0x0, {r, g, b, a} }

#define RT_TEX_PCOLOR                       0
#define RT_TEX_HDR_PCOLOR                   10

struct rt_TEX
{
    rt_si32             tag;
    rt_COL              col;
    rt_void            *ptex;   /* texel array (XRGB), or file name to load */
    rt_si32             tex_num;
    rt_RELATION        *prel;
    rt_si32             rel_num;
    rt_si32             x_dim;  /* power-of-two texture dimensions */
    rt_si32             y_dim;
};

#define RT_TEX(tag, val)                                                      \
    { RT_TEX_##tag, RT_COL(val), RT_NULL, 0, RT_NULL, 0, 0, 0 }

/* a texture named by its BMP file, loaded when the scene is built (from
 * the directory of QR_PATH_TEXTURES, else data/textures/) */
#define RT_TEX_LOAD(tag, pstr)                                                \
    { RT_TEX_##tag, RT_COL(0x0), (rt_pntr)pstr, 0, RT_NULL, 0, 0, 0 }

#define RT_TEX_BIND(tag, ptex)                                                \
    { RT_TEX_##tag, RT_COL(0x0), *ptex, 0, RT_NULL, 0,                        \
      (rt_si32)RT_ARR_SIZE(**ptex), (rt_si32)RT_ARR_SIZE(*ptex) }

struct rt_TEXTURE
{
    rt_vec2             scl;
    rt_real             rot;
    rt_vec2             pos;
    rt_TEX              tex;
    rt_real             wgt;
};

#define RT_MAT_PLAIN                        0
#define RT_MAT_LIGHT                        1
#define RT_MAT_METAL                        2
#define RT_MAT(tag)                         RT_MAT_##tag

struct rt_MATERIAL
{
    rt_si32             tag;
    rt_TEX              tex;
    rt_real             lgt[4]; /* diffuse, specular, specular power */
    rt_real             prp[4]; /* reflect, transparency, refraction index,
                                   extinction (metal) */
};

struct rt_SIDE
{
    rt_vec2             scl;    /* texture transform (implicit 2D) */
    rt_real             rot;
    rt_vec2             pos;
    rt_MATERIAL        *pmat;
};

struct rt_OBJ
{
    rt_si32             tag;
    rt_void            *pobj;
    rt_si32             obj_num;
    rt_RELATION        *prel;
    rt_si32             rel_num;
    rt_MATERIAL        *pmat_outer; /* surface material override */
    rt_MATERIAL        *pmat_inner; /* surface material override */
};

typedef rt_void (*rt_FUNC_ANIM3D)(rt_time time, rt_time last_time,
                                  rt_TRANSFORM3D *trm, rt_pntr pobj);

struct rt_OBJECT
{
    rt_TRANSFORM3D      trm;
    rt_OBJ              obj;
    rt_FUNC_ANIM3D      f_anim;
    rt_time             time;
};

#define RT_OBJ_ARRAY(parr)                                                    \
    { RT_TAG_ARRAY, *parr, (rt_si32)RT_ARR_SIZE(*parr), RT_NULL, 0,           \
      RT_NULL, RT_NULL }

#define RT_OBJ_ARRAY_REL(parr, prel)                                          \
    { RT_TAG_ARRAY, *parr, (rt_si32)RT_ARR_SIZE(*parr),                       \
      *prel, (rt_si32)RT_ARR_SIZE(*prel), RT_NULL, RT_NULL }

#define RT_CAM_PLAIN                        0
#define RT_CAM(tag)                         RT_CAM_##tag

struct rt_CAMERA
{
    rt_si32             tag;
    rt_COL              col;    /* global ambient colour */
    rt_real             lum[1]; /* global ambient intensity */
    rt_real             vpt[1]; /* distance from the eye to a screen 1 wide */
    rt_vec3             dps;    /* movement step per unit of time */
    rt_vec3             drt;    /* rotation step per unit of time */
};

#define RT_LGT_PLAIN                        0
#define RT_LGT(tag)                         RT_LGT_##tag

struct rt_LIGHT
{
    rt_si32             tag;
    rt_COL              col;    /* light colour */
    rt_real             lum[2]; /* ambient and source intensity */
    rt_real             atn[4]; /* range, constant, linear, quadratic */
};

#define RT_OBJ_CAMERA(pobj)                                                   \
    { RT_TAG_CAMERA, pobj, 1, RT_NULL, 0, RT_NULL, RT_NULL }
#define RT_OBJ_LIGHT(pobj)                                                    \
    { RT_TAG_LIGHT, pobj, 1, RT_NULL, 0, RT_NULL, RT_NULL }

struct rt_SURFACE
{
    rt_vec3             min;    /* local-space axis clippers */
    rt_vec3             max;
    rt_SIDE             side_outer;
    rt_SIDE             side_inner;
};

struct rt_PLANE           { rt_SURFACE srf; };
struct rt_CYLINDER        { rt_SURFACE srf; rt_real rad; };
struct rt_SPHERE          { rt_SURFACE srf; rt_real rad; };
struct rt_CONE            { rt_SURFACE srf; rt_real rat; };
struct rt_PARABOLOID      { rt_SURFACE srf; rt_real par; };
struct rt_HYPERBOLOID     { rt_SURFACE srf; rt_real rat; rt_real hyp; };
struct rt_PARACYLINDER    { rt_SURFACE srf; rt_real par; };
struct rt_HYPERCYLINDER   { rt_SURFACE srf; rt_real rat; rt_real hyp; };
struct rt_HYPERPARABOLOID { rt_SURFACE srf; rt_real pr1; rt_real pr2; };

#define QR_OBJ_SURFACE(tg, pobj, po, pi)                                     \
    { tg, pobj, 1, RT_NULL, 0, po, pi }
#define RT_OBJ_PLANE(p)           QR_OBJ_SURFACE(RT_TAG_PLANE, p, 0, 0)
#define RT_OBJ_CYLINDER(p)        QR_OBJ_SURFACE(RT_TAG_CYLINDER, p, 0, 0)
#define RT_OBJ_SPHERE(p)          QR_OBJ_SURFACE(RT_TAG_SPHERE, p, 0, 0)
#define RT_OBJ_CONE(p)            QR_OBJ_SURFACE(RT_TAG_CONE, p, 0, 0)
#define RT_OBJ_PARABOLOID(p)      QR_OBJ_SURFACE(RT_TAG_PARABOLOID, p, 0, 0)
#define RT_OBJ_HYPERBOLOID(p)     QR_OBJ_SURFACE(RT_TAG_HYPERBOLOID, p, 0, 0)
#define RT_OBJ_PARACYLINDER(p)    QR_OBJ_SURFACE(RT_TAG_PARACYLINDER, p, 0, 0)
#define RT_OBJ_HYPERCYLINDER(p)   QR_OBJ_SURFACE(RT_TAG_HYPERCYLINDER, p, 0, 0)
#define RT_OBJ_HYPERPARABOLOID(p) QR_OBJ_SURFACE(RT_TAG_HYPERPARABOLOID, p,0,0)

struct rt_SCENE
{
    rt_OBJ              root;   /* must be an array */
    rt_ui32             opts;   /* option bits this scene turns off */
    rt_pntr             lock;   /* owning engine instance, NULL when free */
};

#endif /* QR_FORMAT_H */

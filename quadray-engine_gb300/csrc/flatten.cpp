/*
 * flatten.cpp: host update phases of the QuadRay engine, restated for the
 * GB300 backend, producing the flat records of qr_gpu.h.
 *
 * Every float expression follows the operation order of the reference
 * (file:line cited per function); build with -ffp-contract=off.
 */
#include <math.h>
#include <string.h>
#include <stdio.h>
#include <stdlib.h>
#include <algorithm>
#include <unordered_map>

#include "flatten.h"
#include "xform.h"
#include "rt_exception.h"

namespace qr
{

#define FLAG_SCL    (1 << 0)    /* RT_UPDATE_FLAG_SCL, core/engine/object.h:74 */
#define FLAG_ROT    (1 << 1)    /* RT_UPDATE_FLAG_ROT, object.h:79 */
#define FLAG_OBJ    (1 << 2)    /* RT_UPDATE_FLAG_OBJ, object.h:83 */

#define K_ARRAY     0
#define K_SURFACE   1
#define K_CAMERA    2
#define K_LIGHT     3

#define DEPS_THRESHOLD  0.00000000001f  /* object.h:41 */
#define TEPS_THRESHOLD  0.0000001f      /* object.h:42 */
#define CLIP_THRESHOLD  0.01f           /* object.h:39 */

static const float iden4[4][4] =
{
    {1.0f, 0.0f, 0.0f, 0.0f},
    {0.0f, 1.0f, 0.0f, 0.0f},
    {0.0f, 0.0f, 1.0f, 0.0f},
    {0.0f, 0.0f, 0.0f, 1.0f},
};

/* ---- scalar helpers (core/config/rtbase.h:827-875) ---------------------- */

static inline float fabs_(float a) { return fabsf(a); }
static inline int sign_(float a) { return a < 0.0f ? -1 : a > 0.0f ? +1 : 0; }
static inline float sqrt_(float a) { return a <= 0.0f ? 0.0f : sqrtf(a); }

/* sine/cosine of an angle in degrees with exact values at multiples of 90
 * (rtbase.h:858-875); other angles go through the platform's sinf/cosf on
 * (float)(deg * pi / 180) computed in double, like the reference */
static float sina_(float a)
{
    if (a == -270.0f) return +1.0f;
    if (a == -180.0f) return  0.0f;
    if (a ==  -90.0f) return -1.0f;
    if (a ==    0.0f) return  0.0f;
    if (a ==  +90.0f) return +1.0f;
    if (a == +180.0f) return  0.0f;
    if (a == +270.0f) return -1.0f;
    return sinf((float)((double)a * RT_PI / 180.0));
}

static float cosa_(float a)
{
    if (a == -270.0f) return  0.0f;
    if (a == -180.0f) return -1.0f;
    if (a ==  -90.0f) return  0.0f;
    if (a ==    0.0f) return +1.0f;
    if (a ==  +90.0f) return  0.0f;
    if (a == +180.0f) return -1.0f;
    if (a == +270.0f) return  0.0f;
    return cosf((float)((double)a * RT_PI / 180.0));
}

float sina(float deg) { return sina_(deg); }
float cosa(float deg) { return cosa_(deg); }

/* ---- 4x4 column-major matrices (core/engine/rtgeom.cpp:59-228) ---------- */

/* T * Rz * Ry * Rx * S (rtgeom.cpp:102-164), scale only with `as` */
static void mat_from_transform(float (*mp)[4], const rt_TRANSFORM3D *t, int as)
{
    const float scl[3] = {as ? t->scl[RT_X] : 1.0f, as ? t->scl[RT_Y] : 1.0f,
                          as ? t->scl[RT_Z] : 1.0f};
    const float s3[3] = {sina_(t->rot[RT_X]), sina_(t->rot[RT_Y]), sina_(t->rot[RT_Z])};
    const float c3[3] = {cosa_(t->rot[RT_X]), cosa_(t->rot[RT_Y]), cosa_(t->rot[RT_Z])};
    const float pos[3] = {t->pos[RT_X], t->pos[RT_Y], t->pos[RT_Z]};
    mat_from_sc(mp, s3, c3, pos, scl);
}

/* packed XRGB to [0,1] colour (object.cpp:435-440, 599-604) */
static void col_hdr(rt_COL *col)
{
    if (col->val != 0x0)
    {
        col->hdr[RT_R] = ((col->val >> 0x10) & 0xFF) / 255.0f;
        col->hdr[RT_G] = ((col->val >> 0x08) & 0xFF) / 255.0f;
        col->hdr[RT_B] = ((col->val >> 0x00) & 0xFF) / 255.0f;
    }
}

/* ======================================================================== */

Flat::Flat(rt_SCENE *scn, int opts_, int x_res_, int y_res_, int fsaa_)
    : opts(opts_), x_res(x_res_), y_res(y_res_), fsaa(fsaa_),
      depth(10), cam_idx(0), hor_sin(0.0f), hor_cos(1.0f), cam_off(0), cam_num(0),
      root(0)
{
    if (scn == RT_NULL || scn->root.tag != RT_TAG_ARRAY)
    {
        throw rt_Exception("scene's root is not an array");
    }
    /* pixel width, aspect ratio (engine.cpp:2901-2903) */
    factor = 1.0f / (rt_real)x_res;
    aspect = (rt_real)y_res * factor;

    memset(&rootobj, 0, sizeof(rootobj));
    rootobj.trm.scl[RT_I] = 1.0f;
    rootobj.trm.scl[RT_J] = 1.0f;
    rootobj.trm.scl[RT_K] = 1.0f;
    rootobj.obj = scn->root;

    root = build(RT_NULL, &rootobj);
    if (cameras.empty())
    {
        throw rt_Exception("scene doesn't contain camera");
    }
    /* the reference keeps its cameras in a list each new one is pushed in
     * front of (object.cpp:429-431, object.h:178) and starts with its head
     * (engine.cpp:2956-2961): the camera created last */
    cam_idx = (int)cameras.size() - 1;
}

Flat::~Flat()
{
    for (size_t i = 0; i < nodes.size(); i++) delete nodes[i];
}

/* resolve a material (rt_Material ctor, object.cpp:4038-4180) */
/* a 24-bit uncompressed BMP as the reference's load_image reads it
 * (rtimag.cpp:47-186): signature, data offset, width, height, one plane,
 * 24 bits, no compression; texels in file order (rows are not flipped),
 * each row padded to 4 bytes, texel = B | G << 8 | R << 16 */
static bool load_bmp(const char *path, std::vector<rt_ui32> &out, int &xd, int &yd)
{
    FILE *f = fopen(path, "rb");
    if (f == NULL) return false;
    unsigned char h[34];
    bool ok = fread(h, 1, sizeof(h), f) == sizeof(h);
    const unsigned sig = h[0] | (h[1] << 8);
    const unsigned off = h[10] | (h[11] << 8) | (h[12] << 16) | ((unsigned)h[13] << 24);
    const int w = (int)(h[18] | (h[19] << 8) | (h[20] << 16) | ((unsigned)h[21] << 24));
    const int hh = (int)(h[22] | (h[23] << 8) | (h[24] << 16) | ((unsigned)h[25] << 24));
    const unsigned planes = h[26] | (h[27] << 8), depth = h[28] | (h[29] << 8);
    const unsigned comp = h[30] | (h[31] << 8) | (h[32] << 16) | ((unsigned)h[33] << 24);
    ok = ok && sig == 0x4D42 && planes == 1 && depth == 24 && comp == 0 && w != 0 && hh != 0;
    if (ok)
    {
        xd = w < 0 ? -w : w;
        yd = hh < 0 ? -hh : hh;
        ok = xd <= 65536 && yd <= 65536 && fseek(f, (long)off, SEEK_SET) == 0;
    }
    if (ok)
    {
        const int pad = ((xd * 3 + 3) / 4) * 4 - xd * 3;
        out.assign((size_t)xd * yd, 0u);
        unsigned char px[3], skip[3];
        for (int y = 0; y < yd && ok; y++)
        {
            for (int x = 0; x < xd && ok; x++)
            {
                ok = fread(px, 1, 3, f) == 3;
                out[(size_t)y * xd + x] = (rt_ui32)px[0] | ((rt_ui32)px[1] << 8) |
                                          ((rt_ui32)px[2] << 16);
            }
            if (ok && pad) ok = fread(skip, 1, (size_t)pad, f) == (size_t)pad;
        }
    }
    fclose(f);
    return ok;
}

int Flat::material(rt_SIDE *sd, rt_MATERIAL *mt)
{
    if (mt == RT_NULL)
    {
        throw rt_Exception("null-pointer in material");
    }
    Material M;
    memset(&M, 0, sizeof(M));
    M.mat = mt;
    M.sd = sd;

    rt_TEX *tx = &mt->tex;
    /* plain colour defined in place (object.cpp:4193-4198) */
    rt_ui32 *ptex = (rt_ui32 *)tx->ptex;
    int x_dim = tx->x_dim, y_dim = tx->y_dim;
    if (x_dim == 0 && y_dim == 0 && ptex == RT_NULL)
    {
        ptex = &tx->col.val;
        x_dim = 1;
        y_dim = 1;
    }
    if (x_dim == 0 && y_dim == 0 && ptex != RT_NULL)
    {
        /* a file name: the texture loads once per scene (rt_Texture,
         * object.cpp:3990-4011; rtimag.cpp:47-186) */
        const std::string name((const char *)tx->ptex);
        size_t k = 0;
        while (k < file_tex_name.size() && file_tex_name[k] != name) k++;
        if (k == file_tex_name.size())
        {
            const char *pfx = getenv("QR_PATH_TEXTURES");
            const std::string path = std::string(pfx ? pfx : "data/textures/") + name;
            std::vector<rt_ui32> t;
            int xd = 0, yd = 0;
            if (!load_bmp(path.c_str(), t, xd, yd))
            {
                throw rt_Exception("failed to load image");
            }
            file_tex.push_back(t);
            file_tex_name.push_back(name);
            file_tex_dim.push_back(xd);
            file_tex_dim.push_back(yd);
        }
        ptex = file_tex[k].data();
        x_dim = file_tex_dim[2 * k];
        y_dim = file_tex_dim[2 * k + 1];
    }
    M.texels = ptex;
    M.x_dim = x_dim;
    M.y_dim = y_dim;

    int props = QR_PROP_NORMAL;
    props |= -((opts & RT_OPTS_GAMMA) == 0) & QR_PROP_GAMMA;
    props |= -((opts & RT_OPTS_FRESNEL) == 0) & QR_PROP_FRESNEL;
    props |= mt->tag == RT_MAT_LIGHT ? QR_PROP_LIGHT : 0;
    props |= mt->tag == RT_MAT_METAL ? QR_PROP_METAL : 0;
    props |= mt->prp[1] == 0.0f ? QR_PROP_OPAQUE : 0;
    props |= mt->prp[1] == 1.0f ? QR_PROP_TRANSP : 0;
    props |= x_dim == 1 && y_dim == 1 ? 0 : QR_PROP_TEXTURE;
    props |= mt->prp[0] == 0.0f ? 0 : QR_PROP_REFLECT;
    props |= mt->prp[2] == 1.0f ? 0 : QR_PROP_REFRACT;
    props |= mt->lgt[0] == 0.0f ? 0 : QR_PROP_DIFFUSE;
    props |= mt->lgt[1] == 0.0f ? 0 : QR_PROP_SPECULAR;
    if (mt->prp[0] + mt->prp[1] >= 1.0f)
    {
        props &= ~QR_PROP_DIFFUSE;
        props &= ~QR_PROP_SPECULAR;
    }
    M.props = props;

    /* texture axis mapping from the side's 2D rotation */
    float mtx[2][2];
    mtx[0][0] = +cosa_(sd->rot);
    mtx[0][1] = +sina_(sd->rot);
    mtx[1][0] = -sina_(sd->rot);
    mtx[1][1] = +cosa_(sd->rot);
    int sgn[2] = {1, 1}, match = 0;
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++)
            if (fabs_(mtx[i][0]) == iden4[j][0] && fabs_(mtx[i][1]) == iden4[j][1])
            {
                M.map[i] = j;
                sgn[i] = sign_(mtx[i][j]);
                match++;
            }
    if (match < 2)
    {
        M.map[RT_X] = RT_U; sgn[RT_X] = 1;
        M.map[RT_Y] = RT_V; sgn[RT_Y] = 1;
    }

    qr_mat &m = M.m;
    m.tmap[0] = M.map[RT_X];
    m.tmap[1] = M.map[RT_Y];
    M.scl[RT_X] = x_dim / (sd->scl[RT_X] * sgn[RT_X]);
    M.scl[RT_Y] = y_dim / (sd->scl[RT_Y] * sgn[RT_Y]);
    m.xscal = M.scl[RT_X];
    m.yscal = M.scl[RT_Y];
    m.xoffs = sd->pos[M.map[RT_X]];
    m.yoffs = sd->pos[M.map[RT_Y]];
    m.xmask = x_dim - 1;
    m.ymask = y_dim - 1;
    int xd = x_dim, xl = 0;
    while (xd >>= 1) xl++;
    m.yshft = xl;

    float f = 1.0f - (mt->prp[0] + mt->prp[1]);
    f = RT_MAX(f, 0.0f);
    m.l_dff = mt->lgt[0] * f;
    m.l_spc = mt->lgt[1] * f;
    m.l_pow = (int32_t)(rt_ui32)(mt->lgt[2] * 16.0f);   /* 28.4 fixed point */
    m.c_rfl = mt->prp[0];
    m.c_trn = mt->prp[1];
    m.c_rfr = mt->prp[2];
    m.rfr_2 = mt->prp[2] * mt->prp[2];
    m.c_rcp = 1.0f / mt->prp[2];
    m.ext_2 = mt->prp[3] * mt->prp[3];
    if (!(mt->prp[1] == 0.0f || mt->prp[1] == 1.0f || mt->prp[2] != 1.0f))
    {
        m.c_rfr = mt->prp[3];
        m.rfr_2 = mt->prp[3] * mt->prp[3];
    }
    m.props = props;
    m.tex_off = -1;

    mats.push_back(M);
    return (int)mats.size() - 1;
}

/* build the tree (rt_Array ctor, object.cpp:1183-1647) */
Node *Flat::build(Node *parent, rt_OBJECT *obj)
{
    Node *n = new Node();
    nodes.push_back(n);
    n->obj = obj;
    n->trm = &obj->trm;
    n->tag = obj->obj.tag;
    n->parent = parent;
    memset(n->mtx, 0, sizeof(n->mtx));
    memset(n->acc, 0, sizeof(n->acc));
    memset(n->hdr, 0, sizeof(n->hdr));
    obj->time = -1;

    if (n->tag == RT_TAG_ARRAY)
    {
        n->kind = K_ARRAY;
        arrays.push_back(n);
        rt_OBJECT *arr = (rt_OBJECT *)obj->obj.pobj;
        for (int i = 0; i < obj->obj.obj_num; i++)
        {
            int t = arr[i].obj.tag;
            if (t == RT_TAG_CAMERA || t == RT_TAG_LIGHT || t == RT_TAG_ARRAY ||
                (t >= RT_TAG_PLANE && t < RT_TAG_SURFACE_MAX))
            {
                n->children.push_back(build(n, &arr[i]));
            }
        }
        /* emission of LIGHT-material surfaces from the array's accumulated
         * light (object.cpp:1347-1388) */
        for (size_t i = 0; i < n->children.size(); i++)
        {
            Node *c = n->children[i];
            if (c->kind != K_SURFACE) continue;
            int sides[2] = {c->outer, c->inner};
            for (int s = 0; s < 2; s++)
            {
                qr_mat &m = mats[sides[s]].m;
                if (mats[sides[s]].props & QR_PROP_LIGHT)
                {
                    m.emit[0] = n->acc[RT_R] * 100.0f;
                    m.emit[1] = n->acc[RT_G] * 100.0f;
                    m.emit[2] = n->acc[RT_B] * 100.0f;
                    m.emit[3] = n->acc[RT_A] * 100.0f;
                }
                else
                {
                    m.emit[0] = m.emit[1] = m.emit[2] = m.emit[3] = 0.0f;
                }
            }
        }
        relations(n);
    }
    else if (n->tag == RT_TAG_CAMERA)
    {
        n->kind = K_CAMERA;
        cameras.push_back(n);
        rt_CAMERA *cam = (rt_CAMERA *)obj->obj.pobj;
        col_hdr(&cam->col);
        /* pov (object.cpp:446-448) */
        n->pov = cam->vpt[0] <= 0.0f ? 1.0f :
                 cam->vpt[0] <= 2 * CLIP_THRESHOLD ? 2 * CLIP_THRESHOLD :
                 cam->vpt[0];
    }
    else if (n->tag == RT_TAG_LIGHT)
    {
        n->kind = K_LIGHT;
        lights.push_back(n);
        rt_LIGHT *lgt = (rt_LIGHT *)obj->obj.pobj;
        col_hdr(&lgt->col);
        /* object.cpp:610-630 */
        n->lcol[0] = lgt->col.hdr[RT_R] * lgt->lum[1];
        n->lcol[1] = lgt->col.hdr[RT_G] * lgt->lum[1];
        n->lcol[2] = lgt->col.hdr[RT_B] * lgt->lum[1];
        parent->acc[RT_R] += n->lcol[0];
        parent->acc[RT_G] += n->lcol[1];
        parent->acc[RT_B] += n->lcol[2];
        parent->acc[RT_R] += lgt->col.hdr[RT_R] * lgt->lum[0];
        parent->acc[RT_G] += lgt->col.hdr[RT_G] * lgt->lum[0];
        parent->acc[RT_B] += lgt->col.hdr[RT_B] * lgt->lum[0];
        parent->acc[RT_A] += lgt->lum[0] + lgt->lum[1];
    }
    else
    {
        n->kind = K_SURFACE;
        n->gen = (int)surfaces.size();
        surfaces.push_back(n);
        n->srf = (rt_SURFACE *)obj->obj.pobj;
        n->outer = material(&n->srf->side_outer, obj->obj.pmat_outer ?
                            obj->obj.pmat_outer : n->srf->side_outer.pmat);
        n->inner = material(&n->srf->side_inner, obj->obj.pmat_inner ?
                            obj->obj.pmat_inner : n->srf->side_inner.pmat);
    }
    return n;
}

/* append relation template "lst" to a surface, or to every surface of an
 * array (rt_Surface::add_relation, object.cpp:2407-2479; the template is
 * reversed there and reversed again when the clip list is built,
 * engine.cpp:1850-1979, so the final order is the scene's order) */
void Flat::add_relation(Node *n, const std::vector<Node::Rel> &lst)
{
    if (n->kind == K_ARRAY)
    {
        for (size_t i = 0; i < n->children.size(); i++)
            add_relation(n->children[i], lst);
        return;
    }
    if (n->kind != K_SURFACE) return;
    for (size_t i = 0; i < lst.size(); i++)
    {
        const Node::Rel &r = lst[i];
        if (r.obj == RT_NULL || r.obj->kind == K_SURFACE)
        {
            n->rel.push_back(r);
        }
        else if (r.obj->kind == K_ARRAY)
        {
            /* expand array clippers into their objects */
            std::vector<Node::Rel> sub;
            for (size_t j = 0; j < r.obj->children.size(); j++)
            {
                Node::Rel e = {r.data, r.obj->children[j]};
                sub.push_back(e);
            }
            add_relation(n, sub);
        }
    }
}

/* relations of an array (object.cpp:1390-1601): custom clippers and boolean
 * accumulator segments; bounding-volume relations only cull and are ignored */
void Flat::relations(Node *arr)
{
    rt_RELATION *rel = arr->obj->obj.prel;
    int rel_num = arr->obj->obj.rel_num;
    std::vector<Node*> *l = &arr->children, *r = &arr->children;
    std::vector<Node::Rel> acc_list;
    int acc = 0;

    for (int i = 0; i < rel_num; i++)
    {
        if (rel[i].obj1 >= (int)l->size() || rel[i].obj2 >= (int)r->size())
        {
            continue;
        }
        std::vector<Node::Rel> elm;
        bool have = false;
        switch (rel[i].rel)
        {
        case RT_REL_INDEX_ARRAY:
            if (rel[i].obj1 >= 0 && rel[i].obj2 >= -1 &&
                (*l)[rel[i].obj1]->kind == K_ARRAY)
                l = &(*l)[rel[i].obj1]->children;
            if (rel[i].obj1 >= -1 && rel[i].obj2 >= 0 &&
                (*r)[rel[i].obj2]->kind == K_ARRAY)
                r = &(*r)[rel[i].obj2]->children;
            break;

        case RT_REL_MINUS_INNER:
        case RT_REL_MINUS_OUTER:
            if (rel[i].obj1 == -1 && rel[i].obj2 >= 0 && acc == 0)
            {
                acc = 1;
                acc_list.clear();
                Node::Rel e = {-1, RT_NULL};    /* accum enter */
                acc_list.push_back(e);
            }
            if (rel[i].obj1 >= -1 && rel[i].obj2 >= 0)
            {
                Node::Rel e = {rel[i].rel, (*r)[rel[i].obj2]};
                r = &arr->children;
                if (rel[i].obj1 == -1)
                {
                    acc_list.push_back(e);
                }
                else
                {
                    elm.push_back(e);
                    have = true;
                }
            }
            break;

        case RT_REL_MINUS_ACCUM:
            if (rel[i].obj1 >= 0 && rel[i].obj2 == -1 && acc == 1)
            {
                acc = 0;
                Node::Rel e = {+1, RT_NULL};    /* accum leave */
                acc_list.push_back(e);
                elm = acc_list;
                have = true;
            }
            break;

        default:
            if (rel[i].obj1 >= 0) l = &arr->children;
            if (rel[i].obj2 >= 0) r = &arr->children;
            break;
        }
        if (rel[i].obj1 >= 0 && have)
        {
            add_relation((*l)[rel[i].obj1], elm);
            l = &arr->children;
        }
    }
}

/* ---- phase 0.5 ---------------------------------------------------------- */

/* rt_Object::update_status (object.cpp:175-216), rt_Array::update_status
 * (object.cpp:1683-1701) */
void Flat::update_status(Node *n, rt_time time, int flags, Node *trnode)
{
    rt_OBJECT *obj = n->obj;
    if (n->kind == K_ARRAY)
    {
        /* every frame is a full update in this engine (the reference skips
         * unchanged subtrees only as an optimisation, results are equal) */
        flags |= FLAG_OBJ;
    }
    if (obj->f_anim != RT_NULL && obj->time != time)
    {
        obj->f_anim(time, obj->time < 0 ? 0 : obj->time, n->trm, RT_NULL);
    }
    obj->time = time;
    n->obj_changed = flags & FLAG_OBJ;
    if (obj->f_anim != RT_NULL)
    {
        n->obj_changed |= FLAG_OBJ;
    }
    if (n->obj_changed == 0)
    {
        return;
    }
    n->obj_has_trm = (flags & FLAG_SCL) | (flags & FLAG_ROT);
    n->trnode = trnode;
}

/* rt_Object::update_matrix (object.cpp:221-389) */
void Flat::update_matrix(Node *n, float (*mtx)[4])
{
    if (n->obj_changed == 0)
    {
        return;
    }
    rt_TRANSFORM3D *trm = n->trm;
    int i, c;

    n->mtx_has_trm = 0;

    const float fsc[] = {-1.0f, +1.0f};
    for (i = 0, c = 0; i < 2; i++)
    {
        if (trm->scl[RT_X] == fsc[i]) c++;
        if (trm->scl[RT_Y] == fsc[i]) c++;
        if (trm->scl[RT_Z] == fsc[i]) c++;
    }
    n->mtx_has_trm |= (c == 3) ? 0 : FLAG_SCL;

    const float frt[] = {-270.0f, -180.0f, -90.0f, 0.0f, +90.0f, +180.0f, +270.0f};
    for (i = 0, c = 0; i < 7; i++)
    {
        if (trm->rot[RT_X] == frt[i]) c++;
        if (trm->rot[RT_Y] == frt[i]) c++;
        if (trm->rot[RT_Z] == frt[i]) c++;
    }
    n->mtx_has_trm |= (c == 3) ? 0 : FLAG_ROT;

    if ((n->mtx_has_trm & FLAG_ROT) == 0)
    {
        float trm_mtx[4][4];
        mat_from_transform(trm_mtx, trm, 1);
        mat_mul_mat(n->mtx, mtx, trm_mtx);

        if (n->obj_has_trm == FLAG_SCL)
        {
            n->mtx_has_trm = n->obj_has_trm;
            n->obj_has_trm = 0;
        }

        for (i = 0; i < 3; i++)
        {
            for (int j = 0; j < 3; j++)
            {
                if ((n->mtx[i][0] != 0.0f) == (iden4[j][0] != 0.0f) &&
                    (n->mtx[i][1] != 0.0f) == (iden4[j][1] != 0.0f) &&
                    (n->mtx[i][2] != 0.0f) == (iden4[j][2] != 0.0f))
                {
                    n->map[i] = j;
                    n->sgn[i] = sign_(n->mtx[i][j]);
                    n->scl[j] = fabs_(n->mtx[i][j]);
                }
            }
        }
        n->map[RT_L] = RT_W;
        n->sgn[RT_L] = 1;
        n->scl[RT_W] = 1.0f;
    }

    if ((n->mtx_has_trm & FLAG_ROT) != 0 && n->trnode == RT_NULL)
    {
        float trm_mtx[4][4];
        mat_from_transform(trm_mtx, trm, 0);
        mat_mul_mat(n->mtx, mtx, trm_mtx);
    }
    if ((n->mtx_has_trm & FLAG_ROT) != 0 && n->trnode != RT_NULL)
    {
        float trm_mtx[4][4], tmp_mtx[4][4];
        mat_from_transform(trm_mtx, trm, 0);
        mat_mul_mat(tmp_mtx, n->trnode->mtx, mtx);
        mat_mul_mat(n->mtx, tmp_mtx, trm_mtx);
    }
    if ((n->mtx_has_trm & FLAG_ROT) != 0)
    {
        n->trnode = n;
        n->obj_has_trm |= FLAG_ROT;
        n->map[RT_I] = RT_X; n->map[RT_J] = RT_Y;
        n->map[RT_K] = RT_Z; n->map[RT_L] = RT_W;
        n->sgn[RT_I] = 1; n->sgn[RT_J] = 1; n->sgn[RT_K] = 1; n->sgn[RT_L] = 1;
        n->scl[RT_X] = trm->scl[RT_X];
        n->scl[RT_Y] = trm->scl[RT_Y];
        n->scl[RT_Z] = trm->scl[RT_Z];
        n->scl[RT_W] = 1.0f;
    }

    if ((n->obj_has_trm & FLAG_ROT) != 0 && (opts & RT_OPTS_FSCALE) == 0)
    {
        n->obj_has_trm |= FLAG_SCL;
    }

    if (n->trnode != RT_NULL && n->trnode != n &&
        ((opts & RT_OPTS_TARRAY) == 0 || n->tag > RT_TAG_SURFACE_MAX))
    {
        float tmp_mtx[4][4];
        mat_mul_mat(tmp_mtx, n->trnode->mtx, n->mtx);
        memcpy(n->mtx, tmp_mtx, sizeof(tmp_mtx));

        n->trnode = n;
        n->obj_has_trm |= n->mtx_has_trm;
        n->map[RT_I] = RT_X; n->map[RT_J] = RT_Y;
        n->map[RT_K] = RT_Z; n->map[RT_L] = RT_W;
        n->sgn[RT_I] = 1; n->sgn[RT_J] = 1; n->sgn[RT_K] = 1; n->sgn[RT_L] = 1;
        n->scl[RT_X] = 1.0f; n->scl[RT_Y] = 1.0f;
        n->scl[RT_Z] = 1.0f; n->scl[RT_W] = 1.0f;
    }

    if (n->kind == K_ARRAY)
    {
        /* rt_Array::update_matrix (object.cpp:1706-1748) */
        n->pmtx = n->mtx;
        if (n->trnode == n)
        {
            memcpy(n->scm, iden4, sizeof(n->scm));
            n->scm[0][0] = n->scl[0];
            n->scm[1][1] = n->scl[1];
            n->scm[2][2] = n->scl[2];
            n->pmtx = n->scm;
        }
    }
}

/* rt_Array::update_object (object.cpp:1753-1781) and the leaf variants
 * (object.cpp:457-465, 636-644, 2484-2492): leaves only remember the
 * parent's matrix, their own matrix is computed in phase 1 */
void Flat::update_object(Node *n, rt_time time, int flags, Node *trnode,
                         float (*mtx)[4])
{
    n->in_flags = flags;
    update_status(n, time, flags, trnode);
    if (n->kind != K_ARRAY)
    {
        n->pmtx = mtx;
        return;
    }
    update_matrix(n, mtx);
    for (size_t i = 0; i < n->children.size(); i++)
    {
        update_object(n->children[i], time,
                      flags | n->mtx_has_trm | n->obj_changed,
                      n->trnode, n->pmtx);
    }
}

/* ---- phase 1 ------------------------------------------------------------ */

/* rt_Node::update_fields (object.cpp:826-857) */
void Flat::fields_node(Node *n)
{
    qr_srf &s = n->rec;
    if (n->trnode == n)
    {
        mat_inverse(n->inv, n->mtx);
        s.tci[0] = n->inv[RT_X][RT_I];
        s.tci[1] = n->inv[RT_Y][RT_I];
        s.tci[2] = n->inv[RT_Z][RT_I];
        s.tcj[0] = n->inv[RT_X][RT_J];
        s.tcj[1] = n->inv[RT_Y][RT_J];
        s.tcj[2] = n->inv[RT_Z][RT_J];
        s.tck[0] = n->inv[RT_X][RT_K];
        s.tck[1] = n->inv[RT_Y][RT_K];
        s.tck[2] = n->inv[RT_Z][RT_K];
    }
    s.pos[0] = n->mtx[3][RT_X];
    s.pos[1] = n->mtx[3][RT_Y];
    s.pos[2] = n->mtx[3][RT_Z];

    int shift = n->trnode != RT_NULL ? 1 : 0;
    s.amap[0] = n->map[RT_I];
    s.amap[1] = n->map[RT_J];
    s.amap[2] = n->map[RT_K];
    s.amap[3] = n->obj_has_trm;
    s.asgn[0] = n->sgn[RT_I] >= 0 ? 0 : 1;
    s.asgn[1] = n->sgn[RT_J] >= 0 ? 0 : 1;
    s.asgn[2] = n->sgn[RT_K] >= 0 ? 0 : 1;
    s.asgn[3] = shift;
}

/* rt_Array::update_fields (object.cpp:1786-1850) */
void Flat::fields_array(Node *n)
{
    memset(&n->rec, 0, sizeof(n->rec));
    n->rec.tag = RT_TAG_ARRAY;
    n->rec.is_node = 1;
    n->rec.trnode = -1;
    fields_node(n);
}

/* surfaces (rt_Surface::update_fields object.cpp:2497-2528, plane
 * 2920-2977, quadrics 3037-3088 and 3145-3936) */
void Flat::fields_surface(Node *n)
{
    update_matrix(n, n->pmtx);
    qr_srf keep = n->rec;
    memset(&n->rec, 0, sizeof(n->rec));
    (void)keep;
    n->rec.tag = n->tag;
    n->rec.trnode = -1;
    n->rec.id = n->gen;
    fields_node(n);

    int mp_i = n->map[RT_I], mp_j = n->map[RT_J], mp_k = n->map[RT_K];
    float *sci = n->sci, *scj = n->scj;

    if (n->tag == RT_TAG_PLANE)
    {
        /* texture scalers (object.cpp:2929-2963) */
        float asc[2], isc[2];
        asc[RT_U] = n->scl[mp_i];
        asc[RT_V] = n->scl[mp_j];
        isc[RT_U] = 1.0f / asc[RT_U];
        isc[RT_V] = 1.0f / asc[RT_V];
        int sides[2] = {n->outer, n->inner};
        for (int s = 0; s < 2; s++)
        {
            Material &M = mats[sides[s]];
            M.m.xscal = M.scl[RT_X] * isc[M.map[RT_X]];
            M.m.yscal = M.scl[RT_Y] * isc[M.map[RT_Y]];
            M.m.xoffs = M.sd->pos[M.map[RT_X]] * asc[M.map[RT_X]];
            M.m.yoffs = M.sd->pos[M.map[RT_Y]] * asc[M.map[RT_Y]];
        }
        sci[0] = sci[1] = sci[2] = sci[3] = 0.0f;
        scj[0] = scj[1] = scj[2] = scj[3] = 0.0f;
        n->rec.sci[0] = n->rec.sci[1] = n->rec.sci[2] = n->rec.sci[3] = 0.0f;
        n->rec.scj[0] = n->rec.scj[1] = n->rec.scj[2] = 0.0f;
        return;
    }

    /* quadric base shape (object.cpp:3046-3053) */
    sci[0] = sci[1] = sci[2] = 1.0f; sci[3] = 0.0f;
    scj[0] = scj[1] = scj[2] = 0.0f; scj[3] = 0.0f;

    rt_OBJECT *o = n->obj;
    switch (n->tag)
    {
    case RT_TAG_CYLINDER:
    {
        rt_CYLINDER *x = (rt_CYLINDER *)o->obj.pobj;
        sci[mp_k] = 0.0f;
        sci[RT_W] = x->rad * x->rad;
    } break;
    case RT_TAG_SPHERE:
    {
        rt_SPHERE *x = (rt_SPHERE *)o->obj.pobj;
        sci[RT_W] = x->rad * x->rad;
    } break;
    case RT_TAG_CONE:
    {
        rt_CONE *x = (rt_CONE *)o->obj.pobj;
        sci[mp_k] = -(x->rat * x->rat);
    } break;
    case RT_TAG_PARABOLOID:
    {
        rt_PARABOLOID *x = (rt_PARABOLOID *)o->obj.pobj;
        sci[mp_k] = 0.0f;
        scj[mp_k] = x->par * (rt_real)n->sgn[RT_K];
    } break;
    case RT_TAG_HYPERBOLOID:
    {
        rt_HYPERBOLOID *x = (rt_HYPERBOLOID *)o->obj.pobj;
        sci[mp_k] = -(x->rat * x->rat);
        sci[RT_W] = x->hyp;
    } break;
    case RT_TAG_PARACYLINDER:
    {
        rt_PARACYLINDER *x = (rt_PARACYLINDER *)o->obj.pobj;
        sci[mp_j] = 0.0f;
        sci[mp_k] = 0.0f;
        scj[mp_k] = x->par * (rt_real)n->sgn[RT_K];
    } break;
    case RT_TAG_HYPERCYLINDER:
    {
        rt_HYPERCYLINDER *x = (rt_HYPERCYLINDER *)o->obj.pobj;
        sci[mp_j] = 0.0f;
        sci[mp_k] = -(x->rat * x->rat);
        sci[RT_W] = x->hyp;
    } break;
    case RT_TAG_HYPERPARABOLOID:
    {
        rt_HYPERPARABOLOID *x = (rt_HYPERPARABOLOID *)o->obj.pobj;
        sci[mp_i] = 1.0f / +fabs_(x->pr1);
        sci[mp_j] = 1.0f / -fabs_(x->pr2);
        sci[mp_k] = 0.0f;
        scj[mp_k] = 1.0f * (rt_real)n->sgn[RT_K];
    } break;
    }

    /* rt_Quadric::commit_fields (object.cpp:3059-3088) */
    float isc[3];
    isc[RT_X] = 1.0f / n->scl[RT_X];
    isc[RT_Y] = 1.0f / n->scl[RT_Y];
    isc[RT_Z] = 1.0f / n->scl[RT_Z];
    sci[RT_X] *= isc[RT_X] * isc[RT_X];
    sci[RT_Y] *= isc[RT_Y] * isc[RT_Y];
    sci[RT_Z] *= isc[RT_Z] * isc[RT_Z];
    scj[RT_X] *= isc[RT_X];
    scj[RT_Y] *= isc[RT_Y];
    scj[RT_Z] *= isc[RT_Z];
    n->rec.sci[0] = sci[RT_X];
    n->rec.sci[1] = sci[RT_Y];
    n->rec.sci[2] = sci[RT_Z];
    n->rec.sci[3] = sci[RT_W];
    n->rec.scj[0] = scj[RT_X] * 0.5f;
    n->rec.scj[1] = scj[RT_Y] * 0.5f;
    n->rec.scj[2] = scj[RT_Z] * 0.5f;
}

/* ---- phase 2: clip boxes (object.cpp:2533-2870 and per-shape
 *      adjust_minmax 2982-3009, 3163-3971) -------------------------------- */

void Flat::adjust_minmax(Node *n, const float *smin, const float *smax,
                         float *bmin, float *bmax, float *cmin, float *cmax)
{
    rt_SURFACE *srf = n->srf;
    rt_OBJECT *o = n->obj;
    const float INF = RT_INF;

    /* rt_Surface::adjust_minmax (object.cpp:2533-2549) */
    if (cmin != RT_NULL && cmax != RT_NULL)
    {
        cmin[RT_I] = smin[RT_I] > srf->min[RT_I] ? -INF : smin[RT_I];
        cmin[RT_J] = smin[RT_J] > srf->min[RT_J] ? -INF : smin[RT_J];
        cmin[RT_K] = smin[RT_K] > srf->min[RT_K] ? -INF : smin[RT_K];
        cmax[RT_I] = smax[RT_I] < srf->max[RT_I] ? +INF : smax[RT_I];
        cmax[RT_J] = smax[RT_J] < srf->max[RT_J] ? +INF : smax[RT_J];
        cmax[RT_K] = smax[RT_K] < srf->max[RT_K] ? +INF : smax[RT_K];
    }
    bool cb = (cmin != RT_NULL && cmax != RT_NULL);

    switch (n->tag)
    {
    case RT_TAG_PLANE:
        if (cb) { cmin[RT_K] = -INF; cmax[RT_K] = +INF; }
        if (bmin != RT_NULL && bmax != RT_NULL)
        {
            bmin[RT_I] = smin[RT_I]; bmin[RT_J] = smin[RT_J]; bmin[RT_K] = 0.0f;
            bmax[RT_I] = smax[RT_I]; bmax[RT_J] = smax[RT_J]; bmax[RT_K] = 0.0f;
        }
        break;

    case RT_TAG_CYLINDER:
    {
        rt_CYLINDER *x = (rt_CYLINDER *)o->obj.pobj;
        float rad = fabs_(x->rad);
        if (cb)
        {
            cmin[RT_I] = cmin[RT_I] <= -rad ? -INF : cmin[RT_I];
            cmin[RT_J] = cmin[RT_J] <= -rad ? -INF : cmin[RT_J];
            cmax[RT_I] = cmax[RT_I] >= +rad ? +INF : cmax[RT_I];
            cmax[RT_J] = cmax[RT_J] >= +rad ? +INF : cmax[RT_J];
        }
        if (bmin != RT_NULL && bmax != RT_NULL)
        {
            bmin[RT_I] = RT_MAX(smin[RT_I], -rad);
            bmin[RT_J] = RT_MAX(smin[RT_J], -rad);
            bmin[RT_K] = smin[RT_K];
            bmax[RT_I] = RT_MIN(smax[RT_I], +rad);
            bmax[RT_J] = RT_MIN(smax[RT_J], +rad);
            bmax[RT_K] = smax[RT_K];
        }
    } break;

    case RT_TAG_SPHERE:
    {
        rt_SPHERE *x = (rt_SPHERE *)o->obj.pobj;
        float top, r = fabs_(x->rad);
        float rad[3] = {r, r, r};
        for (int k = 0; k < 3; k++)
        {
            top = smin[k] > 0.0f ? +smin[k] : smax[k] < 0.0f ? -smax[k] : 0.0f;
            r = sqrt_(RT_MAX(x->rad * x->rad - top * top, 0.0f));
            int i = (k + 1) % 3;
            if (rad[i] > r) rad[i] = r;
            int j = (k + 2) % 3;
            if (rad[j] > r) rad[j] = r;
        }
        if (cb)
        {
            cmin[RT_I] = cmin[RT_I] <= -rad[RT_I] ? -INF : cmin[RT_I];
            cmin[RT_J] = cmin[RT_J] <= -rad[RT_J] ? -INF : cmin[RT_J];
            cmin[RT_K] = cmin[RT_K] <= -rad[RT_K] ? -INF : cmin[RT_K];
            cmax[RT_I] = cmax[RT_I] >= +rad[RT_I] ? +INF : cmax[RT_I];
            cmax[RT_J] = cmax[RT_J] >= +rad[RT_J] ? +INF : cmax[RT_J];
            cmax[RT_K] = cmax[RT_K] >= +rad[RT_K] ? +INF : cmax[RT_K];
        }
        if (bmin != RT_NULL && bmax != RT_NULL)
        {
            bmin[RT_I] = RT_MAX(smin[RT_I], -rad[RT_I]);
            bmin[RT_J] = RT_MAX(smin[RT_J], -rad[RT_J]);
            bmin[RT_K] = RT_MAX(smin[RT_K], -rad[RT_K]);
            bmax[RT_I] = RT_MIN(smax[RT_I], +rad[RT_I]);
            bmax[RT_J] = RT_MIN(smax[RT_J], +rad[RT_J]);
            bmax[RT_K] = RT_MIN(smax[RT_K], +rad[RT_K]);
        }
    } break;

    case RT_TAG_CONE:
    {
        rt_CONE *x = (rt_CONE *)o->obj.pobj;
        float rat = fabs_(x->rat);
        float top = RT_MAX(fabs_(smin[RT_K]), fabs_(smax[RT_K]));
        float rad = top != INF ? top * rat : INF;
        float mxi = RT_MAX(fabs_(smin[RT_I]), fabs_(smax[RT_I]));
        float mxj = RT_MAX(fabs_(smin[RT_J]), fabs_(smax[RT_J]));
        top = RT_MIN(mxi != INF && mxj != INF ?
                     sqrt_(mxi * mxi + mxj * mxj) / rat : top, top);
        if (cb)
        {
            cmin[RT_I] = cmin[RT_I] <= -rad ? -INF : cmin[RT_I];
            cmin[RT_J] = cmin[RT_J] <= -rad ? -INF : cmin[RT_J];
            cmin[RT_K] = cmin[RT_K] <  -top ? -INF : cmin[RT_K];
            cmax[RT_I] = cmax[RT_I] >= +rad ? +INF : cmax[RT_I];
            cmax[RT_J] = cmax[RT_J] >= +rad ? +INF : cmax[RT_J];
            cmax[RT_K] = cmax[RT_K] >  +top ? +INF : cmax[RT_K];
        }
        if (bmin != RT_NULL && bmax != RT_NULL)
        {
            bmin[RT_I] = RT_MAX(smin[RT_I], -rad);
            bmin[RT_J] = RT_MAX(smin[RT_J], -rad);
            bmin[RT_K] = cb ? RT_MAX(smin[RT_K], -top) : smin[RT_K];
            bmax[RT_I] = RT_MIN(smax[RT_I], +rad);
            bmax[RT_J] = RT_MIN(smax[RT_J], +rad);
            bmax[RT_K] = cb ? RT_MIN(smax[RT_K], +top) : smax[RT_K];
        }
    } break;

    case RT_TAG_PARABOLOID:
    {
        rt_PARABOLOID *x = (rt_PARABOLOID *)o->obj.pobj;
        float par = x->par;
        float top = RT_MAX(par < 0.0f ? -smin[RT_K] : +smax[RT_K], 0.0f);
        float rad = top != INF ? sqrt_(top * fabs_(par)) : INF;
        float mxi = RT_MAX(fabs_(smin[RT_I]), fabs_(smax[RT_I]));
        float mxj = RT_MAX(fabs_(smin[RT_J]), fabs_(smax[RT_J]));
        top = RT_MIN(mxi != INF && mxj != INF ?
                     (mxi * mxi + mxj * mxj) / fabs_(par) : top, top);
        if (cb)
        {
            cmin[RT_I] = cmin[RT_I] <= -rad ? -INF : cmin[RT_I];
            cmin[RT_J] = cmin[RT_J] <= -rad ? -INF : cmin[RT_J];
            cmin[RT_K] = (cmin[RT_K] <= 0.0f && par > 0.0f) ||
                         (cmin[RT_K] <  -top && par < 0.0f) ? -INF : cmin[RT_K];
            cmax[RT_I] = cmax[RT_I] >= +rad ? +INF : cmax[RT_I];
            cmax[RT_J] = cmax[RT_J] >= +rad ? +INF : cmax[RT_J];
            cmax[RT_K] = (cmax[RT_K] >= 0.0f && par < 0.0f) ||
                         (cmax[RT_K] >  +top && par > 0.0f) ? +INF : cmax[RT_K];
        }
        if (bmin != RT_NULL && bmax != RT_NULL)
        {
            bmin[RT_I] = RT_MAX(smin[RT_I], -rad);
            bmin[RT_J] = RT_MAX(smin[RT_J], -rad);
            bmin[RT_K] = par > 0.0f ? RT_MAX(smin[RT_K], 0.0f) :
                         cb ? RT_MAX(smin[RT_K], -top) : smin[RT_K];
            bmax[RT_I] = RT_MIN(smax[RT_I], +rad);
            bmax[RT_J] = RT_MIN(smax[RT_J], +rad);
            bmax[RT_K] = par < 0.0f ? RT_MIN(smax[RT_K], 0.0f) :
                         cb ? RT_MIN(smax[RT_K], +top) : smax[RT_K];
        }
    } break;

    case RT_TAG_HYPERBOLOID:
    {
        rt_HYPERBOLOID *x = (rt_HYPERBOLOID *)o->obj.pobj;
        float rat = fabs_(x->rat);
        float hyp = x->hyp;
        float top = RT_MAX(fabs_(smin[RT_K]), fabs_(smax[RT_K]));
        float rad = top != INF ? sqrt_(top * top * rat * rat + hyp) : INF;
        float mxi = RT_MAX(fabs_(smin[RT_I]), fabs_(smax[RT_I]));
        float mxj = RT_MAX(fabs_(smin[RT_J]), fabs_(smax[RT_J]));
        top = RT_MIN(mxi != INF && mxj != INF ?
                     sqrt_(mxi * mxi + mxj * mxj - hyp) / rat : top, top);
        if (cb)
        {
            cmin[RT_I] = cmin[RT_I] <= -rad ? -INF : cmin[RT_I];
            cmin[RT_J] = cmin[RT_J] <= -rad ? -INF : cmin[RT_J];
            cmin[RT_K] = cmin[RT_K] <  -top ? -INF : cmin[RT_K];
            cmax[RT_I] = cmax[RT_I] >= +rad ? +INF : cmax[RT_I];
            cmax[RT_J] = cmax[RT_J] >= +rad ? +INF : cmax[RT_J];
            cmax[RT_K] = cmax[RT_K] >  +top ? +INF : cmax[RT_K];
        }
        if (bmin != RT_NULL && bmax != RT_NULL)
        {
            bmin[RT_I] = RT_MAX(smin[RT_I], -rad);
            bmin[RT_J] = RT_MAX(smin[RT_J], -rad);
            bmin[RT_K] = cb ? RT_MAX(smin[RT_K], -top) : smin[RT_K];
            bmax[RT_I] = RT_MIN(smax[RT_I], +rad);
            bmax[RT_J] = RT_MIN(smax[RT_J], +rad);
            bmax[RT_K] = cb ? RT_MIN(smax[RT_K], +top) : smax[RT_K];
        }
    } break;

    case RT_TAG_PARACYLINDER:
    {
        rt_PARACYLINDER *x = (rt_PARACYLINDER *)o->obj.pobj;
        float par = x->par;
        float top = RT_MAX(par < 0.0f ? -smin[RT_K] : +smax[RT_K], 0.0f);
        float rad = top != INF ? sqrt_(top * fabs_(par)) : INF;
        float mxi = RT_MAX(fabs_(smin[RT_I]), fabs_(smax[RT_I]));
        top = RT_MIN(mxi != INF ? (mxi * mxi) / fabs_(par) : top, top);
        if (cb)
        {
            cmin[RT_I] = cmin[RT_I] <= -rad ? -INF : cmin[RT_I];
            cmin[RT_K] = (cmin[RT_K] <= 0.0f && par > 0.0f) ||
                         (cmin[RT_K] <  -top && par < 0.0f) ? -INF : cmin[RT_K];
            cmax[RT_I] = cmax[RT_I] >= +rad ? +INF : cmax[RT_I];
            cmax[RT_K] = (cmax[RT_K] >= 0.0f && par < 0.0f) ||
                         (cmax[RT_K] >  +top && par > 0.0f) ? +INF : cmax[RT_K];
        }
        if (bmin != RT_NULL && bmax != RT_NULL)
        {
            bmin[RT_I] = RT_MAX(smin[RT_I], -rad);
            bmin[RT_J] = smin[RT_J];
            bmin[RT_K] = par > 0.0f ? RT_MAX(smin[RT_K], 0.0f) :
                         cb ? RT_MAX(smin[RT_K], -top) : smin[RT_K];
            bmax[RT_I] = RT_MIN(smax[RT_I], +rad);
            bmax[RT_J] = smax[RT_J];
            bmax[RT_K] = par < 0.0f ? RT_MIN(smax[RT_K], 0.0f) :
                         cb ? RT_MIN(smax[RT_K], +top) : smax[RT_K];
        }
    } break;

    case RT_TAG_HYPERCYLINDER:
    {
        rt_HYPERCYLINDER *x = (rt_HYPERCYLINDER *)o->obj.pobj;
        float rat = fabs_(x->rat);
        float hyp = x->hyp;
        float top = RT_MAX(fabs_(smin[RT_K]), fabs_(smax[RT_K]));
        float rad = top != INF ? sqrt_(top * top * rat * rat + hyp) : INF;
        float mxi = RT_MAX(fabs_(smin[RT_I]), fabs_(smax[RT_I]));
        top = RT_MIN(mxi != INF ? sqrt_(mxi * mxi - hyp) / rat : top, top);
        if (cb)
        {
            cmin[RT_I] = cmin[RT_I] <= -rad ? -INF : cmin[RT_I];
            cmin[RT_K] = cmin[RT_K] <  -top ? -INF : cmin[RT_K];
            cmax[RT_I] = cmax[RT_I] >= +rad ? +INF : cmax[RT_I];
            cmax[RT_K] = cmax[RT_K] >  +top ? +INF : cmax[RT_K];
        }
        if (bmin != RT_NULL && bmax != RT_NULL)
        {
            bmin[RT_I] = RT_MAX(smin[RT_I], -rad);
            bmin[RT_J] = smin[RT_J];
            bmin[RT_K] = cb ? RT_MAX(smin[RT_K], -top) : smin[RT_K];
            bmax[RT_I] = RT_MIN(smax[RT_I], +rad);
            bmax[RT_J] = smax[RT_J];
            bmax[RT_K] = cb ? RT_MIN(smax[RT_K], +top) : smax[RT_K];
        }
    } break;

    case RT_TAG_HYPERPARABOLOID:
    {
        rt_HYPERPARABOLOID *x = (rt_HYPERPARABOLOID *)o->obj.pobj;
        float rd1 = RT_MAX(-smin[RT_I], +smax[RT_I]);
        float rd2 = RT_MAX(-smin[RT_J], +smax[RT_J]);
        float tp1 = rd1 * rd1 / fabs_(x->pr1);
        float tp2 = rd2 * rd2 / fabs_(x->pr2);
        if (cb)
        {
            cmin[RT_K] = cmin[RT_K] <= -tp2 ? -INF : cmin[RT_K];
            cmax[RT_K] = cmax[RT_K] >= +tp1 ? +INF : cmax[RT_K];
        }
        if (bmin != RT_NULL && bmax != RT_NULL)
        {
            bmin[RT_I] = smin[RT_I];
            bmin[RT_J] = smin[RT_J];
            bmin[RT_K] = cb ? RT_MAX(smin[RT_K], -tp2) : smin[RT_K];
            bmax[RT_I] = smax[RT_I];
            bmax[RT_J] = smax[RT_J];
            bmax[RT_K] = cb ? RT_MIN(smax[RT_K], +tp1) : smax[RT_K];
        }
    } break;
    }
}

/* local IJK box -> sub-world XYZ box (object.cpp:2600-2631) */
void Flat::direct_minmax(Node *n, const float *smin, const float *smax,
                         float *dmin, float *dmax)
{
    const float INF = RT_INF;
    float tmin[4], tmax[4];
    float zro[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    float pos[4] = {n->mtx[3][0], n->mtx[3][1], n->mtx[3][2], 0.0f};
    float *pps = n->trnode == n ? zro : pos;
    int mp_i = n->map[RT_I], mp_j = n->map[RT_J], mp_k = n->map[RT_K];
    int *sgn = n->sgn;
    float *scl = n->scl;

    tmin[mp_i] = sgn[RT_I] > 0 ? +smin[RT_I] : -smax[RT_I];
    tmin[mp_j] = sgn[RT_J] > 0 ? +smin[RT_J] : -smax[RT_J];
    tmin[mp_k] = sgn[RT_K] > 0 ? +smin[RT_K] : -smax[RT_K];
    tmax[mp_i] = sgn[RT_I] > 0 ? +smax[RT_I] : -smin[RT_I];
    tmax[mp_j] = sgn[RT_J] > 0 ? +smax[RT_J] : -smin[RT_J];
    tmax[mp_k] = sgn[RT_K] > 0 ? +smax[RT_K] : -smin[RT_K];

    for (int k = 0; k < 3; k++)
    {
        tmin[k] = tmin[k] == -INF ? -INF : tmin[k] * scl[k];
        tmax[k] = tmax[k] == +INF ? +INF : tmax[k] * scl[k];
    }
    for (int k = 0; k < 3; k++)
    {
        dmin[k] = tmin[k] == -INF ? -INF : tmin[k] + pps[k];
        dmax[k] = tmax[k] == +INF ? +INF : tmax[k] + pps[k];
    }
}

/* sub-world XYZ box -> local IJK box (object.cpp:2559-2590) */
void Flat::invert_minmax(Node *n, const float *smin, const float *smax,
                         float *dmin, float *dmax)
{
    const float INF = RT_INF;
    float tmin[4], tmax[4];
    float zro[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    float pos[4] = {n->mtx[3][0], n->mtx[3][1], n->mtx[3][2], 0.0f};
    float *pps = n->trnode == n ? zro : pos;
    int mp_i = n->map[RT_I], mp_j = n->map[RT_J], mp_k = n->map[RT_K];
    int *sgn = n->sgn;
    float *scl = n->scl;

    for (int k = 0; k < 3; k++)
    {
        tmin[k] = smin[k] == -INF ? -INF : smin[k] - pps[k];
        tmax[k] = smax[k] == +INF ? +INF : smax[k] - pps[k];
    }
    for (int k = 0; k < 3; k++)
    {
        tmin[k] = tmin[k] == -INF ? -INF : tmin[k] / scl[k];
        tmax[k] = tmax[k] == +INF ? +INF : tmax[k] / scl[k];
    }
    dmin[RT_I] = sgn[RT_I] > 0 ? +tmin[mp_i] : -tmax[mp_i];
    dmin[RT_J] = sgn[RT_J] > 0 ? +tmin[mp_j] : -tmax[mp_j];
    dmin[RT_K] = sgn[RT_K] > 0 ? +tmin[mp_k] : -tmax[mp_k];
    dmax[RT_I] = sgn[RT_I] > 0 ? +tmax[mp_i] : -tmin[mp_i];
    dmax[RT_J] = sgn[RT_J] > 0 ? +tmax[mp_j] : -tmin[mp_j];
    dmax[RT_K] = sgn[RT_K] > 0 ? +tmax[mp_k] : -tmin[mp_k];
}

/* rt_Surface::recalc_minmax (object.cpp:2636-2710) */
void Flat::recalc_minmax(Node *n, float *smin, float *smax, float *bmin,
                         float *bmax, float *cmin, float *cmax)
{
    const float INF = RT_INF;
    float tmin[4], tmax[4], lmin[4], lmax[4];
    float *pmin = RT_NULL, *pmax = RT_NULL;
    rt_SURFACE *srf = n->srf;

    if (smin != RT_NULL && smax != RT_NULL && bmin == RT_NULL && bmax == RT_NULL)
    {
        invert_minmax(n, smin, smax, tmin, tmax);
        bmin = lmin;
        bmax = lmax;
        pmin = cmin;
        pmax = cmax;
        cmin = RT_NULL;
        cmax = RT_NULL;
    }
    else if (smin != RT_NULL && smax != RT_NULL && cmin != RT_NULL && cmax != RT_NULL)
    {
        invert_minmax(n, smin, smax, tmin, tmax);
        for (int k = 0; k < 3; k++)
        {
            tmin[k] = RT_MAX(tmin[k], srf->min[k]);
            tmax[k] = RT_MIN(tmax[k], srf->max[k]);
        }
    }
    else if (smin == RT_NULL && smax == RT_NULL)
    {
        for (int k = 0; k < 3; k++)
        {
            tmin[k] = srf->min[k];
            tmax[k] = srf->max[k];
        }
    }

    adjust_minmax(n, tmin, tmax, bmin, bmax, cmin, cmax);

    if (pmin != RT_NULL && pmax != RT_NULL)
    {
        for (int k = 0; k < 3; k++)
        {
            tmin[k] = tmin[k] == bmin[k] ? -INF : bmin[k];
            tmax[k] = tmax[k] == bmax[k] ? +INF : bmax[k];
        }
        direct_minmax(n, tmin, tmax, tmin, tmax);
        for (int k = 0; k < 3; k++)
        {
            pmin[k] = RT_MAX(pmin[k], tmin[k]);
            pmax[k] = RT_MIN(pmax[k], tmax[k]);
        }
        bmin = RT_NULL;
        bmax = RT_NULL;
    }
    if (bmin != RT_NULL && bmax != RT_NULL)
    {
        direct_minmax(n, bmin, bmax, bmin, bmax);
    }
    if (cmin != RT_NULL && cmax != RT_NULL)
    {
        direct_minmax(n, cmin, cmax, cmin, cmax);
    }
}

/* rt_Surface::update_minmax / update_bounds (object.cpp:2715-2870) */
void Flat::bounds(Node *n)
{
    const float INF = RT_INF;
    bool has_clip = false;
    for (size_t i = 0; i < n->rel.size(); i++) has_clip = true;

    if ((opts & RT_OPTS_ADJUST) == 0 || !has_clip || n->trnode == n)
    {
        recalc_minmax(n, RT_NULL, RT_NULL, n->bmin, n->bmax, n->cmin, n->cmax);
    }
    else
    {
        recalc_minmax(n, RT_NULL, RT_NULL, n->bmin, n->bmax, RT_NULL, RT_NULL);
        for (int k = 0; k < 3; k++) { n->cmin[k] = -INF; n->cmax[k] = +INF; }
        int skip = 0;
        for (size_t i = 0; i < n->rel.size(); i++)
        {
            Node *o = n->rel[i].obj;
            if (o == RT_NULL)
            {
                skip = 1 - skip;
            }
            if (o == RT_NULL || skip == 1 || o->kind != K_SURFACE ||
                o->tag == RT_TAG_PLANE || o->trnode != n->trnode ||
                n->rel[i].data != RT_REL_MINUS_OUTER)
            {
                continue;
            }
            recalc_minmax(o, n->bmin, n->bmax, RT_NULL, RT_NULL, n->cmin, n->cmax);
        }
        recalc_minmax(n, n->cmin, n->cmax, n->bmin, n->bmax, n->cmin, n->cmax);
    }

    qr_srf &s = n->rec;
    s.mint = (n->cmin[RT_X] == -INF ? 0 : 1) | (n->cmin[RT_Y] == -INF ? 0 : 2) |
             (n->cmin[RT_Z] == -INF ? 0 : 4);
    s.maxt = (n->cmax[RT_X] == +INF ? 0 : 1) | (n->cmax[RT_Y] == +INF ? 0 : 2) |
             (n->cmax[RT_Z] == +INF ? 0 : 4);
    float zro[3] = {0.0f, 0.0f, 0.0f};
    float pos[3] = {n->mtx[3][0], n->mtx[3][1], n->mtx[3][2]};
    float *pps = n->trnode == n ? zro : pos;
    for (int k = 0; k < 3; k++)
    {
        s.bmin[k] = n->bmin[k] - pps[k];
        s.bmax[k] = n->bmax[k] - pps[k];
    }
}

/* ---- per-frame update --------------------------------------------------- */

void Flat::update(rt_time time)
{
    /* phase 0.5 */
    update_object(root, time, 0, RT_NULL, (float (*)[4])iden4);

    /* phase 1: arrays, cameras, lights, surfaces (engine.cpp:3399-3451) */
    for (size_t i = 0; i < arrays.size(); i++)
    {
        if (arrays[i]->obj_changed) fields_array(arrays[i]);
    }
    for (size_t i = 0; i < cameras.size(); i++)
    {
        Node *c = cameras[i];
        if (c->obj_changed) update_matrix(c, c->pmtx);
    }
    for (size_t i = 0; i < lights.size(); i++)
    {
        Node *l = lights[i];
        if (l->obj_changed) update_matrix(l, l->pmtx);
    }
    for (size_t i = 0; i < surfaces.size(); i++)
    {
        if (surfaces[i]->obj_changed) fields_surface(surfaces[i]);
    }
    /* phase 2: clip boxes */
    for (size_t i = 0; i < surfaces.size(); i++)
    {
        bounds(surfaces[i]);
    }
    /* phase 3: solver kinds (rt_Platform::update0, tracer.cpp:8115-8149) */
    for (size_t i = 0; i < surfaces.size(); i++)
    {
        qr_srf &s = surfaces[i]->rec;
        int tag = surfaces[i]->tag;
        s.solver = tag > RT_TAG_PLANE ?
                   ((tag == RT_TAG_HYPERCYLINDER && s.sci[3] == 0.0f) ? 3 : 2) : 1;
        s.nrmk = tag > RT_TAG_PLANE ?
                 ((tag != RT_TAG_PARABOLOID && tag != RT_TAG_PARACYLINDER &&
                   tag != RT_TAG_HYPERPARABOLOID) ? 3 : 2) : 1;
        s.clpk = s.nrmk;
        s.conic = (tag == RT_TAG_CONE ||
                   (tag == RT_TAG_HYPERBOLOID && s.sci[3] == 0.0f)) ? 1 :
                  (tag == RT_TAG_HYPERCYLINDER && s.sci[3] == 0.0f) ? 2 : 0;
    }
    emit_records();
    emit_lists();
    hor_sin = sina_(cameras[cam_idx]->trm->rot[RT_Z]);
    hor_cos = cosa_(cameras[cam_idx]->trm->rot[RT_Z]);
}

int Flat::next_cam()
{
    const int n = (int)cameras.size();
    int r = n - 1 - cam_idx;
    r = r + 1 < n ? r + 1 : 0;
    cam_idx = n - 1 - r;
    return r;
}

void Flat::camera_action(rt_time time, int action)
{
    Node *cn = cameras[cam_idx];
    rt_CAMERA *cam = (rt_CAMERA *)cn->obj->obj.pobj;
    rt_TRANSFORM3D *trm = cn->trm;
    const rt_real t = (time - cn->obj->time) / 50.0f;
    switch (action)
    {
    case RT_CAMERA_MOVE_UP:     trm->pos[RT_Z] += cam->dps[RT_K] * t; break;
    case RT_CAMERA_MOVE_DOWN:   trm->pos[RT_Z] -= cam->dps[RT_K] * t; break;
    case RT_CAMERA_MOVE_LEFT:
        trm->pos[RT_X] -= cam->dps[RT_I] * t * hor_cos;
        trm->pos[RT_Y] -= cam->dps[RT_I] * t * hor_sin; break;
    case RT_CAMERA_MOVE_RIGHT:
        trm->pos[RT_X] += cam->dps[RT_I] * t * hor_cos;
        trm->pos[RT_Y] += cam->dps[RT_I] * t * hor_sin; break;
    case RT_CAMERA_MOVE_BACK:
        trm->pos[RT_X] += cam->dps[RT_J] * t * hor_sin;
        trm->pos[RT_Y] -= cam->dps[RT_J] * t * hor_cos; break;
    case RT_CAMERA_MOVE_FORWARD:
        trm->pos[RT_X] -= cam->dps[RT_J] * t * hor_sin;
        trm->pos[RT_Y] += cam->dps[RT_J] * t * hor_cos; break;
    case RT_CAMERA_ROTATE_LEFT:
        trm->rot[RT_Z] += cam->drt[RT_I] * t;
        if (trm->rot[RT_Z] >= +180.0f) trm->rot[RT_Z] -= +360.0f; break;
    case RT_CAMERA_ROTATE_RIGHT:
        trm->rot[RT_Z] -= cam->drt[RT_I] * t;
        if (trm->rot[RT_Z] <= -180.0f) trm->rot[RT_Z] += +360.0f; break;
    case RT_CAMERA_ROTATE_UP:
        if (trm->rot[RT_X] < 0.0f)
        {
            trm->rot[RT_X] += cam->drt[RT_J] * t;
            if (trm->rot[RT_X] > 0.0f) trm->rot[RT_X] = 0.0f;
        } break;
    case RT_CAMERA_ROTATE_DOWN:
        if (trm->rot[RT_X] > -180.0f)
        {
            trm->rot[RT_X] -= cam->drt[RT_J] * t;
            if (trm->rot[RT_X] < -180.0f) trm->rot[RT_X] = -180.0f;
        } break;
    default: break;
    }
}

/* ---- device-side update phases ------------------------------------------ */

/* the rotation flag of rt_Object::update_matrix (object.cpp:236-247): set
 * unless every angle is a multiple of 90 degrees */
static int rot_flag(const rt_TRANSFORM3D *trm)
{
    const float frt[] = {-270.0f, -180.0f, -90.0f, 0.0f, +90.0f, +180.0f, +270.0f};
    int c = 0;
    for (int i = 0; i < 7; i++)
    {
        if (trm->rot[RT_X] == frt[i]) c++;
        if (trm->rot[RT_Y] == frt[i]) c++;
        if (trm->rot[RT_Z] == frt[i]) c++;
    }
    return c == 3 ? 0 : FLAG_ROT;
}

static void copy16(float *d, const float (*m)[4])
{
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) d[4 * i + j] = m[i][j];
}

int Flat::anim_table(std::vector<qr_anim_node> &out, std::string *why)
{
    out.clear();
    anim_nodes.clear();
    anim_scl.clear();
    std::vector<int> entry(nodes.size(), -1);
    std::unordered_map<const Node*, int> at;
    for (size_t i = 0; i < nodes.size(); i++) at[nodes[i]] = (int)i;
    /* nodes are in creation order: every parent before its children */
    for (size_t i = 0; i < nodes.size(); i++)
    {
        Node *n = nodes[i];
        const bool animated = n->obj->f_anim != RT_NULL;
        Node *t0 = n->parent != RT_NULL ? n->parent->trnode : RT_NULL;
        const int t0e = t0 != RT_NULL ? entry[at[t0]] : -1;
        const float (*pm)[4] = n->parent != RT_NULL ? (const float (*)[4])n->parent->pmtx : iden4;
        const int rot = rot_flag(n->trm);
        if (animated && !rot)
        {
            if (why) *why = "an animated object has no free rotation";
            return 1;
        }
        if (n->kind == K_CAMERA && (animated || t0e >= 0))
        {
            if (why) *why = "a camera moves with an animated object";
            return 2;
        }
        qr_anim_node e;
        memset(&e, 0, sizeof(e));
        e.parent = -1;
        e.param = -1;
        e.rec = -1;
        e.light = -1;
        float P[4][4], R[4][4];
        bool dyn = false;
        if (rot)
        {
            if (!animated && t0e < 0) continue;
            dyn = true;
            if (t0 == RT_NULL)
            {
                e.kind = QR_ANIM_OWN;
                memcpy(P, pm, sizeof(P));
            }
            else if (t0e < 0)
            {
                e.kind = QR_ANIM_OWN;
                mat_mul_mat(P, t0->mtx, pm);
            }
            else
            {
                e.kind = QR_ANIM_UNDER;
                e.parent = t0e;
                memcpy(P, pm, sizeof(P));
            }
            mat_from_transform(R, n->trm, 0);
            if (animated)
            {
                e.param = (int)anim_nodes.size();
                anim_nodes.push_back(n);
                std::vector<float> sc(n->trm->scl, n->trm->scl + 3);
                anim_scl.push_back(sc);
            }
        }
        else
        {
            const bool clause = t0 != RT_NULL && t0 != n &&
                                ((opts & RT_OPTS_TARRAY) == 0 || n->tag > RT_TAG_SURFACE_MAX);
            if (!clause || t0e < 0) continue;
            dyn = true;
            e.kind = QR_ANIM_NODE;
            e.parent = t0e;
            float trm_mtx[4][4];
            mat_from_transform(trm_mtx, n->trm, 1);
            mat_mul_mat(P, pm, trm_mtx);
            memset(R, 0, sizeof(R));
        }
        if (!dyn || n->trnode != n)
        {
            if (why) *why = "a moving object is not a transform node";
            return 3;
        }
        copy16(e.p, P);
        copy16(e.r, R);
        if (n->kind == K_SURFACE || n->kind == K_ARRAY) e.rec = n->index;
        if (n->kind == K_LIGHT)
        {
            for (size_t j = 0; j < lights.size(); j++)
                if (lights[j] == n) e.light = (int)j;
        }
        entry[i] = (int)out.size();
        out.push_back(e);
    }

    /* the recipes must give the matrices of the last update */
    std::vector<float> M(16 * out.size());
    for (size_t i = 0; i < nodes.size(); i++)
    {
        if (entry[i] < 0) continue;
        const qr_anim_node &e = out[entry[i]];
        float P[4][4], R[4][4], T[4][4], tmp[4][4], m[4][4];
        memcpy(P, e.p, sizeof(P));
        memcpy(R, e.r, sizeof(R));
        if (e.param >= 0) mat_from_transform(R, nodes[i]->trm, 0);
        if (e.parent >= 0) memcpy(T, &M[16 * e.parent], sizeof(T));
        if (e.kind == QR_ANIM_OWN) mat_mul_mat(m, P, R);
        else if (e.kind == QR_ANIM_UNDER) { mat_mul_mat(tmp, T, P); mat_mul_mat(m, tmp, R); }
        else mat_mul_mat(m, T, P);
        memcpy(&M[16 * entry[i]], m, sizeof(m));
        if (memcmp(m, nodes[i]->mtx, sizeof(m)) != 0)
        {
            if (why) *why = "the update table does not reproduce a transform";
            return 4;
        }
    }
    return 0;
}

int Flat::anim_params(rt_time time, std::vector<qr_anim_param> &out)
{
    /* animators and time stamps as in update_status (object.cpp:175-216) */
    for (size_t i = 0; i < nodes.size(); i++)
    {
        rt_OBJECT *obj = nodes[i]->obj;
        if (obj->f_anim != RT_NULL && obj->time != time)
        {
            obj->f_anim(time, obj->time < 0 ? 0 : obj->time, nodes[i]->trm, RT_NULL);
        }
        obj->time = time;
    }
    /* cameras as update() leaves them: phase 0.5 status, phase 1 matrix,
     * and the heading camera actions use */
    for (size_t i = 0; i < cameras.size(); i++)
    {
        Node *c = cameras[i];
        update_status(c, time, c->in_flags, c->parent != RT_NULL ? c->parent->trnode : RT_NULL);
        if (c->obj_changed) update_matrix(c, c->pmtx);
    }
    hor_sin = sina_(cameras[cam_idx]->trm->rot[RT_Z]);
    hor_cos = cosa_(cameras[cam_idx]->trm->rot[RT_Z]);
    out.resize(anim_nodes.size());
    int rc = 0;
    for (size_t i = 0; i < anim_nodes.size(); i++)
    {
        const rt_TRANSFORM3D *t = anim_nodes[i]->trm;
        if (!rot_flag(t)) rc = 1;
        for (int k = 0; k < 3; k++)
            if (memcmp(&t->scl[k], &anim_scl[i][k], sizeof(float)) != 0) rc = 2;
        qr_anim_param &q = out[i];
        memset(&q, 0, sizeof(q));
        for (int k = 0; k < 3; k++)
        {
            q.sin[k] = sina_(t->rot[k]);
            q.cos[k] = cosa_(t->rot[k]);
            q.pos[k] = t->pos[k];
        }
    }
    return rc;
}

void Flat::emit_records()
{
    srf.clear();
    mat.clear();
    lgt.clear();
    texels.clear();

    /* surfaces first (index = creation order), then transform nodes */
    for (size_t i = 0; i < surfaces.size(); i++) surfaces[i]->index = (int)i;
    int k = (int)surfaces.size();
    for (size_t i = 0; i < arrays.size(); i++) arrays[i]->index = k++;

    for (size_t i = 0; i < mats.size(); i++)
    {
        Material &M = mats[i];
        M.m.tex_off = (int32_t)texels.size();
        for (int t = 0; t < M.x_dim * M.y_dim; t++) texels.push_back(M.texels[t]);
        mat.push_back(M.m);
    }
    for (size_t i = 0; i < surfaces.size(); i++)
    {
        Node *n = surfaces[i];
        qr_srf s = n->rec;
        s.mat[0] = n->outer;
        s.mat[1] = n->inner;
        s.props[0] = mats[n->outer].props;
        s.props[1] = mats[n->inner].props;
        s.trnode = (n->trnode != RT_NULL && n->trnode != n) ? n->trnode->index : -1;
        s.is_node = 0;
        srf.push_back(s);
    }
    for (size_t i = 0; i < arrays.size(); i++)
    {
        qr_srf s = arrays[i]->rec;
        s.is_node = 1;
        s.trnode = -1;
        srf.push_back(s);
    }
    for (size_t i = 0; i < lights.size(); i++)
    {
        Node *n = lights[i];
        rt_LIGHT *l = (rt_LIGHT *)n->obj->obj.pobj;
        qr_light L;
        memset(&L, 0, sizeof(L));
        L.pos[0] = n->mtx[3][RT_X];
        L.pos[1] = n->mtx[3][RT_Y];
        L.pos[2] = n->mtx[3][RT_Z];
        L.t_max = 1.0f;
        L.col[0] = n->lcol[0];
        L.col[1] = n->lcol[1];
        L.col[2] = n->lcol[2];
        L.l_src = l->lum[1];
        L.a_qdr = l->atn[3];
        L.a_lnr = l->atn[2];
        L.a_cnt = l->atn[1] + 1.0f;
        L.a_rng = l->atn[0];
        lgt.push_back(L);
    }
}

/* append a surface list with transform-node grouping: surfaces cached under
 * the same node are emitted after one node element whose "last" points at
 * the group's last surface (engine.cpp:1145-1243, 3199-3276) */
int Flat::emit_surface_list(const std::vector<Node*> &order)
{
    int off = (int)elems.size();
    for (size_t i = 0; i < order.size(); i++)
    {
        Node *n = order[i];
        Node *t = (n->trnode != RT_NULL && n->trnode != n) ? n->trnode : RT_NULL;
        if (t != RT_NULL)
        {
            bool grouped = false;
            /* continue an open group of the same node */
            for (int e = (int)elems.size() - 1; e >= off; e--)
            {
                if (elems[e].kind == QR_ELM_TRNODE)
                {
                    if (elems[e].ref == t->index && elems[e].last == (int)elems.size() - 1)
                    {
                        grouped = true;
                        elems[e].last = (int)elems.size();
                    }
                    break;
                }
                if (elems[e].kind == QR_ELM_SURFACE &&
                    srf[elems[e].ref].trnode != t->index)
                {
                    break;
                }
            }
            if (!grouped)
            {
                qr_elem te = {QR_ELM_TRNODE, t->index, (int)elems.size() + 1, 0};
                elems.push_back(te);
            }
        }
        qr_elem se = {QR_ELM_SURFACE, n->index, 0, 0};
        elems.push_back(se);
    }
    return off;
}

void Flat::emit_lists()
{
    elems.clear();
    lelems.clear();

    /* camera list: reverse creation order (the order the reference's
     * hierarchical insert leaves in rt_Scene::clist) */
    std::vector<Node*> rev(surfaces.rbegin(), surfaces.rend());
    cam_off = emit_surface_list(rev);
    cam_num = (int)elems.size() - cam_off;

    /* shadow list (shared by every light): all surfaces; any-hit, so the
     * order does not change results */
    int shd_off = emit_surface_list(rev);
    int shd_num = (int)elems.size() - shd_off;

    /* secondary rays: all surfaces, same order as the camera list */
    int sec_off = cam_off, sec_num = cam_num;

    for (size_t i = 0; i < surfaces.size(); i++)
    {
        Node *n = surfaces[i];
        qr_srf &s = srf[n->index];

        /* custom clippers (engine.cpp:1850-1979) */
        s.clip_off = (int)elems.size();
        for (size_t r = 0; r < n->rel.size(); r++)
        {
            const Node::Rel &rl = n->rel[r];
            if (rl.obj == RT_NULL)
            {
                qr_elem e = {rl.data < 0 ? QR_ELM_ACC_ENTER : QR_ELM_ACC_LEAVE,
                             -1, 0, rl.data};
                elems.push_back(e);
                continue;
            }
            Node *c = rl.obj;
            Node *t = (c->trnode != RT_NULL && c->trnode != c) ? c->trnode : RT_NULL;
            if (t != RT_NULL)
            {
                /* find an existing node element for t in the current accum
                 * segment (or outside any segment) */
                int found = -1, acc = 0;
                for (int e = s.clip_off; e < (int)elems.size(); e++)
                {
                    const qr_elem &x = elems[e];
                    if (x.kind == QR_ELM_ACC_ENTER) acc = 1;
                    if (x.kind == QR_ELM_ACC_LEAVE) acc = 0;
                    if (x.kind == QR_ELM_TRNODE && x.ref == t->index)
                    {
                        /* node in the same segment as the insertion point */
                        int seg = 0;
                        for (int q = e; q < (int)elems.size(); q++)
                        {
                            if (elems[q].kind == QR_ELM_ACC_ENTER ||
                                elems[q].kind == QR_ELM_ACC_LEAVE) seg = 1;
                        }
                        if (seg == 0) found = e;
                    }
                }
                (void)acc;
                if (found >= 0 && elems[found].last == (int)elems.size() - 1)
                {
                    elems[found].last = (int)elems.size();
                }
                else
                {
                    qr_elem te = {QR_ELM_TRNODE, t->index, (int)elems.size() + 1, 0};
                    elems.push_back(te);
                }
            }
            qr_elem ce = {QR_ELM_SURFACE, c->index, 0, rl.data};
            elems.push_back(ce);
        }
        s.clip_num = (int)elems.size() - s.clip_off;

        for (int side = 0; side < 2; side++)
        {
            s.sec_off[side] = sec_off;
            s.sec_num[side] = sec_num;
        }
    }

    /* light lists: every light in creation order, both sides */
    int loff = (int)lelems.size();
    for (size_t l = 0; l < lights.size(); l++)
    {
        qr_lelem le = {(int)l, shd_off, shd_num, 0};
        lelems.push_back(le);
    }
    int lnum = (int)lelems.size() - loff;
    for (size_t i = 0; i < surfaces.size(); i++)
    {
        qr_srf &s = srf[surfaces[i]->index];
        s.lgt_off[0] = s.lgt_off[1] = loff;
        s.lgt_num[0] = s.lgt_num[1] = lnum;
    }
}

/* camera ray basis and ambient (engine.cpp:3078-3101, 3301-3318,
 * 3615-3655) */
void Flat::frame_params(qr_frame_params *fp) const
{
    memset(fp, 0, sizeof(*fp));
    Node *cam = cameras[cam_idx];
    rt_CAMERA *c = (rt_CAMERA *)cam->obj->obj.pobj;
    float pos[3], hor[3], ver[3], nrm[3], dir[3];
    for (int k = 0; k < 3; k++)
    {
        pos[k] = cam->mtx[3][k];
        hor[k] = cam->mtx[0][k];
        ver[k] = cam->mtx[1][k];
        nrm[k] = cam->mtx[2][k];
    }
    float h = -0.5f * 1.0f;
    float v = -0.5f * aspect;
    for (int k = 0; k < 3; k++) dir[k] = nrm[k] * cam->pov;
    for (int k = 0; k < 3; k++) dir[k] += hor[k] * h;
    for (int k = 0; k < 3; k++) dir[k] += ver[k] * v;
    for (int k = 0; k < 3; k++) hor[k] = hor[k] * factor;
    for (int k = 0; k < 3; k++) ver[k] = ver[k] * factor;
    for (int k = 0; k < 3; k++) dir[k] += hor[k] * 0.5f;
    for (int k = 0; k < 3; k++) dir[k] += ver[k] * 0.5f;

    float amb[4];
    for (int k = 0; k < 3; k++) amb[k] = c->col.hdr[k] * c->lum[0];
    amb[3] = c->lum[0];
    /* lights in the registry's order: most recently created first */
    for (int l = (int)lights.size() - 1; l >= 0; l--)
    {
        rt_LIGHT *L = (rt_LIGHT *)lights[l]->obj->obj.pobj;
        for (int k = 0; k < 3; k++) amb[k] += L->col.hdr[k] * L->lum[0];
        amb[3] += L->lum[0];
    }

    for (int k = 0; k < 3; k++)
    {
        fp->org[k] = pos[k];
        fp->dir[k] = dir[k];
        fp->hor[k] = hor[k];
        fp->ver[k] = ver[k];
        fp->amb[k] = amb[k];
    }
    fp->l_amb = amb[3];
    fp->t_min = cam->pov;
    fp->t_max = RT_INF;
    fp->x_res = x_res;
    fp->y_res = y_res;
    fp->x_row = x_res;
    fp->fsaa = fsaa;
    fp->depth = depth;
    fp->ctx_props = -((opts & RT_OPTS_GAMMA) == 0) & QR_PROP_GAMMA;
}

void Flat::desc(qr_scene_desc *d) const
{
    memset(d, 0, sizeof(*d));
    d->nsrf = (int32_t)srf.size();      d->srf = srf.data();
    d->nmat = (int32_t)mat.size();      d->mat = mat.data();
    d->nlgt = (int32_t)lgt.size();      d->lgt = lgt.data();
    d->nelem = (int32_t)elems.size();   d->elems = elems.data();
    d->nlelem = (int32_t)lelems.size(); d->lelems = lelems.data();
    d->ntex = (int32_t)texels.size();   d->texels = texels.data();
    d->cam_off = cam_off;
    d->cam_num = cam_num;
}

} /* namespace qr */

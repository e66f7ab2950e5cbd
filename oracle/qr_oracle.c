/*
 * qr_oracle.c: CPU restatement of the QuadRay Whitted render path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GB300 CUDA tracer and the
 * timed CPU baseline.  Nothing in the product links this file.
 *
 * It restates, one ray at a time in plain fp32 C, the SIMD tracer of the
 * reference engine (VectorChief/QuadRay-engine core/tracer/tracer.cpp,
 * rt_simd_*::render0, lines 2086-7622, built with RT_FEAT_PT=0,
 * RT_FEAT_BUFFERS=0) on the flattened scene of include/qr_gpu.h.  Every
 * arithmetic step follows the reference's instruction order (cited per
 * function) so results are bit-identical; it must be compiled with
 * -ffp-contract=off and without fast-math.
 *
 * The reference processes SIMD groups with lane masks and shades every
 * surface that is the nearest so far ("overdraw", depth test against T_BUF).
 * Per lane that is the same as shading the nearest hit, where hits are
 * ordered by the walk order and a later hit wins only if strictly nearer.
 * Three mask-level shortcuts of the reference depend on neighbouring lanes;
 * this restatement resolves them per lane as noted in place.  They only
 * change results when two roots of one quadric are exactly equal, or in the
 * last bit of a metal surface's specular blend.
 *
 * Parity is pinned against frames rendered by the reference itself
 * (oracle/_ref, tests/golden).
 */
#include <math.h>
#include <string.h>
#include <stdint.h>
#include <float.h>

#include "qr_gpu.h"
#include "qr_oracle.h"

/* the restatement's functions are plain static C; the FP64 GPU oracle
 * (qr_oracle_gpu.cu) compiles this file for the device as well */
#ifdef __CUDACC__
#define ORC static __host__ __device__
#else
#define ORC static
#endif

/* precision of the restatement: float (the checker of the GPU tracer and
 * the CPU baseline) or, built with QR_ORACLE_FP64, double (the FP64 oracle
 * of the path tracer); both builds come from this one source.  The scene
 * records stay float either way. */
#ifdef QR_ORACLE_FP64
typedef double real;
#define R_SQRT  sqrt
#define R_FABS  fabs
#define R_FLOOR floor
#define R_LRINT lrint
#define R_FMA   fma
#else
typedef float real;
#define R_SQRT  sqrtf
#define R_FABS  fabsf
#define R_FLOOR floorf
#define R_LRINT lrintf
#define R_FMA   fmaf
#endif

#define TAG_ARRAY   (-1)
#define FLAG_SIDE   1
#define FLAG_PASS   2           /* 0 pass back (reflect), 2 pass thru */
#define FLAG_SHAD   4
#define SIDE_OUTER  0
#define SIDE_INNER  1

#define D_EPS       0.00000000001f  /* RT_DEPS_THRESHOLD, object.h:41 */
#define T_EPS       0.0000001f      /* RT_TEPS_THRESHOLD, object.h:42 */

typedef struct scene_s
{
    const qr_srf   *srf;
    const qr_mat   *mat;
    const qr_light *lgt;
    const qr_elem  *elems;
    const qr_lelem *lelems;
    const uint32_t *texels;
    real amb[3];
    int   ctx_props;
    uint64_t nrays;         /* traced segments (stats) */
} scene_t;

/* a ray context (rt_SIMD_CONTEXT fields used per lane) */
typedef struct ray_s
{
    real org[3];
    real ray[3];
    real t_min;
    real t_max;
    int   from;             /* originating surface (ctx PARAM OBJ), -1 none */
    int   flags;            /* side | pass | shadow bits of ctx PARAM FLG */
    real phit[3];          /* originating surface's local hit (parent NRM_IJK) */
    int   depth;            /* remaining secondary-ray depth (inf_DEPTH) */
} ray_t;

/* nearest hit found by a list walk */
typedef struct hit_s
{
    int   srf;
    int   side;
    real t;
    real hit[3];           /* world hit point (ctx HIT) */
    real loc[3];           /* local hit in the solver's frame (ctx NEW) */
    real amask;            /* sign of the quadric's a (for the record) */
} hit_t;

/* sign-bit operations of the reference's SIMD code (xor with the sign
 * mask), written as negation so they hold in either precision */
ORC inline real fxor(real a, uint32_t m) { return (m & 0x80000000u) ? -a : a; }
ORC inline uint32_t sgnbit(real a) { return signbit(a) ? 0x80000000u : 0u; }

/* reciprocal square root and reciprocal in the reference's full-precision
 * compat mode (core/config/rtconf.h: rsq = 1/sqrt, rcp = 1/x) */
ORC inline real rsq(real x) { return 1.0f / R_SQRT(x); }

/* M * v with the transform-node coefficients, diagonal terms first
 * (tracer.cpp:2537-2568); fast path keeps only the diagonal (2546) */
ORC void xform(const qr_srf *t, const real v[3], real o[3])
{
    real x = t->tci[0] * v[0];
    real y = t->tcj[1] * v[1];
    real z = t->tck[2] * v[2];
    if (t->amap[3] != 1)
    {
        x = x + t->tci[1] * v[1];
        x = x + t->tci[2] * v[2];
        y = y + t->tcj[0] * v[0];
        y = y + t->tcj[2] * v[2];
        z = z + t->tck[0] * v[0];
        z = z + t->tck[1] * v[1];
    }
    o[0] = x; o[1] = y; o[2] = z;
}

/* ---- clipping subroutine CC_clp (tracer.cpp:2686-3249) ------------------ */

/*
 * Boundary tracking (qr_oracle_boundary, the hit-ID exclusion mask): while
 * a walk carries a tracker, every decision taken for a root that can still
 * matter (its depth test passes or is marginal) records the root's distance
 * when the quantity it compares lies within QR_MARGIN (1e-5) of the
 * decision's boundary, relative to the size of the terms compared: the
 * quadric's discriminant (tangent rays), the depth test between surfaces,
 * the near plane, the axis clippers and the custom clippers.  A pixel whose
 * primary ray recorded such a root no farther than its hit is ill
 * conditioned: float rounding may give it either surface.  Walks without a
 * tracker (every render) skip all of this.
 */
#define QR_MARGIN       1e-5
#define QR_MARGIN_EV    8

typedef struct margin_s
{
    int  nev;                   /* marginal decisions seen */
    real t[QR_MARGIN_EV];       /* their roots' distances */
} margin_t;

ORC void margin_note(margin_t *mg, real t, real num, real den)
{
    if (mg == NULL) return;
    if (!(R_FABS(num) <= (real)QR_MARGIN * den)) return;
    /* beyond the slots, the last one keeps the nearest distance */
    if (mg->nev < QR_MARGIN_EV) mg->t[mg->nev] = t;
    else if (t < mg->t[QR_MARGIN_EV - 1]) mg->t[QR_MARGIN_EV - 1] = t;
    mg->nev++;
}

ORC real rmax3(real a, real b, real c)
{
    a = R_FABS(a);
    b = R_FABS(b);
    c = R_FABS(c);
    if (b > a) a = b;
    return c > a ? c : a;
}

/*
 * Returns 1 if root t of surface s survives depth test, near clip, axis
 * clippers and custom clippers; fills the world hit and the local hit.
 *   ldff   the surface's local diff (ctx DFF in the solver's frame)
 *   lray   the surface's local ray
 *   tbuf   current depth buffer
 *   dmask  this lane's near-zero-determinant flag, amask sign of a
 */
ORC int clip_root(const scene_t *sc, const ray_t *r, int si, real t,
                     real tbuf, const real ldff[3], const real lray[3],
                     int side, int dmask, uint32_t amask, real hit[3],
                     real loc[3], margin_t *mg)
{
    const qr_srf *s = &sc->srf[si];
    int valid = 1;
    int k;

    if (!(tbuf > t)) valid = 0;             /* depth test */
    if (!(r->t_min < t)) valid = 0;         /* near plane */
    if (mg != NULL)
    {
        const int dm = R_FABS(tbuf - t) <= (real)QR_MARGIN * rmax3(t, tbuf, 0.0f);
        const int nm = R_FABS(t - r->t_min) <= (real)QR_MARGIN * rmax3(t, r->t_min, 0.0f);
        if (dm) margin_note(mg, t, 0.0f, 1.0f);
        if (nm) margin_note(mg, t, 0.0f, 1.0f);
        /* the decisions below matter only for a root the depth test and the
         * near plane let through, or nearly so */
        if (!valid && !dm && !nm) mg = NULL;
    }

    for (k = 0; k < 3; k++)
    {
        hit[k] = r->ray[k] * t + r->org[k];
    }
    if (s->amap[3] != 0)
    {
        for (k = 0; k < 3; k++)
        {
            loc[k] = lray[k] * t + ldff[k];
        }
    }
    else
    {
        for (k = 0; k < 3; k++)
        {
            loc[k] = hit[k] - s->pos[k];
        }
    }

    /* conic singularity adjustment near the apex (2795-2945) */
    if (s->conic != 0 && dmask)
    {
        int mi = s->amap[0], mj = s->amap[1], mk = s->amap[2];
        real r2 = loc[mi] * loc[mi];
        if (s->conic != 2)
        {
            r2 = r2 + loc[mj] * loc[mj];
        }
        r2 = r2 + loc[mk] * loc[mk];
        if (r2 < T_EPS)
        {
            real li, lj = 0.0f, lk, lr, sk;
            li = fxor(1.0f, sgnbit(ldff[mi]));
            sk = s->sci[mi];
            lr = 1.0f;
            if (s->conic != 2)
            {
                lj = fxor(1.0f, sgnbit(ldff[mj]));
                sk = sk + s->sci[mj];
                lr = lr + 1.0f;
            }
            sk = sk / s->sci[mk];
            sk = fxor(sk, 0x80000000u);
            lk = R_SQRT(sk);
            {
                real inv = rsq(sk + lr);
                inv = inv * T_EPS;
                li = li * inv;
                lj = lj * inv;
                lk = lk * inv;
            }
            {
                uint32_t tside = side ? 0x80000000u : 0u;
                lk = fxor(lk, sgnbit(ldff[mk]));
                lk = fxor(lk, amask & ~tside);
                li = fxor(li, tside & ~amask);
                lj = fxor(lj, tside & ~amask);
            }
            loc[mi] = li;
            if (s->conic != 2)
            {
                loc[mj] = lj;
            }
            loc[mk] = lk;
        }
    }

    /* axis clippers (2963-3014) */
    for (k = 0; k < 3; k++)
    {
        if ((s->mint >> k) & 1)
        {
            if (!(s->bmin[k] <= loc[k])) valid = 0;
            margin_note(mg, t, loc[k] - s->bmin[k], rmax3(loc[k], s->bmin[k], 1.0f));
        }
        if ((s->maxt >> k) & 1)
        {
            if (!(s->bmax[k] >= loc[k])) valid = 0;
            margin_note(mg, t, loc[k] - s->bmax[k], rmax3(loc[k], s->bmax[k], 1.0f));
        }
    }

    /* custom clippers with boolean accumulator segments (3020-3240) */
    if (s->clip_num > 0)
    {
        int mask = valid, saved = 0, cache_last = -1;
        int e;
        real nx[3] = {0, 0, 0};    /* ctx NRM_X/Y/Z used as scratch */
        for (e = 0; e < s->clip_num; e++)
        {
            int ei = s->clip_off + e;
            const qr_elem *el = &sc->elems[ei];
            const qr_srf *c;
            real p[3], v;
            if (el->kind == QR_ELM_ACC_ENTER)
            {
                saved = mask;
                mask = 1;               /* srf_C_DEF = all lanes */
                continue;
            }
            if (el->kind == QR_ELM_ACC_LEAVE)
            {
                mask = !mask && saved;
                continue;
            }
            c = &sc->srf[el->ref];
            if (el->kind == QR_ELM_TRNODE)
            {
                if (s->trnode == el->ref)
                {
                    /* clipped surface shares the node: local hit back to
                     * node space (3097-3126) */
                    for (k = 0; k < 3; k++) nx[k] = loc[k] + s->pos[k];
                }
                else
                {
                    for (k = 0; k < 3; k++) p[k] = hit[k] - c->pos[k];
                    if (c->amap[3] != 0) xform(c, p, nx);
                    else { nx[0] = p[0]; nx[1] = p[1]; nx[2] = p[2]; }
                }
                cache_last = el->last;
                continue;
            }
            /* surface clipper: its local point (3057-3214) */
            if (cache_last >= 0)
            {
                for (k = 0; k < 3; k++) p[k] = nx[k] - c->pos[k];
                if (ei == cache_last) cache_last = -1;
            }
            else
            {
                real d[3];
                for (k = 0; k < 3; k++) d[k] = hit[k] - c->pos[k];
                if (c->amap[3] != 0) xform(c, d, p);
                else { p[0] = d[0]; p[1] = d[1]; p[2] = d[2]; }
            }
            /* clipper's implicit function (PL_clp 5696, QD_clp 6292,
             * TP_clp 6466) */
            if (c->clpk == 1)
            {
                v = fxor(p[c->amap[2]], c->asgn[2] ? 0x80000000u : 0u);
                margin_note(mg, t, v, rmax3(p[0], p[1], p[2]) + 1.0f);
            }
            else if (c->clpk == 2)
            {
                real d2[3];
                for (k = 0; k < 3; k++)
                {
                    real d1 = (c->scj[k] + c->scj[k]) * p[k];
                    d2[k] = p[k] * p[k] * c->sci[k] - d1;
                }
                v = ((d2[0] - c->sci[3]) + d2[1]) + d2[2];
                margin_note(mg, t, v, R_FABS(d2[0]) + R_FABS(d2[1]) + R_FABS(d2[2]) +
                                      R_FABS(c->sci[3]));
            }
            else
            {
                real d2[3];
                for (k = 0; k < 3; k++) d2[k] = p[k] * p[k] * c->sci[k];
                v = ((d2[0] - c->sci[3]) + d2[1]) + d2[2];
                margin_note(mg, t, v, R_FABS(d2[0]) + R_FABS(d2[1]) + R_FABS(d2[2]) +
                                      R_FABS(c->sci[3]));
            }
            /* APPLY_CLIP (515-523): minus inner keeps v >= 0,
             * minus outer keeps v <= 0 */
            if (el->rel < 0) mask = mask && (v >= 0.0f);
            else             mask = mask && (v <= 0.0f);
        }
        valid = mask;
    }
    return valid;
}

/* ---- list walk OO_cyc (2413-2680) with the plane (5522-5706), quadric
 *      (5714-6335) and two-plane (6341-6497) solvers ---------------------- */

typedef struct walk_s
{
    int     shadow;         /* 1: any-hit test for shadow rays */
    int     occluded;
    real   tbuf;
    hit_t   best;
    margin_t *mg;           /* boundary tracker (NULL: none) */
} walk_t;

/* record a root that passed the clipper; shadow rays test occlusion */
ORC void accept_root(const scene_t *sc, walk_t *w, int si, int side,
                        real t, const real hit[3], const real loc[3],
                        uint32_t amask)
{
    if (w->shadow)
    {
        /* CHECK_SHAD (576-616): light sources and transparent
         * non-refractive surfaces do not occlude */
        int props = sc->srf[si].props[side];
        if (props & QR_PROP_LIGHT) return;
        if ((props & QR_PROP_TRANSP) && !(props & QR_PROP_REFRACT)) return;
        w->occluded = 1;
        return;
    }
    w->tbuf = t;
    w->best.srf = si;
    w->best.side = side;
    w->best.t = t;
    memcpy(w->best.hit, hit, sizeof(w->best.hit));
    memcpy(w->best.loc, loc, sizeof(w->best.loc));
    w->best.amask = amask ? (real)-0.0f : (real)0.0f;
}

/* CHECK_SIDE (558-567): a ray leaving surface s cannot hit it again from
 * the side it could not reach */
ORC int side_blocked(const ray_t *r, int si, int side)
{
    int f;
    if (r->from != si) return 0;
    f = r->flags & (FLAG_SIDE | FLAG_PASS);
    return f == 1 - side || f == 2 + side;
}

ORC void root_pair(const scene_t *sc, const ray_t *r, walk_t *w, int si,
                      const real ldff[3], const real lray[3],
                      real a, real b, real c, real d)
{
    real nb, sd, q, t1n, t1d, t2n, t2d, t1, t2;
    int dmask, m_pos, m_neg, t1m, t2m, first, k;
    uint32_t amask;
    real hit[3], loc[3];

    /* a tangent ray: the double root -b / a */
    if (w->mg != NULL && a != 0.0f)
        margin_note(w->mg, -b / a, d, b * b + R_FABS(c * a));
    /* QD_rts (5785-5799) */
    if (!(0.0f <= d)) return;               /* xmask */
    nb = fxor(b, 0x80000000u);
    dmask = d < D_EPS;

    /* b-mixed roots (5854-5883) */
    sd = R_SQRT(d);
    sd = fxor(sd, sgnbit(nb));
    q = nb + sd;
    m_pos = 0.0f <= sd;
    m_neg = 0.0f > sd;
    t2n = m_neg ? c : m_pos ? q : 0.0f;
    t1n = m_neg ? q : m_pos ? c : 0.0f;
    t2d = m_neg ? q : m_pos ? a : 0.0f;
    t1d = m_neg ? a : m_pos ? q : 0.0f;
    amask = sgnbit(a);

    if (dmask)
    {
        /* near-zero determinant: zero numerators give t = 0 and the two
         * roots are equated and split by T_EPS (5908-5959) */
        real tdff, teps;
        int fmask;
        if (t1n == 0.0f) t1d = 1.0f;
        if (t2n == 0.0f) t2d = 1.0f;
        t1 = t1n / t1d;
        t2 = t2n / t2d;
        t1m = t1d != 0.0f;
        t2m = t2d != 0.0f;
        tdff = t1 - t2;
        tdff = fxor(tdff, amask);
        fmask = 0.0f <= tdff;
        tdff = fmask ? tdff : 0.0f;
        teps = fmask ? T_EPS : 0.0f;
        teps = teps * t1;
        teps = R_FABS(teps);
        tdff = tdff * -0.5f;
        tdff = tdff - teps;
        tdff = fxor(tdff, amask);
        if (!(t1m && t2m)) tdff = 0.0f;
        t1 = t1 + tdff;
        t2 = t2 - tdff;
    }
    else
    {
        t1 = t1n / t1d;
        t2 = t2n / t2d;
        t1m = t1d != 0.0f;
        t2m = t2d != 0.0f;
    }

    /* root order (5982-5994): outer root first unless a < 0; the reference
     * uses the outer-first order for a whole SIMD group with mixed signs
     * of a, which only matters for exactly equal roots */
    first = (0.0f > a) ? SIDE_INNER : SIDE_OUTER;
    for (k = 0; k < 2; k++)
    {
        int side = k == 0 ? first : 1 - first;
        real t = side == SIDE_OUTER ? t1 : t2;
        int tm = side == SIDE_OUTER ? t1m : t2m;
        if (side_blocked(r, si, side)) continue;
        if (!tm) continue;
        if (clip_root(sc, r, si, t, w->tbuf, ldff, lray, side, dmask, amask,
                      hit, loc, w->mg))
        {
            accept_root(sc, w, si, side, t, hit, loc, amask);
            if (w->shadow && w->occluded) return;
        }
    }
}

ORC void walk(const scene_t *sc, const ray_t *r, int off, int num, walk_t *w)
{
    real cdff[3] = {0, 0, 0}, cray[3] = {0, 0, 0};
    int cache_last = -1;
    int e, k;

    for (e = 0; e < num; e++)
    {
        int ei = off + e;
        const qr_elem *el = &sc->elems[ei];
        const qr_srf *s = &sc->srf[el->ref];
        real ldff[3], lray[3];

        if (el->kind == QR_ELM_TRNODE)
        {
            /* transform node: cache its diff and ray (2466-2510,
             * 2574-2589, 2599-2643) */
            real d[3];
            for (k = 0; k < 3; k++) d[k] = r->org[k] - s->pos[k];
            if (s->amap[3] == 0) continue;
            xform(s, d, cdff);
            xform(s, r->ray, cray);
            cache_last = el->last;
            continue;
        }

        if (cache_last >= 0)
        {
            if (r->from == el->ref)
            {
                memcpy(ldff, r->phit, sizeof(ldff));
            }
            else
            {
                for (k = 0; k < 3; k++) ldff[k] = cdff[k] - s->pos[k];
            }
            memcpy(lray, cray, sizeof(lray));
            if (ei == cache_last) cache_last = -1;
        }
        else
        {
            if (r->from == el->ref)
            {
                memcpy(ldff, r->phit, sizeof(ldff));
                if (s->amap[3] != 0) xform(s, r->ray, lray);
                else memcpy(lray, r->ray, sizeof(lray));
            }
            else
            {
                real d[3];
                for (k = 0; k < 3; k++) d[k] = r->org[k] - s->pos[k];
                if (s->amap[3] != 0)
                {
                    xform(s, d, ldff);
                    xform(s, r->ray, lray);
                }
                else
                {
                    memcpy(ldff, d, sizeof(ldff));
                    memcpy(lray, r->ray, sizeof(lray));
                }
            }
        }

        if (s->solver == 1)
        {
            /* plane (5545-5634) */
            int mk = s->amap[2];
            uint32_t sg = s->asgn[2] ? 0x80000000u : 0u;
            real dk, rk, t;
            real hit[3], loc[3];
            if (r->from == el->ref) continue;
            dk = fxor(ldff[mk], sg);
            rk = fxor(lray[mk], sg);
            dk = fxor(dk, 0x80000000u);
            if (!(rk != 0.0f)) continue;
            t = dk / rk;
            if (!clip_root(sc, r, el->ref, t, w->tbuf, ldff, lray, 0, 0, 0,
                           hit, loc, w->mg))
            {
                continue;
            }
            accept_root(sc, w, el->ref, rk < 0.0f ? SIDE_OUTER : SIDE_INNER,
                        t, hit, loc, 0);
        }
        else if (s->solver == 2)
        {
            /* quadric coefficients (5722-5783) */
            real a, b, c, d, ax, bx, cx, sri, sdi;
            a = b = c = 0.0f;
            for (k = 0; k < 3; k++)
            {
                sri = s->sci[k] * lray[k];
                sdi = s->sci[k] * ldff[k];
                sdi = sdi - s->scj[k];
                ax = lray[k] * sri;
                bx = lray[k] * sdi;
                sdi = sdi - s->scj[k];
                cx = ldff[k] * sdi;
                if (k == 0) { a = ax; b = bx; c = cx; }
                else { a = a + ax; b = b + bx; c = c + cx; }
            }
            c = c - s->sci[3];
            d = b * b - c * a;
            root_pair(sc, r, w, el->ref, ldff, lray, a, b, c, d);
        }
        else
        {
            /* two-plane (6349-6402) */
            int mi = s->amap[0], mk = s->amap[2];
            real ri = lray[mi], di = ldff[mi], rk2 = lray[mk], dk2 = ldff[mk];
            real si_ = s->sci[mi], sk = s->sci[mk];
            real dd, bb, cc, aa;
            dd = di * rk2 - dk2 * ri;
            dd = dd * dd;
            dd = dd * si_;
            dd = dd * sk;
            dd = R_FABS(dd);
            bb = si_ * di * ri + sk * dk2 * rk2;
            cc = di * di * si_ + dk2 * dk2 * sk;
            aa = ri * ri * si_ + rk2 * rk2 * sk;
            root_pair(sc, r, w, el->ref, ldff, lray, aa, bb, cc, dd);
        }
        if (w->shadow && w->occluded) return;
    }
}

/* ---- shading: normal (PL 5669-5687, QD 6237-6283, TP 6415-6457), normal
 *      transform (3273-3352), material (3356-3416), lights (3929-4436),
 *      transparency (4438-4936), reflection (4938-5359) -------------------- */

ORC void trace(scene_t *sc, const ray_t *r, int off, int num, real col[3]);

/* normal (side-oriented, world frame) and texel colour of a hit */
ORC void hit_surface(const scene_t *sc, const hit_t *h, real nrm[3], real tex[3])
{
    const qr_srf *s = &sc->srf[h->srf];
    int side = h->side;
    int props = s->props[side];
    const qr_mat *m = &sc->mat[s->mat[side]];
    uint32_t tside = side ? 0x80000000u : 0u;
    real tu = 0.0f, tv = 0.0f;
    int k;

    /* normal in the solver's frame */
    if (s->nrmk == 1)
    {
        real n[3] = {0.0f, 0.0f, 0.0f};
        int mk = s->amap[2];
        n[s->amap[0]] = 0.0f;
        n[s->amap[1]] = 0.0f;
        n[mk] = fxor(fxor(1.0f, tside), s->asgn[2] ? 0x80000000u : 0u);
        memcpy(nrm, n, 3 * sizeof(real));
        if (props & QR_PROP_TEXTURE)
        {
            tu = fxor(h->loc[s->amap[0]], s->asgn[0] ? 0x80000000u : 0u);
            tv = fxor(h->loc[s->amap[1]], s->asgn[1] ? 0x80000000u : 0u);
        }
    }
    else
    {
        real x = h->loc[0] * s->sci[0];
        real y = h->loc[1] * s->sci[1];
        real z = h->loc[2] * s->sci[2];
        real l2, inv;
        if (s->nrmk == 2)
        {
            x = x - s->scj[0];
            y = y - s->scj[1];
            z = z - s->scj[2];
        }
        l2 = x * x + y * y;
        l2 = l2 + z * z;
        inv = rsq(l2);
        inv = fxor(inv, tside);
        nrm[0] = x * inv;
        nrm[1] = y * inv;
        nrm[2] = z * inv;
    }

    if (s->amap[3] != 0)
    {
        /* node's transposed inverse (3273-3352) */
        const qr_srf *t = &sc->srf[s->trnode >= 0 ? s->trnode : h->srf];
        real n1 = nrm[0], n2 = nrm[1], n3 = nrm[2];
        real x = t->tci[0] * n1;
        real y = t->tcj[1] * n2;
        real z = t->tck[2] * n3;
        int renorm = 1;
        if (t->amap[3] != 1)
        {
            x = x + t->tcj[0] * n2;
            x = x + t->tck[0] * n3;
            y = y + t->tci[1] * n1;
            y = y + t->tck[1] * n3;
            z = z + t->tci[2] * n1;
            z = z + t->tcj[2] * n2;
            if (t->amap[3] == 2) renorm = 0;
        }
        if (renorm)
        {
            real l2 = x * x + y * y;
            real inv;
            l2 = l2 + z * z;
            inv = rsq(l2);
            x = x * inv;
            y = y * inv;
            z = z * inv;
        }
        nrm[0] = x; nrm[1] = y; nrm[2] = z;
    }

    /* texel (3380-3416, PAINT_COLX 970-979) */
    {
        uint32_t texel;
        int32_t idx = 0;
        if (props & QR_PROP_TEXTURE)
        {
            real uv[2] = {tu, tv};
            real tx = uv[m->tmap[0]], ty = uv[m->tmap[1]];
            tx = tx - m->xoffs;
            ty = ty - m->yoffs;
            tx = tx * m->xscal;
            ty = ty * m->yscal;
            idx = ((int32_t)R_FLOOR(tx) & m->xmask) +
                  (((int32_t)R_FLOOR(ty) & m->ymask) << m->yshft);
        }
        texel = sc->texels[m->tex_off + idx];
        tex[0] = (real)(int32_t)((texel >> 16) & 0xFF) / 255.0f;
        tex[1] = (real)(int32_t)((texel >> 8) & 0xFF) / 255.0f;
        tex[2] = (real)(int32_t)(texel & 0xFF) / 255.0f;
        if (props & QR_PROP_GAMMA)
        {
            for (k = 0; k < 3; k++) tex[k] = tex[k] * tex[k];
        }
    }

}

ORC void shade(scene_t *sc, const ray_t *r, const hit_t *h, real col[3])
{
    const qr_srf *s = &sc->srf[h->srf];
    int side = h->side;
    int props = s->props[side];
    const qr_mat *m = &sc->mat[s->mat[side]];
    real nrm[3], tex[3], c[3];
    int k;

    hit_surface(sc, h, nrm, tex);

    /* ambient (3931-3996) */
    for (k = 0; k < 3; k++) c[k] = tex[k];
    if (!(props & QR_PROP_LIGHT))
    {
        real f;
        for (k = 0; k < 3; k++) c[k] = c[k] * sc->amb[k];
        f = 1.0f - m->c_trn;
        f = f - m->c_rfl;
        f = (0.0f <= f) ? f : 0.0f;
        for (k = 0; k < 3; k++) c[k] = c[k] * f;

        /* lights (4002-4391) */
        {
            int li;
            int loff = s->lgt_off[side], lnum = s->lgt_num[side];
            for (li = 0; li < lnum; li++)
            {
                const qr_lelem *le = &sc->lelems[loff + li];
                const qr_light *L = &sc->lgt[le->light];
                real lv[3], dot, r2, diff, sdot, lc[3];
                int spec_on = 0;
                real spec = 0.0f;
                for (k = 0; k < 3; k++) lv[k] = L->pos[k] - h->hit[k];
                dot = lv[0] * nrm[0] + lv[1] * nrm[1];
                dot = dot + lv[2] * nrm[2];
                if (!(0.0f < dot)) continue;

                /* shadow ray: origin = hit, direction = L, t in (0, 1) */
                {
                    ray_t sr;
                    walk_t sw;
                    memcpy(sr.org, h->hit, sizeof(sr.org));
                    memcpy(sr.ray, lv, sizeof(sr.ray));
                    sr.t_min = 0.0f;
                    sr.t_max = L->t_max;
                    sr.from = h->srf;
                    sr.flags = side | FLAG_SHAD;
                    memcpy(sr.phit, h->loc, sizeof(sr.phit));
                    sr.depth = r->depth - 1;
                    memset(&sw, 0, sizeof(sw));
                    sw.shadow = 1;
                    sw.tbuf = L->t_max;
                    sw.best.srf = -1;
                    sc->nrays++;
                    walk(sc, &sr, le->shd_off, le->shd_num, &sw);
                    if (sw.occluded) continue;
                }

                r2 = lv[0] * lv[0] + lv[1] * lv[1];
                r2 = r2 + lv[2] * lv[2];

                if (props & QR_PROP_DIFFUSE)
                {
                    real inv_r, r1, att, inv_a;
                    inv_r = rsq(r2);
                    r1 = inv_r * r2;
                    att = r2 * L->a_qdr;
                    r1 = r1 * L->a_lnr;
                    att = att + L->a_cnt;
                    att = att + r1;
                    inv_a = rsq(att);
                    sdot = dot;
                    diff = dot * inv_a;
                    diff = diff * inv_r;
                    diff = diff * m->l_dff;
                }
                else
                {
                    sdot = dot;
                    diff = 0.0f;
                }

                if (props & QR_PROP_SPECULAR)
                {
                    real rx, ry, rz, sv, ray2;
                    real pn;
                    pn = sdot * nrm[0];
                    rx = lv[0] - pn; rx = rx - pn;
                    pn = sdot * nrm[1];
                    ry = lv[1] - pn; ry = ry - pn;
                    pn = sdot * nrm[2];
                    rz = lv[2] - pn; rz = rz - pn;
                    rx = rx * r->ray[0];
                    ry = ry * r->ray[1];
                    rz = rz * r->ray[2];
                    ray2 = r->ray[2] * r->ray[2];
                    ray2 = ray2 + r->ray[0] * r->ray[0];
                    ray2 = ray2 + r->ray[1] * r->ray[1];
                    sv = rx + ry;
                    sv = sv + rz;
                    if (0.0f < sv)
                    {
                        /* power in 28.4 fixed point (4225-4285) */
                        real p1 = 1.0f, p2, p3;
                        uint32_t lp = (uint32_t)m->l_pow;
                        uint32_t fr = lp & 0xF, in = lp >> 4;
                        sv = sv * rsq(ray2);
                        sv = sv * rsq(r2);
                        p2 = sv;
                        if (fr != 0)
                        {
                            real s4 = sv;
                            do
                            {
                                s4 = R_SQRT(s4);
                                if (fr & 0x8) p1 = p1 * s4;
                                fr = (fr << 1) & 0xF;
                            } while (fr != 0);
                        }
                        if (in != 0)
                        {
                            p3 = p1;
                            p1 = 1.0f;
                            do
                            {
                                if (in & 1) p1 = p1 * p2;
                                p2 = p2 * p2;
                                in >>= 1;
                            } while (in != 0);
                            p1 = p1 * p3;
                        }
                        spec = p1 * m->l_spc;
                        spec_on = 1;
                    }
                }

                if (spec_on && !(props & QR_PROP_METAL))
                {
                    /* plain: the highlight takes the light's colour only
                     * (LT_mtl, 4323-4355) */
                    for (k = 0; k < 3; k++)
                    {
                        real t1 = tex[k] * diff;
                        t1 = t1 * L->col[k];
                        lc[k] = t1 + L->col[k] * spec;
                    }
                }
                else
                {
                    /* metal: the highlight is tinted by the surface colour
                     * (4287-4317); also the no-highlight case.  The
                     * reference picks the plain form for a lane without a
                     * highlight when another lane of its SIMD group has one,
                     * which differs only in the last bit */
                    if (spec_on) diff = diff + spec;
                    for (k = 0; k < 3; k++)
                    {
                        lc[k] = tex[k] * L->col[k];
                        lc[k] = lc[k] * diff;
                    }
                }
                for (k = 0; k < 3; k++) c[k] = lc[k] + c[k];
            }
        }
    }

    /* transparency (4442-4936) */
    {
        real c_trn = m->c_trn, c_rfl = m->c_rfl;
        int m_trn = 1;
        real nw[3];
        int do_trn = 0;

        if (!(props & QR_PROP_OPAQUE))
        {
            real dn[3], l2, inv, cosi, nci, kk, sq = 0.0f;
            int fres = (props & QR_PROP_FRESNEL) != 0;
            int refr = (props & QR_PROP_REFRACT) != 0;
            if (refr || fres)
            {
                l2 = r->ray[0] * r->ray[0];
                l2 = l2 + r->ray[1] * r->ray[1];
                l2 = l2 + r->ray[2] * r->ray[2];
                inv = rsq(l2);
                for (k = 0; k < 3; k++) dn[k] = r->ray[k] * inv;
                cosi = dn[0] * nrm[0];
                cosi = cosi + dn[1] * nrm[1];
                cosi = cosi + dn[2] * nrm[2];
                nci = cosi * m->c_rfr;
                kk = nci * nci;
                kk = kk + 1.0f;
                kk = kk - m->rfr_2;
                if (fres)
                {
                    m_trn = 0.0f <= kk;
                }
                if (fres && !m_trn)
                {
                    /* total inner reflection (4537-4552) */
                    c_trn = 0.0f;
                    c_rfl = m->c_rfl + m->c_trn;
                }
                else
                {
                    sq = R_SQRT(kk);
                    nci = nci + sq;
                    if (refr)
                    {
                        for (k = 0; k < 3; k++)
                        {
                            real a1 = nrm[k] * nci;
                            real a2 = dn[k] * m->c_rfr;
                            nw[k] = a2 - a1;
                        }
                    }
                    else
                    {
                        memcpy(nw, r->ray, sizeof(nw));
                    }
                    if (fres)
                    {
                        real x1 = cosi, x2, x3, f0, f1, fr;
                        real sqn;
                        x2 = x1 * m->c_rfr;
                        x2 = x2 - sq;
                        sqn = sq * m->c_rfr;
                        x3 = x1;
                        x1 = x1 + sqn;
                        x3 = x3 - sqn;
                        f0 = nci / x2;
                        f1 = x1 / x3;
                        f0 = f0 * f0;
                        f1 = f1 * f1;
                        fr = f0 + f1;
                        fr = R_FABS(fr * -0.5f);
                        fr = fr * m->c_trn;
                        c_trn = m->c_trn - fr;
                        c_rfl = m->c_rfl + fr;
                    }
                    do_trn = 1;
                }
            }
            else
            {
                memcpy(nw, r->ray, sizeof(nw));
                do_trn = 1;
            }

            if (do_trn && m_trn)
            {
                real tc[3] = {0.0f, 0.0f, 0.0f};
                if (r->depth != 0)
                {
                    ray_t cr;
                    memcpy(cr.org, h->hit, sizeof(cr.org));
                    memcpy(cr.ray, nw, sizeof(cr.ray));
                    cr.t_min = 0.0f;
                    cr.t_max = FLT_MAX;
                    cr.from = h->srf;
                    cr.flags = side | FLAG_PASS;
                    memcpy(cr.phit, h->loc, sizeof(cr.phit));
                    cr.depth = r->depth - 1;
                    trace(sc, &cr, s->sec_off[1 - side], s->sec_num[1 - side], tc);
                    for (k = 0; k < 3; k++) tc[k] = tc[k] * c_trn;
                }
                for (k = 0; k < 3; k++) c[k] = tc[k] + c[k];
            }
        }

        /* reflection (4942-5359) */
        {
            int refl = (props & QR_PROP_REFLECT) != 0;
            int do_rfl = refl;
            if (!refl && !(props & QR_PROP_OPAQUE) && (props & QR_PROP_FRESNEL))
            {
                do_rfl = 1;
            }
            if (do_rfl)
            {
                real dn[3], l2, inv, cosi, rw[3];
                l2 = r->ray[0] * r->ray[0];
                l2 = l2 + r->ray[1] * r->ray[1];
                l2 = l2 + r->ray[2] * r->ray[2];
                inv = rsq(l2);
                for (k = 0; k < 3; k++) dn[k] = r->ray[k] * inv;
                cosi = dn[0] * nrm[0];
                cosi = cosi + dn[1] * nrm[1];
                cosi = cosi + dn[2] * nrm[2];
                for (k = 0; k < 3; k++)
                {
                    real p = nrm[k] * cosi;
                    rw[k] = dn[k] - p;
                    rw[k] = rw[k] - p;
                }
                if ((props & QR_PROP_FRESNEL) && (props & QR_PROP_OPAQUE))
                {
                    real fr;
                    if (props & QR_PROP_METAL)
                    {
                        /* fast complex-IOR Fresnel (5067-5089) */
                        real r6 = m->c_rcp, x4, x0, x1, x2, x3;
                        x4 = cosi * r6;
                        x4 = x4 + x4;
                        x0 = cosi * cosi;
                        r6 = r6 * r6;
                        r6 = r6 + m->ext_2;
                        x1 = x0 * r6;
                        x0 = x0 + r6;
                        x1 = x1 + 1.0f;
                        x2 = x0;
                        x3 = x1;
                        x0 = x0 + x4;
                        x1 = x1 + x4;
                        x2 = x2 - x4;
                        x3 = x3 - x4;
                        x0 = x0 / x2;
                        x1 = x1 / x3;
                        x0 = x0 + x1;
                        fr = R_FABS(x0 * -0.5f);
                    }
                    else
                    {
                        /* dielectric Fresnel for opaque (5108-5134) */
                        real x4 = cosi, n = m->c_rfr, x0, x7, x1, x2, x3, f1;
                        x0 = cosi * n;
                        x7 = x0 * x0;
                        x7 = x7 + 1.0f;
                        x7 = x7 - m->rfr_2;
                        x7 = R_SQRT(x7);
                        x0 = x0 + x7;
                        x1 = x4;
                        x2 = x1 * n;
                        x2 = x2 - x7;
                        x7 = x7 * n;
                        x3 = x1;
                        x1 = x1 + x7;
                        x3 = x3 - x7;
                        x0 = x0 / x2;
                        f1 = x1 / x3;
                        x0 = x0 * x0;
                        f1 = f1 * f1;
                        x0 = x0 + f1;
                        fr = R_FABS(x0 * -0.5f);
                    }
                    fr = fr - 1.0f;
                    fr = fr * m->c_rfl;
                    c_rfl = m->c_rfl + fr;
                }
                {
                    real rc[3] = {0.0f, 0.0f, 0.0f};
                    if (r->depth != 0)
                    {
                        ray_t cr;
                        memcpy(cr.org, h->hit, sizeof(cr.org));
                        memcpy(cr.ray, rw, sizeof(cr.ray));
                        cr.t_min = 0.0f;
                        cr.t_max = FLT_MAX;
                        cr.from = h->srf;
                        cr.flags = side;
                        memcpy(cr.phit, h->loc, sizeof(cr.phit));
                        cr.depth = r->depth - 1;
                        trace(sc, &cr, s->sec_off[side], s->sec_num[side], rc);
                        for (k = 0; k < 3; k++) rc[k] = rc[k] * c_rfl;
                    }
                    for (k = 0; k < 3; k++) c[k] = rc[k] + c[k];
                }
            }
        }
    }
    memcpy(col, c, sizeof(c));
}

ORC void trace(scene_t *sc, const ray_t *r, int off, int num, real col[3])
{
    walk_t w;
    memset(&w, 0, sizeof(w));
    w.tbuf = r->t_max;
    w.best.srf = -1;
    sc->nrays++;
    walk(sc, r, off, num, &w);
    if (w.best.srf < 0)
    {
        col[0] = col[1] = col[2] = 0.0f;
        return;
    }
    shade(sc, r, &w.best, col);
}

/* ---- frame (ray generation 2348-2411, AA offsets engine.cpp:3521-3606,
 *      clamp/AA/gamma/pack 7028-7145 and FRAME_SIMD 1922-1940) ----------- */

static const real aa4_h[4] = {-0.08f - 0.25f, -0.08f + 0.25f,
                               +0.08f - 0.25f, +0.08f + 0.25f};
static const real aa4_v[4] = {+0.08f - 0.25f, -0.08f - 0.25f,
                               +0.08f + 0.25f, -0.08f + 0.25f};
/* 2x alternating (engine.cpp:3536-3570): the pair of offsets depends on
 * the parity of the pixel's column */
static const real aa2_h[2][2] = {{-0.08f + 0.25f, +0.08f - 0.25f},
                                 {+0.08f - 0.25f, -0.08f + 0.25f}};
static const real aa2_v[2][2] = {{+0.08f + 0.25f, -0.08f - 0.25f},
                                 {+0.08f + 0.25f, -0.08f - 0.25f}};

ORC void primary(scene_t *sc, const qr_scene_desc *d,
                    const qr_frame_params *fp, real hs, real vs,
                    real col[3])
{
    ray_t r;
    int k;
    real hx[3], vx[3];
    for (k = 0; k < 3; k++)
    {
        hx[k] = fp->hor[k] * hs;
        vx[k] = fp->ver[k] * vs;
        hx[k] = hx[k] + vx[k];
        r.ray[k] = hx[k] + fp->dir[k];
        r.org[k] = fp->org[k];
        r.phit[k] = 0.0f;
    }
    r.t_min = fp->t_min;
    r.t_max = fp->t_max;
    r.from = -1;
    r.flags = 0;
    r.depth = fp->depth;
    trace(sc, &r, d->cam_off, d->cam_num, col);
}

ORC uint32_t pack(const qr_frame_params *fp, const real col[3])
{
    uint32_t px = 0;
    int k;
    const int sh[3] = {16, 8, 0};
    for (k = 0; k < 3; k++)
    {
        real v = col[k];
        int32_t iv;
        if (fp->ctx_props & QR_PROP_GAMMA) v = R_SQRT(v);
        v = v * 255.0f;
        iv = (isnan(v) || v >= 2147483648.0f || v < -2147483648.0f) ?
             (int32_t)0x80000000 : (int32_t)R_LRINT(v);
        px |= ((uint32_t)iv & 0xFF) << sh[k];
    }
    return px;
}

ORC inline real clamp1(real v) { return v < 1.0f ? v : 1.0f; }

/* the scene view of a descriptor for the walk */
ORC void scene_of(scene_t *sc, const qr_scene_desc *d, const qr_frame_params *fp)
{
    int k;
    memset(sc, 0, sizeof(*sc));
    sc->srf = d->srf;
    sc->mat = d->mat;
    sc->lgt = d->lgt;
    sc->elems = d->elems;
    sc->lelems = d->lelems;
    sc->texels = d->texels;
    for (k = 0; k < 3; k++) sc->amb[k] = fp->amb[k];
    sc->ctx_props = fp->ctx_props;
}

int qr_oracle_render(const qr_scene_desc *d, const qr_frame_params *fp,
                     uint32_t *frame, int y0, int y1, uint64_t *nrays)
{
    scene_t sc;
    int x, y, k;
    if (d == NULL || fp == NULL || frame == NULL) return QR_ERR_ARG;
    memset(&sc, 0, sizeof(sc));
    sc.srf = d->srf;
    sc.mat = d->mat;
    sc.lgt = d->lgt;
    sc.elems = d->elems;
    sc.lelems = d->lelems;
    sc.texels = d->texels;
    for (k = 0; k < 3; k++) sc.amb[k] = fp->amb[k];
    sc.ctx_props = fp->ctx_props;
    if (y1 > fp->y_res) y1 = fp->y_res;

    for (y = y0; y < y1; y++)
    {
        for (x = 0; x < fp->x_res; x++)
        {
            real col[3];
            if (fp->fsaa == 2)
            {
                real cs[4][3];
                int s;
                for (s = 0; s < 4; s++)
                {
                    primary(&sc, d, fp, (real)x + aa4_h[s],
                            (real)y + aa4_v[s], cs[s]);
                    for (k = 0; k < 3; k++) cs[s][k] = clamp1(cs[s][k]);
                }
                for (k = 0; k < 3; k++)
                {
                    real p01 = cs[0][k] * 0.5f + cs[1][k] * 0.5f;
                    real p23 = cs[2][k] * 0.5f + cs[3][k] * 0.5f;
                    col[k] = p01 * 0.5f + p23 * 0.5f;
                }
            }
            else if (fp->fsaa == 1)
            {
                real cs[2][3];
                int s;
                for (s = 0; s < 2; s++)
                {
                    primary(&sc, d, fp, (real)x + aa2_h[x & 1][s],
                            (real)y + aa2_v[x & 1][s], cs[s]);
                    for (k = 0; k < 3; k++) cs[s][k] = clamp1(cs[s][k]);
                }
                for (k = 0; k < 3; k++) col[k] = cs[0][k] * 0.5f + cs[1][k] * 0.5f;
            }
            else
            {
                primary(&sc, d, fp, (real)x, (real)y, col);
                for (k = 0; k < 3; k++) col[k] = clamp1(col[k]);
            }
            frame[(size_t)y * fp->x_row + x] = pack(fp, col);
        }
    }
    if (nrays) *nrays = sc.nrays;
    return QR_OK;
}

/* 1 when the camera ray through (hs, vs) meets a decision within QR_MARGIN
 * of its boundary no farther than its hit (see margin_t) */
ORC int primary_marginal(scene_t *sc, const qr_scene_desc *d, const qr_frame_params *fp,
                         real hs, real vs)
{
    ray_t r;
    walk_t w;
    margin_t mg;
    int k;
    for (k = 0; k < 3; k++)
    {
        real hx = fp->hor[k] * hs;
        real vx = fp->ver[k] * vs;
        hx = hx + vx;
        r.ray[k] = hx + fp->dir[k];
        r.org[k] = fp->org[k];
        r.phit[k] = 0.0f;
    }
    r.t_min = fp->t_min;
    r.t_max = fp->t_max;
    r.from = -1;
    r.flags = 0;
    r.depth = fp->depth;
    memset(&w, 0, sizeof(w));
    memset(&mg, 0, sizeof(mg));
    w.tbuf = r.t_max;
    w.best.srf = -1;
    w.mg = &mg;
    walk(sc, &r, d->cam_off, d->cam_num, &w);
    for (k = 0; k < mg.nev && k < QR_MARGIN_EV; k++)
        if (w.best.srf < 0 || mg.t[k] <= w.tbuf + (real)QR_MARGIN * R_FABS(w.tbuf)) return 1;
    return 0;
}

int qr_oracle_boundary(const qr_scene_desc *d, const qr_frame_params *fp, uint8_t *mask,
                       int y0, int y1)
{
    scene_t sc;
    int x, y, s;
    if (d == NULL || fp == NULL || mask == NULL) return QR_ERR_ARG;
    scene_of(&sc, d, fp);
    if (y1 > fp->y_res) y1 = fp->y_res;
    for (y = y0; y < y1; y++)
    {
        for (x = 0; x < fp->x_res; x++)
        {
            int m = 0;
            if (fp->fsaa == 2)
                for (s = 0; s < 4; s++)
                    m |= primary_marginal(&sc, d, fp, (real)x + aa4_h[s], (real)y + aa4_v[s]);
            else if (fp->fsaa == 1)
                for (s = 0; s < 2; s++)
                    m |= primary_marginal(&sc, d, fp, (real)x + aa2_h[x & 1][s],
                                          (real)y + aa2_v[x & 1][s]);
            else
                m = primary_marginal(&sc, d, fp, (real)x, (real)y);
            mask[(size_t)y * fp->x_res + x] = (uint8_t)m;
        }
    }
    return QR_OK;
}

/* ==== path tracer ==========================================================
 *
 * The estimator of the reference's path-tracer mode (tracer.cpp built with
 * RT_FEAT_PT, rt_Scene::set_pton, RT_FEAT_BUFFERS=0), per sample:
 *   camera ray with a tent-filter jitter of +-0.5 pixel (2267-2342);
 *   at a hit: colour = emission of the material (mat_COL, the light colour
 *   x 100 of a LIGHT material, object.cpp:1346-1375) plus, for a diffuse
 *   material and depth left, l_dff * tex * the colour of a cosine-weighted
 *   bounce (3470-3930, power-series sin/cos 1979-2007), with Russian
 *   roulette at probability max(tex) once the depth left is at most 5
 *   (3484-3528); then the refracted and reflected children of the Whitted
 *   path (4438-5359), where a dielectric, once the depth left is at most
 *   8, follows only one of the two: reflection with
 *   probability P = 0.25 + 0.5 Re, weight c_rfl / P, else refraction with
 *   weight c_trn / (1 - P) (4685-4723); point lights and ambient are not
 *   used (no next-event estimation); colour = rc c_rfl + (tc c_trn + local);
 *   the pixel is the mean of its samples (2115-2139, 2250-2263).
 * Random numbers are counter-based: every draw is a hash of (seed, frame
 * index, pixel index, sample, the drawing node's position in the sample's
 * ray tree, the draw's purpose), so any order of evaluation (depth first
 * here, breadth first in the CUDA wavefront) draws the same numbers.  The
 * hash is the SplitMix64 finaliser (Steele, Lea, Flood 2014) chained over
 * the key; a node's position is its code in base 3: the camera ray 0, the
 * diffuse, refracted and reflected children of node c are 3c + 1, 3c + 2,
 * 3c + 3.
 */

/* depth left at which roulette and the dielectric split start: the
 * reference compares its depth counter with RT_STACK_DEPTH - 5 and - 2
 * (tracer.cpp:3486, 4690; RT_STACK_DEPTH = 10, tracer.h:51) whatever the
 * scene's depth */
#define PT_RR_DEPTH     (10 - 5)
#define PT_SPLIT_DEPTH  (10 - 2)

/* counter-based draws (see the header of this section) */
ORC uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

#define PT_GOLDEN   0x9E3779B97F4A7C15ull
#define PT_CODEMUL  0xD6E8FEB86659FD93ull

/* the key of sample n of a pixel */
ORC uint64_t pt_sample_key(uint64_t seed, int frame, uint64_t pixel, int n)
{
    uint64_t kp = mix64(seed ^ mix64(((uint64_t)(uint32_t)frame << 40) ^ pixel));
    return mix64(kp + (uint64_t)(uint32_t)n * PT_GOLDEN);
}

/* the key of the node with tree code `code` in a sample */
ORC uint64_t pt_node_key(uint64_t ks, uint32_t code)
{
    return mix64(ks ^ ((uint64_t)code * PT_CODEMUL));
}

/* draw d of a node: uniform in [0, 1) with 24 bits, exact in either
 * precision; draws 0 roulette, 1-2 bounce, 3 dielectric split, 4-5 the
 * camera ray's jitter (node 0) */
#define PT_DRAW_RR      0
#define PT_DRAW_BOUNCE  1
#define PT_DRAW_SPLIT   3
#define PT_DRAW_JITTER  4
ORC real pt_draw(uint64_t kn, int d)
{
    uint32_t u = (uint32_t)(mix64(kn + (uint64_t)(d + 1) * PT_GOLDEN) >> 40);
    return (real)(int32_t)u * (real)(1.0f / 16777216.0f);
}

/* power series of sin and cos on [-pi, pi], evaluated with fused
 * multiply-adds like the reference's sinps/cosps (Taylor terms to x^9 and
 * x^8) */
ORC real pt_sin(real x)
{
    real t = x * x, s = x, p = x * t;
    s = R_FMA(p, (real)(-1.0 / 6.0), s);
    p = p * t;
    s = R_FMA(p, (real)(1.0 / 120.0), s);
    p = p * t;
    s = R_FMA(p, (real)(-1.0 / 5040.0), s);
    p = p * t;
    s = R_FMA(p, (real)(1.0 / 362880.0), s);
    return s;
}

ORC real pt_cos(real x)
{
    real t = x * x, c = 1.0f, p = t;
    c = R_FMA(p, (real)(-0.5), c);
    p = p * t;
    c = R_FMA(p, (real)(1.0 / 24.0), c);
    p = p * t;
    c = R_FMA(p, (real)(-1.0 / 720.0), c);
    p = p * t;
    c = R_FMA(p, (real)(1.0 / 40320.0), c);
    return c;
}

#ifdef QR_ORACLE_FP64
#define PT_PI 3.14159265358979323846
#else
#define PT_PI 3.14159265358979323846f
#endif

/* cosine-weighted direction about the unit normal w */
ORC void pt_bounce(const real w[3], real u1, real u2, real d[3])
{
    real a[3] = {0.0f, 0.0f, 0.0f}, u[3], v[3], l, inv, s0, s1, ph, cp, sp;
    int k;
    if (R_FABS(w[0]) > 0.1f) a[1] = 1.0f; else a[0] = 1.0f;
    u[0] = a[1] * w[2] - a[2] * w[1];
    u[1] = a[2] * w[0] - a[0] * w[2];
    u[2] = a[0] * w[1] - a[1] * w[0];
    l = u[0] * u[0] + u[1] * u[1];
    l = l + u[2] * u[2];
    inv = rsq(l);
    for (k = 0; k < 3; k++) u[k] = u[k] * inv;
    v[0] = w[1] * u[2] - w[2] * u[1];
    v[1] = w[2] * u[0] - w[0] * u[2];
    v[2] = w[0] * u[1] - w[1] * u[0];
    s1 = R_SQRT(u1);
    s0 = R_SQRT(1.0f - u1);
    ph = u2 + u2;
    ph = ph * PT_PI;
    ph = ph - PT_PI;
    cp = pt_cos(ph) * s1;
    sp = pt_sin(ph) * s1;
    for (k = 0; k < 3; k++)
    {
        d[k] = w[k] * s0;
        d[k] = d[k] + u[k] * cp;
        d[k] = d[k] + v[k] * sp;
    }
}

/* refracted / reflected children of a hit: the Whitted weights (4442-5359) */
typedef struct pt_sec_s
{
    int  trn, rfl, split;
    real c_trn, c_rfl;
    real nw[3], rw[3];
} pt_sec_t;

ORC void pt_secondary(const scene_t *sc, const ray_t *r, const hit_t *h,
                         const real nrm[3], pt_sec_t *o)
{
    const qr_srf *s = &sc->srf[h->srf];
    int props = s->props[h->side];
    const qr_mat *m = &sc->mat[s->mat[h->side]];
    real c_trn = m->c_trn, c_rfl = m->c_rfl;
    int k;
    o->trn = 0;
    o->rfl = 0;
    o->split = 0;
    if (!(props & QR_PROP_OPAQUE))
    {
        int fres = (props & QR_PROP_FRESNEL) != 0;
        int refr = (props & QR_PROP_REFRACT) != 0;
        int do_trn = 0, m_ok = 1;
        real nw[3];
        if (refr || fres)
        {
            real dn[3], l2, inv, cosi, nci, kk;
            l2 = r->ray[0] * r->ray[0];
            l2 = l2 + r->ray[1] * r->ray[1];
            l2 = l2 + r->ray[2] * r->ray[2];
            inv = rsq(l2);
            for (k = 0; k < 3; k++) dn[k] = r->ray[k] * inv;
            cosi = dn[0] * nrm[0];
            cosi = cosi + dn[1] * nrm[1];
            cosi = cosi + dn[2] * nrm[2];
            nci = cosi * m->c_rfr;
            kk = nci * nci;
            kk = kk + 1.0f;
            kk = kk - m->rfr_2;
            if (fres) m_ok = 0.0f <= kk;
            if (fres && !m_ok)
            {
                c_trn = 0.0f;
                c_rfl = m->c_rfl + m->c_trn;
            }
            else
            {
                real sq = R_SQRT(kk);
                nci = nci + sq;
                if (refr)
                {
                    for (k = 0; k < 3; k++)
                    {
                        real a1 = nrm[k] * nci;
                        real a2 = dn[k] * m->c_rfr;
                        nw[k] = a2 - a1;
                    }
                }
                else
                {
                    for (k = 0; k < 3; k++) nw[k] = r->ray[k];
                }
                if (fres)
                {
                    real x1 = cosi, x2, x3, f0, f1, fr, sqn;
                    x2 = x1 * m->c_rfr;
                    x2 = x2 - sq;
                    sqn = sq * m->c_rfr;
                    x3 = x1;
                    x1 = x1 + sqn;
                    x3 = x3 - sqn;
                    f0 = nci / x2;
                    f1 = x1 / x3;
                    f0 = f0 * f0;
                    f1 = f1 * f1;
                    fr = f0 + f1;
                    fr = R_FABS(fr * -0.5f);
                    fr = fr * m->c_trn;
                    c_trn = m->c_trn - fr;
                    c_rfl = m->c_rfl + fr;
                    o->split = 1;
                }
                do_trn = 1;
            }
        }
        else
        {
            for (k = 0; k < 3; k++) nw[k] = r->ray[k];
            do_trn = 1;
        }
        o->trn = do_trn && m_ok;
        for (k = 0; k < 3; k++) o->nw[k] = nw[k];
    }
    {
        int refl = (props & QR_PROP_REFLECT) != 0;
        int do_rfl = refl || (!(props & QR_PROP_OPAQUE) && (props & QR_PROP_FRESNEL));
        o->rfl = do_rfl;
        if (do_rfl)
        {
            real dn[3], l2, inv, cosi;
            l2 = r->ray[0] * r->ray[0];
            l2 = l2 + r->ray[1] * r->ray[1];
            l2 = l2 + r->ray[2] * r->ray[2];
            inv = rsq(l2);
            for (k = 0; k < 3; k++) dn[k] = r->ray[k] * inv;
            cosi = dn[0] * nrm[0];
            cosi = cosi + dn[1] * nrm[1];
            cosi = cosi + dn[2] * nrm[2];
            for (k = 0; k < 3; k++)
            {
                real p = nrm[k] * cosi;
                real x = dn[k] - p;
                o->rw[k] = x - p;
            }
            if ((props & QR_PROP_FRESNEL) && (props & QR_PROP_OPAQUE))
            {
                real fr;
                if (props & QR_PROP_METAL)
                {
                    real r6 = m->c_rcp, x4, x0, x1, x2, x3;
                    x4 = cosi * r6;
                    x4 = x4 + x4;
                    x0 = cosi * cosi;
                    r6 = r6 * r6;
                    r6 = r6 + m->ext_2;
                    x1 = x0 * r6;
                    x0 = x0 + r6;
                    x1 = x1 + 1.0f;
                    x2 = x0;
                    x3 = x1;
                    x0 = x0 + x4;
                    x1 = x1 + x4;
                    x2 = x2 - x4;
                    x3 = x3 - x4;
                    x0 = x0 / x2;
                    x1 = x1 / x3;
                    x0 = x0 + x1;
                    fr = R_FABS(x0 * -0.5f);
                }
                else
                {
                    real n = m->c_rfr, x0, x7, x1, x2, x3, f1;
                    x0 = cosi * n;
                    x7 = x0 * x0;
                    x7 = x7 + 1.0f;
                    x7 = x7 - m->rfr_2;
                    x7 = R_SQRT(x7);
                    x0 = x0 + x7;
                    x1 = cosi;
                    x2 = x1 * n;
                    x2 = x2 - x7;
                    x7 = x7 * n;
                    x3 = x1;
                    x1 = x1 + x7;
                    x3 = x3 - x7;
                    x0 = x0 / x2;
                    f1 = x1 / x3;
                    x0 = x0 * x0;
                    f1 = f1 * f1;
                    x0 = x0 + f1;
                    fr = R_FABS(x0 * -0.5f);
                }
                fr = fr - 1.0f;
                fr = fr * m->c_rfl;
                c_rfl = m->c_rfl + fr;
            }
        }
    }
    o->c_trn = c_trn;
    o->c_rfl = c_rfl;
}

ORC void pt_trace(scene_t *sc, const ray_t *r, int off, int num, int dmax,
                     uint64_t ks, uint32_t code, real col[3]);

ORC void child(ray_t *cr, const hit_t *h, const real dir[3], int flags, int depth)
{
    int k;
    for (k = 0; k < 3; k++)
    {
        cr->org[k] = h->hit[k];
        cr->ray[k] = dir[k];
        cr->phit[k] = h->loc[k];
    }
    cr->t_min = 0.0f;
    cr->t_max = FLT_MAX;
    cr->from = h->srf;
    cr->flags = flags;
    cr->depth = depth;
}

ORC void pt_shade(scene_t *sc, const ray_t *r, const hit_t *h, int dmax,
                     uint64_t ks, uint32_t code, real col[3])
{
    const uint64_t kn = pt_node_key(ks, code);
    const qr_srf *s = &sc->srf[h->srf];
    int side = h->side;
    int props = s->props[side];
    const qr_mat *m = &sc->mat[s->mat[side]];
    real nrm[3], tex[3], c[3], ddir[3] = {0.0f, 0.0f, 0.0f};
    int dif, k;
    pt_sec_t o;

    hit_surface(sc, h, nrm, tex);

    /* random draws in a fixed order: roulette, bounce, dielectric split */
    dif = (props & QR_PROP_DIFFUSE) && r->depth != 0;
    if (dif && r->depth <= PT_RR_DEPTH)
    {
        real p = tex[0] > tex[1] ? tex[0] : tex[1];
        real u;
        p = p > tex[2] ? p : tex[2];
        u = pt_draw(kn, PT_DRAW_RR);
        if (!(u < p)) dif = 0;
        else
        {
            real rc = 1.0f / p;
            for (k = 0; k < 3; k++) tex[k] = tex[k] * rc;
        }
    }
    if (dif)
    {
        real u1 = pt_draw(kn, PT_DRAW_BOUNCE);
        real u2 = pt_draw(kn, PT_DRAW_BOUNCE + 1);
        pt_bounce(nrm, u1, u2, ddir);
    }
    pt_secondary(sc, r, h, nrm, &o);
    if (o.split && o.trn && o.rfl && r->depth != 0 && r->depth <= PT_SPLIT_DEPTH)
    {
        real u = pt_draw(kn, PT_DRAW_SPLIT);
        real re = o.c_rfl / (o.c_trn + o.c_rfl);
        real pr = re * 0.5f;
        pr = pr + 0.25f;
        if (u < pr)
        {
            o.trn = 0;
            o.c_rfl = o.c_rfl / pr;
        }
        else
        {
            o.rfl = 0;
            o.c_trn = o.c_trn / (1.0f - pr);
        }
    }

    /* diffuse child, then emission */
    for (k = 0; k < 3; k++) c[k] = 0.0f;
    if (dif)
    {
        ray_t cr;
        real lc[3];
        child(&cr, h, ddir, side, r->depth - 1);
        pt_trace(sc, &cr, s->sec_off[side], s->sec_num[side], dmax, ks, 3 * code + 1, lc);
        for (k = 0; k < 3; k++)
        {
            c[k] = lc[k] * m->l_dff;
            c[k] = c[k] * tex[k];
        }
    }
    for (k = 0; k < 3; k++) c[k] = c[k] + m->emit[k];

    if (o.trn)
    {
        real tc[3] = {0.0f, 0.0f, 0.0f};
        if (r->depth != 0)
        {
            ray_t cr;
            child(&cr, h, o.nw, side | FLAG_PASS, r->depth - 1);
            pt_trace(sc, &cr, s->sec_off[1 - side], s->sec_num[1 - side], dmax, ks,
                     3 * code + 2, tc);
            for (k = 0; k < 3; k++) tc[k] = tc[k] * o.c_trn;
        }
        for (k = 0; k < 3; k++) c[k] = tc[k] + c[k];
    }
    if (o.rfl)
    {
        real rc[3] = {0.0f, 0.0f, 0.0f};
        if (r->depth != 0)
        {
            ray_t cr;
            child(&cr, h, o.rw, side, r->depth - 1);
            pt_trace(sc, &cr, s->sec_off[side], s->sec_num[side], dmax, ks, 3 * code + 3, rc);
            for (k = 0; k < 3; k++) rc[k] = rc[k] * o.c_rfl;
        }
        for (k = 0; k < 3; k++) c[k] = rc[k] + c[k];
    }
    for (k = 0; k < 3; k++) col[k] = c[k];
}

ORC void pt_trace(scene_t *sc, const ray_t *r, int off, int num, int dmax,
                     uint64_t ks, uint32_t code, real col[3])
{
    walk_t w;
    memset(&w, 0, sizeof(w));
    w.tbuf = r->t_max;
    w.best.srf = -1;
    sc->nrays++;
    walk(sc, r, off, num, &w);
    if (w.best.srf < 0)
    {
        col[0] = col[1] = col[2] = 0.0f;
        return;
    }
    pt_shade(sc, r, &w.best, dmax, ks, code, col);
}

/* tent filter on [-1, 1] from one uniform number (2267-2342), halved */
ORC real pt_tent(real u)
{
    real r = u + u, d;
    if (r < 1.0f) d = R_SQRT(r) - 1.0f;
    else d = 1.0f - R_SQRT(2.0f - r);
    return d * 0.5f;
}


/* fp->pt_on samples of pixel (x, y) added to its running sums a[3]; the
 * mean is returned packed */
ORC uint32_t pt_pixel(scene_t *sc, const qr_scene_desc *d, const qr_frame_params *fp,
                      int x, int y, real *a)
{
    real sum[3] = {0.0f, 0.0f, 0.0f}, mean[3];
    const int spp = fp->pt_on, n0 = (int)fp->pts_c;
    const uint64_t pixel = (uint64_t)y * fp->x_res + x;
    int n, k;
    for (n = 0; n < spp; n++)
    {
        real hs, vs, col[3];
        ray_t r;
        const uint64_t ks = pt_sample_key(fp->seed, fp->frame_idx, pixel, n0 + n);
        const uint64_t k0 = pt_node_key(ks, 0);
        hs = pt_tent(pt_draw(k0, PT_DRAW_JITTER));
        vs = pt_tent(pt_draw(k0, PT_DRAW_JITTER + 1));
        hs = (real)x + hs;
        vs = (real)y + vs;
        for (k = 0; k < 3; k++)
        {
            real hx = fp->hor[k] * hs;
            real vx = fp->ver[k] * vs;
            hx = hx + vx;
            r.ray[k] = hx + fp->dir[k];
            r.org[k] = fp->org[k];
            r.phit[k] = 0.0f;
        }
        r.t_min = fp->t_min;
        r.t_max = fp->t_max;
        r.from = -1;
        r.flags = 0;
        r.depth = fp->depth;
        pt_trace(sc, &r, d->cam_off, d->cam_num, fp->depth, ks, 0, col);
        for (k = 0; k < 3; k++) sum[k] = sum[k] + col[k];
    }
    for (k = 0; k < 3; k++)
    {
        a[k] = (n0 == 0 ? 0.0f : a[k]) + sum[k];
        mean[k] = a[k] / (real)(n0 + spp);
        mean[k] = clamp1(mean[k]);
    }
    return pack(fp, mean);
}

int qr_oracle_pt(const qr_scene_desc *d, const qr_frame_params *fp, void *acc_,
                 uint32_t *frame, int y0, int y1, uint64_t *nrays)
{
    scene_t sc;
    real *acc = (real *)acc_;
    int x, y;
    scene_of(&sc, d, fp);
    if (fp->pt_on <= 0) return 1;
    for (y = y0; y < y1; y++)
    {
        for (x = 0; x < fp->x_res; x++)
        {
            const uint32_t px = pt_pixel(&sc, d, fp, x, y,
                                         &acc[3 * ((size_t)y * fp->x_row + x)]);
            if (frame != NULL) frame[(size_t)y * fp->x_row + x] = px;
        }
    }
    if (nrays != NULL) *nrays = sc.nrays;
    return 0;
}

/*
 * accel.cpp: conservative world boxes of a flattened scene's surfaces and a
 * binned-SAH bounding-volume hierarchy over its camera list (see accel.h).
 */
#include "accel.h"

#include <math.h>
#include <string.h>
#include <algorithm>

namespace
{

const double INF = HUGE_VAL;

struct Box
{
    double lo[3], hi[3];
    void inf()
    {
        for (int k = 0; k < 3; k++) { lo[k] = -INF; hi[k] = +INF; }
    }
    bool finite() const
    {
        for (int k = 0; k < 3; k++)
            if (!(lo[k] > -INF && hi[k] < INF)) return false;
        return true;
    }
    bool empty() const
    {
        for (int k = 0; k < 3; k++)
            if (lo[k] > hi[k]) return true;
        return false;
    }
    void meet(const Box &b)
    {
        for (int k = 0; k < 3; k++)
        {
            lo[k] = std::max(lo[k], b.lo[k]);
            hi[k] = std::min(hi[k], b.hi[k]);
        }
    }
};

/* a record's 3x3 transform as the tracer applies it (xform in tracer.cu:
 * diagonal only for amap[3] == 1, "scaling only") */
void record_matrix(const qr_srf &t, double m[3][3])
{
    const float *row[3] = {t.tci, t.tcj, t.tck};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            m[i][j] = (t.amap[3] == 1 && i != j) ? 0.0 : (double)row[i][j];
}

bool invert3(const double m[3][3], double r[3][3])
{
    double c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
    double c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
    double c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
    double det = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
    if (!(fabs(det) > 1e-30)) return false;
    double id = 1.0 / det;
    r[0][0] = c00 * id;
    r[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
    r[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
    r[1][0] = c01 * id;
    r[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
    r[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
    r[2][0] = c02 * id;
    r[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
    r[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
    return true;
}

/* interval image of box u under h = a * u + o */
Box affine_image(const double a[3][3], const double o[3], const Box &u)
{
    Box h;
    for (int i = 0; i < 3; i++)
    {
        double lo = o[i], hi = o[i];
        for (int j = 0; j < 3; j++)
        {
            const double c = a[i][j];
            if (c == 0.0) continue;
            const double p = c * u.lo[j], q = c * u.hi[j];
            if (isnan(p) || isnan(q)) { lo = -INF; hi = INF; break; }
            lo += std::min(p, q);
            hi += std::max(p, q);
        }
        h.lo[i] = lo;
        h.hi[i] = hi;
    }
    return h;
}

/* minimum of g(x) = a x^2 - 2 b x over [lo, hi] */
double gmin(double a, double b, double lo, double hi)
{
    if (a > 0.0)
    {
        double x = std::min(std::max(b / a, lo), hi);
        return a * x * x - 2.0 * b * x;
    }
    if (a == 0.0)
    {
        if (b == 0.0) return 0.0;
        double x = b > 0.0 ? hi : lo;
        if (!(x > -INF && x < INF)) return -INF;
        return -2.0 * b * x;
    }
    if (!(lo > -INF && hi < INF)) return -INF;
    return std::min(a * lo * lo - 2.0 * b * lo, a * hi * hi - 2.0 * b * hi);
}

/* tighten box u to the sublevel set  sum_k (a_k x_k^2 - 2 b_k x_k) <= w  */
void quadric_tighten(const double a[3], const double b[3], double w, Box &u)
{
    for (int it = 0; it < 4; it++)
    {
        for (int j = 0; j < 3; j++)
        {
            double U = w;
            for (int k = 0; k < 3; k++)
            {
                if (k == j) continue;
                U -= gmin(a[k], b[k], u.lo[k], u.hi[k]);
            }
            if (!(U < INF)) continue;
            if (a[j] > 0.0)
            {
                double rhs = U + b[j] * b[j] / a[j];
                if (rhs < 0.0) rhs = 0.0;
                const double c = b[j] / a[j], r = sqrt(rhs / a[j]);
                u.lo[j] = std::max(u.lo[j], c - r);
                u.hi[j] = std::min(u.hi[j], c + r);
            }
            else if (a[j] == 0.0 && b[j] != 0.0)
            {
                if (b[j] > 0.0) u.lo[j] = std::max(u.lo[j], -U / (2.0 * b[j]));
                else            u.hi[j] = std::min(u.hi[j], U / (-2.0 * b[j]));
            }
        }
    }
}

/*
 * Rounding allowance.  The tracer evaluates the quadric (its c coefficient,
 * the discriminant) and the hit position in float on local coordinates of
 * magnitude up to D; far from the surface those values are dominated by
 * rounding, and the reference's arithmetic, which the tracer reproduces,
 * then reports hits the exact geometry does not have.  A box must contain
 * them too: the quadric is widened to {f <= eta} with eta = G (sum |sci| D^2
 * + 2 sum |scj| D + |w|), and positions by G D, where G = 32 float epsilons
 * is several times the rounding of those few operations.  Rays whose origin
 * is farther than D allows are walked in list order instead (qr_dscene
 * ray_c / ray_r2).
 */
const double G_ROUND = 32.0 * 1.1920928955078125e-7;

double quadric_eta(const float sci[4], const float scj[3], double D)
{
    double e = fabs((double)sci[3]);
    for (int k = 0; k < 3; k++)
        e += fabs((double)sci[k]) * D * D + 2.0 * fabs((double)scj[k]) * D;
    return G_ROUND * e;
}

/* surface in its local coordinates: quadric {f <= eta} (or the plane k = 0)
 * within the active axis clippers (clip_root, tracer.cu), for local
 * coordinates up to D in magnitude */
Box local_surface_box(const qr_srf &s, double D)
{
    const double m = G_ROUND * D + 1e-6;
    Box u;
    u.inf();
    for (int k = 0; k < 3; k++)
    {
        if ((s.mint >> k) & 1) u.lo[k] = s.bmin[k] - m;
        if ((s.maxt >> k) & 1) u.hi[k] = s.bmax[k] + m;
    }
    if (s.solver == 1)
    {
        const int mk = s.amap[2];
        u.lo[mk] = std::max(u.lo[mk], -m);
        u.hi[mk] = std::min(u.hi[mk], +m);
        return u;
    }
    double a[3], b[3];
    for (int k = 0; k < 3; k++) { a[k] = s.sci[k]; b[k] = s.scj[k]; }
    quadric_tighten(a, b, (double)s.sci[3] + quadric_eta(s.sci, s.scj, D), u);
    for (int k = 0; k < 3; k++) { u.lo[k] -= m; u.hi[k] += m; }
    return u;
}

/* region a clipper keeps when it subtracts its outer subspace (v <= 0 in the
 * clipper evaluation of clip_root, tracer.cu), with the rounding allowance */
Box local_clip_region(const qr_srf &c, double D)
{
    const double m = G_ROUND * D + 1e-6;
    Box u;
    u.inf();
    if (c.clpk == 1)
    {
        const int mk = c.amap[2];
        if (c.asgn[2]) u.lo[mk] = -m;       /* -p_k <= 0 */
        else           u.hi[mk] = +m;       /*  p_k <= 0 */
        return u;
    }
    double a[3], b[3];
    float scj0[3] = {0.0f, 0.0f, 0.0f};
    for (int k = 0; k < 3; k++)
    {
        a[k] = c.sci[k];
        b[k] = c.clpk == 2 ? c.scj[k] : 0.0;
    }
    quadric_tighten(a, b, (double)c.sci[3] +
                    quadric_eta(c.sci, c.clpk == 2 ? c.scj : scj0, D), u);
    for (int k = 0; k < 3; k++) { u.lo[k] -= m; u.hi[k] += m; }
    return u;
}

/* largest row norm of a record's 3x3 transform (1 without one): local
 * coordinates are at most this times the world distance */
double record_gain(const qr_srf &t)
{
    if (t.amap[3] == 0) return 1.0;
    double m[3][3], g = 0.0;
    record_matrix(t, m);
    for (int i = 0; i < 3; i++)
        g = std::max(g, sqrt(m[i][0] * m[i][0] + m[i][1] * m[i][1] + m[i][2] * m[i][2]));
    return std::max(g, 1.0);
}

/*
 * world box of local box u of record s, where the local coordinates are
 *   xf >= 0 (transform node T, am3(T) != 0): loc = M_T (h - T.pos) - s.pos
 *   own transform (am3(s) != 0):             loc = M_s (h - s.pos)
 *   translation only:                        loc = h - s.pos
 * and node_only selects the transform-node form loc = X_T(h) - s.pos with
 * X_T(h) = am3(T) ? M_T (h - T.pos) : h - T.pos (clip-list groups)
 */
bool world_box(const qr_scene_desc *d, const qr_srf &s, int xf, bool node_only,
               const Box &u, Box &w)
{
    double a[3][3], o[3];
    if (xf >= 0 && (node_only || d->srf[xf].amap[3] != 0))
    {
        const qr_srf &t = d->srf[xf];
        Box v = u;
        for (int k = 0; k < 3; k++) { v.lo[k] += s.pos[k]; v.hi[k] += s.pos[k]; }
        if (t.amap[3] != 0)
        {
            double m[3][3];
            record_matrix(t, m);
            if (!invert3(m, a)) return false;
        }
        else
        {
            memset(a, 0, sizeof(a));
            a[0][0] = a[1][1] = a[2][2] = 1.0;
        }
        for (int k = 0; k < 3; k++) o[k] = t.pos[k];
        w = affine_image(a, o, v);
        return true;
    }
    if (s.amap[3] != 0)
    {
        double m[3][3];
        record_matrix(s, m);
        if (!invert3(m, a)) return false;
    }
    else
    {
        memset(a, 0, sizeof(a));
        a[0][0] = a[1][1] = a[2][2] = 1.0;
    }
    for (int k = 0; k < 3; k++) o[k] = s.pos[k];
    w = affine_image(a, o, u);
    return true;
}

void pad(Box &b)
{
    for (int k = 0; k < 3; k++)
    {
        const double m = 1e-3 + 1e-4 * (fabs(b.lo[k]) + fabs(b.hi[k]));
        b.lo[k] -= m;
        b.hi[k] += m;
    }
}

/* transform node of each element of a list (-1 outside groups), following
 * the element layout of qr_elem (QR_ELM_TRNODE with `last`) */
void list_groups(const qr_scene_desc *d, int off, int num, std::vector<int> &xf)
{
    xf.assign(num, -1);
    int node = -1, last = -1;
    for (int e = 0; e < num; e++)
    {
        const qr_elem &el = d->elems[off + e];
        if (node >= 0 && off + e > last) node = -1;
        if (el.kind == QR_ELM_TRNODE)
        {
            node = el.ref;
            last = el.last;
            continue;
        }
        xf[e] = node;
    }
}

/* ---- binned SAH ---------------------------------------------------------- */

struct Prim
{
    Box b;
    double c[3];
    qr_bitem it;
};

double area(const Box &b)
{
    double dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return 2.0 * (dx * dy + dy * dz + dz * dx);
}

Box merge(const Box &a, const Box &b)
{
    Box r;
    for (int k = 0; k < 3; k++)
    {
        r.lo[k] = std::min(a.lo[k], b.lo[k]);
        r.hi[k] = std::max(a.hi[k], b.hi[k]);
    }
    return r;
}

int build_node(std::vector<Prim> &p, int lo, int hi, int depth, qr_accel_host *out)
{
    const int idx = (int)out->nodes.size();
    out->nodes.push_back(qr_bnode());
    Box bb = p[lo].b, cb;
    for (int k = 0; k < 3; k++) cb.lo[k] = cb.hi[k] = p[lo].c[k];
    for (int i = lo + 1; i < hi; i++)
    {
        bb = merge(bb, p[i].b);
        for (int k = 0; k < 3; k++)
        {
            cb.lo[k] = std::min(cb.lo[k], p[i].c[k]);
            cb.hi[k] = std::max(cb.hi[k], p[i].c[k]);
        }
    }
    if (depth > out->depth) out->depth = depth;
    const int n = hi - lo;
    int mid = -1;
    if (n > 2 && depth < QR_BVH_STACK - 8)
    {
        /* binned SAH over the centroid box */
        const int NB = 12;
        double best = area(bb) * n;     /* cost of a leaf */
        int bax = -1, bsplit = -1;
        for (int ax = 0; ax < 3; ax++)
        {
            const double ext = cb.hi[ax] - cb.lo[ax];
            if (!(ext > 0.0)) continue;
            Box bin[NB];
            int cnt[NB] = {0};
            for (int i = lo; i < hi; i++)
            {
                int q = (int)((p[i].c[ax] - cb.lo[ax]) / ext * NB);
                q = std::min(std::max(q, 0), NB - 1);
                bin[q] = cnt[q] ? merge(bin[q], p[i].b) : p[i].b;
                cnt[q]++;
            }
            /* boxes and counts right of every split in one sweep from the
             * right, then the left ones in one sweep from the left */
            Box rb[NB];
            int rn[NB + 1];
            rn[NB] = 0;
            for (int q = NB - 1; q >= 0; q--)
            {
                rn[q] = rn[q + 1] + cnt[q];
                if (cnt[q]) rb[q] = rn[q + 1] ? merge(rb[q + 1], bin[q]) : bin[q];
                else if (rn[q + 1]) rb[q] = rb[q + 1];
            }
            Box l;
            int nl = 0;
            for (int s = 1; s < NB; s++)
            {
                if (cnt[s - 1]) { l = nl ? merge(l, bin[s - 1]) : bin[s - 1]; nl += cnt[s - 1]; }
                const int nr = rn[s];
                if (nl == 0 || nr == 0) continue;
                const double cost = 0.5 * area(bb) + area(l) * nl + area(rb[s]) * nr;
                if (cost < best) { best = cost; bax = ax; bsplit = s; }
            }
        }
        if (bax >= 0)
        {
            const double ext = cb.hi[bax] - cb.lo[bax];
            Prim *m = std::partition(&p[lo], &p[lo] + n, [&](const Prim &x) {
                int q = (int)((x.c[bax] - cb.lo[bax]) / ext * NB);
                q = std::min(std::max(q, 0), NB - 1);
                return q < bsplit;
            });
            mid = (int)(m - &p[0]);
            if (mid <= lo || mid >= hi) mid = -1;
        }
    }
    if (mid < 0 && n > QR_BVH_LEAF_MAX)
    {
        /* a leaf holds at most QR_BVH_LEAF_MAX items: halve the node at
         * the median centroid of its widest axis (or in list order) */
        int ax = 0;
        for (int k = 1; k < 3; k++)
            if (cb.hi[k] - cb.lo[k] > cb.hi[ax] - cb.lo[ax]) ax = k;
        mid = lo + n / 2;
        if (cb.hi[ax] > cb.lo[ax])
            std::nth_element(&p[lo], &p[mid], &p[lo] + n, [ax](const Prim &u, const Prim &v) {
                return u.c[ax] < v.c[ax];
            });
    }
    qr_bnode nd;
    memset(&nd, 0, sizeof(nd));
    for (int k = 0; k < 3; k++)
    {
        nd.lo[k] = (float)bb.lo[k];
        nd.hi[k] = (float)bb.hi[k];
        /* round outwards to float */
        if ((double)nd.lo[k] > bb.lo[k]) nd.lo[k] = nextafterf(nd.lo[k], -HUGE_VALF);
        if ((double)nd.hi[k] < bb.hi[k]) nd.hi[k] = nextafterf(nd.hi[k], +HUGE_VALF);
    }
    if (mid < 0)
    {
        nd.a = (int)out->items.size();
        nd.count = n;
        for (int i = lo; i < hi; i++) out->items.push_back(p[i].it);
        /* items under one transform node next to each other, so the walk
         * transforms the ray once for them (ties between hits are decided
         * by list position, not by the order of the items) */
        std::stable_sort(out->items.begin() + nd.a, out->items.end(),
                         [](const qr_bitem &u, const qr_bitem &v) { return u.xf < v.xf; });
        out->nodes[idx] = nd;
        return idx;
    }
    nd.count = 0;
    out->nodes[idx] = nd;
    const int l = build_node(p, lo, mid, depth + 1, out);
    const int r = build_node(p, mid, hi, depth + 1, out);
    out->nodes[idx].a = l;
    out->nodes[idx].b = r;
    return idx;
}

} /* namespace */

void qr_accel_pairs(const std::vector<qr_bnode> &nodes, std::vector<qr_bpair> &pairs)
{
    pairs.assign(nodes.size(), qr_bpair());
    for (size_t i = 0; i < nodes.size(); i++)
    {
        const qr_bnode &nd = nodes[i];
        qr_bpair &pr = pairs[i];
        memset(&pr, 0, sizeof(pr));
        if (nd.count > 0) continue;
        const qr_bnode &a = nodes[nd.a], &b = nodes[nd.b];
        for (int k = 0; k < 3; k++)
        {
            pr.lo_a[k] = a.lo[k];
            pr.hi_a[k] = a.hi[k];
            pr.lo_b[k] = b.lo[k];
            pr.hi_b[k] = b.hi[k];
        }
        pr.code_a = qr_bnode_code(a, nd.a);
        pr.code_b = qr_bnode_code(b, nd.b);
    }
}

static double node_area(const qr_bnode &n)
{
    const double dx = (double)n.hi[0] - n.lo[0], dy = (double)n.hi[1] - n.lo[1],
                 dz = (double)n.hi[2] - n.lo[2];
    return 2.0 * (dx * dy + dy * dz + dz * dx);
}

/* the record of inner node i and, recursively, of its inner slots; returns
 * its index; *need: the deepest stack below it */
static int32_t make_quad(const std::vector<qr_bnode> &nodes, int32_t i,
                         std::vector<qr_bquad> &quads, std::vector<int32_t> &src,
                         int32_t *need)
{
    int32_t ch[4] = {nodes[i].a, nodes[i].b, -1, -1};
    int n = 2;
    while (n < 4)
    {
        /* open the inner child with the largest box */
        int best = -1;
        double ba = -1.0;
        for (int k = 0; k < n; k++)
        {
            const qr_bnode &c = nodes[ch[k]];
            if (c.count == 0 && node_area(c) > ba) { ba = node_area(c); best = k; }
        }
        if (best < 0) break;
        const qr_bnode &c = nodes[ch[best]];
        ch[best] = c.a;
        ch[n++] = c.b;
    }
    const int32_t q = (int32_t)quads.size();
    quads.push_back(qr_bquad());
    src.resize(4 * quads.size(), -1);
    qr_bquad rec;
    memset(&rec, 0, sizeof(rec));
    int32_t below = 0;
    for (int k = 0; k < 4; k++)
    {
        if (k >= n)
        {
            rec.lo_x[k] = rec.lo_y[k] = rec.lo_z[k] = HUGE_VALF;
            rec.hi_x[k] = rec.hi_y[k] = rec.hi_z[k] = -HUGE_VALF;
            rec.code[k] = QR_BQUAD_EMPTY;
            src[4 * q + k] = -1;
            continue;
        }
        const qr_bnode &c = nodes[ch[k]];
        rec.lo_x[k] = c.lo[0]; rec.lo_y[k] = c.lo[1]; rec.lo_z[k] = c.lo[2];
        rec.hi_x[k] = c.hi[0]; rec.hi_y[k] = c.hi[1]; rec.hi_z[k] = c.hi[2];
        src[4 * q + k] = ch[k];
        if (c.count > 0)
        {
            rec.code[k] = qr_bnode_code(c, ch[k]);
        }
        else
        {
            int32_t nb = 0;
            rec.code[k] = make_quad(nodes, ch[k], quads, src, &nb);
            below = std::max(below, nb);
        }
    }
    quads[q] = rec;
    /* a visit pushes the hit slots but the nearest: n - 1 entries */
    *need = (n - 1) + below;
    return q;
}

void qr_accel_quads(const std::vector<qr_bnode> &nodes, const int *root, int nlev,
                    std::vector<qr_bquad> &quads, std::vector<int32_t> &src,
                    int32_t *quad_root, int32_t *stack_need)
{
    quads.clear();
    src.clear();
    for (int l = 0; l < nlev; l++)
    {
        quad_root[l] = QR_BQUAD_EMPTY;
        stack_need[l] = 0;
        if (root[l] < 0 || root[l] >= (int)nodes.size()) continue;
        const qr_bnode &r = nodes[root[l]];
        if (r.count > 0)
        {
            quad_root[l] = qr_bnode_code(r, root[l]);
            continue;
        }
        int32_t need = 0;
        quad_root[l] = make_quad(nodes, root[l], quads, src, &need);
        stack_need[l] = need;
    }
}

/* node boxes of a tree whose items' boxes changed, bottom-up: nodes are
 * stored parent before children (build_node), so a reverse sweep sees
 * children first */
static void refit(qr_accel_host *out)
{
    for (int i = (int)out->nodes.size() - 1; i >= 0; i--)
    {
        qr_bnode &nd = out->nodes[i];
        float lo[3] = {HUGE_VALF, HUGE_VALF, HUGE_VALF};
        float hi[3] = {-HUGE_VALF, -HUGE_VALF, -HUGE_VALF};
        if (nd.count > 0)
        {
            for (int j = nd.a; j < nd.a + nd.count; j++)
            {
                const float *b = &out->boxes[6 * (size_t)out->items[j].srf];
                for (int k = 0; k < 3; k++)
                {
                    lo[k] = std::min(lo[k], b[k]);
                    hi[k] = std::max(hi[k], b[3 + k]);
                }
            }
        }
        else
        {
            const qr_bnode &a = out->nodes[nd.a], &b = out->nodes[nd.b];
            for (int k = 0; k < 3; k++)
            {
                lo[k] = std::min(a.lo[k], b.lo[k]);
                hi[k] = std::max(a.hi[k], b.hi[k]);
            }
        }
        for (int k = 0; k < 3; k++) { nd.lo[k] = lo[k]; nd.hi[k] = hi[k]; }
    }
}

/* the scene's extent, from which every level's radius and rounding
 * allowance follow: boxes without rounding allowance and record positions,
 * joined with the motion bound `bound` (lo[3], hi[3]; NULL: none) */
struct Extent
{
    std::vector<int> xf;        /* transform node per camera-list element */
    std::vector<int> srf_xf;    /* per record (-2: not in the camera list) */
    double clo[3], chi[3], rs, gain;
};

static void scene_extent(const qr_scene_desc *d, const float *bound, Extent &x)
{
    list_groups(d, d->cam_off, d->cam_num, x.xf);
    x.srf_xf.assign(d->nsrf, -2);
    for (int e = 0; e < d->cam_num; e++)
    {
        const qr_elem &el = d->elems[d->cam_off + e];
        if (el.kind == QR_ELM_SURFACE) x.srf_xf[el.ref] = x.xf[e];
    }
    x.gain = 1.0;
    for (int i = 0; i < d->nsrf; i++) x.gain = std::max(x.gain, record_gain(d->srf[i]));
    double *clo = x.clo, *chi = x.chi;
    for (int k = 0; k < 3; k++) { clo[k] = INF; chi[k] = -INF; }
    for (int i = 0; i < d->nsrf; i++)
    {
        const qr_srf &s = d->srf[i];
        if (s.is_node || x.srf_xf[i] == -2) continue;
        Box u = local_surface_box(s, 0.0), w;
        if (u.empty() || !world_box(d, s, x.srf_xf[i], false, u, w) || !w.finite()) continue;
        for (int k = 0; k < 3; k++)
        {
            clo[k] = std::min(clo[k], w.lo[k]);
            chi[k] = std::max(chi[k], w.hi[k]);
        }
    }
    /* record positions too (transform nodes, surfaces): the local
     * coordinates the walk forms start from them */
    for (int i = 0; i < d->nsrf; i++)
        for (int k = 0; k < 3; k++)
        {
            clo[k] = std::min(clo[k], (double)d->srf[i].pos[k]);
            chi[k] = std::max(chi[k], (double)d->srf[i].pos[k]);
        }
    if (bound != NULL)
        for (int k = 0; k < 3; k++)
        {
            clo[k] = std::min(clo[k], (double)bound[k]);
            chi[k] = std::max(chi[k], (double)bound[3 + k]);
        }
    double rs = 0.0;
    for (int k = 0; k < 3; k++)
    {
        if (!(clo[k] <= chi[k])) { clo[k] = chi[k] = 0.0; }
        rs += 0.25 * (chi[k] - clo[k]) * (chi[k] - clo[k]);
    }
    x.rs = sqrt(rs);
}

/* rays starting within ray_r of the extent's centre use level `level`;
 * their local coordinates stay below D.  Each level covers 8 times the
 * radius of the previous one, with boxes widened for the larger rounding */
static void level_radius(const Extent &x, int level, double *ray_r, double *D)
{
    *ray_r = (6.0 * x.rs + 8.0) * pow(8.0, (double)level);
    *D = x.gain * (*ray_r + 2.0 * x.rs + 1.0) + 1.0;
}

static int accel_build(const qr_scene_desc *d, qr_accel_host *out, int level,
                       const qr_accel_host *topo, const float *bound);

int qr_accel_build(const qr_scene_desc *d, qr_accel_host *out, int level)
{
    return accel_build(d, out, level, NULL, NULL);
}

/* level `level` of the hierarchy; with `topo` (the tree of another level
 * over the same bounded surfaces) its topology is kept and only the boxes
 * are refitted, the tree shape does not change the frame */
static int accel_build(const qr_scene_desc *d, qr_accel_host *out, int level,
                       const qr_accel_host *topo, const float *bound)
{
    out->nodes.clear();
    out->items.clear();
    out->always.clear();
    out->depth = 0;
    out->boxes.assign((size_t)d->nsrf * 6, 0.0f);
    out->bounded.assign(d->nsrf, 0);

    Extent x;
    scene_extent(d, bound, x);
    const std::vector<int> &xf = x.xf, &srf_xf = x.srf_xf;
    for (int k = 0; k < 3; k++)
    {
        out->ray_c[k] = (float)(0.5 * (x.clo[k] + x.chi[k]));
        out->ext[k] = x.clo[k];
        out->ext[3 + k] = x.chi[k];
    }
    out->gain = x.gain;
    double ray_r, D;
    level_radius(x, level, &ray_r, &D);
    out->ray_r2 = (float)(ray_r * ray_r);

    /* world boxes of the surfaces (unclipped by custom clippers) */
    std::vector<Box> wbox(d->nsrf);
    std::vector<char> ok(d->nsrf, 0);
    for (int i = 0; i < d->nsrf; i++)
    {
        const qr_srf &s = d->srf[i];
        if (s.is_node || srf_xf[i] == -2) continue;
        Box u = local_surface_box(s, D), w;
        if (u.empty()) { wbox[i] = u; ok[i] = 0; continue; }
        ok[i] = world_box(d, s, srf_xf[i], false, u, w) ? 1 : 0;
        wbox[i] = w;
    }

    /* clippers that keep only the inside of a surface (v <= 0, relation
     * "minus outer", outside accumulator segments) bound the clipped one */
    for (int i = 0; i < d->nsrf; i++)
    {
        const qr_srf &s = d->srf[i];
        if (!ok[i] || s.clip_num <= 0) continue;
        std::vector<int> cxf;
        list_groups(d, s.clip_off, s.clip_num, cxf);
        int acc = 0;
        for (int e = 0; e < s.clip_num; e++)
        {
            const qr_elem &el = d->elems[s.clip_off + e];
            if (el.kind == QR_ELM_ACC_ENTER) { acc = 1; continue; }
            if (el.kind == QR_ELM_ACC_LEAVE) { acc = 0; continue; }
            if (el.kind != QR_ELM_SURFACE || acc || el.rel <= 0) continue;
            const qr_srf &c = d->srf[el.ref];
            Box u = local_clip_region(c, D), w;
            if (!world_box(d, c, cxf[e], true, u, w)) continue;
            wbox[i].meet(w);
        }
    }

#ifndef QR_ALWAYS_FRAC
#define QR_ALWAYS_FRAC 0.2
#endif
    /* surfaces whose box covers more than a fifth of the bounded extent's
     * surface area (the walls of a room) are tested by every ray, as the
     * unbounded ones are, instead of widening the tree's upper nodes: the
     * 1280x720 64-spp frame of the closed box takes 121.7 against 157.2 ms
     * (at a twelfth of the area 130.2 ms, and the animated frame, whose
     * larger surfaces then leave the tree, 28.6 against 20.1 ms) */
    double ext_area = 0.0;
    if (QR_ALWAYS_FRAC > 0.0)
    {
        Box all;
        bool any = false;
        for (int i = 0; i < d->nsrf; i++)
        {
            if (!ok[i] || wbox[i].empty() || !wbox[i].finite()) continue;
            all = any ? merge(all, wbox[i]) : wbox[i];
            any = true;
        }
        if (any) ext_area = area(all);
    }
    for (int e = 0; e < d->cam_num; e++)
    {
        const qr_elem &el = d->elems[d->cam_off + e];
        if (el.kind != QR_ELM_SURFACE) continue;
        const int i = el.ref;
        qr_bitem it;
        it.pos = e;
        it.srf = i;
        it.xf = (xf[e] >= 0 && d->srf[xf[e]].amap[3] != 0) ? xf[e] : -1;
        it.pad = 0;
        Box b = wbox[i];
        const bool huge = QR_ALWAYS_FRAC > 0.0 && ext_area > 0.0 && ok[i] && !b.empty() &&
                          b.finite() && area(b) > QR_ALWAYS_FRAC * ext_area;
        if (ok[i] && !b.empty() && b.finite() && !huge)
        {
            pad(b);
            for (int k = 0; k < 3; k++)
            {
                out->boxes[6 * i + k] = (float)b.lo[k];
                out->boxes[6 * i + 3 + k] = (float)b.hi[k];
            }
            out->bounded[i] = 1;
        }
        else
        {
            out->always.push_back(it);
        }
    }

    std::vector<Prim> prims;
    for (int e = 0; e < d->cam_num; e++)
    {
        const qr_elem &el = d->elems[d->cam_off + e];
        if (el.kind != QR_ELM_SURFACE || out->bounded[el.ref] != 1) continue;
        Prim p;
        const int i = el.ref;
        for (int k = 0; k < 3; k++)
        {
            p.b.lo[k] = out->boxes[6 * i + k];
            p.b.hi[k] = out->boxes[6 * i + 3 + k];
            p.c[k] = 0.5 * (p.b.lo[k] + p.b.hi[k]);
        }
        p.it.pos = e;
        p.it.srf = i;
        p.it.xf = (xf[e] >= 0 && d->srf[xf[e]].amap[3] != 0) ? xf[e] : -1;
        p.it.pad = 0;
        prims.push_back(p);
    }
    if (topo != NULL && topo->bounded == out->bounded && topo->always.size() == out->always.size())
    {
        out->nodes = topo->nodes;
        out->items = topo->items;
        out->depth = topo->depth;
        refit(out);
        return 0;
    }
    if (!prims.empty()) build_node(prims, 0, (int)prims.size(), 1, out);
    return 0;
}

void qr_accel_build_levels(const qr_scene_desc *d, qr_accel_host *out,
                           int root[QR_BVH_LEVELS], int aoff[QR_BVH_LEVELS],
                           int anum[QR_BVH_LEVELS], float r2[QR_BVH_LEVELS],
                           const float *bound)
{
    out->nodes.clear();
    out->items.clear();
    out->always.clear();
    out->depth = 0;
    qr_accel_host lv0;
    for (int l = 0; l < QR_BVH_LEVELS; l++)
    {
        const int n0 = (int)out->nodes.size();
        root[l] = n0;
        aoff[l] = (int)out->always.size();
        anum[l] = 0;
        r2[l] = -1.0f;
        /* the outer levels' boxes are wide; for short lists a walk in list
         * order is cheaper than traversing them, and they are not built */
        const bool used = l == 0 || d->cam_num >= QR_BVH_OUTER_MIN;
        out->lboxes[l].clear();
        out->lbounded[l].clear();
        if (!used) continue;
        qr_accel_host lv;
        accel_build(d, &lv, l, l == 0 ? NULL : &lv0, bound);
        out->lboxes[l] = lv.boxes;
        out->lbounded[l] = lv.bounded;
        const int i0 = (int)out->items.size();
        anum[l] = (int)lv.always.size();
        r2[l] = (lv.depth < QR_BVH_STACK - 2 && !lv.nodes.empty() &&
                 i0 + lv.items.size() <= (size_t)QR_BVH_MAX_ITEMS) ? lv.ray_r2 : -1.0f;
        if (l == 0)
        {
            for (int k = 0; k < 3; k++) out->ray_c[k] = lv.ray_c[k];
            for (int k = 0; k < 6; k++) out->ext[k] = lv.ext[k];
            out->gain = lv.gain;
            out->ray_r2 = lv.ray_r2;
            out->boxes = lv.boxes;
            out->bounded = lv.bounded;
        }
        out->depth = std::max(out->depth, lv.depth);
        for (size_t k = 0; k < lv.nodes.size(); k++)
        {
            qr_bnode nd = lv.nodes[k];
            if (nd.count > 0) nd.a += i0;
            else { nd.a += n0; nd.b += n0; }
            out->nodes.push_back(nd);
        }
        out->items.insert(out->items.end(), lv.items.begin(), lv.items.end());
        out->always.insert(out->always.end(), lv.always.begin(), lv.always.end());
        if (l == 0) lv0 = lv;
    }
}

void qr_accel_extent(const qr_scene_desc *d, double ext[6])
{
    Extent x;
    scene_extent(d, NULL, x);
    for (int k = 0; k < 3; k++)
    {
        ext[k] = x.clo[k];
        ext[3 + k] = x.chi[k];
    }
}

/* ---- terms of the world boxes that animated records move ------------------ */

/* float bounds that contain [lo, hi] */
static float down(double v)
{
    float f = (float)v;
    return (double)f > v ? nextafterf(f, -HUGE_VALF) : f;
}

static float up(double v)
{
    float f = (float)v;
    return (double)f < v ? nextafterf(f, HUGE_VALF) : f;
}

static void term_local(qr_anim_term &t, int l, const Box &u)
{
    for (int k = 0; k < 3; k++)
    {
        t.u[l][k] = down(u.lo[k]);
        t.u[l][3 + k] = up(u.hi[k]);
    }
}

bool qr_accel_record_frame_d(const qr_srf &t, double a[9])
{
    double m[3][3], r[3][3];
    record_matrix(t, m);
    if (!invert3(m, r)) return false;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) a[3 * i + j] = r[i][j];
    return true;
}

bool qr_accel_record_frame(const qr_srf &t, float a[9])
{
    double r[9];
    if (!qr_accel_record_frame_d(t, r)) return false;
    for (int k = 0; k < 9; k++) a[k] = (float)r[k];
    return true;
}

/* the world_box form for record s in the frame of transform node xf */
static int term_mode(const qr_scene_desc *d, const qr_srf &s, int xf, bool node_only)
{
    if (xf >= 0 && (node_only || d->srf[xf].amap[3] != 0))
        return d->srf[xf].amap[3] != 0 ? QR_TERM_NODE : QR_TERM_NODE_SHIFT;
    return s.amap[3] != 0 ? QR_TERM_OWN : QR_TERM_OWN_SHIFT;
}

int qr_accel_anim_terms(const qr_scene_desc *d, const qr_accel_host *acc,
                        const float *bound, const std::vector<char> &dyn,
                        std::vector<qr_anim_term> &terms,
                        std::vector<qr_anim_target> &targets)
{
    terms.clear();
    targets.clear();
    Extent x;
    scene_extent(d, bound, x);
    double Dl[QR_BVH_LEVELS];
    for (int l = 0; l < QR_BVH_LEVELS; l++)
    {
        double r;
        level_radius(x, l, &r, &Dl[l]);
    }
    for (int i = 0; i < d->nsrf; i++)
    {
        const qr_srf &s = d->srf[i];
        if (s.is_node || x.srf_xf[i] == -2) continue;
        int lv = 0;
        for (int l = 0; l < QR_BVH_LEVELS; l++)
            if (!acc->lbounded[l].empty() && acc->lbounded[l][i]) lv |= 1 << l;
        if (lv == 0) continue;
        const int sx = x.srf_xf[i];
        bool moved = dyn[i] || (sx >= 0 && dyn[sx]);
        qr_anim_target tg;
        tg.srf = i;
        tg.t0 = (int)terms.size();
        tg.levels = lv;

        /* the surface itself */
        qr_anim_term t;
        memset(&t, 0, sizeof(t));
        t.srf = i;
        t.xf = sx;
        t.mode = term_mode(d, s, sx, false);
        for (int l = 0; l < QR_BVH_LEVELS; l++) term_local(t, l, local_surface_box(s, Dl[l]));
        term_local(t, QR_BVH_LEVELS, local_surface_box(s, 0.0));
        terms.push_back(t);

        /* clippers that keep only its inside (as in accel_build) */
        if (s.clip_num > 0)
        {
            std::vector<int> cxf;
            list_groups(d, s.clip_off, s.clip_num, cxf);
            int accm = 0;
            for (int e = 0; e < s.clip_num; e++)
            {
                const qr_elem &el = d->elems[s.clip_off + e];
                if (el.kind == QR_ELM_ACC_ENTER) { accm = 1; continue; }
                if (el.kind == QR_ELM_ACC_LEAVE) { accm = 0; continue; }
                if (el.kind != QR_ELM_SURFACE || accm || el.rel <= 0) continue;
                const qr_srf &c = d->srf[el.ref];
                qr_anim_term ct;
                memset(&ct, 0, sizeof(ct));
                ct.srf = el.ref;
                ct.xf = cxf[e];
                ct.mode = term_mode(d, c, cxf[e], true);
                for (int l = 0; l < QR_BVH_LEVELS; l++)
                    term_local(ct, l, local_clip_region(c, Dl[l]));
                terms.push_back(ct);
                moved = moved || dyn[el.ref] || (cxf[e] >= 0 && dyn[cxf[e]]);
            }
        }
        tg.tn = (int)terms.size() - tg.t0;
        if (moved) targets.push_back(tg);
        else terms.resize(tg.t0);
    }
    return 0;
}

/* ---- the default motion bound of animated scenes ------------------------- */

/* largest singular value of a 3x3 matrix (power iteration on A^T A) */
static double sigma_max(const double a[3][3])
{
    double g[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            g[i][j] = a[0][i] * a[0][j] + a[1][i] * a[1][j] + a[2][i] * a[2][j];
    double v[3] = {1.0, 0.7, 0.4}, lam = 0.0;
    for (int it = 0; it < 64; it++)
    {
        double w[3];
        for (int i = 0; i < 3; i++) w[i] = g[i][0] * v[0] + g[i][1] * v[1] + g[i][2] * v[2];
        const double n = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        if (!(n > 0.0)) return 0.0;
        for (int i = 0; i < 3; i++) v[i] = w[i] / n;
        lam = n;
    }
    /* a little above the estimate: power iteration approaches from below */
    return sqrt(lam) * (1.0 + 1e-6) + 1e-12;
}

/*
 * The default motion bound of qr_scene_anim_init: where moving records and
 * surfaces can be if the
 * animators rotate and never move their transforms' origins.  Along the
 * table (parents first) every entry's origin stays in a ball (c, r) and its
 * linear part has a singular value bound s: an entry of its own keeps its
 * origin, s = |M|; under a parent T the origin is T's origin plus T's linear
 * part applied to a fixed offset, r = r_T + s_T |offset|, s = s_T |P|.  A
 * moving surface stays within its frame's ball widened by s_F times the
 * largest corner of its local box.  The bound holds these balls and the
 * scene's extent; an update that leaves it anyway (an animator that
 * translates) is caught by the update's own check.
 */
void qr_accel_rotation_bound(const qr_scene_desc *d, const qr_anim_node *nodes, int n,
                             float out[6])
{
    Extent x;
    scene_extent(d, NULL, x);
    double lo[3] = {x.clo[0], x.clo[1], x.clo[2]}, hi[3] = {x.chi[0], x.chi[1], x.chi[2]};
    std::vector<double> c(3 * (size_t)n), r(n), sg(n);
    std::vector<int> of_rec(d->nsrf, -1);
    auto grow = [&](const double *cc, double rr) {
        for (int k = 0; k < 3; k++)
        {
            lo[k] = std::min(lo[k], cc[k] - rr);
            hi[k] = std::max(hi[k], cc[k] + rr);
        }
    };
    for (int e = 0; e < n; e++)
    {
        const qr_anim_node &N = nodes[e];
        double P[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) P[i][j] = N.p[4 * j + i];   /* column-major */
        double o[3] = {0.0, 0.0, 0.0};
        double M[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        if (N.rec >= 0)
        {
            const qr_srf &s = d->srf[N.rec];
            float f[9];
            if (qr_accel_record_frame(s, f))
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) M[i][j] = f[3 * i + j];
            for (int k = 0; k < 3; k++) o[k] = s.pos[k];
            of_rec[N.rec] = e;
        }
        else if (N.light >= 0)
        {
            for (int k = 0; k < 3; k++) o[k] = d->lgt[N.light].pos[k];
        }
        if (N.kind == QR_ANIM_OWN)
        {
            for (int k = 0; k < 3; k++) c[3 * e + k] = o[k];
            r[e] = 0.0;
            sg[e] = sigma_max(M);
        }
        else
        {
            const int t = N.parent;
            const qr_srf &T = d->srf[nodes[t].rec >= 0 ? nodes[t].rec : 0];
            /* the offset in T's frame: T's transform rows applied to the
             * origins' difference */
            double q = 0.0;
            const float *row[3] = {T.tci, T.tcj, T.tck};
            for (int i = 0; i < 3; i++)
            {
                double v = 0.0;
                for (int k = 0; k < 3; k++) v += (double)row[i][k] * (o[k] - (double)T.pos[k]);
                q += v * v;
            }
            for (int k = 0; k < 3; k++) c[3 * e + k] = c[3 * t + k];
            r[e] = r[t] + sg[t] * sqrt(q) * (1.0 + 1e-5) + 1e-5;
            sg[e] = sg[t] * sigma_max(P);
        }
        if (N.rec >= 0) grow(&c[3 * e], r[e]);
    }
    /* moving surfaces: their frame's ball and the reach of their local box
     * (without rounding allowance, as the extent has it) */
    for (int i = 0; i < d->nsrf; i++)
    {
        const qr_srf &s = d->srf[i];
        if (s.is_node || x.srf_xf[i] == -2) continue;
        const int sx = x.srf_xf[i];
        const int mode = term_mode(d, s, sx, false);
        const bool node = mode == QR_TERM_NODE || mode == QR_TERM_NODE_SHIFT;
        const int fr = node ? sx : i;
        if (fr < 0 || of_rec[fr] < 0) continue;
        const int e = of_rec[fr];
        const Box u = local_surface_box(s, 0.0);
        double rho = 0.0;
        bool fin = true;
        for (int k = 0; k < 3; k++)
        {
            /* the box in float, rounded outwards, as the terms hold it */
            const double a = down(u.lo[k]), b = up(u.hi[k]);
            const double sh = node ? (double)s.pos[k] : 0.0;
            if (!(a > -HUGE_VAL && b < HUGE_VAL && a <= b)) fin = false;
            const double m = std::max(fabs(a + sh), fabs(b + sh));
            rho += m * m;
        }
        if (!fin) continue;
        grow(&c[3 * e], r[e] + sg[e] * sqrt(rho) * (1.0 + 1e-5) + 1e-5);
    }
    for (int k = 0; k < 3; k++)
    {
        out[k] = (float)lo[k];
        out[3 + k] = (float)hi[k];
    }
}

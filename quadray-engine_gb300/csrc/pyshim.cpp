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
#include "xform.h"
#include "accel.h"
#include "anim_box.h"
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

/* the device update table (Flat::anim_table) into out[cap]; *n receives its
 * length; QR_ERR_LIMIT when cap is short, QR_ERR_STATE (reason in why) when
 * the scene cannot be updated on the device */
int qrpy_flat_anim_table(void *f, qr_anim_node *out, int cap, int *n, char *why, int why_len)
{
    std::vector<qr_anim_node> t;
    std::string reason;
    int rc = ((qr::Flat *)f)->anim_table(t, &reason);
    *n = (int)t.size();
    if (rc != 0)
    {
        if (why != NULL && why_len > 0) snprintf(why, (size_t)why_len, "%s", reason.c_str());
        return QR_ERR_STATE;
    }
    if ((int)t.size() > cap) return QR_ERR_LIMIT;
    if (!t.empty()) memcpy(out, t.data(), sizeof(qr_anim_node) * t.size());
    return QR_OK;
}

/* animators for `time` and the table's transforms (Flat::anim_params) into
 * out[cap]; returns Flat::anim_params' status, or -1 when cap is short */
int qrpy_flat_anim_params(void *f, long long time, qr_anim_param *out, int cap, int *n)
{
    std::vector<qr_anim_param> p;
    int rc = ((qr::Flat *)f)->anim_params((rt_time)time, p);
    *n = (int)p.size();
    if ((int)p.size() > cap) return -1;
    if (!p.empty()) memcpy(out, p.data(), sizeof(qr_anim_param) * p.size());
    return rc;
}

/* the default motion bound of a device update table (lo[3], hi[3]) and the
 * scene extent it is joined with, for host tests of the bound */
void qrpy_rotation_bound(const qr_scene_desc *d, const qr_anim_node *t, int n, float *out)
{
    qr_accel_rotation_bound(d, t, n, out);
}

void qrpy_extent(const qr_scene_desc *d, double *out)
{
    qr_accel_extent(d, out);
}

/* level 0 of the hierarchy of scene d: out[0] surfaces in the tree,
 * out[1] surfaces every ray tests (unbounded, or covering more than a fifth
 * of the bounded extent's area), out[2] nodes */
void qrpy_accel_counts(const qr_scene_desc *d, int *out)
{
    qr_accel_host acc;
    qr_accel_build(d, &acc, 0);
    out[0] = (int)acc.items.size();
    out[1] = (int)acc.always.size();
    out[2] = (int)acc.nodes.size();
}

/* the walk's views of the hierarchy of scene d against its binary tree:
 * per built level, the items a walk of the 4-wide records reaches are
 * those of the binary tree, each once; every slot's box is its source
 * node's and its code the node's (or the record made of it); pairs hold
 * their children's boxes and codes; leaves hold at most QR_BVH_LEAF_MAX
 * items; a level's stack need bounds what its walk pushes.  Returns the
 * number of violations; *levels receives the levels checked */
int qrpy_accel_check(const qr_scene_desc *d, int *levels)
{
    qr_accel_host acc;
    int root[QR_BVH_LEVELS], aoff[QR_BVH_LEVELS], anum[QR_BVH_LEVELS];
    float r2[QR_BVH_LEVELS];
    qr_accel_build_levels(d, &acc, root, aoff, anum, r2, NULL);
    std::vector<qr_bpair> pairs;
    qr_accel_pairs(acc.nodes, pairs);
    std::vector<qr_bquad> quads;
    std::vector<int32_t> src;
    int32_t qroot[QR_BVH_LEVELS], need[QR_BVH_LEVELS];
    qr_accel_quads(acc.nodes, root, QR_BVH_LEVELS, quads, src, qroot, need);
    int bad = 0, nl = 0;
    const int nn = (int)acc.nodes.size();
    for (int i = 0; i < nn; i++)
    {
        const qr_bnode &n = acc.nodes[i];
        if (n.count > 0)
        {
            if (n.count > QR_BVH_LEAF_MAX) bad++;
            continue;
        }
        const qr_bpair &p = pairs[i];
        const qr_bnode &a = acc.nodes[n.a], &b = acc.nodes[n.b];
        for (int k = 0; k < 3; k++)
            if (p.lo_a[k] != a.lo[k] || p.hi_a[k] != a.hi[k] ||
                p.lo_b[k] != b.lo[k] || p.hi_b[k] != b.hi[k]) bad++;
        if (p.code_a != qr_bnode_code(a, n.a) || p.code_b != qr_bnode_code(b, n.b)) bad++;
    }
    for (int l = 0; l < QR_BVH_LEVELS; l++)
    {
        if (r2[l] < 0.0f || root[l] < 0 || root[l] >= nn) continue;
        nl++;
        /* items under the binary tree */
        std::vector<int> want(acc.items.size(), 0), got(acc.items.size(), 0);
        std::vector<int> st(1, root[l]);
        while (!st.empty())
        {
            const int i = st.back();
            st.pop_back();
            const qr_bnode &n = acc.nodes[i];
            if (n.count > 0)
                for (int j = n.a; j < n.a + n.count; j++) want[j]++;
            else { st.push_back(n.a); st.push_back(n.b); }
        }
        /* items the 4-wide walk reaches, with its deepest stack */
        std::vector<std::pair<int32_t, int>> qs(1, std::make_pair(qroot[l], 0));
        int deepest = 0;
        while (!qs.empty())
        {
            const int32_t c = qs.back().first;
            const int depth = qs.back().second;
            qs.pop_back();
            if (c < 0)
            {
                const uint32_t lc = ~(uint32_t)c;
                for (int j = (int)(lc >> 4); j < (int)(lc >> 4) + (int)(lc & 15); j++)
                    if (j >= 0 && j < (int)got.size()) got[j]++; else bad++;
                continue;
            }
            if (c >= (int32_t)quads.size()) { bad++; continue; }
            const qr_bquad &q = quads[c];
            int used = 0;
            for (int k = 0; k < 4; k++)
            {
                const int s = src[4 * (size_t)c + k];
                if (q.code[k] == QR_BQUAD_EMPTY) { if (s != -1) bad++; continue; }
                used++;
                if (s < 0 || s >= nn) { bad++; continue; }
                const qr_bnode &n = acc.nodes[s];
                if (q.lo_x[k] != n.lo[0] || q.lo_y[k] != n.lo[1] || q.lo_z[k] != n.lo[2] ||
                    q.hi_x[k] != n.hi[0] || q.hi_y[k] != n.hi[1] || q.hi_z[k] != n.hi[2]) bad++;
                if (n.count > 0 && q.code[k] != qr_bnode_code(n, s)) bad++;
                if (n.count == 0 && q.code[k] < 0) bad++;
            }
            if (used < 2) bad++;
            deepest = std::max(deepest, depth + used - 1);
            for (int k = 0; k < 4; k++)
                if (q.code[k] != QR_BQUAD_EMPTY)
                    qs.push_back(std::make_pair(q.code[k], depth + used - 1));
        }
        if (deepest > need[l]) bad++;
        for (size_t j = 0; j < want.size(); j++)
            if (want[j] != got[j] || want[j] > 1) bad++;
    }
    if (levels != NULL) *levels = nl;
    return bad;
}

/* the device update's box stage (anim_box.h, the kernel's own float steps)
 * run on the host for the records of scene dt, with the terms and targets
 * taken from scene d0 and its table under the default motion bound;
 * returns how many (surface, level) boxes fail to contain the exact box of
 * the same terms (double arithmetic, no pad), counting a box the float
 * stage refuses (singular or unbounded) a thousand times */
int qrpy_anim_box_check(const qr_scene_desc *d0, const qr_anim_node *table, int n,
                        const qr_scene_desc *dt)
{
    float b[6];
    qr_accel_rotation_bound(d0, table, n, b);
    qr_accel_host acc;
    int root[QR_BVH_LEVELS], aoff[QR_BVH_LEVELS], anum[QR_BVH_LEVELS];
    float r2[QR_BVH_LEVELS];
    qr_accel_build_levels(d0, &acc, root, aoff, anum, r2, b);
    std::vector<char> dyn(d0->nsrf, 0);
    for (int e = 0; e < n; e++)
        if (table[e].rec >= 0) dyn[table[e].rec] = 1;
    std::vector<qr_anim_term> terms;
    std::vector<qr_anim_target> targets;
    qr_accel_anim_terms(d0, &acc, b, dyn, terms, targets);
    std::vector<float> fr((size_t)dt->nsrf * 10);
    for (int i = 0; i < dt->nsrf; i++) qr::record_frame(dt->srf[i], &fr[10 * (size_t)i]);
    int bad = 0;
    for (size_t g = 0; g < targets.size(); g++)
    {
        const qr_anim_target &tg = targets[g];
        for (int l = 0; l < QR_BVH_LEVELS; l++)
        {
            if (((tg.levels >> l) & 1) == 0) continue;
            float fb[6];
            if (!qr::target_box(dt->srf, fr.data(), terms.data(), tg, l, fb))
            {
                bad += 1000;
                continue;
            }
            double lo[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
            double hi[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL};
            for (int j = 0; j < tg.tn; j++)
            {
                const qr_anim_term &t = terms[tg.t0 + j];
                const bool node = t.mode == QR_TERM_NODE || t.mode == QR_TERM_NODE_SHIFT;
                const qr_srf &s = dt->srf[t.srf];
                const qr_srf &F = dt->srf[node ? t.xf : t.srf];
                double v[6];
                for (int k = 0; k < 3; k++)
                {
                    const double sh = node ? (double)s.pos[k] : 0.0;
                    v[k] = (double)t.u[l][k] + sh;
                    v[3 + k] = (double)t.u[l][3 + k] + sh;
                }
                double a[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
                if (t.mode == QR_TERM_NODE || t.mode == QR_TERM_OWN)
                    qr_accel_record_frame_d(F, a);
                for (int i = 0; i < 3; i++)
                {
                    double l0 = F.pos[i], h0 = F.pos[i];
                    for (int k = 0; k < 3; k++)
                    {
                        const double c = a[3 * i + k];
                        if (c == 0.0) continue;
                        const double p = c * v[k], q = c * v[3 + k];
                        l0 += p < q ? p : q;
                        h0 += p < q ? q : p;
                    }
                    if (l0 > lo[i]) lo[i] = l0;
                    if (h0 < hi[i]) hi[i] = h0;
                }
            }
            for (int k = 0; k < 3; k++)
                if (!((double)fb[k] <= lo[k] && (double)fb[3 + k] >= hi[k])) { bad++; break; }
        }
    }
    return bad;
}

/* host restatement of the device update's transform stages (anim.cu stages
 * 1-2, with the same matrix steps of xform.h) applied to table[n] and
 * params, compared with the records and lights of Flat f after its own
 * update; returns how many entries differ in any bit */
int qrpy_anim_check(void *f, const qr_anim_node *table, int n, const qr_anim_param *params)
{
    qr::Flat *fl = (qr::Flat *)f;
    std::vector<float> M(16 * (size_t)(n > 0 ? n : 1));
    int bad = 0;
    for (int e = 0; e < n; e++)
    {
        const qr_anim_node &N = table[e];
        float P[4][4], R[4][4], T[4][4], tmp[4][4], m[4][4], inv[4][4];
        memcpy(P, N.p, sizeof(P));
        memcpy(R, N.r, sizeof(R));
        if (N.param >= 0)
        {
            const float one[3] = {1.0f, 1.0f, 1.0f};
            qr::mat_from_sc(R, params[N.param].sin, params[N.param].cos,
                            params[N.param].pos, one);
        }
        if (N.parent >= 0) memcpy(T, &M[16 * (size_t)N.parent], sizeof(T));
        if (N.kind == QR_ANIM_OWN) qr::mat_mul_mat(m, P, R);
        else if (N.kind == QR_ANIM_UNDER) { qr::mat_mul_mat(tmp, T, P); qr::mat_mul_mat(m, tmp, R); }
        else qr::mat_mul_mat(m, T, P);
        memcpy(&M[16 * (size_t)e], m, sizeof(m));
        bool diff = false;
        if (N.rec >= 0)
        {
            qr::mat_inverse(inv, m);
            const qr_srf &s = fl->srf[N.rec];
            for (int k = 0; k < 3; k++)
            {
                diff |= memcmp(&s.tci[k], &inv[k][0], 4) != 0;
                diff |= memcmp(&s.tcj[k], &inv[k][1], 4) != 0;
                diff |= memcmp(&s.tck[k], &inv[k][2], 4) != 0;
                diff |= memcmp(&s.pos[k], &m[3][k], 4) != 0;
            }
        }
        if (N.light >= 0)
            for (int k = 0; k < 3; k++)
                diff |= memcmp(&fl->lgt[N.light].pos[k], &m[3][k], 4) != 0;
        bad += diff ? 1 : 0;
    }
    return bad;
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

int qrpy_scene_set_device_update(void *h, int on)
{
    return ((qrpy_engine *)h)->scn->set_device_update(on);
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

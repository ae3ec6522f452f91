/*
 * wr_oracle.c — CPU restatement of WalkRay's unidirectional path tracer.
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline); the
 * library never links or calls it.  See wr_oracle.h for what is pinned and
 * how.  Built with -ffp-contract=off.
 *
 * Every function cites the reference code it restates (file:line in the
 * WalkRay tree).
 */
#include "wr_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/walkray.h"

/* macros.h:5-7 */
#define PI_D 3.1415926535897932384626433832795
#define INV_PI_D 0.31830988618379067153776752674503
#define EPS_D 1e-5

/* ========================================================================
 * vec3f with nvVector.h's operation order
 * ====================================================================== */
typedef struct { float x, y, z; } v3;

static inline v3 V3(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vneg(v3 a) { return V3(-a.x, -a.y, -a.z); }
static inline v3 vscale(v3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); } /* vec*T and T*vec */
static inline v3 vmul(v3 a, v3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
/* operator/(vec3, T) leaves the vector unchanged when T == 0 (nvVector.h:376-381) */
static inline v3 vdivs(v3 a, float d) {
    if (d == 0) return a;
    return V3(a.x / d, a.y / d, a.z / d);
}
/* nvVector.h:501-506: r = 0; r += x*x'; r += y*y'; r += z*z' */
static inline float vdot(v3 a, v3 b) {
    float r = 0.f;
    r += a.x * b.x;
    r += a.y * b.y;
    r += a.z * b.z;
    return r;
}
/* nvVector.h:490-499 */
static inline v3 vcross(v3 l, v3 r) { return V3(l.y * r.z - l.z * r.y, l.z * r.x - l.x * r.z, l.x * r.y - l.y * r.x); }
static inline float vlen(v3 a) { return sqrtf(vdot(a, a)); }
/* nvVector.h:522-526 */
static inline v3 vnorm(v3 a) {
    float r = vlen(a);
    if (r > 0) a = vdivs(a, r);
    return a;
}
static inline float vcomp(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
static inline v3 vload(const float* p) { return V3(p[0], p[1], p[2]); }
static inline float fmaxf3(v3 a) { /* *std::max_element over (x, y, z): first maximum */
    float m = a.x;
    if (a.y > m) m = a.y;
    if (a.z > m) m = a.z;
    return m;
}
/* util.h:32-37 */
static inline float luminance(v3 c) { return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z; }
/* MAX(a, EPSILON) with the double literal of macros.h */
static inline float max_eps(float a) { return (double)a > EPS_D ? a : (float)EPS_D; }
/* util.h:8-18 */
static inline int legal_color(v3 c) {
    float a[3] = {c.x, c.y, c.z};
    for (int i = 0; i < 3; i++)
        if (isnan(a[i]) || !isfinite(a[i]) || a[i] < 0) return 0;
    return 1;
}

/* ========================================================================
 * Tree build: KDTree::build(BEST) -> splitBest (kdtree.cpp:141-258)
 * ====================================================================== */
typedef struct {
    int32_t left, right; /* -1 for a leaf */
    float box[6];        /* min xyz, max xyz (BoundingBox, kdtree.cpp:36-40) */
    uint32_t first, count; /* leaf: range in leaf_tris */
} wro_node;

struct wro_tree {
    wro_node* nodes;
    uint32_t n_nodes, cap;
    uint32_t* leaf_tris;
    uint64_t n_leaf_tris, lt_cap;
    const float* v;    /* vertex positions (borrowed) */
    const uint32_t* t; /* triangle vertex indices (borrowed) */
    uint32_t nv, nt;
    /* build scratch */
    uint32_t* stamp;
    uint32_t stamp_id;
    uint32_t* uniq;
    float* coords;
};

static uint32_t tree_alloc(wro_tree* T) {
    if (T->n_nodes == T->cap) {
        T->cap = T->cap ? T->cap * 2 : 1024;
        T->nodes = (wro_node*)realloc(T->nodes, sizeof(wro_node) * T->cap);
    }
    memset(&T->nodes[T->n_nodes], 0, sizeof(wro_node));
    return T->n_nodes++;
}

static void leaf_append(wro_tree* T, const uint32_t* tl, uint32_t cnt, wro_node* nd) {
    if (T->n_leaf_tris + cnt > T->lt_cap) {
        while (T->n_leaf_tris + cnt > T->lt_cap) T->lt_cap = T->lt_cap ? T->lt_cap * 2 : 1024;
        T->leaf_tris = (uint32_t*)realloc(T->leaf_tris, sizeof(uint32_t) * T->lt_cap);
    }
    nd->first = (uint32_t)T->n_leaf_tris;
    nd->count = cnt;
    memcpy(T->leaf_tris + T->n_leaf_tris, tl, sizeof(uint32_t) * cnt);
    T->n_leaf_tris += cnt;
}

/* value at sorted position k (what std::nth_element leaves at begin()+k) */
static float select_kth(float* a, int64_t n, int64_t k) {
    int64_t lo = 0, hi = n - 1;
    while (lo < hi) {
        float x = a[lo], y = a[lo + (hi - lo) / 2], z = a[hi];
        float pivot = (x < y) ? ((y < z) ? y : ((x < z) ? z : x)) : ((x < z) ? x : ((y < z) ? z : y));
        int64_t i = lo, j = hi;
        while (i <= j) {
            while (a[i] < pivot) i++;
            while (a[j] > pivot) j--;
            if (i <= j) {
                float tmp = a[i];
                a[i] = a[j];
                a[j] = tmp;
                i++;
                j--;
            }
        }
        if (k <= j) hi = j;
        else if (k >= i) lo = i;
        else return a[k];
    }
    return a[k];
}

static void build_node(wro_tree* T, uint32_t ni, uint32_t* tl, uint32_t cnt) {
    wro_node* nd = &T->nodes[ni];
    nd->left = nd->right = -1;
    if (cnt == 0) { /* kdtree.cpp:148-149 (box left unset in the reference) */
        nd->first = nd->count = 0;
        return;
    }
    const float* V = T->v;
    const uint32_t* TR = T->t;
    /* bounding box: boundvec<1>/<0> (kdtree.cpp:5-21, 150-164) */
    float mn[3], mx[3];
    {
        const float* p0 = V + 3 * (size_t)TR[3 * (size_t)tl[0]];
        for (int k = 0; k < 3; k++) mn[k] = mx[k] = p0[k];
    }
    for (uint32_t i = 0; i < cnt; i++)
        for (int k = 0; k < 3; k++) {
            const float* p = V + 3 * (size_t)TR[3 * (size_t)tl[i] + k];
            for (int d = 0; d < 3; d++) {
                mn[d] = p[d] < mn[d] ? p[d] : mn[d];
                mx[d] = p[d] > mx[d] ? p[d] : mx[d];
            }
        }
    for (int d = 0; d < 3; d++) {
        nd->box[d] = mn[d];
        nd->box[3 + d] = mx[d];
    }
    /* maxLeafTriangleNum = 1 (kdtree.cpp:24-29, 169-170) */
    if (cnt <= 1) {
        leaf_append(T, tl, cnt, nd);
        return;
    }
    /* the node's distinct vertex indices (the unordered_set, kdtree.cpp:153-163) */
    uint32_t id = ++T->stamp_id, nu = 0;
    for (uint32_t i = 0; i < cnt; i++)
        for (int k = 0; k < 3; k++) {
            uint32_t vi = TR[3 * (size_t)tl[i] + k];
            if (T->stamp[vi] != id) {
                T->stamp[vi] = id;
                T->uniq[nu++] = vi;
            }
        }
    float bestRatio = 10.f, bestSplit = 0.f;
    int bestDim = 0;
    for (int dim = 0; dim < 3; dim++) {
        for (uint32_t k = 0; k < nu; k++) T->coords[k] = V[3 * (size_t)T->uniq[k] + dim];
        float split = select_kth(T->coords, nu, nu >> 1); /* kdtree.cpp:172-182 */
        uint32_t leftCount = 0;
        for (uint32_t i = 0; i < cnt; i++) {
            unsigned mask = 0;
            for (int k = 0; k < 3; k++) mask += (V[3 * (size_t)TR[3 * (size_t)tl[i] + k] + dim] <= split) << k;
            if (mask != 0) leftCount++;
        }
        float ratio = (float)leftCount / (float)cnt;
        /* abs(ratio-0.5) < abs(bestRatio-0.5) evaluated in double (kdtree.cpp:203) */
        if (fabs((double)ratio - 0.5) < fabs((double)bestRatio - 0.5)) {
            bestRatio = ratio;
            bestDim = dim;
            bestSplit = split;
        }
    }
    if (bestRatio == 0 || bestRatio == 1) { /* kdtree.cpp:211-215 */
        leaf_append(T, tl, cnt, nd);
        return;
    }
    /* order-preserving partition: any vertex <= split goes left (kdtree.cpp:220-236) */
    uint32_t* L = (uint32_t*)malloc(sizeof(uint32_t) * cnt);
    uint32_t* R = (uint32_t*)malloc(sizeof(uint32_t) * cnt);
    uint32_t nl = 0, nr = 0;
    for (uint32_t i = 0; i < cnt; i++) {
        unsigned mask = 0;
        for (int k = 0; k < 3; k++) mask += (V[3 * (size_t)TR[3 * (size_t)tl[i] + k] + bestDim] <= bestSplit) << k;
        if (mask == 0) R[nr++] = tl[i];
        else L[nl++] = tl[i];
    }
    uint32_t li = tree_alloc(T);
    T->nodes[ni].left = (int32_t)li;
    build_node(T, li, L, nl);
    free(L);
    uint32_t ri = tree_alloc(T);
    T->nodes[ni].right = (int32_t)ri;
    build_node(T, ri, R, nr);
    free(R);
}

wro_tree* wro_build(const float* verts, uint32_t nv, const uint32_t* tris, uint32_t nt) {
    wro_tree* T = (wro_tree*)calloc(1, sizeof(wro_tree));
    T->v = verts;
    T->t = tris;
    T->nv = nv;
    T->nt = nt;
    T->stamp = (uint32_t*)calloc(nv + 1, sizeof(uint32_t));
    T->uniq = (uint32_t*)malloc(sizeof(uint32_t) * (nv + 1));
    T->coords = (float*)malloc(sizeof(float) * (nv + 1));
    uint32_t* all = (uint32_t*)malloc(sizeof(uint32_t) * (nt + 1));
    for (uint32_t i = 0; i < nt; i++) all[i] = i;
    uint32_t root = tree_alloc(T);
    build_node(T, root, all, nt);
    free(all);
    free(T->stamp);
    free(T->uniq);
    free(T->coords);
    T->stamp = T->uniq = NULL;
    T->coords = NULL;
    return T;
}

void wro_tree_free(wro_tree* T) {
    if (!T) return;
    free(T->nodes);
    free(T->leaf_tris);
    free(T);
}

uint32_t wro_tree_num_nodes(const wro_tree* T) { return T->n_nodes; }

static uint64_t dump_rec(const wro_tree* T, int32_t ni, unsigned char* buf, uint64_t cap, uint64_t off) {
    const wro_node* nd = &T->nodes[ni];
    uint32_t leaf = nd->left < 0 ? 1u : 0u;
    uint32_t cnt = leaf ? nd->count : 0u;
    uint64_t need = 4 + 24 + 4 + 4ull * cnt;
    if (buf && off + need <= cap) {
        memcpy(buf + off, &leaf, 4);
        memcpy(buf + off + 4, nd->box, 24);
        memcpy(buf + off + 28, &cnt, 4);
        if (cnt) memcpy(buf + off + 32, T->leaf_tris + nd->first, 4ull * cnt);
    }
    off += need;
    if (!leaf) {
        off = dump_rec(T, nd->left, buf, cap, off);
        off = dump_rec(T, nd->right, buf, cap, off);
    }
    return off;
}

uint64_t wro_tree_dump(const wro_tree* T, void* buf, uint64_t cap) {
    if (!T->n_nodes) return 0;
    return dump_rec(T, 0, (unsigned char*)buf, cap, 0);
}

/* ========================================================================
 * Traversal
 * ====================================================================== */
/* KDTree::Node::BoundingBox::intersect (kdtree.cpp:46-64): nearest
 * non-negative hit over the six face planes, other two axes checked with
 * inclusive bounds; -1 on a miss. */
static float box_hit(const float* box, v3 o, v3 d) {
    float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    float minDist = -1;
    for (unsigned i = 0; i < 6; i++) {
        unsigned a = i % 3;
        if (dd[a] == 0) continue;
        float dist = (box[i] - oo[a]) / dd[a];
        float p[3];
        for (int k = 0; k < 3; k++) p[k] = oo[k] + dist * dd[k];
        unsigned b = (i + 1) % 3, c = (i + 2) % 3;
        int inter = dist >= 0;
        inter &= box[b] <= p[b];
        inter &= box[3 + b] >= p[b];
        inter &= box[c] <= p[c];
        inter &= box[3 + c] >= p[c];
        minDist = (inter && (dist < minDist || minDist < 0)) ? dist : minDist;
    }
    return minDist;
}

/* KDTree::intersect(ray, tri, cond), geometric part (kdtree.cpp:279-301):
 * edge-function sign masks, then the plane distance along the ray. */
static float tri_hit(v3 v0, v3 v1, v3 v2, v3 o, v3 d) {
    v3 vs[3] = {v0, v1, v2}, lines[3], r2v = V3(0, 0, 0), n;
    unsigned mp = 0, mn = 0;
    for (unsigned i = 0; i < 3; i++) {
        lines[i] = vsub(vs[(i + 1) % 3], vs[i]);
        r2v = vsub(vs[i], o);
        n = vcross(lines[i], r2v);
        float dn = vdot(d, n);
        mp += (dn >= 0) << i;
        mn += (dn <= 0) << i;
    }
    n = vnorm(vcross(lines[0], lines[1]));
    float orthoDist = vdot(n, r2v);
    float dd = vdot(n, d);
    if (dd == 0 || orthoDist / dd < 0 || (mp != 7 && mn != 7)) return -1;
    return orthoDist / dd;
}

/* Mesh::getWorldNormal without vertex normals (mesh.h:47-56): the face normal
 * normalize((v1-v0) x (v2-v0)). */
static inline v3 face_normal(v3 v0, v3 v1, v3 v2) { return vnorm(vcross(vsub(v1, v0), vsub(v2, v0))); }

typedef struct {
    const int32_t* tri_obj;
    int32_t inside, contact; /* object ids, -1 = NULL */
    int filtered;
    uint64_t boxes, tris;
} trace_q;

/* NoSelfCondition::legal (noself.cpp:13-20) */
static int noself_legal(const trace_q* q, int32_t hit_obj, v3 dir, v3 fn) {
    float dd = vdot(dir, fn);
    int in = dd <= 0, out = dd >= 0;
    if (q->inside == q->contact) return !(in && q->contact == hit_obj);
    return !(out && q->inside != hit_obj);
}

/* KDTree::intersect(ray, node, ...) (kdtree.cpp:308-347): descends both
 * children; leaf keeps the first strict minimum; ties between children go
 * to the right child. */
static float node_hit(const wro_tree* T, int32_t ni, v3 o, v3 d, uint32_t* tid, trace_q* q) {
    const wro_node* nd = &T->nodes[ni];
    q->boxes++;
    if (box_hit(nd->box, o, d) < 0) return -1;
    if (nd->left < 0 && nd->right < 0) {
        float minDist = -1;
        for (uint32_t k = 0; k < nd->count; k++) {
            uint32_t ti = T->leaf_tris[nd->first + k];
            const uint32_t* tv = T->t + 3 * (size_t)ti;
            v3 v0 = vload(T->v + 3 * (size_t)tv[0]), v1 = vload(T->v + 3 * (size_t)tv[1]),
               v2 = vload(T->v + 3 * (size_t)tv[2]);
            q->tris++;
            float dist = tri_hit(v0, v1, v2, o, d);
            if (dist >= 0 && q->filtered && !noself_legal(q, q->tri_obj[ti], d, face_normal(v0, v1, v2))) dist = -1;
            if (dist >= 0 && (dist < minDist || minDist < 0)) {
                minDist = dist;
                *tid = ti;
            }
        }
        return minDist;
    }
    uint32_t ltid = 0, rtid = 0;
    float ld = node_hit(T, nd->left, o, d, &ltid, q);
    float rd = node_hit(T, nd->right, o, d, &rtid, q);
    if (ld >= 0 && rd >= 0) {
        *tid = ld < rd ? ltid : rtid;
        return ld < rd ? ld : rd;
    } else if (rd < 0) {
        *tid = ltid;
        return ld;
    } else if (ld < 0) {
        *tid = rtid;
        return rd;
    }
    return -1;
}

static float tree_hit(const wro_tree* T, v3 o, v3 d, uint32_t* tid, trace_q* q) {
    if (!T->n_nodes) return -1;
    return node_hit(T, 0, o, d, tid, q);
}

void wro_trace(const wro_tree* T, const float* rays, uint64_t n, const int32_t* inside, const int32_t* contact,
               const int32_t* tri_obj, uint32_t* out_tri, float* out_t, int nthreads, uint64_t* box_tests,
               uint64_t* tri_tests) {
    uint64_t nb = 0, ntr = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads) reduction(+ : nb, ntr)
#endif
    for (int64_t i = 0; i < (int64_t)n; i++) {
        trace_q q;
        memset(&q, 0, sizeof q);
        q.tri_obj = tri_obj;
        if (inside) {
            q.filtered = 1;
            q.inside = inside[i];
            q.contact = contact[i];
        }
        uint32_t tid = 0xffffffffu;
        float t = tree_hit(T, vload(rays + 6 * i), vload(rays + 6 * i + 3), &tid, &q);
        out_tri[i] = t >= 0 ? tid : 0xffffffffu;
        out_t[i] = t;
        nb += q.boxes;
        ntr += q.tris;
    }
    (void)nthreads;
    if (box_tests) *box_tests = nb;
    if (tri_tests) *tri_tests = ntr;
}

/* ========================================================================
 * Philox4x32-10 (Salmon et al., "Parallel random numbers: as easy as 1, 2,
 * 3", SC'11): two 32x32->64 multiplies per round, Weyl key schedule.
 * ====================================================================== */
void wro_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* Draw `dim` of (pixel, sample): counter {dim/4, sample, pixel, 0}, key =
 * seed; word dim%4; top 24 bits scaled by 2^-24 -> [0, 1). */
float wro_draw(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t dim) {
    uint32_t ctr[4] = {dim >> 2, sample, pixel, 0u}, key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)}, out[4];
    wro_philox4x32_10(ctr, key, out);
    return (float)(out[dim & 3u] >> 8) * (1.0f / 16777216.0f);
}

#include "wr_oracle_pt.inc"
#include "wr_oracle_bpt.inc"
#include "wr_oracle_vcm.inc"
#include "wr_oracle_ppm.inc"

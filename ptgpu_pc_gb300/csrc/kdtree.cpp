// kdtree.cpp -- host KD-tree build with the reference's topology.
//
// KDTree::build (KDTree.cpp:89-182) splits the longest axis of a node's box
// (ties prefer x, then y) at the mean "midpoint" of shapes 1..n-1 (shape 0 is
// skipped), where a triangle's midpoint is p3 / 3 (the comma expression of
// KDTree.cpp:55-57); shapes whose midpoint is <= the mean go right.  A node
// with one shape, or whose split leaves a side empty, is a leaf holding all its
// shapes.  This version keeps that topology exactly but builds iteratively
// with index arrays instead of recursive vector copies, so deep or degenerate
// inputs cannot exhaust the call stack.
#include <cstring>
#include <queue>

#include "host.h"

namespace ptgpu {

namespace {

ptgpu_bound shape_bound(const ptgpu_shape &s) {
    ptgpu_bound b;
    if (s.type == PTGPU_TRIANGLE) {                          // KDTree.cpp:22-34
        const ptgpu_triangle &t = s.g.t;
        auto mn = [](float a, float c) { return a < c ? a : c; };
        auto mx = [](float a, float c) { return a > c ? a : c; };
        b.min_x = mn(mn(t.p1.x, t.p2.x), t.p3.x); b.max_x = mx(mx(t.p1.x, t.p2.x), t.p3.x);
        b.min_y = mn(mn(t.p1.y, t.p2.y), t.p3.y); b.max_y = mx(mx(t.p1.y, t.p2.y), t.p3.y);
        b.min_z = mn(mn(t.p1.z, t.p2.z), t.p3.z); b.max_z = mx(mx(t.p1.z, t.p2.z), t.p3.z);
    } else {                                                   // KDTree.cpp:8-20
        const ptgpu_sphere &sp = s.g.s;
        b.min_x = sp.p.x - sp.rad; b.max_x = sp.p.x + sp.rad;
        b.min_y = sp.p.y - sp.rad; b.max_y = sp.p.y + sp.rad;
        b.min_z = sp.p.z - sp.rad; b.max_z = sp.p.z + sp.rad;
    }
    return b;
}

inline float midpoint_axis(const ptgpu_shape &s, int axis) {
    if (s.type == PTGPU_TRIANGLE) {
        const ptgpu_vec &p3 = s.g.t.p3;
        return (axis == 0 ? p3.x : axis == 1 ? p3.y : p3.z) / 3.0f;
    }
    const ptgpu_vec &p = s.g.s.p;
    return axis == 0 ? p.x : axis == 1 ? p.y : p.z;
}

inline void expand(ptgpu_bound &box, const ptgpu_bound &b) {   // KDTree.h:35-44
    if (b.min_x < box.min_x) box.min_x = b.min_x;
    if (b.min_y < box.min_y) box.min_y = b.min_y;
    if (b.min_z < box.min_z) box.min_z = b.min_z;
    if (b.max_x > box.max_x) box.max_x = b.max_x;
    if (b.max_y > box.max_y) box.max_y = b.max_y;
    if (b.max_z > box.max_z) box.max_z = b.max_z;
}

inline int longest_axis(const ptgpu_bound &b) {                 // KDTree.cpp:72-86
    float xd = b.max_x - b.min_x, yd = b.max_y - b.min_y, zd = b.max_z - b.min_z;
    if (xd >= yd) return xd >= zd ? 0 : 2;
    return yd >= zd ? 1 : 2;
}

struct Item {
    int32_t node;
    int32_t depth;
    std::vector<int32_t> ids;
};

}  // namespace

int kd_build(const ptgpu_shape *shapes, uint32_t n, KdTree &kd) {
    kd = KdTree();
    auto new_node = [&](int32_t depth) {
        kd.leaf.push_back(0); kd.left.push_back(-1); kd.right.push_back(-1);
        kd.depth.push_back(depth); kd.kmin.push_back(0); kd.kmax.push_back(0);
        ptgpu_bound z; std::memset(&z, 0, sizeof(z));
        kd.box.push_back(z);
        if (depth > kd.max_depth) kd.max_depth = depth;
        return (int32_t)kd.leaf.size() - 1;
    };
    std::vector<int32_t> leaf_start, leaf_count;     // per node, into `store`
    std::vector<int32_t> store;
    store.reserve(n);
    std::vector<Item> work;
    {
        Item root;
        root.node = new_node(0);
        root.depth = 0;
        root.ids.resize(n);
        for (uint32_t i = 0; i < n; ++i) root.ids[i] = (int32_t)i;
        work.push_back(std::move(root));
    }
    auto make_leaf = [&](const Item &it) {
        int32_t nd = it.node;
        kd.leaf[nd] = 1;
        if ((int32_t)leaf_start.size() <= nd) { leaf_start.resize(nd + 1, 0); leaf_count.resize(nd + 1, 0); }
        leaf_start[nd] = (int32_t)store.size();
        leaf_count[nd] = (int32_t)it.ids.size();
        store.insert(store.end(), it.ids.begin(), it.ids.end());
        kd.szbuf += (int32_t)it.ids.size();
    };
    std::vector<int32_t> lft, rgt;
    while (!work.empty()) {
        Item it = std::move(work.back());
        work.pop_back();
        const size_t cnt = it.ids.size();
        if (cnt == 0) continue;                        // empty root: box zero, no children
        ptgpu_bound box = shape_bound(shapes[it.ids[0]]);
        if (cnt <= 1) {
            kd.box[it.node] = box;
            make_leaf(it);
            continue;
        }
        const float recp = (float)(1.0 / (double)cnt);
        float mid[3] = {0.f, 0.f, 0.f};
        for (size_t i = 1; i < cnt; ++i) {
            const ptgpu_shape &s = shapes[it.ids[i]];
            expand(box, shape_bound(s));
            for (int a = 0; a < 3; ++a) {
                float m = midpoint_axis(s, a);
                m *= recp;
                mid[a] += m;
            }
        }
        kd.box[it.node] = box;
        const int axis = longest_axis(box);
        lft.clear(); rgt.clear();
        for (size_t i = 0; i < cnt; ++i) {
            if (mid[axis] >= midpoint_axis(shapes[it.ids[i]], axis)) rgt.push_back(it.ids[i]);
            else lft.push_back(it.ids[i]);
        }
        if (lft.size() == cnt || rgt.size() == cnt) {
            make_leaf(it);
            continue;
        }
        Item li, ri;
        li.node = new_node(it.depth + 1);
        ri.node = new_node(it.depth + 1);
        kd.left[it.node] = li.node;
        kd.right[it.node] = ri.node;
        li.depth = ri.depth = it.depth + 1;
        li.ids = lft;
        ri.ids = rgt;
        work.push_back(std::move(ri));
        work.push_back(std::move(li));
    }
    // kn in breadth-first leaf order (KDTree::traverseTree, KDTree.cpp:206-241)
    leaf_start.resize(kd.leaf.size(), 0);
    leaf_count.resize(kd.leaf.size(), 0);
    kd.kn.reserve(kd.szbuf);
    std::queue<int32_t> q;
    if (!kd.leaf.empty()) q.push(0);
    while (!q.empty()) {
        int32_t nd = q.front();
        q.pop();
        if (kd.leaf[nd]) {
            kd.kmin[nd] = (int32_t)kd.kn.size();
            for (int32_t i = 0; i < leaf_count[nd]; ++i) kd.kn.push_back(store[leaf_start[nd] + i]);
            kd.kmax[nd] = (int32_t)kd.kn.size();
        }
        if (kd.left[nd] >= 0) q.push(kd.left[nd]);
        if (kd.right[nd] >= 0) q.push(kd.right[nd]);
    }
    return PTGPU_OK;
}

int kd_heap_size(const KdTree &kd, int64_t *kng_cnt) {
    if (kd.max_depth > 40) { *kng_cnt = -1; return PTGPU_E_RANGE; }
    *kng_cnt = (int64_t)1 << (kd.max_depth + 1);
    return (*kng_cnt > 32768 || kd.szbuf > 32767) ? PTGPU_E_RANGE : PTGPU_OK;
}

int kd_export_heap(const KdTree &kd, ptgpu_kd_node *kng, int64_t kng_cnt, int32_t *kn) {
    int64_t size;
    int st = kd_heap_size(kd, &size);
    if (size < 0 || kng_cnt < size) return PTGPU_E_RANGE;
    std::memset(kng, 0, sizeof(ptgpu_kd_node) * (size_t)size);
    std::vector<int64_t> pos(kd.leaf.size(), 0);
    std::queue<int32_t> q;
    if (!kd.leaf.empty()) { q.push(0); pos[0] = 1; }
    while (!q.empty()) {                            // KDTree::fillNode, KDTree.cpp:184-204
        int32_t nd = q.front();
        q.pop();
        int64_t p = pos[nd];
        ptgpu_kd_node &k = kng[p];
        k.bound = kd.box[nd];
        k.leaf = (int16_t)kd.leaf[nd];
        if (kd.leaf[nd]) { k.min = (int16_t)kd.kmin[nd]; k.max = (int16_t)kd.kmax[nd]; }
        k.nLeft = (int16_t)(2 * p);
        k.nRight = (int16_t)(2 * p + 1);
        k.nParent = (int16_t)(p / 2);
        if (kd.left[nd] >= 0) { pos[kd.left[nd]] = 2 * p; q.push(kd.left[nd]); }
        if (kd.right[nd] >= 0) { pos[kd.right[nd]] = 2 * p + 1; q.push(kd.right[nd]); }
    }
    if (kn && !kd.kn.empty()) std::memcpy(kn, kd.kn.data(), sizeof(int32_t) * kd.kn.size());
    return st;
}

void kd_export_wide(const KdTree &kd, ptgpu_kd_node_wide *nodes) {
    // breadth-first numbering: the heap export's order with its empty slots
    // left out
    const int32_t cnt = kd.node_count();
    if (cnt == 0) return;
    std::vector<int32_t> order;
    std::vector<int32_t> bfs(cnt, -1);
    order.reserve(cnt);
    order.push_back(0);
    bfs[0] = 0;
    for (size_t h = 0; h < order.size(); ++h) {
        const int32_t nd = order[h];
        for (int32_t c : {kd.left[nd], kd.right[nd]})
            if (c >= 0) { bfs[c] = (int32_t)order.size(); order.push_back(c); }
    }
    for (int32_t i = 0; i < (int32_t)order.size(); ++i) {
        const int32_t nd = order[i];
        ptgpu_kd_node_wide &k = nodes[i];
        k.leaf = kd.leaf[nd];
        k.nLeft = kd.left[nd] >= 0 ? bfs[kd.left[nd]] : -1;
        k.nRight = kd.right[nd] >= 0 ? bfs[kd.right[nd]] : -1;
        k.nParent = -1;
        k.bound = kd.box[nd];
        k.min = kd.leaf[nd] ? kd.kmin[nd] : 0;
        k.max = kd.leaf[nd] ? kd.kmax[nd] : 0;
    }
    for (int32_t i = 0; i < (int32_t)order.size(); ++i) {
        if (nodes[i].nLeft >= 0) nodes[nodes[i].nLeft].nParent = i;
        if (nodes[i].nRight >= 0) nodes[nodes[i].nRight].nParent = i;
    }
}

void kd_trace_nodes(const KdTree &kd, std::vector<float> &nodes, int32_t *root_first,
                    int32_t *root_count, float root_box[6]) {
    nodes.clear();
    *root_first = 0;
    *root_count = 0;
    for (int a = 0; a < 6; ++a) root_box[a] = 0.f;
    if (kd.leaf.empty()) return;
    std::memcpy(root_box, &kd.box[0], sizeof(float) * 6);
    if (kd.leaf[0]) {
        *root_first = kd.kmin[0];
        *root_count = kd.kmax[0] - kd.kmin[0];
        return;
    }
    if (kd.left[0] < 0) {          // empty scene
        *root_count = 0;
        return;
    }
    // breadth-first numbering of the internal nodes
    std::vector<int32_t> bfs_id(kd.leaf.size(), -1), order;
    std::queue<int32_t> q;
    q.push(0);
    while (!q.empty()) {
        int32_t nd = q.front();
        q.pop();
        if (kd.leaf[nd]) continue;
        bfs_id[nd] = (int32_t)order.size();
        order.push_back(nd);
        q.push(kd.left[nd]);
        q.push(kd.right[nd]);
    }
    nodes.resize(order.size() * 16);
    for (size_t i = 0; i < order.size(); ++i) {
        int32_t nd = order[i];
        int32_t l = kd.left[nd], r = kd.right[nd];
        const ptgpu_bound &lb = kd.box[l], &rb = kd.box[r];
        float *o = &nodes[i * 16];
        o[0] = lb.min_x; o[1] = lb.max_x; o[2] = lb.min_y; o[3] = lb.max_y;
        o[4] = lb.min_z; o[5] = lb.max_z; o[6] = rb.min_x; o[7] = rb.max_x;
        o[8] = rb.min_y; o[9] = rb.max_y; o[10] = rb.min_z; o[11] = rb.max_z;
        int32_t q3[4];
        q3[0] = kd.leaf[l] ? kd.kmin[l] : bfs_id[l];
        q3[1] = kd.leaf[r] ? kd.kmin[r] : bfs_id[r];
        q3[2] = kd.leaf[l] ? kd.kmax[l] - kd.kmin[l] : 0;
        q3[3] = kd.leaf[r] ? kd.kmax[r] - kd.kmin[r] : 0;
        std::memcpy(o + 12, q3, sizeof(q3));
    }
}

}  // namespace ptgpu

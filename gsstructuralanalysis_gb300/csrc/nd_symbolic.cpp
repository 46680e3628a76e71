// nd_symbolic.cpp -- nested-dissection tree, postorder numbering, fronts and extend-add maps.
#include "nd_symbolic.h"

#include <algorithm>
#include <stdexcept>

namespace klsa {

namespace {

struct Builder {
    NDTree& T;
    const uint8_t* fixed;
    int leaf_max;
    int next_id = 0;

    int build(int i0, int i1, int j0, int j1, int parent) {
        const int p = T.p;
        int idx = (int)T.nodes.size();
        T.nodes.emplace_back();
        {
            NDNode& nd = T.nodes[idx];
            nd.i0 = i0; nd.i1 = i1; nd.j0 = j0; nd.j1 = j1;
            nd.parent = parent;
        }
        int w = i1 - i0, hgt = j1 - j0;
        // split the longer side by a strip p points wide while the box exceeds the leaf size
        bool can_i = w >= p + 2, can_j = hgt >= p + 2;
        bool split_i = false, split_j = false;
        if (std::max(w, hgt) > leaf_max && (can_i || can_j)) {
            if (can_i && (w >= hgt || !can_j)) split_i = true;
            else split_j = true;
        }
        int c0 = -1, c1 = -1, height = 0;
        int si0 = i0, si1 = i1, sj0 = j0, sj1 = j1;
        if (split_i) {
            int mid = i0 + (w - p) / 2;
            si0 = mid; si1 = mid + p;
            c0 = build(i0, mid, j0, j1, idx);
            c1 = build(mid + p, i1, j0, j1, idx);
        } else if (split_j) {
            int mid = j0 + (hgt - p) / 2;
            sj0 = mid; sj1 = mid + p;
            c0 = build(i0, i1, j0, mid, idx);
            c1 = build(i0, i1, mid + p, j1, idx);
        }
        // drop empty children (boxes of zero area cannot occur, but guard anyway)
        NDNode& nd = T.nodes[idx];
        nd.child[0] = c0;
        nd.child[1] = c1;
        for (int c : {c0, c1})
            if (c >= 0) height = std::max(height, T.nodes[c].height + 1);
        nd.height = height;
        nd.si0 = si0; nd.si1 = si1; nd.sj0 = sj0; nd.sj1 = sj1;
        // postorder numbering of own dofs: control points row-major, components interleaved
        nd.own_start = next_id;
        for (int j = sj0; j < sj1; ++j)
            for (int i = si0; i < si1; ++i) {
                int A = j * T.n1 + i;
                for (int c = 0; c < 3; ++c) {
                    size_t full = (size_t)c * T.ncp + A;
                    if (!fixed[full]) T.full2int[full] = next_id++;
                }
            }
        nd.k = next_id - nd.own_start;
        return idx;
    }
};

}  // namespace

int NDTree::local_index(int nd, int id) const {
    const NDNode& n = nodes[nd];
    if (id >= n.own_start && id < n.own_start + n.k) return id - n.own_start;
    auto it = std::lower_bound(n.halo.begin(), n.halo.end(), id);
    if (it == n.halo.end() || *it != id) return -1;
    return n.k + (int)(it - n.halo.begin());
}

double NDTree::factor_flops() const {
    double s = 0;
    for (const NDNode& n : nodes) {
        double k = n.k, f = n.f();
        s += k * f * f - k * k * f + k * k * k / 3.0;
    }
    return s;
}

int64_t NDTree::front_entries() const {
    int64_t s = 0;
    for (const NDNode& n : nodes) s += (int64_t)n.f() * n.f();
    return s;
}

NDTree build_nd_tree(int n1, int n2, int p, const uint8_t* fixed, int leaf_max) {
    if (n1 < 1 || n2 < 1 || p < 1) throw std::invalid_argument("bad grid");
    NDTree T;
    T.n1 = n1; T.n2 = n2; T.p = p; T.ncp = n1 * n2;
    T.full2int.assign(3 * (size_t)T.ncp, -1);
    Builder B{T, fixed, std::max(leaf_max, p + 1)};
    T.nodes.reserve(4 * (size_t)T.ncp / std::max(1, leaf_max * leaf_max) + 16);
    T.root = B.build(0, n1, 0, n2, -1);
    T.nfree = B.next_id;
    T.int2full.assign(T.nfree, -1);
    for (size_t f = 0; f < T.full2int.size(); ++f)
        if (T.full2int[f] >= 0) T.int2full[T.full2int[f]] = (int)f;
    T.node_of.assign(T.nfree, -1);
    for (int nd = 0; nd < (int)T.nodes.size(); ++nd) {
        const NDNode& n = T.nodes[nd];
        for (int id = n.own_start; id < n.own_start + n.k; ++id) T.node_of[id] = nd;
        T.max_height = std::max(T.max_height, n.height);
    }
    // halos: free dofs of control points outside the box within index distance p
    for (NDNode& n : T.nodes) {
        n.halo.clear();
        int a0 = std::max(0, n.i0 - p), a1 = std::min(n1, n.i1 + p);
        int b0 = std::max(0, n.j0 - p), b1 = std::min(n2, n.j1 + p);
        for (int j = b0; j < b1; ++j)
            for (int i = a0; i < a1; ++i) {
                if (i >= n.i0 && i < n.i1 && j >= n.j0 && j < n.j1) continue;
                int A = j * n1 + i;
                for (int c = 0; c < 3; ++c) {
                    int id = T.full2int[(size_t)c * T.ncp + A];
                    if (id >= 0) n.halo.push_back(id);
                }
            }
        std::sort(n.halo.begin(), n.halo.end());
        if (!n.halo.empty() && n.k > 0 && n.halo.front() < n.own_start + n.k)
            throw std::logic_error("nested dissection: halo precedes own dofs");
    }
    // extend-add maps (child halo -> parent front); every child halo id must be in the parent front
    T.parent_map.assign(T.nodes.size(), {});
    for (int nd = 0; nd < (int)T.nodes.size(); ++nd) {
        const NDNode& n = T.nodes[nd];
        if (n.parent < 0) continue;
        std::vector<int>& m = T.parent_map[nd];
        m.resize(n.halo.size());
        for (size_t a = 0; a < n.halo.size(); ++a) {
            int li = T.local_index(n.parent, n.halo[a]);
            if (li < 0) throw std::logic_error("nested dissection: child halo not in parent front");
            m[a] = li;
        }
    }
    return T;
}

}  // namespace klsa

// nd_symbolic.h -- nested-dissection elimination tree of a tensor-product control grid.
//
// The stiffness matrix of a degree-p tensor-product B-spline patch couples two control
// points iff their indices differ by at most p in both directions.  Recursive bisection
// by separator strips p control points wide therefore decouples the two halves exactly,
// so the elimination tree, the fronts and the extend-add maps follow from the grid alone
// (no graph partitioner).  Internal dof numbering = postorder of that tree; the dofs of
// one control point stay consecutive (components interleaved).
#pragma once

#include <cstdint>
#include <vector>

namespace klsa {

struct NDNode {
    int i0, i1, j0, j1;      // box of the subtree (half-open control-point ranges)
    int si0, si1, sj0, sj1;  // own control points (separator strip or the whole leaf box)
    int parent = -1;
    int child[2] = {-1, -1};
    int height = 0;          // 0 for leaves; parent height > child height
    int own_start = 0;       // internal ids [own_start, own_start + k)
    int k = 0;
    std::vector<int> halo;   // internal ids of the front beyond the own dofs, ascending
    int f() const { return k + (int)halo.size(); }
    int h() const { return (int)halo.size(); }
};

struct NDTree {
    int n1 = 0, n2 = 0, p = 0, ncp = 0, nfree = 0;
    std::vector<NDNode> nodes;       // root is nodes[root]
    int root = -1;
    std::vector<int> full2int;       // size 3*ncp (component-blocked full index), -1 = Dirichlet
    std::vector<int> int2full;       // size nfree
    std::vector<int> node_of;        // internal id -> owning node
    int max_height = 0;

    // child halo index -> parent front index, per node (empty for the root)
    std::vector<std::vector<int>> parent_map;

    // front index of internal id `id` in node `nd` (-1 if absent)
    int local_index(int nd, int id) const;
    // flops of the numeric factorisation (k f^2 - k^2 f + k^3/3 per node)
    double factor_flops() const;
    int64_t front_entries() const;  // sum f^2
};

// fixed: 3*ncp mask in the component-blocked full layout (1 = Dirichlet)
NDTree build_nd_tree(int n1, int n2, int p, const uint8_t* fixed, int leaf_max);

}  // namespace klsa

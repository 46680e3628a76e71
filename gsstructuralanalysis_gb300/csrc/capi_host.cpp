// capi_host.cpp -- host-only entry points (no CUDA call): symbolic analysis queries.
#include <cstdint>
#include <cstring>
#include <exception>

#include "../../include/klshell_gb300.h"
#include "nd_symbolic.h"

using namespace klsa;

extern "C" {

int klsa_nd_stats(int n1, int n2, int p, const uint8_t* fixed, int leaf_max, double* out) {
    try {
        NDTree T = build_nd_tree(n1, n2, p, fixed, leaf_max);
        int maxf = 0;
        for (const NDNode& n : T.nodes) maxf = n.f() > maxf ? n.f() : maxf;
        out[0] = (double)T.nodes.size();
        out[1] = (double)T.nfree;
        out[2] = T.factor_flops();
        out[3] = (double)T.front_entries();
        out[4] = (double)T.max_height;
        out[5] = (double)maxf;
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

int klsa_nd_export(int n1, int n2, int p, const uint8_t* fixed, int leaf_max, int32_t* full2int,
                   int32_t* node_info, int32_t* halo_ids, int64_t capacity_nodes, int64_t capacity_halo) {
    try {
        NDTree T = build_nd_tree(n1, n2, p, fixed, leaf_max);
        int64_t nh = 0;
        for (const NDNode& n : T.nodes) nh += n.h();
        if ((int64_t)T.nodes.size() > capacity_nodes || nh > capacity_halo) return -2;
        std::memcpy(full2int, T.full2int.data(), T.full2int.size() * sizeof(int32_t));
        int64_t off = 0;
        for (size_t i = 0; i < T.nodes.size(); ++i) {
            const NDNode& n = T.nodes[i];
            int32_t* r = node_info + 6 * i;
            r[0] = n.own_start; r[1] = n.k; r[2] = n.h(); r[3] = n.parent; r[4] = n.height; r[5] = (int32_t)off;
            std::memcpy(halo_ids + off, n.halo.data(), n.halo.size() * sizeof(int32_t));
            off += n.h();
        }
        return (int)T.nodes.size();
    } catch (const std::exception&) {
        return -1;
    }
}

}  // extern "C"

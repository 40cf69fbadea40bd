// Grouped execution of many independent contraction plans on one stream.
//
// Each plan keeps its own arithmetic form. The group carves one workspace
// into per-plan slices so that all members can be in flight at once and the
// whole group can be captured into one CUDA graph by the caller.
#include <algorithm>
#include <cstring>
#include <vector>

#include "mgb_internal.h"

struct mgb_group_s {
    std::vector<mgb_plan> plans;
    std::vector<const void *> A, B;
    std::vector<void *> C;
    std::vector<uint64_t> ws_off;
    std::vector<int32_t> tiles;
    uint64_t ws_bytes = 0;
};

using namespace mgb;

extern "C" {

int mgb_group_create(mgb_group *group, const mgb_plan *plans, int32_t count, const void *const *A,
                     const void *const *B, void *const *C) {
    if (!group) return fail(MGB_ERR_ARGUMENT, "group output pointer is null");
    *group = nullptr;
    if (count < 0 || (count > 0 && (!plans || !A || !B || !C)))
        return fail(MGB_ERR_ARGUMENT, "group: null arrays");
    auto *g = new mgb_group_s();
    uint64_t off = 0;
    for (int i = 0; i < count; ++i) {
        if (!plans[i] || plans[i]->kind != PlanKind::Contraction) {
            delete g;
            return fail(MGB_ERR_ARGUMENT, "group: member " + std::to_string(i) + " is not a contraction plan");
        }
        g->plans.push_back(plans[i]);
        g->A.push_back(A[i]);
        g->B.push_back(B[i]);
        g->C.push_back(C[i]);
        g->ws_off.push_back(off);
        off += (plans[i]->cp.ws_bytes + 255) & ~uint64_t(255);
    }
    g->tiles.assign(count, -1);
    g->ws_bytes = off;
    *group = g;
    return MGB_OK;
}

int mgb_group_update(mgb_group group, const void *const *A, const void *const *B, void *const *C) {
    if (!group || !A || !B || !C) return fail(MGB_ERR_ARGUMENT, "group: null argument");
    for (size_t i = 0; i < group->plans.size(); ++i) {
        group->A[i] = A[i];
        group->B[i] = B[i];
        group->C[i] = C[i];
    }
    return MGB_OK;
}

int mgb_group_workspace_size(mgb_group group, uint64_t *bytes) {
    if (!group || !bytes) return fail(MGB_ERR_ARGUMENT, "group: null argument");
    *bytes = group->ws_bytes;
    return MGB_OK;
}

int mgb_group_set_tiles(mgb_group group, const int32_t *tile_per_plan) {
    if (!group || !tile_per_plan) return fail(MGB_ERR_ARGUMENT, "group: null argument");
    for (size_t i = 0; i < group->plans.size(); ++i) group->tiles[i] = tile_per_plan[i];
    return MGB_OK;
}

int mgb_group_execute(mgb_group group, void *workspace, uint64_t workspace_bytes, void *stream) {
    if (!group) return fail(MGB_ERR_ARGUMENT, "group: null argument");
    if (workspace_bytes < group->ws_bytes || (group->ws_bytes && !workspace))
        return fail(MGB_ERR_WORKSPACE, "group workspace smaller than mgb_group_workspace_size");
    for (size_t i = 0; i < group->plans.size(); ++i) {
        void *w = group->ws_bytes ? (char *)workspace + group->ws_off[i] : nullptr;
        int st = mgb_contract(group->plans[i], group->A[i], group->B[i], group->C[i], w,
                              group->plans[i]->cp.ws_bytes, stream);
        if (st) return st;
    }
    return MGB_OK;
}

int mgb_group_destroy(mgb_group group) {
    delete group;
    return MGB_OK;
}

}  // extern "C"

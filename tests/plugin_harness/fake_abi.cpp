// TEST INFRASTRUCTURE ONLY: a host-side stand-in for the part of libreaddy_cuda_core.so that the ReaDDy
// plugin's structural topology reactions use, so that the plugin's mapping of ReaDDy's recipes onto the C
// ABI runs without a GPU.  It holds one topology (a chain of three TOPOLOGY particles, ids 10 11 12, types
// 0 0 0, x = 1 2 3), records every rdc_recipe_* call on stdout, and makes rdc_evaluate_topology_reactions call
// each registered reaction's rate function and then its reaction function on that topology.  The plugin's
// other C-ABI calls resolve to stubs that return RDC_OK (generated by the test).
#include <readdy_cuda.h>

#include <cstdio>
#include <vector>

namespace {
struct Registered {
    rdc_topology_rate_fn rate;
    rdc_topology_recipe_fn reaction;
    void *user;
    int type, expect_connected;
};
std::vector<Registered> g_reactions;
int g_dummy;
const uint64_t IDS[3] = {10, 11, 12};
const int64_t EDGES[4] = {0, 1, 1, 2};
}  // namespace

extern "C" {

const char *rdc_last_error(void) { return "fake"; }
const char *rdc_kernel_name(void) { return "CUDA"; }

int rdc_context_create(rdc_context **c, const double *, const int *, double, int, const double *) {
    *c = reinterpret_cast<rdc_context *>(&g_dummy);
    return RDC_OK;
}

int rdc_system_create(rdc_system **s, const rdc_context *, uint64_t) {
    *s = reinterpret_cast<rdc_system *>(&g_dummy);
    g_reactions.clear();
    return RDC_OK;
}

int rdc_add_structural_topology_reaction(rdc_system *, int topology_type, rdc_topology_rate_fn rate,
                                         rdc_topology_recipe_fn reaction, void *user, int expect_connected,
                                         int *reaction_id) {
    g_reactions.push_back({rate, reaction, user, topology_type, expect_connected});
    if (reaction_id) *reaction_id = (int)g_reactions.size() - 1;
    std::printf("register type=%d expect_connected=%d\n", topology_type, expect_connected);
    return RDC_OK;
}

int rdc_get_topology(rdc_system *, int64_t k, int *topology_type, int64_t capacity, uint64_t *ids, int *types,
                     int64_t *n_vertices, int64_t capacity_edges, int64_t *edges2, int64_t *n_edges) {
    if (k != 0) return RDC_ERR_INVALID_ARGUMENT;
    if (topology_type) *topology_type = 0;
    *n_vertices = 3;
    *n_edges = 2;
    if (capacity < 3 || capacity_edges < 2) return RDC_ERR_CAPACITY;
    for (int v = 0; v < 3; ++v) {
        ids[v] = IDS[v];
        types[v] = 0;
    }
    for (int e = 0; e < 4; ++e) edges2[e] = EDGES[e];
    return RDC_OK;
}

int rdc_get_topology_positions(rdc_system *, int64_t k, int64_t capacity, double *positions3) {
    if (k != 0 || capacity < 3) return RDC_ERR_INVALID_ARGUMENT;
    for (int v = 0; v < 3; ++v) {
        positions3[3 * v] = 1.0 + v;
        positions3[3 * v + 1] = 0.0;
        positions3[3 * v + 2] = 0.0;
    }
    return RDC_OK;
}

int rdc_evaluate_topology_reactions(rdc_system *s, double, int64_t *performed) {
    for (const auto &r : g_reactions) {
        std::printf("rate %.6g\n", r.rate(r.user, s, 0));
        rdc_recipe *recipe = reinterpret_cast<rdc_recipe *>(&g_dummy);
        r.reaction(r.user, s, 0, recipe);
    }
    if (performed) *performed = 0;
    return RDC_OK;
}

int rdc_recipe_change_particle_type(rdc_recipe *, int64_t vertex, int type) {
    std::printf("change_particle_type %lld %d\n", (long long)vertex, type);
    return RDC_OK;
}
int rdc_recipe_add_edge(rdc_recipe *, int64_t v1, int64_t v2) {
    std::printf("add_edge %lld %lld\n", (long long)v1, (long long)v2);
    return RDC_OK;
}
int rdc_recipe_remove_edge(rdc_recipe *, int64_t v1, int64_t v2) {
    std::printf("remove_edge %lld %lld\n", (long long)v1, (long long)v2);
    return RDC_OK;
}
int rdc_recipe_separate_vertex(rdc_recipe *, int64_t vertex) {
    std::printf("separate_vertex %lld\n", (long long)vertex);
    return RDC_OK;
}
int rdc_recipe_change_topology_type(rdc_recipe *, int type) {
    std::printf("change_topology_type %d\n", type);
    return RDC_OK;
}
int rdc_recipe_append_particle(rdc_recipe *, int64_t n_neighbors, const int64_t *neighbors, int type,
                               const double *pos3) {
    std::printf("append_particle");
    for (int64_t k = 0; k < n_neighbors; ++k) std::printf(" %lld", (long long)neighbors[k]);
    std::printf(" type %d at %g %g %g\n", type, pos3[0], pos3[1], pos3[2]);
    return RDC_OK;
}
int rdc_recipe_change_particle_position(rdc_recipe *, int64_t vertex, const double *pos3) {
    std::printf("change_particle_position %lld %g %g %g\n", (long long)vertex, pos3[0], pos3[1], pos3[2]);
    return RDC_OK;
}

}  // extern "C"

// TEST INFRASTRUCTURE ONLY: a host-side stand-in for the part of libreaddy_cuda_core.so that the ReaDDy
// plugin calls while it sets a system up and runs structural topology reactions, so that the plugin's
// mapping of ReaDDy's context and recipes onto the C ABI runs without a GPU.
//  * Topology reactions: it holds one topology (a chain of three TOPOLOGY particles, ids 10 11 12, types
//    0 0 0, x = 1 2 3), records every rdc_recipe_* call on stdout, and makes rdc_evaluate_topology_reactions
//    call each registered structural reaction's rate function and then its reaction function on that
//    topology, and each spatial rate function with that topology as both topologies.
//  * Context: after fake_abi_log_context(1) it records every rdc_context_* call with its arguments (doubles
//    in the shortest form that reads back exactly).
//  * System: after fake_abi_log_context(2) it records the state-model, action and observable calls with
//    their arguments instead (particles, topologies with edges, time steps, break pairs, bins).  It keeps
//    the particles and topologies added since the last rdc_system_create and returns them from the
//    particle and topology queries.
// The plugin's other C-ABI calls resolve to stubs that return RDC_OK (generated by the test).
#include <readdy_cuda.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {
struct Registered {
    rdc_topology_rate_fn rate;
    rdc_topology_recipe_fn reaction;
    void *user;
    int type, expect_connected;
};
std::vector<Registered> g_reactions;
struct SpatialFn {
    rdc_spatial_rate_fn rate;
    void *user;
};
std::vector<SpatialFn> g_spatial;  // rate functions of the last context
std::vector<std::string> g_spatial_reactions;  // the spatial reactions of the last context, as logged
int g_dummy;
int g_log_context = 0;  // 1: context calls, 2: system calls
int g_reaction_ids = 0;
uint64_t g_next_id = 100;
// the state of the one system: particles, and topologies as particle ids with id edges
struct Part {
    double x[3];
    int type;
    uint64_t id;
};
struct Top {
    int type;
    std::vector<uint64_t> ids;
    std::vector<uint64_t> edges;
};
std::vector<Part> g_parts;
std::vector<Top> g_tops;

// the shortest %.*g form of x that reads back as x, without an exponent where one of at most 17 digits does
std::string num(double x) {
    char b[40];
    std::string first;
    for (int p = 1; p <= 17; ++p) {
        std::snprintf(b, sizeof b, "%.*g", p, x);
        if (std::strtod(b, nullptr) != x) continue;
        if (!std::strchr(b, 'e')) return b;
        if (first.empty()) first = b;
    }
    return first.empty() ? std::string(b) : first;
}
std::string vec3(const double *v) { return "(" + num(v[0]) + " " + num(v[1]) + " " + num(v[2]) + ")"; }
const uint64_t IDS[3] = {10, 11, 12};
const int64_t EDGES[4] = {0, 1, 1, 2};
}  // namespace

extern "C" {

const char *rdc_last_error(void) { return "fake"; }
const char *rdc_kernel_name(void) { return "CUDA"; }

void fake_abi_log_context(int on) { g_log_context = on; }

int rdc_context_create(rdc_context **c, const double *box, const int *pbc, double kbt, int n_types,
                       const double *D) {
    *c = reinterpret_cast<rdc_context *>(&g_dummy);
    g_reaction_ids = 0;
    g_spatial.clear();
    g_spatial_reactions.clear();
    if (g_log_context == 1) {
        std::printf("context box %s pbc %d %d %d kbt %s D", vec3(box).c_str(), pbc[0], pbc[1], pbc[2], num(kbt).c_str());
        for (int t = 0; t < n_types; ++t) std::printf(" %s", num(D[t]).c_str());
        std::printf("\n");
    }
    return RDC_OK;
}
int rdc_context_set_particle_flavor(rdc_context *, int type, int flavor) {
    if (g_log_context == 1) std::printf("flavor %d %d\n", type, flavor);
    return RDC_OK;
}
int rdc_context_add_spatial_topology_reaction(rdc_context *, int mode, int type1, int topology_type1, int type2,
                                              int topology_type2, int type_to1, int topology_type_to1, int type_to2,
                                              int topology_type_to2, double rate, double radius,
                                              int min_graph_distance, int *reaction_id) {
    char line[256];
    std::snprintf(line, sizeof line, "mode %d %d/%d + %d/%d -> %d/%d + %d/%d rate %s radius %s distance %d", mode,
                  type1, topology_type1, type2, topology_type2, type_to1, topology_type_to1, type_to2,
                  topology_type_to2, num(rate).c_str(), num(radius).c_str(), min_graph_distance);
    if (g_log_context == 1) std::printf("spatial %s\n", line);
    g_spatial_reactions.push_back(line);
    if (reaction_id) *reaction_id = (int)g_spatial_reactions.size() - 1;
    return RDC_OK;
}
int rdc_context_set_spatial_topology_rate_function(rdc_context *, int reaction_id, rdc_spatial_rate_fn rate,
                                                   void *user) {
    if (g_log_context == 1) std::printf("spatial rate function of %s\n", g_spatial_reactions.at(reaction_id).c_str());
    g_spatial.push_back({rate, user});
    return RDC_OK;
}
int rdc_context_set_legacy_topology_self_fusion(rdc_context *, int legacy) {
    if (g_log_context == 1) std::printf("legacy self fusion %d\n", legacy);
    return RDC_OK;
}
int rdc_context_set_record_virial(rdc_context *, int record) {
    if (g_log_context == 1) std::printf("record virial %d\n", record);
    return RDC_OK;
}
int rdc_context_add_harmonic_repulsion(rdc_context *, int t1, int t2, double k, double d) {
    if (g_log_context == 1) std::printf("harmonic repulsion %d %d k %s d %s\n", t1, t2, num(k).c_str(), num(d).c_str());
    return RDC_OK;
}
int rdc_context_add_weak_interaction_piecewise_harmonic(rdc_context *, int t1, int t2, double k, double desired,
                                                        double depth, double cutoff) {
    if (g_log_context == 1)
        std::printf("weak interaction %d %d k %s desired %s depth %s cutoff %s\n", t1, t2, num(k).c_str(), num(desired).c_str(),
                    num(depth).c_str(), num(cutoff).c_str());
    return RDC_OK;
}
int rdc_context_add_lennard_jones(rdc_context *, int t1, int t2, unsigned m, unsigned n, double cutoff, int shift,
                                  double epsilon, double sigma) {
    if (g_log_context == 1)
        std::printf("lennard jones %d %d m %u n %u cutoff %s shift %d epsilon %s sigma %s\n", t1, t2, m, n,
                    num(cutoff).c_str(), shift, num(epsilon).c_str(), num(sigma).c_str());
    return RDC_OK;
}
int rdc_context_add_screened_electrostatics(rdc_context *, int t1, int t2, double strength, double inverse_depth,
                                            double repulsion, double repulsion_distance, unsigned exponent,
                                            double cutoff) {
    if (g_log_context == 1)
        std::printf("screened electrostatics %d %d strength %s kappa %s repulsion %s sigma %s exponent %u cutoff %s\n",
                    t1, t2, num(strength).c_str(), num(inverse_depth).c_str(), num(repulsion).c_str(), num(repulsion_distance).c_str(), exponent,
                    num(cutoff).c_str());
    return RDC_OK;
}
int rdc_context_add_box(rdc_context *, int t, double k, const double *origin, const double *extent, int inclusion) {
    if (g_log_context == 1)
        std::printf("box %d k %s origin %s extent %s inclusion %d\n", t, num(k).c_str(), vec3(origin).c_str(), vec3(extent).c_str(), inclusion);
    return RDC_OK;
}
int rdc_context_add_sphere(rdc_context *, int t, double k, const double *origin, double radius, int inclusion) {
    if (g_log_context == 1)
        std::printf("sphere %d k %s origin %s radius %s inclusion %d\n", t, num(k).c_str(), vec3(origin).c_str(), num(radius).c_str(), inclusion);
    return RDC_OK;
}
int rdc_context_add_capsule(rdc_context *, int t, double k, const double *center, const double *direction,
                            double length, double radius, int inclusion) {
    if (g_log_context == 1)
        std::printf("capsule %d k %s center %s direction %s length %s radius %s inclusion %d\n", t, num(k).c_str(),
                    vec3(center).c_str(), vec3(direction).c_str(), num(length).c_str(), num(radius).c_str(), inclusion);
    return RDC_OK;
}
int rdc_context_add_spherical_barrier(rdc_context *, int t, double height, double width, const double *origin,
                                      double radius) {
    if (g_log_context == 1)
        std::printf("spherical barrier %d height %s width %s origin %s radius %s\n", t, num(height).c_str(), num(width).c_str(),
                    vec3(origin).c_str(), num(radius).c_str());
    return RDC_OK;
}
int rdc_context_add_cylinder(rdc_context *, int t, double k, const double *origin, const double *normal,
                             double radius, int inclusion) {
    if (g_log_context == 1)
        std::printf("cylinder %d k %s origin %s normal %s radius %s inclusion %d\n", t, num(k).c_str(), vec3(origin).c_str(),
                    vec3(normal).c_str(), num(radius).c_str(), inclusion);
    return RDC_OK;
}
int rdc_context_add_conversion(rdc_context *, int from, int to, double rate, int *id) {
    if (g_log_context == 1) std::printf("conversion %d -> %d rate %s\n", from, to, num(rate).c_str());
    if (id) *id = g_reaction_ids++;
    return RDC_OK;
}
int rdc_context_add_decay(rdc_context *, int from, double rate, int *id) {
    if (g_log_context == 1) std::printf("decay %d rate %s\n", from, num(rate).c_str());
    if (id) *id = g_reaction_ids++;
    return RDC_OK;
}
int rdc_context_add_fusion(rdc_context *, int from1, int from2, int to, double rate, double distance, double w1,
                           double w2, int *id) {
    if (g_log_context == 1)
        std::printf("fusion %d + %d -> %d rate %s distance %s weights %s %s\n", from1, from2, to, num(rate).c_str(),
                    num(distance).c_str(), num(w1).c_str(), num(w2).c_str());
    if (id) *id = g_reaction_ids++;
    return RDC_OK;
}
int rdc_context_add_fission(rdc_context *, int from, int to1, int to2, double rate, double distance, double w1,
                            double w2, int *id) {
    if (g_log_context == 1)
        std::printf("fission %d -> %d + %d rate %s distance %s weights %s %s\n", from, to1, to2, num(rate).c_str(),
                    num(distance).c_str(), num(w1).c_str(), num(w2).c_str());
    if (id) *id = g_reaction_ids++;
    return RDC_OK;
}
int rdc_context_add_enzymatic(rdc_context *, int catalyst, int from, int to, double rate, double distance, int *id) {
    if (g_log_context == 1)
        std::printf("enzymatic catalyst %d %d -> %d rate %s distance %s\n", catalyst, from, to, num(rate).c_str(),
                    num(distance).c_str());
    if (id) *id = g_reaction_ids++;
    return RDC_OK;
}
int rdc_context_configure_harmonic_bond(rdc_context *, int t1, int t2, double k, double length) {
    if (g_log_context == 1) std::printf("bond %d %d k %s length %s\n", t1, t2, num(k).c_str(), num(length).c_str());
    return RDC_OK;
}
int rdc_context_configure_harmonic_angle(rdc_context *, int t1, int t2, int t3, double k, double theta0) {
    if (g_log_context == 1) std::printf("angle %d %d %d k %s theta0 %s\n", t1, t2, t3, num(k).c_str(), num(theta0).c_str());
    return RDC_OK;
}
int rdc_context_configure_cosine_dihedral(rdc_context *, int t1, int t2, int t3, int t4, double k,
                                          double multiplicity, double phi0) {
    if (g_log_context == 1)
        std::printf("dihedral %d %d %d %d k %s n %s phi0 %s\n", t1, t2, t3, t4, num(k).c_str(), num(multiplicity).c_str(), num(phi0).c_str());
    return RDC_OK;
}

int rdc_system_create(rdc_system **s, const rdc_context *, uint64_t) {
    *s = reinterpret_cast<rdc_system *>(&g_dummy);
    g_reactions.clear();
    g_parts.clear();
    g_tops.clear();
    if (g_log_context == 2) std::printf("system create\n");
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

int rdc_evaluate_topology_reactions(rdc_system *s, double dt, int64_t *performed) {
    if (g_log_context == 2) std::printf("evaluate topology reactions %s\n", num(dt).c_str());
    for (const auto &r : g_reactions) {
        std::printf("rate %.6g\n", r.rate(r.user, s, 0));
        rdc_recipe *recipe = reinterpret_cast<rdc_recipe *>(&g_dummy);
        r.reaction(r.user, s, 0, recipe);
    }
    for (const auto &f : g_spatial) std::printf("spatial rate %.6g\n", f.rate(f.user, s, 0, 0));
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

int rdc_add_particles(rdc_system *, int64_t n, const double *x, const int *types, uint64_t *ids) {
    for (int64_t i = 0; i < n; ++i) {
        if (g_log_context == 2) std::printf("add particle %s type %d\n", vec3(x + 3 * i).c_str(), types[i]);
        g_parts.push_back({{x[3 * i], x[3 * i + 1], x[3 * i + 2]}, types[i], g_next_id});
        if (ids) ids[i] = g_next_id;
        ++g_next_id;
    }
    return RDC_OK;
}
int rdc_get_n_particles(rdc_system *, int64_t *n) {
    *n = (int64_t)g_parts.size();
    return RDC_OK;
}
int rdc_get_particles(rdc_system *, int64_t capacity, double *x, int *types, uint64_t *ids, int64_t *n_out) {
    const int64_t n = (int64_t)g_parts.size();
    if (n_out) *n_out = n;
    if (capacity < n) return RDC_ERR_CAPACITY;
    for (int64_t i = 0; i < n; ++i) {
        if (x)
            for (int d = 0; d < 3; ++d) x[3 * i + d] = g_parts[i].x[d];
        if (types) types[i] = g_parts[i].type;
        if (ids) ids[i] = g_parts[i].id;
    }
    return RDC_OK;
}
int rdc_get_topologies(rdc_system *, int64_t cap_t, int *types, int64_t *offsets, int64_t cap_i, uint64_t *ids,
                       int64_t *n_t, int64_t *n_i) {
    int64_t ni = 0;
    for (const auto &t : g_tops) ni += (int64_t)t.ids.size();
    *n_t = (int64_t)g_tops.size();
    *n_i = ni;
    if (cap_t < (int64_t)g_tops.size() || cap_i < ni) return RDC_ERR_CAPACITY;
    int64_t at = 0;
    for (std::size_t k = 0; k < g_tops.size(); ++k) {
        if (types) types[k] = g_tops[k].type;
        if (offsets) offsets[k] = at;
        for (uint64_t id : g_tops[k].ids) {
            if (ids) ids[at] = id;
            ++at;
        }
    }
    if (offsets) offsets[g_tops.size()] = at;
    return RDC_OK;
}
int rdc_get_topology_edges(rdc_system *, int64_t cap_t, int64_t *offsets, int64_t cap_e, uint64_t *edges2,
                           int64_t *n_t, int64_t *n_e) {
    int64_t ne = 0;
    for (const auto &t : g_tops) ne += (int64_t)t.edges.size() / 2;
    *n_t = (int64_t)g_tops.size();
    *n_e = ne;
    if (cap_t < (int64_t)g_tops.size() || cap_e < ne) return RDC_ERR_CAPACITY;
    int64_t at = 0;
    for (std::size_t k = 0; k < g_tops.size(); ++k) {
        if (offsets) offsets[k] = at;
        for (std::size_t e = 0; e + 1 < g_tops[k].edges.size(); e += 2) {
            if (edges2) {
                edges2[2 * at] = g_tops[k].edges[e];
                edges2[2 * at + 1] = g_tops[k].edges[e + 1];
            }
            ++at;
        }
    }
    if (offsets) offsets[g_tops.size()] = at;
    return RDC_OK;
}
int rdc_add_topology_typed(rdc_system *, int topology_type, int64_t n, const double *x, const int *types,
                           int64_t n_edges, const int64_t *edges2, uint64_t *ids) {
    if (g_log_context == 2) {
        std::printf("add topology type %d:", topology_type);
        for (int64_t i = 0; i < n; ++i) std::printf(" %s/%d", vec3(x + 3 * i).c_str(), types[i]);
        std::printf(" edges");
        for (int64_t e = 0; e < n_edges; ++e) std::printf(" %lld-%lld", (long long)edges2[2 * e], (long long)edges2[2 * e + 1]);
        std::printf("\n");
    }
    Top top{topology_type, {}, {}};
    for (int64_t i = 0; i < n; ++i) {
        g_parts.push_back({{x[3 * i], x[3 * i + 1], x[3 * i + 2]}, types[i], g_next_id});
        top.ids.push_back(g_next_id);
        if (ids) ids[i] = g_next_id;
        ++g_next_id;
    }
    for (int64_t e = 0; e < n_edges; ++e) {
        top.edges.push_back(top.ids[edges2[2 * e]]);
        top.edges.push_back(top.ids[edges2[2 * e + 1]]);
    }
    g_tops.push_back(std::move(top));
    return RDC_OK;
}
int rdc_break_bonds(rdc_system *, double dt, int n_pairs, const int *t1, const int *t2, const double *thr,
                    const double *rate, int64_t *n_broken) {
    if (g_log_context == 2) {
        std::printf("break bonds dt %s", num(dt).c_str());
        for (int k = 0; k < n_pairs; ++k)
            std::printf(" %d-%d threshold %s rate %s", t1[k], t2[k], num(thr[k]).c_str(), num(rate[k]).c_str());
        std::printf("\n");
    }
    if (n_broken) *n_broken = 0;
    return RDC_OK;
}
int rdc_set_record_virial(rdc_system *, int record) {
    if (g_log_context == 2) std::printf("system record virial %d\n", record);
    return RDC_OK;
}
int rdc_get_virial(rdc_system *, double *virial9) {
    if (g_log_context == 2) std::printf("get virial\n");
    for (int k = 0; k < 9; ++k) virial9[k] = k + 1;
    return RDC_OK;
}
int rdc_initialize(rdc_system *) {
    if (g_log_context == 2) std::printf("initialize\n");
    return RDC_OK;
}
int rdc_nl_create(rdc_system *, double cutoff) {
    if (g_log_context == 2) std::printf("neighbor list create %s\n", num(cutoff).c_str());
    return RDC_OK;
}
int rdc_nl_update(rdc_system *) {
    if (g_log_context == 2) std::printf("neighbor list update\n");
    return RDC_OK;
}
int rdc_nl_clear(rdc_system *) {
    if (g_log_context == 2) std::printf("neighbor list clear\n");
    return RDC_OK;
}
int rdc_calculate_forces(rdc_system *) {
    if (g_log_context == 2) std::printf("calculate forces\n");
    return RDC_OK;
}
int rdc_euler_bd_integrate(rdc_system *, double dt) {
    if (g_log_context == 2) std::printf("euler bd %s\n", num(dt).c_str());
    return RDC_OK;
}
int rdc_uncontrolled_approximation(rdc_system *, double dt) {
    if (g_log_context == 2) std::printf("uncontrolled approximation %s\n", num(dt).c_str());
    return RDC_OK;
}
int rdc_gillespie(rdc_system *, double dt) {
    if (g_log_context == 2) std::printf("gillespie %s\n", num(dt).c_str());
    return RDC_OK;
}
int rdc_get_forces(rdc_system *, int64_t capacity, double *forces3, uint64_t *ids, int64_t *n_out) {
    // particle i's force is (id, -id, 0.5), in storage order
    const int64_t n = (int64_t)g_parts.size();
    if (n_out) *n_out = n;
    if (capacity < n) return RDC_ERR_CAPACITY;
    for (int64_t i = 0; i < n; ++i) {
        if (forces3) {
            forces3[3 * i] = (double)g_parts[i].id;
            forces3[3 * i + 1] = -(double)g_parts[i].id;
            forces3[3 * i + 2] = 0.5;
        }
        if (ids) ids[i] = g_parts[i].id;
    }
    return RDC_OK;
}
int rdc_get_energy(rdc_system *, double *energy) {
    *energy = 42.5;
    return RDC_OK;
}
int rdc_get_reaction_counts(rdc_system *, int n, int64_t *counts) {
    if (g_log_context == 2) std::printf("get reaction counts\n");
    for (int k = 0; k < n; ++k) counts[k] = 100 + k;  // device reaction k performed 100 + k times
    return RDC_OK;
}
int rdc_count_types(rdc_system *, int64_t *counts) {
    if (g_log_context == 2) std::printf("count types\n");
    for (int t = 0; t < 2; ++t) counts[t] = 7 + t;
    return RDC_OK;
}
int rdc_histogram_along_axis(rdc_system *, int n_borders, const double *borders, int n_types, const int *types,
                             int axis, double *counts) {
    if (g_log_context == 2) {
        std::printf("histogram axis %d borders", axis);
        for (int k = 0; k < n_borders; ++k) std::printf(" %s", num(borders[k]).c_str());
        std::printf(" types");
        for (int k = 0; k < n_types; ++k) std::printf(" %d", types[k]);
        std::printf("\n");
    }
    for (int k = 0; k + 1 < n_borders; ++k) counts[k] = k;
    return RDC_OK;
}
int rdc_radial_distribution(rdc_system *, int n_borders, const double *borders, int n_from, const int *from,
                            int n_to, const int *to, double density, double *counts, double *distribution) {
    if (g_log_context == 2) {
        std::printf("radial distribution borders");
        for (int k = 0; k < n_borders; ++k) std::printf(" %s", num(borders[k]).c_str());
        std::printf(" from");
        for (int k = 0; k < n_from; ++k) std::printf(" %d", from[k]);
        std::printf(" to");
        for (int k = 0; k < n_to; ++k) std::printf(" %d", to[k]);
        std::printf(" density %s\n", num(density).c_str());
    }
    for (int k = 0; k + 1 < n_borders; ++k) {
        if (counts) counts[k] = k;
        if (distribution) distribution[k] = 0.5 * k;
    }
    return RDC_OK;
}

}  // extern "C"

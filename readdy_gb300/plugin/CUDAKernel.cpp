// The "CUDA" kernel plugin: each ReaDDy interface method is one call into the C ABI of
// libreaddy_cuda_core.so.  Declarations and the build/installation notes are in CUDAKernel.h.
#include "CUDAKernel.h"

#include <readdy/model/potentials/PotentialsOrder1.h>
#include <readdy/model/potentials/PotentialsOrder2.h>
#include <readdy/model/reactions/Reaction.h>
#include <readdy/model/topologies/reactions/Operations.h>
#include <readdy/model/topologies/reactions/Recipe.h>
#include <readdy/model/topologies/reactions/StructuralTopologyReaction.h>
#include <readdy/model/topologies/reactions/TopologyReactionActionFactory.h>

#include <algorithm>
#include <limits>
#include <map>
#include <cstdlib>
#include <random>
#include <set>
#include <stdexcept>
#include <unordered_map>

namespace readdy::kernel::cuda {

void check(int rc) {
    if (rc == RDC_OK) return;
    const std::string m = rdc_last_error();
    if (rc == RDC_ERR_INVALID_ARGUMENT) throw std::invalid_argument(m);
    if (rc == RDC_ERR_LOGIC) throw std::logic_error(m);
    throw std::runtime_error(m);
}

namespace {

namespace pot = model::potentials;

// Most of ReaDDy's pair and order-1 potential classes keep their parameters as protected members with no
// getters (PotentialsOrder1.h:97-209, PotentialsOrder2.h:54-323).  A class derived from a potential may
// name them, and the pointers-to-member it forms apply to any object of the potential's class, so the
// plugin reads them without a change to ReaDDy's headers.
struct HRAccess : pot::HarmonicRepulsion {
    static constexpr auto forceConstant = &HRAccess::_forceConstant;
    static constexpr auto distance = &HRAccess::_interactionDistance;
};
struct WIPHAccess : pot::WeakInteractionPiecewiseHarmonic {
    static constexpr auto forceConstant = &WIPHAccess::forceConstant;
};
struct LJAccess : pot::LennardJones {
    static constexpr auto m = &LJAccess::m;
    static constexpr auto n = &LJAccess::n;
    static constexpr auto cutoff = &LJAccess::cutoffDistance;
    static constexpr auto shift = &LJAccess::shift;
    static constexpr auto epsilon = &LJAccess::epsilon;
    static constexpr auto sigma = &LJAccess::sigma;
};
struct SEAccess : pot::ScreenedElectrostatics {
    static constexpr auto strength = &SEAccess::electrostaticStrength;
    static constexpr auto inverseDepth = &SEAccess::inverseScreeningDepth;
    static constexpr auto repulsion = &SEAccess::repulsionStrength;
    static constexpr auto repulsionDistance = &SEAccess::repulsionDistance;
    static constexpr auto exponent = &SEAccess::exponent;
    static constexpr auto cutoff = &SEAccess::cutoff;
};
struct BarrierAccess : pot::SphericalBarrier {
    static constexpr auto origin = &BarrierAccess::origin;
    static constexpr auto radius = &BarrierAccess::radius;
    static constexpr auto height = &BarrierAccess::height;
    static constexpr auto width = &BarrierAccess::width;
};
template <bool inclusion>
struct CylinderAccess : pot::Cylinder<inclusion> {
    static constexpr auto origin = &CylinderAccess::origin;
    static constexpr auto normal = &CylinderAccess::normal;
    static constexpr auto forceConstant = &CylinderAccess::forceConstant;
    static constexpr auto radius = &CylinderAccess::radius;
};

// The weak-interaction potential's distances live in a Configuration whose fields only the potential
// itself may read.  Its describe() prints them with {fmt}'s shortest round-trip form, so parsing the
// printed value gives back the exact double (readdy/main/model/potentials/Potentials.cpp:139-144).
double describedValue(const std::string &text, const std::string &label) {
    const auto at = text.find(label);
    if (at == std::string::npos) throw std::invalid_argument("CUDA kernel: cannot read '" + label + "' of: " + text);
    return std::strtod(text.c_str() + at + label.size(), nullptr);
}

void addPairPotential(rdc_context *c, const pot::PotentialOrder2 *p) {
    const int t1 = (int)p->particleType1(), t2 = (int)p->particleType2();
    if (auto *hr = dynamic_cast<const pot::HarmonicRepulsion *>(p)) {
        check(rdc_context_add_harmonic_repulsion(c, t1, t2, hr->*HRAccess::forceConstant, hr->*HRAccess::distance));
    } else if (auto *w = dynamic_cast<const pot::WeakInteractionPiecewiseHarmonic *>(p)) {
        // classified by its class, not by type(), which returns "HarmonicRepulsion" (Potentials.cpp:146-148)
        const std::string d = w->describe();
        check(rdc_context_add_weak_interaction_piecewise_harmonic(c, t1, t2, w->*WIPHAccess::forceConstant,
                                                                  describedValue(d, "desired distance="),
                                                                  describedValue(d, "depth="),
                                                                  describedValue(d, "cutoff=")));
    } else if (auto *lj = dynamic_cast<const pot::LennardJones *>(p)) {
        check(rdc_context_add_lennard_jones(c, t1, t2, (unsigned)(lj->*LJAccess::m), (unsigned)(lj->*LJAccess::n),
                                            lj->*LJAccess::cutoff, lj->*LJAccess::shift ? 1 : 0,
                                            lj->*LJAccess::epsilon, lj->*LJAccess::sigma));
    } else if (auto *se = dynamic_cast<const pot::ScreenedElectrostatics *>(p)) {
        check(rdc_context_add_screened_electrostatics(c, t1, t2, se->*SEAccess::strength, se->*SEAccess::inverseDepth,
                                                      se->*SEAccess::repulsion, se->*SEAccess::repulsionDistance,
                                                      (unsigned)(se->*SEAccess::exponent), se->*SEAccess::cutoff));
    } else {
        throw std::invalid_argument("CUDA kernel: unsupported order-2 potential: " + p->describe());
    }
}

template <bool inclusion>
bool addGeometryPotential(rdc_context *c, int t, const pot::PotentialOrder1 *p) {
    using BoxG = model::geometry::Box<scalar>;
    using SphereG = model::geometry::Sphere<scalar>;
    using CapsuleG = model::geometry::Capsule<scalar>;
    if (auto *b = dynamic_cast<const pot::HarmonicGeometryPotential<BoxG, inclusion> *>(p)) {
        const auto &g = b->geometry();
        const double origin[3] = {g.v0[0], g.v0[1], g.v0[2]};
        const double extent[3] = {g.v1[0] - g.v0[0], g.v1[1] - g.v0[1], g.v1[2] - g.v0[2]};
        check(rdc_context_add_box(c, t, b->forceConstant(), origin, extent, inclusion));
        return true;
    }
    if (auto *s = dynamic_cast<const pot::HarmonicGeometryPotential<SphereG, inclusion> *>(p)) {
        const auto &g = s->geometry();
        const double centre[3] = {g.center[0], g.center[1], g.center[2]};
        check(rdc_context_add_sphere(c, t, s->forceConstant(), centre, g.radius,
                                     inclusion));
        return true;
    }
    if (auto *k = dynamic_cast<const pot::HarmonicGeometryPotential<CapsuleG, inclusion> *>(p)) {
        const auto &g = k->geometry();
        const double centre[3] = {g.center[0], g.center[1], g.center[2]};
        const double dir[3] = {g.direction[0], g.direction[1], g.direction[2]};
        check(rdc_context_add_capsule(c, t, k->forceConstant(), centre, dir,
                                      g.length, g.radius, inclusion));
        return true;
    }
    if (auto *y = dynamic_cast<const pot::Cylinder<inclusion> *>(p)) {
        const Vec3 &o = y->*CylinderAccess<inclusion>::origin, &nrm = y->*CylinderAccess<inclusion>::normal;
        const double origin[3] = {o[0], o[1], o[2]}, normal[3] = {nrm[0], nrm[1], nrm[2]};
        check(rdc_context_add_cylinder(c, t, y->*CylinderAccess<inclusion>::forceConstant, origin, normal,
                                       y->*CylinderAccess<inclusion>::radius, inclusion));
        return true;
    }
    return false;
}

void addExternalPotential(rdc_context *c, const pot::PotentialOrder1 *p) {
    const int t = (int)p->particleType();
    if (addGeometryPotential<true>(c, t, p) || addGeometryPotential<false>(c, t, p)) return;
    if (auto *b = dynamic_cast<const pot::SphericalBarrier *>(p)) {
        const Vec3 &o = b->*BarrierAccess::origin;
        const double origin[3] = {o[0], o[1], o[2]};
        check(rdc_context_add_spherical_barrier(c, t, b->*BarrierAccess::height, b->*BarrierAccess::width, origin,
                                                b->*BarrierAccess::radius));
        return;
    }
    throw std::invalid_argument("CUDA kernel: unsupported order-1 potential: " + p->describe());
}

void addReaction(rdc_context *c, const model::reactions::Reaction *r, std::vector<int> &rx) {
    using RT = model::reactions::ReactionType;
    const auto &e = r->educts();
    const auto &p = r->products();
    int id = -1;
    switch (r->type()) {
        case RT::Conversion: check(rdc_context_add_conversion(c, (int)e[0], (int)p[0], r->rate(), &id)); break;
        case RT::Decay: check(rdc_context_add_decay(c, (int)e[0], r->rate(), &id)); break;
        case RT::Fusion:
            check(rdc_context_add_fusion(c, (int)e[0], (int)e[1], (int)p[0], r->rate(), r->eductDistance(),
                                         r->weight1(), r->weight2(), &id));
            break;
        case RT::Fission:
            check(rdc_context_add_fission(c, (int)e[0], (int)p[0], (int)p[1], r->rate(), r->productDistance(),
                                          r->weight1(), r->weight2(), &id));
            break;
        case RT::Enzymatic:  // educts (from, catalyst), products (to, catalyst) (reactions/Enzymatic.h:53-65)
            check(rdc_context_add_enzymatic(c, (int)e[1], (int)e[0], (int)p[0], r->rate(), r->eductDistance(), &id));
            break;
    }
    if (rx.size() <= r->id()) rx.resize(r->id() + 1, -1);
    rx[r->id()] = id;
}

// the seed of the device's random streams: READDY_CUDA_SEED when set, otherwise a random device draw
uint64_t seedFromEnvironment() {
    if (const char *s = std::getenv("READDY_CUDA_SEED")) return std::strtoull(s, nullptr, 10);
    std::random_device rd;
    return ((uint64_t)rd() << 32) ^ rd();
}

}  // namespace

rdc_context *toDevice(const model::Context &ctx, std::vector<int> &rx,
                      std::vector<std::pair<int, const model::top::reactions::SpatialTopologyReaction *>>
                              *rate_functions) {
    const auto &types = ctx.particleTypes();
    ParticleTypeId maxId = 0;
    for (const auto &[name, id] : types.typeMapping()) maxId = std::max(maxId, id);
    std::vector<double> D(types.nTypes() == 0 ? 1 : (std::size_t)maxId + 1, 0.0);
    for (const auto &[name, id] : types.typeMapping()) D[id] = types.infoOf(id).diffusionConstant;  // ParticleTypeRegistry.h:128-133
    const auto &box = ctx.boxSize();
    const auto &pbc = ctx.periodicBoundaryConditions();
    const double b[3] = {box[0], box[1], box[2]};
    const int p[3] = {pbc[0] ? 1 : 0, pbc[1] ? 1 : 0, pbc[2] ? 1 : 0};
    rdc_context *c = nullptr;
    check(rdc_context_create(&c, b, p, ctx.kBT(), (int)D.size(), D.data()));
    try {
        // flavors (ParticleTypeRegistry.h:58-63): BreakBonds drops one-particle pieces of NORMAL types
        for (const auto &[name, id] : types.typeMapping())
            check(rdc_context_set_particle_flavor(c, (int)id, (int)types.infoOf(id).flavor));
        // spatial topology reactions (TopologyRegistry.h:265-281; each reaction sits in one bucket of the
        // reversal-symmetric map); rate() throws for a reaction with a rate function, which the caller binds
        auto top_id = [](TopologyTypeId t) { return t == EmptyTopologyId ? -1 : (int)t; };
        for (const auto &[key, reactions] : ctx.topologyRegistry().spatialReactionRegistry())
            for (const auto &r : reactions) {
                double rate = 0;
                bool function = false;
                try {
                    rate = r.rate();
                } catch (const std::runtime_error &) {
                    if (!rate_functions)
                        throw std::logic_error("CUDA kernel: a spatial topology reaction with a rate function "
                                               "needs the kernel to bind it");
                    rate = 1.0;  // replaced by the function
                    function = true;
                }
                int id = -1;
                check(rdc_context_add_spatial_topology_reaction(
                        c, (int)r.mode(), (int)r.type1(), top_id(r.top_type1()), (int)r.type2(), top_id(r.top_type2()),
                        (int)r.type_to1(), top_id(r.top_type_to1()), (int)r.type_to2(), top_id(r.top_type_to2()), rate,
                        r.radius(), (int)r.min_graph_distance(), &id));
                if (function) rate_functions->emplace_back(id, &r);
            }
        check(rdc_context_set_legacy_topology_self_fusion(c, ctx.legacyTopologySelfFusion() ? 1 : 0));
        // each unordered type pair once: the registry files a pair's potentials under both orders
        std::set<const pot::PotentialOrder2 *> seen;
        for (const auto &[key, pots] : ctx.potentials().potentialsOrder2())
            for (const auto *q : pots)
                if (seen.insert(q).second) addPairPotential(c, q);
        for (const auto &[type, pots] : ctx.potentials().potentialsOrder1())
            for (const auto *q : pots) addExternalPotential(c, q);
        rx.clear();
        for (const auto *r : ctx.reactions().order1Flat()) addReaction(c, r, rx);
        for (const auto *r : ctx.reactions().order2Flat()) addReaction(c, r, rx);
        // bonded terms of static topologies: TopologyRegistry::potentialConfiguration (PotentialConfiguration.h:136-161)
        const auto &pc = ctx.topologyRegistry().potentialConfiguration();
        for (const auto &[key, bonds] : pc.pairPotentials)
            for (const auto &bd : bonds)
                check(rdc_context_configure_harmonic_bond(c, (int)std::get<0>(key), (int)std::get<1>(key),
                                                          bd.forceConstant, bd.length));
        for (const auto &[key, angles] : pc.anglePotentials)
            for (const auto &a : angles)
                check(rdc_context_configure_harmonic_angle(c, (int)std::get<0>(key), (int)std::get<1>(key),
                                                           (int)std::get<2>(key), a.forceConstant, a.equilibriumAngle));
        for (const auto &[key, torsions] : pc.torsionPotentials)
            for (const auto &d : torsions)
                check(rdc_context_configure_cosine_dihedral(c, (int)std::get<0>(key), (int)std::get<1>(key),
                                                            (int)std::get<2>(key), (int)std::get<3>(key),
                                                            d.forceConstant, d.multiplicity, d.phi_0));
        check(rdc_context_set_record_virial(c, ctx.recordVirial() ? 1 : 0));  // Context.h:168-174
    } catch (...) {
        rdc_context_destroy(c);
        throw;
    }
    return c;
}

// ---- state model ------------------------------------------------------------------------------------

namespace {
struct HostParticles {
    std::vector<double> pos;
    std::vector<int> types;
    std::vector<uint64_t> ids;
};
HostParticles fetch(rdc_system *s) {
    HostParticles h;
    if (!s) return h;
    int64_t n = 0;
    check(rdc_get_n_particles(s, &n));
    h.pos.resize(3 * (std::size_t)n);
    h.types.resize((std::size_t)n);
    h.ids.resize((std::size_t)n);
    int64_t got = 0;
    check(rdc_get_particles(s, n, h.pos.data(), h.types.data(), h.ids.data(), &got));
    h.pos.resize(3 * (std::size_t)got);
    h.types.resize((std::size_t)got);
    h.ids.resize((std::size_t)got);
    return h;
}
}  // namespace

std::vector<Vec3> CUDAStateModel::getParticlePositions() const {
    const auto h = fetch(_kernel->sysIfCreated());
    std::vector<Vec3> out;
    for (std::size_t i = 0; i < h.types.size(); ++i) out.emplace_back(h.pos[3 * i], h.pos[3 * i + 1], h.pos[3 * i + 2]);
    return out;
}

std::vector<model::Particle> CUDAStateModel::getParticles() const {
    const auto h = fetch(_kernel->sysIfCreated());
    std::vector<model::Particle> out;
    for (std::size_t i = 0; i < h.types.size(); ++i)
        out.emplace_back(Vec3(h.pos[3 * i], h.pos[3 * i + 1], h.pos[3 * i + 2]), (ParticleTypeId)h.types[i],
                         (ParticleId)h.ids[i]);
    return out;
}

// the particle whose device id is `index` (topology vertices hold device ids as their particle index)
model::Particle CUDAStateModel::getParticleForIndex(std::size_t index) const {
    if (const auto it = _view.find(index); it != _view.end()) return it->second;
    if (const auto it = _pendingParticles.find(index); it != _pendingParticles.end()) return it->second;
    for (const auto &p : getParticles())
        if (p.id() == index) return p;
    throw std::out_of_range("CUDA kernel: no particle with index " + std::to_string(index));
}

ParticleTypeId CUDAStateModel::getParticleType(std::size_t index) const { return getParticleForIndex(index).type(); }

std::vector<model::Particle> CUDAStateModel::getParticlesForTopology(const model::top::GraphTopology &topology) const {
    std::vector<model::Particle> out;
    for (const auto &p : _pending)  // vertices of a pending topology hold placeholder indices
        if (p.top.get() == &topology) {
            for (const auto &v : topology.graph().vertices())
                if (!v.deactivated()) out.push_back(_pendingParticles.at(v->particleIndex));
            return out;
        }
    const auto h = fetch(_kernel->sysIfCreated());
    std::unordered_map<uint64_t, std::size_t> at;
    for (std::size_t i = 0; i < h.ids.size(); ++i) at[h.ids[i]] = i;
    for (const auto &v : topology.graph().vertices()) {
        if (v.deactivated()) continue;
        const auto it = at.find((uint64_t)v->particleIndex);
        if (it == at.end())
            throw std::out_of_range("CUDA kernel: no particle with index " + std::to_string(v->particleIndex));
        const std::size_t i = it->second;
        out.emplace_back(Vec3(h.pos[3 * i], h.pos[3 * i + 1], h.pos[3 * i + 2]), (ParticleTypeId)h.types[i],
                         (ParticleId)h.ids[i]);
    }
    return out;
}

void CUDAStateModel::initializeNeighborList(scalar cutoff) { check(rdc_nl_create(_kernel->sys(), cutoff)); }
void CUDAStateModel::updateNeighborList() { check(rdc_nl_update(_kernel->sys())); }
void CUDAStateModel::clearNeighborList() { check(rdc_nl_clear(_kernel->sys())); }

void CUDAStateModel::addParticles(const std::vector<model::Particle> &ps) {
    std::vector<double> x(3 * ps.size());
    std::vector<int> t(ps.size());
    for (std::size_t i = 0; i < ps.size(); ++i) {
        for (int d = 0; d < 3; ++d) x[3 * i + d] = ps[i].pos()[d];
        t[i] = (int)ps[i].type();
    }
    check(rdc_add_particles(_kernel->sys(), (int64_t)ps.size(), x.data(), t.data(), nullptr));
}

model::top::GraphTopology *const CUDAStateModel::addTopology(TopologyTypeId type,
                                                            const std::vector<model::Particle> &particles) {
    model::top::Graph graph;
    for (const auto &p : particles) {
        _pendingParticles.emplace(_nextPending, p);
        graph.addVertex(model::top::VertexData{_nextPending++});
    }
    auto top = std::make_unique<model::top::GraphTopology>(type, std::move(graph), _kernel->context(), this);
    auto *raw = top.get();
    _pending.push_back(PendingTopology{std::move(top), particles});
    return raw;
}

void CUDAStateModel::flushTopologies() {
    if (_pending.empty()) return;
    rdc_system *s = _kernel->sysIfCreated();
    if (!s) return;
    for (auto &pt : _pending) {
        auto &g = pt.top->graph();
        const auto n = pt.particles.size();
        std::vector<double> x(3 * n);
        std::vector<int> t(n);
        for (std::size_t i = 0; i < n; ++i) {
            for (int d = 0; d < 3; ++d) x[3 * i + d] = pt.particles[i].pos()[d];
            t[i] = (int)pt.particles[i].type();
        }
        // edges by the vertices' local indices (the position in the list given to addTopology), from their
        // placeholders
        std::unordered_map<std::size_t, int64_t> local;
        for (std::size_t i = 0; i < n; ++i) local[g.vertices().at(model::top::Graph::PersistentVertexIndex{i})->particleIndex] = (int64_t)i;
        std::vector<int64_t> edges;
        for (const auto &[v1, v2] : g.edges()) {
            edges.push_back(local.at(g.vertices().at(v1)->particleIndex));
            edges.push_back(local.at(g.vertices().at(v2)->particleIndex));
        }
        std::vector<uint64_t> ids(n);
        check(rdc_add_topology_typed(s, (int)pt.top->type(), (int64_t)n, x.data(), t.data(),
                                     (int64_t)(edges.size() / 2), edges.data(), ids.data()));
        // from now on a vertex refers to its particle by the device id
        model::top::Graph relabelled;
        for (std::size_t i = 0; i < n; ++i) relabelled.addVertex(model::top::VertexData{(std::size_t)ids[i]});
        for (const auto &[v1, v2] : g.edges())
            relabelled.addEdge(relabelled.vertices().begin_persistent() + local.at(g.vertices().at(v1)->particleIndex),
                               relabelled.vertices().begin_persistent() + local.at(g.vertices().at(v2)->particleIndex));
        for (const auto &[placeholder, i] : local) _pendingParticles.erase(placeholder);
        pt.top->setGraph(std::move(relabelled));
        _topologies.push_back(std::move(pt.top));
    }
    _pending.clear();
}

// the host topologies again from the device's (after BreakBonds split or shrank some): vertices hold
// device ids, edges connect local vertices
void CUDAStateModel::reloadTopologies() {
    rdc_system *s = _kernel->sysIfCreated();
    if (!s) return;
    int64_t nt = 0, ni = 0, ne = 0;
    int st = rdc_get_topologies(s, 0, nullptr, nullptr, 0, nullptr, &nt, &ni);
    if (st != RDC_OK && st != RDC_ERR_CAPACITY) check(st);
    std::vector<int> types(nt);
    std::vector<int64_t> off(nt + 1), eoff(nt + 1);
    std::vector<uint64_t> ids(ni);
    check(rdc_get_topologies(s, nt, types.data(), off.data(), ni, ids.data(), &nt, &ni));
    st = rdc_get_topology_edges(s, 0, nullptr, 0, nullptr, &nt, &ne);
    if (st != RDC_OK && st != RDC_ERR_CAPACITY) check(st);
    std::vector<uint64_t> edges(2 * ne);
    check(rdc_get_topology_edges(s, nt, eoff.data(), ne, edges.data(), &nt, &ne));
    // A topology whose particles are the same as before keeps its host object, with the type and graph the
    // device has now: callers may hold pointers to it (Simulation::addTopology returns one), and the CPU kernel
    // keeps the topologies that reactions left alone.  The others are created anew; vanished ones are dropped.
    std::map<std::vector<std::size_t>, std::unique_ptr<model::top::GraphTopology>> previous;
    for (auto &t : _topologies) {
        std::vector<std::size_t> key;
        for (const auto &v : t->graph().vertices()) key.push_back(v->particleIndex);
        std::sort(key.begin(), key.end());
        previous.emplace(std::move(key), std::move(t));
    }
    _topologies.clear();
    for (int64_t k = 0; k < nt; ++k) {
        model::top::Graph graph;
        std::unordered_map<uint64_t, std::size_t> local;
        std::vector<std::size_t> key;
        for (int64_t v = off[k]; v < off[k + 1]; ++v) {
            local[ids[v]] = (std::size_t)(v - off[k]);
            graph.addVertex(model::top::VertexData{(std::size_t)ids[v]});
            key.push_back((std::size_t)ids[v]);
        }
        for (int64_t e = eoff[k]; e < eoff[k + 1]; ++e)
            graph.addEdge(graph.vertices().begin_persistent() + local.at(edges[2 * e]),
                          graph.vertices().begin_persistent() + local.at(edges[2 * e + 1]));
        std::sort(key.begin(), key.end());
        if (auto it = previous.find(key); it != previous.end()) {
            auto top = std::move(it->second);
            previous.erase(it);
            top->type() = (TopologyTypeId)types[k];
            top->setGraph(std::move(graph));
            _topologies.push_back(std::move(top));
        } else {
            _topologies.push_back(std::make_unique<model::top::GraphTopology>((TopologyTypeId)types[k],
                                                                              std::move(graph), _kernel->context(),
                                                                              this));
        }
    }
}

std::unique_ptr<model::top::GraphTopology> CUDAStateModel::deviceTopology(int64_t k, bool keep_view) {
    rdc_system *s = _kernel->sysIfCreated();
    int type = 0;
    int64_t nv = 0, ne = 0;
    int st = rdc_get_topology(s, k, &type, 0, nullptr, nullptr, &nv, 0, nullptr, &ne);
    if (st != RDC_OK && st != RDC_ERR_CAPACITY) check(st);
    std::vector<uint64_t> ids(nv);
    std::vector<int> types(nv);
    std::vector<int64_t> edges(2 * ne);
    std::vector<double> x(3 * nv);
    check(rdc_get_topology(s, k, &type, nv, ids.data(), types.data(), &nv, ne, edges.data(), &ne));
    check(rdc_get_topology_positions(s, k, nv, x.data()));
    if (!keep_view) _view.clear();
    model::top::Graph graph;
    for (int64_t v = 0; v < nv; ++v) {
        graph.addVertex(model::top::VertexData{(std::size_t)ids[v]});
        _view.emplace((std::size_t)ids[v], model::Particle(Vec3(x[3 * v], x[3 * v + 1], x[3 * v + 2]),
                                                           (ParticleTypeId)types[v], (ParticleId)ids[v]));
    }
    for (int64_t e = 0; e < ne; ++e)
        graph.addEdge(graph.vertices().begin_persistent() + edges[2 * e],
                      graph.vertices().begin_persistent() + edges[2 * e + 1]);
    return std::make_unique<model::top::GraphTopology>((TopologyTypeId)type, std::move(graph), _kernel->context(),
                                                       this);
}

std::vector<model::top::GraphTopology *> CUDAStateModel::getTopologies() {
    std::vector<model::top::GraphTopology *> out;
    for (auto &t : _topologies) out.push_back(t.get());
    for (auto &p : _pending) out.push_back(p.top.get());
    return out;
}

void CUDAStateModel::removeParticle(const model::Particle &) {
    throw std::logic_error("CUDA kernel: removing single particles is not supported (decay reactions remove them)");
}

void CUDAStateModel::removeAllParticles() {
    _pending.clear();
    _pendingParticles.clear();
    _topologies.clear();
    _kernel->dropSystem();
}

CUDAStateModel::Snapshot CUDAStateModel::snapshot() const {
    Snapshot snap;
    rdc_system *s = _kernel->sysIfCreated();
    if (!s) return snap;
    const auto h = fetch(s);
    std::unordered_map<uint64_t, std::size_t> at;  // device id -> index in h
    for (std::size_t i = 0; i < h.ids.size(); ++i) at[h.ids[i]] = i;
    int64_t nt = 0, ni = 0, ne = 0;
    int st = rdc_get_topologies(s, 0, nullptr, nullptr, 0, nullptr, &nt, &ni);
    if (st != RDC_OK && st != RDC_ERR_CAPACITY) check(st);
    std::vector<int> types(nt);
    std::vector<int64_t> off(nt + 1), eoff(nt + 1);
    std::vector<uint64_t> ids(ni);
    if (nt > 0) check(rdc_get_topologies(s, nt, types.data(), off.data(), ni, ids.data(), &nt, &ni));
    st = rdc_get_topology_edges(s, 0, nullptr, 0, nullptr, &nt, &ne);
    if (st != RDC_OK && st != RDC_ERR_CAPACITY) check(st);
    std::vector<uint64_t> edges(2 * ne);
    if (nt > 0) check(rdc_get_topology_edges(s, nt, eoff.data(), ne, edges.data(), &nt, &ne));
    std::vector<char> in_topology(h.ids.size(), 0);
    for (int64_t k = 0; k < nt; ++k) {
        Snapshot::Top top;
        top.type = types[k];
        std::unordered_map<uint64_t, int64_t> local;
        for (int64_t v = off[k]; v < off[k + 1]; ++v) {
            const std::size_t i = at.at(ids[v]);
            in_topology[i] = 1;
            local[ids[v]] = v - off[k];
            for (int d = 0; d < 3; ++d) top.x.push_back(h.pos[3 * i + d]);
            top.t.push_back(h.types[i]);
        }
        for (int64_t e = eoff[k]; e < eoff[k + 1]; ++e) {
            top.edges.push_back(local.at(edges[2 * e]));
            top.edges.push_back(local.at(edges[2 * e + 1]));
        }
        snap.topologies.push_back(std::move(top));
    }
    for (std::size_t i = 0; i < h.ids.size(); ++i)
        if (!in_topology[i])
            snap.free.emplace_back(Vec3(h.pos[3 * i], h.pos[3 * i + 1], h.pos[3 * i + 2]), (ParticleTypeId)h.types[i],
                                   (ParticleId)h.ids[i]);
    return snap;
}

void CUDAStateModel::restore(const Snapshot &snap) {
    rdc_system *s = _kernel->sysIfCreated();
    if (!s) return;
    if (!snap.free.empty()) addParticles(snap.free);
    for (const auto &top : snap.topologies) {
        std::vector<uint64_t> ids(top.t.size());
        check(rdc_add_topology_typed(s, top.type, (int64_t)top.t.size(), top.x.data(), top.t.data(),
                                     (int64_t)(top.edges.size() / 2), top.edges.data(), ids.data()));
    }
    if (!snap.topologies.empty()) reloadTopologies();
}

scalar CUDAStateModel::energy() const {
    double e = 0.0;
    if (_kernel->sysIfCreated()) check(rdc_get_energy(_kernel->sysIfCreated(), &e));
    _energy = e;
    return _energy;
}

scalar &CUDAStateModel::energy() {
    double e = 0.0;
    if (_kernel->sysIfCreated()) check(rdc_get_energy(_kernel->sysIfCreated(), &e));
    _energy = e;
    return _energy;
}

void CUDAStateModel::toDenseParticleIndices(std::vector<std::size_t>::iterator begin,
                                            std::vector<std::size_t>::iterator end) const {
    // device ids -> positions in getParticles()'s order
    const auto h = fetch(_kernel->sysIfCreated());
    std::unordered_map<uint64_t, std::size_t> dense;
    for (std::size_t i = 0; i < h.ids.size(); ++i) dense[h.ids[i]] = i;
    for (auto it = begin; it != end; ++it) *it = dense.at(*it);
}

// ---- actions ----------------------------------------------------------------------------------------

namespace act = model::actions;

namespace {
template <typename Base, typename... Args>
struct CallAction : Base {
    std::function<void()> fn;
    CallAction(std::function<void()> f, Args... args) : Base(args...), fn(std::move(f)) {}
    void perform() override { fn(); }
};
}  // namespace

std::unique_ptr<act::AddParticles> CUDAActionFactory::addParticles(const std::vector<model::Particle> &particles) const {
    return std::make_unique<act::AddParticles>(_kernel, particles);
}
std::unique_ptr<act::EulerBDIntegrator> CUDAActionFactory::eulerBDIntegrator(scalar dt) const {
    auto *k = _kernel;
    return std::make_unique<CallAction<act::EulerBDIntegrator, scalar>>([k, dt] { check(rdc_euler_bd_integrate(k->sys(), dt)); }, dt);
}
std::unique_ptr<act::CalculateForces> CUDAActionFactory::calculateForces() const {
    auto *k = _kernel;
    return std::make_unique<CallAction<act::CalculateForces>>([k] { check(rdc_calculate_forces(k->sys())); });
}
std::unique_ptr<act::CreateNeighborList> CUDAActionFactory::createNeighborList(scalar cutoff) const {
    // the cutoff as the action holds it when performed: SimulationLoop raises it to the context's largest
    // (SimulationLoop.h:266-268) and ReaDDy's Python API adds its skin through the same reference
    struct Create : act::CreateNeighborList {
        CUDAKernel *k;
        Create(CUDAKernel *k, scalar c) : act::CreateNeighborList(c), k(k) {}
        void perform() override { check(rdc_nl_create(k->sys(), cutoffDistance())); }
    };
    return std::make_unique<Create>(_kernel, cutoff);
}
std::unique_ptr<act::UpdateNeighborList> CUDAActionFactory::updateNeighborList() const {
    auto *k = _kernel;
    return std::make_unique<CallAction<act::UpdateNeighborList>>([k] { check(rdc_nl_update(k->sys())); });
}
std::unique_ptr<act::ClearNeighborList> CUDAActionFactory::clearNeighborList() const {
    auto *k = _kernel;
    return std::make_unique<CallAction<act::ClearNeighborList>>([k] { check(rdc_nl_clear(k->sys())); });
}
std::unique_ptr<act::EvaluateCompartments> CUDAActionFactory::evaluateCompartments() const {
    auto *k = _kernel;
    return std::make_unique<CallAction<act::EvaluateCompartments>>([k] {
        if (!k->context().compartments().get().empty())
            throw std::logic_error("CUDA kernel: compartments are not supported");
    });
}
std::unique_ptr<act::reactions::UncontrolledApproximation> CUDAActionFactory::uncontrolledApproximation(scalar dt) const {
    auto *k = _kernel;
    return std::make_unique<CallAction<act::reactions::UncontrolledApproximation, scalar>>(
            [k, dt] { check(rdc_uncontrolled_approximation(k->sys(), dt)); }, dt);
}
std::unique_ptr<act::reactions::Gillespie> CUDAActionFactory::gillespie(scalar dt) const {
    auto *k = _kernel;
    return std::make_unique<CallAction<act::reactions::Gillespie, scalar>>([k, dt] { check(rdc_gillespie(k->sys(), dt)); }, dt);
}
std::unique_ptr<act::reactions::DetailedBalance> CUDAActionFactory::detailedBalance(scalar) const {
    throw std::logic_error("CUDA kernel: the detailed-balance reaction handler is not supported");
}
// EvaluateTopologyReactions (kernels/cpu/src/actions/CPUEvaluateTopologyReactions.cpp): spatial and
// structural reactions run through rdc_evaluate_topology_reactions (the structural ones call back into the
// registry's functions), and the host topologies are read back when any event was performed
std::unique_ptr<act::top::EvaluateTopologyReactions> CUDAActionFactory::evaluateTopologyReactions(scalar dt) const {
    auto *k = _kernel;
    return std::make_unique<CallAction<act::top::EvaluateTopologyReactions, scalar>>([k, dt] {
        const auto &reg = k->context().topologyRegistry();
        if (reg.nStructuralReactions() == 0 && reg.spatialReactionRegistry().empty()) return;
        int64_t performed = 0;
        const int rc = rdc_evaluate_topology_reactions(k->sys(), dt, &performed);
        if (rc == RDC_OK && performed > 0) k->cudaStateModel().reloadTopologies();
        k->rethrowCallbackError();
        check(rc);
    }, dt);
}
// BreakBonds (include/readdy/model/actions/Actions.h:213-290): the break configuration's pairs go to
// rdc_break_bonds; the host topologies are then read back from the device
std::unique_ptr<act::top::BreakBonds> CUDAActionFactory::breakBonds(scalar dt, act::top::BreakConfig config) const {
    struct Break : act::top::BreakBonds {
        CUDAKernel *k;
        Break(CUDAKernel *k, scalar dt, act::top::BreakConfig c) : act::top::BreakBonds(dt, std::move(c)), k(k) {}
        void perform() override {
            std::vector<int> t1, t2;
            std::vector<double> thr, rate;
            for (const auto &[key, e] : thresholdEnergies()) {
                t1.push_back((int)std::get<0>(key));
                t2.push_back((int)std::get<1>(key));
                thr.push_back(e);
                rate.push_back(breakRates().at(key));
            }
            check(rdc_break_bonds(k->sys(), timeStep(), (int)t1.size(), t1.data(), t2.data(), thr.data(), rate.data(),
                                  nullptr));
            k->cudaStateModel().reloadTopologies();
        }
    };
    return std::make_unique<Break>(_kernel, dt, std::move(config));
}
std::unique_ptr<act::EvaluateObservables> CUDAActionFactory::evaluateObservables() const {
    struct Evaluate : act::EvaluateObservables {
        CUDAKernel *k;
        explicit Evaluate(CUDAKernel *k) : k(k) {}
        void perform(TimeStep t) override { k->evaluateObservables(t); }
    };
    return std::make_unique<Evaluate>(_kernel);
}
std::unique_ptr<act::MakeCheckpoint> CUDAActionFactory::makeCheckpoint(std::string, std::size_t) const {
    throw std::logic_error("CUDA kernel: checkpoints are not supported");
}
// InitializeKernel (CPUMiscActions.h:80-89 calls Kernel::initialize, which reads the context again): the
// system keeps its particles and topologies; the one context flag that ReaDDy's observables set after
// particles may have been added, recordVirial, is applied to it here
std::unique_ptr<act::InitializeKernel> CUDAActionFactory::initializeKernel() const {
    auto *k = _kernel;
    return std::make_unique<CallAction<act::InitializeKernel>>([k] {
        check(rdc_set_record_virial(k->sys(), k->context().recordVirial() ? 1 : 0));
        check(rdc_initialize(k->sys()));
    });
}

// ---- observables ------------------------------------------------------------------------------------

namespace obs = model::observables;

namespace {
struct NParticlesCUDA : obs::NParticles {
    CUDAKernel *k;
    NParticlesCUDA(CUDAKernel *k, Stride s, std::vector<std::string> t) : obs::NParticles(k, s, std::move(t)), k(k) {}
    void evaluate() override {  // CPUObservables.cpp:153-171
        const auto nt = (std::size_t)k->context().particleTypes().nTypes();
        std::vector<int64_t> c(std::max<std::size_t>(nt, 1) + 32);
        check(rdc_count_types(k->sys(), c.data()));
        result.clear();
        if (typesToCount.empty()) {
            unsigned long sum = 0;
            for (std::size_t i = 0; i < nt; ++i) sum += (unsigned long)c[i];
            result.push_back(sum);
        } else {
            for (auto t : typesToCount) result.push_back((unsigned long)c[t]);
        }
    }
};

struct ForcesCUDA : obs::Forces {
    CUDAKernel *k;
    ForcesCUDA(CUDAKernel *k, Stride s, std::vector<std::string> t) : obs::Forces(k, s, std::move(t)), k(k) {}
    void evaluate() override {  // CPUObservables.cpp:177-197
        int64_t n = 0;
        check(rdc_get_n_particles(k->sys(), &n));
        std::vector<double> f(3 * (std::size_t)n);
        std::vector<uint64_t> ids((std::size_t)n);
        int64_t got = 0;
        check(rdc_get_forces(k->sys(), n, f.data(), ids.data(), &got));
        std::vector<int> types((std::size_t)n);
        check(rdc_get_particles(k->sys(), n, nullptr, types.data(), nullptr, &got));
        result.clear();
        for (int64_t i = 0; i < got; ++i)
            if (typesToCount.empty() ||
                std::find(typesToCount.begin(), typesToCount.end(), (ParticleTypeId)types[i]) != typesToCount.end())
                result.emplace_back(f[3 * i], f[3 * i + 1], f[3 * i + 2]);
    }
};

struct PositionsCUDA : obs::Positions {
    CUDAKernel *k;
    PositionsCUDA(CUDAKernel *k, Stride s, std::vector<std::string> t) : obs::Positions(k, s, std::move(t)), k(k) {}
    void evaluate() override {
        result.clear();
        for (const auto &p : k->stateModel().getParticles())
            if (typesToCount.empty() ||
                std::find(typesToCount.begin(), typesToCount.end(), p.type()) != typesToCount.end())
                result.push_back(p.pos());
    }
};

struct ParticlesCUDA : obs::Particles {
    CUDAKernel *k;
    ParticlesCUDA(CUDAKernel *k, Stride s) : obs::Particles(k, s), k(k) {}
    void evaluate() override {
        auto &[types, ids, positions] = result;
        types.clear(); ids.clear(); positions.clear();
        for (const auto &p : k->stateModel().getParticles()) {
            types.push_back(p.type());
            ids.push_back(p.id());
            positions.push_back(p.pos());
        }
    }
};

struct HistogramCUDA : obs::HistogramAlongAxis {
    CUDAKernel *k;
    unsigned axis_;
    HistogramCUDA(CUDAKernel *k, Stride s, std::vector<scalar> b, std::vector<std::string> t, unsigned axis)
        : obs::HistogramAlongAxis(k, s, std::move(b), std::move(t), axis), k(k), axis_(axis) {}
    void evaluate() override {  // CPUObservables.cpp:85-146
        std::vector<int> types(typesToCount.begin(), typesToCount.end());
        result.assign(binBorders.size() - 1, 0);
        check(rdc_histogram_along_axis(k->sys(), (int)binBorders.size(), binBorders.data(), (int)types.size(),
                                       types.data(), (int)axis_, result.data()));
    }
};

struct RadialDistributionCUDA : obs::RadialDistribution {
    CUDAKernel *k;
    RadialDistributionCUDA(CUDAKernel *k, Stride s, std::vector<scalar> b, std::vector<std::string> from,
                           std::vector<std::string> to, scalar density)
        : obs::RadialDistribution(k, s, b, from, to, density), k(k) {}
    void evaluate() override {  // RadialDistribution.cpp:75-128, evaluated on the device
        std::vector<int> from(typeCountFrom.begin(), typeCountFrom.end()), to(typeCountTo.begin(), typeCountTo.end());
        auto &[centers, distribution] = result;
        distribution.assign(binBorders.size() - 1, 0);
        counts.assign(binBorders.size() - 1, 0);
        check(rdc_radial_distribution(k->sys(), (int)binBorders.size(), binBorders.data(), (int)from.size(), from.data(),
                                      (int)to.size(), to.data(), particleToDensity, counts.data(), distribution.data()));
    }
};

struct ReactionCountsCUDA : obs::ReactionCounts {
    CUDAKernel *k;
    ReactionCountsCUDA(CUDAKernel *k, Stride s) : obs::ReactionCounts(k, s), k(k) {}
    void evaluate() override {  // CPUStateModel.cpp:126-144
        const auto &rx = k->reactionIds();
        std::vector<int64_t> c(rx.size() + 1, 0);
        check(rdc_get_reaction_counts(k->sys(), (int)c.size(), c.data()));
        auto &counts = std::get<0>(result);
        counts.clear();
        for (std::size_t rid = 0; rid < rx.size(); ++rid)
            if (rx[rid] >= 0) counts[(ReactionId)rid] = (std::size_t)c[(std::size_t)rx[rid]];
    }
};

struct VirialCUDA : obs::Virial {
    CUDAKernel *k;
    VirialCUDA(CUDAKernel *k, Stride s) : obs::Virial(k, s), k(k) {}
    void evaluate() override {
        double v[9];
        check(rdc_get_virial(k->sys(), v));
        result = Matrix33{{{v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8]}}};
    }
};
}  // namespace

CUDAObservableFactory::CUDAObservableFactory(CUDAKernel *kernel) : obs::ObservableFactory(kernel), _kernel(kernel) {}

std::unique_ptr<obs::Energy> CUDAObservableFactory::energy(Stride s, ObsCallback<obs::Energy> cb) const {
    auto o = std::make_unique<obs::Energy>(_kernel, s);  // evaluates StateModel::energy()
    o->setCallback(cb);
    return o;
}
std::unique_ptr<obs::Virial> CUDAObservableFactory::virial(Stride s, ObsCallback<obs::Virial> cb) const {
    auto o = std::make_unique<VirialCUDA>(_kernel, s);
    o->setCallback(cb);
    _kernel->context().recordVirial() = true;
    if (auto *sys = _kernel->sysIfCreated()) check(rdc_set_record_virial(sys, 1));
    return o;
}
std::unique_ptr<obs::HistogramAlongAxis>
CUDAObservableFactory::histogramAlongAxis(Stride s, std::vector<scalar> b, std::vector<std::string> t, unsigned int axis,
                                          ObsCallback<obs::HistogramAlongAxis> cb) const {
    auto o = std::make_unique<HistogramCUDA>(_kernel, s, std::move(b), std::move(t), axis);
    o->setCallback(cb);
    return o;
}
std::unique_ptr<obs::NParticles>
CUDAObservableFactory::nParticles(Stride s, std::vector<std::string> t, ObsCallback<obs::NParticles> cb) const {
    auto o = std::make_unique<NParticlesCUDA>(_kernel, s, std::move(t));
    o->setCallback(cb);
    return o;
}
std::unique_ptr<obs::Forces>
CUDAObservableFactory::forces(Stride s, std::vector<std::string> t, ObsCallback<obs::Forces> cb) const {
    auto o = std::make_unique<ForcesCUDA>(_kernel, s, std::move(t));
    o->setCallback(cb);
    return o;
}
std::unique_ptr<obs::Positions>
CUDAObservableFactory::positions(Stride s, std::vector<std::string> t, ObsCallback<obs::Positions> cb) const {
    auto o = std::make_unique<PositionsCUDA>(_kernel, s, std::move(t));
    o->setCallback(cb);
    return o;
}
std::unique_ptr<obs::RadialDistribution>
CUDAObservableFactory::radialDistribution(Stride s, std::vector<scalar> b, std::vector<std::string> from,
                                          std::vector<std::string> to, scalar density,
                                          ObsCallback<obs::RadialDistribution> cb) const {
    auto o = std::make_unique<RadialDistributionCUDA>(_kernel, s, std::move(b), std::move(from), std::move(to), density);
    o->setCallback(cb);
    return o;
}
std::unique_ptr<obs::Particles> CUDAObservableFactory::particles(Stride s, ObsCallback<obs::Particles> cb) const {
    auto o = std::make_unique<ParticlesCUDA>(_kernel, s);
    o->setCallback(cb);
    return o;
}
std::unique_ptr<obs::Reactions> CUDAObservableFactory::reactions(Stride, ObsCallback<obs::Reactions>) const {
    throw std::logic_error("CUDA kernel: the Reactions observable (records with positions) is not supported");
}
std::unique_ptr<obs::ReactionCounts> CUDAObservableFactory::reactionCounts(Stride s, ObsCallback<obs::ReactionCounts> cb) const {
    auto o = std::make_unique<ReactionCountsCUDA>(_kernel, s);
    o->setCallback(cb);
    _kernel->context().recordReactionCounts() = true;
    return o;
}

// ---- topology action factory ----------------------------------------------------------------------

namespace {
[[noreturn]] void noHostTopologyAction() {
    throw std::logic_error("CUDA kernel: bonded terms, BreakBonds and topology reactions are evaluated on the "
                           "device; per-topology host actions are not provided");
}
}  // namespace

std::unique_ptr<model::top::pot::CalculateHarmonicBondPotential>
CUDATopologyActionFactory::createCalculateHarmonicBondPotential(const harmonic_bond *) const {
    noHostTopologyAction();
}
std::unique_ptr<model::top::pot::CalculateHarmonicAnglePotential>
CUDATopologyActionFactory::createCalculateHarmonicAnglePotential(const harmonic_angle *) const {
    noHostTopologyAction();
}
std::unique_ptr<model::top::pot::CalculateCosineDihedralPotential>
CUDATopologyActionFactory::createCalculateCosineDihedralPotential(const cos_dihedral *) const {
    noHostTopologyAction();
}
CUDATopologyActionFactory::ActionPtr CUDATopologyActionFactory::createChangeParticleType(
        model::top::GraphTopology *, const model::top::Graph::PersistentVertexIndex &, const ParticleTypeId &) const {
    noHostTopologyAction();
}
CUDATopologyActionFactory::ActionPtr CUDATopologyActionFactory::createChangeParticlePosition(
        model::top::GraphTopology *, const model::top::Graph::PersistentVertexIndex &, Vec3) const {
    noHostTopologyAction();
}
CUDATopologyActionFactory::ActionPtr CUDATopologyActionFactory::createAppendParticle(
        model::top::GraphTopology *, const std::vector<model::top::Graph::PersistentVertexIndex> &, ParticleTypeId,
        const Vec3 &) const {
    noHostTopologyAction();
}
CUDATopologyActionFactory::ActionPtr CUDATopologyActionFactory::createChangeTopologyType(model::top::GraphTopology *,
                                                                                         const std::string &) const {
    noHostTopologyAction();
}

// ---- kernel -----------------------------------------------------------------------------------------

CUDAKernel::CUDAKernel() : model::Kernel("CUDA"), _state(this), _actions(this), _observables(this) {}

CUDAKernel::~CUDAKernel() {
    if (_sys) rdc_system_destroy(_sys);
    if (_ctx) rdc_context_destroy(_ctx);
}

// Kernel::initialize (CPUKernel.cpp:63-83): a device context from the current model::Context and a fresh
// system; particles added before are kept (read back and added to the new system)
void CUDAKernel::initialize() {
    model::Kernel::initialize();
    CUDAStateModel::Snapshot keep;
    if (_sys) keep = _state.snapshot();
    std::vector<std::pair<int, const model::top::reactions::SpatialTopologyReaction *>> functions;
    rdc_context *c = toDevice(context(), _rx, &functions);
    // the new context's rate functions: bound here, kept once the old system (which uses the old ones) is gone
    std::vector<std::unique_ptr<SpatialBinding>> spatial;
    try {
        spatial = bindSpatialRateFunctions(c, functions);
    } catch (...) {
        rdc_context_destroy(c);
        throw;
    }
    rdc_system *s = nullptr;
    const int rc = rdc_system_create(&s, c, seedFromEnvironment());
    if (rc != RDC_OK) {
        rdc_context_destroy(c);
        check(rc);
    }
    if (_sys) rdc_system_destroy(_sys);
    if (_ctx) rdc_context_destroy(_ctx);
    _ctx = c;
    _sys = s;
    _spatial = std::move(spatial);
    registerStructuralReactions();
    _state.restore(keep);
    check(rdc_initialize(_sys));
}

void CUDAKernel::dropSystem() {
    if (_sys) rdc_system_destroy(_sys);
    _sys = nullptr;
}

namespace {

namespace rop = model::top::reactions::op;
namespace ract = model::top::reactions::actions;

// A recipe's steps (Recipe.h) hand their data only to the action factory that Operation::create_action
// (Operations.h) is given.  This factory passes each step on to the rdc_recipe being filled and returns an
// action that does nothing; the library applies the steps to the device topology.
class RecipeRecorder : public ract::TopologyReactionActionFactory {
public:
    RecipeRecorder(rdc_recipe *recipe, const model::Context &ctx) : _r(recipe), _ctx(ctx) {}

    ActionPtr createChangeParticleType(model::top::GraphTopology *top, const model::top::Graph::PersistentVertexIndex &v,
                                       const ParticleTypeId &type_to) const override {
        check(rdc_recipe_change_particle_type(_r, (int64_t)v.value, (int)type_to));
        return done(top);
    }
    ActionPtr createChangeParticlePosition(model::top::GraphTopology *top,
                                           const model::top::Graph::PersistentVertexIndex &v, Vec3 pos) const override {
        const double x[3] = {pos[0], pos[1], pos[2]};
        check(rdc_recipe_change_particle_position(_r, (int64_t)v.value, x));
        return done(top);
    }
    ActionPtr createAppendParticle(model::top::GraphTopology *top,
                                   const std::vector<model::top::Graph::PersistentVertexIndex> &neighbors,
                                   ParticleTypeId type, const Vec3 &pos) const override {
        std::vector<int64_t> nb;
        for (const auto &v : neighbors) nb.push_back((int64_t)v.value);
        const double x[3] = {pos[0], pos[1], pos[2]};
        check(rdc_recipe_append_particle(_r, (int64_t)nb.size(), nb.data(), (int)type, x));
        return done(top);
    }
    ActionPtr createChangeTopologyType(model::top::GraphTopology *top, const std::string &type_to) const override {
        check(rdc_recipe_change_topology_type(_r, (int)_ctx.topologyRegistry().idOf(type_to)));
        return done(top);
    }

private:
    struct Done : ract::TopologyReactionAction {
        using ract::TopologyReactionAction::TopologyReactionAction;
        void execute() override {}
    };
    static ActionPtr done(model::top::GraphTopology *top) { return std::make_unique<Done>(top); }
    rdc_recipe *_r;
    const model::Context &_ctx;
};

// op::AddEdge and op::RemoveEdge keep their edge private and pass it only to the factory's non-virtual
// createAddEdge/createRemoveEdge.  Access is not checked for the names in an explicit instantiation
// ([temp.spec.general]), so the two instantiations below form pointers to those members.
template <typename Tag, typename Tag::type M>
struct MemberOf {
    friend typename Tag::type member(Tag) { return M; }
};
struct AddEdgeMember {
    using type = model::top::Graph::Edge rop::AddEdge::*;
    friend type member(AddEdgeMember);
};
struct RemoveEdgeMember {
    using type = model::top::Graph::Edge rop::RemoveEdge::*;
    friend type member(RemoveEdgeMember);
};
template struct MemberOf<AddEdgeMember, &rop::AddEdge::_edge>;
template struct MemberOf<RemoveEdgeMember, &rop::RemoveEdge::_edge>;

// rdc_spatial_rate_fn: SpatialTopologyReaction::rate(top1, top2) on the device topologies g1 and g2 (the
// first and second educt's)
double spatialRate(void *user, rdc_system *, int64_t g1, int64_t g2) {
    auto *b = static_cast<CUDAKernel::SpatialBinding *>(user);
    auto &state = b->kernel->cudaStateModel();
    double rate = std::numeric_limits<double>::quiet_NaN();  // makes the evaluation fail after an exception
    try {
        const auto t1 = state.deviceTopology(g1);
        const auto t2 = state.deviceTopology(g2, true);
        rate = b->reaction.rate(*t1, *t2);
    } catch (...) {
        b->kernel->keepCallbackError(std::current_exception());
    }
    state.clearTopologyView();
    return rate;
}

// rdc_topology_rate_fn: StructuralTopologyReaction::rate on the device topology k
double structuralRate(void *user, rdc_system *, int64_t k) {
    auto *b = static_cast<CUDAKernel::StructuralBinding *>(user);
    auto &state = b->kernel->cudaStateModel();
    double rate = 0;
    try {
        const auto top = state.deviceTopology(k);
        rate = b->reaction.rate(*top);
    } catch (...) {
        b->kernel->keepCallbackError(std::current_exception());
    }
    state.clearTopologyView();
    return rate;
}

// rdc_topology_recipe_fn: StructuralTopologyReaction::operations on the device topology k, its steps in
// order into the rdc_recipe (vertex v of a step is local vertex v of rdc_get_topology)
void structuralRecipe(void *user, rdc_system *, int64_t k, rdc_recipe *recipe) {
    auto *b = static_cast<CUDAKernel::StructuralBinding *>(user);
    auto &state = b->kernel->cudaStateModel();
    try {
        auto top = state.deviceTopology(k);
        const auto steps = b->reaction.operations(*top);
        const RecipeRecorder rec(recipe, b->kernel->context());
        for (const auto &op : steps.steps()) {
            if (const auto *a = dynamic_cast<const rop::AddEdge *>(op.get())) {
                const auto &e = a->*member(AddEdgeMember{});
                check(rdc_recipe_add_edge(recipe, (int64_t)std::get<0>(e).value, (int64_t)std::get<1>(e).value));
            } else if (const auto *r = dynamic_cast<const rop::RemoveEdge *>(op.get())) {
                const auto &e = r->*member(RemoveEdgeMember{});
                check(rdc_recipe_remove_edge(recipe, (int64_t)std::get<0>(e).value, (int64_t)std::get<1>(e).value));
            } else {
                op->create_action(top.get(), &rec);
            }
        }
    } catch (...) {
        b->kernel->keepCallbackError(std::current_exception());
    }
    state.clearTopologyView();
}

}  // namespace

// every structural reaction of the topology registry (TopologyRegistry.h:91-113), with its mode
// (StructuralTopologyReaction.h: expect connected or create children)
void CUDAKernel::registerStructuralReactions() {
    _structural.clear();
    for (const auto &tt : context().topologyRegistry().types())
        for (const auto &r : tt.structuralReactions) {
            _structural.push_back(std::make_unique<StructuralBinding>(StructuralBinding{this, r}));
            check(rdc_add_structural_topology_reaction(_sys, (int)tt.type, structuralRate, structuralRecipe,
                                                       _structural.back().get(),
                                                       r.expects_connected_after_reaction() ? 1 : 0, nullptr));
        }
}

std::vector<std::unique_ptr<CUDAKernel::SpatialBinding>> CUDAKernel::bindSpatialRateFunctions(
        rdc_context *c,
        const std::vector<std::pair<int, const model::top::reactions::SpatialTopologyReaction *>> &functions) {
    std::vector<std::unique_ptr<SpatialBinding>> bound;
    for (const auto &[id, r] : functions) {
        bound.push_back(std::make_unique<SpatialBinding>(SpatialBinding{this, *r}));
        check(rdc_context_set_spatial_topology_rate_function(c, id, spatialRate, bound.back().get()));
    }
    return bound;
}

void CUDAKernel::rethrowCallbackError() {
    if (!_callbackError) return;
    std::exception_ptr e;
    std::swap(e, _callbackError);
    std::rethrow_exception(e);
}

rdc_system *CUDAKernel::sys() {
    if (!_sys) initialize();
    _state.flushTopologies();
    return _sys;
}

}  // namespace readdy::kernel::cuda

extern "C" const char *name() { return rdc_kernel_name(); }  // "CUDA"; CPUKernel.cpp:89-91

extern "C" readdy::model::Kernel *createKernel() { return new readdy::kernel::cuda::CUDAKernel(); }  // :93-95

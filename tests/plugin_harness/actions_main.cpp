// TEST INFRASTRUCTURE ONLY: drives the ReaDDy plugin's state model, actions and binning observables the way
// SimulationLoop and ReaDDy's observables do, against the logging stand-in C ABI of fake_abi.cpp, with ReaDDy's
// model library from the reference build.  Prints the stand-in's log of the system calls and the observables'
// results; the test compares them with the values given here.
#include "../../readdy_gb300/plugin/CUDAKernel.h"

#include <cstdio>

extern "C" void fake_abi_log_context(int on);

namespace top = readdy::model::top;
using PV = top::Graph::PersistentVertexIndex;

int main() {
    readdy::kernel::cuda::CUDAKernel k;
    auto &ctx = k.context();
    ctx.boxSize() = {10., 10., 10.};
    ctx.particleTypes().add("A", 1.0);
    ctx.particleTypes().add("T", 1.0, readdy::model::particleflavor::TOPOLOGY);
    ctx.particleTypes().add("B", 1.0);
    // ReaDDy numbers reactions in registration order; the device numbers order-1 reactions first
    const auto fus = ctx.reactions().addFusion("fus", "A", "A", "B", 1.0, 1.0);
    const auto conv = ctx.reactions().addConversion("conv", "B", "A", 0.5);
    ctx.topologyRegistry().addType("chain");
    ctx.topologyRegistry().configureBondPotential("T", "T", {5.0, 1.0});
    k.initialize();
    fake_abi_log_context(2);
    k.stateModel().addParticles({readdy::model::Particle(0.5, 1.5, -2.5, 0), readdy::model::Particle(1., 2., 3., 0)});
    auto *t = k.stateModel().addTopology(ctx.topologyRegistry().idOf("chain"),
                                         {readdy::model::Particle(0., 0., 0., 1), readdy::model::Particle(1., 0., 0., 1),
                                          readdy::model::Particle(2., 0., 0.25, 1)});
    t->addEdge(PV{0}, PV{1});
    t->addEdge(PV{1}, PV{2});
    auto print_particles = [&](const char *when) {
        std::printf("topology particles %s:", when);
        for (const auto &p : k.stateModel().getParticlesForTopology(*t))
            std::printf(" (%g %g %g)/%d", p.pos()[0], p.pos()[1], p.pos()[2], (int)p.type());
        std::printf("\n");
    };
    print_particles("pending");
    std::printf("pending vertex 2 type %d x %g\n", (int)t->particleForVertex(PV{2}).type(),
                t->particleForVertex(PV{2}).pos()[0]);
    // a Virial observable registered after the system holds particles (the flag reaches the live system)
    auto &o = k.observe();
    auto v = o.virial(1, [](const auto &) {});
    // the SimulationLoop order (SimulationLoop.h:256-306)
    auto &a = k.actions();
    a.initializeKernel()->perform();
    a.createNeighborList(2.5)->perform();
    a.calculateForces()->perform();
    a.eulerBDIntegrator(0.01)->perform();
    a.updateNeighborList()->perform();
    a.uncontrolledApproximation(0.02)->perform();
    a.gillespie(0.03)->perform();
    readdy::model::actions::top::BreakConfig cfg;
    cfg.addBreakablePair(1, 1, 2.0, 0.5);
    a.breakBonds(0.04, cfg)->perform();
    // the topology the caller holds is still the state model's after the reload (its particles are unchanged)
    std::printf("same topology object after reload %d\n", (int)(k.stateModel().getTopologies().at(0) == t));
    print_particles("uploaded");
    a.clearNeighborList()->perform();
    v->evaluate();
    auto rc = o.reactionCounts(1, [](const auto &) {});
    rc->evaluate();
    const auto &counts = std::get<0>(rc->getResult());
    std::printf("reaction counts fus %zu conv %zu\n", (std::size_t)counts.at(fus), (std::size_t)counts.at(conv));
    auto fo = o.forces(1, {"A"}, [](const auto &) {});
    fo->evaluate();
    for (const auto &f : fo->getResult()) std::printf("force of A %g %g %g\n", f[0], f[1], f[2]);
    auto po = o.positions(1, {"T"}, [](const auto &) {});
    po->evaluate();
    for (const auto &x : po->getResult()) std::printf("position of T %g %g %g\n", x[0], x[1], x[2]);
    auto pa = o.particles(1, [](const auto &) {});
    pa->evaluate();
    const auto &[ptypes, pids, ppos] = pa->getResult();
    std::printf("particles %zu:", ptypes.size());
    for (std::size_t i = 0; i < ptypes.size(); ++i) std::printf(" %d/%zu", (int)ptypes[i], (std::size_t)pids[i]);
    std::printf("\n");
    auto en = o.energy(1, [](const auto &) {});
    en->evaluate();
    std::printf("energy %g\n", en->getResult());
    auto n = o.nParticles(1, {"A", "T"}, [](const auto &) {});
    n->evaluate();
    auto h = o.histogramAlongAxis(1, {0., 1., 2.5}, {"T"}, 2, [](const auto &) {});
    h->evaluate();
    auto r = o.radialDistribution(1, {0., 0.5, 1.0, 2.0}, {"A"}, {"A", "T"}, 0.25, [](const auto &) {});
    r->evaluate();
    // ReaDDy's own Topologies observable (Topologies.cpp:61-82) over the plugin's getTopologies and
    // toDenseParticleIndices
    auto tobs = o.topologies(1);
    tobs->evaluate();
    for (const auto &rec : tobs->getResult()) {
        std::printf("topology record type %d particles", (int)rec.type);
        for (auto i : rec.particleIndices) std::printf(" %zu", (std::size_t)i);
        std::printf(" edges");
        for (const auto &[a, b] : rec.edges) std::printf(" %zu-%zu", (std::size_t)a, (std::size_t)b);
        std::printf("\n");
    }
    // Kernel::initialize again (the CPU kernel's InitializeKernel action calls it): a new system takes over
    // the free particles and the topology with its edges
    k.initialize();
    const auto tops = k.stateModel().getTopologies();
    std::printf("after initialize: %zu particles, %zu topologies, %zu vertices, %zu edges\n",
                k.stateModel().getParticles().size(), tops.size(), tops.at(0)->graph().vertices().size(),
                tops.at(0)->graph().edges().size());
    k.stateModel().removeAllParticles();
    std::printf("after removeAllParticles: %zu particles, %zu topologies\n", k.stateModel().getParticles().size(),
                k.stateModel().getTopologies().size());
    fake_abi_log_context(0);
    std::printf("virial %g %g %g\n", v->getResult().at(0, 0), v->getResult().at(1, 1), v->getResult().at(2, 2));
    std::printf("n particles %lu %lu\n", n->getResult()[0], n->getResult()[1]);
    std::printf("histogram %g %g\n", h->getResult()[0], h->getResult()[1]);
    const auto &[centers, distribution] = r->getResult();
    std::printf("radial distribution centers %g %g %g values %g %g %g\n", centers[0], centers[1], centers[2],
                distribution[0], distribution[1], distribution[2]);
    return 0;
}

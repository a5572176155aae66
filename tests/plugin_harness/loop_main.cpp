// TEST INFRASTRUCTURE ONLY: ReaDDy's own SimulationLoop (include/readdy/api/SimulationLoop.h:256-306) drives the
// plugin for two steps of a system with a pair potential, a topology and a topology-particle reaction, against
// the logging stand-in C ABI of fake_abi.cpp.  Prints whether ReaDDy sees topology support and the stand-in's log
// of the system calls the loop makes.
#include "../../readdy_gb300/plugin/CUDAKernel.h"

#include <readdy/api/SimulationLoop.h>

#include <cstdio>

extern "C" void fake_abi_log_context(int on);

using PV = readdy::model::top::Graph::PersistentVertexIndex;

int main() {
    readdy::kernel::cuda::CUDAKernel k;
    auto &ctx = k.context();
    ctx.boxSize() = {10., 10., 10.};
    ctx.particleTypes().add("A", 1.0);
    ctx.particleTypes().add("T", 1.0, readdy::model::particleflavor::TOPOLOGY);
    ctx.potentials().addHarmonicRepulsion("A", "A", 1.0, 1.5);
    ctx.topologyRegistry().addType("chain");
    ctx.topologyRegistry().configureBondPotential("T", "T", {5.0, 1.0});
    ctx.topologyRegistry().addSpatialReaction("attach: chain(T)+(A)->chain(T--T)", 1.0, 1.0);
    // Kernel::supportsTopologies gates Simulation::addTopology and SimulationLoop's topology reactions
    std::printf("supports topologies %d\n", (int)k.supportsTopologies());
    k.stateModel().addParticles({readdy::model::Particle(3., 0., 0., 0)});
    auto *t = k.stateModel().addTopology(ctx.topologyRegistry().idOf("chain"),
                                         {readdy::model::Particle(0., 0., 0., 1), readdy::model::Particle(1., 0., 0., 1)});
    t->addEdge(PV{0}, PV{1});
    fake_abi_log_context(2);
    readdy::api::SimulationLoop loop(&k, 0.01);
    loop.neighborListCutoff() += 0.5;  // a skin, as ReaDDy's Python API adds it (simulation.py:555-556)
    loop.run(2);
    fake_abi_log_context(0);
    return 0;
}

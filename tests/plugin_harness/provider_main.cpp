// TEST INFRASTRUCTURE ONLY: ReaDDy's KernelProvider loads the plugin library from the directory given as argv[1]
// (readdy/main/plugin/KernelProvider.cpp:99-175), and ReaDDy's Simulation (include/readdy/api/Simulation.h) runs
// two steps on the "CUDA" kernel it creates, with a particle, a topology and an observable.  The plugin library
// carries the logging stand-in C ABI of fake_abi.cpp; its log switch is looked up with dlsym.  Prints the
// available kernels, the selected one and the stand-in's log.
#include <readdy/api/Simulation.h>
#include <readdy/plugin/KernelProvider.h>

#include <dlfcn.h>

#include <cstdio>

using PV = readdy::model::top::Graph::PersistentVertexIndex;

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    auto &provider = readdy::plugin::KernelProvider::getInstance();
    provider.loadKernelsFromDirectory(argv[1]);
    bool found = false;
    for (const auto &name : provider.availableKernels()) found |= name == "CUDA";
    std::printf("CUDA kernel available %d\n", (int)found);

    readdy::model::Context ctx;
    ctx.boxSize() = {10., 10., 10.};
    ctx.particleTypes().add("A", 1.0);
    ctx.particleTypes().add("T", 1.0, readdy::model::particleflavor::TOPOLOGY);
    ctx.potentials().addHarmonicRepulsion("A", "A", 1.0, 1.5);
    ctx.topologyRegistry().addType("chain");
    ctx.topologyRegistry().configureBondPotential("T", "T", {5.0, 1.0});
    readdy::Simulation sim("CUDA", ctx);
    std::printf("selected %s supports topologies %d\n", sim.selectedKernelType().c_str(),
                (int)sim.kernelSupportsTopologies());

    auto log = reinterpret_cast<void (*)(int)>(dlsym(RTLD_DEFAULT, "fake_abi_log_context"));
    if (!log) return 3;
    log(2);
    sim.addParticle("A", 0.5, 0.5, 0.5);
    auto *t = sim.addTopology("chain", {sim.createTopologyParticle("T", {0., 0., 0.}),
                                        sim.createTopologyParticle("T", {1., 0., 0.})});
    t->addEdge(PV{0}, PV{1});
    sim.registerObservable(sim.observe().nParticles(1, std::vector<std::string>{"A"}, [](const auto &r) {
        std::printf("observed %zu particles of A\n", (std::size_t)r.at(0));
    }));
    sim.run(2, 0.01);
    log(0);
    return 0;
}

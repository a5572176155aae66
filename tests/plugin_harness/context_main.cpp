// TEST INFRASTRUCTURE ONLY: initializes the ReaDDy plugin on a model::Context that holds every potential,
// reaction and topology term the plugin translates, built through ReaDDy's own registries (the reference
// build's model library), against the logging stand-in C ABI of fake_abi.cpp.  Prints the stand-in's log
// of the rdc_context_* calls; the test compares every call's arguments with the values given here.
#include "../../readdy_gb300/plugin/CUDAKernel.h"

#include <cstdio>

extern "C" void fake_abi_log_context(int on);

int main() {
    readdy::kernel::cuda::CUDAKernel k;
    auto &ctx = k.context();
    ctx.boxSize() = {10., 12., 14.};
    ctx.periodicBoundaryConditions() = {true, true, false};
    ctx.kBT() = 1.5;
    ctx.particleTypes().add("A", 1.0);
    ctx.particleTypes().add("B", 0.5);
    ctx.particleTypes().add("C", 0.25, readdy::model::particleflavor::TOPOLOGY);
    ctx.particleTypes().add("D", 2.0, readdy::model::particleflavor::TOPOLOGY);
    auto &pots = ctx.potentials();
    pots.addHarmonicRepulsion("A", "B", 10.0, 1.1);
    pots.addWeakInteractionPiecewiseHarmonic("B", "B", 5.0, 0.7, 0.3, 1.9);
    pots.addLennardJones("A", "A", 12, 6, 2.5, true, 1.25, 0.9);
    pots.addScreenedElectrostatics("A", "C", -1.0, 0.8, 1.2, 0.6, 6, 3.5);
    pots.addBox("A", 2.0, {-4., -5., -6.}, {8., 10., 12.});
    pots.addSphere("B", 3.0, {0.5, 0.25, -0.5}, 4.0, true);
    pots.addSphere("B", 3.5, {0., 0., 0.}, 2.0, false);
    pots.addCapsule("C", 4.0, {0., 1., 0.}, {1., 0., 0.}, 3.0, 1.5);
    pots.addSphericalBarrier("D", 2.5, 0.5, {1., 1., 1.}, 2.0);
    pots.addCylinder("A", 1.5, {0., 0., 0.}, {0., 0., 2.}, 3.0, true);
    auto &rx = ctx.reactions();
    rx.addConversion("conv", "A", "B", 0.1);
    rx.addDecay("dec", "B", 0.02);
    rx.addFusion("fus", "A", "B", "C", 1.0, 1.2, 1.0, 3.0);
    rx.addFission("fis", "C", "A", "B", 0.5, 0.8, 2.0, 2.0);
    rx.addEnzymatic("enz", "D", "A", "B", 0.7, 1.1);
    auto &top = ctx.topologyRegistry();
    top.addType("T1");
    top.addType("T2");
    top.configureBondPotential("C", "D", {10.0, 1.0});
    top.configureAnglePotential("C", "D", "C", {2.0, 3.0});
    top.configureTorsionPotential("C", "D", "D", "C", {1.0, 3.0, 0.5});
    top.addSpatialReaction("tt: T1(C)+T1(D)->T2(C--D)", 2.0, 1.5);
    top.addSpatialReaction("tf: T2(C)+T2(D)->T1(C--D)",
                           [](const readdy::model::top::GraphTopology &, const readdy::model::top::GraphTopology &) {
                               return 1.0;
                           },
                           0.75);
    std::printf("ids A=%d B=%d C=%d D=%d T1=%d T2=%d\n", (int)ctx.particleTypes().idOf("A"),
                (int)ctx.particleTypes().idOf("B"), (int)ctx.particleTypes().idOf("C"),
                (int)ctx.particleTypes().idOf("D"), (int)top.idOf("T1"), (int)top.idOf("T2"));
    fake_abi_log_context(1);
    k.initialize();
    fake_abi_log_context(0);
    return 0;
}

// TEST INFRASTRUCTURE ONLY: runs the ReaDDy plugin's structural topology reactions against the stand-in C ABI
// of fake_abi.cpp, with ReaDDy's own model library (Context, TopologyRegistry, GraphTopology, Recipe) from the
// reference build.  Prints the stand-in's log; the test compares it with the expected C-ABI calls.
#include "../../readdy_gb300/plugin/CUDAKernel.h"

#include <readdy/model/topologies/reactions/Recipe.h>
#include <readdy/model/topologies/reactions/StructuralTopologyReaction.h>

#include <cstdio>
#include <stdexcept>

namespace top = readdy::model::top;
using readdy::Vec3;
using PV = top::Graph::PersistentVertexIndex;

int main() {
    readdy::kernel::cuda::CUDAKernel k;
    auto &ctx = k.context();
    ctx.particleTypes().add("A", 1.0, readdy::model::particleflavor::TOPOLOGY);
    ctx.particleTypes().add("B", 1.0, readdy::model::particleflavor::TOPOLOGY);
    const auto t1 = ctx.topologyRegistry().addType("T1");
    const auto t2 = ctx.topologyRegistry().addType("T2");
    std::printf("ids A=%d B=%d T1=%d T2=%d\n", (int)ctx.particleTypes().idOf("A"), (int)ctx.particleTypes().idOf("B"),
                (int)t1, (int)t2);
    // rate: the sum of the vertices' x coordinates plus 10 per particle of type A, read through the topology
    auto rate = [](const top::GraphTopology &t) {
        double r = 0;
        for (const auto &v : t.graph().vertices()) {
            const auto p = t.particleForVertex(v);
            r += p.pos()[0] + (p.type() == 0 ? 10.0 : 0.0);
        }
        return r;
    };
    auto recipe = [](top::GraphTopology &t) {
        top::reactions::Recipe r(t);
        r.changeParticleType(PV{0}, "B");
        r.addEdge(PV{0}, PV{2});
        r.removeEdge(PV{0}, PV{1});
        r.separateVertex(PV{1});
        r.appendNewParticle({PV{2}, PV{0}}, "B", Vec3(4, 5, 6));
        r.changeParticlePosition(PV{1}, Vec3(7, 8, 9));
        r.changeTopologyType("T2");
        return r;
    };
    top::reactions::StructuralTopologyReaction all("all steps", recipe, rate);
    all.expect_connected_after_reaction();
    ctx.topologyRegistry().addStructuralReaction("T1", all);
    top::reactions::StructuralTopologyReaction fixed(
            "fixed rate", [](top::GraphTopology &t) { return top::reactions::Recipe(t).changeParticleType(PV{2}, 1); },
            2.5);
    fixed.create_child_topologies_after_reaction();
    ctx.topologyRegistry().addStructuralReaction("T1", fixed);
    // a spatial reaction whose rate is a function of the two topologies: 100 x the first's vertices plus the
    // second's x coordinates
    ctx.topologyRegistry().addSpatialReaction(
            "sp: T1(A)+T1(B)->T1(A--B)",
            [](const top::GraphTopology &t1, const top::GraphTopology &t2) {
                double r = 100.0 * (double)t1.graph().vertices().size();
                for (const auto &v : t2.graph().vertices()) r += t2.particleForVertex(v).pos()[0];
                return r;
            },
            1.2);
    k.initialize();
    k.actions().evaluateTopologyReactions(1.0)->perform();

    // an exception in a reaction's function reaches the caller of the action
    readdy::kernel::cuda::CUDAKernel k2;
    auto &ctx2 = k2.context();
    ctx2.particleTypes().add("A", 1.0, readdy::model::particleflavor::TOPOLOGY);
    ctx2.topologyRegistry().addType("T1");
    ctx2.topologyRegistry().addStructuralReaction(
            "T1", top::reactions::StructuralTopologyReaction(
                          "throws", [](top::GraphTopology &t) { return top::reactions::Recipe(t); },
                          [](const top::GraphTopology &) -> double { throw std::domain_error("rate failed"); }));
    k2.initialize();
    try {
        k2.actions().evaluateTopologyReactions(1.0)->perform();
        std::printf("no exception\n");
    } catch (const std::domain_error &e) {
        std::printf("caught %s\n", e.what());
    }
    return 0;
}

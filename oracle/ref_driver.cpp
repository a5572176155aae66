// TEST INFRASTRUCTURE ONLY: a C ABI around the reference's own pthread CPU kernel (kernels/cpu, compiled
// from the reference sources by oracle/ref_build.py into oracle/_ref/), so that bench.py can time the
// reference implementation of the hot path on the host cores.  It builds a readdy::model::Context from
// plain arguments, creates readdy::kernel::cpu::CPUKernel directly (as KernelProvider::create would,
// readdy/main/plugin/KernelProvider.cpp:183-189), adds particles and runs readdy::api::SimulationLoop
// (include/readdy/api/SimulationLoop.h:256-306) with the chosen reaction handler.  Nothing here is on
// the product path.
#include <readdy/api/SimulationLoop.h>
#include <readdy/io/BloscFilter.h>
#include <readdy/kernel/cpu/CPUKernel.h>

#include <chrono>
#include <cstdint>
#include <exception>
#include <memory>
#include <string>
#include <vector>

// The HDF5 compression filter of the reference needs the blosc library, which this image lacks; no
// output file is written here, so these stand-in definitions only report that the filter is missing.
namespace readdy::io {
BloscFilter::BloscFilter(Compressor compressor, unsigned int compressionLevel, bool shuffle)
    : shuffle(shuffle), compressor(compressor), compressionLevel(compressionLevel) {}
bool BloscFilter::available() const { return false; }
void BloscFilter::activate(h5rd::PropertyList &) {}
void BloscFilter::registerFilter() {}
}  // namespace readdy::io

namespace {
thread_local std::string g_error;

struct RefSystem {
    std::unique_ptr<readdy::kernel::cpu::CPUKernel> kernel;
    int ntypes = 0;
    int nreactions = 0;
};

std::string type_name(int t) { return "T" + std::to_string(t); }

template <typename F>
int guarded(F &&f) {
    try {
        f();
        return 0;
    } catch (const std::exception &e) {
        g_error = e.what();
        return 1;
    }
}
}  // namespace

extern "C" {

const char *refk_last_error() { return g_error.c_str(); }

// a CPU kernel with n_types species (names T0, T1, ...) and n_threads worker threads (0: the
// reference's default, include/readdy/common/common.h:80-95)
void *refk_create(const double box[3], const int pbc[3], double kbt, int n_types, const double *D, int n_threads) {
    RefSystem *s = nullptr;
    if (guarded([&] {
            auto k = std::make_unique<readdy::kernel::cpu::CPUKernel>();
            auto &ctx = k->context();
            ctx.boxSize() = {box[0], box[1], box[2]};
            ctx.periodicBoundaryConditions() = {pbc[0] != 0, pbc[1] != 0, pbc[2] != 0};
            ctx.kBT() = kbt;
            for (int t = 0; t < n_types; ++t) ctx.particleTypes().add(type_name(t), D[t]);
            if (n_threads > 0) ctx.kernelConfiguration().cpu.threadConfig.nThreads = n_threads;
            s = new RefSystem{std::move(k), n_types, 0};
        }) != 0)
        return nullptr;
    return s;
}

void refk_destroy(void *h) { delete static_cast<RefSystem *>(h); }

int refk_add_harmonic_repulsion(void *h, int t1, int t2, double k, double d) {
    return guarded([&] {
        static_cast<RefSystem *>(h)->kernel->context().potentials().addHarmonicRepulsion(type_name(t1), type_name(t2), k, d);
    });
}

int refk_add_weak_interaction_piecewise_harmonic(void *h, int t1, int t2, double k, double desired, double depth,
                                                 double cutoff) {
    return guarded([&] {
        static_cast<RefSystem *>(h)->kernel->context().potentials().addWeakInteractionPiecewiseHarmonic(
                type_name(t1), type_name(t2), k, desired, depth, cutoff);
    });
}

int refk_add_lennard_jones(void *h, int t1, int t2, unsigned m, unsigned n, double cutoff, int shift, double epsilon,
                           double sigma) {
    return guarded([&] {
        static_cast<RefSystem *>(h)->kernel->context().potentials().addLennardJones(type_name(t1), type_name(t2), m, n,
                                                                                   cutoff, shift != 0, epsilon, sigma);
    });
}

int refk_add_fusion(void *h, int a, int b, int c, double rate, double educt_distance) {
    auto *s = static_cast<RefSystem *>(h);
    return guarded([&] {
        s->kernel->context().reactions().addFusion("fusion" + std::to_string(s->nreactions++), type_name(a), type_name(b),
                                                   type_name(c), rate, educt_distance);
    });
}

int refk_add_fission(void *h, int a, int b, int c, double rate, double product_distance) {
    auto *s = static_cast<RefSystem *>(h);
    return guarded([&] {
        s->kernel->context().reactions().addFission("fission" + std::to_string(s->nreactions++), type_name(a), type_name(b),
                                                    type_name(c), rate, product_distance);
    });
}

int refk_add_particles(void *h, int64_t n, const double *pos3, const int *types) {
    auto *s = static_cast<RefSystem *>(h);
    return guarded([&] {
        std::vector<readdy::model::Particle> ps;
        ps.reserve((std::size_t)n);
        for (int64_t i = 0; i < n; ++i)
            ps.emplace_back(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], (readdy::ParticleTypeId)types[i]);
        s->kernel->stateModel().addParticles(ps);
    });
}

// the reference's CalculateForces on the current particles (neighbour list set up at the context's largest
// cutoff): per active particle its id and force (ids in the order the kernel stores them), and the energy
int refk_calculate_forces(void *h, int64_t capacity, uint64_t *ids, double *forces3, int64_t *n_out, double *energy) {
    auto *s = static_cast<RefSystem *>(h);
    return guarded([&] {
        auto &k = *s->kernel;
        k.initialize();
        k.stateModel().initializeNeighborList(k.context().calculateMaxCutoff());
        k.actions().calculateForces()->perform();
        int64_t n = 0;
        for (const auto &e : *k.getCPUKernelStateModel().getParticleData()) {
            if (e.deactivated) continue;
            if (n < capacity) {
                if (ids) ids[n] = e.id;
                if (forces3) {
                    forces3[3 * n] = e.force[0];
                    forces3[3 * n + 1] = e.force[1];
                    forces3[3 * n + 2] = e.force[2];
                }
            }
            ++n;
        }
        if (n_out) *n_out = n;
        if (energy) *energy = k.stateModel().energy();
    });
}

// runs n_steps of the simulation loop with handler 0 = UncontrolledApproximation, 1 = Gillespie; writes
// the final per-type counts (n_types values) and the wall-clock seconds of the run
int refk_run(void *h, int64_t n_steps, double dt, int handler, int64_t *counts, double *seconds) {
    auto *s = static_cast<RefSystem *>(h);
    return guarded([&] {
        s->kernel->initialize();
        readdy::api::SimulationLoop loop(s->kernel.get(), dt);
        loop.useReactionScheduler(handler == 1 ? "Gillespie" : "UncontrolledApproximation");
        const auto t0 = std::chrono::steady_clock::now();
        loop.run(n_steps);
        const auto t1 = std::chrono::steady_clock::now();
        if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
        if (counts) {
            for (int t = 0; t < s->ntypes; ++t) counts[t] = 0;
            for (const auto &p : s->kernel->stateModel().getParticles())
                if ((int)p.type() < s->ntypes) ++counts[p.type()];
        }
    });
}

}  // extern "C"

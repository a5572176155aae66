// The "CUDA" kernel plugin for ReaDDy: model::Kernel, StateModel, ActionFactory and ObservableFactory of
// the reference's plugin interface (include/readdy/model/Kernel.h:71-235, StateModel.h:53-118,
// actions/ActionFactory.h:56-129, observables/ObservableFactory.h:62-185), each method one call into the C
// ABI of libreaddy_cuda_core.so (include/readdy_cuda.h).  Built against ReaDDy's headers like the CPU
// kernel (kernels/cpu) and linked to libreaddy and libreaddy_cuda_core.so; install it as
// libreaddy_kernel_cuda.so in READDY_PLUGIN_DIR, whose loader accepts file names that contain ".so" and
// none of ".a", ".lib", ".obj", ... anywhere in the path (readdy/main/plugin/KernelProvider.cpp:123-133).
#pragma once

#include <readdy/model/Kernel.h>
#include <readdy/model/actions/Actions.h>
#include <readdy/model/observables/ObservableFactory.h>
#include <readdy/model/topologies/GraphTopology.h>
#include <readdy/model/topologies/TopologyActionFactory.h>
#include <readdy_cuda.h>

#include <exception>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

namespace readdy::kernel::cuda {

// status code of the C ABI -> the exception type the CPU kernel throws for the same failure
void check(int rc);

class CUDAKernel;

// StateModel over one rdc_system.  Particles added through addParticles go to the device at once.
// Topology particles stay on the host until the first action after they were added: their graph's
// edges are only complete then (the API adds edges after addTopology returns), and rdc_add_topology
// takes particles and edges together.
class CUDAStateModel : public model::StateModel {
public:
    explicit CUDAStateModel(CUDAKernel *kernel) : _kernel(kernel) {}

    std::vector<Vec3> getParticlePositions() const override;
    std::vector<model::Particle> getParticles() const override;
    model::Particle getParticleForIndex(std::size_t index) const override;
    // the particles of a topology by vertex: one read-back of the system (StateModel.cpp:47-55 looks each vertex
    // up by itself); a topology not uploaded yet gives the particles it was added with
    std::vector<model::Particle> getParticlesForTopology(const model::top::GraphTopology &topology) const override;
    ParticleTypeId getParticleType(std::size_t index) const override;
    void initializeNeighborList(scalar interactionDistance) override;
    void updateNeighborList() override;
    void clearNeighborList() override;
    void addParticle(const model::Particle &p) override { addParticles({p}); }
    void addParticles(const std::vector<model::Particle> &p) override;
    model::top::GraphTopology *const addTopology(TopologyTypeId type,
                                                 const std::vector<model::Particle> &particles) override;
    std::vector<model::top::GraphTopology *> getTopologies() override;
    void removeParticle(const model::Particle &p) override;
    void removeAllParticles() override;
    scalar energy() const override;
    scalar &energy() override;
    scalar time() const override { return _time; }
    void setTime(scalar t) override { _time = t; }
    void toDenseParticleIndices(std::vector<std::size_t>::iterator begin,
                                std::vector<std::size_t>::iterator end) const override;
    void clear() override { removeAllParticles(); }

    // uploads the pending topologies (particles and graph edges) to the device
    void flushTopologies();
    // rebuilds the host topologies from the device's
    void reloadTopologies();
    // The live system's particles outside topologies and its topologies (type, particles by local vertex,
    // edges), read back so that a new system of the same state can replace it (Kernel::initialize).
    struct Snapshot {
        std::vector<model::Particle> free;
        struct Top {
            int type = 0;
            std::vector<double> x;
            std::vector<int> t;
            std::vector<int64_t> edges;  // local vertex pairs
        };
        std::vector<Top> topologies;
    };
    Snapshot snapshot() const;
    // uploads a snapshot into the current system (particle ids are those the new system gives)
    void restore(const Snapshot &snap);
    // topology k of the device (rdc_get_topologies order) as a host GraphTopology for a structural reaction's
    // functions: local vertex v has persistent index v and holds the device id; until the next call,
    // getParticleForIndex serves its particles without reading the whole system back
    std::unique_ptr<model::top::GraphTopology> deviceTopology(int64_t k, bool keep_view = false);
    void clearTopologyView() { _view.clear(); }

private:
    struct PendingTopology {
        std::unique_ptr<model::top::GraphTopology> top;
        std::vector<model::Particle> particles;
    };
    CUDAKernel *_kernel;
    std::vector<PendingTopology> _pending;
    std::vector<std::unique_ptr<model::top::GraphTopology>> _topologies;
    std::unordered_map<std::size_t, model::Particle> _view;  // particles of the last deviceTopology
    // Until its upload, a topology's vertices hold placeholder indices (above any device id) of the particles it
    // was added with, so that particle lookups by vertex (GraphTopology::particleForVertex) find them.
    static constexpr std::size_t PENDING_INDEX = std::size_t(1) << 62;
    std::unordered_map<std::size_t, model::Particle> _pendingParticles;
    std::size_t _nextPending = PENDING_INDEX;
    mutable scalar _energy = 0;
    scalar _time = 0;
};

class CUDAActionFactory : public model::actions::ActionFactory {
public:
    explicit CUDAActionFactory(CUDAKernel *kernel) : _kernel(kernel) {}

    std::unique_ptr<model::actions::AddParticles> addParticles(const std::vector<model::Particle> &particles) const override;
    std::unique_ptr<model::actions::EulerBDIntegrator> eulerBDIntegrator(scalar timeStep) const override;
    std::unique_ptr<model::actions::CalculateForces> calculateForces() const override;
    std::unique_ptr<model::actions::CreateNeighborList> createNeighborList(scalar interactionDistance) const override;
    std::unique_ptr<model::actions::UpdateNeighborList> updateNeighborList() const override;
    std::unique_ptr<model::actions::ClearNeighborList> clearNeighborList() const override;
    std::unique_ptr<model::actions::EvaluateCompartments> evaluateCompartments() const override;
    std::unique_ptr<model::actions::reactions::UncontrolledApproximation> uncontrolledApproximation(scalar timeStep) const override;
    std::unique_ptr<model::actions::reactions::Gillespie> gillespie(scalar timeStep) const override;
    std::unique_ptr<model::actions::reactions::DetailedBalance> detailedBalance(scalar timeStep) const override;
    std::unique_ptr<model::actions::top::EvaluateTopologyReactions> evaluateTopologyReactions(scalar timeStep) const override;
    std::unique_ptr<model::actions::top::BreakBonds> breakBonds(scalar timeStep, model::actions::top::BreakConfig config) const override;
    std::unique_ptr<model::actions::EvaluateObservables> evaluateObservables() const override;
    std::unique_ptr<model::actions::MakeCheckpoint> makeCheckpoint(std::string base, std::size_t maxNSaves) const override;
    std::unique_ptr<model::actions::InitializeKernel> initializeKernel() const override;

private:
    CUDAKernel *_kernel;
};

class CUDAObservableFactory : public model::observables::ObservableFactory {
public:
    explicit CUDAObservableFactory(CUDAKernel *kernel);

    std::unique_ptr<model::observables::Energy> energy(Stride stride, ObsCallback<model::observables::Energy> callback) const override;
    std::unique_ptr<model::observables::Virial> virial(Stride stride, ObsCallback<model::observables::Virial> callback) const override;
    std::unique_ptr<model::observables::HistogramAlongAxis>
    histogramAlongAxis(Stride stride, std::vector<scalar> binBorders, std::vector<std::string> typesToCount,
                       unsigned int axis, ObsCallback<model::observables::HistogramAlongAxis> callback) const override;
    std::unique_ptr<model::observables::NParticles>
    nParticles(Stride stride, std::vector<std::string> typesToCount, ObsCallback<model::observables::NParticles> callback) const override;
    std::unique_ptr<model::observables::Forces>
    forces(Stride stride, std::vector<std::string> typesToCount, ObsCallback<model::observables::Forces> callback) const override;
    std::unique_ptr<model::observables::Positions>
    positions(Stride stride, std::vector<std::string> typesToCount, ObsCallback<model::observables::Positions> callback) const override;
    std::unique_ptr<model::observables::RadialDistribution>
    radialDistribution(Stride stride, std::vector<scalar> binBorders, std::vector<std::string> typeCountFrom,
                       std::vector<std::string> typeCountTo, scalar particleDensity,
                       ObsCallback<model::observables::RadialDistribution> callback) const override;
    std::unique_ptr<model::observables::Particles> particles(Stride stride, ObsCallback<model::observables::Particles> callback) const override;
    std::unique_ptr<model::observables::Reactions> reactions(Stride stride, ObsCallback<model::observables::Reactions> callback) const override;
    std::unique_ptr<model::observables::ReactionCounts> reactionCounts(Stride stride, ObsCallback<model::observables::ReactionCounts> callback) const override;

private:
    CUDAKernel *_kernel;
};

// The kernel's topology action factory (Kernel.h:177-199).  ReaDDy treats a kernel as supporting topologies
// when it has one (Kernel::supportsTopologies): Simulation::addTopology and SimulationLoop's topology
// reactions depend on it.  The plugin evaluates bonded terms, BreakBonds and topology reactions on the device
// through its own actions, so none of its paths creates the per-topology host actions of this factory; a
// caller that asks for one gets std::logic_error.
class CUDATopologyActionFactory : public model::top::TopologyActionFactory {
public:
    std::unique_ptr<model::top::pot::CalculateHarmonicBondPotential>
    createCalculateHarmonicBondPotential(const harmonic_bond *) const override;
    std::unique_ptr<model::top::pot::CalculateHarmonicAnglePotential>
    createCalculateHarmonicAnglePotential(const harmonic_angle *) const override;
    std::unique_ptr<model::top::pot::CalculateCosineDihedralPotential>
    createCalculateCosineDihedralPotential(const cos_dihedral *) const override;
    ActionPtr createChangeParticleType(model::top::GraphTopology *, const model::top::Graph::PersistentVertexIndex &,
                                       const ParticleTypeId &) const override;
    ActionPtr createChangeParticlePosition(model::top::GraphTopology *, const model::top::Graph::PersistentVertexIndex &,
                                           Vec3) const override;
    ActionPtr createAppendParticle(model::top::GraphTopology *,
                                   const std::vector<model::top::Graph::PersistentVertexIndex> &, ParticleTypeId,
                                   const Vec3 &) const override;
    ActionPtr createChangeTopologyType(model::top::GraphTopology *, const std::string &) const override;
};

class CUDAKernel : public model::Kernel {
public:
    CUDAKernel();
    ~CUDAKernel() override;

    const model::StateModel &stateModel() const override { return _state; }
    model::StateModel &stateModel() override { return _state; }
    const model::actions::ActionFactory &actions() const override { return _actions; }
    model::actions::ActionFactory &actions() override { return _actions; }
    const model::observables::ObservableFactory &observe() const override { return _observables; }
    model::observables::ObservableFactory &observe() override { return _observables; }
    // topology reactions and BreakBonds run in the C ABI (no per-operation actions are created); the factory
    // is there so that ReaDDy sees topology support (Kernel::supportsTopologies)
    const model::top::TopologyActionFactory *const getTopologyActionFactory() const override { return &_topologyActions; }
    model::top::TopologyActionFactory *const getTopologyActionFactory() override { return &_topologyActions; }
    // Kernel::initialize (CPUKernel.cpp:63-83): the context is read again into a new device system, which
    // takes over the particles and topologies (their bonded terms derived again, reaction counts and virial
    // reset, as the CPU kernel resets them); particle ids are renumbered
    void initialize() override;
    // drops the system: the next use creates an empty one (StateModel::removeAllParticles)
    void dropSystem();
    bool supportsGillespie() const override { return true; }

    // the device system of the current context (created by initialize); pending topologies are uploaded
    // first, so every action sees all particles
    rdc_system *sys();
    rdc_system *sysIfCreated() const { return _sys; }
    CUDAStateModel &cudaStateModel() { return _state; }
    // reference reaction id -> device reaction id (-1: not registered on the device)
    const std::vector<int> &reactionIds() const { return _rx; }

    // A structural topology reaction of the registry (a copy, so that later changes of the registry leave
    // the registered system's functions in place), registered with rdc_add_structural_topology_reaction;
    // its rate and reaction functions run on a host GraphTopology of the device topology.  An exception they
    // throw cannot cross the C ABI: the first one is kept and rethrown when the library call returns.
    struct StructuralBinding {
        CUDAKernel *kernel;
        model::top::reactions::StructuralTopologyReaction reaction;
    };
    // a spatial topology reaction with a rate function (SpatialTopologyReaction.h:77-99), registered with
    // rdc_context_set_spatial_topology_rate_function
    struct SpatialBinding {
        CUDAKernel *kernel;
        model::top::reactions::SpatialTopologyReaction reaction;
    };
    void keepCallbackError(std::exception_ptr e) {
        if (!_callbackError) _callbackError = std::move(e);
    }
    void rethrowCallbackError();

private:
    void registerStructuralReactions();
    std::vector<std::unique_ptr<SpatialBinding>> bindSpatialRateFunctions(
            rdc_context *c,
            const std::vector<std::pair<int, const model::top::reactions::SpatialTopologyReaction *>> &functions);

    rdc_context *_ctx = nullptr;
    rdc_system *_sys = nullptr;
    std::vector<int> _rx;
    std::vector<std::unique_ptr<StructuralBinding>> _structural;
    std::vector<std::unique_ptr<SpatialBinding>> _spatial;
    std::exception_ptr _callbackError;
    CUDAStateModel _state;
    CUDAActionFactory _actions;
    CUDAObservableFactory _observables;
    CUDATopologyActionFactory _topologyActions;
};

// model::Context -> a device context; fills rx with the device id of each reference reaction id, and
// rate_functions (when given) with the device id of each spatial topology reaction that has a rate function
rdc_context *toDevice(const model::Context &ctx, std::vector<int> &rx,
                      std::vector<std::pair<int, const model::top::reactions::SpatialTopologyReaction *>>
                              *rate_functions = nullptr);

}  // namespace readdy::kernel::cuda

extern "C" const char *name();
extern "C" readdy::model::Kernel *createKernel();

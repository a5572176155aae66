/*
 * readdy_cuda.h -- C ABI of the GB300-native ReaDDy compute kernel ("CUDA" kernel plugin).
 *
 * libreaddy_cuda_core.so exports these symbols.  They take plain pointers, sizes and PODs, return an
 * int status (RDC_OK or an RDC_ERR_* code) and never throw; rdc_last_error() returns the message of
 * the calling thread's last failure.  A ReaDDy kernel plugin (model::Kernel, StateModel,
 * ActionFactory) binds one call per action.
 *
 * Each entry point names the reference interface it replaces (paths inside readdy/readdy).
 * Positions, box sizes and parameters are passed in FP64 like the reference's `scalar`
 * (include/readdy/common/common.h:62) and are held on the device in FP32; box edges are rounded to
 * FP32 on entry.  Particle ids are 64-bit on this interface and count per system from 0.
 */
#ifndef READDY_CUDA_H
#define READDY_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes; the plugin maps them onto the reference's exception types
 * (KernelProvider.cpp:188, CellLinkedList.cpp:55,245, CPUActionFactory.cpp:109) */
#define RDC_OK 0
#define RDC_ERR_INVALID_ARGUMENT 1 /* std::invalid_argument */
#define RDC_ERR_LOGIC 2            /* std::logic_error */
#define RDC_ERR_RUNTIME 3          /* std::runtime_error */
#define RDC_ERR_CUDA 4             /* a CUDA runtime call failed */
#define RDC_ERR_CAPACITY 5         /* device buffer capacity exceeded (particles or events) */

#define RDC_UNCONTROLLED_APPROXIMATION 0
#define RDC_GILLESPIE 1

typedef struct rdc_context rdc_context;
typedef struct rdc_system rdc_system;
typedef struct rdc_batch rdc_batch;

/* ---- library ---------------------------------------------------------------------------------- */
/* message of the calling thread's last failed call ("" if none) */
const char *rdc_last_error(void);
/* ABI version of this header (major*1000 + minor) */
int rdc_version(void);
/* KernelProvider plugin identity: name() of kernels/cpu .. CPUKernel.h:150-152; returns "CUDA" */
const char *rdc_kernel_name(void);
/* the GPU that the calling thread's later calls create their objects on (cudaSetDevice); objects stay
 * on the device they were created on.  No reference counterpart: the CPU kernel has no device. */
int rdc_set_device(int device);

/* ---- model::Context (include/readdy/model/Context.h) ------------------------------------------ */
/* box, periodicity, kBT (Context.h:76-108) and species with diffusion constants
 * (ParticleTypeRegistry::add, include/readdy/model/ParticleTypeRegistry.h:128-133) */
int rdc_context_create(rdc_context **out, const double box[3], const int periodic[3], double kbt, int n_types,
                       const double *diffusion);
int rdc_context_destroy(rdc_context *ctx);
/* TopologyRegistry::addSpatialReaction (readdy/main/model/topologies/TopologyRegistry.cpp:195-236;
 * SpatialTopologyReaction.h:64-191): (type1 in a topology of topology_type1) + (type2 in a topology of
 * topology_type2, or a free particle: topology_type2 = -1) -> (type_to1, topology_type_to1) +
 * (type_to2, topology_type_to2) with a constant rate within radius.  mode in STRMode order: 0 TT_ENZYMATIC,
 * 1 TT_FUSION, 2 TT_FUSION_ALLOW_SELF, 3 TP_ENZYMATIC, 4 TP_FUSION; a fusion adds the edge between the two
 * and the result takes topology_type_to1; a self fusion needs the two more than min_graph_distance edges
 * apart (the descriptor's "distance>").  At least one educt type must be TOPOLOGY flavored (checked when a
 * system is created). */
int rdc_context_add_spatial_topology_reaction(rdc_context *ctx, int mode, int type1, int topology_type1, int type2,
                                              int topology_type2, int type_to1, int topology_type_to1, int type_to2,
                                              int topology_type_to2, double rate, double radius,
                                              int min_graph_distance, int *reaction_id);
/* the rate of a topology-topology spatial reaction as a function of the two topologies (SpatialTopologyReaction's
 * rate function, SpatialTopologyReaction.h:77-99,179-191): topology1 and topology2 are the indices
 * (rdc_get_topologies order) of the topologies of the particles that take the reaction's first and second educt.
 * It is called for every candidate pair at every evaluation (CPUEvaluateTopologyReactions.cpp:296-303), with
 * the system only to be read; a rate below 0 or not a number raises RDC_ERR_RUNTIME. */
typedef double (*rdc_spatial_rate_fn)(void *user, rdc_system *s, int64_t topology1, int64_t topology2);
/* gives spatial reaction reaction_id (of rdc_context_add_spatial_topology_reaction) a rate function in place of
 * its constant rate; topology-particle modes take constant rates only (the reference's rate() throws for them) */
int rdc_context_set_spatial_topology_rate_function(rdc_context *ctx, int reaction_id, rdc_spatial_rate_fn rate,
                                                   void *user);
/* Context::legacyTopologySelfFusion: with 1, self fusions may also join vertices that share an edge */
int rdc_context_set_legacy_topology_self_fusion(rdc_context *ctx, int legacy);
/* ParticleTypeRegistry::add(name, D, flavor) (include/readdy/model/ParticleTypeRegistry.h:58-63,114):
 * 0 NORMAL (the default), 1 TOPOLOGY, 2 MEMBRANE.  Read by rdc_break_bonds. */
int rdc_context_set_particle_flavor(rdc_context *ctx, int type, int flavor);
/* Context::recordVirial (include/readdy/model/Context.h:168-174): systems created from ctx afterwards
 * accumulate the pair virial in CalculateForces */
int rdc_context_set_record_virial(rdc_context *ctx, int record);
/* Context::calculateMaxCutoff, readdy/main/model/Context.cpp:126-144 */
int rdc_context_max_cutoff(const rdc_context *ctx, double *cutoff);

/* PotentialRegistry::addHarmonicRepulsion (PotentialsOrder2.h:54-103) */
int rdc_context_add_harmonic_repulsion(rdc_context *ctx, int type1, int type2, double force_constant,
                                       double interaction_distance);
/* PotentialRegistry::addWeakInteractionPiecewiseHarmonic (PotentialsOrder2.h:105-194) */
int rdc_context_add_weak_interaction_piecewise_harmonic(rdc_context *ctx, int type1, int type2,
                                                        double force_constant, double desired_distance,
                                                        double depth, double no_interaction_distance);
/* PotentialRegistry::addLennardJones (PotentialsOrder2.h:199-272, readdy/main/model/potentials/Potentials.cpp:157-171) */
int rdc_context_add_lennard_jones(rdc_context *ctx, int type1, int type2, unsigned m, unsigned n, double cutoff,
                                  int shift, double epsilon, double sigma);
/* PotentialRegistry::addScreenedElectrostatics (PotentialsOrder2.h:274-323, Potentials.cpp:183-202) */
int rdc_context_add_screened_electrostatics(rdc_context *ctx, int type1, int type2, double electrostatic_strength,
                                            double inverse_screening_depth, double repulsion_strength,
                                            double repulsion_distance, unsigned exponent, double cutoff);

/* order-1 (external) potentials of one particle type, PotentialRegistry (PotentialRegistry.h:99-345) with
 * the classes of include/readdy/model/potentials/PotentialsOrder1.h and the geometries of
 * include/readdy/model/geometry.h.  Box and capsule also take the exclusion form of
 * addHarmonicGeometry (PotentialRegistry.h:335-345); addBox itself is inclusion. */
/* harmonic box: the box spans origin .. origin + extent */
int rdc_context_add_box(rdc_context *ctx, int type, double force_constant, const double origin[3],
                        const double extent[3], int inclusion);
int rdc_context_add_sphere(rdc_context *ctx, int type, double force_constant, const double origin[3], double radius,
                           int inclusion);
int rdc_context_add_capsule(rdc_context *ctx, int type, double force_constant, const double center[3],
                            const double direction[3], double length, double radius, int inclusion);
/* SphericalBarrier (PotentialsOrder1.h:97-152); width must not exceed radius (Potentials.cpp:86-92) */
int rdc_context_add_spherical_barrier(rdc_context *ctx, int type, double height, double width,
                                      const double origin[3], double radius);
/* Cylinder (PotentialsOrder1.h:154-209); the normal is normalised */
int rdc_context_add_cylinder(rdc_context *ctx, int type, double force_constant, const double origin[3],
                             const double normal[3], double radius, int inclusion);

/* ReactionRegistry::addConversion / addDecay / addFusion / addFission / addEnzymatic
 * (include/readdy/model/reactions/{Conversion,Decay,Fusion,Fission,Enzymatic}.h); *reaction_id is the
 * reaction's index in registration order (Reaction.h:93-96) */
int rdc_context_add_conversion(rdc_context *ctx, int type_from, int type_to, double rate, int *reaction_id);
int rdc_context_add_decay(rdc_context *ctx, int type_from, double rate, int *reaction_id);
int rdc_context_add_fusion(rdc_context *ctx, int type_from1, int type_from2, int type_to, double rate,
                           double educt_distance, double weight1, double weight2, int *reaction_id);
int rdc_context_add_fission(rdc_context *ctx, int type_from, int type_to1, int type_to2, double rate,
                            double product_distance, double weight1, double weight2, int *reaction_id);
int rdc_context_add_enzymatic(rdc_context *ctx, int type_catalyst, int type_from, int type_to, double rate,
                              double educt_distance, int *reaction_id);

/* TopologyRegistry::configureBondPotential / configureAnglePotential / configureTorsionPotential
 * (include/readdy/api/PotentialConfiguration.h:136-161; lookups are reversal-symmetric) */
int rdc_context_configure_harmonic_bond(rdc_context *ctx, int type1, int type2, double force_constant,
                                        double length);
int rdc_context_configure_harmonic_angle(rdc_context *ctx, int type1, int type2, int type3,
                                         double force_constant, double equilibrium_angle);
int rdc_context_configure_cosine_dihedral(rdc_context *ctx, int type1, int type2, int type3, int type4,
                                          double force_constant, double multiplicity, double phi0);

/* ---- model::Kernel + StateModel (include/readdy/model/{Kernel,StateModel}.h) ----------------- */
/* KernelProvider::create("CUDA") with a copy of ctx (KernelProvider.cpp:183-189); seed keys every
 * Philox stream of the system */
int rdc_system_create(rdc_system **out, const rdc_context *ctx, uint64_t seed);
int rdc_system_destroy(rdc_system *s);
/* StateModel::addParticles (StateModel.h:69-117); writes the assigned ids if ids_out != NULL */
int rdc_add_particles(rdc_system *s, int64_t n, const double *positions3, const int *types, uint64_t *ids_out);
/* StateModel::addTopology with the graph's edges (local vertex indices); builds the bond, angle and
 * dihedral term lists as GraphTopology::configure does
 * (readdy/main/model/topologies/GraphTopology.cpp:59-143, include/graphs/bits/Graph_detail.h:39-76) */
int rdc_add_topology(rdc_system *s, int64_t n, const double *positions3, const int *types, int64_t n_edges,
                     const int64_t *edges2, uint64_t *ids_out);
/* StateModel::addTopology(type, particles) (StateModel.h:69-117): rdc_add_topology with a topology type
 * id (>= 0; rdc_add_topology uses 0) that the topology and the pieces it breaks into keep */
int rdc_add_topology_typed(rdc_system *s, int topology_type, int64_t n, const double *positions3, const int *types,
                           int64_t n_edges, const int64_t *edges2, uint64_t *ids_out);
/* ActionFactory::breakBonds(timeStep, BreakConfig) + perform (include/readdy/model/actions/Actions.h:190-290):
 * BreakConfig::addBreakablePair(type1[k], type2[k], threshold_energy[k], rate[k]) for k < n_pairs (pairs
 * are unordered).  Every graph edge whose harmonic bond energy exceeds its type pair's threshold breaks
 * with probability 1 - exp(-rate time_step).  A topology that falls apart becomes its connected
 * components, of the same topology type; a component of one particle whose type has NORMAL flavor leaves
 * the topologies (include/readdy/model/actions/Utils.h:59-79).  Bonds, angles and dihedrals are derived
 * again from the remaining edges.  Unlike the reference action, which also adds the evaluated bonds'
 * forces to the particles' force accumulators (CPUTopologyActions.cpp:55-70), this leaves the forces as
 * they were until the next rdc_calculate_forces.  n_broken (may be NULL) receives the edges removed. */
int rdc_break_bonds(rdc_system *s, double time_step, int n_pairs, const int *type1, const int *type2,
                    const double *threshold_energy, const double *rate, int64_t *n_broken);
/* EvaluateTopologyReactions (kernels/cpu/src/actions/CPUEvaluateTopologyReactions.cpp:86-475) for the spatial
 * topology reactions of the context: candidate pairs found on the device, events drawn as algo::performEvents
 * draws them (proportional to rate, without replacement, an accepted event removing those that share its
 * topologies or free particle), then type changes, graph merges, self edges and particles taken into
 * topologies; bonded terms derived again.  Needs the neighbor list.  rdc_run evaluates them every step
 * between the reactions and the forces when the context has any.  n_performed may be NULL. */
int rdc_evaluate_topology_reactions(rdc_system *s, double time_step, int64_t *n_performed);
/* performed events per spatial topology reaction (n = the number registered) since creation */
int rdc_get_topology_reaction_counts(rdc_system *s, int n, int64_t *counts);

/* ---- structural topology reactions (TopologyRegistry::addStructuralReaction,
 * include/readdy/model/topologies/reactions/StructuralTopologyReaction.h): functions of the embedding ---- */
typedef struct rdc_recipe rdc_recipe;
/* rate of a structural reaction for the topology with index `topology` (rdc_get_topologies order); called
 * when the topology is created or changed (GraphTopology::updateReactionRates) and cached until then */
typedef double (*rdc_topology_rate_fn)(void *user, rdc_system *s, int64_t topology);
/* the reaction function: fills `recipe` for the topology with index `topology` (Recipe.h) */
typedef void (*rdc_topology_recipe_fn)(void *user, rdc_system *s, int64_t topology, rdc_recipe *recipe);
/* registers a structural reaction on topologies of topology_type.  Events of all topologies join the
 * spatial events of rdc_evaluate_topology_reactions.  With expect_connected a topology that falls apart
 * raises RDC_ERR_LOGIC; without it the pieces become topologies of the same type (one-particle pieces of
 * NORMAL flavor leave; StructuralTopologyReaction.cpp:70-130, Utils.h:52-81).  During the functions the
 * system may only be read (rdc_get_topology, rdc_get_topology_positions, rdc_get_topologies ...). */
int rdc_add_structural_topology_reaction(rdc_system *s, int topology_type, rdc_topology_rate_fn rate,
                                         rdc_topology_recipe_fn reaction, void *user, int expect_connected,
                                         int *reaction_id);
/* performed events per structural reaction (n = the number registered) since registration */
int rdc_get_structural_reaction_counts(rdc_system *s, int n, int64_t *counts);
/* recipe steps (Recipe.h:74-110), applied in order; vertices are local indices of the topology (the order of
 * rdc_get_topology) */
int rdc_recipe_change_particle_type(rdc_recipe *r, int64_t vertex, int type);
int rdc_recipe_add_edge(rdc_recipe *r, int64_t v1, int64_t v2);
int rdc_recipe_remove_edge(rdc_recipe *r, int64_t v1, int64_t v2);
int rdc_recipe_separate_vertex(rdc_recipe *r, int64_t vertex);
int rdc_recipe_change_topology_type(rdc_recipe *r, int type);
/* a new particle of `type` at pos3, joined to the given vertices (CPUAppendParticle,
 * include/readdy/kernel/cpu/actions/topologies/CPUTopologyActions.h:112-131); it becomes the topology's last vertex */
int rdc_recipe_append_particle(rdc_recipe *r, int64_t n_neighbors, const int64_t *neighbors, int type,
                               const double *pos3);
/* moves a vertex's particle to pos3 (wrapped into the box on periodic axes) */
int rdc_recipe_change_particle_position(rdc_recipe *r, int64_t vertex, const double *pos3);
/* one topology (index k of rdc_get_topologies): type, particle ids and types by local vertex, edges as local
 * vertex pairs; counts are written first, RDC_ERR_CAPACITY if an output does not fit; outputs may be NULL */
int rdc_get_topology(rdc_system *s, int64_t k, int *topology_type, int64_t capacity, uint64_t *ids, int *types,
                     int64_t *n_vertices, int64_t capacity_edges, int64_t *edges2, int64_t *n_edges);
/* positions of topology k's particles by local vertex */
int rdc_get_topology_positions(rdc_system *s, int64_t k, int64_t capacity, double *positions3);
/* StateModel::getTopologies (StateModel.h:69-117): the active topologies as CSR, topology k has type
 * topology_types[k] and the particles ids[offsets[k] .. offsets[k+1]) (offsets holds n_topologies + 1
 * entries).  n_topologies and n_ids are written first; RDC_ERR_CAPACITY if either capacity is smaller.
 * Any output array may be NULL. */
int rdc_get_topologies(rdc_system *s, int64_t capacity_topologies, int *topology_types, int64_t *offsets,
                       int64_t capacity_ids, uint64_t *ids, int64_t *n_topologies, int64_t *n_ids);
/* GraphTopology::graph().edges() of every active topology, in the order of rdc_get_topologies: topology k
 * has the edges edges2[2e], edges2[2e+1] (particle ids) for e in [offsets[k], offsets[k+1]) */
int rdc_get_topology_edges(rdc_system *s, int64_t capacity_topologies, int64_t *offsets, int64_t capacity_edges,
                           uint64_t *edges2, int64_t *n_topologies, int64_t *n_edges);
/* active particle count (StateModel::getParticles().size()) */
int rdc_get_n_particles(rdc_system *s, int64_t *n);
/* StateModel::getParticles: positions, types and ids of active particles; order is the device's
 * cell-sorted storage order; any output may be NULL */
int rdc_get_particles(rdc_system *s, int64_t capacity, double *positions3, int *types, uint64_t *ids,
                      int64_t *n_out);
/* Forces observable (CPUObservables.cpp): per-particle forces, same order as rdc_get_particles */
int rdc_get_forces(rdc_system *s, int64_t capacity, double *forces3, uint64_t *ids, int64_t *n_out);
/* each particle's share of the energy of the last force calculation: half of each of its pair energies,
 * its order-1 energies and the energies of the bonded terms it is listed first in; the shares sum to
 * StateModel::energy() (CPUCalculateForces.cpp:46-212 sums the same terms); same order as rdc_get_particles */
int rdc_get_particle_energies(rdc_system *s, int64_t capacity, double *energies, uint64_t *ids, int64_t *n_out);
/* StateModel::virial() after the last CalculateForces (row-major 3x3): the sum over pairs of
 * outer(-x_ij, f_i) (CPUCalculateForces.cpp:247-249); zero unless the context records the virial */
int rdc_get_virial(rdc_system *s, double *virial9);
/* Context::recordVirial for a system that exists already: ReaDDy reads the flag at every force calculation
 * (CPUCalculateForces.cpp:154), and its Virial observable sets it after particles may have been added; from the
 * next CalculateForces on the system records (1) or stops recording (0) the virial */
int rdc_set_record_virial(rdc_system *s, int record);
/* StateModel::energy() after the last CalculateForces */
int rdc_get_energy(rdc_system *s, double *energy);
/* particles advanced by the integrator since the system was created, summed over steps (the
 * particle-steps of the throughput figures; no reference counterpart) */
int rdc_get_particle_steps(rdc_system *s, uint64_t *particle_steps);
/* NParticles observable per type (kernels/cpu/src/observables/CPUObservables.cpp:153-171) */
int rdc_count_types(rdc_system *s, int64_t *counts);
/* ReactionCounts observable: performed events per reaction id since creation
 * (kernels/cpu/src/CPUStateModel.cpp:126-144) */
int rdc_get_reaction_counts(rdc_system *s, int n, int64_t *counts);
/* HistogramAlongAxis observable of the CPU kernel (kernels/cpu/src/observables/CPUObservables.cpp:85-146):
 * counts (n_borders - 1 values) of the active particles of the listed types by their coordinate on axis
 * 0..2 and std::upper_bound over the ascending borders; like the CPU kernel, the last bin is never counted */
int rdc_histogram_along_axis(rdc_system *s, int n_borders, const double *borders, int n_types, const int *types,
                             int axis, double *counts);
/* RadialDistribution observable (readdy/main/model/observables/RadialDistribution.cpp:75-128): pair counts
 * (n_borders - 1) over all ordered pairs of distinct active particles, the first of a from type and the
 * second of a to type, by their FP64 minimum-image distance; distribution = count / (4/3 pi (r_hi^3 -
 * r_lo^3) n_from particle_to_density).  A distance below the first border is not counted (the reference
 * would write before its counts). */
int rdc_radial_distribution(rdc_system *s, int n_borders, const double *borders, int n_from, const int *from_types,
                            int n_to, const int *to_types, double particle_to_density, double *counts,
                            double *distribution);
/* particle capacity on the device (reaction products beyond it raise RDC_ERR_CAPACITY) */
int rdc_reserve(rdc_system *s, int64_t capacity);
/* cell-list tuning: cells per cutoff (the reference's cll_radius, KernelConfiguration.h:63) */
int rdc_set_cell_radius(rdc_system *s, int radius);

/* ---- ActionFactory actions (include/readdy/model/actions/Actions.h:81-453) -------------------- */
/* InitializeKernel: Kernel::initialize, resets reaction counts (kernels/cpu/src/CPUKernel.cpp:63-83) */
int rdc_initialize(rdc_system *s);
/* CreateNeighborList(cutoff) = StateModel::initializeNeighborList (CPUStateModel.h:96-99) */
int rdc_nl_create(rdc_system *s, double cutoff);
/* UpdateNeighborList (CPUStateModel.h:101-103, CellLinkedList.cpp:230-247) */
int rdc_nl_update(rdc_system *s);
/* ClearNeighborList (CPUStateModel.h:170-172) */
int rdc_nl_clear(rdc_system *s);
/* CalculateForces (kernels/cpu/src/actions/CPUCalculateForces.cpp:46-212) */
int rdc_calculate_forces(rdc_system *s);
/* EulerBDIntegrator(dt) (kernels/cpu/src/actions/CPUEulerBDIntegrator.cpp:51-103) */
int rdc_euler_bd_integrate(rdc_system *s, double dt);
/* UncontrolledApproximation(dt) (kernels/cpu/src/actions/reactions/CPUUncontrolledApproximation.cpp:135-256) */
int rdc_uncontrolled_approximation(rdc_system *s, double dt);
/* Gillespie(dt) (kernels/cpu/src/actions/reactions/CPUGillespie.cpp:53-93) */
int rdc_gillespie(rdc_system *s, double dt);
/* SimulationLoop::run(n_steps) (include/readdy/api/SimulationLoop.h:256-306) on the device, captured
 * in a CUDA graph.  Per-type counts are recorded every count_stride steps including t=0 when
 * counts != NULL (n_types values per record, at most max_records records); *n_records receives the
 * number written. */
int rdc_run(rdc_system *s, int64_t n_steps, double dt, int handler, int64_t count_stride, int64_t *counts,
            int64_t max_records, int64_t *n_records);
/* neighbour pair set of the current cell list for one cutoff: every unordered pair of active
 * in-box particles with d^2 < cutoff^2 (the consumers' contract, CPUCalculateForces.cpp:240-243),
 * as (min id, max id) sorted ascending; parity/debug path */
int rdc_nl_pairs(rdc_system *s, double cutoff, int64_t capacity, uint64_t *pairs2, int64_t *n_pairs);
/* wait for the system's stream and report device-side status */
int rdc_synchronize(rdc_system *s);

/* ---- batched replicas (no reference counterpart: thousands of independent copies of one
 *      Context advanced together, one fused launch per step) ------------------------------------ */
/* n_replicas systems sharing ctx's species, potentials and reactions; boxes3 gives each replica's
 * box (FP32-rounded), capacities its particle capacity */
int rdc_batch_create(rdc_batch **out, const rdc_context *ctx, int n_replicas, const double *boxes3,
                     const int64_t *capacities, uint64_t seed);
int rdc_batch_destroy(rdc_batch *b);
/* initial particles of every replica: offsets (n_replicas+1) into positions3/types */
int rdc_batch_set_particles(rdc_batch *b, const int64_t *offsets, const double *positions3, const int *types);
/* the same from one host array per replica: counts[r] particles at positions3[r] (3 doubles each) and
 * types[r], without concatenating them first */
int rdc_batch_set_particles_list(rdc_batch *b, const int64_t *counts, const double *const *positions3,
                                 const int *const *types);
/* handler, time step and the launch knobs: cell width as a multiple (>= 1) of the largest cutoff, and
 * threads per block (one block advances one replica at a time) */
int rdc_batch_configure(rdc_batch *b, int handler, double dt, double cell_width_scale, int threads_per_block);
/* on (the default): a replica with reactions and shared-memory cells sums its pair forces in the
 * stencil walk of its event search and carries them to the next step's Euler update (two float4
 * per particle slot); off: the forces are summed at the start of every step.  Trajectories are
 * bitwise the same either way. */
int rdc_batch_set_carry_forces(rdc_batch *b, int on);
/* advance every replica n_steps; each step is one fused launch replayed from a CUDA graph */
int rdc_batch_step(rdc_batch *b, int64_t n_steps);
/* rdc_batch_step bracketed by CUDA events on the batch's stream; *device_ms receives the device time */
int rdc_batch_step_timed(rdc_batch *b, int64_t n_steps, double *device_ms);
/* particles advanced so far, summed over replicas and steps (the particle-steps of the throughput metric) */
int rdc_batch_particle_steps(rdc_batch *b, uint64_t *particle_steps);
/* per-replica, per-type counts (n_replicas * n_types) */
int rdc_batch_count_types(rdc_batch *b, int64_t *counts);
/* active particles per replica */
int rdc_batch_n_particles(rdc_batch *b, int64_t *n_per_replica);
/* particles of one replica, same layout as rdc_get_particles */
int rdc_batch_get_particles(rdc_batch *b, int replica, int64_t capacity, double *positions3, int *types,
                            uint64_t *ids, int64_t *n_out);
/* the Forces observable of one replica (kernels/cpu/src/observables/CPUObservables.cpp:177-197): the force its next Euler update applies to each particle, pair forces (carried from the
 * last event walk, or summed over the sorted state) plus order-1 potentials, in the order and with
 * the ids of rdc_batch_get_particles */
int rdc_batch_get_forces(rdc_batch *b, int replica, int64_t capacity, double *forces3, uint64_t *ids,
                         int64_t *n_out);
/* NParticles time series of every replica, streamed: from now on each replica records its per-type counts
 * (record 0 now, then after every `stride` steps of its step count, at most max_records records; the
 * NParticles observable with a stride, CPUObservables.cpp:153-171, written the way TimeSeriesWriter appends
 * a time series, include/readdy/model/observables/io/TimeSeriesWriter.h:56-92).  The records stay on the
 * device until polled. */
int rdc_batch_record_counts(rdc_batch *b, int64_t stride, int64_t max_records);
/* Trajectory observable (readdy/main/model/observables/Trajectory.cpp:100-160) of the replicas
 * replicas[0, n_replicas), streamed: a frame of their live particles is taken now and at every step
 * count that is a multiple of `stride` (as observables with a stride are evaluated), up to max_frames
 * frames (later ones are dropped).  The frames stay on the
 * device until polled; the buffer holds max_frames x the replicas' capacities.  n_replicas = 0 switches
 * the trajectory off; rdc_batch_set_particles* ends it. */
int rdc_batch_record_trajectory(rdc_batch *b, int n_replicas, const int *replicas, int64_t stride, int64_t max_frames);
/* The frames taken since the last poll, whole frames only, as many as capacity_frames and
 * capacity_entries take, copied on a stream of their own once the batch's stream has reached this call.
 * Per frame f: its step in steps[f] and, per selected replica k, its particle count in
 * counts[f * n_replicas + k]; the particles (positions3, types, ids) follow frame by frame and replica by
 * replica.  RDC_ERR_CAPACITY if not even the next frame fits (n_entries then holds its size). */
int rdc_batch_poll_trajectory(rdc_batch *b, int64_t capacity_frames, int64_t capacity_entries, int64_t *steps,
                              int64_t *counts, double *positions3, int *types, uint64_t *ids, int64_t *n_frames,
                              int64_t *n_entries);
/* copies the records written since the last poll (at most capacity records): steps[k] is the time step of
 * record k, counts holds n_replicas * n_types values per record (record-major).  The copy runs on a stream
 * of its own after the steps already queued; the batch's own stream keeps going.  *n_out = records copied */
int rdc_batch_poll_count_records(rdc_batch *b, int64_t capacity, int64_t *steps, int64_t *counts, int64_t *n_out);
/* the Virial observable of every replica (Context::recordVirial, CPUCalculateForces.cpp:247-249): the pair
 * virial of the forces its next Euler update applies, row-major 3x3 per replica (n_replicas * 9).  Taken
 * from forces summed over the sorted state, so carried forces must be off (rdc_batch_set_carry_forces(b, 0);
 * RDC_ERR_LOGIC otherwise) */
int rdc_batch_get_virial(rdc_batch *b, double *virial9);
/* performed events per replica and reaction since the batch was created (n_replicas * n, by reaction
 * id; the ReactionCounts observable, CPUStateModel.cpp:126-144, of every replica) */
int rdc_batch_reaction_counts(rdc_batch *b, int n, int64_t *counts);
/* the cell grid a replica runs on (cells per axis) and whether its cell starts live in shared memory
 * during a step (1) or in global memory (0) */
int rdc_batch_replica_grid(rdc_batch *b, int replica, int *dims3, int *shared_cells);
int rdc_batch_synchronize(rdc_batch *b);

/* ---- served form (no reference counterpart: a request loop over independent simulations) --------
 * Requests of different sizes and chemistries arrive with their own context, particles, step count,
 * time step, count stride (per-type counts at t = 0 and every count_stride steps, like the NParticles
 * observable, CPUObservables.cpp:153-171) and seed.  They are admitted first come, first served, while
 * the device bytes of the admitted requests stay within budget_bytes; each keeps its particle state in
 * device memory until it finishes.  Requests of up to plain_threshold particles (0: all) run together
 * in the fused replica engine, one launch per step; larger ones run as per-system simulations on their
 * own stream.  A request's result depends only on the request, not on the others in the mix. */
typedef struct rdc_server rdc_server;
int rdc_server_create(rdc_server **out, uint64_t budget_bytes, int max_active, int handler, int64_t plain_threshold);
int rdc_server_destroy(rdc_server *s);
/* how many per-system requests run at once, each on its own stream and pool thread (default 24) */
int rdc_server_set_plain_workers(rdc_server *s, int n);
/* device bytes a request would hold while active, and whether it would take the per-system leg
 * (host arithmetic only, no device needed) */
int rdc_server_request_bytes(const rdc_context *ctx, int64_t n, int64_t n_steps, int64_t count_stride,
                             int64_t plain_threshold, uint64_t *bytes, int *plain);
/* queue a request (the context is copied); *request_id identifies it from now on.  A request larger than
 * the whole budget returns RDC_ERR_INVALID_ARGUMENT. */
int rdc_server_submit(rdc_server *s, const rdc_context *ctx, int64_t n, const double *positions3, const int *types,
                      int64_t n_steps, double dt, int64_t count_stride, uint64_t seed, int64_t *request_id);
/* admit what fits, advance the engine requests by up to max_steps engine launches (fewer when one of them
 * finishes first; in one launch a request takes as many steps as fit into one step of the largest active
 * engine request), retire finished requests of both legs */
int rdc_server_progress(rdc_server *s, int64_t max_steps, int64_t *n_finished);
/* ids of requests finished since the last poll */
int rdc_server_poll(rdc_server *s, int64_t capacity, int64_t *ids, int64_t *n_out);
/* count records (n_records x n_types of the request's context), status (-1 while unfinished) and the
 * submit, admit and finish times in seconds since the server was created */
int rdc_server_result(rdc_server *s, int64_t id, int64_t capacity, int64_t *counts, int64_t *n_records, int *status,
                      double *times3);
/* The count records request `id` has written so far, streamed while it runs: a request in the engine leg
 * shows the records of the steps done by the last rdc_server_progress call, a per-system request those of
 * its completed chunks (its run goes in chunks of about 2000 steps, a whole number of strides), a finished
 * request all of them (as rdc_server_result).  n_records is written first; RDC_ERR_CAPACITY if capacity
 * (in int64 entries) is below n_records x ntypes.  counts may be NULL. */
int rdc_server_peek_records(rdc_server *s, int64_t id, int64_t capacity, int64_t *counts, int64_t *n_records);
/* forget a finished request */
int rdc_server_release(rdc_server *s, int64_t id);
/* particles advanced so far (summed over requests and steps), device bytes held by admitted requests,
 * requests running and waiting */
int rdc_server_stats(rdc_server *s, uint64_t *particle_steps, uint64_t *bytes_in_use, int64_t *n_active,
                     int64_t *n_pending);

/* ---- forces without device allocation (no counterpart in the reference) ----------------------
 * For callers that cannot let the library call cudaMalloc where they need forces: embeddings whose
 * own pool owns all of the GPU's memory (an MD engine, a framework with its own caching allocator, a
 * service that carves HBM into fixed pools) and step loops that must not stall on the allocator.
 * Pair forces and the pair energy of n particles held in the caller's device arrays -- positions3
 * (n*3 floats), types (n ints in [0, n_types)) -- are written to the caller's device arrays forces3
 * (n*3 floats) and *energy (one double), on `stream` (a cudaStream_t; NULL is the legacy default
 * stream), asynchronously.  Same pair potentials, exact cutoff test and FP32 terms as
 * rdc_calculate_forces; the neighbour summation order may differ.  The context's order-1 (external)
 * potentials are not applied here.  Positions on a periodic axis must lie in [-L/2, L/2), the range
 * bcs::fixPosition keeps them in; on a closed axis a particle outside the box gets no force, as in the
 * reference's cell list.
 *
 * Working space is one static device array of RDC_NOALLOC_SCRATCH_BYTES per device, so at most
 * RDC_NOALLOC_MAX_PARTICLES particles are accepted (more returns RDC_ERR_INVALID_ARGUMENT) and the
 * cell grid is widened to at most RDC_NOALLOC_MAX_CELLS cells.  The first call on a device, and the
 * first call after the context's potentials changed, finds the array (cudaGetSymbolAddress with that
 * device current) and copies the potential tables into it, synchronising the stream; that call should
 * come before any stream capture (during capture it returns RDC_ERR_LOGIC).  All calls on one device
 * share the array and it keeps the last call's contents: calls that overlap on the GPU (different
 * streams or threads without ordering) race and give wrong results; when such a call has replaced
 * the tables with another context's, the forces and *energy come out NaN.  A type outside
 * [0, n_types), a coordinate that is not a number, or one outside the box on a periodic axis gives
 * that particle no force and makes *energy NaN. */
#define RDC_NOALLOC_MAX_PARTICLES 65536
#define RDC_NOALLOC_MAX_CELLS 131072
#define RDC_NOALLOC_SCRATCH_BYTES 3185408
int rdc_forces_noalloc(const rdc_context *ctx, int64_t n, const float *positions3, const int *types,
                       float *forces3, double *energy, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* READDY_CUDA_H */

/*
 * TEST INFRASTRUCTURE ONLY -- not part of the product.
 *
 * C interface of the FP64 CPU restatement of ReaDDy's CPU-kernel hot path (cell-linked neighbour
 * list, pair and bonded forces, Euler Brownian dynamics, uncontrolled-approximation and Gillespie
 * reaction handlers).  Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg load it,
 * as the checker the CUDA path is compared against.
 *
 * Indices ("storage indices") follow the reference data container: particles live in a vector with
 * blanks that are reused LIFO (kernels/cpu .. DefaultDataContainer.h:79-139).
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_system orc_system;
/* structural topology reactions: functions of the caller (StructuralTopologyReaction.h) */
typedef struct orc_recipe orc_recipe;
typedef double (*orc_topology_rate_fn)(void *user, orc_system *s, int64_t topology);
/* SpatialTopologyReaction's rate function (SpatialTopologyReaction.h:77-99,179-191): the rate of a
 * topology-topology event from the topologies of its two particles, in the order the reference lists them
 * (CPUEvaluateTopologyReactions.cpp:296-303) */
typedef double (*orc_spatial_rate_fn)(void *user, orc_system *s, int64_t topology1, int64_t topology2);
typedef void (*orc_topology_recipe_fn)(void *user, orc_system *s, int64_t topology, orc_recipe *recipe);

enum orc_handler { ORC_UNCONTROLLED_APPROXIMATION = 0, ORC_GILLESPIE = 1 };

orc_system *orc_create(const double box[3], const int periodic[3], double kbt, int n_types,
                       const double *diffusion, uint64_t seed, int n_threads, int cll_radius);
void orc_destroy(orc_system *s);
const char *orc_last_error(void);

/* pair potentials (PotentialsOrder2.h); return 0 on success */
/* order-1 (external) potentials (include/readdy/model/potentials/PotentialsOrder1.h) */
int orc_add_box(orc_system *s, int type, double k, const double *origin3, const double *extent3, int inclusion);
int orc_add_sphere(orc_system *s, int type, double k, const double *origin3, double radius, int inclusion);
int orc_add_capsule(orc_system *s, int type, double k, const double *center3, const double *direction3, double length,
                    double radius, int inclusion);
int orc_add_spherical_barrier(orc_system *s, int type, double height, double width, const double *origin3,
                              double radius);
int orc_add_cylinder(orc_system *s, int type, double k, const double *origin3, const double *normal3, double radius,
                     int inclusion);
/* Context::recordVirial and StateModel::virial() (row-major 3x3) of the last force calculation */
int orc_set_record_virial(orc_system *s, int record);
int orc_get_virial(const orc_system *s, double *out9);
int orc_add_harmonic_repulsion(orc_system *s, int t1, int t2, double k, double interaction_distance);
int orc_add_weak_interaction_piecewise_harmonic(orc_system *s, int t1, int t2, double k, double desired_distance,
                                                double depth, double no_interaction_distance);
int orc_add_lennard_jones(orc_system *s, int t1, int t2, unsigned m, unsigned n, double cutoff, int shift,
                          double epsilon, double sigma);
int orc_add_screened_electrostatics(orc_system *s, int t1, int t2, double electrostatic_strength,
                                    double inverse_screening_depth, double repulsion_strength,
                                    double repulsion_distance, unsigned exponent, double cutoff);

/* reactions (include/readdy/model/reactions); return reaction id >= 0 or -1 */
int orc_add_conversion(orc_system *s, int from, int to, double rate);
int orc_add_decay(orc_system *s, int from, double rate);
int orc_add_fusion(orc_system *s, int from1, int from2, int to, double rate, double educt_distance, double w1,
                   double w2);
int orc_add_fission(orc_system *s, int from, int to1, int to2, double rate, double product_distance, double w1,
                    double w2);
int orc_add_enzymatic(orc_system *s, int catalyst, int from, int to, double rate, double educt_distance);

/* bonded terms of static topologies, indices are storage indices */
int orc_add_harmonic_bonds(orc_system *s, int n, const int *idx2, const double *k, const double *l0);
int orc_add_harmonic_angles(orc_system *s, int n, const int *idx3, const double *k, const double *theta0);
int orc_add_cosine_dihedrals(orc_system *s, int n, const int *idx4, const double *k, const double *multiplicity,
                             const double *phi0);

/* topology registry (PotentialConfiguration.h:136-161), particle flavors, topologies with their graphs
 * (bonded terms derived as GraphTopology::configure does; explicit terms above are kept beside them) and
 * BreakBonds (Actions.h:236-290) */
int orc_set_particle_flavor(orc_system *s, int type, int flavor);
int orc_configure_harmonic_bond(orc_system *s, int t1, int t2, double k, double l0);
int orc_configure_harmonic_angle(orc_system *s, int t1, int t2, int t3, double k, double theta0);
int orc_configure_cosine_dihedral(orc_system *s, int t1, int t2, int t3, int t4, double k, double mult, double phi0);
int orc_add_topology(orc_system *s, int type, int n, const double *pos3, const int *types, int n_edges,
                     const int *edges2, uint64_t *ids_out);
int orc_break_bonds(orc_system *s, double dt, int n, const int *t1, const int *t2, const double *threshold,
                    const double *rate, int64_t *n_broken);
int orc_get_topologies(const orc_system *s, int *types, int64_t *offsets, uint64_t *ids, int64_t *n_top,
                       int64_t *n_ids);
int orc_get_topology_edges(const orc_system *s, int64_t *offsets, uint64_t *edges2, int64_t *n_edges);
/* spatial topology reactions (TopologyRegistry::addSpatialReaction; mode in STRMode order, tt2 = -1 for a free
 * particle) and EvaluateTopologyReactions (kernels/cpu/src/actions/CPUEvaluateTopologyReactions.cpp) */
int orc_add_spatial_topology_reaction(orc_system *s, int mode, int t1, int tt1, int t2, int tt2, int to1, int tto1,
                                      int to2, int tto2, double rate, double radius, int min_graph_distance);
int orc_set_legacy_topology_self_fusion(orc_system *s, int legacy);
int orc_evaluate_topology_reactions(orc_system *s, double dt, int64_t *n_performed);
int orc_topology_reaction_counts(const orc_system *s, int64_t *counts, int n);
int orc_set_spatial_topology_rate_function(orc_system *s, int reaction_id, orc_spatial_rate_fn rate, void *user);
int orc_add_structural_topology_reaction(orc_system *s, int topology_type, orc_topology_rate_fn rate,
                                         orc_topology_recipe_fn reaction, void *user, int expect_connected);
int orc_structural_reaction_counts(const orc_system *s, int64_t *counts, int n);
/* recipe steps (Recipe.h:74-110), vertices by local index */
int orc_recipe_change_particle_type(orc_recipe *r, int64_t vertex, int type);
int orc_recipe_add_edge(orc_recipe *r, int64_t v1, int64_t v2);
int orc_recipe_remove_edge(orc_recipe *r, int64_t v1, int64_t v2);
int orc_recipe_separate_vertex(orc_recipe *r, int64_t vertex);
int orc_recipe_change_topology_type(orc_recipe *r, int type);
int orc_recipe_append_particle(orc_recipe *r, int64_t n_neighbors, const int64_t *neighbors, int type, const double *pos3);
int orc_recipe_change_particle_position(orc_recipe *r, int64_t vertex, const double *pos3);
/* topology k: type, particle ids, types and positions by local vertex, edges as local pairs (outputs may be NULL) */
int orc_get_topology(const orc_system *s, int64_t k, int *type, uint64_t *ids, int *types, double *pos3,
                     int64_t *n_vertices, int64_t *edges2, int64_t *n_edges);

/* particles */
int orc_add_particles(orc_system *s, int n, const double *pos3, const int *types);
int orc_n_particles(const orc_system *s);       /* active */
int orc_n_entries(const orc_system *s);         /* storage size incl. blanks */
/* active particles in storage order; any output pointer may be NULL */
int orc_get_particles(const orc_system *s, double *pos3, int *types, uint64_t *ids, double *force3,
                      int *storage_index);
double orc_calculate_max_cutoff(const orc_system *s);
/* per active particle (storage order): sum over the force terms of the last CalculateForces of their
 * magnitudes -- the scale of the rounding error of an FP32 evaluation of the same sum */
int orc_get_force_scales(const orc_system *s, double *out);

/* neighbour list (CellLinkedList.cpp) */
int orc_nl_setup(orc_system *s, double cutoff);
int orc_nl_update(orc_system *s);
/* candidate pairs from the cell list, each unordered pair once, filtered by d^2 < cutoff^2;
 * writes particle ids (min,max) sorted ascending; returns the number of pairs or -1 if cap too small */
int64_t orc_nl_pairs(const orc_system *s, double cutoff, int64_t cap, uint64_t *pairs);
int64_t orc_brute_force_pairs(const orc_system *s, double cutoff, int64_t cap, uint64_t *pairs);

/* actions */
double orc_calculate_forces(orc_system *s);     /* returns total energy */
double orc_energy(const orc_system *s);
int orc_euler_bd(orc_system *s, double dt);
int orc_uncontrolled_approximation(orc_system *s, double dt);
int orc_gillespie(orc_system *s, double dt);
/* SimulationLoop::run step order; counts (n_types per record) every count_stride steps incl. t=0,
 * returns the number of records written (counts may be NULL) */
int orc_run(orc_system *s, int64_t n_steps, double dt, int handler, int count_stride, int64_t *counts,
            int64_t max_records);
/* per-reaction count of performed events accumulated since creation */
int orc_reaction_counts(const orc_system *s, int64_t *counts, int cap);
/* HistogramAlongAxis observable of the CPU kernel: counts (n_borders - 1 values) of the active particles of
 * the listed types along one axis */
int orc_histogram_along_axis(const orc_system *s, int n_borders, const double *borders, int n_types,
                             const int *types, int axis, double *counts);
/* RadialDistribution observable: pair counts (n_borders - 1) over ordered pairs of distinct particles (from
 * types x to types) and the distribution normalised by shell volume, from-particle count and density */
int orc_radial_distribution(const orc_system *s, int n_borders, const double *borders, int n_from,
                            const int *from_types, int n_to, const int *to_types, double particle_to_density,
                            double *counts, double *distribution);

#ifdef __cplusplus
}
#endif

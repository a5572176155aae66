// Host-side structures of the CUDA core: the context registries, the device tables built from
// them, and the per-system device state.  Internal to libreaddy_cuda_core.so.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/readdy_cuda.h"
#include "rdc_types.h"

namespace rdc {

// ---- errors -----------------------------------------------------------------------------------
struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct CapacityError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

#define RDC_CUDA(call)                                                                                 \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            throw ::rdc::CudaError(std::string(#call) + ": " + cudaGetErrorString(e_));                \
    } while (0)

// ---- context (model::Context) -------------------------------------------------------------------
struct HostPot {
    int t1, t2;
    PairPot pot;
    double cutoff;
};
struct HostReaction {
    int kind, n_educts, n_products;
    int educt[2], product[2];
    double rate, educt_distance, product_distance, w1, w2;
};
struct HostO1 {
    int type;
    int kind, inclusion;
    double k, a[3], b[3], radius, length, height, width;
};
struct BondCfg { int t1, t2; double k, l0; };
struct AngleCfg { int t1, t2, t3; double k, theta0; };
struct DihedralCfg { int t1, t2, t3, t4; double k, mult, phi0; };

// particle flavors (include/readdy/model/ParticleTypeRegistry.h:58-63)
constexpr int FLAVOR_NORMAL = 0, FLAVOR_TOPOLOGY = 1, FLAVOR_MEMBRANE = 2;

// spatial topology reaction (include/readdy/model/topologies/reactions/SpatialTopologyReaction.h:64-191):
// educts (t1 in a topology of type tt1) + (t2 in a topology of type tt2, or tt2 = -1: a free particle),
// products (to1, tto1) and (to2, tto2); fusions add the edge to1 -- to2 and the merged topology takes
// tto1.  Modes in STRMode order.
enum : int { STR_TT_ENZYMATIC = 0, STR_TT_FUSION = 1, STR_TT_FUSION_ALLOW_SELF = 2, STR_TP_ENZYMATIC = 3,
             STR_TP_FUSION = 4 };
struct SpatialTopReaction {
    int mode;
    int t1, tt1, t2, tt2, to1, tto1, to2, tto2;
    double rate, radius;
    int min_graph_distance;  // self fusion: vertices at most this far apart in the graph do not react
    rdc_spatial_rate_fn rate_fn = nullptr;  // topology-topology modes: the rate from the two topologies
    void *rate_user = nullptr;
};

struct ContextData {
    double box[3];
    int pbc[3];
    double kbt;
    int ntypes;
    bool record_virial = false;  // Context::recordVirial (include/readdy/model/Context.h:168-174)
    std::vector<double> D;
    std::vector<int> flavor;  // per type: FLAVOR_NORMAL, FLAVOR_TOPOLOGY or FLAVOR_MEMBRANE
    std::vector<HostPot> pots;
    std::vector<HostO1> o1pots;
    std::vector<HostReaction> reactions;
    std::vector<BondCfg> bonds;
    std::vector<AngleCfg> angles;
    std::vector<DihedralCfg> dihedrals;
    std::vector<SpatialTopReaction> spatial_top;
    bool legacy_self_fusion = false;  // Context::legacyTopologySelfFusion: graph neighbours may self-fuse

    double max_cutoff() const;
    bool structural_reactions() const;  // fusion, fission or decay present (particles appear/vanish/move)
};

// device-resident tables: potentials by type pair, reactions by educt types, per-type integration
struct Tables {
    int ntypes, npots, nreactions;
    int has_o2_any;
    float bd_drift[MAX_TYPES];  // D dt / kBT
    float bd_scale[MAX_TYPES];  // sqrt(2 D dt)
    int pair_tab[MAX_TYPES * MAX_TYPES];  // (first << 8) | count into pots, 0 = none
    float pair_screen[MAX_TYPES * MAX_TYPES];  // largest cutoff^2 + band of the pair's potentials (screening)
    float rx_screen[MAX_TYPES * MAX_TYPES];    // largest educt distance^2 + band of the pair's reactions
    PairPot pots[MAX_PAIR_POTENTIALS];
    ReactionDev reactions[MAX_REACTIONS];
    int o1_tab[MAX_TYPES];                 // (first << 8) | count into o1_list
    int o1_list[MAX_REACTIONS];
    int o2_tab[MAX_TYPES * MAX_TYPES];     // (first << 8) | count into o2_list
    int o2_list[MAX_REACTIONS * 2];
    int o2_any[MAX_TYPES];                 // type has any order-2 reaction
    int o1pot_tab[MAX_TYPES];              // (first << 8) | count into o1pots
    O1Pot o1pots[MAX_O1_POTENTIALS];
};

// builds the tables from a context for a box (band widths depend on the GPU machine) and time step
void build_tables(const ContextData &c, const double box[3], double dt, Tables &t);
void set_time_step(const ContextData &c, double dt, Tables &t);
// FP32-rounded box, cell grid for cutoff/radius with cells at least min_width wide
Geo make_geo(const double box[3], const int pbc[3], double cutoff, int radius, double min_width = 0.0);

// ---- per-system device state -------------------------------------------------------------------
enum Counter : int {
    C_N = 0,         // particles in storage (cells + OUT), sorted
    C_N_TOTAL = 1,   // including particles appended by reactions since the last sort
    C_N_INCELLS = 2, // particles inside cells (storage [0, C_N_INCELLS))
    C_STATUS = 3,    // Status bits
    C_N_EVENTS = 4,
    C_NEXT_ID = 5,
    C_REC = 6,       // observable records written
    C_N_BIRTHS = 7,  // births of the last reaction step (host statistics)
    C_BIG = 8,       // cells with more than CELL_SORT_SMALL entries found by the last sort
    C_DONE = 9,      // blocks finished in the current launch (the last one advances a step or record counter)
    C_COUNT = 10
};

struct SysDev {
    Geo geo;
    int radius;
    const Tables *tab;
    float4 *pos;
    uint32_t *id;
    int *tslot;
    float4 *force;
    float4 *pos_alt;
    uint32_t *id_alt;
    int *tslot_alt;
    float4 *force_alt;
    int *bin, *rank, *src;
    int *big_cells;  // cells too full for the per-thread insertion sort (capacity ncells)
    int *cnt, *start;
    int *scan_blocks;
    int *tloc;
    int *counters;
    uint64_t *step;
    int capacity;
    uint64_t seed;
    // reactions
    EventRec *events;
    int event_capacity;
    int *claim;
    int *taken;
    unsigned long long *reaction_counts;
    // energy
    double *epart;     // per-block partial energies (pair kernel blocks, then bonded blocks)
    double *energy;
    double *vpart;     // per-block partial virials (9 per pair kernel block); null: virial not recorded
    double *virial;    // row-major 3x3 pair virial of the last force calculation
    // bonded (topology slots)
    int n_top;             // topology slots whose bonded terms are live
    int tloc_size;         // slots covered by tloc
    const int *top_off;    // CSR offsets per topology slot
    const int *top_terms;  // (kind << 28) | (role << 24) | term index
    const int4 *bond_idx;  // slots (i, j, -, -)
    const float4 *bond_par;  // (k, l0, l0^2 hi, l0^2 lo)
    const int4 *angle_idx;
    const float4 *angle_par; // (k, theta0, pi - theta0, -)
    const int4 *dih_idx;
    const float4 *dih_par;
    // where each term's role forces go: its entries in top_terms (bond: x, y; angle: x, y, z; dihedral:
    // x, y, z, w), and the per-entry forces (w: the term's energy on its role-0 entry)
    int n_bonds, n_angles, n_dihedrals;
    const int2 *bond_at;
    const int4 *angle_at;
    const int4 *dih_at;
    float4 *term_force;
    // observables
    unsigned long long *counts_ring;
    int counts_stride;
    int counts_max;
    uint64_t rec_base;  // BD step at which the current recording started
};

constexpr int FORCE_BLOCKS = 4 * 152;
constexpr int FORCE_THREADS = 256;
#ifndef RDC_BONDED_BLOCKS
#define RDC_BONDED_BLOCKS (4 * 152)
#endif
constexpr int BONDED_BLOCKS = RDC_BONDED_BLOCKS;
constexpr int GRID_BLOCKS = 8 * 152;
constexpr int GRID_THREADS = 256;

// ---- launchers (rdc_kernels.cu) -----------------------------------------------------------------
void launch_integrate_bin(const SysDev &s, bool integrate, cudaStream_t st);
void launch_bin(const SysDev &s, cudaStream_t st);
void launch_sort(const SysDev &s, bool permute_force, cudaStream_t st);  // scan, scatter, per-cell order, gather
// pair (and bonded) forces; with finals the energy and virial reductions follow (a run does them once
// after its last step instead, see launch_force_finals)
void launch_forces(const SysDev &s, bool pair, bool bonded, cudaStream_t st, bool finals = true);
void launch_force_finals(const SysDev &s, bool bonded, cudaStream_t st);
void launch_events(const SysDev &s, int handler, cudaStream_t st);
void launch_resolve_apply(const SysDev &s, int handler, cudaStream_t st);
void launch_count_types(const SysDev &s, unsigned long long *out, cudaStream_t st);
// HistogramAlongAxis / RadialDistribution bin counts into out (nb - 1 zeroed counters)
void launch_histogram_axis(const SysDev &s, const double *borders, int nb, uint32_t types, int axis,
                           unsigned long long *out, cudaStream_t st);
void launch_radial_distribution(const SysDev &s, int n, const double *borders, int nb, uint32_t from, uint32_t to,
                                float reach2, unsigned long long *out, cudaStream_t st);
void launch_record_counts(const SysDev &s, cudaStream_t st);
void launch_step_advance(const SysDev &s, cudaStream_t st);
void launch_pairs(const SysDev &s, float c2f, float band, double c2, uint64_t *out, int cap, int *n_out,
                  cudaStream_t st);
void launch_fill_ids(uint32_t *id, uint32_t first, int n, cudaStream_t st);
// spatial topology reaction candidates: pairs (i < j) of particles in cells whose types pair_mask names
// (bit u of pair_mask[t]) within sqrt(r2max), as TopCandidate records; the count in out_n (capped at cap)
struct TopCandidate {
    int i, j;          // storage indices
    int ti, tj;        // particle types
    int si, sj;        // topology slots (-1: none)
    uint32_t idi, idj;
    double d2;         // squared minimum-image distance in FP64 from the FP32 positions
};
// (r2screen: an FP32 screen above r2max by the rounding of an FP32 squared distance)
void launch_topology_candidates(const SysDev &s, const uint32_t *pair_mask, double r2max, float r2screen,
                                TopCandidate *out, int *out_n, int cap, cudaStream_t st);
// writes (storage index, new type, new topology slot or -1 to keep, 0) edits; a new slot also maps to the
// index; with w = 1 the x names the topology slot of the particle instead of its storage index
void launch_particle_edits(const SysDev &s, const int4 *edits, int n, cudaStream_t st);
void launch_gather_slots(const SysDev &s, const int *slots, int n, float4 *out, cudaStream_t st);
void launch_position_edits(const SysDev &s, const int2 *targets, const float4 *to, int n, cudaStream_t st);
// edges: (slot1, slot2, first bond term, bond terms); thr and coin: T x T per type pair
void launch_break_bonds(const SysDev &s, const int4 *edges, int n_edges, const double2 *bond_kl, const double *thr,
                        const uint64_t *coin, int T, uint64_t seed, uint64_t counter, int *out, int *out_n,
                        cudaStream_t st);
int scan_block_count(int n);
size_t resolve_smem_bytes();
void init_kernel_attributes();

}  // namespace rdc

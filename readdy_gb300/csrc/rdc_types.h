// Plain data shared by host orchestration and device kernels.
#pragma once
#include <cstdint>

namespace rdc {

constexpr int MAX_TYPES = 32;          // particle species per system
constexpr int MAX_PAIR_POTENTIALS = 128;
constexpr int MAX_REACTIONS = 64;
constexpr int MAX_O1_POTENTIALS = 64;  // order-1 (external) potentials per system
constexpr int RESOLVE_MAX_EVENTS = 8192;  // accepted events one step may resolve (device-checked)

enum PotKind : int {
    POT_HARMONIC_REPULSION = 0,
    POT_WEAK_PIECEWISE_HARMONIC = 1,
    POT_LENNARD_JONES = 2,
    POT_SCREENED_ELECTROSTATICS = 3,
};

// order-1 (external) potentials, include/readdy/model/potentials/PotentialsOrder1.h
enum O1Kind : int { O1_BOX = 0, O1_SPHERE = 1, O1_CAPSULE = 2, O1_SPHERICAL_BARRIER = 3, O1_CYLINDER = 4 };

// Parameters in FP32 (positions are FP32 on the device).  Layouts of p[]:
//   box:      k, v0[3], v1[3]
//   sphere:   k, centre[3], radius, radius^2 (hi, lo)
//   capsule:  k, centre[3], unit direction[3] (hi), length/2, radius, radius^2 (hi, lo), direction (lo)
//   barrier:  centre[3], radius, width, height, keff, r1, r2, r3, r4, radius^2 (hi, lo)
//   cylinder: k, origin[3], unit normal[3] (hi), radius, radius^2 (hi, lo), normal (lo)
struct O1Pot {
    int kind;
    int inclusion;
    float p[14];
};

enum ReactionKind : int { R_CONVERSION = 0, R_FUSION = 1, R_FISSION = 2, R_ENZYMATIC = 3, R_DECAY = 4 };

enum Handler : int { H_UNCONTROLLED_APPROXIMATION = 0, H_GILLESPIE = 1 };

// status bits raised on the device, read by the host after a step
enum Status : int {
    ST_CAPACITY = 1,       // particle capacity exceeded by reaction products
    ST_EVENTS = 2,         // event buffer overflow
    ST_ID_OVERFLOW = 4,    // 32-bit particle id counter exhausted
    ST_RESOLVE_ROUNDS = 8, // conflict resolution did not converge within its round limit
    ST_TYPE = 16,          // particle type out of range
    ST_INDEX = 32,         // a replica step met a storage index outside its particles (access skipped)
};

struct Geo {
    float L[3], hL[3], invW[3];
    double Ld[3];
    int pbc[3];
    int dims[3];
    int ncells;
    int exact_always;  // FP64 pair predicate for every candidate (box small relative to cutoff)
};

struct PairPot {
    int kind;
    int pad;
    float p[12];
    double cutoff2;   // FP64 squared cutoff, computed as the reference does
    float cutoff2f;
    float band;       // half-width of the FP32 rounding band around cutoff2f
};

struct ReactionDev {
    int kind;
    int n_educts, n_products;
    int educt[2], product[2];
    int id;
    float w1, w2, product_distance;
    float educt_distance2f, band;
    double educt_distance2;
    double rate;
    float inv_rate;      // 1 / rate (0 when the rate is 0)
    int active;          // rate > 0: the reaction takes part in event generation
    uint64_t coin_threshold;  // floor((1 - exp(-rate dt)) * 2^64), refreshed when dt changes
};

// accepted reaction event, before conflict resolution
struct EventRec {
    uint64_t key;   // priority (smaller wins); ties impossible in practice, broken by index
    int p1, p2;     // particle slots (p2 == p1 for order-1)
    int reaction;   // index into the reaction table
    int pad;
};

}  // namespace rdc

// The fused replica engine shared by the batched form (rdc_batch.cu) and the served form
// (rdc_serve.cu).  A replica is one independent system: its own box, particles, seed, step counter
// and reaction/potential tables.  Every step is ONE persistent launch over the replicas of a work
// list: each CTA takes replicas from a work counter (largest first) and runs the whole step of one
// replica in block-level phases (the served form lets a small replica take several steps in a launch)
//
//   forces (pair stencil) -> Euler BD -> bin -> counting sort -> reaction events -> conflict
//   resolution + application -> (re-sort if particles appeared or vanished) -> observables
//
// The arithmetic is the per-system path's (rdc_phases.cuh), so a replica gives the same trajectory
// alone, inside any batch or request mix, or through rdc_run with the replica's seed.  Forces act on
// the state left by the previous step's reactions, which is where SimulationLoop::run computes them
// (SimulationLoop.h:283-289).  A replica with reactions and shared-memory cells computes them one
// walk earlier: the stencil walk that looks for reaction partners after the sort also sums every
// particle's pair force and stores it.  Its reactions then change the state in place (removed
// particles keep their slots, births are appended) and no re-sort follows; only particles whose
// 27-cell stencil held a reacting particle walk again, over that state, with the candidates in the
// order of the sorted one.  Every sort orders a cell by particle id, so the sorted order does not
// depend on the order of the source arrays, and the stored forces are the ones a walk over the
// sorted final state gives, bit for bit.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "rdc_host.h"

namespace rdc {

// Cell counts and starts of a replica of fewer than 65536 particles live in shared memory during its
// step as uint16_t, SMEM_CELLS entries (92 KB): at cells of the cutoff's width and density 0.25 that
// holds replicas of up to ~11.7k particles, and larger ones get proportionally wider cells.  Replicas
// of more particles keep int starts in global memory at the natural cell width.  The size keeps one
// CTA's shared memory within the 164 KB configuration, so that 92 KB of the SM stay L1 for the
// neighbour positions (measured: 6.49 ms per step of the 4096-replica ensemble against 6.93 ms with
// 49152 entries and the 196 KB configuration, and 6.75 ms with 32768 entries).
#ifndef RDC_ENGINE_SMEM_CELLS
#define RDC_ENGINE_SMEM_CELLS 47104
#endif
#ifndef RDC_ENGINE_MAX_EVENTS_SM
#define RDC_ENGINE_MAX_EVENTS_SM 1024
#endif
// The launch bound of the fused step, which also caps its registers (65536 / 768 -> 80 per thread).
// Measured on the 4096-replica ensemble (one CTA per SM, the shared-memory cell array above): 4.88 ms
// per step at 512 threads and 128 registers, 4.33 ms at 640 threads and 96 registers, 4.02 ms at 768
// and 80 (84 bytes of spills), 4.03 ms at 896 and 72 (596 bytes of spills).  The walk phases are bound
// by the latency of dependent loads and arithmetic; more warps per SM hide more of it.
#ifndef RDC_ENGINE_THREADS_MAX
#define RDC_ENGINE_THREADS_MAX 768
#endif
constexpr int SMEM_CELLS = RDC_ENGINE_SMEM_CELLS;
constexpr int ENGINE_THREADS_MAX = RDC_ENGINE_THREADS_MAX;
// accepted events one replica step resolves in shared memory (more raise ST_EVENTS)
constexpr int ENGINE_MAX_EVENTS_SM = RDC_ENGINE_MAX_EVENTS_SM;

struct RepDesc {
    Geo geo;
    float4 *pos[2];              // double buffer; state.cur selects the current one
    uint32_t *id[2];
    float4 *force[2];            // pair forces on pos[k] between steps (null: summed at the step start)
    int *bin, *rank, *src, *claim, *taken;   // capacity entries each
    int *start;                  // cell starts between steps, ncells + 3 entries
    EventRec *events;            // ecap entries
    unsigned long long *records; // per-type counts, max_records x ntypes (null: none)
    unsigned long long *rx_counts;  // performed events per reaction (null: none)
    uint64_t seed;
    int64_t n_steps;             // the replica idles once it has run this many steps
    int cap, ecap;
    int smem_cells;              // 1: uint16_t cell array in shared memory during the step
    int table;                   // index into EngineDev::tabs
    int count_stride;            // record counts at t = 0 and after every count_stride steps (0: never)
    int max_records;
    int64_t record_pitch;        // entries between successive count records of this replica (0: ntypes)
};

struct RepState {
    int n, n_in, cur, next_id, status, rec;  // rec: count records written
    int fvalid;                              // force[cur] holds the pair forces on pos[cur]
    int64_t step;                            // steps run (keys the random streams)
};

struct EngineDev {
    const RepDesc *desc;
    RepState *state;
    const int *order;   // work item -> replica
    const int *n_work;  // work items of a step; on the device, so one captured graph serves any list
    int *work;          // work counter, reset after each step
    const Tables *tabs;
    int handler;
    int max_events_sm;  // events one replica step resolves in shared memory
    unsigned long long *particle_steps;  // particles advanced, summed over replicas and steps
    // steps each replica takes per launch, one after the other on its CTA (null: one).  The served form
    // gives small requests more, so that a launch's length is not the largest request's step for all.
    const int *launch_steps;
};

// decides the cell grid of a replica: cells at least cutoff * cell_scale wide, widened until the
// grid fits the shared-memory cell array when the replica is small enough for 16-bit starts
Geo replica_geo(const double box[3], const int pbc[3], double cutoff, double cell_scale, int64_t capacity,
                int &smem_cells);

size_t engine_smem_bytes(int max_events_sm);
// kernel attributes for the dynamic shared memory; returns the persistent grid (CTAs resident at once)
int engine_grid(int threads, size_t smem);
// one step of every listed replica (or, with E.launch_steps, that many steps of each), then the work
// counter reset (both captured in the step graph)
void launch_engine_step(const EngineDev &E, int blocks, int threads, size_t smem, cudaStream_t st);
// binning and sort of the listed replicas (list: device array of replica indices), after setting the
// ids to 0..n-1 when fill_ids; replicas with records and none written yet get their t = 0 record
void launch_engine_admit(const EngineDev &E, const int *list, int count, bool fill_ids, cudaStream_t st);
// current per-type counts of replicas [0, R) into out (R x ntypes)
void launch_engine_count(const EngineDev &E, int R, int ntypes, unsigned long long *out, cudaStream_t st);
// the force the next step applies to each of the n storage slots of replica r's current state (pair
// forces carried or walked, plus order-1 potentials) into out (float4 per slot, removed slots zero)
void launch_engine_forces(const EngineDev &E, int r, int n, float4 *out, cudaStream_t st);
// current per-type counts of replicas [0, R) written as count record `rec` of each
void launch_engine_record_now(const EngineDev &E, int R, int ntypes, int rec, cudaStream_t st);
// the live particles of replicas sel[0, n_sel) into the slots slot_off[k] of a trajectory frame
void launch_engine_snapshot(const EngineDev &E, const int *sel, int n_sel, const int64_t *slot_off, float4 *out_pos,
                            uint32_t *out_id, int *out_n, cudaStream_t st);
// pair virial (9 doubles, row-major) of replicas [0, R) on their current states into out (R x 9); NaN for a
// replica that carries its forces (its state is not sorted)
void launch_engine_virial(const EngineDev &E, int R, double *out, cudaStream_t st);
// multiprocessors of the current device
int sm_count();

}  // namespace rdc

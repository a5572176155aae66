// Kernels of the per-system ("plain") path: one simulation, every stage a grid-wide launch.
//
//   K1  cell list as a deterministic counting sort            (CellLinkedList.cpp:52-247)
//   K3  pair forces over the 27-cell stencil                  (CPUCalculateForces.cpp:214-268)
//   K4  bonded bond/angle/dihedral terms per topology particle (CPUTopologyActions.cpp:55-123)
//   K5  Euler Brownian dynamics fused with binning            (CPUEulerBDIntegrator.cpp:51-103)
//   K6  reaction events (order 1 per particle, order 2 per pair)   (CPUUncontrolledApproximation.cpp:70-133,
//                                                                    ReactionUtils.h:83-144)
//   K7  conflict resolution by seeded priority + application   (CPUUncontrolledApproximation.cpp:197-253,
//                                                                algorithm.h:62-136, ReactionUtils.h:146-227)
// Storage is structure-of-arrays in cell order; a sort writes the alternate buffers.
#include <cuda_runtime.h>

#include <cfloat>
#include <climits>
#include <cstdint>

#include "rdc_phases.cuh"
#include "rdc_host.h"

namespace rdc {

#define GRID_STRIDE(i, n) for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

// ------------------------------------------------------------------------------------------------
// K5 (+ bin): Euler-Maruyama step, then the bin of the new position and its rank inside the bin
// ------------------------------------------------------------------------------------------------
// true in one thread of the last block of the grid to finish (C_DONE counts the finished blocks and is
// reset by that block): the place for a counter update that every block must see unchanged
__device__ inline bool last_block_done(int *counters) {
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(&counters[C_DONE], 1) == (int)(gridDim.x * gridDim.y) - 1;
        if (last) counters[C_DONE] = 0;
    }
    __syncthreads();
    return last && threadIdx.x == 0;
}

__global__ void k_integrate_bin(SysDev s, int integrate, int bin) {
    const int n = s.counters[C_N_TOTAL];
    const uint64_t step = s.step[0];
    const GeoR g = geo_r(s.geo);
    unsigned advanced = 0;
    GRID_STRIDE(i, n) {
        float4 p = s.pos[i];
        const int t = itype(p);
        if (integrate && t >= 0) {
            const float4 f = s.force[i];
            p = euler_bd(p, f.x, f.y, f.z, s.id[i], s.seed, step, s.tab->bd_drift[t], s.tab->bd_scale[t], g);
            s.pos[i] = p;
            ++advanced;
        }
        if (bin) {
            const int b = bin_of(p, s.geo);
            s.bin[i] = b;
            s.rank[i] = atomicAdd(&s.cnt[b], 1);
        }
    }
    // particles advanced, summed over steps (the particle-steps of the throughput figures)
    if (integrate) {
        advanced = __reduce_add_sync(0xffffffffu, advanced);
        if ((threadIdx.x & 31) == 0 && advanced) atomicAdd(reinterpret_cast<unsigned long long *>(&s.step[2]),
                                                           (unsigned long long)advanced);
    }
    // the integrator step counter (Philox key) advances once every block has read it
    if (integrate && last_block_done(s.counters)) s.step[0] = step + 1;
}

// ------------------------------------------------------------------------------------------------
// exclusive scan of the bin counts (tiles of 2048, one pass over tile sums, one add pass)
// ------------------------------------------------------------------------------------------------
constexpr int SCAN_THREADS = 256, SCAN_ITEMS = 8, SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__global__ void k_scan_tiles(const int *__restrict__ in, int *__restrict__ out, int *__restrict__ tile_sums, int n) {
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int sum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        sum += v[k];
    }
    int total;
    int run = block_exclusive_scan(sum, total);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// single block: exclusive scan of the tile sums in place; out[n] = grand total
__global__ void k_scan_top(int *tile_sums, int ntiles, int *out, int n) {
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < ntiles; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = i < ntiles ? tile_sums[i] : 0;
        int total;
        const int ex = block_exclusive_scan(v, total);
        if (i < ntiles) tile_sums[i] = ex + carry;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = carry;
}

__global__ void k_scan_add(int *out, const int *tile_sums, int n) {
    const int add = tile_sums[blockIdx.x];
    const int base = blockIdx.x * SCAN_TILE;
    for (int k = threadIdx.x; k < SCAN_TILE; k += blockDim.x)
        if (base + k < n) out[base + k] += add;
}

int scan_block_count(int n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }

// the whole scan in one block, tile after tile with a running carry (one launch instead of three for
// grids of up to SCAN_ONE_BLOCK cells, where the launches cost more than the work)
constexpr int SCAN_ONE_BLOCK = 16384, SCAN_ONE_THREADS = 1024;
__global__ void __launch_bounds__(SCAN_ONE_THREADS) k_scan_one_block(const int *__restrict__ in, int *__restrict__ out,
                                                                     int n) {
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int tile = SCAN_ONE_THREADS * SCAN_ITEMS;
    for (int base = 0; base < n; base += tile) {
        const int b = base + (int)threadIdx.x * SCAN_ITEMS;
        int v[SCAN_ITEMS];
        int sum = 0;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            v[k] = (b + k < n) ? in[b + k] : 0;
            sum += v[k];
        }
        int total;
        int run = block_exclusive_scan(sum, total) + carry;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            if (b + k < n) out[b + k] = run;
            run += v[k];
        }
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = carry;
}

static void launch_scan(const int *in, int *out, int *tiles, int n, cudaStream_t st) {
    if (n <= SCAN_ONE_BLOCK) {
        k_scan_one_block<<<1, SCAN_ONE_THREADS, 0, st>>>(in, out, n);
        return;
    }
    const int nt = scan_block_count(n);
    k_scan_tiles<<<nt, SCAN_THREADS, 0, st>>>(in, out, tiles, n);
    k_scan_top<<<1, 1024, 0, st>>>(tiles, nt, out, n);
    k_scan_add<<<nt, SCAN_THREADS, 0, st>>>(out, tiles, n);
}

// ------------------------------------------------------------------------------------------------
// K1 counting sort: scatter source indices, order each cell by particle id (deterministic, and
// independent of the order of the source arrays), gather the particle arrays into the alternate buffers
// ------------------------------------------------------------------------------------------------
__global__ void k_scatter(SysDev s) {
    const int n = s.counters[C_N_TOTAL];
    const int nc = s.geo.ncells;
    GRID_STRIDE(i, n) {
        const int b = s.bin[i];
        if (b <= nc) s.src[s.start[b] + s.rank[i]] = i;
    }
}

__global__ void k_cell_order(SysDev s) {
    GRID_STRIDE(c, s.geo.ncells) {
        const int b = s.start[c], e = s.start[c + 1];
        if (e - b > CELL_SORT_SMALL) {
            s.big_cells[atomicAdd(&s.counters[C_BIG], 1)] = c;
            continue;
        }
        insertion_sort_by(s.src, b, e, s.id);
    }
}

// cells with many entries: one block per cell, every entry's rank is the number of entries with a
// smaller id (ids are distinct); rank[] is free scratch once the scatter is done
__global__ void k_big_cell_order(SysDev s) {
    const int nbig = s.counters[C_BIG];
    for (int q = blockIdx.x; q < nbig; q += gridDim.x) {
        const int c = s.big_cells[q];
        block_rank_sort_by(s.src, s.rank, s.start[c], s.start[c + 1], s.id);
    }
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x == 0) s.counters[C_BIG] = 0;
}

__global__ void k_gather(SysDev s, int permute_force) {
    const int nc = s.geo.ncells;
    const int n_new = s.start[nc + 1];  // cells + OUT, without the dead
    GRID_STRIDE(j, n_new) {
        const int k = s.src[j];
        s.pos_alt[j] = s.pos[k];
        s.id_alt[j] = s.id[k];
        const int ts = s.tslot[k];
        s.tslot_alt[j] = ts;
        if (ts >= 0 && ts < s.tloc_size) s.tloc[ts] = j;
        if (permute_force) s.force_alt[j] = s.force[k];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        s.counters[C_N] = n_new;
        s.counters[C_N_TOTAL] = n_new;
        s.counters[C_N_INCELLS] = s.start[nc];
    }
}

// ------------------------------------------------------------------------------------------------
// K3 pair forces: one thread per particle, full (both-direction) stencil, force and half the pair
// energies accumulated in registers; per-block FP64 energy partials in a fixed order
// ------------------------------------------------------------------------------------------------
// Three 256-thread blocks per SM (80 registers): 0.203 ms per step of the 200k-particle crowded system
// against 0.221 ms at two blocks (92 registers) and 0.206 ms at four (64 registers, spills).
template <bool VIRIAL>
__global__ void __launch_bounds__(FORCE_THREADS, 3) k_pair_forces(SysDev s) {
    __shared__ int sh_tab[MAX_TYPES * MAX_TYPES];
    __shared__ float sh_scr[MAX_TYPES * MAX_TYPES];
    __shared__ PairPot sh_pots[MAX_PAIR_POTENTIALS];
    const Tables *tab = s.tab;
    const int T = tab->ntypes, NP = tab->npots;
    for (int k = threadIdx.x; k < T * T; k += blockDim.x) {
        sh_tab[k] = tab->pair_tab[k];
        sh_scr[k] = tab->pair_screen[k];
    }
    for (int k = threadIdx.x; k < NP; k += blockDim.x) sh_pots[k] = tab->pots[k];
    __syncthreads();
    const int n = s.counters[C_N], n_in = s.counters[C_N_INCELLS];
    const GeoR g = geo_r(s.geo);
    double esum = 0.0;
    float vir[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    double vsum[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    GRID_STRIDE(i, n) {
        float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
        const float4 p = s.pos[i];
        if (i < n_in && NP > 0)
            pair_force_at(i, p, s.pos, s.start, g, s.radius, sh_tab, sh_scr, sh_pots, T, fx, fy, fz, e,
                          VIRIAL ? vir : nullptr);
        if (VIRIAL) {
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                vsum[k] += (double)vir[k];
                vir[k] = 0.f;
            }
        }
        const int ti = itype(p);
        if (ti >= 0) {  // order-1 potentials act on every active particle, in the box or not (CPUCalculateForces.cpp:295-314)
            const int o1 = tab->o1pot_tab[ti];
            if (o1) order1_force(p, tab->o1pots, o1 >> 8, o1 & 0xff, fx, fy, fz, e);
        }
        s.force[i] = make_float4(fx, fy, fz, e);
        esum += (double)e;
    }
    const double b = block_sum_double(esum);
    if (threadIdx.x == 0) s.epart[blockIdx.x] = b;
    if (VIRIAL) {
        for (int k = 0; k < 9; ++k) {
            const double v = block_sum_double(vsum[k]);
            if (threadIdx.x == 0) s.vpart[9 * blockIdx.x + k] = v;
        }
    }
    // the final sums read FORCE_BLOCKS partials: those of the blocks this launch has not are zero
    if (blockIdx.x == 0)
        for (int k = gridDim.x + threadIdx.x; k < FORCE_BLOCKS; k += blockDim.x) {
            s.epart[k] = 0.0;
            if (VIRIAL)
                for (int c = 0; c < 9; ++c) s.vpart[9 * k + c] = 0.0;
        }
}

// virial of the last force calculation: block partials summed in a fixed order
__global__ void k_virial_final(SysDev s) {
    for (int k = 0; k < 9; ++k) {
        double v = 0.0;
        for (int b = threadIdx.x; b < FORCE_BLOCKS; b += blockDim.x) v += s.vpart[9 * b + k];
        const double t = block_sum_double(v);
        if (threadIdx.x == 0) s.virial[k] = t;
    }
}

// ------------------------------------------------------------------------------------------------
// K4 bonded terms: one thread per term evaluates it once and writes every participant's force to the
// term's entries of the per-particle term lists; one thread per topology particle then sums its
// entries in list order and adds them to its force.  The term kernel is bound by the latency of its
// FP64 dihedral arithmetic; two 256-thread blocks per SM (128 registers) ran the 200k polymer step in
// 0.227 ms against 0.230 ms at 142 registers and 0.229 ms at three blocks (80 registers, spills).
// ------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 2) k_bonded_terms(SysDev s) {
    const Geo &g = s.geo;
    const int nb = s.n_bonds, na = s.n_angles, nd = s.n_dihedrals;
    double esum = 0.0;
    GRID_STRIDE(t, nb + na + nd) {
        float e = 0.f;
        if (t < nb) {
            const int4 I = s.bond_idx[t];
            const float4 P = s.bond_par[t];
            const int2 at = s.bond_at[t];
            F3 f = f3(0.f, 0.f, 0.f);
            if (P.x != 0.0f)  // terms with k = 0 are skipped (CPUTopologyActions.cpp:62)
                f = bond_force(s.pos[s.tloc[I.x]], s.pos[s.tloc[I.y]], P, g, e);
            s.term_force[at.x] = make_float4(f.x, f.y, f.z, e);
            s.term_force[at.y] = make_float4(-f.x, -f.y, -f.z, 0.f);
        } else if (t < nb + na) {
            const int k = t - nb;
            const int4 I = s.angle_idx[k];
            const int4 at = s.angle_at[k];
            F3 f[3];
            angle_force(s.pos[s.tloc[I.x]], s.pos[s.tloc[I.y]], s.pos[s.tloc[I.z]], s.angle_par[k], g, f, e);
            s.term_force[at.x] = make_float4(f[0].x, f[0].y, f[0].z, e);
            s.term_force[at.y] = make_float4(f[1].x, f[1].y, f[1].z, 0.f);
            s.term_force[at.z] = make_float4(f[2].x, f[2].y, f[2].z, 0.f);
        } else {
            const int k = t - nb - na;
            const int4 I = s.dih_idx[k];
            const float4 P = s.dih_par[k];
            const int4 at = s.dih_at[k];
            F3 f[4];
            dihedral_force(s.pos[s.tloc[I.x]], s.pos[s.tloc[I.y]], s.pos[s.tloc[I.z]], s.pos[s.tloc[I.w]], P.x, P.y,
                           P.z, g, f, e);
            s.term_force[at.x] = make_float4(f[0].x, f[0].y, f[0].z, e);
            s.term_force[at.y] = make_float4(f[1].x, f[1].y, f[1].z, 0.f);
            s.term_force[at.z] = make_float4(f[2].x, f[2].y, f[2].z, 0.f);
            s.term_force[at.w] = make_float4(f[3].x, f[3].y, f[3].z, 0.f);
        }
        esum += (double)e;
    }
    const double b = block_sum_double(esum);
    if (threadIdx.x == 0) s.epart[FORCE_BLOCKS + blockIdx.x] = b;
}

__global__ void k_bonded_gather(SysDev s) {
    GRID_STRIDE(t, s.n_top) {
        const int j = s.tloc[t];
        float fx = 0.f, fy = 0.f, fz = 0.f, eown = 0.f;
        for (int q = s.top_off[t]; q < s.top_off[t + 1]; ++q) {
            const float4 f = s.term_force[q];
            fx += f.x; fy += f.y; fz += f.z; eown += f.w;
        }
        float4 cur = s.force[j];
        cur.x += fx; cur.y += fy; cur.z += fz; cur.w += eown;
        s.force[j] = cur;
    }
}

// ------------------------------------------------------------------------------------------------
// BreakBonds (include/readdy/model/actions/Actions.h:236-290): one thread per graph edge of the
// topologies.  The edge's energy is the sum of its harmonic bonds, k (|x_ij| - l0)^2 over the bond
// configurations of its type pair (BondedPotential.h harmonic bond energy), taken in FP64 from the FP32
// positions with bcs::shortestDifference (boundary_condition_operations.h:71-80).  An edge above its
// type pair's threshold energy breaks when its coin, keyed by the ordered ids of its particles and the
// call counter, falls below 1 - exp(-rate dt); the indices of the broken edges are appended to out.
// Edges are independent: the reference evaluates every edge of a topology on the positions before
// any removal.
// ------------------------------------------------------------------------------------------------
__global__ void k_break_bonds(SysDev s, const int4 *__restrict__ edges, int n_edges, const double2 *__restrict__ bond_kl,
                              const double *__restrict__ thr, const uint64_t *__restrict__ coin, int T, uint64_t seed,
                              uint64_t counter, int *out, int *out_n) {
    const Geo &g = s.geo;
    GRID_STRIDE(e, n_edges) {
        const int4 E = edges[e];
        const int i = s.tloc[E.x], j = s.tloc[E.y];
        const float4 pi = s.pos[i], pj = s.pos[j];
        const int ti = itype(pi), tj = itype(pj);
        if (ti < 0 || tj < 0 || ti >= T || tj >= T) continue;
        const double th = thr[ti * T + tj];
        if (th != th) continue;  // NaN: the type pair is not breakable
        double x[3] = {(double)pj.x - (double)pi.x, (double)pj.y - (double)pi.y, (double)pj.z - (double)pi.z};
#pragma unroll
        for (int a = 0; a < 3; ++a)
            if (g.pbc[a]) {
                const double L = (double)g.L[a];
                if (x[a] > 0.5 * L) x[a] -= L;
                else if (x[a] <= -0.5 * L) x[a] += L;
            }
        const double d = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
        double energy = 0.0;
        for (int b = E.z; b < E.z + E.w; ++b) {
            const double2 kl = bond_kl[b];
            energy += kl.x * (d - kl.y) * (d - kl.y);
        }
        if (!(energy > th)) continue;
        const uint32_t a = s.id[i], b = s.id[j];
        const U4 u = rng_draw(seed, min(a, b), max(a, b), counter, RNG_BREAK, 0u);
        if (coin_bits(u) < coin[ti * T + tj]) out[atomicAdd(out_n, 1)] = e;
    }
}

// ------------------------------------------------------------------------------------------------
// Spatial topology reactions, device part: the candidate pairs of the event gathering of
// CPUEvaluateTopologyReactions::gatherEvents (kernels/cpu/src/actions/CPUEvaluateTopologyReactions.cpp:
// 225-320) -- pairs of particles in cells whose types some spatial reaction names, closer than the largest
// reaction radius -- one thread per particle over the stencil cells, each unordered pair once (j > i).
// The squared distance is bcs::distSquared in FP64 from the FP32 positions; the host applies each
// reaction's own radius, the topology conditions and the selection.
// ------------------------------------------------------------------------------------------------
__global__ void k_topology_candidates(SysDev s, const uint32_t *__restrict__ pair_mask, float r2screen, double r2max,
                                      TopCandidate *out, int *out_n, int cap) {
    const GeoR g = geo_r(s.geo);
    const int n_in = s.counters[C_N_INCELLS];
    GRID_STRIDE(i, n_in) {
        const float4 p = s.pos[i];
        const int ti = itype(p);
        if (ti < 0) continue;
        const uint32_t mi = pair_mask[ti];
        if (!mi) continue;
        for_each_candidate(p, g, s.start, s.radius, i + 1, [&](int j) {
            const float4 q = s.pos[j];
            const int tj = itype(q);
            if (tj < 0 || !((mi >> tj) & 1u)) return;
            if (screen_d2(p, q, g) > r2screen) return;
            double x[3] = {(double)q.x - (double)p.x, (double)q.y - (double)p.y, (double)q.z - (double)p.z};
#pragma unroll
            for (int a = 0; a < 3; ++a)
                if (g.pbc[a]) {
                    const double L = (double)g.L[a];
                    if (x[a] > 0.5 * L) x[a] -= L;
                    else if (x[a] <= -0.5 * L) x[a] += L;
                }
            const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(x[0], x[0]), __dmul_rn(x[1], x[1])), __dmul_rn(x[2], x[2]));
            if (!(d2 < r2max)) return;
            const int k = atomicAdd(out_n, 1);
            if (k < cap) out[k] = TopCandidate{i, j, ti, tj, s.tslot[i], s.tslot[j], s.id[i], s.id[j], d2};
        });
    }
}

void launch_topology_candidates(const SysDev &s, const uint32_t *pair_mask, double r2max, float r2screen,
                                TopCandidate *out, int *out_n, int cap, cudaStream_t st) {
    RDC_CUDA(cudaMemsetAsync(out_n, 0, sizeof(int), st));
    k_topology_candidates<<<GRID_BLOCKS, GRID_THREADS, 0, st>>>(s, pair_mask, r2screen, r2max, out, out_n, cap);
}

__global__ void k_particle_edits(SysDev s, const int4 *__restrict__ edits, int n) {
    GRID_STRIDE(k, n) {
        const int4 e = edits[k];
        int i = e.x;
        if (e.w == 1) {  // x names a topology slot
            if (e.x < 0 || e.x >= s.tloc_size) continue;
            i = s.tloc[e.x];
        }
        float4 p = s.pos[i];
        p.w = __int_as_float(e.y);
        s.pos[i] = p;
        if (e.z >= 0) {
            s.tslot[i] = e.z;
            if (e.z < s.tloc_size) s.tloc[e.z] = i;
        }
    }
}

// position changes: target x is a storage index (y = 0) or a topology slot (y = 1); the type is kept
__global__ void k_position_edits(SysDev s, const int2 *__restrict__ targets, const float4 *__restrict__ to, int n) {
    GRID_STRIDE(k, n) {
        const int2 t = targets[k];
        int i = t.x;
        if (t.y == 1) {
            if (t.x < 0 || t.x >= s.tloc_size) continue;
            i = s.tloc[t.x];
        }
        float4 p = s.pos[i];
        p.x = to[k].x;
        p.y = to[k].y;
        p.z = to[k].z;
        s.pos[i] = p;
    }
}

void launch_position_edits(const SysDev &s, const int2 *targets, const float4 *to, int n, cudaStream_t st) {
    if (n > 0) k_position_edits<<<std::min((n + 255) / 256, GRID_BLOCKS), 256, 0, st>>>(s, targets, to, n);
}

// positions of the particles of topology slots slots[0, n)
__global__ void k_gather_slots(SysDev s, const int *__restrict__ slots, int n, float4 *out) {
    GRID_STRIDE(k, n) {
        const int t = slots[k];
        out[k] = (t >= 0 && t < s.tloc_size) ? s.pos[s.tloc[t]] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

void launch_gather_slots(const SysDev &s, const int *slots, int n, float4 *out, cudaStream_t st) {
    if (n > 0) k_gather_slots<<<std::min((n + 255) / 256, GRID_BLOCKS), 256, 0, st>>>(s, slots, n, out);
}

void launch_particle_edits(const SysDev &s, const int4 *edits, int n, cudaStream_t st) {
    if (n > 0) k_particle_edits<<<std::min((n + 255) / 256, GRID_BLOCKS), 256, 0, st>>>(s, edits, n);
}

void launch_break_bonds(const SysDev &s, const int4 *edges, int n_edges, const double2 *bond_kl, const double *thr,
                        const uint64_t *coin, int T, uint64_t seed, uint64_t counter, int *out, int *out_n,
                        cudaStream_t st) {
    RDC_CUDA(cudaMemsetAsync(out_n, 0, sizeof(int), st));
    if (n_edges > 0)
        k_break_bonds<<<std::min((n_edges + 255) / 256, GRID_BLOCKS), 256, 0, st>>>(s, edges, n_edges, bond_kl, thr, coin,
                                                                               T, seed, counter, out, out_n);
}

__global__ void k_energy_final(SysDev s, int pair, int bonded) {
    double v = 0.0;
    if (pair)
        for (int k = threadIdx.x; k < FORCE_BLOCKS; k += blockDim.x) v += s.epart[k];
    if (bonded)
        for (int k = threadIdx.x; k < BONDED_BLOCKS; k += blockDim.x) v += s.epart[FORCE_BLOCKS + k];
    const double b = block_sum_double(v);
    if (threadIdx.x == 0) *s.energy = b;
}

// ------------------------------------------------------------------------------------------------
// K6 reaction events that pass their acceptance coin
// ------------------------------------------------------------------------------------------------
__global__ void k_events(SysDev s, int handler) {
    __shared__ int sh_rt_ints[MAX_TYPES + MAX_REACTIONS * 3 + MAX_TYPES * MAX_TYPES + MAX_TYPES];
    __shared__ float sh_rt_scr[MAX_TYPES * MAX_TYPES];
    __shared__ ReactionDev sh_rx[MAX_REACTIONS];
    const RxnTables rt = stage_rxn_tables(s.tab, sh_rt_ints, sh_rt_scr, sh_rx);
    __syncthreads();
    const GeoR g = geo_r(s.geo);
    const int n = s.counters[C_N], n_in = s.counters[C_N_INCELLS];
    const uint64_t step = s.step[1];
    auto emit = [&](uint64_t key, int p1, int p2, int r) {
        const int k = atomicAdd(&s.counters[C_N_EVENTS], 1);
        if (k < s.event_capacity) {
            EventRec ev;
            ev.key = key; ev.p1 = p1; ev.p2 = p2; ev.reaction = r; ev.pad = 0;
            s.events[k] = ev;
        } else {
            atomicOr(&s.counters[C_STATUS], ST_EVENTS);
        }
    };
    __shared__ int q1[EVENT_QUEUE], q2[EVENT_QUEUE], qn;
    __shared__ unsigned char qr[EVENT_QUEUE];
    const TupleQueue Q{q1, q2, qr, &qn};
    block_events(blockIdx.x * blockDim.x, gridDim.x * blockDim.x, n, n_in, s.pos, s.id, s.start, g, s.radius, rt,
                 s.seed, step, handler, Q, emit);
}

// ------------------------------------------------------------------------------------------------
// K7 one block: priority order, greedy maximal independent set, application of the winners
// ------------------------------------------------------------------------------------------------
constexpr int RESOLVE_THREADS = 1024;

size_t resolve_smem_bytes() {
    return (size_t)RESOLVE_MAX_EVENTS * (sizeof(uint64_t) + sizeof(int) + sizeof(int)) + 64;
}

__global__ void __launch_bounds__(RESOLVE_THREADS) k_resolve_apply(SysDev s, int handler) {
    extern __shared__ unsigned char smem[];
    uint64_t *key = reinterpret_cast<uint64_t *>(smem);
    int *idx = reinterpret_cast<int *>(key + RESOLVE_MAX_EVENTS);
    int *state = idx + RESOLVE_MAX_EVENTS;
    int E = s.counters[C_N_EVENTS];
    if (E > s.event_capacity) E = s.event_capacity;
    ApplyTarget t;
    t.pos = s.pos; t.id = s.id; t.tslot = s.tslot; t.force = s.force;
    t.claim = s.claim; t.taken = s.taken; t.reaction_counts = s.reaction_counts;
    t.n_total = s.counters[C_N_TOTAL];
    t.capacity = s.capacity;
    t.next_id = (uint32_t)s.counters[C_NEXT_ID];
    ApplyResult res;
    block_resolve_apply(s.events, E, RESOLVE_MAX_EVENTS, key, idx, state, s.tab, s.geo, s.seed, s.step[1], t, res);
    if (threadIdx.x == 0) {
        s.counters[C_N_TOTAL] = t.n_total + res.births;
        s.counters[C_NEXT_ID] = (int)(t.next_id + (uint32_t)res.ids);
        s.counters[C_N_BIRTHS] = res.births;
        s.counters[C_N_EVENTS] = 0;
        if (res.status) atomicOr(&s.counters[C_STATUS], res.status);
        s.step[1] += 1;
    }
    (void)handler;
}

// ------------------------------------------------------------------------------------------------
// observables and the parity pair list
// ------------------------------------------------------------------------------------------------
__global__ void k_count_types(SysDev s, unsigned long long *out) {
    __shared__ unsigned int hist[MAX_TYPES];
    const int T = s.tab->ntypes;
    for (int k = threadIdx.x; k < T; k += blockDim.x) hist[k] = 0;
    __syncthreads();
    const int n = s.counters[C_N_TOTAL];
    GRID_STRIDE(i, n) {
        const int t = itype(s.pos[i]);
        if (t >= 0 && t < T) atomicAdd(&hist[t], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < T; k += blockDim.x)
        if (hist[k]) atomicAdd(&out[k], (unsigned long long)hist[k]);
}

// counts into the record ring when the step is a multiple of the stride; the record counter advances
// once every block has added its counts
__global__ void k_record_counts(SysDev s) {
    const uint64_t t = s.step[0] - s.rec_base;
    if (s.counts_stride <= 0 || t % (uint64_t)s.counts_stride != 0) return;
    const int rec = s.counters[C_REC];
    if (rec >= s.counts_max) return;
    __shared__ unsigned int hist[MAX_TYPES];
    const int T = s.tab->ntypes;
    for (int k = threadIdx.x; k < T; k += blockDim.x) hist[k] = 0;
    __syncthreads();
    const int n = s.counters[C_N_TOTAL];
    GRID_STRIDE(i, n) {
        const int ty = itype(s.pos[i]);
        if (ty >= 0 && ty < T) atomicAdd(&hist[ty], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < T; k += blockDim.x)
        if (hist[k]) atomicAdd(&s.counts_ring[(size_t)rec * T + k], (unsigned long long)hist[k]);
    if (last_block_done(s.counters)) s.counters[C_REC] = rec + 1;
}

__global__ void k_pairs(SysDev s, float c2f, float band, double c2, uint64_t *out, int cap, int *n_out) {
    const int n_in = s.counters[C_N_INCELLS];
    const GeoR g = geo_r(s.geo);
    GRID_STRIDE(i, n_in) {
        const float4 p = s.pos[i];
        const uint32_t idi = s.id[i];
        for_each_candidate(p, g, s.start, s.radius, i + 1, [&](int j) {
            const float4 q = s.pos[j];
            const PairGeom g0 = pair_geom(p, q, g);
            PairGeom gg = g0;
            if (!within(g0, gg, p, q, g, c2f, band, c2)) return;
            const uint32_t idj = s.id[j];
            const int k = atomicAdd(n_out, 1);
            if (k < cap) out[k] = ((uint64_t)min(idi, idj) << 32) | max(idi, idj);
        });
    }
}

__global__ void k_fill_ids(uint32_t *id, uint32_t first, int n) {
    GRID_STRIDE(i, n) id[i] = first + (uint32_t)i;
}

// ------------------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------------------
void init_kernel_attributes() {
    RDC_CUDA(cudaFuncSetAttribute(k_resolve_apply, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)resolve_smem_bytes()));
}

// Blocks of a grid-stride launch over `items` particles or cells: one item per thread, at most `cap`
// blocks.  A small system's kernels then start and drain sooner, and leave the SMs to kernels of other
// systems on other streams (the served form runs several per-system requests at once).  Particle
// launches are sized by the capacity, which bounds the particles of every step a graph replays.
inline int blocks_for(int items, int cap) { return std::max(1, std::min(cap, (items + 255) / 256)); }
inline int particle_blocks(const SysDev &s) { return blocks_for(s.capacity, GRID_BLOCKS); }

void launch_integrate_bin(const SysDev &s, bool integrate, cudaStream_t st) {
    RDC_CUDA(cudaMemsetAsync(s.cnt, 0, sizeof(int) * (s.geo.ncells + 2), st));
    k_integrate_bin<<<particle_blocks(s), GRID_THREADS, 0, st>>>(s, integrate ? 1 : 0, 1);
}

void launch_bin(const SysDev &s, cudaStream_t st) { launch_integrate_bin(s, false, st); }

void launch_sort(const SysDev &s, bool permute_force, cudaStream_t st) {
    const int nb = s.geo.ncells + 2;
    launch_scan(s.cnt, s.start, s.scan_blocks, nb, st);
    k_scatter<<<particle_blocks(s), GRID_THREADS, 0, st>>>(s);
    k_cell_order<<<blocks_for(s.geo.ncells, GRID_BLOCKS), GRID_THREADS, 0, st>>>(s);
    k_big_cell_order<<<152, 512, 0, st>>>(s);
    k_gather<<<particle_blocks(s), GRID_THREADS, 0, st>>>(s, permute_force ? 1 : 0);
}

void launch_force_finals(const SysDev &s, bool bonded, cudaStream_t st) {
    if (s.virial) k_virial_final<<<1, 256, 0, st>>>(s);
    k_energy_final<<<1, 256, 0, st>>>(s, 1, (bonded && s.n_top > 0) ? 1 : 0);
}

void launch_forces(const SysDev &s, bool pair, bool bonded, cudaStream_t st, bool finals) {
    const int fb = blocks_for(s.capacity, FORCE_BLOCKS);
    if (s.virial) k_pair_forces<true><<<fb, FORCE_THREADS, 0, st>>>(s);
    else k_pair_forces<false><<<fb, FORCE_THREADS, 0, st>>>(s);
    if (bonded && s.n_top > 0) {
        k_bonded_terms<<<BONDED_BLOCKS, 256, 0, st>>>(s);
        k_bonded_gather<<<BONDED_BLOCKS, 256, 0, st>>>(s);
    }
    if (finals) launch_force_finals(s, bonded, st);
    (void)pair;
}

void launch_events(const SysDev &s, int handler, cudaStream_t st) {
    k_events<<<particle_blocks(s), GRID_THREADS, 0, st>>>(s, handler);
}

void launch_resolve_apply(const SysDev &s, int handler, cudaStream_t st) {
    k_resolve_apply<<<1, RESOLVE_THREADS, resolve_smem_bytes(), st>>>(s, handler);
}

// ------------------------------------------------------------------------------------------------
// observables of ReaDDy's CPU kernel that bin particles or pairs (readdy/main/model/observables)
// ------------------------------------------------------------------------------------------------
// bins counted in a shared-memory histogram per block (more go straight to global memory)
constexpr int OBS_SMEM_BINS = 4096;
constexpr int RDF_TILE = 256;

// std::upper_bound over borders[0, n): the first border greater than x (FP64 comparisons)
__device__ inline int upper_bound_d(const double *__restrict__ b, int n, double x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (!(x < b[mid])) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// HistogramAlongAxis of the CPU kernel (kernels/cpu/src/observables/CPUObservables.cpp:85-146): every
// active particle of a type in `types` (bit mask) adds one to bin k - 1 of k = upper_bound(borders, x),
// x its coordinate on `axis`, when 1 <= k < nb - 1 (the CPU kernel compares k with the nb - 1 bins of
// its result, so the last bin stays empty).  The FP32 coordinate widened to FP64 compares exactly.
__global__ void k_histogram_axis(SysDev s, const double *__restrict__ borders, int nb, uint32_t types, int axis,
                                 unsigned long long *out) {
    extern __shared__ unsigned int hist[];
    const int size = nb - 1;
    const bool in_smem = size <= OBS_SMEM_BINS;
    if (in_smem)
        for (int k = threadIdx.x; k < size; k += blockDim.x) hist[k] = 0u;
    __syncthreads();
    const int n = s.counters[C_N_TOTAL];
    GRID_STRIDE(i, n) {
        const float4 p = s.pos[i];
        const int t = itype(p);
        if (t < 0 || !((types >> t) & 1u)) continue;
        const double x = (double)(axis == 0 ? p.x : (axis == 1 ? p.y : p.z));
        const int k = upper_bound_d(borders, nb, x);
        if (k < 1 || k >= size) continue;
        if (in_smem) atomicAdd(&hist[k - 1], 1u);
        else atomicAdd(&out[k - 1], 1ull);
    }
    __syncthreads();
    if (in_smem)
        for (int k = threadIdx.x; k < size; k += blockDim.x)
            if (hist[k]) atomicAdd(&out[k], (unsigned long long)hist[k]);
}

// RadialDistribution (readdy/main/model/observables/RadialDistribution.cpp:75-128): every ordered pair of
// active particles with distinct ids, the first of a `from` type and the second of a `to` type, adds one to
// bin k - 1 of k = upper_bound(borders, |x_to - x_from|) when 1 <= k < nb.  All pairs, like the reference:
// each block holds RDF_TILE `from` particles and streams every particle through shared memory in tiles.  A
// pair whose FP32 distance is beyond the last border by more than FP32 rounding (reach2) is dropped; the
// others get the reference's FP64 distance (minimum image, squares summed x, y, z, sqrt), on positions that
// are exact in FP64.
__global__ void __launch_bounds__(RDF_TILE) k_radial_distribution(SysDev s, const double *__restrict__ borders,
                                                                   int nb, uint32_t from, uint32_t to, float reach2,
                                                                   unsigned long long *out) {
    extern __shared__ __align__(16) unsigned char rdf_smem[];
    float4 *tp = reinterpret_cast<float4 *>(rdf_smem);
    uint32_t *tid = reinterpret_cast<uint32_t *>(tp + RDF_TILE);
    unsigned int *hist = tid + RDF_TILE;
    const int size = nb - 1;
    const bool in_smem = size <= OBS_SMEM_BINS;
    if (in_smem)
        for (int k = threadIdx.x; k < size; k += blockDim.x) hist[k] = 0u;
    const int n = s.counters[C_N_TOTAL];
    const GeoR g = geo_r(s.geo);
    const double L[3] = {(double)s.geo.L[0], (double)s.geo.L[1], (double)s.geo.L[2]};
    for (int base = blockIdx.x * RDF_TILE; base < n; base += gridDim.x * RDF_TILE) {
        const int i = base + (int)threadIdx.x;
        float4 p = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
        uint32_t idi = 0;
        if (i < n) {
            p = s.pos[i];
            idi = s.id[i];
        }
        const int ti = itype(p);
        const bool counts_from = ti >= 0 && ((from >> ti) & 1u);
        for (int j0 = 0; j0 < n; j0 += RDF_TILE) {
            __syncthreads();
            if (j0 + (int)threadIdx.x < n) {
                tp[threadIdx.x] = s.pos[j0 + threadIdx.x];
                tid[threadIdx.x] = s.id[j0 + threadIdx.x];
            }
            __syncthreads();
            if (!counts_from) continue;
            const int m = min(RDF_TILE, n - j0);
            for (int k = 0; k < m; ++k) {
                const float4 q = tp[k];
                const int tj = itype(q);
                if (tj < 0 || !((to >> tj) & 1u) || tid[k] == idi) continue;
                if (screen_d2(p, q, g) > reach2) continue;
                double dv[3] = {(double)q.x - (double)p.x, (double)q.y - (double)p.y, (double)q.z - (double)p.z};
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    if (s.geo.pbc[d]) {
                        if (dv[d] > L[d] * .5) dv[d] -= L[d];
                        else if (dv[d] <= -L[d] * .5) dv[d] += L[d];
                    }
                const double d2 =
                    __dadd_rn(__dadd_rn(__dmul_rn(dv[0], dv[0]), __dmul_rn(dv[1], dv[1])), __dmul_rn(dv[2], dv[2]));
                const int kb = upper_bound_d(borders, nb, __dsqrt_rn(d2));
                if (kb < 1 || kb >= nb) continue;
                if (in_smem) atomicAdd(&hist[kb - 1], 1u);
                else atomicAdd(&out[kb - 1], 1ull);
            }
        }
    }
    __syncthreads();
    if (in_smem)
        for (int k = threadIdx.x; k < size; k += blockDim.x)
            if (hist[k]) atomicAdd(&out[k], (unsigned long long)hist[k]);
}

void launch_histogram_axis(const SysDev &s, const double *borders, int nb, uint32_t types, int axis,
                           unsigned long long *out, cudaStream_t st) {
    const size_t smem = nb - 1 <= OBS_SMEM_BINS ? sizeof(unsigned int) * (nb - 1) : 0;
    k_histogram_axis<<<GRID_BLOCKS, GRID_THREADS, smem, st>>>(s, borders, nb, types, axis, out);
}

void launch_radial_distribution(const SysDev &s, int n, const double *borders, int nb, uint32_t from, uint32_t to,
                                float reach2, unsigned long long *out, cudaStream_t st) {
    const size_t smem = (sizeof(float4) + sizeof(uint32_t)) * RDF_TILE +
                        (nb - 1 <= OBS_SMEM_BINS ? sizeof(unsigned int) * (nb - 1) : 0);
    const int blocks = std::max(1, std::min((n + RDF_TILE - 1) / RDF_TILE, 8 * 152));
    k_radial_distribution<<<blocks, RDF_TILE, smem, st>>>(s, borders, nb, from, to, reach2, out);
}

void launch_count_types(const SysDev &s, unsigned long long *out, cudaStream_t st) {
    RDC_CUDA(cudaMemsetAsync(out, 0, sizeof(unsigned long long) * MAX_TYPES, st));
    k_count_types<<<GRID_BLOCKS, GRID_THREADS, 0, st>>>(s, out);
}

void launch_record_counts(const SysDev &s, cudaStream_t st) {
    k_record_counts<<<particle_blocks(s), GRID_THREADS, 0, st>>>(s);
}

void launch_pairs(const SysDev &s, float c2f, float band, double c2, uint64_t *out, int cap, int *n_out,
                  cudaStream_t st) {
    k_pairs<<<GRID_BLOCKS, GRID_THREADS, 0, st>>>(s, c2f, band, c2, out, cap, n_out);
}

void launch_fill_ids(uint32_t *id, uint32_t first, int n, cudaStream_t st) {
    if (n > 0) k_fill_ids<<<(n + 255) / 256, 256, 0, st>>>(id, first, n);
}

}  // namespace rdc

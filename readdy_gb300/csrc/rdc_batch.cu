// Batched replicas: thousands of independent copies of one context (own box, own particles) advanced
// together.  Every step is ONE persistent launch: each CTA takes replicas from a work queue ordered
// largest first and runs the whole step for one replica in block-level phases
//
//   forces (pair stencil) -> Euler BD -> bin -> counting sort -> reaction events -> conflict
//   resolution + application -> (re-sort if particles appeared or vanished) -> observables
//
// The step is replayed from a CUDA graph.  The arithmetic is the per-system path's (rdc_phases.cuh),
// so a replica gives the same trajectory alone, inside any batch, or through rdc_run with the
// replica's seed.  Forces are computed at the start of a step from the state left by the previous
// step's reactions, which is where SimulationLoop::run computes them (SimulationLoop.h:283-289).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/readdy_cuda.h"
#include "rdc_phases.cuh"

using namespace rdc;

namespace rdc {

// Cell counts and starts of a replica of fewer than 65536 particles live in shared memory during its
// step as uint16_t, SMEM_CELLS entries (96 KB): at cells of the cutoff's width and density 0.25 that
// holds replicas of up to ~12k particles, and larger ones get proportionally wider cells.  Replicas of
// more particles keep int starts in global memory at the natural cell width.
constexpr int SMEM_CELLS = 49152;

struct RepDesc {
    Geo geo;
    int poff, cap;     // particle slots [poff, poff + cap) in every per-particle array
    int soff;          // cell starts at start[soff .. soff + ncells + 3) between steps
    int eoff, ecap;    // event buffer
    int smem_cells;    // 1: uint16_t cell array in shared memory during the step, 0: int in global
    int pad;
    uint64_t seed;
};

struct RepState {
    int n, n_in, cur, next_id, status, pad;
};

struct BatchDev {
    int R;
    const RepDesc *desc;
    RepState *state;
    const int *order;
    int *work;
    float4 *posA, *posB;
    uint32_t *idA, *idB;
    int *bin, *rank, *src, *claim, *taken;
    int *start;
    EventRec *events;
    const Tables *tab;
    uint64_t *step;  // [0] integrator step, [1] reaction step (shared by all replicas)
    int handler, reactions;
    unsigned long long *counts;  // replica-major per-type counts, refreshed every count_stride steps
    int count_stride;
    int max_events_sm;
    unsigned long long *reaction_counts;
    unsigned long long *particle_steps;  // sum over replicas and steps of the particles advanced
};

template <typename T>
__device__ inline void block_zero(T *a, int n) {
    for (int k = threadIdx.x; k < n; k += blockDim.x) a[k] = 0;
    __syncthreads();
}

template <typename D, typename T>
__device__ inline void block_copy(D *dst, const T *src, int n) {
    for (int k = threadIdx.x; k < n; k += blockDim.x) dst[k] = (D)src[k];
    __syncthreads();
}

// in-place exclusive scan of a[0..n) by one block (shared or global memory); a[n] = total
template <typename T>
__device__ inline void block_scan_inplace(T *a, int n) {
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    constexpr int ITEMS = 4;
    const int tile = blockDim.x * ITEMS;
    for (int base = 0; base < n; base += tile) {
        const int b = base + threadIdx.x * ITEMS;
        int v[ITEMS];
        int sum = 0;
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            v[k] = (b + k < n) ? a[b + k] : 0;
            sum += v[k];
        }
        int total;
        int run = block_exclusive_scan(sum, total) + carry;
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            if (b + k < n) a[b + k] = (T)run;
            run += v[k];
        }
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) a[n] = (T)carry;
    __syncthreads();
}

// ranks of the particles inside their bins (bin[] already set); cells receives the counts
__device__ inline void block_rank(int n, const int *bin, int *rank, int *cells, int nbins) {
    block_zero(cells, nbins);
    for (int i = threadIdx.x; i < n; i += blockDim.x) rank[i] = atomicAdd(&cells[bin[i]], 1);
    __syncthreads();
}

// 16-bit counters, two per 32-bit word (4-byte aligned array); a count never exceeds the replica's
// particles (< 65536), so an increment never carries into the neighbouring counter
__device__ inline void block_rank(int n, const int *bin, int *rank, uint16_t *cells, int nbins) {
    block_zero(cells, nbins);
    unsigned *w = reinterpret_cast<unsigned *>(cells);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int b = bin[i];
        const unsigned sh = (unsigned)(b & 1) * 16u;
        rank[i] = (int)((atomicAdd(&w[b >> 1], 1u << sh) >> sh) & 0xffffu);
    }
    __syncthreads();
}

__device__ inline void block_bin(const float4 *pos, int n, int *bin, const Geo &g) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) bin[i] = bin_of(pos[i], g);
    __syncthreads();
}

// counting sort of one replica from counts in cells: scan to cell starts, scatter, order each cell
// by source index (deterministic), gather into the destination arrays
template <typename C>
__device__ inline void block_sort(const float4 *spos, const uint32_t *sid, int n, float4 *dpos, uint32_t *did,
                                  const int *bin, const int *rank, int *src, C *cells, const Geo &g, int &n_new,
                                  int &n_in) {
    const int nc = g.ncells;
    block_scan_inplace(cells, nc + 2);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int b = bin[i];
        if (b <= nc) src[cells[b] + rank[i]] = i;
    }
    __syncthreads();
    __shared__ int big[64];
    __shared__ int nbig;
    if (threadIdx.x == 0) nbig = 0;
    __syncthreads();
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const int b = cells[c], e = cells[c + 1];
        if (e - b > CELL_SORT_SMALL) {
            const int q = atomicAdd(&nbig, 1);
            if (q < 64) big[q] = c;
            continue;
        }
        insertion_sort(src, b, e);
    }
    __syncthreads();
    // crowded cells: ordered by the whole block (rank[] is free scratch after the scatter)
    if (nbig <= 64) {
        for (int q = 0; q < nbig; ++q) block_rank_sort(src, const_cast<int *>(rank), cells[big[q]], cells[big[q] + 1]);
    } else {
        for (int c = 0; c < nc; ++c)
            if (cells[c + 1] - cells[c] > CELL_SORT_SMALL) block_rank_sort(src, const_cast<int *>(rank), cells[c], cells[c + 1]);
    }
    n_new = cells[nc + 1];
    n_in = cells[nc];
    for (int j = threadIdx.x; j < n_new; j += blockDim.x) {
        const int k = src[j];
        dpos[j] = spos[k];
        did[j] = sid[k];
    }
    __syncthreads();
}

__device__ inline void block_count_types(const float4 *pos, int n, int T, unsigned long long *out) {
    __shared__ unsigned int hist[MAX_TYPES];
    for (int k = threadIdx.x; k < T; k += blockDim.x) hist[k] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int t = itype(pos[i]);
        if (t >= 0 && t < T) atomicAdd(&hist[t], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < T; k += blockDim.x) out[k] = hist[k];
    __syncthreads();
}

struct SmemLayout {
    int *tab;
    float *screen;
    float *drift, *scale;
    PairPot *pots;
    uint64_t *key;
    int *idx, *state;
    TupleQueue queue;
    uint16_t *cells;
};

__device__ inline SmemLayout carve(unsigned char *smem, int T, int NP, int max_events) {
    SmemLayout L;
    size_t off = 0;
    L.key = reinterpret_cast<uint64_t *>(smem + off);
    off += sizeof(uint64_t) * max_events;
    L.pots = reinterpret_cast<PairPot *>(smem + off);
    off += sizeof(PairPot) * (NP > 0 ? NP : 1);
    L.tab = reinterpret_cast<int *>(smem + off);
    off += sizeof(int) * T * T;
    L.idx = reinterpret_cast<int *>(smem + off);
    off += sizeof(int) * max_events;
    L.state = reinterpret_cast<int *>(smem + off);
    off += sizeof(int) * max_events;
    L.queue.p1 = reinterpret_cast<int *>(smem + off);
    off += sizeof(int) * EVENT_QUEUE;
    L.queue.p2 = reinterpret_cast<int *>(smem + off);
    off += sizeof(int) * EVENT_QUEUE;
    L.queue.count = reinterpret_cast<int *>(smem + off);
    off += sizeof(int) * 4;
    L.queue.r = smem + off;
    off += EVENT_QUEUE;
    L.cells = reinterpret_cast<uint16_t *>(smem + off);
    return L;
}

size_t batch_smem_bytes(int T, int NP, int max_events) {
    return sizeof(uint64_t) * max_events + sizeof(PairPot) * (NP > 0 ? NP : 1) + sizeof(int) * T * T +
           2 * sizeof(int) * max_events + (2 * sizeof(int) + 1) * EVENT_QUEUE + 4 * sizeof(int) +
           sizeof(uint16_t) * (SMEM_CELLS + 4) + 16;
}

// one step of one replica by the whole block; C is the cell array's type (uint16_t in shared memory
// or int in global memory)
template <typename C>
__device__ void replica_body(const BatchDev &B, int r, const SmemLayout &S, const RxnTables &rt, uint64_t bd_step,
                             uint64_t rx_step, const RepDesc &D, const RepState &st, int &sh_nev, int &sh_status,
                             C *cells) {
    const Tables *tab = B.tab;
    const int T = tab->ntypes, NP = tab->npots;
    const Geo &gs = D.geo;
    const GeoR g = geo_r(gs);
    const int nc = gs.ncells;
    float4 *posX = (st.cur ? B.posB : B.posA) + D.poff;
    uint32_t *idX = (st.cur ? B.idB : B.idA) + D.poff;
    float4 *posY = (st.cur ? B.posA : B.posB) + D.poff;
    uint32_t *idY = (st.cur ? B.idA : B.idB) + D.poff;
    int *bin = B.bin + D.poff, *rank = B.rank + D.poff, *src = B.src + D.poff;
    int *gstart = B.start + D.soff;
    constexpr bool in_smem = sizeof(C) == sizeof(uint16_t);
    if (in_smem) block_copy(cells, gstart, nc + 3);
    const int n = st.n, n_in = st.n_in;

    // forces on the current state, Euler step into Y, bins of the new positions
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float4 p = posX[i];
        float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
        if (i < n_in && NP > 0) pair_force_at(i, p, posX, cells, g, 1, S.tab, S.screen, S.pots, T, fx, fy, fz, e);
        const uint32_t id = idX[i];
        const int t = itype(p);
        const float4 q = euler_bd(p, fx, fy, fz, id, D.seed, bd_step, S.drift[t], S.scale[t], g);
        posY[i] = q;
        idY[i] = id;
        bin[i] = bin_of(q, gs);
    }
    __syncthreads();
    block_rank(n, bin, rank, cells, nc + 2);
    int n1, nin1;
    block_sort(posY, idY, n, posX, idX, bin, rank, src, cells, gs, n1, nin1);

    int n_final = n1, nin_final = nin1, cur = st.cur, next_id = st.next_id;
    if (B.reactions) {
        EventRec *ev = B.events + D.eoff;
        const int ecap = D.ecap;
        auto emit = [&](uint64_t key, int p1, int p2, int rr) {
            const int k = atomicAdd(&sh_nev, 1);
            if (k < ecap) {
                EventRec e;
                e.key = key; e.p1 = p1; e.p2 = p2; e.reaction = rr; e.pad = 0;
                ev[k] = e;
            } else {
                atomicOr(&sh_status, ST_EVENTS);
            }
        };
        block_events(0, blockDim.x, n1, nin1, posX, idX, cells, g, 1, rt, D.seed, rx_step, B.handler, S.queue, emit);
        const int E = min(sh_nev, ecap);
        if (E > 0) {
            ApplyTarget t;
            t.pos = posX; t.id = idX; t.tslot = nullptr; t.force = nullptr;
            t.claim = B.claim + D.poff; t.taken = B.taken + D.poff;
            t.reaction_counts = B.reaction_counts;
            t.n_total = n1;
            t.capacity = D.cap;
            t.next_id = (uint32_t)st.next_id;
            ApplyResult res;
            block_resolve_apply(ev, E, B.max_events_sm, S.key, S.idx, S.state, tab, gs, D.seed, rx_step, t, res);
            next_id = st.next_id + res.ids;
            if (threadIdx.x == 0) sh_status |= res.status;
            if (res.winners > 0) {
                // particles changed cells, appeared or vanished: sort again, into Y
                const int n_total = n1 + res.births;
                block_bin(posX, n_total, bin, gs);
                block_rank(n_total, bin, rank, cells, nc + 2);
                int n2, nin2;
                block_sort(posX, idX, n_total, posY, idY, bin, rank, src, cells, gs, n2, nin2);
                n_final = n2;
                nin_final = nin2;
                cur ^= 1;
            }
        }
    }
    if (in_smem) block_copy(gstart, cells, nc + 3);
    if (B.count_stride > 0 && (bd_step + 1) % (uint64_t)B.count_stride == 0) {
        const float4 *pf = (cur ? B.posB : B.posA) + D.poff;
        block_count_types(pf, n_final, T, B.counts + (size_t)r * T);
    }
    if (threadIdx.x == 0) {
        atomicAdd(B.particle_steps, (unsigned long long)n);
        RepState o;
        o.n = n_final;
        o.n_in = nin_final;
        o.cur = cur;
        o.next_id = next_id;
        o.status = st.status | sh_status;
        o.pad = 0;
        B.state[r] = o;
    }
    __syncthreads();
}

__device__ void replica_step(const BatchDev &B, int r, const SmemLayout &S, const RxnTables &rt, uint64_t bd_step,
                             uint64_t rx_step) {
    __shared__ RepDesc D;
    __shared__ RepState st;
    __shared__ int sh_nev, sh_status;
    if (threadIdx.x == 0) {
        D = B.desc[r];
        st = B.state[r];
        sh_nev = 0;
        sh_status = 0;
    }
    __syncthreads();
    if (D.smem_cells) replica_body(B, r, S, rt, bd_step, rx_step, D, st, sh_nev, sh_status, S.cells);
    else replica_body(B, r, S, rt, bd_step, rx_step, D, st, sh_nev, sh_status, B.start + D.soff);
}

__global__ void __launch_bounds__(512, 1) k_batch_step(BatchDev B) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int sh_r;
    __shared__ int sh_rt_ints[MAX_TYPES + MAX_REACTIONS * 3 + MAX_TYPES * MAX_TYPES + MAX_TYPES];
    __shared__ float sh_rt_scr[MAX_TYPES * MAX_TYPES];
    __shared__ float sh_pair_scr[MAX_TYPES * MAX_TYPES];
    __shared__ ReactionDev sh_rx[MAX_REACTIONS];
    __shared__ float sh_drift[MAX_TYPES], sh_scale[MAX_TYPES];
    const Tables *tab = B.tab;
    const int T = tab->ntypes, NP = tab->npots;
    SmemLayout S = carve(smem, T, NP, B.max_events_sm);
    S.drift = sh_drift;
    S.scale = sh_scale;
    S.screen = sh_pair_scr;
    for (int k = threadIdx.x; k < T * T; k += blockDim.x) {
        S.tab[k] = tab->pair_tab[k];
        sh_pair_scr[k] = tab->pair_screen[k];
    }
    for (int k = threadIdx.x; k < NP; k += blockDim.x) S.pots[k] = tab->pots[k];
    for (int k = threadIdx.x; k < T; k += blockDim.x) {
        sh_drift[k] = tab->bd_drift[k];
        sh_scale[k] = tab->bd_scale[k];
    }
    const RxnTables rt = stage_rxn_tables(tab, sh_rt_ints, sh_rt_scr, sh_rx);
    const uint64_t bd_step = B.step[0], rx_step = B.step[1];
    __syncthreads();
    for (;;) {
        if (threadIdx.x == 0) sh_r = atomicAdd(B.work, 1);
        __syncthreads();
        const int w = sh_r;
        __syncthreads();
        if (w >= B.R) break;
        replica_step(B, B.order[w], S, rt, bd_step, rx_step);
    }
}

__global__ void k_batch_advance(BatchDev B) {
    B.step[0] += 1;
    B.step[1] += 1;
    *B.work = 0;
}

// initial binning and sort of every replica (state.cur selects the source); the cell starts are
// sorted in the global start array
__global__ void k_batch_sort(BatchDev B) {
    __shared__ int sh_r;
    for (;;) {
        if (threadIdx.x == 0) sh_r = atomicAdd(B.work, 1);
        __syncthreads();
        const int r = sh_r;
        __syncthreads();
        if (r >= B.R) break;
        const RepDesc D = B.desc[r];
        RepState st = B.state[r];
        float4 *posX = (st.cur ? B.posB : B.posA) + D.poff;
        uint32_t *idX = (st.cur ? B.idB : B.idA) + D.poff;
        float4 *posY = (st.cur ? B.posA : B.posB) + D.poff;
        uint32_t *idY = (st.cur ? B.idA : B.idB) + D.poff;
        int *bin = B.bin + D.poff, *rank = B.rank + D.poff, *src = B.src + D.poff;
        int *cells = B.start + D.soff;
        block_bin(posX, st.n, bin, D.geo);
        block_rank(st.n, bin, rank, cells, D.geo.ncells + 2);
        int n2, nin2;
        block_sort(posX, idX, st.n, posY, idY, bin, rank, src, cells, D.geo, n2, nin2);
        if (threadIdx.x == 0) {
            st.n = n2;
            st.n_in = nin2;
            st.cur ^= 1;
            B.state[r] = st;
        }
        __syncthreads();
    }
}

__global__ void k_batch_count(BatchDev B, unsigned long long *out) {
    for (int r = blockIdx.x; r < B.R; r += gridDim.x) {
        const RepDesc &D = B.desc[r];
        const RepState st = B.state[r];
        const float4 *pos = (st.cur ? B.posB : B.posA) + D.poff;
        block_count_types(pos, st.n, B.tab->ntypes, out + (size_t)r * B.tab->ntypes);
    }
}

__global__ void k_fill_ids_batch(BatchDev B) {
    for (int r = blockIdx.x; r < B.R; r += gridDim.x) {
        const RepDesc &D = B.desc[r];
        const RepState st = B.state[r];
        uint32_t *id = (st.cur ? B.idB : B.idA) + D.poff;
        for (int i = threadIdx.x; i < st.n; i += blockDim.x) id[i] = (uint32_t)i;
    }
}

}  // namespace rdc

// ---------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------
namespace {
thread_local std::string b_err;

template <typename T>
T *balloc(size_t n) {
    void *p = nullptr;
    if (n == 0) n = 1;
    RDC_CUDA(cudaMalloc(&p, n * sizeof(T)));
    return static_cast<T *>(p);
}
template <typename T>
void bfree(T *&p) {
    if (p) cudaFree((void *)p);
    p = nullptr;
}

uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
}  // namespace

// context accessor shared with rdc_api.cu
namespace rdc {
const ContextData &context_data(const rdc_context *ctx);
uint64_t replica_seed(uint64_t seed, int replica) { return splitmix64(seed ^ (0x5DEECE66Dull * (uint64_t)(replica + 1))); }
}  // namespace rdc

struct rdc_batch {
    ContextData ctx;
    int R = 0;
    uint64_t seed = 0;
    cudaStream_t stream = nullptr;
    std::vector<RepDesc> desc;
    std::vector<int64_t> caps;
    std::vector<double> boxes;
    BatchDev d{};
    RepDesc *desc_dev = nullptr;
    RepState *state_dev = nullptr;
    int *order_dev = nullptr;
    Tables tab{};
    Tables *tab_dev = nullptr;
    double dt = 0;
    int handler = H_GILLESPIE;
    double cell_scale = 1.0;  // cell width = cutoff * cell_scale (at least)
    int threads = 256;
    int blocks = 0;
    size_t smem = 0;
    cudaGraphExec_t graph = nullptr;
    unsigned long long *count_dev = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    ~rdc_batch() { release(); }

    void release() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        bfree(desc_dev); bfree(state_dev); bfree(order_dev); bfree(tab_dev); bfree(count_dev);
        bfree(d.posA); bfree(d.posB); bfree(d.idA); bfree(d.idB);
        bfree(d.bin); bfree(d.rank); bfree(d.src); bfree(d.claim); bfree(d.taken);
        bfree(d.start); bfree(d.events); bfree(d.work); bfree(d.step); bfree(d.counts);
        bfree(d.reaction_counts); bfree(d.particle_steps);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }

    void sync() { RDC_CUDA(cudaStreamSynchronize(stream)); }

    void invalidate_graph() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
    }

    // cell grids and offsets: cells at least cutoff * cell_scale wide, widened for a replica whose
    // grid would not fit the shared-memory cell array
    void layout() {
        const double cutoff = ctx.max_cutoff();
        int64_t poff = 0, soff = 0, eoff = 0;
        desc.resize(R);
        for (int r = 0; r < R; ++r) {
            RepDesc &D = desc[r];
            double w = cutoff * cell_scale;
            D.geo = make_geo(&boxes[3 * r], ctx.pbc, cutoff, 1, w);
            const bool small = caps[r] < 65536;  // cell starts fit 16 bits
            if (small)
                for (int k = 0; k < 64 && D.geo.ncells + 3 > SMEM_CELLS && cutoff > 0; ++k) {
                    w *= 1.05;
                    D.geo = make_geo(&boxes[3 * r], ctx.pbc, cutoff, 1, w);
                }
            D.smem_cells = (small && D.geo.ncells + 3 <= SMEM_CELLS) ? 1 : 0;
            if (!D.smem_cells) D.geo = make_geo(&boxes[3 * r], ctx.pbc, cutoff, 1, cutoff * cell_scale);
            D.pad = 0;
            D.poff = (int)poff;
            D.cap = (int)caps[r];
            D.soff = (int)soff;
            D.ecap = 64 + D.cap / 32;
            D.eoff = (int)eoff;
            D.seed = replica_seed(seed, r);
            poff += D.cap;
            soff += D.geo.ncells + 3;
            eoff += D.ecap;
            if (poff > INT_MAX / 2 || soff > INT_MAX / 2 || eoff > INT_MAX / 2)
                throw std::invalid_argument("batch too large for 32-bit offsets");
        }
        bfree(d.start); bfree(d.events);
        d.start = balloc<int>(soff);
        d.events = balloc<EventRec>(eoff);
        RDC_CUDA(cudaMemsetAsync(d.start, 0, sizeof(int) * soff, stream));
        bfree(desc_dev);
        desc_dev = balloc<RepDesc>(R);
        RDC_CUDA(cudaMemcpyAsync(desc_dev, desc.data(), sizeof(RepDesc) * R, cudaMemcpyHostToDevice, stream));
        d.desc = desc_dev;
        invalidate_graph();
    }

    void init(const ContextData &c, int nrep, const double *bx, const int64_t *cp, uint64_t s) {
        ctx = c;
        R = nrep;
        seed = s;
        boxes.assign(bx, bx + 3 * R);
        for (double &b : boxes) b = (double)(float)b;
        caps.assign(cp, cp + R);
        RDC_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        int64_t total = 0;
        for (int r = 0; r < R; ++r) {
            if (caps[r] <= 0) throw std::invalid_argument("replica capacity must be > 0");
            total += caps[r];
        }
        if (total > INT_MAX / 2) throw std::invalid_argument("batch capacity too large");
        d.R = R;
        d.posA = balloc<float4>(total); d.posB = balloc<float4>(total);
        d.idA = balloc<uint32_t>(total); d.idB = balloc<uint32_t>(total);
        d.bin = balloc<int>(total); d.rank = balloc<int>(total); d.src = balloc<int>(total);
        d.claim = balloc<int>(total); d.taken = balloc<int>(total);
        RDC_CUDA(cudaMemsetAsync(d.claim, 0x7f, sizeof(int) * total, stream));
        RDC_CUDA(cudaMemsetAsync(d.taken, 0, sizeof(int) * total, stream));
        d.work = balloc<int>(1);
        RDC_CUDA(cudaMemsetAsync(d.work, 0, sizeof(int), stream));
        d.step = balloc<uint64_t>(2);
        RDC_CUDA(cudaMemsetAsync(d.step, 0, sizeof(uint64_t) * 2, stream));
        d.counts = balloc<unsigned long long>((size_t)R * ctx.ntypes);
        RDC_CUDA(cudaMemsetAsync(d.counts, 0, sizeof(unsigned long long) * R * ctx.ntypes, stream));
        count_dev = balloc<unsigned long long>((size_t)R * ctx.ntypes);
        d.reaction_counts = balloc<unsigned long long>(MAX_REACTIONS);
        RDC_CUDA(cudaMemsetAsync(d.reaction_counts, 0, sizeof(unsigned long long) * MAX_REACTIONS, stream));
        d.particle_steps = balloc<unsigned long long>(1);
        RDC_CUDA(cudaMemsetAsync(d.particle_steps, 0, sizeof(unsigned long long), stream));
        RDC_CUDA(cudaEventCreate(&ev0));
        RDC_CUDA(cudaEventCreate(&ev1));
        state_dev = balloc<RepState>(R);
        RDC_CUDA(cudaMemsetAsync(state_dev, 0, sizeof(RepState) * R, stream));
        d.state = state_dev;
        // largest replicas first (longest-processing-time order for the work queue)
        order_dev = balloc<int>(R);
        d.order = order_dev;
        // tables: rounding bands sized for the largest box
        double bmax[3] = {0, 0, 0};
        for (int r = 0; r < R; ++r)
            for (int k = 0; k < 3; ++k) bmax[k] = std::max(bmax[k], boxes[3 * r + k]);
        build_tables(ctx, bmax, 0.0, tab);
        tab_dev = balloc<Tables>(1);
        RDC_CUDA(cudaMemcpyAsync(tab_dev, &tab, sizeof(Tables), cudaMemcpyHostToDevice, stream));
        d.tab = tab_dev;
        d.handler = handler;
        d.reactions = ctx.reactions.empty() ? 0 : 1;
        d.max_events_sm = 1024;
        layout();
        sync();
    }

    void set_order(const std::vector<int64_t> &n) {
        std::vector<int> ord(R);
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return n[a] > n[b]; });
        RDC_CUDA(cudaMemcpyAsync(order_dev, ord.data(), sizeof(int) * R, cudaMemcpyHostToDevice, stream));
        sync();
    }

    void sort_all() {
        RDC_CUDA(cudaMemsetAsync(d.work, 0, sizeof(int), stream));
        k_batch_sort<<<std::min(R, 4 * 152), 256, 0, stream>>>(d);
        RDC_CUDA(cudaMemsetAsync(d.work, 0, sizeof(int), stream));
    }

    void configure_launch() {
        smem = batch_smem_bytes(tab.ntypes, tab.npots, d.max_events_sm);
        RDC_CUDA(cudaFuncSetAttribute(k_batch_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        RDC_CUDA(cudaFuncSetAttribute(k_batch_step, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        int per_sm = 0;
        RDC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_step, threads, smem));
        int dev = 0, sms = 0;
        RDC_CUDA(cudaGetDevice(&dev));
        RDC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        blocks = std::max(1, std::min(R, std::max(1, per_sm) * sms));
    }

    void step(int64_t n) {
        if (dt <= 0) throw std::logic_error("rdc_batch_configure must set a time step first");
        if (!graph) {
            configure_launch();
            cudaGraph_t g;
            RDC_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            k_batch_step<<<blocks, threads, smem, stream>>>(d);
            k_batch_advance<<<1, 1, 0, stream>>>(d);
            RDC_CUDA(cudaStreamEndCapture(stream, &g));
            RDC_CUDA(cudaGraphInstantiate(&graph, g, 0));
            cudaGraphDestroy(g);
        }
        for (int64_t k = 0; k < n; ++k) RDC_CUDA(cudaGraphLaunch(graph, stream));
    }

    std::vector<RepState> states() {
        std::vector<RepState> h(R);
        RDC_CUDA(cudaMemcpyAsync(h.data(), state_dev, sizeof(RepState) * R, cudaMemcpyDeviceToHost, stream));
        sync();
        return h;
    }

    void check_status() {
        auto st = states();
        int any = 0;
        for (auto &s : st) any |= s.status;
        if (any) {
            for (auto &s : st) s.status = 0;
            RDC_CUDA(cudaMemcpyAsync(state_dev, st.data(), sizeof(RepState) * R, cudaMemcpyHostToDevice, stream));
            sync();
            if (any & ST_CAPACITY) throw rdc::CapacityError("replica particle capacity exceeded by reaction products");
            if (any & ST_EVENTS) throw rdc::CapacityError("replica reaction event buffer overflow");
            throw std::runtime_error("replica device status " + std::to_string(any));
        }
    }
};

namespace {
template <typename F>
int bguard(F &&f) {
    try {
        f();
        return RDC_OK;
    } catch (const rdc::CapacityError &e) {
        b_err = e.what();
        return RDC_ERR_CAPACITY;
    } catch (const rdc::CudaError &e) {
        b_err = e.what();
        return RDC_ERR_CUDA;
    } catch (const std::invalid_argument &e) {
        b_err = e.what();
        return RDC_ERR_INVALID_ARGUMENT;
    } catch (const std::logic_error &e) {
        b_err = e.what();
        return RDC_ERR_LOGIC;
    } catch (const std::exception &e) {
        b_err = e.what();
        return RDC_ERR_RUNTIME;
    }
}
}  // namespace

namespace rdc {
void set_last_error(const std::string &m);
}

#define BATCH_CALL(...)                                   \
    do {                                                  \
        int rc_ = bguard([&] { __VA_ARGS__; });           \
        if (rc_ != RDC_OK) rdc::set_last_error(b_err);    \
        return rc_;                                       \
    } while (0)

extern "C" {

int rdc_batch_create(rdc_batch **out, const rdc_context *ctx, int n_replicas, const double *boxes3,
                     const int64_t *capacities, uint64_t seed) {
    BATCH_CALL({
        if (!out || !ctx || !boxes3 || !capacities) throw std::invalid_argument("null argument");
        if (n_replicas <= 0) throw std::invalid_argument("n_replicas must be > 0");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            throw rdc::CudaError("no CUDA device available");
        }
        auto b = std::make_unique<rdc_batch>();
        b->init(rdc::context_data(ctx), n_replicas, boxes3, capacities, seed);
        *out = b.release();
    });
}

int rdc_batch_destroy(rdc_batch *b) {
    if (b) {
        if (b->stream) cudaStreamSynchronize(b->stream);
        delete b;
    }
    return RDC_OK;
}

int rdc_batch_set_particles(rdc_batch *b, const int64_t *offsets, const double *pos, const int *types) {
    BATCH_CALL({
        if (!b || !offsets || !pos || !types) throw std::invalid_argument("null argument");
        const int R = b->R;
        std::vector<float4> hp;
        std::vector<RepState> st(R);
        std::vector<int64_t> n(R);
        int64_t total = 0;
        for (int r = 0; r < R; ++r) total += b->desc[r].cap;
        hp.assign(total, make_float4(0, 0, 0, 0));
        for (int r = 0; r < R; ++r) {
            n[r] = offsets[r + 1] - offsets[r];
            if (n[r] < 0 || n[r] > b->desc[r].cap) throw std::invalid_argument("replica particle count exceeds capacity");
            for (int64_t i = 0; i < n[r]; ++i) {
                const int64_t k = offsets[r] + i;
                const int t = types[k];
                if (t < 0 || t >= b->ctx.ntypes) throw std::invalid_argument("particle type out of range");
                float4 p;
                p.x = (float)pos[3 * k]; p.y = (float)pos[3 * k + 1]; p.z = (float)pos[3 * k + 2];
                std::memcpy(&p.w, &t, 4);
                hp[b->desc[r].poff + i] = p;
            }
            st[r] = RepState{(int)n[r], 0, 0, (int)n[r], 0, 0};
        }
        RDC_CUDA(cudaMemcpyAsync(b->d.posA, hp.data(), sizeof(float4) * total, cudaMemcpyHostToDevice, b->stream));
        RDC_CUDA(cudaMemcpyAsync(b->state_dev, st.data(), sizeof(RepState) * R, cudaMemcpyHostToDevice, b->stream));
        k_fill_ids_batch<<<std::min(R, 1024), 256, 0, b->stream>>>(b->d);
        b->set_order(n);
        b->sort_all();
        b->sync();
    });
}

int rdc_batch_configure(rdc_batch *b, int handler, double dt, double cell_width_scale, int threads_per_block) {
    BATCH_CALL({
        if (!b) throw std::invalid_argument("null argument");
        if (handler != H_UNCONTROLLED_APPROXIMATION && handler != H_GILLESPIE)
            throw std::invalid_argument("unknown reaction handler");
        if (!(dt > 0)) throw std::invalid_argument("time step must be > 0");
        if (!(cell_width_scale >= 1.0 && cell_width_scale <= 8.0))
            throw std::invalid_argument("cell width scale must be in [1, 8]");
        if (threads_per_block < 64 || threads_per_block > 1024 || threads_per_block % 32)
            throw std::invalid_argument("threads per block must be a multiple of 32 in [64, 1024]");
        b->handler = handler;
        b->d.handler = handler;
        b->dt = dt;
        set_time_step(b->ctx, dt, b->tab);
        RDC_CUDA(cudaMemcpyAsync(b->tab_dev, &b->tab, sizeof(Tables), cudaMemcpyHostToDevice, b->stream));
        b->threads = threads_per_block;
        if (cell_width_scale != b->cell_scale) {
            b->cell_scale = cell_width_scale;
            b->layout();
            b->sort_all();
        }
        b->invalidate_graph();
        b->sync();
    });
}

int rdc_batch_step(rdc_batch *b, int64_t n_steps) {
    BATCH_CALL({
        if (!b) throw std::invalid_argument("null argument");
        if (n_steps < 0) throw std::invalid_argument("n_steps must be >= 0");
        b->step(n_steps);
    });
}

int rdc_batch_step_timed(rdc_batch *b, int64_t n_steps, double *device_ms) {
    BATCH_CALL({
        if (!b || !device_ms) throw std::invalid_argument("null argument");
        if (n_steps < 0) throw std::invalid_argument("n_steps must be >= 0");
        RDC_CUDA(cudaEventRecord(b->ev0, b->stream));
        b->step(n_steps);
        RDC_CUDA(cudaEventRecord(b->ev1, b->stream));
        RDC_CUDA(cudaEventSynchronize(b->ev1));
        float ms = 0.f;
        RDC_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
        *device_ms = ms;
    });
}

int rdc_batch_particle_steps(rdc_batch *b, uint64_t *particle_steps) {
    BATCH_CALL({
        if (!b || !particle_steps) throw std::invalid_argument("null argument");
        unsigned long long v = 0;
        RDC_CUDA(cudaMemcpyAsync(&v, b->d.particle_steps, sizeof(v), cudaMemcpyDeviceToHost, b->stream));
        b->sync();
        *particle_steps = v;
    });
}

int rdc_batch_count_types(rdc_batch *b, int64_t *counts) {
    BATCH_CALL({
        if (!b || !counts) throw std::invalid_argument("null argument");
        k_batch_count<<<std::min(b->R, 4 * 152), 256, 0, b->stream>>>(b->d, b->count_dev);
        std::vector<unsigned long long> h((size_t)b->R * b->ctx.ntypes);
        RDC_CUDA(cudaMemcpyAsync(h.data(), b->count_dev, sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost,
                                 b->stream));
        b->sync();
        for (size_t i = 0; i < h.size(); ++i) counts[i] = (int64_t)h[i];
    });
}

int rdc_batch_n_particles(rdc_batch *b, int64_t *n) {
    BATCH_CALL({
        if (!b || !n) throw std::invalid_argument("null argument");
        auto st = b->states();
        for (int r = 0; r < b->R; ++r) n[r] = st[r].n;
    });
}

int rdc_batch_get_particles(rdc_batch *b, int replica, int64_t cap, double *pos, int *types, uint64_t *ids,
                            int64_t *n_out) {
    BATCH_CALL({
        if (!b) throw std::invalid_argument("null argument");
        if (replica < 0 || replica >= b->R) throw std::invalid_argument("replica out of range");
        auto st = b->states();
        const RepState s = st[replica];
        const RepDesc &D = b->desc[replica];
        std::vector<float4> hp(s.n);
        std::vector<uint32_t> hid(s.n);
        if (s.n > 0) {
            RDC_CUDA(cudaMemcpyAsync(hp.data(), (s.cur ? b->d.posB : b->d.posA) + D.poff, sizeof(float4) * s.n,
                                     cudaMemcpyDeviceToHost, b->stream));
            RDC_CUDA(cudaMemcpyAsync(hid.data(), (s.cur ? b->d.idB : b->d.idA) + D.poff, sizeof(uint32_t) * s.n,
                                     cudaMemcpyDeviceToHost, b->stream));
        }
        b->sync();
        int64_t k = 0;
        for (int i = 0; i < s.n; ++i) {
            int t;
            std::memcpy(&t, &hp[i].w, 4);
            if (t < 0) continue;
            if (k < cap) {
                if (pos) { pos[3 * k] = hp[i].x; pos[3 * k + 1] = hp[i].y; pos[3 * k + 2] = hp[i].z; }
                if (types) types[k] = t;
                if (ids) ids[k] = hid[i];
            }
            ++k;
        }
        if (n_out) *n_out = k;
        if (k > cap) throw rdc::CapacityError("output capacity too small for the particles");
    });
}

int rdc_batch_synchronize(rdc_batch *b) {
    BATCH_CALL({
        if (!b) throw std::invalid_argument("null argument");
        b->sync();
        RDC_CUDA(cudaGetLastError());
        b->check_status();
    });
}

}  // extern "C"

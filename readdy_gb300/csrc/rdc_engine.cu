// Device side of the fused replica engine (declarations and overview in rdc_engine.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "rdc_engine.h"
#include "rdc_phases.cuh"

namespace rdc {

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

// 16-bit cell starts between global and shared memory, 8 entries per 16-byte access; both arrays are
// 16-byte aligned and padded to a multiple of 8 entries
__device__ inline void copy_starts16(uint16_t *dst, const uint16_t *src, int n) {
    const int nv = (n + 7) >> 3;
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
    for (int k = threadIdx.x; k < nv; k += blockDim.x) d4[k] = s4[k];
    __syncthreads();
}

// int cell starts narrowed to 16 bits in place (values < 65536): chunk by chunk every thread reads its
// int before any thread writes, and the 16-bit writes of a chunk only cover ints already read
__device__ inline void narrow_starts_inplace(int *a, int n) {
    uint16_t *b = reinterpret_cast<uint16_t *>(a);
    for (int base = 0; base < n; base += blockDim.x) {
        const int k = base + (int)threadIdx.x;
        const int v = k < n ? a[k] : 0;
        __syncthreads();
        if (k < n) b[k] = (uint16_t)v;
        __syncthreads();
    }
}

// in-place exclusive scan of a[0..n) by one block (shared or global memory); a[n] = total
template <typename T>
__device__ inline void block_scan_inplace(T *a, int n) {
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    constexpr int ITEMS = 8;
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
    {   // zero 8 counters per 16-byte store (the shared array is 16-byte aligned and padded)
        uint4 *c4 = reinterpret_cast<uint4 *>(cells);
        for (int k = threadIdx.x; k < (nbins + 7) >> 3; k += blockDim.x) c4[k] = make_uint4(0u, 0u, 0u, 0u);
        __syncthreads();
    }
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
// by particle id (deterministic, and independent of the order of the source arrays), gather into the
// destination arrays
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
    // order every bin (cells and the out-of-box bin) holding two or more particles by id;
    // the particle of rank 0 in a bin does it, so the loop runs over particles, not over the 4x more cells
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int c = bin[i];
        if (c > nc || rank[i] != 0) continue;
        const int b = cells[c], e = cells[c + 1];
        if (e - b < 2) continue;
        if (e - b > CELL_SORT_SMALL) {
            const int q = atomicAdd(&nbig, 1);
            if (q < 64) big[q] = c;
            continue;
        }
        insertion_sort_by(src, b, e, sid);
    }
    __syncthreads();
    // crowded cells: ordered by the whole block (rank[] is free scratch now)
    if (nbig <= 64) {
        for (int q = 0; q < nbig; ++q)
            block_rank_sort_by(src, const_cast<int *>(rank), cells[big[q]], cells[big[q] + 1], sid);
    } else {
        for (int c = 0; c <= nc; ++c)
            if (cells[c + 1] - cells[c] > CELL_SORT_SMALL)
                block_rank_sort_by(src, const_cast<int *>(rank), cells[c], cells[c + 1], sid);
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

// dynamic shared memory: event keys, potentials and the type-pair table of the largest context,
// resolution scratch, the event tuple queue, then the 16-bit cell array
__device__ inline SmemLayout carve(unsigned char *smem, int max_events) {
    SmemLayout L;
    size_t off = 0;
    L.key = reinterpret_cast<uint64_t *>(smem + off);
    off += sizeof(uint64_t) * max_events;
    L.pots = reinterpret_cast<PairPot *>(smem + off);
    off += sizeof(PairPot) * MAX_PAIR_POTENTIALS;
    L.tab = reinterpret_cast<int *>(smem + off);
    off += sizeof(int) * MAX_TYPES * MAX_TYPES;
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

size_t engine_smem_bytes(int max_events) {
    return sizeof(uint64_t) * max_events + sizeof(PairPot) * MAX_PAIR_POTENTIALS + sizeof(int) * MAX_TYPES * MAX_TYPES +
           2 * sizeof(int) * max_events + (2 * sizeof(int) + 1) * EVENT_QUEUE + 4 * sizeof(int) +
           sizeof(uint16_t) * (SMEM_CELLS + 4) + 16;
}

// The candidate pass of block_events and the pair forces of the same sorted state in one stencil walk
// per particle: the walk that sums particle i's pair forces also finds its reaction partners j > i,
// and force[i] receives the sum (zero outside the cells).  The walk runs without block barriers, like
// the plain force walk.  It keeps up to two partner candidates in registers, tries their reactions
// after the walk and lists the tuples then (measured: an atomic list append inside the divergent
// candidate loop made the walk 8x slower); a particle with more candidates lists its tuples by its
// own event walk.  The list holds up to `room`
// tuples in global scratch (tp1, tp2, tr) and the coins are drawn after it with all lanes converged;
// a list that overflows is dropped and block_events generates the tuples again.  Tuples, coins and
// forces are those of block_events and pair_force_at on their own.
template <typename G, typename Emit>
__device__ __forceinline__ void block_events_forces(int n, int n_in, const float4 *__restrict__ pos,
                                                    const uint32_t *__restrict__ id,
                                                    const uint16_t *__restrict__ start, const G &g,
                                                    const SmemLayout &S, int T, bool pair_pots, const RxnTables &rt,
                                                    uint64_t seed, uint64_t step, int handler,
                                                    float4 *__restrict__ force, int *tp1, int *tp2, int *tr, int room,
                                                    int *status, Emit emit) {
    int *count = S.queue.count;
    auto push = [&](int a, int b, int r) {
        const int k = atomicAdd(count, 1);
        if (k < room) {
            tp1[k] = a;
            tp2[k] = b;
            tr[k] = r;
        }
    };
    // warps take 32-particle chunks from a counter: the walks differ in length, and a static split
    // leaves warps waiting at the barrier after the walk
    int *next = S.queue.count + 3;
    if (threadIdx.x == 0) {
        *count = 0;
        *next = 0;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    // per type: the largest force or reaction screen, as far as the walk of a particle of that type reaches,
    // and the types it has a pair potential or a pair reaction with
    __shared__ float sh_reach[MAX_TYPES];
    __shared__ uint32_t sh_mask[MAX_TYPES];
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
        float r2 = 0.f;
        uint32_t m = 0u;
        for (int u = 0; u < T; ++u) {
            if (S.tab[t * T + u]) {
                r2 = fmaxf(r2, S.screen[t * T + u]);
                m |= 1u << u;
            }
            if (rt.o2_any[t] && rt.o2_tab[t * rt.T + u]) {
                r2 = fmaxf(r2, rt.screen[t * rt.T + u]);
                m |= 1u << u;
            }
        }
        sh_reach[t] = r2;
        sh_mask[t] = m;
    }
    __syncthreads();
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(next, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const int i = base + lane;
        if (i >= n) continue;
        const float4 p = pos[i];
        const int ti = itype(p);
        float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
        if (ti >= 0) {
            const bool pairs = i < n_in && rt.o2_any[ti];
            int t0 = 0, t1 = 0, nt = 0;  // partner tuples j | r << 16 (j < 65536 in shared-memory replicas)
            if (i < n_in && (pairs || pair_pots)) {
                const int *rrow = rt.o2_tab + ti * rt.T;
                const float *rsrow = rt.screen + ti * rt.T;
                // the cells walked reach as far as the largest force or reaction screen of i's type (a walking
                // particle is inside the cells, so its type's reaction screens count when it has any)
                // partner candidates j > i inside a reaction screen, in candidate order; their reactions are
                // tried after the walk, with the lanes converged, instead of inside the divergent loop
                int c0 = 0, c1 = 0, nc = 0;
                auto partner = [&](int j, float4, int tj, float d2s) {
                    if (!pairs || j < i) return;
                    const int o2 = rrow[tj];
                    if (o2 == 0 || d2s > rsrow[tj]) return;
                    if (nc == 0) c0 = j;
                    else if (nc == 1) c1 = j;
                    ++nc;
                };
                pair_force_at(i, p, pos, start, g, 1, S.tab, S.screen, S.pots, T, fx, fy, fz, e, nullptr, partner,
                              sh_reach[ti], sh_mask[ti]);
                if (nc > 2) {
                    nt = 3;  // more candidates than registers: its own event walk lists the tuples
                } else {
                    for (int c = 0; c < nc; ++c) {
                        const int j = c == 0 ? c0 : c1;
                        const float4 q = pos[j];
                        const int o2 = rrow[itype(q)];
                        const PairGeom g0 = pair_geom(p, q, g);
                        for (int k = (o2 >> 8); k < (o2 >> 8) + (o2 & 0xff); ++k) {
                            const int r = rt.o2_list[k];
                            const ReactionDev &R = rt.rx[r];
                            if (!R.active) continue;
                            PairGeom gg = g0;
                            if (within(g0, gg, p, q, g, R.educt_distance2f, R.band, R.educt_distance2)) {
                                if (nt == 0) t0 = j | (r << 16);
                                else if (nt == 1) t1 = j | (r << 16);
                                ++nt;
                            }
                        }
                    }
                }
            }
            if (nt > 2) {
                event_tuples_at(i, true, pos, start, g, 1, rt, push);
            } else {
                const int o1 = rt.o1_tab[ti];
                for (int k = (o1 >> 8); k < (o1 >> 8) + (o1 & 0xff); ++k) {
                    const int r = rt.o1_list[k];
                    if (rt.rx[r].active) push(i, i, r);
                }
                if (nt > 0) push(i, t0 & 0xffff, t0 >> 16);
                if (nt > 1) push(i, t1 & 0xffff, t1 >> 16);
            }
        }
        force[i] = make_float4(fx, fy, fz, 0.f);
    }
    __syncthreads();
    const int nq = *count;
    __syncthreads();
    if (nq > room) {
        block_events(0, blockDim.x, n, n_in, pos, id, start, g, 1, rt, seed, step, handler, S.queue, emit);
        return;
    }
    for (int k = threadIdx.x; k < nq; k += blockDim.x) {
        const int a = tp1[k], b = tp2[k], r = tr[k];
        if ((unsigned)a < (unsigned)n && (unsigned)b < (unsigned)n && (unsigned)r < (unsigned)MAX_REACTIONS)
            event_coin(a, b, r, id, rt, seed, step, handler, emit);
        else
            atomicOr(status, ST_INDEX);
    }
    __syncthreads();
}

// sets the bits of the cells of the 3x3x3 stencil around cell c: the cells whose particles see c
// (the stencil relation is symmetric)
__device__ inline void mark_stencil(uint32_t *mark, int c, const Geo &g) {
    const int dy = g.dims[1], dz = g.dims[2];
    int ax[3], ay[3], az[3];
    const int nx = axis_cells(c / (dy * dz), g.dims[0], g.pbc[0], 1, ax);
    const int ny = axis_cells((c / dz) % dy, dy, g.pbc[1], 1, ay);
    const int nz = axis_cells(c % dz, dz, g.pbc[2], 1, az);
    for (int a = 0; a < nx; ++a)
        for (int b = 0; b < ny; ++b)
            for (int k = 0; k < nz; ++k) {
                const int m = az[k] + dz * (ay[b] + dy * ax[a]);
                atomicOr(&mark[m >> 5], 1u << (m & 31));
            }
}

__device__ inline bool marked(const uint32_t *mark, int c) { return (mark[c >> 5] >> (c & 31)) & 1u; }

// first entry of the ascending keys[0, n) that is >= v
__device__ inline int lower_bound_u64(const uint64_t *keys, int n, uint64_t v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (keys[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Particles a step's reactions changed, in a state they left unsorted: the sorted storage of the step
// (cell starts `start`, cells in particle-id order) with removed particles (type < 0), particles that
// took part in a performed reaction (flagged in `taken`: they may have moved and have new ids) and the
// births appended.  `mkey` lists the changed particles inside the box as cell << 32 | id, ascending,
// with their storage indices in `midx`.
struct Changed {
    const uint64_t *mkey;
    const int *midx;
    int n;
    const int *taken;
    const uint32_t *bloom;  // CHANGED_BLOOM_BITS bits over the cells of mkey, then as many over changed indices
    int nstore;             // storage slots of the state; an index outside raises ST_INDEX
    int *status;
};

// single-hash Bloom filters in shared memory that spare the walks a search or a global flag load for
// the cells and particles no reaction touched (a hit is confirmed exactly)
constexpr int CHANGED_BLOOM_BITS = 4096;
static_assert(2 * CHANGED_BLOOM_BITS / 8 <= EVENT_QUEUE, "the filters live in the tuple queue's reaction bytes");
__device__ inline bool bloom_has(const uint32_t *b, int v) {
    const int h = v & (CHANGED_BLOOM_BITS - 1);
    return (b[h >> 5] >> (h & 31)) & 1u;
}
__device__ inline void bloom_add(uint32_t *b, int v) {
    const int h = v & (CHANGED_BLOOM_BITS - 1);
    atomicOr(&b[h >> 5], 1u << (h & 31));
}

// Pair force on particle i of such a state, with the candidates in the order of the sorted state: per
// stencil cell, the cell's unchanged storage range merged by id with the changed particles now in the
// cell -- the order in which block_sort would store them.  The candidates are listed first (shared
// memory only, up to UNSORTED_CANDIDATES) and then walked with the next position loaded ahead, as in
// for_each_candidate_q; a longer list is walked cell by cell.  The arithmetic is pair_force_at's.
constexpr int UNSORTED_CANDIDATES = 48;

template <typename G>
__device__ inline void pair_force_unsorted(int i, float4 p, const float4 *__restrict__ pos,
                                           const uint32_t *__restrict__ id, const uint16_t *__restrict__ start,
                                           const G &g, const Changed &X, const int *tab, const float *screen,
                                           const PairPot *pots, int T, float &fx, float &fy, float &fz) {
    const int ti = itype(p);
    const int *trow = tab + ti * T;
    const float *srow = screen + ti * T;
    float e = 0.f;
    auto visit = [&](int j, float4 q) {
        if (j == i) return;
        const int tj = itype(q);
        if (tj < 0 || trow[tj] == 0) return;
        if (screen_d2(p, q, g) > srow[tj]) return;
        pair_force_body(p, q, g, trow[tj], pots, fx, fy, fz, e);
    };
    const uint32_t *bloom_idx = X.bloom + CHANGED_BLOOM_BITS / 32;
    // f(j) for the candidates in order; an index outside the storage raises ST_INDEX and is skipped
    auto candidates = [&](auto f) {
        for_each_neighbor_cell(p, g, [&](int c) {
            const int je = start[c + 1];
            // the next member of the cell's storage range that is unchanged (a removed one is skipped
            // by visit; one that reacted is flagged in taken)
            auto member = [&](int j) {
                while (j < je && bloom_has(bloom_idx, j) && X.taken[j]) ++j;
                return j;
            };
            int j = member(start[c]);
            // changed particles now in c: entries x with cell c, from the first key >= c << 32
            int x = bloom_has(X.bloom, c) ? lower_bound_u64(X.mkey, X.n, (uint64_t)c << 32) : X.n;
            auto in_c = [&](int x) { return x < X.n && (int)(X.mkey[x] >> 32) == c; };
            while (j < je || in_c(x)) {
                int k;
                if (in_c(x) && (j >= je || (uint32_t)X.mkey[x] < id[j])) {
                    k = X.midx[x];
                    ++x;
                } else {
                    k = j;
                    j = member(j + 1);
                }
                if ((unsigned)k < (unsigned)X.nstore) f(k);
                else atomicOr(X.status, ST_INDEX);
            }
        });
    };
    int cand[UNSORTED_CANDIDATES];
    int nc = 0;
    candidates([&](int k) {
        if (nc < UNSORTED_CANDIDATES) cand[nc] = k;
        ++nc;
    });
    if (nc > UNSORTED_CANDIDATES) {
        candidates([&](int k) { visit(k, pos[k]); });
        return;
    }
    if (nc == 0) return;
    float4 q = pos[cand[0]];
    for (int k = 0; k < nc; ++k) {
        float4 qn = q;
        if (k + 1 < nc) qn = pos[cand[k + 1]];
        visit(cand[k], q);
        q = qn;
    }
}

// After the reactions of a replica that carries its forces, without sorting again: the particles of
// the marked cells get their pair forces again (in force[], by storage index), walked over the state
// as the reactions left it.  The performed events are events[idx[k]] for state[k] == 1, k < n_events
// (block_resolve_apply's scratch); births are storage slots [n1, n1 + births).  Scratch: mkey and midx
// (cap entries), tmp and list (one entry per storage slot), cnt (2 ints), bloom (2 CHANGED_BLOOM_BITS
// bits).  Returns false when the
// changed particles do not fit mkey; only zero forces of changed particles outside the box are
// written then.  Every storage index is checked against the n1 + births slots; one outside raises
// ST_INDEX in *status and its access is skipped.
template <typename G>
__device__ inline bool refresh_in_place(const float4 *__restrict__ pos, const uint32_t *__restrict__ id, int n1,
                                        int births, const EventRec *events, const int *idx, const int *state,
                                        int n_events, const uint32_t *mark, const uint16_t *start,
                                        const Geo &gs, const G &g, int *taken, uint64_t *mkey, int *midx, int cap,
                                        int *tmp,
                                        int *list, int *cnt, uint32_t *bloom, const SmemLayout &S, int T,
                                        bool pair_pots, float4 *force, int *status) {
    const int nc = gs.ncells;
    const int nstore = n1 + births;
    auto inside = [&](int q) {
        if ((unsigned)q < (unsigned)nstore) return true;
        atomicOr(status, ST_INDEX);
        return false;
    };
    // every particle of a performed event and every birth: flagged, listed when inside the box
    auto each_changed = [&](auto f) {
        for (int k = threadIdx.x; k < n_events + births; k += blockDim.x) {
            if (k < n_events) {
                if (state[k] != 1) continue;
                const EventRec e = events[idx[k]];
                f(e.p1);
                if (e.p2 != e.p1) f(e.p2);
            } else {
                f(n1 + k - n_events);
            }
        }
    };
    if (threadIdx.x == 0) { cnt[0] = 0; cnt[1] = 0; }
    for (int k = threadIdx.x; k < 2 * CHANGED_BLOOM_BITS / 32; k += blockDim.x) bloom[k] = 0u;
    __syncthreads();
    each_changed([&](int q) {
        if (!inside(q)) return;
        const float4 p = pos[q];
        if (itype(p) < 0) return;  // removed
        taken[q] = 1;
        bloom_add(bloom + CHANGED_BLOOM_BITS / 32, q);
        const int c = bin_of(p, gs);
        if (c == nc) {  // outside the box: no pair forces
            force[q] = make_float4(0.f, 0.f, 0.f, 0.f);
            return;
        }
        bloom_add(bloom, c);
        const int x = atomicAdd(&cnt[0], 1);
        if (x < cap) {
            mkey[x] = ((uint64_t)c << 32) | id[q];
            midx[x] = q;
        }
    });
    __syncthreads();
    const int nm = cnt[0];
    const bool fits = nm <= cap;
    if (fits) {
        // ascending keys (distinct: ids are): ranks place the indices, the keys follow
        for (int x = threadIdx.x; x < nm; x += blockDim.x) {
            const uint64_t v = mkey[x];
            int r = 0;
            for (int y = 0; y < nm; ++y) r += mkey[y] < v;
            tmp[r] = midx[x];
        }
        __syncthreads();
        for (int x = threadIdx.x; x < nm; x += blockDim.x) {
            const int q = tmp[x];
            if (!inside(q)) continue;
            midx[x] = q;
            mkey[x] = ((uint64_t)bin_of(pos[q], gs) << 32) | id[q];
        }
        __syncthreads();
        // the particles now in marked cells: unchanged storage-range members, then the changed ones
        for (int w = threadIdx.x; w < (nc + 31) / 32; w += blockDim.x) {
            uint32_t bits = mark[w];
            while (bits) {
                const int c = w * 32 + __ffs(bits) - 1;
                bits &= bits - 1;
                for (int j = start[c]; j < start[c + 1]; ++j)
                    if (!(bloom_has(bloom + CHANGED_BLOOM_BITS / 32, j) && taken[j]) && itype(pos[j]) >= 0) {
                        const int l = atomicAdd(&cnt[1], 1);
                        if (inside(l)) list[l] = j;
                    }
            }
        }
        for (int x = threadIdx.x; x < nm; x += blockDim.x) {
            const int l = atomicAdd(&cnt[1], 1);
            if (inside(l)) list[l] = midx[x];
        }
        __syncthreads();
        // each particle is listed once (a storage-range member of its own cell, or changed)
        const int nl = min(cnt[1], nstore);
        const Changed X{mkey, midx, nm, taken, bloom, nstore, status};
        // entry l goes to lane l / warps of warp l % warps: the few walks spread over the warps instead
        // of diverging inside the first one
        const int warps = blockDim.x >> 5;
        for (int l0 = 0; l0 < nl; l0 += blockDim.x) {
            const int l = l0 + (int)(threadIdx.x & 31) * warps + (int)(threadIdx.x >> 5);
            if (l >= nl) continue;
            const int k = list[l];
            if (!inside(k)) continue;
            float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
            if (pair_pots)
                pair_force_unsorted(k, pos[k], pos, id, start, g, X, S.tab, S.screen, S.pots, T, f.x, f.y, f.z);
            force[k] = f;
        }
    }
    __syncthreads();
    each_changed([&](int q) {
        if ((unsigned)q < (unsigned)nstore) taken[q] = 0;
    });
    __syncthreads();
    return fits;
}

// one step of one replica by the whole block; C is the cell array's type (uint16_t in shared memory
// or int in global memory).  Inlined into the kernel: compiled as a call it took a 700-byte stack frame
// per thread (the arguments it passes down by reference live in local memory), 232 bytes inlined.
template <typename C>
__device__ __forceinline__ void replica_body(const EngineDev &E, int r, const SmemLayout &S, const RxnTables &rt,
                                             const Tables *tab, const RepDesc &D, const RepState &st, int &sh_nev,
                                             int &sh_status, C *cells) {
    const int T = tab->ntypes, NP = tab->npots;
    const uint64_t step = (uint64_t)st.step;
    const Geo &gs = D.geo;
    const GeoR g = geo_r(gs);
    const int nc = gs.ncells;
    float4 *posX = D.pos[st.cur];
    uint32_t *idX = D.id[st.cur];
    float4 *posY = D.pos[st.cur ^ 1];
    uint32_t *idY = D.id[st.cur ^ 1];
    int *bin = D.bin, *rank = D.rank, *src = D.src;
    int *gstart = D.start;
    constexpr bool in_smem = sizeof(C) == sizeof(uint16_t);
    const int n = st.n, n_in = st.n_in;
    // forces stored by the previous step's event walk (replicas with reactions and shared-memory cells);
    // the state is then the one the reactions left, unsorted, with removed particles in place
    const bool fuse = in_smem && tab->nreactions > 0 && D.force[0] != nullptr;
    const float4 *fX = (fuse && st.fvalid) ? D.force[st.cur] : nullptr;
    // otherwise the state is sorted and a shared-memory replica keeps its starts as 16-bit entries in
    // its start array between steps
    if (in_smem && !fX)
        copy_starts16(reinterpret_cast<uint16_t *>(cells), reinterpret_cast<const uint16_t *>(gstart), nc + 3);

    // forces on the current state, Euler step into Y, bins of the new positions
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float4 p = posX[i];
        float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
        if (fX) {
            const float4 f = fX[i];
            fx = f.x; fy = f.y; fz = f.z;
        } else if (i < n_in && NP > 0) {
            pair_force_at(i, p, posX, cells, g, 1, S.tab, S.screen, S.pots, T, fx, fy, fz, e);
        }
        const uint32_t id = idX[i];
        const int t = itype(p);
        if (t >= 0) {  // order-1 potentials
            const int o1 = tab->o1pot_tab[t];
            if (o1) order1_force(p, tab->o1pots, o1 >> 8, o1 & 0xff, fx, fy, fz, e);
        }
        const float4 q = t >= 0 ? euler_bd(p, fx, fy, fz, id, D.seed, step, S.drift[t], S.scale[t], g) : p;
        posY[i] = q;
        idY[i] = id;
        bin[i] = bin_of(q, gs);
    }
    __syncthreads();
    block_rank(n, bin, rank, cells, nc + 2);
    int n1, nin1;
    block_sort(posY, idY, n, posX, idX, bin, rank, src, cells, gs, n1, nin1);

    int n_final = n1, nin_final = nin1, cur = st.cur, next_id = st.next_id, fvalid = 0;
    if (tab->nreactions > 0) {
        // the next step's forces come from this step's event walk unless this is the replica's last step
        const bool keep = fuse && st.step + 1 < D.n_steps;
        uint32_t *mark = reinterpret_cast<uint32_t *>(S.queue.p1);  // cell bitmap, free after the coins
        EventRec *ev = D.events;
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
        if (keep)
            // the sort scratch (bin, rank, src) is free until the re-sort: it holds the tuple list
            block_events_forces(n1, nin1, posX, idX, reinterpret_cast<const uint16_t *>(cells), g, S, T, NP > 0, rt,
                                D.seed, step, E.handler, D.force[st.cur], bin, rank, src, D.cap, &sh_status, emit);
        else
            block_events(0, blockDim.x, n1, nin1, posX, idX, cells, g, 1, rt, D.seed, step, E.handler, S.queue, emit);
        fvalid = keep ? 1 : 0;
        const int Ev = min(sh_nev, ecap);
        if (Ev > 0 && keep) {
            // cells around the educts, before the reactions move or remove them
            for (int k = threadIdx.x; k < (nc + 31) / 32; k += blockDim.x) mark[k] = 0u;
            __syncthreads();
            for (int k = threadIdx.x; k < 2 * Ev; k += blockDim.x) {
                const EventRec e = ev[k >> 1];
                const int c = bin_of(posX[(k & 1) ? e.p2 : e.p1], gs);
                if (c < nc) mark_stencil(mark, c, gs);
            }
            __syncthreads();
        }
        if (Ev > 0) {
            ApplyTarget t;
            t.pos = posX; t.id = idX; t.tslot = nullptr; t.force = nullptr;
            t.claim = D.claim; t.taken = D.taken;
            t.reaction_counts = D.rx_counts;
            t.n_total = n1;
            t.capacity = D.cap;
            t.next_id = (uint32_t)st.next_id;
            ApplyResult res;
            block_resolve_apply(ev, Ev, E.max_events_sm, S.key, S.idx, S.state, tab, gs, D.seed, step, t, res);
            next_id = st.next_id + res.ids;
            if (threadIdx.x == 0) sh_status |= res.status;
            const int n_total = n1 + res.births;
            bool sort_again = res.winners > 0;
            if (sort_again && keep) {
                // cells around the products and the births
                for (int k = threadIdx.x; k < 2 * Ev + res.births; k += blockDim.x) {
                    int q;
                    if (k < 2 * Ev) {
                        const EventRec e = ev[k >> 1];
                        q = (k & 1) ? e.p2 : e.p1;
                    } else {
                        q = n1 + k - 2 * Ev;
                    }
                    const int c = bin_of(posX[q], gs);
                    if (c < nc) mark_stencil(mark, c, gs);
                }
                __syncthreads();
                // the particles around them walk again over the state as it is; it stays unsorted (the
                // next step sorts after its Euler update anyway)
                if (refresh_in_place(posX, idX, n1, res.births, ev, S.idx, S.state, min(Ev, E.max_events_sm), mark,
                                     reinterpret_cast<const uint16_t *>(cells), gs, g, D.taken, S.key,
                                     S.queue.p2, E.max_events_sm, src, rank, S.queue.count + 1,
                                     reinterpret_cast<uint32_t *>(S.queue.r), S, T, NP > 0, D.force[st.cur],
                                     &sh_status)) {
                    n_final = n_total;
                    sort_again = false;
                }
            }
            if (sort_again) {
                // particles changed cells, appeared or vanished: sort again, into Y
                block_bin(posX, n_total, bin, gs);
                block_rank(n_total, bin, rank, cells, nc + 2);
                int n2, nin2;
                block_sort(posX, idX, n_total, posY, idY, bin, rank, src, cells, gs, n2, nin2);
                if (keep) {
                    // forces follow their particles; a particle whose stencil saw a reaction walks again
                    const float4 *fi = D.force[st.cur];
                    float4 *fo = D.force[st.cur ^ 1];
                    for (int i = threadIdx.x; i < n2; i += blockDim.x) {
                        const int k = src[i];
                        float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
                        if (i < nin2) {
                            if (!marked(mark, bin[k])) {
                                f = fi[k];
                            } else if (NP > 0) {
                                float e = 0.f;
                                pair_force_at(i, posY[i], posY, cells, g, 1, S.tab, S.screen, S.pots, T, f.x, f.y,
                                              f.z, e);
                            }
                        }
                        fo[i] = f;
                    }
                    __syncthreads();
                }
                n_final = n2;
                nin_final = nin2;
                cur ^= 1;
            }
        }
    }
    // a replica that carries its forces does not read its starts at the next step
    if (in_smem && !fvalid)
        copy_starts16(reinterpret_cast<uint16_t *>(gstart), reinterpret_cast<const uint16_t *>(cells), nc + 3);
    int rec = st.rec;
    if (D.records && D.count_stride > 0 && (step + 1) % (uint64_t)D.count_stride == 0 && rec < D.max_records) {
        block_count_types(D.pos[cur], n_final, T, D.records + (size_t)rec * (D.record_pitch ? (size_t)D.record_pitch : (size_t)T));
        ++rec;
    }
    if (threadIdx.x == 0) {
        atomicAdd(E.particle_steps, (unsigned long long)n1);
        RepState o;
        o.n = n_final;
        o.n_in = nin_final;
        o.cur = cur;
        o.next_id = next_id;
        o.status = st.status | sh_status;
        o.rec = rec;
        o.fvalid = fvalid;
        o.step = st.step + 1;
        E.state[r] = o;
    }
    __syncthreads();
}

// Stages the potential and reaction tables of a context into shared memory (whole block).
__device__ inline RxnTables stage_tables(const Tables *tab, const SmemLayout &S, int *rt_ints, float *rt_screen,
                                         ReactionDev *rt_rx) {
    const int T = tab->ntypes, NP = tab->npots;
    for (int k = threadIdx.x; k < T * T; k += blockDim.x) {
        S.tab[k] = tab->pair_tab[k];
        S.screen[k] = tab->pair_screen[k];
    }
    for (int k = threadIdx.x; k < NP; k += blockDim.x) S.pots[k] = tab->pots[k];
    for (int k = threadIdx.x; k < T; k += blockDim.x) {
        S.drift[k] = tab->bd_drift[k];
        S.scale[k] = tab->bd_scale[k];
    }
    return stage_rxn_tables(tab, rt_ints, rt_screen, rt_rx);
}

// MULTI: replicas may take several steps per launch (E.launch_steps).  A separate instantiation, so that
// the batched form, which always takes one, keeps the register allocation of the single step (the loop
// cost it 5 %).
template <bool MULTI>
__global__ void __launch_bounds__(ENGINE_THREADS_MAX, 1) k_engine_step(EngineDev E) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int sh_r, sh_table, sh_nev, sh_status;
    __shared__ RepDesc D;
    __shared__ RepState st;
    __shared__ int sh_rt_ints[MAX_TYPES + MAX_REACTIONS * 3 + MAX_TYPES * MAX_TYPES + MAX_TYPES];
    __shared__ float sh_rt_scr[MAX_TYPES * MAX_TYPES];
    __shared__ float sh_pair_scr[MAX_TYPES * MAX_TYPES];
    __shared__ ReactionDev sh_rx[MAX_REACTIONS];
    __shared__ float sh_drift[MAX_TYPES], sh_scale[MAX_TYPES];
    SmemLayout S = carve(smem, E.max_events_sm);
    S.drift = sh_drift;
    S.scale = sh_scale;
    S.screen = sh_pair_scr;
    RxnTables rt{};
    const int n_work = *E.n_work;
    if (threadIdx.x == 0) sh_table = -1;
    __syncthreads();
    for (;;) {
        if (threadIdx.x == 0) sh_r = atomicAdd(E.work, 1);
        __syncthreads();
        const int w = sh_r;
        if (w >= n_work) break;
        const int r = E.order[w];
        if (threadIdx.x == 0) {
            D = E.desc[r];
            st = E.state[r];
            sh_nev = 0;
            sh_status = 0;
        }
        __syncthreads();
        // a replica that has run its steps, or whose state is in error, idles
        if (st.step >= D.n_steps || st.status != 0) continue;
        const Tables *tab = E.tabs + D.table;
        if (D.table != sh_table) {
            rt = stage_tables(tab, S, sh_rt_ints, sh_rt_scr, sh_rx);
            __syncthreads();
            if (threadIdx.x == 0) sh_table = D.table;
        }
        __syncthreads();
        if constexpr (!MULTI) {
            if (D.smem_cells) replica_body(E, r, S, rt, tab, D, st, sh_nev, sh_status, S.cells);
            else replica_body(E, r, S, rt, tab, D, st, sh_nev, sh_status, D.start);
        } else {
            const int m = max(1, E.launch_steps[r]);
            for (int k = 0;;) {
                if (D.smem_cells) replica_body(E, r, S, rt, tab, D, st, sh_nev, sh_status, S.cells);
                else replica_body(E, r, S, rt, tab, D, st, sh_nev, sh_status, D.start);
                if (++k >= m) break;
                // the replica's next step: its state as the body stored it (the body ended at a barrier)
                if (threadIdx.x == 0) {
                    st = E.state[r];
                    sh_nev = 0;
                    sh_status = 0;
                }
                __syncthreads();
                if (st.step >= D.n_steps || st.status != 0) break;
            }
        }
    }
}

__global__ void k_engine_reset(EngineDev E) { *E.work = 0; }

// ids 0..n-1 (fill_ids), binning and sort of each listed replica (state.cur selects the source; the cell starts
// are sorted in the replica's global start array), and its t = 0 count record
__global__ void k_engine_admit(EngineDev E, const int *list, int count, int fill_ids) {
    for (int w = blockIdx.x; w < count; w += gridDim.x) {
        const int r = list[w];
        const RepDesc D = E.desc[r];
        RepState st = E.state[r];
        float4 *posX = D.pos[st.cur];
        uint32_t *idX = D.id[st.cur];
        if (fill_ids) {
            for (int i = threadIdx.x; i < st.n; i += blockDim.x) idX[i] = (uint32_t)i;
            __syncthreads();
        }
        block_bin(posX, st.n, D.bin, D.geo);
        block_rank(st.n, D.bin, D.rank, D.start, D.geo.ncells + 2);
        int n2, nin2;
        block_sort(posX, idX, st.n, D.pos[st.cur ^ 1], D.id[st.cur ^ 1], D.bin, D.rank, D.src, D.start, D.geo, n2,
                   nin2);
        st.n = n2;
        st.n_in = nin2;
        st.cur ^= 1;
        st.fvalid = 0;
        if (D.smem_cells) narrow_starts_inplace(D.start, D.geo.ncells + 3);
        if (D.records && D.count_stride > 0 && st.rec == 0 && D.max_records > 0) {
            block_count_types(D.pos[st.cur], st.n, E.tabs[D.table].ntypes, D.records);
            st.rec = 1;
        }
        if (threadIdx.x == 0) E.state[r] = st;
        __syncthreads();
    }
}

// current per-type counts of replicas [0, R) as count record `rec` of each (its records array and pitch)
__global__ void k_engine_record_now(EngineDev E, int R, int T, int rec) {
    for (int r = blockIdx.x; r < R; r += gridDim.x) {
        const RepDesc &D = E.desc[r];
        const RepState st = E.state[r];
        if (!D.records) continue;
        const size_t pitch = D.record_pitch ? (size_t)D.record_pitch : (size_t)T;
        block_count_types(D.pos[st.cur], st.n, T, D.records + (size_t)rec * pitch);
    }
}

// One frame of the Trajectory observable (FlatTrajectory records, readdy/main/model/observables/
// Trajectory.cpp:100-160) for the selected replicas sel[0, n_sel): the live particles of replica sel[k]
// (removed ones skipped, storage order kept) into slot k, positions with their type bits at
// out_pos + slot_off[k], ids at out_id + slot_off[k], their number in out_n[k].  One CTA per selected
// replica compacts by block scans.
__global__ void k_engine_snapshot(EngineDev E, const int *sel, int n_sel, const int64_t *slot_off, float4 *out_pos,
                                  uint32_t *out_id, int *out_n) {
    for (int k = blockIdx.x; k < n_sel; k += gridDim.x) {
        const RepDesc &D = E.desc[sel[k]];
        const RepState st = E.state[sel[k]];
        const float4 *pos = D.pos[st.cur];
        const uint32_t *id = D.id[st.cur];
        float4 *op = out_pos + slot_off[k];
        uint32_t *oi = out_id + slot_off[k];
        int base = 0;
        for (int c = 0; c < st.n; c += blockDim.x) {
            const int i = c + threadIdx.x;
            float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
            int live = 0;
            if (i < st.n) {
                p = pos[i];
                live = itype(p) >= 0;
            }
            int total = 0;
            const int at = block_exclusive_scan(live, total);
            if (live) {
                op[base + at] = p;
                oi[base + at] = id[i];
            }
            base += total;
        }
        if (threadIdx.x == 0) out_n[k] = base;
        __syncthreads();
    }
}

__global__ void k_engine_count(EngineDev E, int R, int T, unsigned long long *out) {
    for (int r = blockIdx.x; r < R; r += gridDim.x) {
        const RepDesc &D = E.desc[r];
        const RepState st = E.state[r];
        block_count_types(D.pos[st.cur], st.n, T, out + (size_t)r * T);
    }
}

// The force the next Euler update of replica r applies to each particle of its current state, in
// storage order (fx, fy, fz, 0): the pair forces it carries from its last event walk where it carries
// them, otherwise a pair walk over its sorted state (16-bit or int starts, as the replica keeps them
// between steps), plus the order-1 potentials.  Removed particles get zero.
template <typename C>
__device__ inline void engine_forces_of(const RepDesc &D, const RepState &st, const Tables *tab, const C *start,
                                        float4 *out) {
    const GeoR g = geo_r(D.geo);
    const float4 *pos = D.pos[st.cur];
    const float4 *carried = (st.fvalid && D.force[st.cur]) ? D.force[st.cur] : nullptr;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < st.n; i += gridDim.x * blockDim.x) {
        const float4 p = pos[i];
        const int t = itype(p);
        float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
        if (t >= 0) {
            if (carried) {
                const float4 f = carried[i];
                fx = f.x; fy = f.y; fz = f.z;
            } else if (i < st.n_in && tab->npots > 0) {
                pair_force_at(i, p, pos, start, g, 1, tab->pair_tab, tab->pair_screen, tab->pots, tab->ntypes, fx, fy,
                              fz, e);
            }
            const int o1 = tab->o1pot_tab[t];
            if (o1) order1_force(p, tab->o1pots, o1 >> 8, o1 & 0xff, fx, fy, fz, e);
        }
        out[i] = make_float4(fx, fy, fz, 0.f);
    }
}

// The pair virial of every listed replica's current state (Context::recordVirial; the sum over pairs of
// outer(-x_ij, f_i) that calculateOrder2<true> accumulates, CPUCalculateForces.cpp:247-249, seen here once
// from each side with half the weight), one block per replica, FP32 per thread and FP64 per block, into
// out (9 doubles per replica, row-major).  The state must be sorted (forces not carried), so that its
// cell starts are valid; a replica that carries its forces gets NaN.
template <typename C>
__device__ inline void engine_virial_of(const RepDesc &D, const RepState &st, const Tables *tab, const C *start,
                                        double *out) {
    const GeoR g = geo_r(D.geo);
    const float4 *pos = D.pos[st.cur];
    float vir[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < st.n_in; i += blockDim.x) {
        const float4 p = pos[i];
        if (itype(p) < 0 || tab->npots == 0) continue;
        float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
        pair_force_at(i, p, pos, start, g, 1, tab->pair_tab, tab->pair_screen, tab->pots, tab->ntypes, fx, fy, fz, e,
                      vir);
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            acc[k] += (double)vir[k];
            vir[k] = 0.f;
        }
    }
    for (int k = 0; k < 9; ++k) {
        const double v = block_sum_double(acc[k]);
        if (threadIdx.x == 0) out[k] = v;
    }
}

__global__ void k_engine_virial(EngineDev E, int R, double *out) {
    for (int r = blockIdx.x; r < R; r += gridDim.x) {
        const RepDesc D = E.desc[r];
        const RepState st = E.state[r];
        if (st.fvalid) {
            if (threadIdx.x < 9) out[(size_t)r * 9 + threadIdx.x] = __longlong_as_double(0x7ff8000000000000LL);
            __syncthreads();
            continue;
        }
        const Tables *tab = E.tabs + D.table;
        if (D.smem_cells) engine_virial_of(D, st, tab, reinterpret_cast<const uint16_t *>(D.start), out + (size_t)r * 9);
        else engine_virial_of(D, st, tab, D.start, out + (size_t)r * 9);
        __syncthreads();
    }
}

__global__ void k_engine_forces(EngineDev E, int r, float4 *out) {
    const RepDesc D = E.desc[r];
    const RepState st = E.state[r];
    const Tables *tab = E.tabs + D.table;
    if (D.smem_cells) engine_forces_of(D, st, tab, reinterpret_cast<const uint16_t *>(D.start), out);
    else engine_forces_of(D, st, tab, D.start, out);
}

// ---- host side ----------------------------------------------------------------------------------

Geo replica_geo(const double box[3], const int pbc[3], double cutoff, double cell_scale, int64_t capacity,
                int &smem_cells) {
    double w = cutoff * cell_scale;
    Geo g = make_geo(box, pbc, cutoff, 1, w);
    const bool small = capacity < 65536;  // cell starts fit 16 bits
    if (small)
        for (int k = 0; k < 64 && g.ncells + 3 > SMEM_CELLS && cutoff > 0; ++k) {
            w *= 1.05;
            g = make_geo(box, pbc, cutoff, 1, w);
        }
    smem_cells = (small && g.ncells + 3 <= SMEM_CELLS) ? 1 : 0;
    if (!smem_cells) g = make_geo(box, pbc, cutoff, 1, cutoff * cell_scale);
    return g;
}

int sm_count() {
    int dev = 0, sms = 0;
    RDC_CUDA(cudaGetDevice(&dev));
    RDC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    return std::max(1, sms);
}

int engine_grid(int threads, size_t smem) {
    RDC_CUDA(cudaFuncSetAttribute(k_engine_step<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    RDC_CUDA(cudaFuncSetAttribute(k_engine_step<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int dev = 0, sms = 0, smem_sm = 0;
    RDC_CUDA(cudaGetDevice(&dev));
    RDC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    RDC_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    // Ask for just the shared memory one CTA needs: the rest of the SM's unified L1/shared array stays
    // L1, which caches the neighbour positions of the candidate walks (a 100 % carveout leaves 28 KB).
    cudaFuncAttributes fa{};
    RDC_CUDA(cudaFuncGetAttributes(&fa, k_engine_step<false>));
    const size_t need = smem + fa.sharedSizeBytes + 1024;  // + the per-CTA reservation
    const int carveout = (int)std::min<size_t>(100, (need * 100 + smem_sm - 1) / std::max(smem_sm, 1));
    RDC_CUDA(cudaFuncSetAttribute(k_engine_step<false>, cudaFuncAttributePreferredSharedMemoryCarveout, carveout));
    RDC_CUDA(cudaFuncSetAttribute(k_engine_step<true>, cudaFuncAttributePreferredSharedMemoryCarveout, carveout));
    int per_sm = 0;
    RDC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_engine_step<false>, threads, smem));
    return std::max(1, per_sm) * sms;
}

void launch_engine_step(const EngineDev &E, int blocks, int threads, size_t smem, cudaStream_t st) {
    if (E.launch_steps) k_engine_step<true><<<blocks, threads, smem, st>>>(E);
    else k_engine_step<false><<<blocks, threads, smem, st>>>(E);
    k_engine_reset<<<1, 1, 0, st>>>(E);
}

void launch_engine_admit(const EngineDev &E, const int *list, int count, bool fill_ids, cudaStream_t st) {
    if (count > 0) k_engine_admit<<<std::min(count, 4 * sm_count()), 256, 0, st>>>(E, list, count, fill_ids ? 1 : 0);
}

void launch_engine_count(const EngineDev &E, int R, int ntypes, unsigned long long *out, cudaStream_t st) {
    if (R > 0) k_engine_count<<<std::min(R, 4 * sm_count()), 256, 0, st>>>(E, R, ntypes, out);
}

void launch_engine_record_now(const EngineDev &E, int R, int ntypes, int rec, cudaStream_t st) {
    if (R > 0) k_engine_record_now<<<std::min(R, 4 * sm_count()), 256, 0, st>>>(E, R, ntypes, rec);
}

void launch_engine_snapshot(const EngineDev &E, const int *sel, int n_sel, const int64_t *slot_off, float4 *out_pos,
                            uint32_t *out_id, int *out_n, cudaStream_t st) {
    if (n_sel > 0)
        k_engine_snapshot<<<std::min(n_sel, 4 * sm_count()), 256, 0, st>>>(E, sel, n_sel, slot_off, out_pos, out_id,
                                                                           out_n);
}

void launch_engine_virial(const EngineDev &E, int R, double *out, cudaStream_t st) {
    if (R > 0) k_engine_virial<<<std::min(R, 4 * sm_count()), 256, 0, st>>>(E, R, out);
}

void launch_engine_forces(const EngineDev &E, int r, int n, float4 *out, cudaStream_t st) {
    if (n > 0) k_engine_forces<<<std::min((n + 255) / 256, 4 * sm_count()), 256, 0, st>>>(E, r, out);
}

}  // namespace rdc

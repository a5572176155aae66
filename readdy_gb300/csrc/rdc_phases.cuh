// Per-particle and per-block phases shared by the grid-wide per-system kernels and the fused
// batched-replica kernel.  Both paths call the same functions, so one replica advanced alone or
// inside a batch performs the same arithmetic in the same order.
#pragma once
#include <climits>
#include <cstdint>
#include <type_traits>

#include "rdc_device.cuh"
#include "rdc_host.h"

namespace rdc {

// cells along one axis of the (2r+1)-stencil around c, each cell once
__device__ inline int axis_cells(int c, int dim, int pbc, int r, int *out) {
    int n = 0;
    if (pbc && dim <= 2 * r + 1) {
        for (int v = 0; v < dim; ++v) out[n++] = v;
        return n;
    }
    for (int o = -r; o <= r; ++o) {
        int v = c + o;
        if (pbc) v = (v + dim) % dim;
        else if (v < 0 || v >= dim) continue;
        out[n++] = v;
    }
    return n;
}

// cells up to this many entries are ordered by one thread (insertion sort)
constexpr int CELL_SORT_SMALL = 32;

// orders the source indices a[b..e) by their particles' ids key[a[.]] (distinct within a system), so
// that a cell's storage order does not depend on the order of the source arrays.  A pair -- nearly
// every cell to order at the densities of the workloads -- loads both keys at once.
__device__ inline void insertion_sort_by(int *a, int b, int e, const uint32_t *__restrict__ key) {
    if (e - b == 2) {
        const int v0 = a[b], v1 = a[b + 1];
        if (key[v0] > key[v1]) {
            a[b] = v1;
            a[b + 1] = v0;
        }
        return;
    }
    for (int j = b + 1; j < e; ++j) {
        const int v = a[j];
        const uint32_t kv = key[v];
        int k = j - 1;
        while (k >= b && key[a[k]] > kv) {
            a[k + 1] = a[k];
            --k;
        }
        a[k + 1] = v;
    }
}

// insertion_sort_by for crowded cells, by the whole block: each index's rank is the count of smaller
// keys; tmp[b..e) is scratch
__device__ inline void block_rank_sort_by(int *a, int *tmp, int b, int e, const uint32_t *__restrict__ key) {
    const int k = e - b;
    for (int t = threadIdx.x; t < k; t += blockDim.x) {
        const int v = a[b + t];
        const uint32_t kv = key[v];
        int r = 0;
        for (int u = 0; u < k; ++u) r += key[a[b + u]] < kv;
        tmp[b + r] = v;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < k; t += blockDim.x) a[b + t] = tmp[b + t];
    __syncthreads();
}

// Calls f(jb, je) for the storage ranges of every cell of the (2r+1)^3 stencil around the particle's
// cell, cells in x-major, z-fastest order.  start[] holds the cell starts as int or, for systems of
// fewer than 65536 particles, as uint16_t.  For r = 1 on grids of at least 3 cells along each periodic
// axis the three z-cells of a column are contiguous in storage and are visited as one range (two if
// the column wraps); other grids take the general per-cell path.
template <typename G>
__device__ inline bool stencil_fast(const G &g, int radius) {
    return radius == 1 && (!g.pbc[0] || g.dims[0] >= 3) && (!g.pbc[1] || g.dims[1] >= 3) &&
           (!g.pbc[2] || g.dims[2] >= 3);
}

template <typename G, typename S, typename F>
__device__ inline void for_each_neighbor_range(float4 p, const G &g, const S *__restrict__ start, int radius,
                                               F f, bool skip_lower_columns = false, float reach2 = INFINITY) {
    int cx, cy, cz;
    cell_coords(p, g, cx, cy, cz);
    const int dx0 = g.dims[0], dy0 = g.dims[1], dz0 = g.dims[2];
    if (stencil_fast(g, radius)) {
        // a column stored wholly before the particle's own column holds only smaller storage indices;
        // walks that want partners j > i (skip_lower_columns) need not read its starts
        const int own_base = (cx * dy0 + cy) * dz0;
        // Lower bounds of the distance from p to the cell below (lo) and above (hi) along each axis: its
        // offset inside its own cell, less a margin that covers the rounding of the offset.  A column or an
        // end cell farther than sqrt(reach2) holds no candidate that can pass the caller's screen, so it is
        // skipped; the candidates that remain keep their order.
        float lo[3], hi[3];
        {
            const float pc[3] = {p.x, p.y, p.z};
            const int cc[3] = {cx, cy, cz};
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                float w, m;
                cell_width_margin(g, d, w, m);
                const float u = (pc[d] + g.hL[d]) - (float)cc[d] * w;
                lo[d] = fmaxf(u - m, 0.f);
                hi[d] = fmaxf(w - u - m, 0.f);
            }
        }
#pragma unroll 1
        for (int ox = -1; ox <= 1; ++ox) {
            const float dx2 = ox < 0 ? lo[0] * lo[0] : (ox > 0 ? hi[0] * hi[0] : 0.f);
            if (dx2 > reach2) continue;
            int x = cx + ox;
            if (x < 0) {
                if (!g.pbc[0]) continue;
                x += dx0;
            } else if (x >= dx0) {
                if (!g.pbc[0]) continue;
                x -= dx0;
            }
#pragma unroll 1
            for (int oy = -1; oy <= 1; ++oy) {
                const float dxy2 = dx2 + (oy < 0 ? lo[1] * lo[1] : (oy > 0 ? hi[1] * hi[1] : 0.f));
                if (dxy2 > reach2) continue;
                int y = cy + oy;
                if (y < 0) {
                    if (!g.pbc[1]) continue;
                    y += dy0;
                } else if (y >= dy0) {
                    if (!g.pbc[1]) continue;
                    y -= dy0;
                }
                const int base = (x * dy0 + y) * dz0;
                if (skip_lower_columns && base < own_base) continue;
                int z0 = dxy2 + lo[2] * lo[2] > reach2 ? cz : cz - 1;
                int z1 = dxy2 + hi[2] * hi[2] > reach2 ? cz : cz + 1;
                if (z0 < 0) {
                    if (g.pbc[2]) f(start[base + dz0 - 1], start[base + dz0]);
                    z0 = 0;
                }
                bool wrap_hi = false;
                if (z1 >= dz0) {
                    wrap_hi = g.pbc[2] != 0;
                    z1 = dz0 - 1;
                }
                f(start[base + z0], start[base + z1 + 1]);
                if (wrap_hi) f(start[base], start[base + 1]);
            }
        }
        return;
    }
    int ax[7], ay[7], az[7];
    const int nx = axis_cells(cx, dx0, g.pbc[0], radius, ax);
    const int ny = axis_cells(cy, dy0, g.pbc[1], radius, ay);
    const int nz = axis_cells(cz, dz0, g.pbc[2], radius, az);
    for (int a = 0; a < nx; ++a)
        for (int b = 0; b < ny; ++b)
            for (int c = 0; c < nz; ++c) {
                const int cell = az[c] + dz0 * (ay[b] + dy0 * ax[a]);
                f(start[cell], start[cell + 1]);
            }
}

// Calls f(cell) for every cell of the radius-1 stencil around the particle's cell, in the order in
// which for_each_neighbor_range visits their storage ranges.
template <typename G, typename F>
__device__ inline void for_each_neighbor_cell(float4 p, const G &g, F f) {
    int cx, cy, cz;
    cell_coords(p, g, cx, cy, cz);
    const int dx0 = g.dims[0], dy0 = g.dims[1], dz0 = g.dims[2];
    if (stencil_fast(g, 1)) {
        // loops kept rolled: f is inlined once, not once per stencil cell
#pragma unroll 1
        for (int ox = -1; ox <= 1; ++ox) {
            int x = cx + ox;
            if (x < 0) {
                if (!g.pbc[0]) continue;
                x += dx0;
            } else if (x >= dx0) {
                if (!g.pbc[0]) continue;
                x -= dx0;
            }
#pragma unroll 1
            for (int oy = -1; oy <= 1; ++oy) {
                int y = cy + oy;
                if (y < 0) {
                    if (!g.pbc[1]) continue;
                    y += dy0;
                } else if (y >= dy0) {
                    if (!g.pbc[1]) continue;
                    y -= dy0;
                }
                const int base = (x * dy0 + y) * dz0;
                int z0 = cz - 1, z1 = cz + 1;
                if (z0 < 0) z0 = 0;
                bool wrap_hi = false;
                if (z1 >= dz0) {
                    wrap_hi = g.pbc[2] != 0;
                    z1 = dz0 - 1;
                }
                // the column's cells in storage order: the wrapped low cell, z0..z1, the wrapped high cell
                const int zs = (cz - 1 < 0 && g.pbc[2]) ? -1 : z0;
                const int ze = wrap_hi ? z1 + 1 : z1;
#pragma unroll 1
                for (int z = zs; z <= ze; ++z) f(base + (z < 0 ? dz0 - 1 : (z > z1 ? 0 : z)));
            }
        }
        return;
    }
    int ax[7], ay[7], az[7];
    const int nx = axis_cells(cx, dx0, g.pbc[0], 1, ax);
    const int ny = axis_cells(cy, dy0, g.pbc[1], 1, ay);
    const int nz = axis_cells(cz, dz0, g.pbc[2], 1, az);
#pragma unroll 1
    for (int a = 0; a < nx; ++a)
#pragma unroll 1
        for (int b = 0; b < ny; ++b)
#pragma unroll 1
            for (int c = 0; c < nz; ++c) f(az[c] + dz0 * (ay[b] + dy0 * ax[a]));
}

// Calls f(j) for every candidate j >= jmin of the stencil, in the order of for_each_neighbor_range.
// The non-empty ranges are gathered first and then walked as one flat sequence, so the lanes of a
// warp run the candidate body together until each has exhausted its own candidates (short per-cell
// loops would cost every range the longest lane's length).  Measured on the batched ensemble this is
// faster than producing the ranges column by column inside the walk, although the range list lives
// in local memory.
constexpr int MAX_RANGES = 18;

template <typename G, typename S, typename F>
__device__ inline void for_each_candidate(float4 p, const G &g, const S *__restrict__ start, int radius, int jmin,
                                          F f) {
    if (!stencil_fast(g, radius)) {
        for_each_neighbor_range(p, g, start, radius, [&](int jb, int je) {
            for (int j = max(jb, jmin); j < je; ++j) f(j);
        });
        return;
    }
    int rb[MAX_RANGES], re[MAX_RANGES];
    int nr = 0;
    for_each_neighbor_range(p, g, start, radius, [&](int jb, int je) {
        jb = max(jb, jmin);
        if (jb < je) {
            rb[nr] = jb;
            re[nr] = je;
            ++nr;
        }
    });
    int r = 0;
    int j = nr > 0 ? rb[0] : 0, je = nr > 0 ? re[0] : 0;
    while (r < nr) {
        f(j);
        if (++j == je && ++r < nr) {
            j = rb[r];
            je = re[r];
        }
    }
}

// for_each_candidate that also hands f the candidate's position: f(j, pos[j]).  On the fast stencil the
// position of the next candidate is loaded before f runs on the current one, so each thread keeps a
// load in flight while it screens; the walk is latency bound on these loads.
template <typename G, typename S, typename F>
__device__ inline void for_each_candidate_q(float4 p, const G &g, const S *__restrict__ start,
                                            const float4 *__restrict__ pos, int radius, int jmin, F f,
                                            float reach2 = INFINITY) {
    if (!stencil_fast(g, radius)) {
        for_each_neighbor_range(p, g, start, radius, [&](int jb, int je) {
            for (int j = max(jb, jmin); j < je; ++j) f(j, pos[j]);
        });
        return;
    }
    int rb[MAX_RANGES], re[MAX_RANGES];
    int nr = 0;
    for_each_neighbor_range(p, g, start, radius, [&](int jb, int je) {
        jb = max(jb, jmin);
        if (jb < je) {
            rb[nr] = jb;
            re[nr] = je;
            ++nr;
        }
    }, jmin > 0, reach2);
    if (nr == 0) return;
    int r = 0, j = rb[0], je = re[0];
    float4 q = pos[j];
    for (;;) {
        int jn = j + 1, rn = r, jen = je;
        bool more = true;
        if (jn == jen) {
            if (++rn < nr) {
                jn = rb[rn];
                jen = re[rn];
            } else {
                more = false;
            }
        }
        float4 qn = q;
        if (more) qn = pos[jn];
        f(j, q);
        if (!more) break;
        j = jn;
        r = rn;
        je = jen;
        q = qn;
    }
}

// exclusive scan of one value per thread across the block; total receives the block sum
__device__ inline int block_exclusive_scan(int v, int &total) {
    __shared__ int warp_sums[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    const int before = (wid > 0 ? warp_sums[wid - 1] : 0) + x - v;
    total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before;
}

__device__ inline double block_sum_double(double v) {
    __shared__ double red[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double r = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += red[w];
    __syncthreads();
    return r;
}

// Pair force and half pair energy on particle i (storage index inside the cells) from every
// neighbour of the stencil; the full both-direction iteration of CPUCalculateForces.cpp:214-268.
// The walk only screens candidates (cheap FP32 distance test) and keeps up to PAIR_BUFFER survivors in
// registers; their forces are evaluated afterwards, with the lanes of a warp evaluating their k-th
// survivors together.  Evaluated inside the walk, the force body ran for the one lane in six or so
// that had met a neighbour.  Survivors keep the walk order, so the summation order is unchanged.
constexpr int PAIR_BUFFER = 4;

// With vir non-null, vir[3a+b] also receives half of -x_ij[a] f_i[b] per pair: the virial
// sum over pairs of outer(-x_ij, f_i) of calculateOrder2<true> (CPUCalculateForces.cpp:247-249), seen
// here once from each side.
// With an `extra` callable, extra(j, q, tj, d2) also sees the live candidates j != i of the walk with
// their FP32 screening distance, before the force filters: the replica engine finds its reaction
// pairs in the same walk.  The force arithmetic and its order do not depend on it.  reach2 bounds the
// cells walked (default, reach2 < 0: the largest pair-potential screen of i's type); a caller with an
// `extra` passes the largest screen that either needs, and in tmask (bit t: type t) the candidate types
// that either takes; candidates of other types or beyond reach2 are not handed on.  (Measured: the two
// register tests speed up the engine's fused walk 3 % and slow the force-only walk 2 %, so the
// force-only walk keeps its table tests.)
struct NoExtra {
    __device__ void operator()(int, float4, int, float) const {}
};

// the pair potentials of one surviving candidate q (pt: its entry of the type-pair table) on p
template <typename G>
__device__ inline void pair_force_body(float4 p, float4 q, const G &g, int pt, const PairPot *pots, float &fx,
                                       float &fy, float &fz, float &e) {
    const PairGeom g0 = pair_geom(p, q, g);
    const int first = pt >> 8, cnt = pt & 0xff;
    for (int k = first; k < first + cnt; ++k) {
        const PairPot &pp = pots[k];
        PairGeom gg = g0;
        if (within(g0, gg, p, q, g, pp.cutoff2f, pp.band, pp.cutoff2)) pair_force(pp, gg, p, q, g, fx, fy, fz, e);
    }
}

template <typename G, typename S, typename Extra = NoExtra>
__device__ inline void pair_force_at(int i, float4 p, const float4 *__restrict__ pos, const S *__restrict__ start,
                                     const G &g, int radius, const int *tab, const float *screen, const PairPot *pots,
                                     int T, float &fx, float &fy, float &fz, float &e, float *vir = nullptr,
                                     Extra extra = Extra(), float reach2 = -1.f, uint32_t tmask = 0u) {
    constexpr bool has_extra = !std::is_same<Extra, NoExtra>::value;
    const int ti = itype(p);
    const int *trow = tab + ti * T;
    const float *srow = screen + ti * T;
    if (reach2 < 0.f) {  // the largest screen of the type's pair potentials: cells beyond it are not walked
        reach2 = 0.f;
        tmask = 0u;
        for (int t = 0; t < T; ++t)
            if (trow[t]) {
                reach2 = fmaxf(reach2, srow[t]);
                tmask |= 1u << t;
            }
    }
    auto body = [&](int j) {
        const float4 q = pos[j];
        const int pt = trow[itype(q)];
        if (!vir) {
            pair_force_body(p, q, g, pt, pots, fx, fy, fz, e);
            return;
        }
        const PairGeom g0 = pair_geom(p, q, g);
        const int first = pt >> 8, cnt = pt & 0xff;
        for (int k = first; k < first + cnt; ++k) {
            const PairPot &pp = pots[k];
            PairGeom gg = g0;
            if (within(g0, gg, p, q, g, pp.cutoff2f, pp.band, pp.cutoff2)) {
                float tx = 0.f, ty = 0.f, tz = 0.f;
                pair_force(pp, gg, p, q, g, tx, ty, tz, e);
                fx += tx; fy += ty; fz += tz;
                const float d[3] = {-0.5f * gg.dx, -0.5f * gg.dy, -0.5f * gg.dz}, f[3] = {tx, ty, tz};
#pragma unroll
                for (int a = 0; a < 3; ++a)
#pragma unroll
                    for (int b = 0; b < 3; ++b) vir[3 * a + b] += d[a] * f[b];
            }
        }
    };
    int b0 = 0, b1 = 0, b2 = 0, b3 = 0, nb = 0;
    for_each_candidate_q(p, g, start, pos, radius, 0, [&](int j, float4 q) {
        if (j == i) return;
        const int tj = itype(q);
        if constexpr (has_extra) {
            // register tests first: a type neither filter takes, a candidate beyond every screen of i's type
            if ((unsigned)tj >= 32u || !((tmask >> tj) & 1u)) return;
            const float d2s = screen_d2(p, q, g);
            if (d2s > reach2) return;
            extra(j, q, tj, d2s);
            if (trow[tj] == 0 || d2s > srow[tj]) return;
        } else {
            if (tj < 0) return;
            if (trow[tj] == 0) return;
            if (screen_d2(p, q, g) > srow[tj]) return;
        }
        if (nb == PAIR_BUFFER) {  // full: evaluate the oldest survivor now and shift
            body(b0);
            b0 = b1; b1 = b2; b2 = b3;
            --nb;
        }
        if (nb == 0) b0 = j;
        else if (nb == 1) b1 = j;
        else if (nb == 2) b2 = j;
        else b3 = j;
        ++nb;
    }, reach2);
    for (int k = 0; k < nb; ++k) {
        body(b0);
        b0 = b1; b1 = b2; b2 = b3;
    }
}

// Euler-Maruyama update of one particle (CPUEulerBDIntegrator.cpp:66-73), FP32, Philox noise
// keyed by (seed, particle id, integrator step)
template <typename G>
__device__ inline float4 euler_bd(float4 p, float fx, float fy, float fz, uint32_t id, uint64_t seed, uint64_t step,
                                  float drift, float sc, const G &g) {
    float n0, n1, n2, n3;
    normal4(rng_draw(seed, id, 0u, step, RNG_BD, 0u), n0, n1, n2, n3);
    p.x = wrap1(p.x + (sc * n0 + fx * drift), g.L[0], g.hL[0], g.pbc[0]);
    p.y = wrap1(p.y + (sc * n1 + fy * drift), g.L[1], g.hL[1], g.pbc[1]);
    p.z = wrap1(p.z + (sc * n2 + fz * drift), g.L[2], g.hL[2], g.pbc[2]);
    return p;
}

// ------------------------------------------------------------------------------------------------
// reaction events that pass the acceptance coin u < 1 - exp(-k dt) (ReactionUtils.h:64-71)
// ------------------------------------------------------------------------------------------------
__device__ inline uint64_t coin_bits(U4 r) { return ((uint64_t)r.x << 32) | r.y; }

// Priority of an accepted event (smaller resolves first).  Uncontrolled approximation: a uniformly
// random order (the shuffle of CPUUncontrolledApproximation.cpp:198).  Gillespie: the exponential
// clock E / k with E ~ Exp(1), whose order is proportional-to-rate selection without replacement
// (algorithm.h:80-88).  The clock is an FP32 value in the high word (positive floats order like their
// bits) and a random word breaks ties; everything stays off the FP64 pipe.
__device__ inline uint64_t priority_key(U4 r, const ReactionDev &R, int handler) {
    if (handler == H_GILLESPIE) {
        const float clock = -logf(u01(r.z)) * R.inv_rate;
        return ((uint64_t)__float_as_uint(clock) << 32) | r.w;
    }
    return ((uint64_t)r.z << 32) | r.w;
}

// the reaction lookup tables of Tables, staged in shared memory by the kernels that generate events
struct RxnTables {
    const int *o1_tab, *o1_list, *o2_tab, *o2_list, *o2_any;
    const float *screen;
    const ReactionDev *rx;
    int T;
};

// all threads of the block copy the reaction tables into smem (ints, T*T screening floats, reactions)
__device__ inline RxnTables stage_rxn_tables(const Tables *tab, int *smem_ints, float *smem_screen,
                                             ReactionDev *smem_rx) {
    const int T = tab->ntypes, NR = tab->nreactions;
    int *o1t = smem_ints, *o1l = o1t + T, *o2t = o1l + NR, *o2l = o2t + T * T, *o2a = o2l + 2 * NR;
    for (int k = threadIdx.x; k < T; k += blockDim.x) { o1t[k] = tab->o1_tab[k]; o2a[k] = tab->o2_any[k]; }
    for (int k = threadIdx.x; k < NR; k += blockDim.x) { o1l[k] = tab->o1_list[k]; smem_rx[k] = tab->reactions[k]; }
    for (int k = threadIdx.x; k < 2 * NR; k += blockDim.x) o2l[k] = tab->o2_list[k];
    for (int k = threadIdx.x; k < T * T; k += blockDim.x) {
        o2t[k] = tab->o2_tab[k];
        smem_screen[k] = tab->rx_screen[k];
    }
    return RxnTables{o1t, o1l, o2t, o2l, o2a, smem_screen, smem_rx, T};
}

// Event generation in two passes.  The candidate pass walks the stencil and pushes every educt
// tuple that can react -- (i, i, r) for the order-1 reactions of particle i and (i, j, r) for the
// pairs (i, j > i) inside the educt distance -- into a per-block queue.  The coin pass then draws the
// acceptance coin of each queued tuple with all lanes converged: drawn inside the walk, the Philox
// rounds ran for the one or two lanes of a warp that had met a pair.  The coins are keyed by ids,
// step and reaction, so the accepted events do not depend on the queue order.

// order-1 tuples of particle i and order-2 tuples of the pairs (i, j > i); push(p1, p2, r)
template <typename G, typename S, typename Push>
__device__ inline void event_tuples_at(int i, bool in_cells, const float4 *__restrict__ pos,
                                       const S *__restrict__ start, const G &g, int radius, const RxnTables &rt,
                                       Push push) {
    const float4 p = pos[i];
    const int ti = itype(p);
    if (ti < 0) return;
    const int o1 = rt.o1_tab[ti];
    for (int k = (o1 >> 8); k < (o1 >> 8) + (o1 & 0xff); ++k) {
        const int r = rt.o1_list[k];
        if (rt.rx[r].active) push(i, i, r);
    }
    if (!in_cells || !rt.o2_any[ti]) return;
    const int *trow = rt.o2_tab + ti * rt.T;
    const float *srow = rt.screen + ti * rt.T;
    for_each_candidate_q(p, g, start, pos, radius, i + 1, [&](int j, float4 q) {
        const int tj = itype(q);
        if (tj < 0) return;
        const int o2 = trow[tj];
        if (o2 == 0) return;
        if (screen_d2(p, q, g) > srow[tj]) return;  // cheap FP32 reject before the exact geometry
        const PairGeom g0 = pair_geom(p, q, g);
        for (int k = (o2 >> 8); k < (o2 >> 8) + (o2 & 0xff); ++k) {
            const int r = rt.o2_list[k];
            const ReactionDev &R = rt.rx[r];
            if (!R.active) continue;
            PairGeom gg = g0;
            if (within(g0, gg, p, q, g, R.educt_distance2f, R.band, R.educt_distance2)) push(i, j, r);
        }
    });
}

// the acceptance coin u < 1 - exp(-k dt) of one tuple (ReactionUtils.h:64-71); emit(key, p1, p2, r)
// with p1 the particle of smaller id
template <typename Emit>
__device__ inline void event_coin(int p1, int p2, int r, const uint32_t *__restrict__ id, const RxnTables &rt,
                                  uint64_t seed, uint64_t step, int handler, Emit emit) {
    const ReactionDev &R = rt.rx[r];
    if (p1 == p2) {
        const U4 u = rng_draw(seed, id[p1], 0u, step, RNG_COIN1, (uint32_t)r);
        if (coin_bits(u) < R.coin_threshold) emit(priority_key(u, R, handler), p1, p1, r);
        return;
    }
    const uint32_t a = id[p1], b = id[p2];
    const U4 u = rng_draw(seed, min(a, b), max(a, b), step, RNG_COIN2, (uint32_t)r);
    if (coin_bits(u) < R.coin_threshold) {
        if (a < b) emit(priority_key(u, R, handler), p1, p2, r);
        else emit(priority_key(u, R, handler), p2, p1, r);
    }
}

// per-block queue of educt tuples between the two passes, in shared memory
constexpr int EVENT_QUEUE = 2048;
struct TupleQueue {
    int *p1, *p2;
    unsigned char *r;
    int *count;
};

// Both passes over particles [0, n) by one block (all threads must call it), in rounds of blockDim.x
// particles: particle `first + k * stride` for k = 0, 1, ...  A full queue never loses a tuple: its
// coin is drawn on the spot.
template <typename G, typename S, typename Emit>
__device__ inline void block_events(int first, int stride, int n, int n_in, const float4 *__restrict__ pos,
                                    const uint32_t *__restrict__ id, const S *__restrict__ start, const G &g,
                                    int radius, const RxnTables &rt, uint64_t seed, uint64_t step, int handler,
                                    const TupleQueue &Q, Emit emit) {
    auto push = [&](int a, int b, int r) {
        const int k = atomicAdd(Q.count, 1);
        if (k < EVENT_QUEUE) {
            Q.p1[k] = a;
            Q.p2[k] = b;
            Q.r[k] = (unsigned char)r;
        } else {
            event_coin(a, b, r, id, rt, seed, step, handler, emit);
        }
    };
    if (threadIdx.x == 0) *Q.count = 0;
    __syncthreads();
    for (int base = first; base < n; base += stride) {
        const int i = base + (int)threadIdx.x;
        if (i < n) event_tuples_at(i, i < n_in, pos, start, g, radius, rt, push);
        __syncthreads();
        const int nq = min(*Q.count, EVENT_QUEUE);
        for (int k = threadIdx.x; k < nq; k += blockDim.x)
            event_coin(Q.p1[k], Q.p2[k], (int)Q.r[k], id, rt, seed, step, handler, emit);
        __syncthreads();
        if (threadIdx.x == 0) *Q.count = 0;
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------------------
// block-level conflict resolution and application of accepted events
// ------------------------------------------------------------------------------------------------
struct ApplyTarget {
    float4 *pos;
    uint32_t *id;
    int *tslot;    // may be null (replicas carry no topologies)
    float4 *force; // may be null
    int *claim, *taken;
    unsigned long long *reaction_counts;
    int n_total;   // storage size before the births
    int capacity;
    uint32_t next_id;
};

struct ApplyResult {
    int births, ids, status, winners;
};

__device__ inline F3 fission_direction(uint64_t seed, uint32_t id1, uint64_t step, int r) {
    float n0, n1, n2, n3;
    normal4(rng_draw(seed, id1, 0u, step, RNG_FISSION, (uint32_t)r), n0, n1, n2, n3);
    const float inv = rsqrtf(n0 * n0 + n1 * n1 + n2 * n2);
    return f3(n0 * inv, n1 * inv, n2 * inv);
}

// All threads of the block call this.  key/idx/state are shared-memory arrays of max_events
// entries.  An event wins iff no earlier winner (by priority) shares a particle: the greedy scan of
// CPUUncontrolledApproximation.cpp:206-253 and algorithm.h:62-136, computed in parallel rounds
// (each round the undecided events that are minimal among the undecided events of both their
// particles win, and the events touching a winner lose).
__device__ inline void block_resolve_apply(const EventRec *events, int E, int max_events, uint64_t *key, int *idx,
                                           int *state, const Tables *tab, const Geo &g, uint64_t seed,
                                           uint64_t step, ApplyTarget t, ApplyResult &res) {
    __shared__ int sh_any, sh_births, sh_ids, sh_status, sh_win;
    if (threadIdx.x == 0) sh_status = 0;
    if (E > max_events) {
        if (threadIdx.x == 0) sh_status |= ST_EVENTS;
        E = max_events;
    }
    int P = 1;
    while (P < E) P <<= 1;
    for (int k = threadIdx.x; k < P; k += blockDim.x) {
        key[k] = k < E ? events[k].key : ~0ull;
        idx[k] = k < E ? k : INT_MAX;
    }
    __syncthreads();
    for (int size = 2; size <= P; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int k = threadIdx.x; k < P; k += blockDim.x) {
                const int l = k ^ stride;
                if (l > k) {
                    const bool up = (k & size) == 0;
                    const bool gt = key[k] > key[l] || (key[k] == key[l] && idx[k] > idx[l]);
                    if (gt == up) {
                        const uint64_t tk = key[k]; key[k] = key[l]; key[l] = tk;
                        const int ti = idx[k]; idx[k] = idx[l]; idx[l] = ti;
                    }
                }
            }
            __syncthreads();
        }
    for (int k = threadIdx.x; k < E; k += blockDim.x) state[k] = 0;
    __syncthreads();
    for (int round = 0;; ++round) {
        for (int k = threadIdx.x; k < E; k += blockDim.x)
            if (state[k] == 0) {
                const EventRec ev = events[idx[k]];
                atomicMin(&t.claim[ev.p1], k);
                if (ev.p2 != ev.p1) atomicMin(&t.claim[ev.p2], k);
            }
        __syncthreads();
        for (int k = threadIdx.x; k < E; k += blockDim.x)
            if (state[k] == 0) {
                const EventRec ev = events[idx[k]];
                if (t.claim[ev.p1] == k && t.claim[ev.p2] == k) {
                    state[k] = 1;
                    t.taken[ev.p1] = 1;
                    t.taken[ev.p2] = 1;
                }
            }
        if (threadIdx.x == 0) sh_any = 0;
        __syncthreads();
        for (int k = threadIdx.x; k < E; k += blockDim.x) {
            const EventRec ev = events[idx[k]];
            if (state[k] == 0) {
                if (t.taken[ev.p1] || t.taken[ev.p2]) state[k] = 2;
                else sh_any = 1;
            }
            t.claim[ev.p1] = INT_MAX;
            t.claim[ev.p2] = INT_MAX;
        }
        __syncthreads();
        if (!sh_any) break;
        if (round >= 255) {
            if (threadIdx.x == 0) sh_status |= ST_RESOLVE_ROUNDS;
            break;
        }
        __syncthreads();
    }
    // births and new ids of the winners in priority order; offsets reuse the key storage
    int *boff = reinterpret_cast<int *>(key);
    int *ioff = boff + max_events;
    if (threadIdx.x == 0) {
        int nb = 0, ni = 0, nw = 0;
        for (int k = 0; k < E; ++k) {
            boff[k] = nb;
            ioff[k] = ni;
            if (state[k] != 1) continue;
            ++nw;
            switch (tab->reactions[events[idx[k]].reaction].kind) {
                case R_CONVERSION: ni += 1; break;
                case R_ENZYMATIC: ni += 1; break;
                case R_FISSION: nb += 1; ni += 2; break;
                case R_FUSION: nb += 1; ni += 1; break;
                default: break;
            }
        }
        sh_births = nb;
        sh_ids = ni;
        sh_win = nw;
    }
    __syncthreads();
    const bool room = t.n_total + sh_births <= t.capacity;
    for (int k = threadIdx.x; k < E; k += blockDim.x) {
        const EventRec ev = events[idx[k]];
        t.taken[ev.p1] = 0;
        t.taken[ev.p2] = 0;
        if (state[k] != 1) continue;
        const ReactionDev &R = tab->reactions[ev.reaction];
        const int bslot = t.n_total + boff[k];
        const uint32_t nid = t.next_id + (uint32_t)ioff[k];
        float4 p1 = t.pos[ev.p1];
        switch (R.kind) {
            case R_DECAY:  // ReactionUtils.h:164-167
                p1.w = __int_as_float(-1);
                t.pos[ev.p1] = p1;
                break;
            case R_CONVERSION:  // :168-173
                p1.w = __int_as_float(R.product[0]);
                t.pos[ev.p1] = p1;
                t.id[ev.p1] = nid;
                break;
            case R_ENZYMATIC: {  // :174-189, the non-catalyst converts
                if (itype(p1) == R.educt[1]) {
                    float4 p2 = t.pos[ev.p2];
                    p2.w = __int_as_float(R.product[0]);
                    t.pos[ev.p2] = p2;
                    t.id[ev.p2] = nid;
                } else {
                    p1.w = __int_as_float(R.product[0]);
                    t.pos[ev.p1] = p1;
                    t.id[ev.p1] = nid;
                }
                break;
            }
            case R_FISSION: {  // :190-207
                if (!room) break;
                const F3 dir = fission_direction(seed, t.id[ev.p1], step, ev.reaction);
                const float a = R.w2 * R.product_distance, b = R.w1 * R.product_distance;
                float4 q;
                q.x = wrap1(p1.x - a * dir.x, g.L[0], g.hL[0], g.pbc[0]);
                q.y = wrap1(p1.y - a * dir.y, g.L[1], g.hL[1], g.pbc[1]);
                q.z = wrap1(p1.z - a * dir.z, g.L[2], g.hL[2], g.pbc[2]);
                q.w = __int_as_float(R.product[1]);
                t.pos[bslot] = q;
                t.id[bslot] = nid;
                if (t.tslot) t.tslot[bslot] = -1;
                if (t.force) t.force[bslot] = make_float4(0.f, 0.f, 0.f, 0.f);
                p1.x = wrap1(p1.x + b * dir.x, g.L[0], g.hL[0], g.pbc[0]);
                p1.y = wrap1(p1.y + b * dir.y, g.L[1], g.hL[1], g.pbc[1]);
                p1.z = wrap1(p1.z + b * dir.z, g.L[2], g.hL[2], g.pbc[2]);
                p1.w = __int_as_float(R.product[0]);
                t.pos[ev.p1] = p1;
                t.id[ev.p1] = nid + 1u;
                break;
            }
            case R_FUSION: {  // :208-225
                if (!room) break;
                const float4 p2 = t.pos[ev.p2];
                const float w = (R.educt[0] == itype(p1)) ? R.w1 : R.w2;
                const float dx = mi_diff(p2.x, p1.x, g.L[0], g.hL[0], g.pbc[0]);
                const float dy = mi_diff(p2.y, p1.y, g.L[1], g.hL[1], g.pbc[1]);
                const float dz = mi_diff(p2.z, p1.z, g.L[2], g.hL[2], g.pbc[2]);
                float4 q;
                q.x = wrap1(p1.x + w * dx, g.L[0], g.hL[0], g.pbc[0]);
                q.y = wrap1(p1.y + w * dy, g.L[1], g.hL[1], g.pbc[1]);
                q.z = wrap1(p1.z + w * dz, g.L[2], g.hL[2], g.pbc[2]);
                q.w = __int_as_float(R.product[0]);
                t.pos[bslot] = q;
                t.id[bslot] = nid;
                if (t.tslot) t.tslot[bslot] = -1;
                if (t.force) t.force[bslot] = make_float4(0.f, 0.f, 0.f, 0.f);
                p1.w = __int_as_float(-1);
                t.pos[ev.p1] = p1;
                float4 d2 = p2;
                d2.w = __int_as_float(-1);
                t.pos[ev.p2] = d2;
                break;
            }
            default:
                break;
        }
        if (t.reaction_counts) atomicAdd(&t.reaction_counts[R.id], 1ull);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int st = sh_status;
        if (!room && sh_births > 0) st |= ST_CAPACITY;
        if ((uint64_t)t.next_id + (uint64_t)sh_ids > 0xFFFFFF00ull) st |= ST_ID_OVERFLOW;
        sh_status = st;
    }
    __syncthreads();
    res.births = room ? sh_births : 0;
    res.ids = sh_ids;
    res.status = sh_status;
    res.winners = sh_win;
    __syncthreads();
}

}  // namespace rdc

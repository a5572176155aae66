// Device-side building blocks shared by the per-system kernels and the batched replica kernel.
//
// Semantics follow ReaDDy's CPU kernel (paths relative to the readdy/readdy project root):
//   minimum image / wrap ........ include/readdy/common/boundary_condition_operations.h:53-80
//   pair potentials .............. include/readdy/model/potentials/PotentialsOrder2.h:54-305
//   harmonic bond ................ include/readdy/model/topologies/potentials/BondedPotential.h:105-113
//   harmonic angle ............... readdy/main/model/topologies/potentials/AnglePotential.cpp:58-104
//   cosine dihedral .............. readdy/main/model/topologies/potentials/TorsionPotential.cpp:53-153
//   reaction coin ................ include/readdy/kernel/cpu/actions/reactions/ReactionUtils.h:64-76
// Arithmetic is FP32 except the pair-membership predicate: pairs whose FP32 squared distance lies
// within a rounding band of the cutoff are re-decided in FP64 exactly as the reference does, so the
// neighbour pair set is bit-identical to the FP64 CPU kernel on the same (FP32) positions.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "rdc_types.h"

namespace rdc {

// ------------------------------------------------------------------------------------------------
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel random numbers:
// as easy as 1, 2, 3", SC'11).  Constants are the published round multipliers and Weyl increments.
// ------------------------------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };

__host__ __device__ inline void mulhilo32(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}

__host__ __device__ inline U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c.x, hi0, lo0);
        mulhilo32(0xCD9E8D57u, c.z, hi1, lo1);
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// purposes (the 4th counter word) keep the streams of different uses disjoint
enum : uint32_t {
    RNG_BD = 1u, RNG_COIN1 = 2u, RNG_COIN2 = 3u, RNG_PRIO1 = 4u, RNG_PRIO2 = 5u, RNG_FISSION = 6u, RNG_BREAK = 7u,
    RNG_TOPOLOGY = 8u, RNG_STRUCTURAL = 9u
};

__host__ __device__ inline U4 rng_draw(uint64_t seed, uint32_t a, uint32_t b, uint64_t step, uint32_t purpose,
                                       uint32_t reaction) {
    U4 c{a, b, (uint32_t)step, purpose | ((uint32_t)(step >> 32) << 8) | (reaction << 16)};
    return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

// uniform in (0,1), 24-bit resolution, never 0
__device__ inline float u01(uint32_t r) { return ((float)(r >> 8) + 0.5f) * (1.0f / 16777216.0f); }

// four standard normals by the Box-Muller transform of two uniform pairs
__device__ inline void normal4(U4 r, float &n0, float &n1, float &n2, float &n3) {
    float u1 = u01(r.x), u2 = u01(r.y), u3 = u01(r.z), u4 = u01(r.w);
    float r1 = sqrtf(-2.0f * logf(u1)), r2 = sqrtf(-2.0f * logf(u3));
    float s1, c1, s2, c2;
    sincospif(2.0f * u2, &s1, &c1);
    sincospif(2.0f * u4, &s2, &c2);
    n0 = r1 * c1; n1 = r1 * s1; n2 = r2 * c2; n3 = r2 * s2;
}

// ------------------------------------------------------------------------------------------------
// geometry
// ------------------------------------------------------------------------------------------------
__device__ inline float type_of(float4 p) { return p.w; }
__device__ inline int itype(float4 p) { return __float_as_int(p.w); }

// bcs::fixPosition in FP32 with a bounded number of wraps (the box is FP32-exact, so the
// comparisons against +-L/2 are exact)
__device__ inline float wrap1(float x, float L, float hL, int pbc) {
    if (pbc) {
#pragma unroll 1
        for (int k = 0; k < 4 && x >= hL; ++k) x -= L;
#pragma unroll 1
        for (int k = 0; k < 4 && x < -hL; ++k) x += L;
    }
    return x;
}

// bcs::shortestDifference(lhs, rhs) component rhs - lhs, FP32.  A wrapped difference is formed
// as (rhs -+ L) - lhs rather than (rhs - lhs) -+ L: shifting first is exact for coordinates inside
// the box, so the result carries one rounding instead of an error of order ulp(L).
__device__ inline float mi_diff(float rhs, float lhs, float L, float hL, int pbc) {
    float dv = rhs - lhs;
    if (pbc) {
        if (dv > hL) dv = (rhs - L) - lhs;
        else if (dv <= -hL) dv = (rhs + L) - lhs;
    }
    return dv;
}

// geometry held in registers by the hot loops (same member names as Geo; the box edges are FP32-exact,
// so (double)L is the FP64 box of the reference)
struct GeoR {
    float L[3], hL[3], invW[3], invL[3];
    float W[3], M[3];  // cell widths, and the rounding margins of distance bounds to neighbour cells
    int dims[3];
    int pbc[3];
    int exact_always;
};

__device__ inline GeoR geo_r(const Geo &g) {
    GeoR r;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        r.L[d] = g.L[d];
        r.hL[d] = g.hL[d];
        r.invW[d] = g.invW[d];
        r.invL[d] = 1.0f / g.L[d];
        r.dims[d] = g.dims[d];
        r.pbc[d] = g.pbc[d];
        r.W[d] = g.L[d] / (float)g.dims[d];
        r.M[d] = r.W[d] * (1e-4f + 4e-7f * (float)g.dims[d]);
    }
    r.exact_always = g.exact_always;
    return r;
}

// cell width along axis d and the margin that covers the rounding of a particle's offset inside its cell
// (precomputed once per system in GeoR; computed on the spot from a Geo)
__device__ inline void cell_width_margin(const GeoR &g, int d, float &w, float &m) {
    w = g.W[d];
    m = g.M[d];
}
__device__ inline void cell_width_margin(const Geo &g, int d, float &w, float &m) {
    w = g.L[d] / (float)g.dims[d];
    m = w * (1e-4f + 4e-7f * (float)g.dims[d]);
}

// result of the FP64 pair predicate: the rounded FP64 difference and whether d^2 < c^2
struct ExactPair {
    float dx, dy, dz, d2;
    int inside;
};

// bcs::shortestDifference + inner product in FP64 with the reference's rounding order
// ((0 + x*x) + y*y) + z*z and no fused multiply-add.  Out of line: it runs only for the rare pairs
// within the FP32 rounding band of a cutoff and keeps the hot loops small.
static __device__ __noinline__ ExactPair pair_exact_fp64(float4 lhs, float4 rhs, float L0, float L1, float L2, int pbcmask,
                                                  double c2) {
    double d[3] = {__dsub_rn((double)rhs.x, (double)lhs.x), __dsub_rn((double)rhs.y, (double)lhs.y),
                   __dsub_rn((double)rhs.z, (double)lhs.z)};
    const double L[3] = {(double)L0, (double)L1, (double)L2};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (pbcmask & (1 << i)) {
            const double h = L[i] * 0.5;
            if (d[i] > h) d[i] = __dsub_rn(d[i], L[i]);
            else if (d[i] <= -h) d[i] = __dadd_rn(d[i], L[i]);
        }
    }
    double s = __dmul_rn(d[0], d[0]);
    s = __dadd_rn(s, __dmul_rn(d[1], d[1]));
    s = __dadd_rn(s, __dmul_rn(d[2], d[2]));
    ExactPair r;
    r.dx = (float)d[0]; r.dy = (float)d[1]; r.dz = (float)d[2];
    r.d2 = (float)s;
    r.inside = s < c2;
    return r;
}

// ------------------------------------------------------------------------------------------------
// compensated FP32 (error-free transformations) for the terms that cancel near a cutoff, a rest
// length or a potential minimum: the difference of two positions is carried exactly as hi + lo and
// the squared distance as a float-float pair, so r - d, d0 - r, 2 sigma^6 - r^6 ... keep ~24 bits.
// Intrinsics keep the compiler from contracting the products whose rounding errors are captured.
// ------------------------------------------------------------------------------------------------
// rounding error of s = fl(a + b) (Knuth's TwoSum)
__device__ inline float two_sum_err(float a, float b, float s) {
    const float bb = __fsub_rn(s, a);
    return __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// minimum-image rhs - lhs as an unevaluated sum hi + lo; hi equals mi_diff()
__device__ inline void mi_diff2(float rhs, float lhs, float L, float hL, int pbc, float &hi, float &lo) {
    float a = rhs, ea = 0.f;
    const float dv = __fsub_rn(rhs, lhs);
    if (pbc) {
        if (dv > hL) {
            a = __fsub_rn(rhs, L);
            ea = two_sum_err(rhs, -L, a);
        } else if (dv <= -hL) {
            a = __fadd_rn(rhs, L);
            ea = two_sum_err(rhs, L, a);
        }
    }
    hi = __fsub_rn(a, lhs);
    lo = __fadd_rn(two_sum_err(a, -lhs, hi), ea);
}

struct FF { float hi, lo; };

// exact differences and their squared norm as float-float
struct PairExact {
    float dx, dy, dz;  // hi parts (the FP32 minimum-image difference)
    FF d2;
};

__device__ inline float sq_err(float h, float l, float p) {  // (h + l)^2 - p, to first order in l
    return __fadd_rn(__fmaf_rn(h, h, -p), 2.0f * h * l);
}

template <typename G>
__device__ inline PairExact pair_exact(float4 lhs, float4 rhs, const G &g) {
    PairExact r;
    float lx, ly, lz;
    mi_diff2(rhs.x, lhs.x, g.L[0], g.hL[0], g.pbc[0], r.dx, lx);
    mi_diff2(rhs.y, lhs.y, g.L[1], g.hL[1], g.pbc[1], r.dy, ly);
    mi_diff2(rhs.z, lhs.z, g.L[2], g.hL[2], g.pbc[2], r.dz, lz);
    const float px = __fmul_rn(r.dx, r.dx), py = __fmul_rn(r.dy, r.dy), pz = __fmul_rn(r.dz, r.dz);
    const float s1 = __fadd_rn(px, py);
    const float t1 = two_sum_err(px, py, s1);
    const float h = __fadd_rn(s1, pz);
    const float t2 = two_sum_err(s1, pz, h);
    const float e = sq_err(r.dx, lx, px) + sq_err(r.dy, ly, py) + sq_err(r.dz, lz, pz);
    r.d2.hi = h;
    r.d2.lo = __fadd_rn(__fadd_rn(t1, t2), e);
    return r;
}

// (d2 - c) for a float-float d2 and a constant c = chi + clo; accurate when d2 is close to c
__device__ inline float ff_sub(FF d2, float chi, float clo) {
    return __fadd_rn(__fsub_rn(d2.hi, chi), __fsub_rn(d2.lo, clo));
}

// a*b - c*d with one rounding error (Kahan's difference of products)
__device__ inline float diff_prod(float a, float b, float c, float d) {
    const float w = __fmul_rn(c, d);
    const float e = __fmaf_rn(c, d, -w);
    const float f = __fmaf_rn(a, b, -w);
    return __fsub_rn(f, e);
}

// Screening distance: a branch-free minimum image (d - L rint(d / L) on periodic axes) and its squared
// norm.  It differs from the reference-order difference by a few ulp of the box, which the screening
// radius covers; a candidate that passes is re-evaluated exactly.
template <typename G>
__device__ inline float screen_d2(float4 lhs, float4 rhs, const G &g) {
    float dx = rhs.x - lhs.x, dy = rhs.y - lhs.y, dz = rhs.z - lhs.z;
    if (g.pbc[0]) dx = fmaf(-g.L[0], rintf(dx * g.invL[0]), dx);
    if (g.pbc[1]) dy = fmaf(-g.L[1], rintf(dy * g.invL[1]), dy);
    if (g.pbc[2]) dz = fmaf(-g.L[2], rintf(dz * g.invL[2]), dz);
    return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

// Minimum-image difference rhs - lhs in FP32 and its squared norm.
struct PairGeom {
    float dx, dy, dz, d2;
};

template <typename G>
__device__ inline PairGeom pair_geom(float4 lhs, float4 rhs, const G &g) {
    PairGeom r;
    r.dx = mi_diff(rhs.x, lhs.x, g.L[0], g.hL[0], g.pbc[0]);
    r.dy = mi_diff(rhs.y, lhs.y, g.L[1], g.hL[1], g.pbc[1]);
    r.dz = mi_diff(rhs.z, lhs.z, g.L[2], g.hL[2], g.pbc[2]);
    r.d2 = fmaf(r.dx, r.dx, fmaf(r.dy, r.dy, r.dz * r.dz));
    return r;
}

// d^2 < c^2 decided exactly as the FP64 reference: FP32 outside the rounding band, FP64 inside it.
// On an FP64 decision the FP32 difference is replaced by the rounded FP64 one.
template <typename G>
__device__ inline bool within(const PairGeom &pg0, PairGeom &pg, float4 lhs, float4 rhs, const G &g, float c2f,
                              float band, double c2) {
    if (!g.exact_always) {
        if (pg0.d2 < c2f - band) return true;
        if (pg0.d2 > c2f + band) return false;
    }
    const ExactPair e = pair_exact_fp64(lhs, rhs, g.L[0], g.L[1], g.L[2],
                                        (g.pbc[0] ? 1 : 0) | (g.pbc[1] ? 2 : 0) | (g.pbc[2] ? 4 : 0), c2);
    pg.dx = e.dx; pg.dy = e.dy; pg.dz = e.dz;
    pg.d2 = e.d2;
    return e.inside != 0;
}

// in-box test of the cell list (CellLinkedList.cpp:188-192), exact because the box is FP32-exact
__device__ inline bool in_box(float4 p, const Geo &g) {
    return -g.hL[0] <= p.x && g.hL[0] > p.x && -g.hL[1] <= p.y && g.hL[1] > p.y && -g.hL[2] <= p.z &&
           g.hL[2] > p.z;
}

__device__ inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// cell of a particle; the grid is row-major with z fastest (include/readdy/common/Index.h:130-141)
template <typename G>
__device__ inline void cell_coords(float4 p, const G &g, int &cx, int &cy, int &cz) {
    cx = clampi(__float2int_rd((p.x + g.hL[0]) * g.invW[0]), 0, g.dims[0] - 1);
    cy = clampi(__float2int_rd((p.y + g.hL[1]) * g.invW[1]), 0, g.dims[1] - 1);
    cz = clampi(__float2int_rd((p.z + g.hL[2]) * g.invW[2]), 0, g.dims[2] - 1);
}
__device__ inline int cell_index(int cx, int cy, int cz, const Geo &g) {
    return cz + g.dims[2] * (cy + g.dims[1] * cx);
}

// bin of a particle: its cell, OUT (outside the box on a non-periodic axis) or DEAD
__device__ inline int bin_of(float4 p, const Geo &g) {
    if (itype(p) < 0) return g.ncells + 1;  // DEAD
    if (!in_box(p, g)) return g.ncells;     // OUT
    int cx, cy, cz;
    cell_coords(p, g, cx, cy, cz);
    return cell_index(cx, cy, cz, g);
}

// neighbour-cell offsets along one axis without duplicates: dims 1 -> {0}, 2 -> {0,+1} (periodic)
__device__ inline int axis_offsets(int c, int dim, int pbc, int *out) {
    int n = 0;
    if (dim == 1) { out[n++] = 0; return n; }
    for (int o = -1; o <= 1; ++o) {
        int v = c + o;
        if (pbc) {
            v = (v + dim) % dim;
            bool dup = false;
            for (int k = 0; k < n; ++k) dup |= (out[k] == v);
            if (dup) continue;
        } else if (v < 0 || v >= dim) {
            continue;
        }
        out[n++] = v;
    }
    return n;
}

// ------------------------------------------------------------------------------------------------
// pair potentials (force on the particle at lhs, x = rhs - lhs, half the pair energy added to e)
// ------------------------------------------------------------------------------------------------
__device__ inline float ipow(float x, int n) {
    float r = 1.0f;
#pragma unroll 1
    while (n > 0) {
        if (n & 1) r *= x;
        x *= x;
        n >>= 1;
    }
    return r;
}

// Parameter layout of PairPot::p (set by the context registry):
//   harmonic repulsion: k, d, d^2 hi, d^2 lo
//   weak piecewise harmonic: k, d0, depth, rc, d0^2 hi, d0^2 lo, rc^2 hi, rc^2 lo, mid^2 (mid = (d0 + rc) / 2)
//   Lennard-Jones: m, n, rc, shift, epsilon, sigma^2, k, E(rc) shift, is-12-6, sigma^6 hi, sigma^6 lo
//   screened electrostatics: C, kappa, D, sigma, exponent
template <typename G>
__device__ inline void pair_force(const PairPot &pp, const PairGeom &g, float4 lhs, float4 rhs, const G &geo,
                                  float &fx, float &fy, float &fz, float &e) {
    switch (pp.kind) {
        case POT_HARMONIC_REPULSION: {  // PotentialsOrder2.h:73-91; r - d = (d2 - d^2) / (r + d)
            const float k = pp.p[0], d = pp.p[1];
            const PairExact x = pair_exact(lhs, rhs, geo);
            const float d2 = __fadd_rn(x.d2.hi, x.d2.lo);
            const float r = sqrtf(d2);
            const float rd = ff_sub(x.d2, pp.p[2], pp.p[3]) / (r + d);
            if (d2 > 0.0f) {
                const float s = k * rd / r;
                fx += s * x.dx; fy += s * x.dy; fz += s * x.dz;
            }
            e += 0.25f * k * rd * rd;  // half of 0.5 k (r - d)^2
            break;
        }
        case POT_WEAK_PIECEWISE_HARMONIC: {  // PotentialsOrder2.h:131-183
            const float k = pp.p[0], d0 = pp.p[1], depth = pp.p[2], rc = pp.p[3];
            const PairExact x = pair_exact(lhs, rhs, geo);
            const float d2 = __fadd_rn(x.d2.hi, x.d2.lo);
            const float dist = sqrtf(d2);
            const float half = 0.5f * (rc - d0);
            const float c = depth / (half * half);
            const float diff0 = ff_sub(x.d2, pp.p[4], pp.p[5]);  // d2 - d0^2
            float en, factor;
            if (diff0 < 0.0f) {  // dist < d0
                const float t = -diff0 / (d0 + dist);  // d0 - dist
                en = 0.5f * k * t * t - depth;
                factor = -k * t;
            } else if (d2 < pp.p[8]) {  // dist < d0 + half
                const float t = -diff0 / (d0 + dist);  // d0 - dist (<= 0)
                en = 0.5f * c * t * t - depth;
                factor = -c * t;
            } else {  // dist < rc (pre-filtered)
                const float u = -ff_sub(x.d2, pp.p[6], pp.p[7]) / (rc + dist);  // rc - dist
                en = -0.5f * c * u * u;
                factor = c * u;
            }
            e += 0.5f * en;
            if (dist > 0.0f && factor != 0.0f) {
                const float s = factor / dist;
                fx += s * x.dx; fy += s * x.dy; fz += s * x.dz;
            }
            break;
        }
        case POT_LENNARD_JONES: {  // PotentialsOrder2.h:240-264
            const float kk = pp.p[6], eshift = pp.p[7];
            if (pp.p[8] != 0.0f) {
                // 12-6: F = -6k s^6 (2 s^6 - 1) / r^2 x and E = k s^6 (s^6 - 1), s^6 = sigma^6 / r^6, with
                // 2 sigma^6 - r^6 and sigma^6 - r^6 from a float-float r^6 (they cancel at the minimum and at sigma)
                const PairExact x = pair_exact(lhs, rhs, geo);
                const float h = x.d2.hi, l = x.d2.lo;
                const float q = __fmul_rn(h, h);
                const float eq = __fmaf_rn(h, h, -q);
                const float c = __fmul_rn(q, h);
                const float ec = __fmaf_rn(q, h, -c);
                const float cerr = ec + eq * h + 3.0f * q * l;  // r^6 = c + cerr
                const float s6h = pp.p[9], s6l = pp.p[10];
                const float numF = __fadd_rn(__fsub_rn(2.0f * s6h, c), __fsub_rn(2.0f * s6l, cerr));
                const float numE = __fadd_rn(__fsub_rn(s6h, c), __fsub_rn(s6l, cerr));
                const float t = s6h / c;
                const float s = -6.0f * kk * t * (numF / c) / h;
                fx += s * x.dx; fy += s * x.dy; fz += s * x.dz;
                e += 0.5f * (kk * t * (numE / c) - eshift);
            } else {
                // general exponents: integer powers by multiplication
                const int m = (int)pp.p[0], n = (int)pp.p[1];
                const float sigma2 = pp.p[5];
                const float s2 = sigma2 / g.d2;  // (sigma/r)^2
                float sm, sn;
                if ((m & 1) == 0 && (n & 1) == 0) {
                    sm = ipow(s2, m >> 1);
                    sn = ipow(s2, n >> 1);
                } else {
                    const float s1 = sqrtf(s2);
                    sm = ipow(s1, m);
                    sn = ipow(s1, n);
                }
                // F = -k/sigma^2 (m (s/r)^(m+2) - n (s/r)^(n+2)) x
                const float s = -kk / sigma2 * (m * sm - n * sn) * s2;
                fx += s * g.dx; fy += s * g.dy; fz += s * g.dz;
                e += 0.5f * (kk * (sm - sn) - eshift);
            }
            break;
        }
        case POT_SCREENED_ELECTROSTATICS: {  // PotentialsOrder2.h:291-305
            const float C = pp.p[0], kappa = pp.p[1], D = pp.p[2], sigma = pp.p[3];
            const int ex = (int)pp.p[4];
            const float r = sqrtf(g.d2);
            const float ir = 1.0f / r;
            const float ekr = C * expf(-kappa * r);
            const float sr = sigma * ir;
            const float srn = ipow(sr, ex);
            e += 0.5f * (ekr * ir + D * srn);
            float ff = ekr * (kappa * ir + ir * ir);
            ff += D * (float)ex / sigma * srn * sr;
            const float s = -ff * ir;
            fx += s * g.dx; fy += s * g.dy; fz += s * g.dz;
            break;
        }
        default:
            break;
    }
}

// ------------------------------------------------------------------------------------------------
// bonded terms.  Each term is evaluated once and yields the force on every participant (its roles);
// the forces are summed per particle in a fixed order by a gather (no atomics, deterministic).
// ------------------------------------------------------------------------------------------------
struct F3 { float x, y, z; };
__device__ inline F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ inline F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ inline F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ inline F3 operator*(float s, F3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ inline float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ inline F3 cross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
// cross product with each component as a Kahan difference of products (error ~1 ulp of the result)
__device__ inline F3 cross_k(F3 a, F3 b) {
    return {diff_prod(a.y, b.z, a.z, b.y), diff_prod(a.z, b.x, a.x, b.z), diff_prod(a.x, b.y, a.y, b.x)};
}

__device__ inline F3 shortest3(float4 lhs, float4 rhs, const Geo &g) {
    return F3{mi_diff(rhs.x, lhs.x, g.L[0], g.hL[0], g.pbc[0]), mi_diff(rhs.y, lhs.y, g.L[1], g.hL[1], g.pbc[1]),
              mi_diff(rhs.z, lhs.z, g.L[2], g.hL[2], g.pbc[2])};
}

// the same difference as an unevaluated sum hi + lo (hi equals shortest3)
__device__ inline void shortest3_ff(float4 lhs, float4 rhs, const Geo &g, F3 &hi, F3 &lo) {
    mi_diff2(rhs.x, lhs.x, g.L[0], g.hL[0], g.pbc[0], hi.x, lo.x);
    mi_diff2(rhs.y, lhs.y, g.L[1], g.hL[1], g.pbc[1], hi.y, lo.y);
    mi_diff2(rhs.z, lhs.z, g.L[2], g.hL[2], g.pbc[2], hi.z, lo.z);
}

// (ah + al) x (bh + bl) to first order in the low parts: accurate to a few ulp of the result even
// when the two vectors are nearly parallel and the result is much shorter than |a||b|
__device__ inline F3 cross_ff(F3 ah, F3 al, F3 bh, F3 bl) {
    return cross_k(ah, bh) + (cross(ah, bl) + cross(al, bh));
}

// (ah + al) + s (bh + bl) rounded once per component (s = +-1), from the exact sum of the high parts
__device__ inline F3 ff_sum3(F3 ah, F3 al, F3 bh, F3 bl, float sgn) {
    auto one = [&](float a, float la, float b, float lb) {
        const float bb = sgn * b;
        const float h = __fadd_rn(a, bb);
        return __fadd_rn(h, __fadd_rn(two_sum_err(a, bb, h), __fadd_rn(la, sgn * lb)));
    };
    return F3{one(ah.x, al.x, bh.x, bl.x), one(ah.y, al.y, bh.y, bl.y), one(ah.z, al.z, bh.z, bl.z)};
}

// FP64 vectors for the few quantities that need more than FP32 (the dihedral angle)
struct D3 { double x, y, z; };
__device__ inline D3 d3(F3 hi, F3 lo) {
    return D3{(double)hi.x + (double)lo.x, (double)hi.y + (double)lo.y, (double)hi.z + (double)lo.z};
}
__device__ inline D3 dcross(D3 a, D3 b) {
    return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ inline D3 dneg(D3 a) { return D3{-a.x, -a.y, -a.z}; }
__device__ inline double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ inline D3 dadd(D3 a, D3 b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ inline D3 dsub(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ inline D3 dlin(double a, D3 u, double b, D3 v) {
    return D3{a * u.x + b * v.x, a * u.y + b * v.y, a * u.z + b * v.z};
}
__device__ inline F3 f3of(D3 a) { return F3{(float)a.x, (float)a.y, (float)a.z}; }
__device__ inline D3 operator+(D3 a, D3 b) { return dadd(a, b); }
__device__ inline D3 operator-(D3 a, D3 b) { return dsub(a, b); }
__device__ inline D3 operator-(D3 a) { return dneg(a); }
__device__ inline D3 operator*(double s, D3 a) { return D3{s * a.x, s * a.y, s * a.z}; }

// harmonic bond: E = k (r - l0)^2, force on i = 2k (r-l0)/r x_ij, on j its negative
// (BondedPotential.h:105-113, CPUTopologyActions.cpp:61-74); r - l0 = (d2 - l0^2) / (r + l0)
// from the float-float d2.  P = (k, l0, l0^2 hi, l0^2 lo)
// ------------------------------------------------------------------------------------------------
// order-1 (external) potentials (include/readdy/model/potentials/PotentialsOrder1.h:60-225, geometries of
// include/readdy/model/geometry.h).  Differences to the geometry come from TwoSum, and every (d - r)
// near a surface is formed as (d^2 - r^2)/(d + r) from a float-float d^2, so forces keep their digits
// where they vanish.
// ------------------------------------------------------------------------------------------------
struct FF3 { F3 hi, lo; };
__device__ inline FF3 diff_ff(float4 x, const float *c) {  // x - c, exactly
    FF3 r;
    r.hi.x = __fsub_rn(x.x, c[0]); r.lo.x = two_sum_err(x.x, -c[0], r.hi.x);
    r.hi.y = __fsub_rn(x.y, c[1]); r.lo.y = two_sum_err(x.y, -c[1], r.hi.y);
    r.hi.z = __fsub_rn(x.z, c[2]); r.lo.z = two_sum_err(x.z, -c[2], r.hi.z);
    return r;
}
__device__ inline FF norm2_ff(const FF3 &v) {  // |hi + lo|^2 as float-float, to first order in lo
    const float px = __fmul_rn(v.hi.x, v.hi.x), py = __fmul_rn(v.hi.y, v.hi.y), pz = __fmul_rn(v.hi.z, v.hi.z);
    const float s1 = __fadd_rn(px, py);
    const float t1 = two_sum_err(px, py, s1);
    const float h = __fadd_rn(s1, pz);
    const float t2 = two_sum_err(s1, pz, h);
    const float e = sq_err(v.hi.x, v.lo.x, px) + sq_err(v.hi.y, v.lo.y, py) + sq_err(v.hi.z, v.lo.z, pz);
    return FF{h, __fadd_rn(__fadd_rn(t1, t2), e)};
}
__device__ inline F3 ff_value(const FF3 &v) { return v.hi + v.lo; }

// v + s * u as float-float (v float-float, s and u FP32): the products' rounding errors are kept
__device__ inline FF3 axpy_ff(const FF3 &v, float s, F3 u) {
    auto one = [&](float vh, float vl, float uu) {
        const float ph = __fmul_rn(s, uu), pe = __fmaf_rn(s, uu, -ph);
        const float h = __fadd_rn(vh, ph);
        return FF{h, __fadd_rn(__fadd_rn(two_sum_err(vh, ph, h), vl), pe)};
    };
    const FF x = one(v.hi.x, v.lo.x, u.x), y = one(v.hi.y, v.lo.y, u.y), z = one(v.hi.z, v.lo.z, u.z);
    return FF3{f3(x.hi, y.hi, z.hi), f3(x.lo, y.lo, z.lo)};
}

// (ah + al) x (bh + bl) as float-float: a1 b2 - a2 b1 per component with both products' rounding
// errors and the first-order low-part terms kept
__device__ inline FF3 cross_ff3(const FF3 &a, const FF3 &b) {
    auto one = [](float a1h, float a1l, float b2h, float b2l, float a2h, float a2l, float b1h, float b1l) {
        const float p1 = __fmul_rn(a1h, b2h), e1 = __fmaf_rn(a1h, b2h, -p1);
        const float p2 = __fmul_rn(a2h, b1h), e2 = __fmaf_rn(a2h, b1h, -p2);
        const float h = __fsub_rn(p1, p2);
        const float l = two_sum_err(p1, -p2, h) + (e1 - e2) + (a1l * b2h - a2l * b1h) + (a1h * b2l - a2h * b1l);
        return FF{h, l};
    };
    const FF x = one(a.hi.y, a.lo.y, b.hi.z, b.lo.z, a.hi.z, a.lo.z, b.hi.y, b.lo.y);
    const FF y = one(a.hi.z, a.lo.z, b.hi.x, b.lo.x, a.hi.x, a.lo.x, b.hi.z, b.lo.z);
    const FF z = one(a.hi.x, a.lo.x, b.hi.y, b.lo.y, a.hi.y, a.lo.y, b.hi.x, b.lo.x);
    return FF3{f3(x.hi, y.hi, z.hi), f3(x.lo, y.lo, z.lo)};
}

// geometry::Sphere::smallestDifference (geometry.h:25-49) for a difference `delta` from the centre
__device__ inline F3 sphere_diff(const FF3 &delta, float radius, float r2hi, float r2lo, int inclusion) {
    const FF d2 = norm2_ff(delta);
    const float d2f = __fadd_rn(d2.hi, d2.lo);
    if (inclusion ? d2f < r2hi : d2f > r2hi) return f3(0.f, 0.f, 0.f);
    const float d = sqrtf(d2f);
    if (!inclusion && d < 1e-5f) return f3(-radius, 0.f, 0.f);
    const float dr = ff_sub(d2, r2hi, r2lo) / (d + radius);  // d - r
    return (dr / d) * ff_value(delta);
}

// adds the force and energy of the order-1 potentials first..first+cnt-1 on a particle at p
__device__ inline void order1_force(float4 p, const O1Pot *pots, int first, int cnt, float &fx, float &fy, float &fz,
                                    float &e) {
    for (int q = first; q < first + cnt; ++q) {
        const O1Pot &o = pots[q];
        const float *P = o.p;
        F3 f = f3(0.f, 0.f, 0.f);
        switch (o.kind) {
            case O1_BOX: {  // HarmonicGeometryPotential<Box>, geometry.h:77-116
                const float x[3] = {p.x, p.y, p.z};
                float dv[3] = {0.f, 0.f, 0.f};
                if (o.inclusion) {
                    for (int d = 0; d < 3; ++d) {
                        if (x[d] < P[1 + d]) dv[d] = x[d] - P[1 + d];
                        else if (x[d] > P[4 + d]) dv[d] = x[d] - P[4 + d];
                    }
                } else {
                    bool inside = true;
                    for (int d = 0; d < 3; ++d) inside = inside && x[d] > P[1 + d] && x[d] < P[4 + d];
                    if (inside) {  // nearest face; the first minimum wins, like std::min_element
                        int best = 0;
                        float bd = fabsf(x[0] - P[1]);
                        for (int k = 1; k < 6; ++k) {
                            const float v = fabsf(x[k / 2] - P[(k % 2 == 0 ? 1 : 4) + k / 2]);
                            if (v < bd) { bd = v; best = k; }
                        }
                        dv[best / 2] = x[best / 2] - P[(best % 2 == 0 ? 1 : 4) + best / 2];
                    }
                }
                e += 0.5f * P[0] * (dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
                f = f3(-P[0] * dv[0], -P[0] * dv[1], -P[0] * dv[2]);
                break;
            }
            case O1_SPHERE: {  // HarmonicGeometryPotential<Sphere>
                const F3 dv = sphere_diff(diff_ff(p, P + 1), P[4], P[5], P[6], o.inclusion);
                e += 0.5f * P[0] * dot(dv, dv);
                f = (-P[0]) * dv;
                break;
            }
            case O1_CAPSULE: {  // HarmonicGeometryPotential<Capsule>, closest circle centre geometry.h:132-150
                const FF3 xc = diff_ff(p, P + 1);
                const F3 n = f3(P[4], P[5], P[6]);
                const float lambda = fminf(P[7], fmaxf(-P[7], dot(ff_value(xc), n)));
                FF3 delta = axpy_ff(xc, -lambda, n);  // x - (c + lambda n) as float-float, n = hi + lo
                delta.lo = delta.lo + (-lambda) * f3(P[11], P[12], P[13]);
                const F3 dv = sphere_diff(delta, P[8], P[9], P[10], o.inclusion);
                e += 0.5f * P[0] * dot(dv, dv);
                f = (-P[0]) * dv;
                break;
            }
            case O1_SPHERICAL_BARRIER: {  // SphericalBarrier, PotentialsOrder1.h:103-146
                const FF3 df = diff_ff(p, P);
                const FF d2 = norm2_ff(df);
                const float dist = sqrtf(__fadd_rn(d2.hi, d2.lo));
                const float radius = P[3], width = P[4], height = P[5], keff = P[6];
                if (dist < P[7] || P[10] <= dist) break;
                const float dr = ff_sub(d2, P[11], P[12]) / (dist + radius);  // dist - radius
                const F3 u = (1.0f / dist) * ff_value(df);
                if (dist < P[8]) {
                    const float s = dr + width;
                    e += 0.5f * keff * s * s;
                    f = (-keff * s) * u;
                } else if (dist < P[9]) {
                    e += height - 0.5f * keff * dr * dr;
                    f = (keff * dr) * u;
                } else {
                    const float s = dr - width;
                    e += 0.5f * keff * s * s;
                    f = (-keff * s) * u;
                }
                break;
            }
            case O1_CYLINDER: {  // Cylinder, PotentialsOrder1.h:168-209; perp = n x (pos x n)
                const FF3 pos = diff_ff(p, P + 1);
                const F3 n = f3(P[4], P[5], P[6]);
                const FF3 pxn = cross_ff3(pos, FF3{n, f3(P[10], P[11], P[12])});
                const FF d2 = norm2_ff(pxn);
                const float dist = sqrtf(__fadd_rn(d2.hi, d2.lo));
                const float radius = P[7];
                if (o.inclusion ? dist > radius : dist < radius) {
                    const F3 perp = cross_k(n, ff_value(pxn));
                    const float dr = ff_sub(d2, P[8], P[9]) / (dist + radius);
                    e += 0.5f * P[0] * dr * dr;
                    f = (-P[0] * dr / dist) * perp;
                }
                break;
            }
        }
        fx += f.x;
        fy += f.y;
        fz += f.z;
    }
}

// harmonic bond, E = k (|x_ij| - l0)^2 (BondedPotential.h): the force on particle i (role 0); particle j
// (role 1) takes its negative
__device__ inline F3 bond_force(float4 pi, float4 pj, float4 P, const Geo &g, float &e) {
    const PairExact x = pair_exact(pi, pj, g);
    const float r = sqrtf(__fadd_rn(x.d2.hi, x.d2.lo));
    const float rd = ff_sub(x.d2, P.z, P.w) / (r + P.y);
    e = P.x * rd * rd;
    const float s = 2.0f * P.x * rd / r;
    return s * f3(x.dx, x.dy, x.dz);
}

// harmonic angle, E = k (theta - theta0)^2 (AnglePotential.cpp:58-104) with the reference's clamps
// (|x|^2, |x_ji||x_jk|, sin theta >= 1e-10).  theta comes from atan2(|x_ji x x_jk|, x_ji . x_jk)
// (cross product by Kahan's difference of products); for obtuse angles theta - theta0 is formed as
// (pi - theta0) - atan2(|cross|, -dot), which stays exact at the straight-chain minimum theta0 = pi.
// P = (k, theta0, pi - theta0, -)
__device__ inline void angle_force(float4 pi, float4 pj, float4 pk, float4 P, const Geo &g, F3 f[3], float &e) {
    const float SMALL = 1e-10f;
    const float kf = P.x;
    F3 a, la, b, lb;
    shortest3_ff(pj, pi, g, a, la);  // x_ji
    shortest3_ff(pj, pk, g, b, lb);  // x_jk
    const F3 cr = cross_ff(a, la, b, lb);  // short near theta = 0 and pi: formed from the exact differences
    const float cn = sqrtf(dot(cr, cr));
    const float sp = dot(a, b);
    const float na2 = fmaxf(dot(a, a), SMALL), nb2 = fmaxf(dot(b, b), SMALL);
    const float np = fmaxf(sqrtf(na2) * sqrtf(nb2), SMALL);
    float dth;
    if (sp < 0.0f) dth = P.z - atan2f(cn, -sp);
    else dth = atan2f(cn, sp) - P.y;
    e = kf * dth * dth;
    // The reference's force_i = c cos(theta)/|a|^2 a - c/(|a||b|) b with c = 2k dth / sin(theta) is
    // -(c/(|a||b|)) times the part of b perpendicular to a, ((a x b) x a)/|a|^2; force_k likewise
    // with (b x (a x b))/|b|^2.  Formed from the cross product, that part keeps its relative accuracy
    // near theta = 0 and pi, where the two terms of the reference's expression cancel.  The
    // reference's clamp sin(theta) >= SMALL becomes |a x b| >= SMALL |a||b|.
    const float q = 2.0f * kf * dth / fmaxf(cn, SMALL * np);
    const F3 fi = (-q / na2) * cross_k(cr, a);
    const F3 fk = (-q / nb2) * cross_k(b, cr);
    f[0] = (-1.0f) * fi;
    f[1] = fi + fk;
    f[2] = (-1.0f) * fk;
}

// cosine dihedral, the analytic gradient of TorsionPotential.cpp:70-153 written with explicit
// cross products; same clamps (1e-4) and the same zero-force rule for |cos phi| < 1e-4.  f[r] receives
// the force on the term's particle r (i, j, k, l)
__device__ inline void dihedral_force(float4 pi, float4 pj, float4 pk, float4 pl, float kf, float mult, float phi0,
                                      const Geo &g, F3 f[4], float &e) {
    const float SMALL = 1e-4f;
    F3 xji, lji, xkj, lkj, xkl, lkl;
    shortest3_ff(pj, pi, g, xji, lji);  // x_i - x_j
    shortest3_ff(pk, pj, g, xkj, lkj);  // x_j - x_k
    shortest3_ff(pk, pl, g, xkl, lkl);  // x_l - x_k
    // m = x_ji x x_kj and n = x_kl x x_jk are formed from the exact differences: near a straight bond
    // angle m or n is short, and rounded differences would cost it most of its digits.
    // The dihedral angle is taken in FP64 from the exact differences.  Its force is dV/dphi times a
    // gradient of length ~1/(|x_ji| sin theta); near n phi - phi0 = 0 mod pi, dV/dphi is small and an
    // FP32 phi (error ~1e-7 rad) would leave it with few correct digits.
    const D3 Fd = d3(xji, lji), Gd = d3(xkj, lkj), Hd = d3(xkl, lkl);
    const D3 md = dcross(Fd, Gd), nd = dneg(dcross(Hd, Gd)), jkd = dneg(Gd);  // m, n, x_jk of the reference
    const double mm_d = ddot(md, md), nn_d = ddot(nd, nd), jk2_d = ddot(jkd, jkd);
    const double mxn_jk = ddot(dcross(md, nd), jkd), m_n = ddot(md, nd);
    // force (TorsionPotential.cpp:70-159): clamps on |x_jk|^2, |m|^2, |n|^2 and |m||n|
    const double nmn_d = fmax(sqrt(fmax(mm_d, (double)SMALL)) * sqrt(fmax(nn_d, (double)SMALL)), (double)SMALL);
    const double cphi_d = m_n / nmn_d;
    const double sphi_d = mxn_jk / (nmn_d * sqrt(fmax(jk2_d, (double)SMALL)));
    const bool unclamped = jk2_d >= SMALL && mm_d >= SMALL && nn_d >= SMALL && sqrt(mm_d) * sqrt(nn_d) >= SMALL;
    double sn, cs;
    if (unclamped) {
        // the energy's clamps (TorsionPotential.cpp:53-68, on |x_jk| and |m||n|) are inactive as well: its
        // angle is the force's, bit for bit, and one sincos gives both
        sincos((double)mult * -atan2(sphi_d, cphi_d) - (double)phi0, &sn, &cs);
        e = (float)((double)kf * (1.0 + cs));
    } else {
        const double xjkn_e = fmax(sqrt(jk2_d), (double)SMALL);
        const double mnn_e = fmax(sqrt(mm_d) * sqrt(nn_d), (double)SMALL);
        const double dih = -atan2(mxn_jk / (mnn_e * xjkn_e), m_n / mnn_e);
        e = (float)((double)kf * (1.0 + cos((double)mult * dih - (double)phi0)));
        sn = sin((double)mult * -atan2(sphi_d, cphi_d) - (double)phi0);
    }
    if (fabs(cphi_d) < (double)SMALL) {
        f[0] = f[1] = f[2] = f[3] = f3(0.f, 0.f, 0.f);
        return;
    }
    const double dVdphi_d = -(double)kf * (double)mult * sn;
    if (unclamped) {
        // No clamp of the reference is active, so its gradient equals the analytic one.  Taken in the
        // form of Blondel & Karplus (J. Comput. Chem. 17, 1132 (1996)) with F = x_ji, G = x_kj,
        // H = x_kl, A = F x G (= m), B = H x G (= -n).  The coefficients of the middle atoms,
        // |G|/|A|^2 + F.G/(|A|^2 |G|) and H.G/(|B|^2 |G|) - |G|/|B|^2, are G.(x_i - x_k)/(|A|^2 |G|) and
        // G.(x_l - x_j)/(|B|^2 |G|).  The middle atoms' forces are differences of an A and a B part that
        // can cancel, so the gradient is formed in FP64 from the exact differences (once per term, next
        // to the FP64 angle).  The reference's phi is -(phi_BK +- pi), so its force
        // -dV/dphi dphi/dx = dV/dphi dphi_BK/dx.
        const D3 Ad = md, Bd = dneg(nd);
        const double A2 = mm_d, B2 = nn_d, Gn = sqrt(jk2_d);
        const D3 xik = dadd(Fd, Gd), xlj = dsub(Hd, Gd);  // x_i - x_k, x_l - x_j
        const double cA = dVdphi_d / (A2 * Gn), cB = dVdphi_d / (B2 * Gn);
        f[0] = f3of(dlin(-dVdphi_d * Gn / A2, Ad, 0.0, Bd));
        f[1] = f3of(dlin(cA * ddot(Gd, xik), Ad, -cB * ddot(Hd, Gd), Bd));
        f[2] = f3of(dlin(-cA * ddot(Fd, Gd), Ad, cB * ddot(Gd, xlj), Bd));
        f[3] = f3of(dlin(0.0, Ad, dVdphi_d * Gn / B2, Bd));
        return;
    }
    // A clamp is active: the reference's own gradient expression (TorsionPotential.cpp:70-159), with m
    // and n of the reference, in FP64 from the exact differences (near-collinear atoms make it
    // ill-conditioned).  With the skew tensors of the reference:
    //   v * dm_dxi = x_kj x v, v * dm_dxk = x_ji x v, v * dn_dxj = x_kl x v, v * dn_dxl = -(x_kj x v)
    //   x_jk * dmxn_dx = d(m x n) contracted with x_jk
    const D3 &xji_d = Fd, &xkj_d = Gd, &xkl_d = Hd, &xjk_d = jkd, &m = md, &n = nd;
    const double S = (double)SMALL;
    const double xjkn2 = fmax(jk2_d, S), xjkn = sqrt(xjkn2);
    const double mn = sqrt(fmax(mm_d, S)), nn = sqrt(fmax(nn_d, S));
    const double nmn = fmax(mn * nn, S);
    const D3 mxn = dcross(m, n);
    const double cphi = cphi_d, sphi = sphi_d;
    const double sbc = sphi / cphi;
    const double ppre = -1.0 / (cphi * (1.0 + sbc * sbc));
    const double cpre = 1.0 / nmn, spre = 1.0 / (nmn * xjkn);
    // gradients of |m| and |n| (TorsionPotential.cpp:95-106)
    const double jikj = ddot(xji_d, xkj_d), kljk = ddot(xkl_d, xjk_d);
    const D3 dmn2_dxi = (2.0 * xjkn2) * xji_d - (2.0 * jikj) * xkj_d;
    const D3 dmn2_dxk = (-2.0 * ddot(xji_d, xji_d)) * xkj_d + (2.0 * jikj) * xji_d;
    const D3 dnn2_dxl = (2.0 * xjkn2) * xkl_d - (2.0 * kljk) * xjk_d;
    const D3 dnn2_dxj = (-2.0 * ddot(xkl_d, xkl_d)) * xjk_d + (2.0 * kljk) * xkl_d;
    const double i2m = 1.0 / (2.0 * mn), i2n = 1.0 / (2.0 * nn);
    const D3 nxj = dcross(n, xjk_d), jxm = dcross(xjk_d, m);
    auto force_of = [&](const D3 &dc, const D3 &ds) { return f3of((-dVdphi_d * ppre) * (ds - sbc * dc)); };
    {  // x_i: m depends on x_ji, n does not
        const D3 dmn = i2m * dmn2_dxi;
        const D3 dc = cpre * (dcross(xkj_d, n) - (cphi * nn) * dmn);
        // x_jk . (dm/dxi_c x n) = (n x x_jk) . dm/dxi_c = (x_kj x (n x x_jk))_c
        const D3 ds = spre * (dcross(xkj_d, nxj) - (sphi * nn * xjkn) * dmn);
        f[0] = force_of(dc, ds);
    }
    {  // x_j: dm_dxj = -(dm_dxk + dm_dxi), dn_dxj = skew(x_kl)
        const D3 dmn = i2m * (-(dmn2_dxi + dmn2_dxk));
        const D3 dnn = i2n * dnn2_dxj;
        const D3 n_dm = -(dcross(xji_d, n) + dcross(xkj_d, n));
        const D3 dc = cpre * (n_dm + dcross(xkl_d, m) - (cphi * nn) * dmn - (cphi * mn) * dnn);
        const D3 v = -(dcross(xji_d, nxj) + dcross(xkj_d, nxj)) + dcross(xkl_d, jxm);
        const D3 ds = spre * (v - mxn - (sphi * nn * xjkn) * dmn - (sphi * mn * xjkn) * dnn + (sphi * nmn / xjkn) * xjk_d);
        f[1] = force_of(dc, ds);
    }
    {  // x_k: dm_dxk = skew(x_ji), dn_dxk = -(dn_dxj + dn_dxl) = -(skew(x_kl) - skew(x_kj))
        const D3 dmn = i2m * dmn2_dxk;
        const D3 dnn = i2n * (-(dnn2_dxl + dnn2_dxj));
        const D3 m_dn = -(dcross(xkl_d, m) - dcross(xkj_d, m));
        const D3 dc = cpre * (dcross(xji_d, n) + m_dn - (cphi * nn) * dmn - (cphi * mn) * dnn);
        const D3 v = dcross(xji_d, nxj) - (dcross(xkl_d, jxm) - dcross(xkj_d, jxm));
        const D3 ds = spre * (v + mxn - (sphi * nn * xjkn) * dmn - (sphi * mn * xjkn) * dnn - (sphi * nmn / xjkn) * xjk_d);
        f[2] = force_of(dc, ds);
    }
    {  // x_l: only n depends on x_kl; dn/dxl_c = -(skew(x_kj) col c)
        const D3 dnn = i2n * dnn2_dxl;
        const D3 dc = cpre * (-dcross(xkj_d, m) - (cphi * mn) * dnn);
        // x_jk . (m x dn/dxl_c) = (x_jk x m) . dn/dxl_c
        const D3 ds = spre * (-dcross(xkj_d, jxm) - (sphi * mn * xjkn) * dnn);
        f[3] = force_of(dc, ds);
    }
}

}  // namespace rdc

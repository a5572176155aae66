// rdc_forces_noalloc: pair forces and energy of caller-owned device arrays, with no device allocation.
//
// rdc_calculate_forces works on a system whose particle arrays, cell list and energy partials this
// library allocated when the system was created.  Some callers cannot let a library call cudaMalloc
// at the point where they want forces: embeddings (an MD engine, a PyTorch extension with its own
// caching allocator, a service that carves HBM into fixed pools) own all device memory and hand none
// of it to a library, and a step loop that must not stall on the allocator's implicit
// synchronisation cannot afford one either.
//
// This entry point reads positions and types from the caller's device arrays and writes forces and
// the energy into the caller's device arrays.  Its working space (cell counts and starts, the
// cell-sorted copy of the particles, per-block energy partials and the potential tables) is one
// statically sized array in this library's device image, g_noalloc_scratch below, whose address is
// taken once per device with cudaGetSymbolAddress.  The arithmetic is the per-system force kernel's
// (pair_force_at of rdc_phases.cuh: same stencil walk, exact cutoff predicate and FP32 terms); only
// the summation order over neighbours can differ, because the cell-sorted order is built here from
// the caller's order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>

#include "../../include/readdy_cuda.h"
#include "rdc_phases.cuh"

using namespace rdc;

namespace rdc {
const ContextData &context_data(const rdc_context *ctx);
void set_last_error(const std::string &m);
}  // namespace rdc

namespace {

constexpr int NA_MAX_PARTICLES = RDC_NOALLOC_MAX_PARTICLES;
constexpr int NA_MAX_CELLS = RDC_NOALLOC_MAX_CELLS;
constexpr int NA_FORCE_BLOCKS = 256;
constexpr int NA_THREADS = 256;
constexpr int NA_MAX_DEVICES = 64;

constexpr size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

// byte offsets inside the scratch array (every region starts on a 256-byte boundary)
constexpr size_t OFF_TAB = 0;
constexpr size_t OFF_CNT = up256(OFF_TAB + sizeof(Tables));                          // int[cells + 2]
constexpr size_t OFF_START = up256(OFF_CNT + sizeof(int) * (NA_MAX_CELLS + 2));      // int[cells + 3]
constexpr size_t OFF_BIN = up256(OFF_START + sizeof(int) * (NA_MAX_CELLS + 3));      // int[n]
constexpr size_t OFF_RANK = up256(OFF_BIN + sizeof(int) * NA_MAX_PARTICLES);         // int[n]
constexpr size_t OFF_SRC1 = up256(OFF_RANK + sizeof(int) * NA_MAX_PARTICLES);        // int[n]
constexpr size_t OFF_SRC = up256(OFF_SRC1 + sizeof(int) * NA_MAX_PARTICLES);         // int[n]
constexpr size_t OFF_POS = up256(OFF_SRC + sizeof(int) * NA_MAX_PARTICLES);          // float4[n]
constexpr size_t OFF_EPART = up256(OFF_POS + sizeof(float4) * NA_MAX_PARTICLES);     // double[blocks]
constexpr size_t OFF_STATUS = up256(OFF_EPART + sizeof(double) * NA_FORCE_BLOCKS);   // int
constexpr size_t OFF_FPRINT = OFF_STATUS + 8;  // uint64: fingerprint of the tables held at OFF_TAB
constexpr size_t NA_SCRATCH_BYTES = up256(OFF_FPRINT + sizeof(uint64_t));
static_assert(NA_SCRATCH_BYTES == RDC_NOALLOC_SCRATCH_BYTES, "scratch size in the header is stale");

}  // namespace

// The working space of rdc_forces_noalloc, one per device (the array lives in every device's copy of
// this library's module).  Its contents at load time do not matter: each call zeroes the cell counts
// and the status word before using them, and writes every other region before reading it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_SCRATCH_BYTES];

namespace {

// status bits of one call: a type outside [0, n_types); a position outside the box on a periodic axis
// or not a number; tables in the scratch other than the call's (an overlapping call for another context)
enum : int { NA_BAD_TYPE = 1, NA_BAD_POSITION = 2, NA_STALE_TABLES = 4 };

struct NaScratch {
    Tables *tab;
    int *cnt, *start, *bin, *rank, *src1, *src;
    float4 *pos;
    double *epart;
    int *status;
    unsigned long long *fprint;
};

NaScratch carve(unsigned char *base) {
    NaScratch s;
    s.tab = reinterpret_cast<Tables *>(base + OFF_TAB);
    s.cnt = reinterpret_cast<int *>(base + OFF_CNT);
    s.start = reinterpret_cast<int *>(base + OFF_START);
    s.bin = reinterpret_cast<int *>(base + OFF_BIN);
    s.rank = reinterpret_cast<int *>(base + OFF_RANK);
    s.src1 = reinterpret_cast<int *>(base + OFF_SRC1);
    s.src = reinterpret_cast<int *>(base + OFF_SRC);
    s.pos = reinterpret_cast<float4 *>(base + OFF_POS);
    s.epart = reinterpret_cast<double *>(base + OFF_EPART);
    s.status = reinterpret_cast<int *>(base + OFF_STATUS);
    s.fprint = reinterpret_cast<unsigned long long *>(base + OFF_FPRINT);
    return s;
}

// FNV-1a over the bytes of the tables: the fingerprint a call expects to find next to them
uint64_t tables_fingerprint(const Tables &t) {
    const unsigned char *b = reinterpret_cast<const unsigned char *>(&t);
    uint64_t h = 0xcbf29ce484222325ull;
    for (size_t k = 0; k < sizeof(Tables); ++k) h = (h ^ b[k]) * 0x100000001b3ull;
    return h;
}

// particle i of the caller's arrays as the device layout (type bits in .w; -1 marks a bad type)
__device__ inline float4 load_particle(const float *__restrict__ pos3, const int *__restrict__ types, int i,
                                       int ntypes, bool &bad) {
    int t = types[i];
    bad = t < 0 || t >= ntypes;
    if (bad) t = -1;
    return make_float4(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], __int_as_float(t));
}

// zeroes the bin counts and the status word; a fingerprint other than the one of the tables this call
// was made for raises NA_STALE_TABLES
__global__ void k_na_clear(NaScratch s, int nbins, unsigned long long fprint) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nbins; k += gridDim.x * blockDim.x) s.cnt[k] = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) *s.status = (*s.fprint == fprint) ? 0 : NA_STALE_TABLES;
}

// a coordinate that is not a number, or outside [-L/2, L/2) on a periodic axis (the range of
// bcs::fixPosition, include/readdy/common/boundary_condition_operations.h:53-61)
__device__ inline bool bad_position(float4 p, const Geo &g) {
    const float c[3] = {p.x, p.y, p.z};
    bool bad = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) bad |= !(c[d] == c[d]) || (g.pbc[d] && !(c[d] >= -g.hL[d] && c[d] < g.hL[d]));
    return bad;
}

__global__ void k_na_bin(NaScratch s, Geo geo, const float *__restrict__ pos3, const int *__restrict__ types, int n,
                         int ntypes) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    bool bad;
    const float4 p = load_particle(pos3, types, i, ntypes, bad);
    if (bad) atomicOr(s.status, NA_BAD_TYPE);
    if (bad_position(p, geo)) atomicOr(s.status, NA_BAD_POSITION);
    const int b = bin_of(p, geo);  // cells, then OUT (outside the box), then DEAD (bad type)
    s.bin[i] = b;
    s.rank[i] = atomicAdd(&s.cnt[b], 1);
}

// exclusive scan of the bin counts by one block; start[nbins] = n
__global__ void __launch_bounds__(1024) k_na_scan(NaScratch s, int nbins) {
    const int per = (nbins + blockDim.x - 1) / blockDim.x;
    const int b0 = min(nbins, (int)threadIdx.x * per), b1 = min(nbins, b0 + per);
    int local = 0;
    for (int k = b0; k < b1; ++k) local += s.cnt[k];
    int total;
    int run = block_exclusive_scan(local, total);
    for (int k = b0; k < b1; ++k) {
        s.start[k] = run;
        run += s.cnt[k];
    }
    if (threadIdx.x == 0) s.start[nbins] = total;
}

__global__ void k_na_scatter(NaScratch s, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    s.src1[s.start[s.bin[i]] + s.rank[i]] = i;
}

// final slot = bin start + number of the bin's particles with a smaller caller index, so the sorted
// order of a cell does not depend on the order in which the atomics above were served (a scan of the
// cell: quadratic in the particles of a cell, a handful at the cutoff's cell width).  Particles outside
// the cells (OUT and DEAD bins) get no force, so their order does not matter: they keep the slot the
// atomics gave them, which bounds the work when many particles are outside.
__global__ void k_na_place(NaScratch s, Geo geo, const float *__restrict__ pos3, const int *__restrict__ types, int n,
                           int ntypes) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = s.bin[i];
    const int sb = s.start[b], se = s.start[b + 1];
    int r = s.rank[i];
    if (b < geo.ncells) {
        r = 0;
        for (int k = sb; k < se; ++k) r += s.src1[k] < i;
    }
    bool bad;
    s.src[sb + r] = i;
    s.pos[sb + r] = load_particle(pos3, types, i, ntypes, bad);
}

__global__ void __launch_bounds__(NA_THREADS, 2) k_na_forces(NaScratch s, Geo geo, float *__restrict__ forces3,
                                                             int n) {
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
    const int n_in = s.start[geo.ncells];  // particles inside cells
    const GeoR g = geo_r(geo);
    // tables replaced by a call for another context: every force is NaN (and the energy, below)
    const bool stale = (*s.status & NA_STALE_TABLES) != 0;
    double esum = 0.0;
    for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < n; slot += gridDim.x * blockDim.x) {
        float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
        if (stale) {
            fx = fy = fz = __int_as_float(0x7fc00000);
        } else if (slot < n_in && NP > 0) {
            pair_force_at(slot, s.pos[slot], s.pos, s.start, g, 1, sh_tab, sh_scr, sh_pots, T, fx, fy, fz, e);
        }
        const int i = s.src[slot];
        forces3[3 * i] = fx;
        forces3[3 * i + 1] = fy;
        forces3[3 * i + 2] = fz;
        esum += (double)e;
    }
    const double b = block_sum_double(esum);
    if (threadIdx.x == 0) s.epart[blockIdx.x] = b;
}

// energy = sum of the block partials in block order; NaN when a type or a position was out of range or
// the tables were not the call's
__global__ void k_na_energy(NaScratch s, double *energy, int nblocks) {
    double v = 0.0;
    for (int k = threadIdx.x; k < nblocks; k += blockDim.x) v += s.epart[k];
    const double b = block_sum_double(v);
    if (threadIdx.x == 0) *energy = *s.status ? __longlong_as_double(0x7ff8000000000000LL) : b;
}

// per-device set-up state: the scratch address and the tables last copied into it
struct NaDevice {
    unsigned char *base = nullptr;
    bool tables_valid = false;
    Tables tab;
    uint64_t fprint = 0;
};

std::mutex g_na_mutex;
std::unique_ptr<NaDevice> g_na_devices[NA_MAX_DEVICES];

// cell grid for the potentials' largest cutoff, widened until it fits the scratch cell arrays
Geo noalloc_geo(const ContextData &c) {
    double cutoff = 0.0;
    for (auto &p : c.pots) cutoff = std::max(cutoff, p.cutoff);
    Geo g = make_geo(c.box, c.pbc, cutoff, 1);
    if (g.ncells <= NA_MAX_CELLS) return g;
    double w = std::max(cutoff, std::cbrt((double)g.L[0] * g.L[1] * g.L[2] / NA_MAX_CELLS));
    for (int it = 0; it < 200; ++it, w *= 1.05) {
        g = make_geo(c.box, c.pbc, cutoff, 1, w);
        if (g.ncells <= NA_MAX_CELLS) return g;
    }
    throw std::invalid_argument("rdc_forces_noalloc: no cell grid of the box fits the scratch cell arrays");
}

void forces_noalloc(const rdc_context *ctx, int64_t n, const float *pos3, const int *types, float *forces3,
                    double *energy, void *stream_ptr) {
    if (!ctx || !energy || (n > 0 && (!pos3 || !types || !forces3)))
        throw std::invalid_argument("rdc_forces_noalloc: null argument");
    if (n < 0) throw std::invalid_argument("rdc_forces_noalloc: n must be >= 0");
    if (n > NA_MAX_PARTICLES)
        throw std::invalid_argument("rdc_forces_noalloc: " + std::to_string(n) + " particles exceed the scratch limit of " +
                                    std::to_string(NA_MAX_PARTICLES) + " (use a system and rdc_calculate_forces)");
    cudaStream_t st = static_cast<cudaStream_t>(stream_ptr);
    const ContextData &c = context_data(ctx);
    const Geo geo = noalloc_geo(c);
    auto tab = std::make_unique<Tables>();  // host memory: the tables as this context defines them
    build_tables(c, c.box, 0.0, *tab);

    int dev = 0;
    RDC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NA_MAX_DEVICES) throw std::invalid_argument("rdc_forces_noalloc: device index too large");
    unsigned char *base;
    uint64_t fprint;
    {
        std::lock_guard<std::mutex> lock(g_na_mutex);
        auto &slot = g_na_devices[dev];
        if (!slot) slot = std::make_unique<NaDevice>();
        NaDevice &d = *slot;
        const bool setup = d.base == nullptr || !d.tables_valid || std::memcmp(&d.tab, tab.get(), sizeof(Tables)) != 0;
        if (setup) {
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            RDC_CUDA(cudaStreamIsCapturing(st, &cs));
            if (cs != cudaStreamCaptureStatusNone)
                throw std::logic_error("rdc_forces_noalloc: the first call on a device, and the first after the context "
                                       "changed, sets up the scratch and must come before any stream capture");
            if (d.base == nullptr) {
                void *p = nullptr;
                const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
                if (e != cudaSuccess || p == nullptr) {
                    cudaGetLastError();
                    throw CudaError(std::string("rdc_forces_noalloc: cudaGetSymbolAddress of the scratch failed: ") +
                                    cudaGetErrorString(e));
                }
                d.base = static_cast<unsigned char *>(p);
            }
            d.tables_valid = false;
            const uint64_t fp = tables_fingerprint(*tab);
            RDC_CUDA(cudaMemcpyAsync(d.base + OFF_TAB, tab.get(), sizeof(Tables), cudaMemcpyHostToDevice, st));
            RDC_CUDA(cudaMemcpyAsync(d.base + OFF_FPRINT, &fp, sizeof(fp), cudaMemcpyHostToDevice, st));
            RDC_CUDA(cudaStreamSynchronize(st));
            d.tab = *tab;
            d.fprint = fp;
            d.tables_valid = true;
        }
        base = d.base;
        fprint = d.fprint;
    }

    const NaScratch s = carve(base);
    const int nn = (int)n;
    const int nbins = geo.ncells + 2;
    k_na_clear<<<std::min(1024, (nbins + NA_THREADS - 1) / NA_THREADS), NA_THREADS, 0, st>>>(s, nbins, fprint);
    if (nn > 0) {
        const int blocks = (nn + NA_THREADS - 1) / NA_THREADS;
        k_na_bin<<<blocks, NA_THREADS, 0, st>>>(s, geo, pos3, types, nn, c.ntypes);
        k_na_scan<<<1, 1024, 0, st>>>(s, nbins);
        k_na_scatter<<<blocks, NA_THREADS, 0, st>>>(s, nn);
        k_na_place<<<blocks, NA_THREADS, 0, st>>>(s, geo, pos3, types, nn, c.ntypes);
        k_na_forces<<<std::min(NA_FORCE_BLOCKS, blocks), NA_THREADS, 0, st>>>(s, geo, forces3, nn);
    }
    k_na_energy<<<1, NA_THREADS, 0, st>>>(s, energy, nn > 0 ? std::min(NA_FORCE_BLOCKS, (nn + NA_THREADS - 1) / NA_THREADS)
                                                              : 0);
    RDC_CUDA(cudaGetLastError());
}

}  // namespace

extern "C" int rdc_forces_noalloc(const rdc_context *ctx, int64_t n, const float *positions3, const int *types,
                                  float *forces3, double *energy, void *stream) {
    try {
        forces_noalloc(ctx, n, positions3, types, forces3, energy, stream);
        return RDC_OK;
    } catch (const CudaError &e) {
        set_last_error(e.what());
        return RDC_ERR_CUDA;
    } catch (const std::invalid_argument &e) {
        set_last_error(e.what());
        return RDC_ERR_INVALID_ARGUMENT;
    } catch (const std::logic_error &e) {
        set_last_error(e.what());
        return RDC_ERR_LOGIC;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return RDC_ERR_RUNTIME;
    }
}

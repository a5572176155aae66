// C ABI of libreaddy_cuda_core.so (include/readdy_cuda.h) and the host orchestration of the
// per-system path: context registries, device tables, particle storage, the action sequence of
// SimulationLoop::run (include/readdy/api/SimulationLoop.h:256-306) captured in a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <climits>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/readdy_cuda.h"
#include "rdc_device.cuh"  // Philox streams (rng_draw) for the host's topology-reaction draws
#include "rdc_host.h"

using namespace rdc;

namespace {
thread_local std::string g_err;

struct InvalidArgument : std::invalid_argument {
    using std::invalid_argument::invalid_argument;
};
struct LogicError : std::logic_error {
    using std::logic_error::logic_error;
};

template <typename F>
int guarded(F &&f) {
    try {
        f();
        g_err.clear();
        return RDC_OK;
    } catch (const CapacityError &e) {
        g_err = e.what();
        return RDC_ERR_CAPACITY;
    } catch (const CudaError &e) {
        g_err = e.what();
        return RDC_ERR_CUDA;
    } catch (const std::invalid_argument &e) {
        g_err = e.what();
        return RDC_ERR_INVALID_ARGUMENT;
    } catch (const std::logic_error &e) {
        g_err = e.what();
        return RDC_ERR_LOGIC;
    } catch (const std::exception &e) {
        g_err = e.what();
        return RDC_ERR_RUNTIME;
    }
}

void require(bool c, const std::string &msg) {
    if (!c) throw InvalidArgument(msg);
}

template <typename T>
T *dalloc(size_t n) {
    void *p = nullptr;
    if (n == 0) n = 1;
    RDC_CUDA(cudaMalloc(&p, n * sizeof(T)));
    return static_cast<T *>(p);
}
template <typename T>
void dfree(T *&p) {
    if (p) cudaFree((void *)p);
    p = nullptr;
}

uint64_t coin_threshold(double rate, double dt) {
    // acceptance probability 1 - exp(-k dt) (ReactionUtils.h:64-71) as a 64-bit threshold
    const double p = 1.0 - std::exp(-rate * dt);
    if (!(p > 0)) return 0;
    const double x = p * 18446744073709551616.0;
    if (x >= 18446744073709551615.0) return ~0ull;
    return (uint64_t)x;
}

// x as an unevaluated float sum hi + lo
void split_ff(double x, float &hi, float &lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

float4 bond_params(double k, double l0) {
    float hi, lo;
    split_ff(l0 * l0, hi, lo);
    return make_float4((float)k, (float)l0, hi, lo);
}

float4 angle_params(double k, double theta0) {
    return make_float4((float)k, (float)theta0, (float)(M_PI - theta0), 0.f);
}

float band_for(double cutoff, const float L[3]) {
    const double Lmax = std::max(L[0], std::max(L[1], L[2]));
    const double c2 = cutoff * cutoff;
    return (float)(1e-5 * c2 + 4e-6 * Lmax * cutoff);
}
}  // namespace

// ---------------------------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------------------------
namespace rdc {

double ContextData::max_cutoff() const {
    double c = 0;
    for (auto &p : pots) c = std::max(c, p.cutoff);
    for (auto &r : reactions)
        if (r.n_educts == 2) c = std::max(c, r.educt_distance);
    for (auto &r : spatial_top) c = std::max(c, r.radius);  // Context::calculateMaxCutoff
    return c;
}

bool ContextData::structural_reactions() const {
    for (auto &r : reactions)
        if (r.kind == R_FUSION || r.kind == R_FISSION || r.kind == R_DECAY) return true;
    return false;
}

Geo make_geo(const double box[3], const int pbc[3], double cutoff, int radius, double min_width) {
    Geo g{};
    double Lmax = 0;
    for (int d = 0; d < 3; ++d) {
        g.L[d] = (float)box[d];
        g.hL[d] = g.L[d] * 0.5f;
        g.Ld[d] = (double)g.L[d];
        g.pbc[d] = pbc[d] ? 1 : 0;
        Lmax = std::max(Lmax, g.Ld[d]);
    }
    g.exact_always = 0;
    for (int d = 0; d < 3; ++d) {
        int dims = 1;
        if (cutoff > 0) {
            // cell width >= cutoff/radius with a margin covering FP32 binning error
            const double w = cutoff / radius + std::ldexp(g.Ld[d], -19) / radius + 1e-6 * cutoff;
            dims = (int)std::max(1.0, std::floor(g.Ld[d] / std::max(w, min_width)));
        }
        g.dims[d] = dims;
        g.invW[d] = (float)((double)dims / g.Ld[d]);
        if (g.pbc[d] && cutoff > 0.45 * g.Ld[d]) g.exact_always = 1;
    }
    const long long nc = (long long)g.dims[0] * g.dims[1] * g.dims[2];
    if (nc > (1LL << 28)) throw InvalidArgument("cell grid too large for the box and cutoff");
    g.ncells = (int)nc;
    return g;
}

void set_time_step(const ContextData &c, double dt, Tables &t) {
    for (int i = 0; i < c.ntypes; ++i) {
        t.bd_drift[i] = (float)(c.D[i] * dt / c.kbt);
        t.bd_scale[i] = (float)std::sqrt(2.0 * c.D[i] * dt);
    }
    for (int r = 0; r < t.nreactions; ++r) t.reactions[r].coin_threshold = coin_threshold(t.reactions[r].rate, dt);
}

void build_tables(const ContextData &c, const double box[3], double dt, Tables &t) {
    std::memset(&t, 0, sizeof(Tables));
    const int T = c.ntypes;
    t.ntypes = T;
    float L[3] = {(float)box[0], (float)box[1], (float)box[2]};
    // pair potentials grouped by unordered type pair, registration order kept within a pair
    std::map<std::pair<int, int>, std::vector<const HostPot *>> groups;
    for (auto &p : c.pots) groups[{std::min(p.t1, p.t2), std::max(p.t1, p.t2)}].push_back(&p);
    int np = 0;
    for (auto &kv : groups) {
        const int first = np;
        for (auto *hp : kv.second) {
            if (np >= MAX_PAIR_POTENTIALS) throw InvalidArgument("too many pair potentials");
            t.pots[np] = hp->pot;
            t.pots[np].band = band_for(hp->cutoff, L);
            ++np;
        }
        const int cnt = np - first;
        if (cnt > 255) throw InvalidArgument("too many potentials for one type pair");
        const int v = (first << 8) | cnt;
        float scr = 0.f;
        for (int k = first; k < np; ++k) scr = std::max(scr, t.pots[k].cutoff2f + 2.0f * t.pots[k].band);
        t.pair_tab[kv.first.first * T + kv.first.second] = v;
        t.pair_tab[kv.first.second * T + kv.first.first] = v;
        t.pair_screen[kv.first.first * T + kv.first.second] = scr;
        t.pair_screen[kv.first.second * T + kv.first.first] = scr;
    }
    t.npots = np;
    // reactions
    t.nreactions = (int)c.reactions.size();
    if (t.nreactions > MAX_REACTIONS) throw InvalidArgument("too many reactions");
    for (int r = 0; r < t.nreactions; ++r) {
        const auto &h = c.reactions[r];
        ReactionDev &d = t.reactions[r];
        d.kind = h.kind;
        d.n_educts = h.n_educts;
        d.n_products = h.n_products;
        d.educt[0] = h.educt[0]; d.educt[1] = h.educt[1];
        d.product[0] = h.product[0]; d.product[1] = h.product[1];
        d.id = r;
        d.w1 = (float)h.w1; d.w2 = (float)h.w2;
        d.product_distance = (float)h.product_distance;
        d.educt_distance2 = h.educt_distance * h.educt_distance;
        d.educt_distance2f = (float)d.educt_distance2;
        d.band = band_for(h.educt_distance, L);
        d.rate = h.rate;
        d.inv_rate = h.rate > 0 ? (float)(1.0 / h.rate) : 0.f;
        d.active = (h.rate > 0 && std::isfinite(d.inv_rate)) ? 1 : 0;
    }
    std::vector<std::vector<int>> o1(T);
    std::map<std::pair<int, int>, std::vector<int>> o2;
    for (int r = 0; r < t.nreactions; ++r) {
        const auto &h = c.reactions[r];
        if (h.n_educts == 1) o1[h.educt[0]].push_back(r);
        else o2[{std::min(h.educt[0], h.educt[1]), std::max(h.educt[0], h.educt[1])}].push_back(r);
    }
    int k = 0;
    for (int ty = 0; ty < T; ++ty) {
        t.o1_tab[ty] = o1[ty].empty() ? 0 : ((k << 8) | (int)o1[ty].size());
        for (int r : o1[ty]) t.o1_list[k++] = r;
    }
    k = 0;
    for (auto &kv : o2) {
        const int v = (k << 8) | (int)kv.second.size();
        float scr = 0.f;
        for (int r : kv.second) scr = std::max(scr, t.reactions[r].educt_distance2f + 2.0f * t.reactions[r].band);
        t.rx_screen[kv.first.first * T + kv.first.second] = scr;
        t.rx_screen[kv.first.second * T + kv.first.first] = scr;
        t.o2_tab[kv.first.first * T + kv.first.second] = v;
        t.o2_tab[kv.first.second * T + kv.first.first] = v;
        t.o2_any[kv.first.first] = 1;
        t.o2_any[kv.first.second] = 1;
        t.has_o2_any = 1;
        for (int r : kv.second) t.o2_list[k++] = r;
    }
    // order-1 potentials grouped by type, registration order kept within a type
    int q = 0;
    for (int ty = 0; ty < T; ++ty) {
        const int first = q;
        for (const auto &h : c.o1pots) {
            if (h.type != ty) continue;
            if (q >= MAX_O1_POTENTIALS) throw InvalidArgument("too many order-1 potentials");
            O1Pot &o = t.o1pots[q++];
            o.kind = h.kind;
            o.inclusion = h.inclusion;
            float *p = o.p;
            switch (h.kind) {
                case O1_BOX:
                    p[0] = (float)h.k;
                    for (int d = 0; d < 3; ++d) { p[1 + d] = (float)h.a[d]; p[4 + d] = (float)(h.a[d] + h.b[d]); }
                    break;
                case O1_SPHERE:
                    p[0] = (float)h.k;
                    for (int d = 0; d < 3; ++d) p[1 + d] = (float)h.a[d];
                    p[4] = (float)h.radius;
                    split_ff(h.radius * h.radius, p[5], p[6]);
                    break;
                case O1_CAPSULE: {
                    const double nn = std::sqrt(h.b[0] * h.b[0] + h.b[1] * h.b[1] + h.b[2] * h.b[2]);
                    p[0] = (float)h.k;
                    for (int d = 0; d < 3; ++d) { p[1 + d] = (float)h.a[d]; split_ff(h.b[d] / nn, p[4 + d], p[11 + d]); }
                    p[7] = (float)(h.length / 2);
                    p[8] = (float)h.radius;
                    split_ff(h.radius * h.radius, p[9], p[10]);
                    break;
                }
                case O1_SPHERICAL_BARRIER:
                    for (int d = 0; d < 3; ++d) p[d] = (float)h.a[d];
                    p[3] = (float)h.radius;
                    split_ff(h.radius * h.radius, p[11], p[12]);
                    p[4] = (float)h.width;
                    p[5] = (float)h.height;
                    p[6] = (float)(4.0 * h.height / h.width / h.width);
                    p[7] = (float)(h.radius - h.width);
                    p[8] = (float)(h.radius - h.width / 2.0);
                    p[9] = (float)(h.radius + h.width / 2.0);
                    p[10] = (float)(h.radius + h.width);
                    break;
                case O1_CYLINDER: {
                    const double nn = std::sqrt(h.b[0] * h.b[0] + h.b[1] * h.b[1] + h.b[2] * h.b[2]);
                    p[0] = (float)h.k;
                    for (int d = 0; d < 3; ++d) { p[1 + d] = (float)h.a[d]; split_ff(h.b[d] / nn, p[4 + d], p[10 + d]); }
                    p[7] = (float)h.radius;
                    split_ff(h.radius * h.radius, p[8], p[9]);
                    break;
                }
            }
        }
        t.o1pot_tab[ty] = q > first ? ((first << 8) | (q - first)) : 0;
    }
    set_time_step(c, dt, t);
}

}  // namespace rdc

struct rdc_context {
    ContextData d;
};

namespace rdc {
const ContextData &context_data(const rdc_context *ctx) { return ctx->d; }
rdc_context *context_clone(const ContextData &d) { return new rdc_context{d}; }
void set_last_error(const std::string &m) { g_err = m; }
}  // namespace rdc

// ---------------------------------------------------------------------------------------------
// system
// ---------------------------------------------------------------------------------------------
struct Topology {
    // terms refer to topology slots
    std::vector<int4> bonds;
    std::vector<float4> bond_par;
    std::vector<int4> angles;
    std::vector<float4> angle_par;
    std::vector<int4> dihedrals;
    std::vector<float4> dih_par;
    // graph edges: (slot1, slot2, first bond term, bond terms), and each bond term's (k, l0) in FP64
    std::vector<int4> edges;
    std::vector<double2> bond_kl;
    std::vector<std::pair<int, int>> edge_owner;  // (graph, local edge) of each edge
};

// one topology: its type, its particles (vertex -> topology slot) and its graph's edges (local vertices)
struct TopGraph {
    int type = 0;
    std::vector<int> slots;
    std::vector<std::pair<int, int>> edges;
    std::vector<double> rates;  // per structural reaction, from its rate function
    bool rates_valid = false;   // false once the topology was created or changed
};

// recipe operations of a structural topology reaction (include/readdy/model/topologies/reactions/Recipe.h)
enum : int { RECIPE_CHANGE_PARTICLE_TYPE = 0, RECIPE_ADD_EDGE = 1, RECIPE_REMOVE_EDGE = 2, RECIPE_SEPARATE_VERTEX = 3,
             RECIPE_CHANGE_TOPOLOGY_TYPE = 4, RECIPE_APPEND_PARTICLE = 5, RECIPE_CHANGE_PARTICLE_POSITION = 6 };
struct RecipeOp {
    int kind;
    int64_t a, b;
    int type;
    std::vector<int64_t> neighbors;  // append: the new particle's neighbours
    double pos[3];                   // append, change position
};

struct StructuralReaction {
    int topology_type;
    rdc_topology_rate_fn rate;
    rdc_topology_recipe_fn reaction;
    void *user;
    bool expect_connected;
};

struct rdc_recipe {
    std::vector<RecipeOp> ops;
};

struct rdc_system {
    ContextData ctx;
    uint64_t seed = 0;
    cudaStream_t stream = nullptr;
    SysDev d{};
    Tables *tab_dev = nullptr;
    Tables tab{};
    double tab_dt = 0;
    int radius = 1;
    double nl_cutoff = 0;
    bool nl_ready = false;
    bool forces_live = false;
    int n_top = 0;
    Topology top;
    std::vector<TopGraph> graphs;     // the active topologies
    std::vector<int> slot_type;       // particle type per topology slot
    std::vector<uint32_t> slot_id;    // particle id per topology slot
    uint64_t break_calls = 0;         // BreakBonds calls so far: keys their coins
    uint64_t topo_calls = 0;          // topology reaction evaluations so far: keys their clocks and coins
    std::vector<uint64_t> topo_counts;  // performed events per spatial topology reaction
    std::vector<StructuralReaction> structural;  // registered with callbacks of the embedding
    std::vector<uint64_t> structural_counts;
    bool in_callback = false;           // a structural reaction's function is running
    TopCandidate *cand_dev = nullptr;
    int cand_cap = 0;
    uint32_t *top_mask_dev = nullptr;  // MAX_TYPES pair masks of the spatial reactions
    int *top_n_dev = nullptr;
    int4 *edit_dev = nullptr;
    int edit_cap = 0;
    double topo_dt = 0;               // > 0: run() evaluates topology reactions every step with this time step
    int4 *edge_dev = nullptr;
    double2 *bond_kl_dev = nullptr;
    int2 *bond_at_dev = nullptr;
    int4 *angle_at_dev = nullptr, *dih_at_dev = nullptr;
    float4 *term_force_dev = nullptr;
    int *top_off_dev = nullptr, *top_terms_dev = nullptr;
    int4 *bond_idx_dev = nullptr, *angle_idx_dev = nullptr, *dih_idx_dev = nullptr;
    float4 *bond_par_dev = nullptr, *angle_par_dev = nullptr;
    float4 *dih_par_dev = nullptr;
    int top_capacity = 0;
    int ncells_alloc = -1;
    unsigned long long *count_buf = nullptr;  // MAX_TYPES scratch for count_types
    int *pairs_n = nullptr;
    // graph of the run loop (captured per run: device pointers and the recording base are baked in)
    cudaGraphExec_t graph = nullptr;

    ~rdc_system() { release(); }

    void release() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        dfree(d.pos); dfree(d.id); dfree(d.tslot); dfree(d.force);
        dfree(d.pos_alt); dfree(d.id_alt); dfree(d.tslot_alt); dfree(d.force_alt);
        dfree(d.bin); dfree(d.rank); dfree(d.src);
        dfree(d.cnt); dfree(d.start); dfree(d.scan_blocks); dfree(d.big_cells);
        dfree(d.tloc); dfree(d.counters); dfree(d.step);
        dfree(d.events); dfree(d.claim); dfree(d.taken); dfree(d.reaction_counts);
        dfree(d.epart); dfree(d.energy); dfree(d.counts_ring); dfree(d.vpart); dfree(d.virial);
        dfree(tab_dev); dfree(count_buf); dfree(pairs_n);
        dfree(top_off_dev); dfree(top_terms_dev);
        dfree(bond_idx_dev); dfree(angle_idx_dev); dfree(dih_idx_dev);
        dfree(bond_par_dev); dfree(angle_par_dev); dfree(dih_par_dev);
        dfree(edge_dev); dfree(bond_kl_dev);
        dfree(bond_at_dev); dfree(angle_at_dev); dfree(dih_at_dev); dfree(term_force_dev);
        dfree(cand_dev); dfree(top_mask_dev); dfree(top_n_dev); dfree(edit_dev);
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }

    void sync() { RDC_CUDA(cudaStreamSynchronize(stream)); }

    void read_counters(int *c) {
        RDC_CUDA(cudaMemcpyAsync(c, d.counters, sizeof(int) * C_COUNT, cudaMemcpyDeviceToHost, stream));
        sync();
    }

    // raise device-side status as an error and clear it
    void check_status() {
        int c[C_COUNT];
        read_counters(c);
        const int st = c[C_STATUS];
        if (st) {
            int zero = 0;
            RDC_CUDA(cudaMemcpyAsync(d.counters + C_STATUS, &zero, sizeof(int), cudaMemcpyHostToDevice, stream));
            sync();
            if (st & ST_CAPACITY) throw CapacityError("particle capacity exceeded by reaction products (rdc_reserve)");
            if (st & ST_EVENTS) throw CapacityError("reaction event buffer overflow");
            if (st & ST_ID_OVERFLOW) throw std::runtime_error("32-bit particle id space exhausted");
            if (st & ST_RESOLVE_ROUNDS) throw std::runtime_error("reaction conflict resolution did not converge");
            throw std::runtime_error("device status " + std::to_string(st));
        }
    }

    void init(const ContextData &c, uint64_t s) {
        ctx = c;
        seed = s;
        RDC_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        init_kernel_attributes();
        tab_dev = dalloc<Tables>(1);
        build_tables(ctx, ctx.box, 0.0, tab);
        tab_dt = 0;
        upload_tables();
        d.tab = tab_dev;
        d.seed = seed;
        d.radius = radius;
        d.counters = dalloc<int>(C_COUNT);
        RDC_CUDA(cudaMemsetAsync(d.counters, 0, sizeof(int) * C_COUNT, stream));
        d.step = dalloc<uint64_t>(3);  // integrator step, reaction step, particles advanced
        RDC_CUDA(cudaMemsetAsync(d.step, 0, sizeof(uint64_t) * 3, stream));
        d.reaction_counts = dalloc<unsigned long long>(MAX_REACTIONS);
        RDC_CUDA(cudaMemsetAsync(d.reaction_counts, 0, sizeof(unsigned long long) * MAX_REACTIONS, stream));
        d.epart = dalloc<double>(FORCE_BLOCKS + BONDED_BLOCKS);
        RDC_CUDA(cudaMemsetAsync(d.epart, 0, sizeof(double) * (FORCE_BLOCKS + BONDED_BLOCKS), stream));
        d.energy = dalloc<double>(1);
        RDC_CUDA(cudaMemsetAsync(d.energy, 0, sizeof(double), stream));
        if (ctx.record_virial) {
            d.vpart = dalloc<double>(9 * FORCE_BLOCKS);
            d.virial = dalloc<double>(9);
            RDC_CUDA(cudaMemsetAsync(d.virial, 0, sizeof(double) * 9, stream));
        }
        d.event_capacity = 1 << 16;
        d.events = dalloc<EventRec>(d.event_capacity);
        count_buf = dalloc<unsigned long long>(MAX_TYPES);
        pairs_n = dalloc<int>(1);
        d.geo = make_geo(ctx.box, ctx.pbc, 0.0, 1);
        alloc_cells(d.geo.ncells);
        reserve(1024);
        sync();
    }

    void upload_tables() {
        RDC_CUDA(cudaMemcpyAsync(tab_dev, &tab, sizeof(Tables), cudaMemcpyHostToDevice, stream));
    }

    void set_dt(double dt) {
        if (dt != tab_dt) {
            set_time_step(ctx, dt, tab);
            tab_dt = dt;
            upload_tables();
        }
    }

    void alloc_cells(int ncells) {
        if (ncells == ncells_alloc) return;
        dfree(d.cnt); dfree(d.start); dfree(d.scan_blocks); dfree(d.big_cells);
        d.big_cells = dalloc<int>(ncells + 2);
        d.cnt = dalloc<int>(ncells + 2);
        d.start = dalloc<int>(ncells + 3);
        d.scan_blocks = dalloc<int>(scan_block_count(ncells + 2) + 1);
        RDC_CUDA(cudaMemsetAsync(d.cnt, 0, sizeof(int) * (ncells + 2), stream));
        RDC_CUDA(cudaMemsetAsync(d.start, 0, sizeof(int) * (ncells + 3), stream));
        ncells_alloc = ncells;
        invalidate_graph();
    }

    void invalidate_graph() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
    }

    // Context::recordVirial switched on a live system: ReaDDy reads the flag from the context at every
    // force calculation (CPUCalculateForces.cpp:154), and its Virial observable sets it after the state
    // model may already hold particles.  The next force calculation records (or stops recording) the virial.
    void set_record_virial(bool on) {
        if (on == (d.virial != nullptr)) return;
        sync();
        if (on) {
            d.vpart = dalloc<double>(9 * FORCE_BLOCKS);
            d.virial = dalloc<double>(9);
            RDC_CUDA(cudaMemsetAsync(d.vpart, 0, sizeof(double) * 9 * FORCE_BLOCKS, stream));
            RDC_CUDA(cudaMemsetAsync(d.virial, 0, sizeof(double) * 9, stream));
        } else {
            dfree(d.vpart);
            dfree(d.virial);
        }
        ctx.record_virial = on;
        invalidate_graph();
        sync();
    }

    // grow the per-particle arrays (host-synchronous)
    void reserve(int cap) {
        if (cap <= d.capacity) return;
        int c[C_COUNT] = {0};
        if (d.capacity > 0) read_counters(c);
        const int n = c[C_N_TOTAL];
        auto grow = [&](auto *&p, int keep) {
            using T = std::remove_reference_t<decltype(*p)>;
            T *np = dalloc<T>(cap);
            if (p && keep > 0) RDC_CUDA(cudaMemcpyAsync(np, p, sizeof(T) * keep, cudaMemcpyDeviceToDevice, stream));
            sync();
            dfree(p);
            p = np;
        };
        grow(d.pos, n); grow(d.id, n); grow(d.tslot, n); grow(d.force, n);
        grow(d.pos_alt, 0); grow(d.id_alt, 0); grow(d.tslot_alt, 0); grow(d.force_alt, 0);
        grow(d.bin, 0); grow(d.rank, 0); grow(d.src, 0);
        grow(d.claim, 0); grow(d.taken, 0);
        RDC_CUDA(cudaMemsetAsync(d.claim, 0x7f, sizeof(int) * cap, stream));
        RDC_CUDA(cudaMemsetAsync(d.taken, 0, sizeof(int) * cap, stream));
        d.capacity = cap;
        sync();
        invalidate_graph();
    }

    void swap_buffers() {
        std::swap(d.pos, d.pos_alt);
        std::swap(d.id, d.id_alt);
        std::swap(d.tslot, d.tslot_alt);
        std::swap(d.force, d.force_alt);
    }

    // append particles (host-synchronous): they join the cell list at the next sort
    void append(int64_t n, const double *pos, const int *types, const int *tslots, uint64_t *ids_out) {
        if (n <= 0) return;
        for (int64_t i = 0; i < n; ++i)
            if (types[i] < 0 || types[i] >= ctx.ntypes) throw InvalidArgument("particle type out of range");
        int c[C_COUNT];
        read_counters(c);
        const int64_t need = (int64_t)c[C_N_TOTAL] + n;
        if (need > INT_MAX / 2) throw InvalidArgument("too many particles");
        // room for the products a reaction step appends before the next sort compacts the storage
        const int64_t want = need + need / 4 + 64;
        if (want > d.capacity) {
            int64_t cap = std::max(d.capacity, 1024);
            while (cap < want) cap *= 2;
            reserve((int)std::min<int64_t>(cap, INT_MAX / 2));
        }
        std::vector<float4> hp(n);
        std::vector<int> ht(n);
        for (int64_t i = 0; i < n; ++i) {
            float4 p;
            p.x = (float)pos[3 * i]; p.y = (float)pos[3 * i + 1]; p.z = (float)pos[3 * i + 2];
            int ty = types[i];
            std::memcpy(&p.w, &ty, 4);
            hp[i] = p;
            ht[i] = tslots ? tslots[i] : -1;
        }
        const int base = c[C_N_TOTAL];
        RDC_CUDA(cudaMemcpyAsync(d.pos + base, hp.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, stream));
        RDC_CUDA(cudaMemcpyAsync(d.tslot + base, ht.data(), sizeof(int) * n, cudaMemcpyHostToDevice, stream));
        RDC_CUDA(cudaMemsetAsync(d.force + base, 0, sizeof(float4) * n, stream));
        launch_fill_ids(d.id + base, (uint32_t)c[C_NEXT_ID], (int)n, stream);
        int upd[2] = {(int)need, c[C_NEXT_ID] + (int)n};
        RDC_CUDA(cudaMemcpyAsync(d.counters + C_N_TOTAL, &upd[0], sizeof(int), cudaMemcpyHostToDevice, stream));
        RDC_CUDA(cudaMemcpyAsync(d.counters + C_NEXT_ID, &upd[1], sizeof(int), cudaMemcpyHostToDevice, stream));
        if (ids_out)
            for (int64_t i = 0; i < n; ++i) ids_out[i] = (uint64_t)(c[C_NEXT_ID] + i);
        sync();
        // without a neighbour list the storage is kept unsorted: every particle is storage, none is in a
        // cell; topology slots map to their insertion index
        if (!nl_ready) {
            int upd2[2] = {(int)need, 0};
            RDC_CUDA(cudaMemcpyAsync(d.counters + C_N, &upd2[0], sizeof(int), cudaMemcpyHostToDevice, stream));
            RDC_CUDA(cudaMemcpyAsync(d.counters + C_N_INCELLS, &upd2[1], sizeof(int), cudaMemcpyHostToDevice,
                                     stream));
            if (tslots) {
                std::vector<int> loc(n);
                for (int64_t i = 0; i < n; ++i) loc[i] = base + (int)i;
                RDC_CUDA(cudaMemcpyAsync(d.tloc + tslots[0], loc.data(), sizeof(int) * n, cudaMemcpyHostToDevice,
                                         stream));
            }
            sync();
        }
    }

    // ---- actions ----
    void nl_create(double cutoff) {
        if (!(cutoff > 0)) throw LogicError("The cutoff distance for setting up a neighbor list must be > 0");
        nl_cutoff = cutoff;
        d.geo = make_geo(ctx.box, ctx.pbc, cutoff, radius);
        d.radius = radius;
        alloc_cells(d.geo.ncells);
        build_tables(ctx, ctx.box, tab_dt, tab);
        upload_tables();
        nl_ready = true;
        invalidate_graph();
        nl_update();
    }
    void nl_update() {
        if (!nl_ready) throw LogicError("Attempting to fill neighborlist bins, but cell structure is not set up yet");
        launch_bin(d, stream);
        launch_sort(d, forces_live, stream);
        swap_buffers();
    }
    void nl_clear() {
        nl_ready = false;
        nl_cutoff = 0;
    }
    void calculate_forces() {
        if (!ctx.pots.empty() && !nl_ready) throw LogicError("calculate forces: the neighbor list is not set up");
        launch_forces(d, true, n_top > 0, stream);
        forces_live = true;
    }
    void integrate(double dt) {
        set_dt(dt);
        // integrate + bin: the bins are refreshed at the next nl_update, so only integrate here
        integrate_only();
        forces_live = false;
    }
    void integrate_only();
    void react(double dt, int handler) {
        if (ctx.reactions.empty()) return;
        if (!nl_ready) throw LogicError("reactions: the neighbor list is not set up");
        set_dt(dt);
        launch_events(d, handler, stream);
        launch_resolve_apply(d, handler, stream);
        if (ctx.structural_reactions()) {
            // reaction products must be in the cell list before the next consumer
            launch_bin(d, stream);
            launch_sort(d, false, stream);
            swap_buffers();
        }
    }

    // ---- topology ----
    void add_topology(int topology_type, int64_t n, const double *pos, const int *types, int64_t n_edges,
                      const int64_t *edges, uint64_t *ids_out);
    void configure(const TopGraph &g, int graph_index, Topology &out) const;
    void upload_topology(bool sort_new_particles = true);
    int64_t break_bonds(double dt, int n_pairs, const int *t1, const int *t2, const double *threshold,
                        const double *rate);
    int64_t evaluate_topology_reactions(double dt);
    void grow_topology_slots(int n_new);

    // ---- SimulationLoop::run ----
    void run(int64_t n_steps, double dt, int handler, int64_t stride, int64_t *counts, int64_t max_rec,
             int64_t *n_rec);
    void step_sequence(int handler, bool reactions, bool structural, int nsteps);
};

void rdc_system::integrate_only() {
    // k_integrate_bin with binning into the count array; the bin results are discarded by the
    // next nl_update, which re-bins. Counting here keeps the launch identical to the fused one.
    launch_integrate_bin(d, true, stream);
}

// findNTuples over one topology graph (include/graphs/bits/Graph_detail.h:39-76) and the type-tuple
// lookup of GraphTopology::configure (readdy/main/model/topologies/GraphTopology.cpp:59-143): appends the
// graph's bond, angle and dihedral terms and its edges to out; throws if an edge has no bond configured
void rdc_system::configure(const TopGraph &gr, int graph_index, Topology &out) const {
    const int n = (int)gr.slots.size();
    std::vector<std::vector<int>> adj(n);
    std::vector<std::vector<int>> adj_edge(n);  // local edge index of each adjacency entry
    for (size_t e = 0; e < gr.edges.size(); ++e) {
        const int a = gr.edges[e].first, b = gr.edges[e].second;
        adj[a].push_back(b);
        adj_edge[a].push_back((int)e);
        adj[b].push_back(a);
        adj_edge[b].push_back((int)e);
    }
    auto ty = [&](int v) { return slot_type[gr.slots[v]]; };
    auto sl = [&](int v) { return gr.slots[v]; };
    std::vector<char> visited(n, 0);
    for (int v1 = 0; v1 < n; ++v1) {
        visited[v1] = 1;
        for (size_t a = 0; a < adj[v1].size(); ++a) {
            const int nb = adj[v1][a];
            if (!visited[nb]) {
                const int first = (int)out.bonds.size();
                for (auto &c : ctx.bonds) {
                    if ((c.t1 == ty(v1) && c.t2 == ty(nb)) || (c.t1 == ty(nb) && c.t2 == ty(v1))) {
                        out.bonds.push_back(make_int4(sl(v1), sl(nb), 0, 0));
                        out.bond_par.push_back(bond_params(c.k, c.l0));
                        out.bond_kl.push_back(make_double2(c.k, c.l0));
                    }
                }
                const int count = (int)out.bonds.size() - first;
                if (count == 0)
                    throw InvalidArgument("The edge " + std::to_string(v1) + " -- " + std::to_string(nb) +
                                          " has no bond configured!");
                out.edges.push_back(make_int4(sl(v1), sl(nb), first, count));
                out.edge_owner.emplace_back(graph_index, adj_edge[v1][a]);
                for (int q1 : adj[v1]) {
                    if (q1 == nb) continue;
                    for (int q2 : adj[nb]) {
                        if (q2 == v1 || q2 == q1) continue;
                        const int tt[4] = {ty(q1), ty(v1), ty(nb), ty(q2)};
                        for (auto &c : ctx.dihedrals) {
                            const bool fwd = c.t1 == tt[0] && c.t2 == tt[1] && c.t3 == tt[2] && c.t4 == tt[3];
                            const bool bwd = c.t1 == tt[3] && c.t2 == tt[2] && c.t3 == tt[1] && c.t4 == tt[0];
                            if (fwd || bwd) {
                                out.dihedrals.push_back(make_int4(sl(q1), sl(v1), sl(nb), sl(q2)));
                                out.dih_par.push_back(make_float4((float)c.k, (float)c.mult, (float)c.phi0, 0.f));
                            }
                        }
                    }
                }
            }
            for (int nb2 : adj[v1]) {
                if (nb2 != nb && nb2 < nb) {
                    const int tt[3] = {ty(nb2), ty(v1), ty(nb)};
                    for (auto &c : ctx.angles) {
                        const bool fwd = c.t1 == tt[0] && c.t2 == tt[1] && c.t3 == tt[2];
                        const bool bwd = c.t1 == tt[2] && c.t2 == tt[1] && c.t3 == tt[0];
                        if (fwd || bwd) {
                            out.angles.push_back(make_int4(sl(nb2), sl(v1), sl(nb), 0));
                            out.angle_par.push_back(angle_params(c.k, c.theta0));
                        }
                    }
                }
            }
        }
    }
}

template <typename T>
static void append_all(std::vector<T> &to, const std::vector<T> &from) {
    to.insert(to.end(), from.begin(), from.end());
}

void rdc_system::add_topology(int topology_type, int64_t n, const double *pos, const int *types, int64_t n_edges,
                              const int64_t *edges, uint64_t *ids_out) {
    require(n > 0, "topology needs particles");
    require(topology_type >= 0, "topology type must be >= 0");
    for (int64_t i = 0; i < n; ++i) require(types[i] >= 0 && types[i] < ctx.ntypes, "particle type out of range");
    const int base = n_top;
    TopGraph g;
    g.type = topology_type;
    g.slots.resize(n);
    for (int64_t i = 0; i < n; ++i) g.slots[i] = base + (int)i;
    for (int64_t e = 0; e < n_edges; ++e) {
        const int64_t a = edges[2 * e], b = edges[2 * e + 1];
        require(a >= 0 && b >= 0 && a < n && b < n && a != b, "bad topology edge");
        g.edges.emplace_back((int)a, (int)b);
    }
    // terms first, into a scratch list: an edge without a bond configuration leaves the system unchanged
    const size_t old_slots = slot_type.size();
    slot_type.insert(slot_type.end(), types, types + n);
    Topology add;
    try {
        configure(g, (int)graphs.size(), add);
    } catch (...) {
        slot_type.resize(old_slots);
        throw;
    }
    std::vector<int> slots(n);
    for (int64_t i = 0; i < n; ++i) slots[i] = base + (int)i;
    // the slot -> storage map grows with its entries kept, and covers the new slots before any sort
    // gathers them
    int *tloc_new = dalloc<int>(n_top + n);
    if (n_top > 0 && d.tloc)
        RDC_CUDA(cudaMemcpyAsync(tloc_new, d.tloc, sizeof(int) * n_top, cudaMemcpyDeviceToDevice, stream));
    sync();
    dfree(d.tloc);
    d.tloc = tloc_new;
    n_top += (int)n;
    d.tloc_size = n_top;
    d.n_top = 0;  // bonded terms are uploaded below; until then the force kernel skips them
    std::vector<uint64_t> ids(n);
    append(n, pos, types, slots.data(), ids.data());
    if (ids_out) std::copy(ids.begin(), ids.end(), ids_out);
    for (auto v : ids) slot_id.push_back((uint32_t)v);
    graphs.push_back(std::move(g));
    // shift the scratch list's bond term indices behind the existing ones
    const int bond_base = (int)top.bonds.size();
    for (auto &e : add.edges) e.z += bond_base;
    append_all(top.bonds, add.bonds);
    append_all(top.bond_par, add.bond_par);
    append_all(top.bond_kl, add.bond_kl);
    append_all(top.angles, add.angles);
    append_all(top.angle_par, add.angle_par);
    append_all(top.dihedrals, add.dihedrals);
    append_all(top.dih_par, add.dih_par);
    append_all(top.edges, add.edges);
    append_all(top.edge_owner, add.edge_owner);
    upload_topology();
}

// BreakBonds (include/readdy/model/actions/Actions.h:236-290): the device draws which edges break; the
// graphs lose those edges, a graph that falls apart becomes its connected components (same topology
// type; a component of one particle of NORMAL flavor leaves the topologies,
// include/readdy/model/actions/Utils.h:59-79, GraphTopology.cpp:161-173), and the bonded terms are
// derived again from the remaining graphs (StructuralTopologyReaction.cpp:115-127).  The reference
// action also adds the evaluated bonds' forces to the particles' force accumulators
// (CPUTopologyActions.cpp:55-70); here forces stay as they were until the next CalculateForces.
int64_t rdc_system::break_bonds(double dt, int n_pairs, const int *t1, const int *t2, const double *threshold,
                                const double *rate) {
    require(dt > 0, "time step must be > 0");
    require(n_pairs >= 0, "n_pairs must be >= 0");
    const int T = ctx.ntypes;
    std::vector<double> thr(T * T, std::numeric_limits<double>::quiet_NaN());
    std::vector<uint64_t> coin(T * T, 0);
    for (int k = 0; k < n_pairs; ++k) {
        require(t1[k] >= 0 && t1[k] < T && t2[k] >= 0 && t2[k] < T, "particle type out of range");
        require(!std::isnan(threshold[k]), "threshold energy must be a number");
        require(rate[k] >= 0, "break rate must be >= 0");
        for (int o = 0; o < 2; ++o) {
            const int a = o ? t2[k] : t1[k], b = o ? t1[k] : t2[k];
            thr[a * T + b] = threshold[k];
            coin[a * T + b] = coin_threshold(rate[k], dt);
        }
    }
    const int ne = (int)top.edges.size();
    const uint64_t call = break_calls++;
    if (ne == 0 || n_pairs == 0) return 0;
    double *thr_dev = dalloc<double>(T * T);
    uint64_t *coin_dev = dalloc<uint64_t>(T * T);
    int *out_dev = dalloc<int>(ne + 1);
    RDC_CUDA(cudaMemcpyAsync(thr_dev, thr.data(), sizeof(double) * T * T, cudaMemcpyHostToDevice, stream));
    RDC_CUDA(cudaMemcpyAsync(coin_dev, coin.data(), sizeof(uint64_t) * T * T, cudaMemcpyHostToDevice, stream));
    launch_break_bonds(d, edge_dev, ne, bond_kl_dev, thr_dev, coin_dev, T, seed, call, out_dev + 1, out_dev, stream);
    int nb = 0;
    RDC_CUDA(cudaMemcpyAsync(&nb, out_dev, sizeof(int), cudaMemcpyDeviceToHost, stream));
    sync();
    std::vector<int> broken(nb);
    if (nb > 0) RDC_CUDA(cudaMemcpyAsync(broken.data(), out_dev + 1, sizeof(int) * nb, cudaMemcpyDeviceToHost, stream));
    sync();
    dfree(thr_dev);
    dfree(coin_dev);
    dfree(out_dev);
    if (nb == 0) return 0;
    // remove the broken edges from their graphs
    std::vector<std::vector<char>> gone(graphs.size());
    for (int e : broken) {
        require(e >= 0 && e < ne, "broken edge index out of range");
        const auto [gi, le] = top.edge_owner[e];
        if (gone[gi].empty()) gone[gi].assign(graphs[gi].edges.size(), 0);
        gone[gi][le] = 1;
    }
    std::vector<TopGraph> next;
    next.reserve(graphs.size());
    for (size_t gi = 0; gi < graphs.size(); ++gi) {
        TopGraph &g = graphs[gi];
        if (gone[gi].empty()) {
            next.push_back(std::move(g));
            continue;
        }
        std::vector<std::pair<int, int>> kept;
        for (size_t e = 0; e < g.edges.size(); ++e)
            if (!gone[gi][e]) kept.push_back(g.edges[e]);
        // connected components over the kept edges, each listing its vertices in their graph order
        const int n = (int)g.slots.size();
        std::vector<std::vector<int>> adj(n);
        for (auto &e : kept) {
            adj[e.first].push_back(e.second);
            adj[e.second].push_back(e.first);
        }
        std::vector<int> comp(n, -1);
        int nc = 0;
        for (int v = 0; v < n; ++v) {
            if (comp[v] >= 0) continue;
            std::vector<int> stack{v};
            comp[v] = nc;
            while (!stack.empty()) {
                const int u = stack.back();
                stack.pop_back();
                for (int w : adj[u])
                    if (comp[w] < 0) {
                        comp[w] = nc;
                        stack.push_back(w);
                    }
            }
            ++nc;
        }
        std::vector<TopGraph> parts(nc);
        std::vector<int> local(n);
        for (int v = 0; v < n; ++v) {
            local[v] = (int)parts[comp[v]].slots.size();
            parts[comp[v]].slots.push_back(g.slots[v]);
            parts[comp[v]].type = g.type;
        }
        for (auto &e : kept) parts[comp[e.first]].edges.emplace_back(local[e.first], local[e.second]);
        for (auto &part : parts) {
            const bool single_normal = nc > 1 && part.slots.size() == 1 &&
                                       ctx.flavor[slot_type[part.slots[0]]] == FLAVOR_NORMAL;
            if (!single_normal) next.push_back(std::move(part));
        }
    }
    graphs = std::move(next);
    Topology fresh;
    for (size_t gi = 0; gi < graphs.size(); ++gi) configure(graphs[gi], (int)gi, fresh);
    top = std::move(fresh);
    upload_topology(false);
    return nb;
}

// the slot -> storage map grows by n_new slots, its entries kept
void rdc_system::grow_topology_slots(int n_new) {
    if (n_new <= 0) return;
    int *tloc_new = dalloc<int>(n_top + n_new);
    if (n_top > 0 && d.tloc)
        RDC_CUDA(cudaMemcpyAsync(tloc_new, d.tloc, sizeof(int) * n_top, cudaMemcpyDeviceToDevice, stream));
    sync();
    dfree(d.tloc);
    d.tloc = tloc_new;
    n_top += n_new;
    d.tloc_size = n_top;
}

// EvaluateTopologyReactions (kernels/cpu/src/actions/CPUEvaluateTopologyReactions.cpp:86-475).
// Structural reactions: every topology contributes one event per structural reaction of its type, at the
// rate its rate function gave when the topology was created or last changed (GraphTopology::
// updateReactionRates).  Spatial reactions: the device lists the candidate pairs (k_topology_candidates);
// each pair becomes an event per reaction that matches its particle and topology types in either order,
// within the reaction's radius (a self fusion also needs a graph distance above min_graph_distance and,
// unless the legacy rule is set, above 1).  Events are drawn as algo::performEvents does
// (include/readdy/common/algorithm.h:62-136) -- proportional to rate, without replacement, each with its
// coin u < 1 - exp(-rate dt), an accepted event removing the events that share one of its topologies or its
// free particle -- by exponential clocks E/rate with the coins drawn up front (the same distribution;
// Philox keyed by the ordered ids or the topology's first particle, the call count and the reaction).
// Accepted events are applied in clock order, so a reaction function sees the topologies as the earlier
// events left them: structural ones apply their recipe (a topology that falls apart becomes its
// components, or raises when the reaction expects it connected; Utils.h:52-81,
// StructuralTopologyReaction.cpp:70-130), spatial ones change types, merge graphs, add an edge or take a free
// particle into a topology.  The bonded terms are then derived again from the graphs.  Each spatial pair is
// one candidate; the reference lists a topology-particle pair a second time from the free particle's side
// when that particle's storage index is the lower one.
int64_t rdc_system::evaluate_topology_reactions(double dt) {
    require(dt > 0, "time step must be > 0");
    if (in_callback) throw LogicError("topology reactions cannot be evaluated from a reaction's own function");
    const auto &RS = ctx.spatial_top;
    const uint64_t call = topo_calls++;
    if (topo_counts.size() != RS.size()) topo_counts.assign(RS.size(), 0);
    if (structural_counts.size() != structural.size()) structural_counts.assign(structural.size(), 0);
    if ((RS.empty() && structural.empty()) || graphs.empty()) return 0;
    // structural rates of topologies created or changed since their last evaluation
    if (!structural.empty())
        for (size_t gi = 0; gi < graphs.size(); ++gi) {
            TopGraph &g = graphs[gi];
            if (g.rates_valid) continue;
            g.rates.assign(structural.size(), 0.0);
            for (size_t k = 0; k < structural.size(); ++k)
                if (structural[k].topology_type == g.type) {
                    in_callback = true;
                    const double r = structural[k].rate(structural[k].user, this, (int64_t)gi);
                    in_callback = false;
                    if (!(r >= 0)) throw std::runtime_error("a structural topology reaction's rate function gave a rate "
                                                            "below 0 or not a number");
                    g.rates[k] = r;
                }
            g.rates_valid = true;
        }
    std::vector<TopCandidate> cand;
    if (!RS.empty()) {
        if (!nl_ready) throw LogicError("topology reactions: the neighbor list is not set up");
        const int T = ctx.ntypes;
        std::vector<uint32_t> mask(T, 0u);
        double rmax = 0;
        for (const auto &r : RS) {
            mask[r.t1] |= 1u << r.t2;
            mask[r.t2] |= 1u << r.t1;
            rmax = std::max(rmax, r.radius);
        }
        if (!top_mask_dev) {
            top_mask_dev = dalloc<uint32_t>(MAX_TYPES);
            top_n_dev = dalloc<int>(1);
        }
        RDC_CUDA(cudaMemcpyAsync(top_mask_dev, mask.data(), sizeof(uint32_t) * T, cudaMemcpyHostToDevice, stream));
        const double r2max = rmax * rmax;
        const float r2screen = (float)r2max + 2.0f * band_for(rmax, d.geo.L);
        int nc = 0;
        for (int attempt = 0; attempt < 2; ++attempt) {
            if (cand_cap == 0) {
                cand_cap = 4096;
                cand_dev = dalloc<TopCandidate>(cand_cap);
            }
            launch_topology_candidates(d, top_mask_dev, r2max, r2screen, cand_dev, top_n_dev, cand_cap, stream);
            RDC_CUDA(cudaMemcpyAsync(&nc, top_n_dev, sizeof(int), cudaMemcpyDeviceToHost, stream));
            sync();
            if (nc <= cand_cap) break;
            dfree(cand_dev);
            cand_cap = nc + nc / 2;
            cand_dev = dalloc<TopCandidate>(cand_cap);
        }
        cand.resize(std::min(nc, cand_cap));
        if (!cand.empty())
            RDC_CUDA(cudaMemcpyAsync(cand.data(), cand_dev, sizeof(TopCandidate) * cand.size(), cudaMemcpyDeviceToHost,
                                     stream));
        sync();
    }
    // topology and vertex of every slot
    std::vector<int> slot_graph(n_top, -1), slot_vertex(n_top, -1);
    for (size_t gi = 0; gi < graphs.size(); ++gi)
        for (size_t v = 0; v < graphs[gi].slots.size(); ++v) {
            slot_graph[graphs[gi].slots[v]] = (int)gi;
            slot_vertex[graphs[gi].slots[v]] = (int)v;
        }
    auto graph_of = [&](int slot) { return slot >= 0 && slot < n_top ? slot_graph[slot] : -1; };
    // graph distance (breadth first) between two vertices of one graph, -1 if not connected
    auto graph_distance = [&](const TopGraph &g, int from, int to) {
        const int n = (int)g.slots.size();
        std::vector<std::vector<int>> adj(n);
        for (auto &e : g.edges) {
            adj[e.first].push_back(e.second);
            adj[e.second].push_back(e.first);
        }
        std::vector<int> dist(n, -1);
        std::vector<int> queue{from};
        dist[from] = 0;
        for (size_t q = 0; q < queue.size(); ++q)
            for (int w : adj[queue[q]])
                if (dist[w] < 0) {
                    dist[w] = dist[queue[q]] + 1;
                    queue.push_back(w);
                }
        return dist[to];
    };
    struct Event {
        int r;          // reaction (spatial or structural)
        int c;          // spatial: candidate; structural: -1
        bool swap;      // the candidate's j side is the reaction's first educt
        int g1, g2;     // topologies of the first and second educt (g2 = -1: free particle or structural)
        double clock;
        bool fire;
    };
    std::vector<Event> ev;
    for (size_t gi = 0; gi < graphs.size() && !structural.empty(); ++gi)
        for (int k = 0; k < (int)structural.size(); ++k) {
            const double rate = graphs[gi].rates[k];
            if (!(rate > 0)) continue;
            const U4 u = rng_draw(seed, slot_id[graphs[gi].slots[0]], (uint32_t)k, call, RNG_STRUCTURAL, 0u);
            const double e1 = -std::log(((double)(u.x >> 8) + 0.5) * (1.0 / 16777216.0));
            const bool fire = (((uint64_t)u.y << 32) | u.z) < coin_threshold(rate, dt);
            ev.push_back(Event{k, -1, false, (int)gi, -1, e1 / rate, fire});
        }
    for (int c = 0; c < (int)cand.size(); ++c) {
        const TopCandidate &q = cand[c];
        const int ga = graph_of(q.si), gb = graph_of(q.sj);
        if (ga < 0 && gb < 0) continue;
        const int tta = ga >= 0 ? graphs[ga].type : -1, ttb = gb >= 0 ? graphs[gb].type : -1;
        for (int k = 0; k < (int)RS.size(); ++k) {
            const auto &r = RS[k];
            const bool fwd = r.t1 == q.ti && r.tt1 == tta && r.t2 == q.tj && r.tt2 == ttb;
            const bool bwd = r.t1 == q.tj && r.tt1 == ttb && r.t2 == q.ti && r.tt2 == tta;
            if (!fwd && !bwd) continue;
            const bool swap = !fwd;
            const int g1 = swap ? gb : ga, g2 = swap ? ga : gb;
            if (g1 < 0) continue;
            const bool self = g2 >= 0 && g1 == g2;
            if (self && r.mode != STR_TT_FUSION_ALLOW_SELF) continue;
            if (!(q.d2 < r.radius * r.radius)) continue;
            if (self) {
                const int dgr = graph_distance(graphs[g1], slot_vertex[q.si], slot_vertex[q.sj]);
                if ((dgr != -1 && dgr <= r.min_graph_distance) || (!ctx.legacy_self_fusion && dgr == 1)) continue;
            }
            double rate = r.rate;
            if (r.rate_fn) {  // SpatialTopologyReaction::rate(top1, top2), every candidate, every evaluation
                in_callback = true;
                rate = r.rate_fn(r.rate_user, this, (int64_t)g1, (int64_t)g2);
                in_callback = false;
                if (!(rate >= 0))
                    throw std::runtime_error("a spatial topology reaction's rate function gave a rate below 0 or "
                                             "not a number");
                if (rate == 0) continue;
            }
            const U4 u = rng_draw(seed, std::min(q.idi, q.idj), std::max(q.idi, q.idj), call, RNG_TOPOLOGY, (uint32_t)k);
            const double e1 = -std::log(((double)(u.x >> 8) + 0.5) * (1.0 / 16777216.0));
            const bool fire = (((uint64_t)u.y << 32) | u.z) < coin_threshold(rate, dt);
            ev.push_back(Event{k, c, swap, g1, g2, e1 / rate, fire});
        }
    }
    if (ev.empty()) return 0;
    std::vector<int> order(ev.size());
    for (size_t k = 0; k < ev.size(); ++k) order[k] = (int)k;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ev[a].clock < ev[b].clock; });
    std::vector<char> used(graphs.size(), 0), dead(graphs.size(), 0);
    std::vector<TopGraph> children;  // pieces of topologies that structural reactions split
    std::unordered_set<uint32_t> used_free;
    std::vector<int4> edits;  // (storage index or topology slot, type, new slot or -1, 1: x is a slot)
    std::vector<int2> moved;  // position changes: (storage index or topology slot, 1: x is a slot)
    std::vector<float4> moved_to;
    std::unordered_map<int, int> appended;  // topology slot -> storage index of particles appended now
    auto target_of = [&](int slot) {       // a slot's particle for the edit kernels
        auto it = appended.find(slot);
        return it != appended.end() ? make_int2(it->second, 0) : make_int2(slot, 1);
    };
    auto wrapped = [&](const double p[3]) {  // bcs::fixPosition on the periodic axes
        double q[3] = {p[0], p[1], p[2]};
        for (int a = 0; a < 3; ++a)
            if (ctx.pbc[a]) {
                const double L = (double)d.geo.L[a];
                q[a] -= L * std::floor(q[a] / L + 0.5);
                if (q[a] >= 0.5 * L) q[a] -= L;
            }
        return std::array<double, 3>{q[0], q[1], q[2]};
    };
    int64_t performed = 0;
    // The reference's structural events all carry the second particle index 0 and no second topology, so its
    // eventsDependent (CPUEvaluateTopologyReactions.cpp:459-468) takes any two of them as dependent: one
    // accepted structural event removes every other one of the evaluation
    bool structural_done = false;
    for (int k : order) {
        const Event &e = ev[k];
        if (e.c < 0) {  // structural
            if (used[e.g1] || structural_done) continue;
            if (!e.fire) continue;
            structural_done = true;
            const auto &sr = structural[e.r];
            rdc_recipe recipe;
            in_callback = true;
            sr.reaction(sr.user, this, (int64_t)e.g1, &recipe);
            in_callback = false;
            TopGraph &g = graphs[e.g1];
            for (const auto &op : recipe.ops) {
                const int nv_now = (int)g.slots.size();
                auto vertex = [&](int64_t v) {
                    if (v < 0 || v >= nv_now) throw InvalidArgument("recipe vertex index out of range");
                    return (int)v;
                };
                auto find_edge = [&](int a, int b) {
                    for (size_t x = 0; x < g.edges.size(); ++x)
                        if ((g.edges[x].first == a && g.edges[x].second == b) ||
                            (g.edges[x].first == b && g.edges[x].second == a))
                            return (int)x;
                    return -1;
                };
                switch (op.kind) {
                    case RECIPE_CHANGE_PARTICLE_TYPE: {
                        const int v = vertex(op.a);
                        if (op.type < 0 || op.type >= ctx.ntypes) throw InvalidArgument("particle type out of range");
                        slot_type[g.slots[v]] = op.type;
                        const int2 t = target_of(g.slots[v]);
                        edits.push_back(make_int4(t.x, op.type, -1, t.y));
                        break;
                    }
                    case RECIPE_CHANGE_PARTICLE_POSITION: {
                        const int v = vertex(op.a);
                        const auto q = wrapped(op.pos);
                        moved.push_back(target_of(g.slots[v]));
                        moved_to.push_back(make_float4((float)q[0], (float)q[1], (float)q[2], 0.f));
                        break;
                    }
                    case RECIPE_APPEND_PARTICLE: {  // CPUAppendParticle (CPUTopologyActions.h:112-131)
                        if (op.neighbors.empty()) throw InvalidArgument("recipe: a new particle needs a neighbour");
                        if (op.type < 0 || op.type >= ctx.ntypes) throw InvalidArgument("particle type out of range");
                        std::vector<int> nbrs;
                        for (int64_t x : op.neighbors) nbrs.push_back(vertex(x));
                        const auto q = wrapped(op.pos);
                        const double xyz[3] = {q[0], q[1], q[2]};
                        int c[C_COUNT];
                        read_counters(c);
                        const int slot = n_top;
                        grow_topology_slots(1);
                        uint64_t id = 0;
                        append(1, xyz, &op.type, &slot, &id);
                        appended[slot] = c[C_N_TOTAL];
                        slot_type.push_back(op.type);
                        slot_id.push_back((uint32_t)id);
                        g.slots.push_back(slot);
                        const int nvx = (int)g.slots.size() - 1;
                        for (int nb : nbrs)
                            if (find_edge(nb, nvx) < 0) g.edges.emplace_back(nb, nvx);
                        break;
                    }
                    case RECIPE_ADD_EDGE: {
                        const int a = vertex(op.a), b = vertex(op.b);
                        if (a == b) throw InvalidArgument("recipe: an edge needs two vertices");
                        if (find_edge(a, b) < 0) g.edges.emplace_back(a, b);
                        break;
                    }
                    case RECIPE_REMOVE_EDGE: {
                        const int x = find_edge(vertex(op.a), vertex(op.b));
                        if (x < 0) throw InvalidArgument("recipe: the edge to remove does not exist");
                        g.edges.erase(g.edges.begin() + x);
                        break;
                    }
                    case RECIPE_SEPARATE_VERTEX: {
                        const int v = vertex(op.a);
                        std::vector<std::pair<int, int>> kept;
                        for (auto &x : g.edges)
                            if (x.first != v && x.second != v) kept.push_back(x);
                        g.edges = std::move(kept);
                        break;
                    }
                    case RECIPE_CHANGE_TOPOLOGY_TYPE:
                        if (op.type < 0) throw InvalidArgument("topology type must be >= 0");
                        g.type = op.type;
                        break;
                }
            }
            g.rates_valid = false;
            const int nv = (int)g.slots.size();
            // connected components: a topology that falls apart becomes its pieces (or raises)
            std::vector<std::vector<int>> adj(nv);
            for (auto &x : g.edges) {
                adj[x.first].push_back(x.second);
                adj[x.second].push_back(x.first);
            }
            std::vector<int> comp(nv, -1);
            int ncomp = 0;
            for (int v = 0; v < nv; ++v) {
                if (comp[v] >= 0) continue;
                std::vector<int> stack{v};
                comp[v] = ncomp;
                while (!stack.empty()) {
                    const int u = stack.back();
                    stack.pop_back();
                    for (int w : adj[u])
                        if (comp[w] < 0) {
                            comp[w] = ncomp;
                            stack.push_back(w);
                        }
                }
                ++ncomp;
            }
            if (ncomp > 1) {
                if (sr.expect_connected)
                    throw LogicError("The topology was expected to still be connected after the reaction, but it was "
                                     "not");
                std::vector<TopGraph> parts(ncomp);
                std::vector<int> local(nv);
                for (int v = 0; v < nv; ++v) {
                    local[v] = (int)parts[comp[v]].slots.size();
                    parts[comp[v]].slots.push_back(g.slots[v]);
                    parts[comp[v]].type = g.type;
                }
                for (auto &x : g.edges) parts[comp[x.first]].edges.emplace_back(local[x.first], local[x.second]);
                for (auto &part : parts)
                    if (!(part.slots.size() == 1 && ctx.flavor[slot_type[part.slots[0]]] == FLAVOR_NORMAL))
                        children.push_back(std::move(part));
                dead[e.g1] = 1;
            } else if (nv == 1 && ctx.flavor[slot_type[g.slots[0]]] == FLAVOR_NORMAL) {
                dead[e.g1] = 1;  // a single particle of NORMAL flavor is no topology (Utils.h:70-80)
            }
            used[e.g1] = 1;
            ++structural_counts[e.r];
            ++performed;
            continue;
        }
        const TopCandidate &q = cand[e.c];
        const uint32_t free_id = e.g2 < 0 ? (e.swap ? q.idi : q.idj) : 0;
        if (used[e.g1] || (e.g2 >= 0 && used[e.g2]) || (e.g2 < 0 && used_free.count(free_id))) continue;
        if (!e.fire) continue;  // a rejected event blocks nothing
        const auto &r = RS[e.r];
        // first and second educt: storage index, slot
        const int i1 = e.swap ? q.j : q.i, i2 = e.swap ? q.i : q.j;
        const int s1 = e.swap ? q.sj : q.si, s2 = e.swap ? q.si : q.sj;
        const uint32_t id2 = e.swap ? q.idi : q.idj;
        TopGraph &g1 = graphs[e.g1];
        edits.push_back(make_int4(i1, r.to1, -1, 0));
        slot_type[s1] = r.to1;
        if (r.mode == STR_TP_ENZYMATIC || r.mode == STR_TP_FUSION) {
            if (r.mode == STR_TP_FUSION) {
                const int slot = n_top;
                grow_topology_slots(1);
                slot_type.push_back(r.to2);
                slot_id.push_back(id2);
                g1.slots.push_back(slot);
                g1.edges.emplace_back(slot_vertex[s1], (int)g1.slots.size() - 1);
                edits.push_back(make_int4(i2, r.to2, slot, 0));
            } else {
                edits.push_back(make_int4(i2, r.to2, -1, 0));
            }
            g1.type = r.tto1;
            used_free.insert(free_id);
        } else {
            edits.push_back(make_int4(i2, r.to2, -1, 0));
            slot_type[s2] = r.to2;
            TopGraph &g2 = graphs[e.g2];
            if (e.g1 == e.g2) {  // self fusion: the edge unless present
                const std::pair<int, int> edge(slot_vertex[s1], slot_vertex[s2]);
                bool present = false;
                for (auto &x : g1.edges)
                    present |= (x.first == edge.first && x.second == edge.second) ||
                               (x.first == edge.second && x.second == edge.first);
                if (!present) g1.edges.push_back(edge);
                g1.type = r.tto1;
            } else if (r.mode == STR_TT_ENZYMATIC) {
                g1.type = r.tto1;
                g2.type = r.tto2;
            } else {  // fusion of two topologies: the second joins the first with the new edge
                const int off = (int)g1.slots.size();
                for (int sl : g2.slots) g1.slots.push_back(sl);
                for (auto &x : g2.edges) g1.edges.emplace_back(x.first + off, x.second + off);
                g1.edges.emplace_back(slot_vertex[s1], off + slot_vertex[s2]);
                for (size_t v = 0; v < g2.slots.size(); ++v) slot_vertex[g2.slots[v]] = off + (int)v;
                g1.type = r.tto1;
                g2.slots.clear();
                g2.edges.clear();
                dead[e.g2] = 1;
            }
            g2.rates_valid = false;
            used[e.g2] = 1;
        }
        g1.rates_valid = false;
        used[e.g1] = 1;
        ++topo_counts[e.r];
        ++performed;
    }
    if (performed == 0) return 0;
    if (!moved.empty()) {
        int2 *t_dev = dalloc<int2>(moved.size());
        float4 *p_dev = dalloc<float4>(moved.size());
        RDC_CUDA(cudaMemcpyAsync(t_dev, moved.data(), sizeof(int2) * moved.size(), cudaMemcpyHostToDevice, stream));
        RDC_CUDA(cudaMemcpyAsync(p_dev, moved_to.data(), sizeof(float4) * moved.size(), cudaMemcpyHostToDevice, stream));
        launch_position_edits(d, t_dev, p_dev, (int)moved.size(), stream);
        sync();
        dfree(t_dev);
        dfree(p_dev);
    }
    if (!edits.empty()) {
        if ((int)edits.size() > edit_cap) {
            dfree(edit_dev);
            edit_cap = (int)edits.size() * 2;
            edit_dev = dalloc<int4>(edit_cap);
        }
        RDC_CUDA(cudaMemcpyAsync(edit_dev, edits.data(), sizeof(int4) * edits.size(), cudaMemcpyHostToDevice, stream));
        launch_particle_edits(d, edit_dev, (int)edits.size(), stream);
        sync();
    }
    std::vector<TopGraph> kept;
    for (size_t gi = 0; gi < graphs.size(); ++gi)
        if (!dead[gi]) kept.push_back(std::move(graphs[gi]));
    for (auto &c : children) kept.push_back(std::move(c));
    graphs = std::move(kept);
    Topology fresh;
    for (size_t gi = 0; gi < graphs.size(); ++gi) configure(graphs[gi], (int)gi, fresh);
    top = std::move(fresh);
    // appended particles join the cells (and the slot map) with a sort; moved ones likewise
    upload_topology(!appended.empty() || !moved.empty());
    return performed;
}

void rdc_system::upload_topology(bool sort_new_particles) {
    // CSR: per topology slot, every (kind, role, term) it takes part in
    std::vector<std::vector<int>> per(n_top);
    for (size_t i = 0; i < top.bonds.size(); ++i) {
        per[top.bonds[i].x].push_back((0 << 28) | (0 << 24) | (int)i);
        per[top.bonds[i].y].push_back((0 << 28) | (1 << 24) | (int)i);
    }
    for (size_t i = 0; i < top.angles.size(); ++i) {
        per[top.angles[i].x].push_back((1 << 28) | (0 << 24) | (int)i);
        per[top.angles[i].y].push_back((1 << 28) | (1 << 24) | (int)i);
        per[top.angles[i].z].push_back((1 << 28) | (2 << 24) | (int)i);
    }
    for (size_t i = 0; i < top.dihedrals.size(); ++i) {
        per[top.dihedrals[i].x].push_back((2 << 28) | (0 << 24) | (int)i);
        per[top.dihedrals[i].y].push_back((2 << 28) | (1 << 24) | (int)i);
        per[top.dihedrals[i].z].push_back((2 << 28) | (2 << 24) | (int)i);
        per[top.dihedrals[i].w].push_back((2 << 28) | (3 << 24) | (int)i);
    }
    if (top.bonds.size() >= (1u << 24) || top.angles.size() >= (1u << 24) || top.dihedrals.size() >= (1u << 24))
        throw InvalidArgument("too many bonded terms");
    std::vector<int> off(n_top + 1, 0), terms;
    for (int t = 0; t < n_top; ++t) {
        off[t + 1] = off[t] + (int)per[t].size();
        terms.insert(terms.end(), per[t].begin(), per[t].end());
    }
    // each term's entries in the lists, by role: the term kernel writes its role forces there
    std::vector<int2> bond_at(top.bonds.size());
    std::vector<int4> angle_at(top.angles.size()), dih_at(top.dihedrals.size());
    for (int q = 0; q < (int)terms.size(); ++q) {
        const int kind = terms[q] >> 28, role = (terms[q] >> 24) & 0xf, idx = terms[q] & 0xffffff;
        int *slot = kind == 0 ? &bond_at[idx].x : (kind == 1 ? &angle_at[idx].x : &dih_at[idx].x);
        slot[role] = q;
    }
    auto up = [&](auto *&dptr, const auto &vec) {
        using T = std::remove_reference_t<decltype(*dptr)>;
        dfree(dptr);
        dptr = dalloc<T>(vec.size());
        if (!vec.empty())
            RDC_CUDA(cudaMemcpyAsync(dptr, vec.data(), sizeof(T) * vec.size(), cudaMemcpyHostToDevice, stream));
    };
    up(top_off_dev, off);
    up(top_terms_dev, terms);
    up(bond_idx_dev, top.bonds);
    up(bond_par_dev, top.bond_par);
    up(angle_idx_dev, top.angles);
    up(angle_par_dev, top.angle_par);
    up(dih_idx_dev, top.dihedrals);
    up(dih_par_dev, top.dih_par);
    up(edge_dev, top.edges);
    up(bond_kl_dev, top.bond_kl);
    up(bond_at_dev, bond_at);
    up(angle_at_dev, angle_at);
    up(dih_at_dev, dih_at);
    dfree(term_force_dev);
    term_force_dev = dalloc<float4>(terms.size());
    d.n_bonds = (int)top.bonds.size();
    d.n_angles = (int)top.angles.size();
    d.n_dihedrals = (int)top.dihedrals.size();
    d.bond_at = bond_at_dev;
    d.angle_at = angle_at_dev;
    d.dih_at = dih_at_dev;
    d.term_force = term_force_dev;
    d.n_top = n_top;
    d.top_off = top_off_dev;
    d.top_terms = top_terms_dev;
    d.bond_idx = bond_idx_dev; d.bond_par = bond_par_dev;
    d.angle_idx = angle_idx_dev; d.angle_par = angle_par_dev;
    d.dih_idx = dih_idx_dev; d.dih_par = dih_par_dev;
    // with a neighbour list the new particles join the cells and tloc is rebuilt by a sort
    if (nl_ready && sort_new_particles) {
        launch_bin(d, stream);
        launch_sort(d, forces_live, stream);
        swap_buffers();
    }
    sync();
    invalidate_graph();
}

// One or more loop iterations: integrate, update NL, react, update NL, forces, observables.
void rdc_system::step_sequence(int handler, bool reactions, bool structural, int nsteps) {
    for (int k = 0; k < nsteps; ++k) {
        launch_integrate_bin(d, true, stream);
        launch_sort(d, false, stream);
        swap_buffers();
        if (reactions) {
            launch_events(d, handler, stream);
            launch_resolve_apply(d, handler, stream);
            if (structural) {
                launch_bin(d, stream);
                launch_sort(d, false, stream);
                swap_buffers();
            }
        }
        // runTopologyReactions (SimulationLoop.h:285): host work, so a run with spatial topology reactions
        // is not replayed from a graph
        if (topo_dt > 0) evaluate_topology_reactions(topo_dt);
        launch_forces(d, true, n_top > 0, stream, false);  // energy and virial: once, after the run
        launch_record_counts(d, stream);
    }
}

void rdc_system::run(int64_t n_steps, double dt, int handler, int64_t stride, int64_t *counts, int64_t max_rec,
                     int64_t *n_rec) {
    require(n_steps >= 0, "n_steps must be >= 0");
    require(dt > 0, "time step must be > 0");
    require(handler == H_UNCONTROLLED_APPROXIMATION || handler == H_GILLESPIE, "unknown reaction handler");
    set_dt(dt);
    // runInitialize + runInitializeNeighborList + runForces (SimulationLoop.h:257-272)
    RDC_CUDA(cudaMemsetAsync(d.reaction_counts, 0, sizeof(unsigned long long) * MAX_REACTIONS, stream));
    const double cutoff = std::max(nl_cutoff, ctx.max_cutoff());
    const bool need_nl = cutoff > 0;
    if (need_nl) nl_create(cutoff);
    else {
        nl_ready = true;
        nl_update();
    }
    calculate_forces();
    // observables ring
    dfree(d.counts_ring);
    const bool rec = counts != nullptr && stride > 0 && max_rec > 0;
    d.counts_stride = rec ? (int)std::min<int64_t>(stride, INT_MAX) : 0;
    d.counts_max = rec ? (int)std::min<int64_t>(max_rec, 1 << 24) : 0;
    d.counts_ring = dalloc<unsigned long long>((size_t)std::max(1, d.counts_max) * ctx.ntypes);
    RDC_CUDA(cudaMemsetAsync(d.counts_ring, 0, sizeof(unsigned long long) * std::max(1, d.counts_max) * ctx.ntypes,
                             stream));
    {
        int zero = 0;
        RDC_CUDA(cudaMemcpyAsync(d.counters + C_REC, &zero, sizeof(int), cudaMemcpyHostToDevice, stream));
    }
    uint64_t steps_now[2];
    RDC_CUDA(cudaMemcpyAsync(steps_now, d.step, sizeof(steps_now), cudaMemcpyDeviceToHost, stream));
    sync();
    d.rec_base = steps_now[0];
    if (rec) launch_record_counts(d, stream);  // t = 0
    const bool reactions = !ctx.reactions.empty();
    const bool structural = reactions && ctx.structural_reactions();
    const int swaps = 1 + (structural ? 1 : 0);
    const int per_graph = (swaps % 2 == 0) ? 1 : 2;
    // the device state pointers are baked into the graph; a graph of an even number of buffer
    // swaps starts and ends on the same buffers and can be replayed
    // with spatial topology reactions every step evaluates them on the host, between the reactions and the
    // forces: the steps run one by one
    topo_dt = ((!ctx.spatial_top.empty() || !this->structural.empty()) && !graphs.empty()) ? dt : 0.0;
    const int64_t reps = topo_dt > 0 ? 0 : n_steps / per_graph;
    if (reps > 0) {
        invalidate_graph();
        cudaGraph_t g;
        RDC_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        SysDev saved = d;
        step_sequence(handler, reactions, structural, per_graph);
        const bool same = d.pos == saved.pos;
        RDC_CUDA(cudaStreamEndCapture(stream, &g));
        if (!same) {
            cudaGraphDestroy(g);
            throw std::logic_error("graph capture ended on the alternate buffers");
        }
        RDC_CUDA(cudaGraphInstantiate(&graph, g, 0));
        cudaGraphDestroy(g);
        for (int64_t r = 0; r < reps; ++r) RDC_CUDA(cudaGraphLaunch(graph, stream));
    }
    const int64_t rest = n_steps - reps * per_graph;
    if (topo_dt > 0) {
        for (int64_t k = 0; k < rest; ++k) step_sequence(handler, reactions, structural, 1);
        invalidate_graph();
    } else if (rest > 0) {
        step_sequence(handler, reactions, structural, (int)rest);
    }
    topo_dt = 0;
    // the energy and virial of the last force calculation (its per-block partials are still in place)
    if (n_steps > 0) launch_force_finals(d, n_top > 0, stream);
    forces_live = true;
    sync();
    check_status();
    if (rec) {
        int c[C_COUNT];
        read_counters(c);
        const int nr = std::min(c[C_REC], d.counts_max);
        std::vector<unsigned long long> h((size_t)nr * ctx.ntypes);
        if (nr > 0)
            RDC_CUDA(cudaMemcpyAsync(h.data(), d.counts_ring, sizeof(unsigned long long) * h.size(),
                                     cudaMemcpyDeviceToHost, stream));
        sync();
        for (size_t i = 0; i < h.size(); ++i) counts[i] = (int64_t)h[i];
        if (n_rec) *n_rec = nr;
    } else if (n_rec) {
        *n_rec = 0;
    }
    d.counts_stride = 0;
}

// ---------------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------------
extern "C" {

const char *rdc_last_error(void) { return g_err.c_str(); }
int rdc_version(void) { return 1000; }
const char *rdc_kernel_name(void) { return "CUDA"; }

int rdc_set_device(int device) {
    return guarded([&] {
        int n = 0;
        RDC_CUDA(cudaGetDeviceCount(&n));
        require(device >= 0 && device < n, "device index out of range");
        RDC_CUDA(cudaSetDevice(device));
    });
}

int rdc_context_create(rdc_context **out, const double box[3], const int periodic[3], double kbt, int n_types,
                       const double *diffusion) {
    return guarded([&] {
        require(out && box && periodic && diffusion, "null argument");
        require(n_types > 0 && n_types <= MAX_TYPES, "n_types must be in [1, 32]");
        require(kbt > 0, "kBT must be > 0");
        for (int d = 0; d < 3; ++d) require(box[d] > 0, "box edges must be > 0");
        auto c = std::make_unique<rdc_context>();
        for (int d = 0; d < 3; ++d) {
            c->d.box[d] = (double)(float)box[d];
            c->d.pbc[d] = periodic[d] ? 1 : 0;
        }
        c->d.kbt = kbt;
        c->d.ntypes = n_types;
        c->d.D.assign(diffusion, diffusion + n_types);
        c->d.flavor.assign(n_types, FLAVOR_NORMAL);
        for (double D : c->d.D) require(D >= 0, "diffusion constants must be >= 0");
        *out = c.release();
    });
}
int rdc_context_destroy(rdc_context *ctx) {
    delete ctx;
    return RDC_OK;
}
int rdc_context_set_particle_flavor(rdc_context *ctx, int type, int flavor) {
    return guarded([&] {
        require(ctx != nullptr, "null context");
        require(type >= 0 && type < ctx->d.ntypes, "particle type out of range");
        require(flavor == FLAVOR_NORMAL || flavor == FLAVOR_TOPOLOGY || flavor == FLAVOR_MEMBRANE,
                "flavor must be NORMAL (0), TOPOLOGY (1) or MEMBRANE (2)");
        ctx->d.flavor[type] = flavor;
    });
}
int rdc_context_set_record_virial(rdc_context *ctx, int record) {
    return guarded([&] {
        require(ctx != nullptr, "null context");
        ctx->d.record_virial = record != 0;
    });
}
int rdc_context_max_cutoff(const rdc_context *ctx, double *cutoff) {
    return guarded([&] {
        require(ctx && cutoff, "null argument");
        *cutoff = ctx->d.max_cutoff();
    });
}

static void check_types(const rdc_context *ctx, std::initializer_list<int> ts) {
    require(ctx != nullptr, "null context");
    for (int t : ts) require(t >= 0 && t < ctx->d.ntypes, "particle type out of range");
}

static void add_o1(rdc_context *ctx, int type, int kind, int inclusion, double k, const double *a, const double *b,
                   double radius, double length, double height, double width) {
    HostO1 h{type, kind, inclusion ? 1 : 0, k, {0, 0, 0}, {0, 0, 0}, radius, length, height, width};
    for (int d = 0; d < 3; ++d) {
        h.a[d] = a[d];
        if (b) h.b[d] = b[d];
    }
    ctx->d.o1pots.push_back(h);
}
int rdc_context_add_box(rdc_context *ctx, int type, double k, const double origin[3], const double extent[3],
                        int inclusion) {
    return guarded([&] {
        check_types(ctx, {type});
        require(origin && extent, "null argument");
        add_o1(ctx, type, O1_BOX, inclusion, k, origin, extent, 0, 0, 0, 0);
    });
}
int rdc_context_add_sphere(rdc_context *ctx, int type, double k, const double origin[3], double radius, int inclusion) {
    return guarded([&] {
        check_types(ctx, {type});
        require(origin != nullptr, "null argument");
        add_o1(ctx, type, O1_SPHERE, inclusion, k, origin, nullptr, radius, 0, 0, 0);
    });
}
int rdc_context_add_capsule(rdc_context *ctx, int type, double k, const double center[3], const double direction[3],
                            double length, double radius, int inclusion) {
    return guarded([&] {
        check_types(ctx, {type});
        require(center && direction, "null argument");
        require(direction[0] != 0 || direction[1] != 0 || direction[2] != 0, "capsule direction must be nonzero");
        add_o1(ctx, type, O1_CAPSULE, inclusion, k, center, direction, radius, length, 0, 0);
    });
}
int rdc_context_add_spherical_barrier(rdc_context *ctx, int type, double height, double width, const double origin[3],
                                      double radius) {
    return guarded([&] {
        check_types(ctx, {type});
        require(origin != nullptr, "null argument");
        require(width > 0, "spherical barrier width must be > 0");
        require(!(width > radius), "SphericalBarrier must have a radius larger than its width");  // Potentials.cpp:89-91
        add_o1(ctx, type, O1_SPHERICAL_BARRIER, 1, 0, origin, nullptr, radius, 0, height, width);
    });
}
int rdc_context_add_cylinder(rdc_context *ctx, int type, double k, const double origin[3], const double normal[3],
                             double radius, int inclusion) {
    return guarded([&] {
        check_types(ctx, {type});
        require(origin && normal, "null argument");
        require(normal[0] != 0 || normal[1] != 0 || normal[2] != 0, "cylinder normal must be nonzero");
        add_o1(ctx, type, O1_CYLINDER, inclusion, k, origin, normal, radius, 0, 0, 0);
    });
}

int rdc_context_add_harmonic_repulsion(rdc_context *ctx, int t1, int t2, double k, double d) {
    return guarded([&] {
        check_types(ctx, {t1, t2});
        require(d > 0, "interaction distance must be > 0");
        HostPot h{t1, t2, {}, d};
        h.pot.kind = POT_HARMONIC_REPULSION;
        h.pot.p[0] = (float)k;
        h.pot.p[1] = (float)d;
        split_ff(d * d, h.pot.p[2], h.pot.p[3]);
        h.pot.cutoff2 = d * d;
        h.pot.cutoff2f = (float)h.pot.cutoff2;
        ctx->d.pots.push_back(h);
    });
}
int rdc_context_add_weak_interaction_piecewise_harmonic(rdc_context *ctx, int t1, int t2, double k, double d0,
                                                        double depth, double rc) {
    return guarded([&] {
        check_types(ctx, {t1, t2});
        require(rc > d0 && d0 >= 0, "need 0 <= desired distance < no-interaction distance");
        HostPot h{t1, t2, {}, rc};
        h.pot.kind = POT_WEAK_PIECEWISE_HARMONIC;
        h.pot.p[0] = (float)k; h.pot.p[1] = (float)d0; h.pot.p[2] = (float)depth; h.pot.p[3] = (float)rc;
        split_ff(d0 * d0, h.pot.p[4], h.pot.p[5]);
        split_ff(rc * rc, h.pot.p[6], h.pot.p[7]);
        const double mid = d0 + 0.5 * (rc - d0);
        h.pot.p[8] = (float)(mid * mid);
        h.pot.cutoff2 = rc * rc;
        h.pot.cutoff2f = (float)h.pot.cutoff2;
        ctx->d.pots.push_back(h);
    });
}
int rdc_context_add_lennard_jones(rdc_context *ctx, int t1, int t2, unsigned m, unsigned n, double cutoff, int shift,
                                  double epsilon, double sigma) {
    return guarded([&] {
        check_types(ctx, {t1, t2});
        // Potentials.cpp:163-166
        if (m <= n)
            throw InvalidArgument("When constructing the LJ potential, the first exponent m=" + std::to_string(m) +
                                  " was not greater than the second exponent n=" + std::to_string(n) + "!");
        require(cutoff > 0 && sigma > 0, "LJ cutoff and sigma must be > 0");
        require(m <= 64, "LJ exponent too large");
        const double dm = m, dn = n;
        const double rmin = sigma * std::pow(dn / dm, 1. / (dn - dm));  // Potentials.cpp:167-170
        const double kk = -epsilon / (std::pow(sigma / rmin, dm) - std::pow(sigma / rmin, dn));
        const double eshift = shift ? kk * (std::pow(sigma / cutoff, dm) - std::pow(sigma / cutoff, dn)) : 0.0;
        HostPot h{t1, t2, {}, cutoff};
        h.pot.kind = POT_LENNARD_JONES;
        h.pot.p[0] = (float)m; h.pot.p[1] = (float)n; h.pot.p[2] = (float)cutoff; h.pot.p[3] = shift ? 1.f : 0.f;
        h.pot.p[4] = (float)epsilon; h.pot.p[5] = (float)(sigma * sigma); h.pot.p[6] = (float)kk;
        h.pot.p[7] = (float)eshift;
        h.pot.p[8] = (m == 12 && n == 6) ? 1.f : 0.f;
        split_ff(std::pow(sigma, 6.0), h.pot.p[9], h.pot.p[10]);
        h.pot.cutoff2 = cutoff * cutoff;
        h.pot.cutoff2f = (float)h.pot.cutoff2;
        ctx->d.pots.push_back(h);
    });
}
int rdc_context_add_screened_electrostatics(rdc_context *ctx, int t1, int t2, double C, double kappa, double D,
                                            double sigma, unsigned exponent, double cutoff) {
    return guarded([&] {
        check_types(ctx, {t1, t2});
        // Potentials.cpp:188-201
        if (kappa < 0) throw InvalidArgument("inverse screening depth must be positive!");
        if (D < 0) throw InvalidArgument("repulsion strength must be positive!");
        if (sigma < 0) throw InvalidArgument("repulsion distance must be positive!");
        if (cutoff < 0) throw InvalidArgument("cutoff must be positive!");
        require(exponent <= 64, "exponent too large");
        HostPot h{t1, t2, {}, cutoff};
        h.pot.kind = POT_SCREENED_ELECTROSTATICS;
        h.pot.p[0] = (float)C; h.pot.p[1] = (float)kappa; h.pot.p[2] = (float)D; h.pot.p[3] = (float)sigma;
        h.pot.p[4] = (float)exponent;
        h.pot.cutoff2 = cutoff * cutoff;
        h.pot.cutoff2f = (float)h.pot.cutoff2;
        ctx->d.pots.push_back(h);
    });
}

static int add_reaction(rdc_context *ctx, HostReaction r, int *id) {
    return guarded([&] {
        require(ctx != nullptr, "null context");
        require((int)ctx->d.reactions.size() < MAX_REACTIONS, "too many reactions");
        require(r.rate >= 0, "reaction rate must be >= 0");
        for (int k = 0; k < r.n_educts; ++k) check_types(ctx, {r.educt[k]});
        for (int k = 0; k < r.n_products; ++k) check_types(ctx, {r.product[k]});
        const double sum = r.w1 + r.w2;  // Fusion.h:62-68, Fission.h:64-70
        if (sum != 1 && sum > 0) {
            r.w1 /= sum;
            r.w2 /= sum;
        }
        ctx->d.reactions.push_back(r);
        if (id) *id = (int)ctx->d.reactions.size() - 1;
    });
}
int rdc_context_add_conversion(rdc_context *ctx, int from, int to, double rate, int *id) {
    return add_reaction(ctx, HostReaction{R_CONVERSION, 1, 1, {from, 0}, {to, 0}, rate, 0, 0, .5, .5}, id);
}
int rdc_context_add_decay(rdc_context *ctx, int from, double rate, int *id) {
    return add_reaction(ctx, HostReaction{R_DECAY, 1, 0, {from, 0}, {0, 0}, rate, 0, 0, .5, .5}, id);
}
int rdc_context_add_fusion(rdc_context *ctx, int from1, int from2, int to, double rate, double ed, double w1, double w2,
                           int *id) {
    if (!(ed > 0)) {
        g_err = "educt distance must be > 0";
        return RDC_ERR_INVALID_ARGUMENT;
    }
    return add_reaction(ctx, HostReaction{R_FUSION, 2, 1, {from1, from2}, {to, 0}, rate, ed, 0, w1, w2}, id);
}
int rdc_context_add_fission(rdc_context *ctx, int from, int to1, int to2, double rate, double pd, double w1, double w2,
                            int *id) {
    return add_reaction(ctx, HostReaction{R_FISSION, 1, 2, {from, 0}, {to1, to2}, rate, 0, pd, w1, w2}, id);
}
int rdc_context_add_enzymatic(rdc_context *ctx, int catalyst, int from, int to, double rate, double ed, int *id) {
    if (!(ed > 0)) {
        g_err = "educt distance must be > 0";
        return RDC_ERR_INVALID_ARGUMENT;
    }
    return add_reaction(ctx, HostReaction{R_ENZYMATIC, 2, 2, {from, catalyst}, {to, catalyst}, rate, ed, 0, .5, .5},
                        id);
}

int rdc_context_configure_harmonic_bond(rdc_context *ctx, int t1, int t2, double k, double l0) {
    return guarded([&] {
        check_types(ctx, {t1, t2});
        ctx->d.bonds.push_back(BondCfg{t1, t2, k, l0});
    });
}
int rdc_context_configure_harmonic_angle(rdc_context *ctx, int t1, int t2, int t3, double k, double theta0) {
    return guarded([&] {
        check_types(ctx, {t1, t2, t3});
        ctx->d.angles.push_back(AngleCfg{t1, t2, t3, k, theta0});
    });
}
int rdc_context_configure_cosine_dihedral(rdc_context *ctx, int t1, int t2, int t3, int t4, double k, double mult,
                                          double phi0) {
    return guarded([&] {
        check_types(ctx, {t1, t2, t3, t4});
        // TorsionPotential.h:63-67
        if (phi0 > M_PI || phi0 < -M_PI)
            throw InvalidArgument("the equilibrium angle should be within [-pi, pi], but was " + std::to_string(phi0));
        ctx->d.dihedrals.push_back(DihedralCfg{t1, t2, t3, t4, k, mult, phi0});
    });
}

int rdc_context_add_spatial_topology_reaction(rdc_context *ctx, int mode, int type1, int topology_type1, int type2,
                                              int topology_type2, int type_to1, int topology_type_to1, int type_to2,
                                              int topology_type_to2, double rate, double radius,
                                              int min_graph_distance, int *reaction_id) {
    return guarded([&] {
        check_types(ctx, {type1, type2, type_to1, type_to2});
        require(mode >= STR_TT_ENZYMATIC && mode <= STR_TP_FUSION, "unknown spatial topology reaction mode");
        const bool tp = mode == STR_TP_ENZYMATIC || mode == STR_TP_FUSION;
        require(topology_type1 >= 0 && topology_type_to1 >= 0, "topology types must be >= 0");
        require(tp ? topology_type2 == -1 : (topology_type2 >= 0 && topology_type_to2 >= 0),
                "topology-particle reactions take topology_type2 = -1, topology-topology ones a type >= 0");
        // SpatialTopologyReaction.h:88-91, TopologyRegistry.cpp:238-242
        if (!(rate > 0)) throw InvalidArgument("The rate of a spatial topology reaction should always be positive");
        if (!(radius > 0)) throw InvalidArgument("The radius of a spatial topology reaction should always be positive");
        require(min_graph_distance >= 0, "min_graph_distance must be >= 0");
        ctx->d.spatial_top.push_back(SpatialTopReaction{mode, type1, topology_type1, type2, topology_type2, type_to1,
                                                        topology_type_to1, type_to2, tp ? -1 : topology_type_to2, rate,
                                                        radius, min_graph_distance});
        if (reaction_id) *reaction_id = (int)ctx->d.spatial_top.size() - 1;
    });
}
int rdc_context_set_spatial_topology_rate_function(rdc_context *ctx, int reaction_id, rdc_spatial_rate_fn rate,
                                                   void *user) {
    return guarded([&] {
        require(ctx && rate, "null argument");
        require(reaction_id >= 0 && reaction_id < (int)ctx->d.spatial_top.size(), "unknown spatial reaction id");
        auto &r = ctx->d.spatial_top[reaction_id];
        require(r.mode == STR_TT_ENZYMATIC || r.mode == STR_TT_FUSION || r.mode == STR_TT_FUSION_ALLOW_SELF,
                "rate functions apply to topology-topology reactions (the reference's rate() throws for "
                "topology-particle ones)");
        r.rate_fn = rate;
        r.rate_user = user;
    });
}
int rdc_context_set_legacy_topology_self_fusion(rdc_context *ctx, int legacy) {
    return guarded([&] {
        require(ctx != nullptr, "null context");
        ctx->d.legacy_self_fusion = legacy != 0;
    });
}

int rdc_system_create(rdc_system **out, const rdc_context *ctx, uint64_t seed) {
    return guarded([&] {
        require(out && ctx, "null argument");
        // TopologyRegistry::validateSpatialReaction (TopologyRegistry.cpp:243-253)
        for (const auto &r : ctx->d.spatial_top)
            if (ctx->d.flavor[r.t1] != FLAVOR_TOPOLOGY && ctx->d.flavor[r.t2] != FLAVOR_TOPOLOGY)
                throw InvalidArgument("At least one of the educt types of a spatial topology reaction needs to be "
                                      "topology flavored");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            throw CudaError("no CUDA device available");
        }
        auto s = std::make_unique<rdc_system>();
        s->init(ctx->d, seed);
        *out = s.release();
    });
}
int rdc_system_destroy(rdc_system *s) {
    if (s) {
        if (s->stream) cudaStreamSynchronize(s->stream);
        delete s;
    }
    return RDC_OK;
}

int rdc_add_particles(rdc_system *s, int64_t n, const double *pos, const int *types, uint64_t *ids_out) {
    return guarded([&] {
        require(s != nullptr && (n == 0 || (pos && types)), "null argument");
        require(n >= 0, "n must be >= 0");
        s->append(n, pos, types, nullptr, ids_out);
        s->invalidate_graph();
    });
}
int rdc_add_topology(rdc_system *s, int64_t n, const double *pos, const int *types, int64_t n_edges,
                     const int64_t *edges, uint64_t *ids_out) {
    return rdc_add_topology_typed(s, 0, n, pos, types, n_edges, edges, ids_out);
}
int rdc_add_topology_typed(rdc_system *s, int topology_type, int64_t n, const double *pos, const int *types,
                           int64_t n_edges, const int64_t *edges, uint64_t *ids_out) {
    return guarded([&] {
        require(s && pos && types && (n_edges == 0 || edges), "null argument");
        s->add_topology(topology_type, n, pos, types, n_edges, edges, ids_out);
    });
}
int rdc_break_bonds(rdc_system *s, double time_step, int n_pairs, const int *type1, const int *type2,
                    const double *threshold_energy, const double *rate, int64_t *n_broken) {
    return guarded([&] {
        require(s && (n_pairs == 0 || (type1 && type2 && threshold_energy && rate)), "null argument");
        const int64_t nb = s->break_bonds(time_step, n_pairs, type1, type2, threshold_energy, rate);
        if (n_broken) *n_broken = nb;
    });
}
int rdc_evaluate_topology_reactions(rdc_system *s, double time_step, int64_t *n_performed) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        const int64_t n = s->evaluate_topology_reactions(time_step);
        if (n_performed) *n_performed = n;
    });
}
int rdc_add_structural_topology_reaction(rdc_system *s, int topology_type, rdc_topology_rate_fn rate,
                                         rdc_topology_recipe_fn reaction, void *user, int expect_connected,
                                         int *reaction_id) {
    return guarded([&] {
        require(s && rate && reaction, "null argument");
        require(topology_type >= 0, "topology type must be >= 0");
        if (s->in_callback) throw LogicError("reactions cannot be added from a reaction's own function");
        s->structural.push_back(StructuralReaction{topology_type, rate, reaction, user, expect_connected != 0});
        for (auto &g : s->graphs) g.rates_valid = false;
        if (reaction_id) *reaction_id = (int)s->structural.size() - 1;
    });
}
int rdc_get_structural_reaction_counts(rdc_system *s, int n, int64_t *counts) {
    return guarded([&] {
        require(s && (n == 0 || counts), "null argument");
        require(n == (int)s->structural.size(), "n must equal the number of structural topology reactions");
        for (int k = 0; k < n; ++k)
            counts[k] = k < (int)s->structural_counts.size() ? (int64_t)s->structural_counts[k] : 0;
    });
}
static int recipe_op(rdc_recipe *r, RecipeOp op) {
    return guarded([&] {
        require(r != nullptr, "null recipe");
        r->ops.push_back(op);
    });
}
int rdc_recipe_change_particle_type(rdc_recipe *r, int64_t vertex, int type) {
    return recipe_op(r, RecipeOp{RECIPE_CHANGE_PARTICLE_TYPE, vertex, 0, type});
}
int rdc_recipe_add_edge(rdc_recipe *r, int64_t v1, int64_t v2) { return recipe_op(r, RecipeOp{RECIPE_ADD_EDGE, v1, v2, 0}); }
int rdc_recipe_remove_edge(rdc_recipe *r, int64_t v1, int64_t v2) {
    return recipe_op(r, RecipeOp{RECIPE_REMOVE_EDGE, v1, v2, 0});
}
int rdc_recipe_separate_vertex(rdc_recipe *r, int64_t vertex) {
    return recipe_op(r, RecipeOp{RECIPE_SEPARATE_VERTEX, vertex, 0, 0});
}
int rdc_recipe_change_topology_type(rdc_recipe *r, int type) {
    return recipe_op(r, RecipeOp{RECIPE_CHANGE_TOPOLOGY_TYPE, 0, 0, type});
}
int rdc_recipe_change_particle_position(rdc_recipe *r, int64_t vertex, const double *pos3) {
    return guarded([&] {
        require(r && pos3, "null argument");
        r->ops.push_back(RecipeOp{RECIPE_CHANGE_PARTICLE_POSITION, vertex, 0, 0, {}, {pos3[0], pos3[1], pos3[2]}});
    });
}
int rdc_recipe_append_particle(rdc_recipe *r, int64_t n_neighbors, const int64_t *neighbors, int type,
                               const double *pos3) {
    return guarded([&] {
        require(r && pos3 && (n_neighbors == 0 || neighbors), "null argument");
        require(n_neighbors >= 0, "n_neighbors must be >= 0");
        r->ops.push_back(RecipeOp{RECIPE_APPEND_PARTICLE, 0, 0, type,
                                  std::vector<int64_t>(neighbors, neighbors + n_neighbors), {pos3[0], pos3[1], pos3[2]}});
    });
}
int rdc_get_topology(rdc_system *s, int64_t k, int *topology_type, int64_t capacity, uint64_t *ids, int *types,
                     int64_t *n_vertices, int64_t capacity_edges, int64_t *edges2, int64_t *n_edges) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        require(k >= 0 && k < (int64_t)s->graphs.size(), "topology index out of range");
        const TopGraph &g = s->graphs[k];
        if (topology_type) *topology_type = g.type;
        if (n_vertices) *n_vertices = (int64_t)g.slots.size();
        if (n_edges) *n_edges = (int64_t)g.edges.size();
        if ((ids || types) && capacity < (int64_t)g.slots.size())
            throw CapacityError("output capacity too small for the topology's particles");
        if (edges2 && capacity_edges < (int64_t)g.edges.size())
            throw CapacityError("output capacity too small for the topology's edges");
        for (size_t v = 0; v < g.slots.size(); ++v) {
            if (ids) ids[v] = s->slot_id[g.slots[v]];
            if (types) types[v] = s->slot_type[g.slots[v]];
        }
        if (edges2)
            for (size_t e = 0; e < g.edges.size(); ++e) {
                edges2[2 * e] = g.edges[e].first;
                edges2[2 * e + 1] = g.edges[e].second;
            }
    });
}
int rdc_get_topology_positions(rdc_system *s, int64_t k, int64_t capacity, double *positions3) {
    return guarded([&] {
        require(s && positions3, "null argument");
        require(k >= 0 && k < (int64_t)s->graphs.size(), "topology index out of range");
        const TopGraph &g = s->graphs[k];
        const int n = (int)g.slots.size();
        if (capacity < n) throw CapacityError("output capacity too small for the topology's particles");
        int *slots_dev = dalloc<int>(n);
        float4 *out_dev = dalloc<float4>(n);
        RDC_CUDA(cudaMemcpyAsync(slots_dev, g.slots.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s->stream));
        launch_gather_slots(s->d, slots_dev, n, out_dev, s->stream);
        std::vector<float4> h(n);
        RDC_CUDA(cudaMemcpyAsync(h.data(), out_dev, sizeof(float4) * n, cudaMemcpyDeviceToHost, s->stream));
        s->sync();
        dfree(slots_dev);
        dfree(out_dev);
        for (int v = 0; v < n; ++v) {
            positions3[3 * v] = h[v].x;
            positions3[3 * v + 1] = h[v].y;
            positions3[3 * v + 2] = h[v].z;
        }
    });
}
int rdc_get_topology_reaction_counts(rdc_system *s, int n, int64_t *counts) {
    return guarded([&] {
        require(s && (n == 0 || counts), "null argument");
        require(n == (int)s->ctx.spatial_top.size(), "n must equal the number of spatial topology reactions");
        for (int k = 0; k < n; ++k) counts[k] = k < (int)s->topo_counts.size() ? (int64_t)s->topo_counts[k] : 0;
    });
}
int rdc_get_topologies(rdc_system *s, int64_t capacity_topologies, int *topology_types, int64_t *offsets,
                       int64_t capacity_ids, uint64_t *ids, int64_t *n_topologies, int64_t *n_ids) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        const int64_t nt = (int64_t)s->graphs.size();
        int64_t total = 0;
        for (const auto &g : s->graphs) total += (int64_t)g.slots.size();
        if (n_topologies) *n_topologies = nt;
        if (n_ids) *n_ids = total;
        if (nt > capacity_topologies || total > capacity_ids)
            throw CapacityError("output capacity too small for the topologies");
        int64_t at = 0;
        for (int64_t k = 0; k < nt; ++k) {
            const auto &g = s->graphs[k];
            if (topology_types) topology_types[k] = g.type;
            if (offsets) offsets[k] = at;
            for (int slot : g.slots) {
                if (ids) ids[at] = s->slot_id[slot];
                ++at;
            }
        }
        if (offsets) offsets[nt] = at;
    });
}
int rdc_get_topology_edges(rdc_system *s, int64_t capacity_topologies, int64_t *offsets, int64_t capacity_edges,
                           uint64_t *edges2, int64_t *n_topologies, int64_t *n_edges) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        const int64_t nt = (int64_t)s->graphs.size();
        int64_t total = 0;
        for (const auto &g : s->graphs) total += (int64_t)g.edges.size();
        if (n_topologies) *n_topologies = nt;
        if (n_edges) *n_edges = total;
        if (nt > capacity_topologies || total > capacity_edges)
            throw CapacityError("output capacity too small for the topology edges");
        int64_t at = 0;
        for (int64_t k = 0; k < nt; ++k) {
            const auto &g = s->graphs[k];
            if (offsets) offsets[k] = at;
            for (const auto &e : g.edges) {
                if (edges2) {
                    edges2[2 * at] = s->slot_id[g.slots[e.first]];
                    edges2[2 * at + 1] = s->slot_id[g.slots[e.second]];
                }
                ++at;
            }
        }
        if (offsets) offsets[nt] = at;
    });
}
int rdc_get_n_particles(rdc_system *s, int64_t *n) {
    return guarded([&] {
        require(s && n, "null argument");
        // active = storage minus the dead still awaiting a sort
        launch_count_types(s->d, s->count_buf, s->stream);
        std::vector<unsigned long long> h(s->ctx.ntypes);
        RDC_CUDA(cudaMemcpyAsync(h.data(), s->count_buf, sizeof(unsigned long long) * h.size(),
                                 cudaMemcpyDeviceToHost, s->stream));
        s->sync();
        int64_t k = 0;
        for (auto v : h) k += (int64_t)v;
        *n = k;
    });
}

static void fetch(rdc_system *s, std::vector<float4> &p, std::vector<uint32_t> &id, std::vector<float4> *f) {
    int c[C_COUNT];
    s->read_counters(c);
    const int n = c[C_N_TOTAL];
    p.resize(n);
    id.resize(n);
    if (n > 0) {
        RDC_CUDA(cudaMemcpyAsync(p.data(), s->d.pos, sizeof(float4) * n, cudaMemcpyDeviceToHost, s->stream));
        RDC_CUDA(cudaMemcpyAsync(id.data(), s->d.id, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s->stream));
        if (f) {
            f->resize(n);
            RDC_CUDA(cudaMemcpyAsync(f->data(), s->d.force, sizeof(float4) * n, cudaMemcpyDeviceToHost, s->stream));
        }
    }
    s->sync();
}

int rdc_get_particles(rdc_system *s, int64_t cap, double *pos, int *types, uint64_t *ids, int64_t *n_out) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        std::vector<float4> p;
        std::vector<uint32_t> id;
        fetch(s, p, id, nullptr);
        int64_t k = 0;
        for (size_t i = 0; i < p.size(); ++i) {
            int t;
            std::memcpy(&t, &p[i].w, 4);
            if (t < 0) continue;
            if (k < cap) {
                if (pos) { pos[3 * k] = p[i].x; pos[3 * k + 1] = p[i].y; pos[3 * k + 2] = p[i].z; }
                if (types) types[k] = t;
                if (ids) ids[k] = id[i];
            }
            ++k;
        }
        if (n_out) *n_out = k;
        if (k > cap) throw CapacityError("output capacity too small for the particles");
    });
}
int rdc_get_forces(rdc_system *s, int64_t cap, double *forces, uint64_t *ids, int64_t *n_out) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        std::vector<float4> p, f;
        std::vector<uint32_t> id;
        fetch(s, p, id, &f);
        int64_t k = 0;
        for (size_t i = 0; i < p.size(); ++i) {
            int t;
            std::memcpy(&t, &p[i].w, 4);
            if (t < 0) continue;
            if (k < cap) {
                if (forces) { forces[3 * k] = f[i].x; forces[3 * k + 1] = f[i].y; forces[3 * k + 2] = f[i].z; }
                if (ids) ids[k] = id[i];
            }
            ++k;
        }
        if (n_out) *n_out = k;
        if (k > cap) throw CapacityError("output capacity too small for the particles");
    });
}
int rdc_get_particle_energies(rdc_system *s, int64_t cap, double *energies, uint64_t *ids, int64_t *n_out) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        std::vector<float4> p, f;
        std::vector<uint32_t> id;
        fetch(s, p, id, &f);
        int64_t k = 0;
        for (size_t i = 0; i < p.size(); ++i) {
            int t;
            std::memcpy(&t, &p[i].w, 4);
            if (t < 0) continue;
            if (k < cap) {
                if (energies) energies[k] = f[i].w;
                if (ids) ids[k] = id[i];
            }
            ++k;
        }
        if (n_out) *n_out = k;
        if (k > cap) throw CapacityError("output capacity too small for the particles");
    });
}
int rdc_set_record_virial(rdc_system *s, int record) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        s->set_record_virial(record != 0);
    });
}
int rdc_get_virial(rdc_system *s, double *virial9) {
    return guarded([&] {
        require(s && virial9, "null argument");
        for (int k = 0; k < 9; ++k) virial9[k] = 0.0;
        if (s->d.virial)
            RDC_CUDA(cudaMemcpyAsync(virial9, s->d.virial, sizeof(double) * 9, cudaMemcpyDeviceToHost, s->stream));
        s->sync();
    });
}
int rdc_get_energy(rdc_system *s, double *e) {
    return guarded([&] {
        require(s && e, "null argument");
        RDC_CUDA(cudaMemcpyAsync(e, s->d.energy, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        s->sync();
    });
}
int rdc_get_particle_steps(rdc_system *s, uint64_t *particle_steps) {
    return guarded([&] {
        require(s && particle_steps, "null argument");
        unsigned long long v = 0;
        RDC_CUDA(cudaMemcpyAsync(&v, s->d.step + 2, sizeof(v), cudaMemcpyDeviceToHost, s->stream));
        s->sync();
        *particle_steps = v;
    });
}
int rdc_count_types(rdc_system *s, int64_t *counts) {
    return guarded([&] {
        require(s && counts, "null argument");
        launch_count_types(s->d, s->count_buf, s->stream);
        std::vector<unsigned long long> h(s->ctx.ntypes);
        RDC_CUDA(cudaMemcpyAsync(h.data(), s->count_buf, sizeof(unsigned long long) * h.size(),
                                 cudaMemcpyDeviceToHost, s->stream));
        s->sync();
        for (int t = 0; t < s->ctx.ntypes; ++t) counts[t] = (int64_t)h[t];
    });
}
}  // extern "C"

namespace {
// bit mask of the listed particle types (each in range)
static_assert(MAX_TYPES <= 32, "type selections are 32-bit masks");
uint32_t type_mask(const rdc_system *s, int n, const int *types) {
    uint32_t m = 0;
    for (int k = 0; k < n; ++k) {
        require(types[k] >= 0 && types[k] < s->ctx.ntypes, "particle type out of range");
        m |= 1u << types[k];
    }
    return m;
}

// bin counts of one observable: borders uploaded, counters zeroed, `launch` run, counts read back
template <typename Launch>
std::vector<unsigned long long> observe_bins(rdc_system *s, int n_borders, const double *borders, Launch launch) {
    require(n_borders >= 2, "at least two bin borders");
    require(std::is_sorted(borders, borders + n_borders), "bin borders must be ascending");
    double *bd = dalloc<double>(n_borders);
    unsigned long long *od = dalloc<unsigned long long>(n_borders - 1);
    struct Release {
        double *&b;
        unsigned long long *&o;
        ~Release() { dfree(b); dfree(o); }
    } release{bd, od};
    RDC_CUDA(cudaMemcpyAsync(bd, borders, sizeof(double) * n_borders, cudaMemcpyHostToDevice, s->stream));
    RDC_CUDA(cudaMemsetAsync(od, 0, sizeof(unsigned long long) * (n_borders - 1), s->stream));
    launch(bd, od);
    RDC_CUDA(cudaGetLastError());
    std::vector<unsigned long long> h(n_borders - 1);
    RDC_CUDA(cudaMemcpyAsync(h.data(), od, sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost, s->stream));
    s->sync();
    return h;
}
}  // namespace

extern "C" {

int rdc_histogram_along_axis(rdc_system *s, int n_borders, const double *borders, int n_types, const int *types,
                             int axis, double *counts) {
    return guarded([&] {
        require(s && borders && counts && (n_types == 0 || types), "null argument");
        require(axis >= 0 && axis <= 2, "axis must be 0, 1 or 2");
        const uint32_t mask = type_mask(s, n_types, types);
        const auto h = observe_bins(s, n_borders, borders, [&](const double *bd, unsigned long long *od) {
            launch_histogram_axis(s->d, bd, n_borders, mask, axis, od, s->stream);
        });
        for (size_t k = 0; k < h.size(); ++k) counts[k] = (double)h[k];
    });
}

int rdc_radial_distribution(rdc_system *s, int n_borders, const double *borders, int n_from, const int *from_types,
                            int n_to, const int *to_types, double particle_to_density, double *counts,
                            double *distribution) {
    return guarded([&] {
        require(s && borders && counts && distribution && (n_from == 0 || from_types) && (n_to == 0 || to_types),
                "null argument");
        const uint32_t from = type_mask(s, n_from, from_types), to = type_mask(s, n_to, to_types);
        // FP32 screen: beyond the last border by more than the rounding of an FP32 squared distance
        const double rmax = borders[n_borders - 1];
        const float reach2 = rmax > 0 ? (float)(rmax * rmax * (1.0 + 1e-5)) : 0.f;
        int n_store = 0;
        RDC_CUDA(cudaMemcpyAsync(&n_store, s->d.counters + C_N_TOTAL, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
        s->sync();
        const auto h = observe_bins(s, n_borders, borders, [&](const double *bd, unsigned long long *od) {
            launch_radial_distribution(s->d, n_store, bd, n_borders, from, to, reach2, od, s->stream);
        });
        // from-particle count (the reference's count_if over the active particles)
        launch_count_types(s->d, s->count_buf, s->stream);
        std::vector<unsigned long long> tc(s->ctx.ntypes);
        RDC_CUDA(cudaMemcpyAsync(tc.data(), s->count_buf, sizeof(unsigned long long) * tc.size(), cudaMemcpyDeviceToHost,
                                 s->stream));
        s->sync();
        double n_from_particles = 0;
        for (int t = 0; t < s->ctx.ntypes; ++t)
            if ((from >> t) & 1u) n_from_particles += (double)tc[t];
        // RadialDistribution.cpp:108-118, in the same operation order
        const double pi = 3.14159265358979323846;
        for (size_t k = 0; k < h.size(); ++k) {
            counts[k] = (double)h[k];
            distribution[k] = counts[k] / (4. / 3. * pi * (std::pow(borders[k + 1], 3.) - std::pow(borders[k], 3.)) *
                                           n_from_particles * particle_to_density);
        }
    });
}

int rdc_get_reaction_counts(rdc_system *s, int n, int64_t *counts) {
    return guarded([&] {
        require(s && (n == 0 || counts), "null argument");
        std::vector<unsigned long long> h(MAX_REACTIONS);
        RDC_CUDA(cudaMemcpyAsync(h.data(), s->d.reaction_counts, sizeof(unsigned long long) * MAX_REACTIONS,
                                 cudaMemcpyDeviceToHost, s->stream));
        s->sync();
        for (int i = 0; i < n && i < MAX_REACTIONS; ++i) counts[i] = (int64_t)h[i];
    });
}
int rdc_reserve(rdc_system *s, int64_t capacity) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        require(capacity > 0 && capacity < INT_MAX / 2, "capacity out of range");
        s->reserve((int)capacity);
    });
}
int rdc_set_cell_radius(rdc_system *s, int radius) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        require(radius >= 1 && radius <= 3, "cell radius must be 1, 2 or 3");
        s->radius = radius;
        s->d.radius = radius;
        if (s->nl_ready && s->nl_cutoff > 0) s->nl_create(s->nl_cutoff);
    });
}

int rdc_initialize(rdc_system *s) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        RDC_CUDA(cudaMemsetAsync(s->d.reaction_counts, 0, sizeof(unsigned long long) * MAX_REACTIONS, s->stream));
    });
}
int rdc_nl_create(rdc_system *s, double cutoff) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        s->nl_create(cutoff);
    });
}
int rdc_nl_update(rdc_system *s) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        s->nl_update();
    });
}
int rdc_nl_clear(rdc_system *s) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        s->nl_clear();
    });
}
int rdc_calculate_forces(rdc_system *s) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        s->calculate_forces();
    });
}
int rdc_euler_bd_integrate(rdc_system *s, double dt) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        require(dt > 0, "time step must be > 0");
        s->integrate(dt);
    });
}
int rdc_uncontrolled_approximation(rdc_system *s, double dt) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        s->react(dt, H_UNCONTROLLED_APPROXIMATION);
    });
}
int rdc_gillespie(rdc_system *s, double dt) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        s->react(dt, H_GILLESPIE);
    });
}
int rdc_run(rdc_system *s, int64_t n_steps, double dt, int handler, int64_t stride, int64_t *counts, int64_t max_rec,
            int64_t *n_rec) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        s->run(n_steps, dt, handler, stride, counts, max_rec, n_rec);
    });
}
int rdc_nl_pairs(rdc_system *s, double cutoff, int64_t cap, uint64_t *pairs, int64_t *n_pairs) {
    return guarded([&] {
        require(s && n_pairs, "null argument");
        if (!s->nl_ready || s->nl_cutoff <= 0) throw LogicError("neighbor list not set up");
        require(cutoff > 0 && cutoff <= s->nl_cutoff * (1 + 1e-12), "pair cutoff exceeds the neighbor-list cutoff");
        int c[C_COUNT];
        s->read_counters(c);
        int dcap = (int)std::min<int64_t>(std::max<int64_t>(cap, 1), 1 << 28);
        uint64_t *buf = dalloc<uint64_t>(dcap);
        RDC_CUDA(cudaMemsetAsync(s->pairs_n, 0, sizeof(int), s->stream));
        const double c2 = cutoff * cutoff;
        const float L[3] = {s->d.geo.L[0], s->d.geo.L[1], s->d.geo.L[2]};
        launch_pairs(s->d, (float)c2, band_for(cutoff, L), c2, buf, dcap, s->pairs_n, s->stream);
        int n = 0;
        RDC_CUDA(cudaMemcpyAsync(&n, s->pairs_n, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
        s->sync();
        *n_pairs = n;
        if (n > cap) {
            dfree(buf);
            throw CapacityError("pair output capacity too small");
        }
        std::vector<uint64_t> h(n);
        if (n > 0) RDC_CUDA(cudaMemcpyAsync(h.data(), buf, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, s->stream));
        s->sync();
        dfree(buf);
        std::sort(h.begin(), h.end());
        for (int i = 0; i < n; ++i) {
            pairs[2 * i] = h[i] >> 32;
            pairs[2 * i + 1] = h[i] & 0xffffffffull;
        }
    });
}
int rdc_synchronize(rdc_system *s) {
    return guarded([&] {
        require(s != nullptr, "null argument");
        s->sync();
        RDC_CUDA(cudaGetLastError());
        s->check_status();
    });
}

}  // extern "C"

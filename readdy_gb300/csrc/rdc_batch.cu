// Batched replicas: thousands of independent copies of one context (own box, own particles) advanced
// together by the fused replica engine (rdc_engine.h), one persistent launch per step replayed from a
// CUDA graph.  A replica gives the same trajectory alone, inside any batch, or through rdc_run with
// the replica's seed (replica_seed).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/readdy_cuda.h"
#include "rdc_engine.h"

using namespace rdc;

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

// the packed particles of every replica (packed_off[r] .. packed_off[r + 1]) into the replica slices
// (slice_off[r] ..): one block per replica
__global__ void k_unpack_replicas(const float4 *__restrict__ packed, const int64_t *__restrict__ packed_off,
                                  const int64_t *__restrict__ slice_off, float4 *__restrict__ dst, int R) {
    for (int r = blockIdx.x; r < R; r += gridDim.x) {
        const int64_t b = packed_off[r], n = packed_off[r + 1] - b, d = slice_off[r];
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) dst[d + i] = packed[b + i];
    }
}

// float4 (x, y, z, type bits) of replicas [r0, r1) into packed[], from per-replica host arrays; false
// when a type is outside [0, ntypes)
bool pack_replicas(int r0, int r1, const int64_t *n, const int64_t *packed_off, const double *const *pos,
                   const int *const *types, int ntypes, float4 *packed) {
    for (int r = r0; r < r1; ++r) {
        float4 *out = packed + packed_off[r];
        const double *p = pos[r];
        const int *t = types[r];
        for (int64_t i = 0; i < n[r]; ++i) {
            if (t[i] < 0 || t[i] >= ntypes) return false;
            float4 q;
            q.x = (float)p[3 * i];
            q.y = (float)p[3 * i + 1];
            q.z = (float)p[3 * i + 2];
            std::memcpy(&q.w, &t[i], 4);
            out[i] = q;
        }
    }
    return true;
}
}  // namespace

namespace rdc {
const ContextData &context_data(const rdc_context *ctx);
void set_last_error(const std::string &m);
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
    // flat per-particle arrays; replica r owns slots [poff[r], poff[r] + caps[r])
    float4 *posA = nullptr, *posB = nullptr;
    float4 *forceA = nullptr, *forceB = nullptr;  // pair forces carried between steps
    uint32_t *idA = nullptr, *idB = nullptr;
    int *bin = nullptr, *rank = nullptr, *src = nullptr, *claim = nullptr, *taken = nullptr;
    int *start = nullptr;
    EventRec *events = nullptr;
    std::vector<int64_t> poff;
    EngineDev e{};
    RepDesc *desc_dev = nullptr;
    RepState *state_dev = nullptr;
    int *order_dev = nullptr, *n_work_dev = nullptr, *work_dev = nullptr, *all_dev = nullptr;
    unsigned long long *reaction_counts = nullptr, *particle_steps = nullptr, *count_dev = nullptr;
    Tables tab{};
    Tables *tab_dev = nullptr;
    double dt = 0;
    int handler = H_GILLESPIE;
    double cell_scale = 1.0;  // cell width = cutoff * cell_scale (at least)
    int threads = 256;
    int blocks = 0;
    size_t smem = 0;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // per-type count records streamed to the host (NParticles time series): record k of every replica is one
    // contiguous block of R x ntypes counters, so a poll copies new records with one copy on its own stream
    unsigned long long *records = nullptr;
    int64_t rec_stride = 0, rec_max = 0, rec_polled = 0, rec_start = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copy = nullptr;
    // trajectory frames of selected replicas streamed to the host (Trajectory observable): frame f holds,
    // per selected replica k, up to its capacity of particles at slot traj_off[k] of the frame
    std::vector<int> traj_sel;
    std::vector<int64_t> traj_off;  // n_sel + 1 slot offsets; traj_off[n_sel] = entries per frame
    int *traj_sel_dev = nullptr;
    int64_t *traj_off_dev = nullptr;
    float4 *traj_pos = nullptr;
    uint32_t *traj_id = nullptr;
    int *traj_n = nullptr;
    int64_t traj_stride = 0, traj_max = 0, traj_polled = 0, traj_now = 0;
    std::vector<int64_t> traj_steps;  // step of every frame written

    ~rdc_batch() { release(); }

    void release() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        bfree(desc_dev); bfree(state_dev); bfree(order_dev); bfree(n_work_dev); bfree(work_dev); bfree(all_dev);
        bfree(tab_dev); bfree(count_dev); bfree(reaction_counts); bfree(particle_steps);
        bfree(posA); bfree(posB); bfree(forceA); bfree(forceB); bfree(idA); bfree(idB);
        bfree(bin); bfree(rank); bfree(src); bfree(claim); bfree(taken); bfree(start); bfree(events);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (ev_copy) cudaEventDestroy(ev_copy);
        bfree(records);
        traj_off_all();
        if (copy_stream) cudaStreamDestroy(copy_stream);
        copy_stream = nullptr;
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }

    void sync() { RDC_CUDA(cudaStreamSynchronize(stream)); }

    void traj_off_all() {
        bfree(traj_sel_dev); bfree(traj_off_dev); bfree(traj_pos); bfree(traj_id); bfree(traj_n);
        traj_sel.clear();
        traj_off.clear();
        traj_steps.clear();
        traj_stride = traj_max = traj_polled = 0;
    }
    // the next trajectory frame, taken now (dropped once max_frames are written)
    void traj_snapshot() {
        const int64_t f = (int64_t)traj_steps.size();
        if (f >= traj_max) return;
        const int ns = (int)traj_sel.size();
        const int64_t per = traj_off[ns];
        launch_engine_snapshot(e, traj_sel_dev, ns, traj_off_dev, traj_pos + f * per, traj_id + f * per,
                               traj_n + f * ns, stream);
        traj_steps.push_back(traj_now);
    }

    void invalidate_graph() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
    }

    // cell grids and the per-replica slices of the cell and event arrays
    void layout() {
        const double cutoff = ctx.max_cutoff();
        int64_t soff = 0, eoff = 0;
        std::vector<int64_t> so(R), eo(R);
        desc.resize(R);
        for (int r = 0; r < R; ++r) {
            RepDesc &D = desc[r];
            D.geo = replica_geo(&boxes[3 * r], ctx.pbc, cutoff, cell_scale, caps[r], D.smem_cells);
            D.cap = (int)caps[r];
            D.ecap = 64 + D.cap / 32;
            D.table = 0;
            D.seed = replica_seed(seed, r);
            D.n_steps = INT64_MAX;
            D.count_stride = 0;
            D.max_records = 0;
            D.records = nullptr;
            so[r] = soff;
            eo[r] = eoff;
            soff += (D.geo.ncells + 3 + 3) / 4 * 4;  // 16-byte aligned slices (vector copies of 16-bit starts)
            eoff += D.ecap;
            if (soff > INT_MAX / 2 || eoff > INT_MAX / 2) throw std::invalid_argument("batch too large");
        }
        bfree(start); bfree(events);
        start = balloc<int>(soff);
        events = balloc<EventRec>(eoff);
        RDC_CUDA(cudaMemsetAsync(start, 0, sizeof(int) * soff, stream));
        for (int r = 0; r < R; ++r) {
            RepDesc &D = desc[r];
            const int64_t p = poff[r];
            D.pos[0] = posA + p; D.pos[1] = posB + p;
            D.force[0] = forceA ? forceA + p : nullptr;
            D.force[1] = forceB ? forceB + p : nullptr;
            D.id[0] = idA + p; D.id[1] = idB + p;
            D.bin = bin + p; D.rank = rank + p; D.src = src + p; D.claim = claim + p; D.taken = taken + p;
            D.start = start + so[r];
            D.events = events + eo[r];
            D.rx_counts = reaction_counts + (size_t)r * MAX_REACTIONS;
            apply_records(r);
        }
        RDC_CUDA(cudaMemcpyAsync(desc_dev, desc.data(), sizeof(RepDesc) * R, cudaMemcpyHostToDevice, stream));
        invalidate_graph();
    }

    // count-record fields of replica r's descriptor (none until recording is switched on)
    void apply_records(int r) {
        RepDesc &D = desc[r];
        D.records = records ? records + (size_t)r * ctx.ntypes : nullptr;
        D.record_pitch = (int64_t)R * ctx.ntypes;
        D.count_stride = records ? (int)rec_stride : 0;
        D.max_records = records ? (int)rec_max : 0;
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
        poff.resize(R);
        for (int r = 0; r < R; ++r) {
            if (caps[r] <= 0) throw std::invalid_argument("replica capacity must be > 0");
            poff[r] = total;
            total += caps[r];
        }
        if (total > INT_MAX / 2) throw std::invalid_argument("batch capacity too large");
        posA = balloc<float4>(total); posB = balloc<float4>(total);
        forceA = balloc<float4>(total); forceB = balloc<float4>(total);
        idA = balloc<uint32_t>(total); idB = balloc<uint32_t>(total);
        bin = balloc<int>(total); rank = balloc<int>(total); src = balloc<int>(total);
        claim = balloc<int>(total); taken = balloc<int>(total);
        RDC_CUDA(cudaMemsetAsync(claim, 0x7f, sizeof(int) * total, stream));
        RDC_CUDA(cudaMemsetAsync(taken, 0, sizeof(int) * total, stream));
        // performed events per replica and reaction (MAX_REACTIONS counters per replica)
        reaction_counts = balloc<unsigned long long>((size_t)R * MAX_REACTIONS);
        RDC_CUDA(cudaMemsetAsync(reaction_counts, 0, sizeof(unsigned long long) * MAX_REACTIONS * R, stream));
        particle_steps = balloc<unsigned long long>(1);
        RDC_CUDA(cudaMemsetAsync(particle_steps, 0, sizeof(unsigned long long), stream));
        count_dev = balloc<unsigned long long>((size_t)R * ctx.ntypes);
        RDC_CUDA(cudaEventCreate(&ev0));
        RDC_CUDA(cudaEventCreate(&ev1));
        desc_dev = balloc<RepDesc>(R);
        state_dev = balloc<RepState>(R);
        RDC_CUDA(cudaMemsetAsync(state_dev, 0, sizeof(RepState) * R, stream));
        order_dev = balloc<int>(R);
        all_dev = balloc<int>(R);
        std::vector<int> all(R);
        std::iota(all.begin(), all.end(), 0);
        RDC_CUDA(cudaMemcpyAsync(all_dev, all.data(), sizeof(int) * R, cudaMemcpyHostToDevice, stream));
        n_work_dev = balloc<int>(1);
        RDC_CUDA(cudaMemcpyAsync(n_work_dev, &R, sizeof(int), cudaMemcpyHostToDevice, stream));
        work_dev = balloc<int>(1);
        RDC_CUDA(cudaMemsetAsync(work_dev, 0, sizeof(int), stream));
        // tables: rounding bands sized for the largest box
        double bmax[3] = {0, 0, 0};
        for (int r = 0; r < R; ++r)
            for (int k = 0; k < 3; ++k) bmax[k] = std::max(bmax[k], boxes[3 * r + k]);
        build_tables(ctx, bmax, 0.0, tab);
        tab_dev = balloc<Tables>(1);
        RDC_CUDA(cudaMemcpyAsync(tab_dev, &tab, sizeof(Tables), cudaMemcpyHostToDevice, stream));
        e.desc = desc_dev;
        e.state = state_dev;
        e.order = order_dev;
        e.n_work = n_work_dev;
        e.work = work_dev;
        e.tabs = tab_dev;
        e.handler = handler;
        e.max_events_sm = ENGINE_MAX_EVENTS_SM;
        e.particle_steps = particle_steps;
        layout();
        sync();
    }

    // largest replicas first (longest-processing-time order for the work counter)
    void set_order(const std::vector<int64_t> &n) {
        std::vector<int> ord(R);
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return n[a] > n[b]; });
        RDC_CUDA(cudaMemcpyAsync(order_dev, ord.data(), sizeof(int) * R, cudaMemcpyHostToDevice, stream));
        sync();
    }

    // binning and sort of every replica from its current buffer (new ids only for new particles)
    void sort_all(bool fill_ids) { launch_engine_admit(e, all_dev, R, fill_ids, stream); }

    void step(int64_t n) {
        if (dt <= 0) throw std::logic_error("rdc_batch_configure must set a time step first");
        if (!graph) {
            smem = engine_smem_bytes(e.max_events_sm);
            blocks = std::max(1, std::min(R, engine_grid(threads, smem)));
            cudaGraph_t g;
            RDC_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            launch_engine_step(e, blocks, threads, smem, stream);
            RDC_CUDA(cudaStreamEndCapture(stream, &g));
            RDC_CUDA(cudaGraphInstantiate(&graph, g, 0));
            cudaGraphDestroy(g);
        }
        if (!traj_stride) {
            for (int64_t k = 0; k < n; ++k) RDC_CUDA(cudaGraphLaunch(graph, stream));
            return;
        }
        for (int64_t k = 0; k < n; ++k) {
            RDC_CUDA(cudaGraphLaunch(graph, stream));
            if (++traj_now % traj_stride == 0) traj_snapshot();  // observable strides count absolute steps
        }
    }

    std::vector<RepState> states() {
        std::vector<RepState> h(R);
        RDC_CUDA(cudaMemcpyAsync(h.data(), state_dev, sizeof(RepState) * R, cudaMemcpyDeviceToHost, stream));
        sync();
        return h;
    }

    // pair forces carried between steps (allocated) or summed at the start of every step (freed)
    void set_carry_forces(bool on) {
        int64_t total = 0;
        for (int64_t c : caps) total += c;
        if (on && !forceA) {
            forceA = balloc<float4>(total);
            forceB = balloc<float4>(total);
        } else if (!on && forceA) {
            sync();
            bfree(forceA); bfree(forceB);
            forceA = forceB = nullptr;
        }
        for (int r = 0; r < R; ++r) {
            desc[r].force[0] = forceA ? forceA + poff[r] : nullptr;
            desc[r].force[1] = forceB ? forceB + poff[r] : nullptr;
        }
        RDC_CUDA(cudaMemcpyAsync(desc_dev, desc.data(), sizeof(RepDesc) * R, cudaMemcpyHostToDevice, stream));
        // sorted again, cell starts in place, no forces carried
        sort_all(false);
        sync();
    }

    void check_status() { check_status(states()); }

    // a device status raised by any replica becomes an error (and is cleared)
    void check_status(std::vector<RepState> st) {
        int any = 0;
        for (auto &s : st) any |= s.status;
        if (any) {
            for (auto &s : st) s.status = 0;
            RDC_CUDA(cudaMemcpyAsync(state_dev, st.data(), sizeof(RepState) * R, cudaMemcpyHostToDevice, stream));
            sync();
            if (any & ST_CAPACITY) throw rdc::CapacityError("replica particle capacity exceeded by reaction products");
            if (any & ST_EVENTS) throw rdc::CapacityError("replica reaction event buffer overflow");
            if (any & ST_INDEX) throw std::runtime_error("replica step met a storage index out of range");
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

namespace {
// Initial particles of every replica from per-replica host arrays: converted to float4 by host threads
// into one packed buffer, copied once into the second position buffer (free until the first sort) and
// unpacked into the replica slices on the device.
void set_particles_impl(rdc_batch *b, const int64_t *n, const double *const *pos, const int *const *types) {
    const int R = b->R;
    std::vector<int64_t> packed_off(R + 1, 0);
    for (int r = 0; r < R; ++r) {
        if (n[r] < 0 || n[r] > b->caps[r]) throw std::invalid_argument("replica particle count exceeds capacity");
        if (n[r] > 0 && (!pos[r] || !types[r])) throw std::invalid_argument("null argument");
        packed_off[r + 1] = packed_off[r] + n[r];
    }
    const int64_t total = packed_off[R];
    std::unique_ptr<float4[]> packed(new float4[std::max<int64_t>(total, 1)]);
    // replicas split into contiguous runs of about equal particle counts, one per host thread
    const int nt = (int)std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    std::vector<int> cut(nt + 1, R);
    cut[0] = 0;
    for (int t = 1, r = 0; t < nt; ++t) {
        while (r < R && packed_off[r] < total * t / nt) ++r;
        cut[t] = r;
    }
    std::vector<char> ok(nt, 1);
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; ++t)
        pool.emplace_back([&, t] { ok[t] = pack_replicas(cut[t], cut[t + 1], n, packed_off.data(), pos, types,
                                                         b->ctx.ntypes, packed.get()); });
    ok[0] = pack_replicas(cut[0], cut[1], n, packed_off.data(), pos, types, b->ctx.ntypes, packed.get());
    for (auto &th : pool) th.join();
    for (char o : ok)
        if (!o) throw std::invalid_argument("particle type out of range");
    std::vector<RepState> st(R);
    for (int r = 0; r < R; ++r) st[r] = RepState{(int)n[r], 0, 0, (int)n[r], 0, 0, 0, 0};
    int64_t *offs_dev = balloc<int64_t>(2 * (size_t)R + 1);
    struct Release {
        int64_t *&p;
        ~Release() { bfree(p); }
    } release{offs_dev};
    std::vector<int64_t> offs(packed_off);
    offs.insert(offs.end(), b->poff.begin(), b->poff.end());
    RDC_CUDA(cudaMemcpyAsync(offs_dev, offs.data(), sizeof(int64_t) * offs.size(), cudaMemcpyHostToDevice, b->stream));
    if (total > 0)
        RDC_CUDA(cudaMemcpyAsync(b->posB, packed.get(), sizeof(float4) * total, cudaMemcpyHostToDevice, b->stream));
    k_unpack_replicas<<<std::min(R, 4 * sm_count()), 256, 0, b->stream>>>(b->posB, offs_dev, offs_dev + R + 1, b->posA, R);
    RDC_CUDA(cudaGetLastError());
    RDC_CUDA(cudaMemcpyAsync(b->state_dev, st.data(), sizeof(RepState) * R, cudaMemcpyHostToDevice, b->stream));
    b->rec_polled = 0;  // with records on, the admission below writes record 0 again (t = 0)
    b->rec_start = 0;
    b->traj_off_all();  // new replicas: a trajectory of the old ones ends
    b->set_order(std::vector<int64_t>(n, n + R));
    b->sort_all(true);
    b->sync();
}
}  // namespace

int rdc_batch_set_particles(rdc_batch *b, const int64_t *offsets, const double *pos, const int *types) {
    BATCH_CALL({
        if (!b || !offsets || !pos || !types) throw std::invalid_argument("null argument");
        const int R = b->R;
        std::vector<int64_t> n(R);
        std::vector<const double *> p(R);
        std::vector<const int *> t(R);
        for (int r = 0; r < R; ++r) {
            n[r] = offsets[r + 1] - offsets[r];
            p[r] = pos + 3 * offsets[r];
            t[r] = types + offsets[r];
        }
        set_particles_impl(b, n.data(), p.data(), t.data());
    });
}

int rdc_batch_set_particles_list(rdc_batch *b, const int64_t *counts, const double *const *positions3,
                                 const int *const *types) {
    BATCH_CALL({
        if (!b || !counts || !positions3 || !types) throw std::invalid_argument("null argument");
        set_particles_impl(b, counts, positions3, types);
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
        if (threads_per_block < 64 || threads_per_block > ENGINE_THREADS_MAX || threads_per_block % 32)
            throw std::invalid_argument("threads per block must be a multiple of 32 in [64, " +
                                        std::to_string(ENGINE_THREADS_MAX) + "]");
        b->handler = handler;
        b->e.handler = handler;
        b->dt = dt;
        set_time_step(b->ctx, dt, b->tab);
        RDC_CUDA(cudaMemcpyAsync(b->tab_dev, &b->tab, sizeof(Tables), cudaMemcpyHostToDevice, b->stream));
        b->threads = threads_per_block;
        if (cell_width_scale != b->cell_scale) {
            b->cell_scale = cell_width_scale;
            b->layout();
            b->sort_all(false);
        }
        b->invalidate_graph();
        b->sync();
    });
}

int rdc_batch_set_carry_forces(rdc_batch *b, int on) {
    BATCH_CALL({
        if (!b) throw std::invalid_argument("null argument");
        b->set_carry_forces(on != 0);
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
        RDC_CUDA(cudaMemcpyAsync(&v, b->particle_steps, sizeof(v), cudaMemcpyDeviceToHost, b->stream));
        b->sync();
        *particle_steps = v;
    });
}

int rdc_batch_count_types(rdc_batch *b, int64_t *counts) {
    BATCH_CALL({
        if (!b || !counts) throw std::invalid_argument("null argument");
        b->check_status();
        launch_engine_count(b->e, b->R, b->ctx.ntypes, b->count_dev, b->stream);
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
        b->check_status();
        // the per-type counts: a replica's storage may still hold the slots of removed particles
        const int T = b->ctx.ntypes;
        launch_engine_count(b->e, b->R, T, b->count_dev, b->stream);
        std::vector<unsigned long long> h((size_t)b->R * T);
        RDC_CUDA(cudaMemcpyAsync(h.data(), b->count_dev, sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost,
                                 b->stream));
        b->sync();
        for (int r = 0; r < b->R; ++r) {
            int64_t sum = 0;
            for (int t = 0; t < T; ++t) sum += (int64_t)h[(size_t)r * T + t];
            n[r] = sum;
        }
    });
}

int rdc_batch_get_particles(rdc_batch *b, int replica, int64_t cap, double *pos, int *types, uint64_t *ids,
                            int64_t *n_out) {
    BATCH_CALL({
        if (!b) throw std::invalid_argument("null argument");
        if (replica < 0 || replica >= b->R) throw std::invalid_argument("replica out of range");
        auto st = b->states();
        b->check_status(st);
        const RepState s = st[replica];
        const RepDesc &D = b->desc[replica];
        std::vector<float4> hp(s.n);
        std::vector<uint32_t> hid(s.n);
        if (s.n > 0) {
            RDC_CUDA(cudaMemcpyAsync(hp.data(), D.pos[s.cur], sizeof(float4) * s.n, cudaMemcpyDeviceToHost, b->stream));
            RDC_CUDA(cudaMemcpyAsync(hid.data(), D.id[s.cur], sizeof(uint32_t) * s.n, cudaMemcpyDeviceToHost,
                                     b->stream));
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

int rdc_batch_get_forces(rdc_batch *b, int replica, int64_t cap, double *forces, uint64_t *ids, int64_t *n_out) {
    BATCH_CALL({
        if (!b) throw std::invalid_argument("null argument");
        if (replica < 0 || replica >= b->R) throw std::invalid_argument("replica out of range");
        auto st = b->states();
        b->check_status(st);
        const RepState s = st[replica];
        const RepDesc &D = b->desc[replica];
        std::vector<float4> hp(s.n), hf(s.n);
        std::vector<uint32_t> hid(s.n);
        if (s.n > 0) {
            float4 *f = balloc<float4>(s.n);
            struct Release {
                float4 *&p;
                ~Release() { bfree(p); }
            } release{f};
            launch_engine_forces(b->e, replica, s.n, f, b->stream);
            RDC_CUDA(cudaGetLastError());
            RDC_CUDA(cudaMemcpyAsync(hf.data(), f, sizeof(float4) * s.n, cudaMemcpyDeviceToHost, b->stream));
            RDC_CUDA(cudaMemcpyAsync(hp.data(), D.pos[s.cur], sizeof(float4) * s.n, cudaMemcpyDeviceToHost, b->stream));
            RDC_CUDA(cudaMemcpyAsync(hid.data(), D.id[s.cur], sizeof(uint32_t) * s.n, cudaMemcpyDeviceToHost,
                                     b->stream));
            b->sync();
        }
        int64_t k = 0;
        for (int i = 0; i < s.n; ++i) {
            int t;
            std::memcpy(&t, &hp[i].w, 4);
            if (t < 0) continue;
            if (k < cap) {
                if (forces) { forces[3 * k] = hf[i].x; forces[3 * k + 1] = hf[i].y; forces[3 * k + 2] = hf[i].z; }
                if (ids) ids[k] = hid[i];
            }
            ++k;
        }
        if (n_out) *n_out = k;
        if (k > cap) throw rdc::CapacityError("output capacity too small for the particles");
    });
}

int rdc_batch_record_counts(rdc_batch *b, int64_t stride, int64_t max_records) {
    BATCH_CALL({
        if (!b) throw std::invalid_argument("null argument");
        if (stride < 1 || max_records < 1) throw std::invalid_argument("stride and max_records must be >= 1");
        const size_t per_record = (size_t)b->R * b->ctx.ntypes;
        if ((double)per_record * (double)max_records * 8.0 > 16e9)
            throw std::invalid_argument("count records would take more than 16 GB of device memory");
        if (max_records > INT_MAX / 2) throw std::invalid_argument("max_records too large");
        auto st = b->states();
        b->check_status(st);
        bfree(b->records);
        b->records = balloc<unsigned long long>(per_record * (size_t)max_records);
        b->rec_stride = stride;
        b->rec_max = max_records;
        b->rec_polled = 0;
        b->rec_start = st.empty() ? 0 : st[0].step;
        if (!b->copy_stream) {
            RDC_CUDA(cudaStreamCreateWithFlags(&b->copy_stream, cudaStreamNonBlocking));
            RDC_CUDA(cudaEventCreateWithFlags(&b->ev_copy, cudaEventDisableTiming));
        }
        for (int r = 0; r < b->R; ++r) b->apply_records(r);
        RDC_CUDA(cudaMemcpyAsync(b->desc_dev, b->desc.data(), sizeof(RepDesc) * b->R, cudaMemcpyHostToDevice,
                                 b->stream));
        // record 0: the counts now; later records follow every stride steps of the replicas' own step count
        launch_engine_record_now(b->e, b->R, b->ctx.ntypes, 0, b->stream);
        RDC_CUDA(cudaGetLastError());
        for (auto &x : st) x.rec = 1;
        RDC_CUDA(cudaMemcpyAsync(b->state_dev, st.data(), sizeof(RepState) * b->R, cudaMemcpyHostToDevice, b->stream));
        b->sync();
    });
}

int rdc_batch_record_trajectory(rdc_batch *b, int n_replicas, const int *replicas, int64_t stride, int64_t max_frames) {
    BATCH_CALL({
        if (!b || (n_replicas > 0 && !replicas)) throw std::invalid_argument("null argument");
        if (n_replicas < 0) throw std::invalid_argument("n_replicas must be >= 0");
        b->sync();
        b->traj_off_all();
        if (n_replicas == 0) return;
        if (stride <= 0) throw std::invalid_argument("stride must be > 0");
        if (max_frames <= 0) throw std::invalid_argument("max_frames must be > 0");
        std::vector<int64_t> off(n_replicas + 1, 0);
        for (int k = 0; k < n_replicas; ++k) {
            if (replicas[k] < 0 || replicas[k] >= b->R) throw std::invalid_argument("replica out of range");
            off[k + 1] = off[k] + b->caps[replicas[k]];
        }
        const int64_t per = off[n_replicas];
        if (per * max_frames > (int64_t)1 << 34)
            throw std::invalid_argument("trajectory buffer above 2^34 entries: fewer replicas or frames");
        auto st = b->states();
        b->check_status(st);
        b->traj_sel.assign(replicas, replicas + n_replicas);
        b->traj_off = off;
        b->traj_sel_dev = balloc<int>(n_replicas);
        b->traj_off_dev = balloc<int64_t>(n_replicas + 1);
        b->traj_pos = balloc<float4>(per * max_frames);
        b->traj_id = balloc<uint32_t>(per * max_frames);
        b->traj_n = balloc<int>(n_replicas * max_frames);
        RDC_CUDA(cudaMemcpyAsync(b->traj_sel_dev, replicas, sizeof(int) * n_replicas, cudaMemcpyHostToDevice, b->stream));
        RDC_CUDA(cudaMemcpyAsync(b->traj_off_dev, off.data(), sizeof(int64_t) * off.size(), cudaMemcpyHostToDevice,
                                 b->stream));
        b->traj_stride = stride;
        b->traj_max = max_frames;
        b->traj_now = st.empty() ? 0 : st[0].step;
        if (!b->copy_stream) {
            RDC_CUDA(cudaStreamCreateWithFlags(&b->copy_stream, cudaStreamNonBlocking));
            RDC_CUDA(cudaEventCreateWithFlags(&b->ev_copy, cudaEventDisableTiming));
        }
        b->traj_snapshot();  // frame 0: now
        b->sync();
    });
}

int rdc_batch_poll_trajectory(rdc_batch *b, int64_t capacity_frames, int64_t capacity_entries, int64_t *steps,
                              int64_t *counts, double *positions3, int *types, uint64_t *ids, int64_t *n_frames,
                              int64_t *n_entries) {
    BATCH_CALL({
        if (!b) throw std::invalid_argument("null argument");
        if (!b->traj_stride) throw std::logic_error("the trajectory is off (rdc_batch_record_trajectory switches it on)");
        if (n_frames) *n_frames = 0;
        if (n_entries) *n_entries = 0;
        // the frames written so far, copied on the copy stream once the batch's stream has reached this point
        RDC_CUDA(cudaEventRecord(b->ev_copy, b->stream));
        RDC_CUDA(cudaStreamWaitEvent(b->copy_stream, b->ev_copy, 0));
        const int ns = (int)b->traj_sel.size();
        const int64_t per = b->traj_off[ns];
        const int64_t avail = (int64_t)b->traj_steps.size() - b->traj_polled;
        int64_t nf = std::max<int64_t>(0, std::min(avail, capacity_frames));
        std::vector<int> cnt((size_t)nf * ns);
        if (nf > 0)
            RDC_CUDA(cudaMemcpyAsync(cnt.data(), b->traj_n + b->traj_polled * ns, sizeof(int) * cnt.size(),
                                     cudaMemcpyDeviceToHost, b->copy_stream));
        RDC_CUDA(cudaStreamSynchronize(b->copy_stream));
        // whole frames only, as many as the entry capacity takes
        int64_t total = 0, fit = 0;
        for (int64_t f = 0; f < nf; ++f) {
            int64_t t = 0;
            for (int k = 0; k < ns; ++k) t += cnt[f * ns + k];
            if (total + t > capacity_entries) {
                if (fit == 0) {
                    if (n_entries) *n_entries = t;
                    throw rdc::CapacityError("entry capacity too small for the next trajectory frame");
                }
                break;
            }
            total += t;
            ++fit;
        }
        nf = fit;
        std::vector<float4> hp((size_t)total);
        std::vector<uint32_t> hid((size_t)total);
        int64_t at = 0;
        for (int64_t f = 0; f < nf; ++f)
            for (int k = 0; k < ns; ++k) {
                const int64_t c = cnt[f * ns + k];
                const int64_t src = (b->traj_polled + f) * per + b->traj_off[k];
                if (c > 0) {
                    RDC_CUDA(cudaMemcpyAsync(hp.data() + at, b->traj_pos + src, sizeof(float4) * c,
                                             cudaMemcpyDeviceToHost, b->copy_stream));
                    RDC_CUDA(cudaMemcpyAsync(hid.data() + at, b->traj_id + src, sizeof(uint32_t) * c,
                                             cudaMemcpyDeviceToHost, b->copy_stream));
                }
                at += c;
            }
        RDC_CUDA(cudaStreamSynchronize(b->copy_stream));
        for (int64_t f = 0; f < nf; ++f) {
            if (steps) steps[f] = b->traj_steps[b->traj_polled + f];
            if (counts)
                for (int k = 0; k < ns; ++k) counts[f * ns + k] = cnt[f * ns + k];
        }
        for (int64_t i = 0; i < total; ++i) {
            if (positions3) {
                positions3[3 * i] = hp[i].x;
                positions3[3 * i + 1] = hp[i].y;
                positions3[3 * i + 2] = hp[i].z;
            }
            if (types) std::memcpy(&types[i], &hp[i].w, 4);
            if (ids) ids[i] = hid[i];
        }
        b->traj_polled += nf;
        if (n_frames) *n_frames = nf;
        if (n_entries) *n_entries = total;
    });
}

int rdc_batch_poll_count_records(rdc_batch *b, int64_t capacity, int64_t *steps, int64_t *counts, int64_t *n_out) {
    BATCH_CALL({
        if (!b || !n_out || (capacity > 0 && !counts)) throw std::invalid_argument("null argument");
        if (!b->records) throw std::logic_error("count records are off (rdc_batch_record_counts switches them on)");
        // the copies run on their own stream after the steps queued so far; the batch's stream goes on
        RDC_CUDA(cudaEventRecord(b->ev_copy, b->stream));
        RDC_CUDA(cudaStreamWaitEvent(b->copy_stream, b->ev_copy, 0));
        std::vector<RepState> st(b->R);
        RDC_CUDA(cudaMemcpyAsync(st.data(), b->state_dev, sizeof(RepState) * b->R, cudaMemcpyDeviceToHost,
                                 b->copy_stream));
        RDC_CUDA(cudaStreamSynchronize(b->copy_stream));
        int64_t written = b->rec_max;
        for (const auto &x : st) {
            if (x.status) throw std::runtime_error("replica device status " + std::to_string(x.status));
            written = std::min<int64_t>(written, x.rec);
        }
        const int64_t n = std::max<int64_t>(0, std::min<int64_t>(written - b->rec_polled, capacity));
        const size_t per_record = (size_t)b->R * b->ctx.ntypes;
        if (n > 0) {
            std::vector<unsigned long long> h(per_record * (size_t)n);
            RDC_CUDA(cudaMemcpyAsync(h.data(), b->records + per_record * (size_t)b->rec_polled,
                                     sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost, b->copy_stream));
            RDC_CUDA(cudaStreamSynchronize(b->copy_stream));
            for (size_t k = 0; k < h.size(); ++k) counts[k] = (int64_t)h[k];
        }
        if (steps) {
            // record 0 at the step recording started, record k >= 1 after the k-th later multiple of stride
            const int64_t first = (b->rec_start / b->rec_stride + 1) * b->rec_stride;
            for (int64_t k = 0; k < n; ++k) {
                const int64_t idx = b->rec_polled + k;
                steps[k] = idx == 0 ? b->rec_start : first + (idx - 1) * b->rec_stride;
            }
        }
        b->rec_polled += n;
        *n_out = n;
    });
}

int rdc_batch_get_virial(rdc_batch *b, double *virial9) {
    BATCH_CALL({
        if (!b || !virial9) throw std::invalid_argument("null argument");
        if (b->forceA)
            throw std::logic_error("the virial is taken from forces summed over the sorted state: switch carried "
                                   "forces off first (rdc_batch_set_carry_forces(b, 0))");
        b->check_status();
        double *d = balloc<double>((size_t)b->R * 9);
        struct Release {
            double *&p;
            ~Release() { bfree(p); }
        } release{d};
        launch_engine_virial(b->e, b->R, d, b->stream);
        RDC_CUDA(cudaGetLastError());
        RDC_CUDA(cudaMemcpyAsync(virial9, d, sizeof(double) * 9 * b->R, cudaMemcpyDeviceToHost, b->stream));
        b->sync();
    });
}

int rdc_batch_reaction_counts(rdc_batch *b, int n, int64_t *counts) {
    BATCH_CALL({
        if (!b || !counts) throw std::invalid_argument("null argument");
        if (n < 0 || n > MAX_REACTIONS) throw std::invalid_argument("reaction count out of range");
        b->check_status();
        std::vector<unsigned long long> h((size_t)b->R * MAX_REACTIONS);
        RDC_CUDA(cudaMemcpyAsync(h.data(), b->reaction_counts, sizeof(unsigned long long) * h.size(),
                                 cudaMemcpyDeviceToHost, b->stream));
        b->sync();
        for (int r = 0; r < b->R; ++r)
            for (int k = 0; k < n; ++k) counts[(size_t)r * n + k] = (int64_t)h[(size_t)r * MAX_REACTIONS + k];
    });
}

int rdc_batch_replica_grid(rdc_batch *b, int replica, int *dims3, int *shared_cells) {
    BATCH_CALL({
        if (!b || !dims3) throw std::invalid_argument("null argument");
        if (replica < 0 || replica >= b->R) throw std::invalid_argument("replica out of range");
        const RepDesc &D = b->desc[replica];
        for (int k = 0; k < 3; ++k) dims3[k] = D.geo.dims[k];
        if (shared_cells) *shared_cells = D.smem_cells;
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

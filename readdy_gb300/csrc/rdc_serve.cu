// Served form: a request loop over independent simulations of different sizes and chemistries.
//
// Requests arrive with their own context (species, diffusion, potentials, reactions, box), particles,
// step count, time step, count stride and seed.  The server admits them first-come first-served
// against a device-memory budget, keeps every admitted request's particle state resident in HBM until
// it finishes, and returns its per-type count records with submit/admit/finish times.
//
// Two legs share the GPU:
//  * requests of up to plain_threshold particles become replicas of the fused engine (rdc_engine.h):
//    each engine launch is one persistent kernel over all of them with as many CTAs as active requests
//    (at most one per SM; the other SMs stay free for the per-system leg), replayed from a CUDA graph
//    captured per grid size, and requests join and leave between chunks of launches (continuous
//    batching).  In one launch a request takes as many steps as fit into one step of the largest active
//    request, so small requests are not held to the large ones' pace;
//  * larger requests run as plain per-system simulations (rdc_run: grid-wide kernels replayed from a
//    CUDA graph), each on its own stream, taken by a fixed pool of host worker threads (at most that many
//    run at once): on one CTA their steps would take too long for their own latency.
// A request's random streams are keyed by its own seed, particle ids and step counter, and its cell grid
// by its own box, so its result does not depend on which other requests share the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/readdy_cuda.h"
#include "rdc_engine.h"

using namespace rdc;

namespace rdc {
const ContextData &context_data(const rdc_context *ctx);
rdc_context *context_clone(const ContextData &d);
void set_last_error(const std::string &m);
}  // namespace rdc

namespace {
thread_local std::string s_err;

constexpr size_t ALIGN = 256;
size_t up(size_t x) { return (x + ALIGN - 1) / ALIGN * ALIGN; }

// device footprint of an engine replica, carved from one allocation in this order
struct EngineLayout {
    size_t pos, id, ints, start, events, records, rx, total;
};
EngineLayout engine_layout(int64_t cap, int ncells, int ecap, int max_records, int ntypes) {
    EngineLayout L{};
    size_t off = 0;
    L.pos = off; off += up(4 * sizeof(float4) * cap);  // two position and two force buffers
    L.id = off; off += up(2 * sizeof(uint32_t) * cap);
    L.ints = off; off += up(5 * sizeof(int) * cap);
    L.start = off; off += up(sizeof(int) * (ncells + 3));
    L.events = off; off += up(sizeof(EventRec) * ecap);
    L.records = off; off += up(sizeof(unsigned long long) * (size_t)max_records * ntypes);
    L.rx = off; off += up(sizeof(unsigned long long) * MAX_REACTIONS);
    L.total = off;
    return L;
}

// device footprint estimate of a plain per-system simulation (double-buffered particle state, sort
// scratch, cell arrays, the 64k-entry event buffer and the count ring)
size_t plain_bytes(int64_t cap, int64_t ncells, int max_records, int ntypes) {
    return (size_t)cap * (2 * (16 + 4 + 4 + 16) + 6 * 4) + (size_t)ncells * 12 + (size_t)(1 << 16) * 32 +
           (size_t)max_records * ntypes * 8 + (4u << 20);
}

double now_s(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// The cost of one engine step of a replica on its CTA, measured: about 20 us plus 0.027 us per particle,
// i.e. the fixed part is worth about 740 particles.
constexpr double ENGINE_FIXED_PARTICLES = 740.0;
constexpr int ENGINE_MAX_LAUNCH_STEPS = 64;

// particle capacity of a request: reactions may add particles (fission, two-product conversions), so
// room for a quarter more plus a margin; a request that outgrows it ends with RDC_ERR_CAPACITY status
int64_t request_capacity(int64_t n) { return n + n / 4 + 64; }

struct Request {
    int64_t id = 0;
    ContextData ctx;
    std::vector<float4> pos;  // initial particles, type bits in .w
    int64_t n = 0, n_steps = 0, stride = 0, cap = 0;
    double dt = 0;
    uint64_t seed = 0;
    int max_records = 0;
    size_t bytes = 0;
    bool plain = false;
    // engine leg
    Geo geo{};
    int smem_cells = 0;
    int slot = -1;
    void *block = nullptr;
    EngineLayout L{};
    int64_t steps_done = 0;
    // plain leg (run by a worker of the pool); the worker runs in chunks and appends each chunk's count
    // records to `partial` so that rdc_server_peek_records can stream them
    std::atomic<int> worker_done{0};
    int worker_rc = RDC_OK;
    std::string worker_err;
    std::mutex partial_mutex;
    std::vector<int64_t> partial;  // n_partial x ntypes
    int64_t n_partial = 0;
    // result
    double t_submit = 0, t_admit = -1, t_finish = -1;
    int status = RDC_OK;
    std::string message;
    bool finished = false;
    std::vector<int64_t> records;  // n_records x ntypes
    int64_t n_records = 0;
    uint64_t particle_steps = 0;
};
}  // namespace

struct rdc_server {
    cudaStream_t stream = nullptr;
    int device = 0;
    size_t budget = 0, in_use = 0;
    int max_active = 0;
    int handler = H_GILLESPIE;
    int64_t plain_threshold = 0;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    int64_t next_id = 1;
    std::map<int64_t, std::unique_ptr<Request>> requests;
    std::deque<int64_t> pending;
    std::vector<int64_t> slot_owner;  // engine slot -> request id (0: free)
    std::vector<int64_t> plain_running;
    std::vector<int64_t> unpolled;
    // worker pool of the per-system leg: admitted requests wait in plain_queue for a worker
    int plain_workers = 24;
    std::vector<std::thread> workers;
    std::deque<Request *> plain_queue;
    std::mutex plain_mutex;
    std::condition_variable plain_cv;
    bool stopping = false;
    // engine state
    EngineDev e{};
    RepDesc *desc_dev = nullptr;
    RepState *state_dev = nullptr;
    Tables *tabs_dev = nullptr;
    int *order_dev = nullptr, *n_work_dev = nullptr, *work_dev = nullptr, *list_dev = nullptr;
    int *launch_steps_dev = nullptr;    // steps per launch of each engine slot
    std::vector<int> launch_steps;      // the same on the host
    unsigned long long *particle_steps_dev = nullptr;
    uint64_t plain_particle_steps = 0;
    int threads = ENGINE_THREADS_MAX, blocks = 0;
    size_t smem = 0;
    std::map<int, cudaGraphExec_t> graphs;  // the engine step captured per grid size

    ~rdc_server() {
        {
            std::lock_guard<std::mutex> lock(plain_mutex);
            stopping = true;
            plain_queue.clear();  // queued requests that no worker took are dropped with the server
        }
        plain_cv.notify_all();
        for (auto &t : workers) t.join();
        if (stream) cudaStreamSynchronize(stream);
        for (auto &kv : requests)
            if (kv.second->block) cudaFreeAsync(kv.second->block, stream);
        for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
        cudaFree(desc_dev); cudaFree(state_dev); cudaFree(tabs_dev); cudaFree(order_dev);
        cudaFree(n_work_dev); cudaFree(work_dev); cudaFree(list_dev); cudaFree(particle_steps_dev);
        cudaFree(launch_steps_dev);
        if (stream) {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
    }

    template <typename T>
    T *dalloc(size_t n) {
        void *p = nullptr;
        RDC_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
        return static_cast<T *>(p);
    }

    void init(uint64_t budget_bytes, int max_act, int h, int64_t thr) {
        budget = budget_bytes;
        max_active = max_act;
        handler = h;
        plain_threshold = thr;
        RDC_CUDA(cudaGetDevice(&device));
        RDC_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        // keep freed request blocks in the stream-ordered pool for the next admissions
        cudaMemPool_t pool;
        RDC_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
        uint64_t keep = budget;
        RDC_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
        desc_dev = dalloc<RepDesc>(max_active);
        state_dev = dalloc<RepState>(max_active);
        tabs_dev = dalloc<Tables>(max_active);
        order_dev = dalloc<int>(max_active);
        list_dev = dalloc<int>(max_active);
        launch_steps_dev = dalloc<int>(max_active);
        launch_steps.assign(max_active, 1);
        RDC_CUDA(cudaMemcpyAsync(launch_steps_dev, launch_steps.data(), sizeof(int) * max_active,
                                 cudaMemcpyHostToDevice, stream));
        n_work_dev = dalloc<int>(1);
        work_dev = dalloc<int>(1);
        particle_steps_dev = dalloc<unsigned long long>(1);
        RDC_CUDA(cudaMemsetAsync(state_dev, 0, sizeof(RepState) * max_active, stream));
        RDC_CUDA(cudaMemsetAsync(n_work_dev, 0, sizeof(int), stream));
        RDC_CUDA(cudaMemsetAsync(work_dev, 0, sizeof(int), stream));
        RDC_CUDA(cudaMemsetAsync(particle_steps_dev, 0, sizeof(unsigned long long), stream));
        slot_owner.assign(max_active, 0);
        e.desc = desc_dev;
        e.state = state_dev;
        e.order = order_dev;
        e.n_work = n_work_dev;
        e.work = work_dev;
        e.tabs = tabs_dev;
        e.handler = handler;
        e.max_events_sm = ENGINE_MAX_EVENTS_SM;
        e.particle_steps = particle_steps_dev;
        e.launch_steps = launch_steps_dev;
        smem = engine_smem_bytes(e.max_events_sm);
        blocks = engine_grid(threads, smem);
        RDC_CUDA(cudaStreamSynchronize(stream));
        for (int k = 0; k < plain_workers; ++k) workers.emplace_back([this] { worker_loop(); });
    }

    // a pool worker: runs queued per-system requests one after another until the server stops
    void worker_loop() {
        for (;;) {
            Request *q = nullptr;
            {
                std::unique_lock<std::mutex> lock(plain_mutex);
                plain_cv.wait(lock, [this] { return stopping || !plain_queue.empty(); });
                if (stopping) return;
                q = plain_queue.front();
                plain_queue.pop_front();
            }
            run_plain(q, device, handler);
        }
    }

    int free_slot() const {
        for (int k = 0; k < max_active; ++k)
            if (slot_owner[k] == 0) return k;
        return -1;
    }

    // the plain leg: one simulation through the per-system C ABI on this worker thread
    static void run_plain(Request *q, int device, int handler) {
        rdc_context *ctx = nullptr;
        rdc_system *sys = nullptr;
        int rc = RDC_OK;
        cudaSetDevice(device);
        ctx = context_clone(q->ctx);
        std::vector<double> x(3 * q->n);
        std::vector<int> t(q->n);
        for (int64_t i = 0; i < q->n; ++i) {
            x[3 * i] = q->pos[i].x; x[3 * i + 1] = q->pos[i].y; x[3 * i + 2] = q->pos[i].z;
            std::memcpy(&t[i], &q->pos[i].w, 4);
        }
        const int T = q->ctx.ntypes;
        std::vector<int64_t> counts((size_t)q->max_records * T, 0);
        int64_t nrec = 0;
        uint64_t advanced = 0;
        rc = rdc_system_create(&sys, ctx, q->seed);
        if (rc == RDC_OK) rc = rdc_reserve(sys, q->cap);
        if (rc == RDC_OK) rc = rdc_add_particles(sys, q->n, x.data(), t.data(), nullptr);
        if (rc == RDC_OK && q->max_records > 0) {
            // SimulationLoop::run in chunks of whole strides (about 2000 steps): each chunk starts where the
            // last one ended (its neighbour list and forces are rebuilt from the same state, and the random
            // streams are keyed by the step counters), so the trajectory is the single run's; the first
            // record of a later chunk repeats the previous chunk's last one
            const int64_t chunk = q->stride * std::max<int64_t>(1, (2000 + q->stride - 1) / q->stride);
            std::vector<int64_t> buf;
            for (int64_t done = 0; done < q->n_steps && rc == RDC_OK;) {
                const int64_t m = std::min(chunk, q->n_steps - done);
                const int64_t cap = m / q->stride + 1;
                buf.assign((size_t)cap * T, 0);
                int64_t got = 0;
                rc = rdc_run(sys, m, q->dt, handler, q->stride, buf.data(), cap, &got);
                const int64_t first = done > 0 ? 1 : 0;
                for (int64_t r = first; r < got && nrec < q->max_records; ++r, ++nrec)
                    std::copy(buf.begin() + r * T, buf.begin() + (r + 1) * T, counts.begin() + nrec * T);
                {
                    std::lock_guard<std::mutex> g(q->partial_mutex);
                    q->partial.assign(counts.begin(), counts.begin() + nrec * T);
                    q->n_partial = nrec;
                }
                done += m;
            }
        } else if (rc == RDC_OK) {
            rc = rdc_run(sys, q->n_steps, q->dt, handler, q->stride, nullptr, 0, &nrec);
        }
        if (rc == RDC_OK) rc = rdc_get_particle_steps(sys, &advanced);  // counted on the device
        if (rc != RDC_OK) q->worker_err = rdc_last_error();
        q->particle_steps = advanced;
        if (sys) rdc_system_destroy(sys);
        rdc_context_destroy(ctx);
        q->records = std::move(counts);
        q->n_records = nrec;
        q->worker_rc = rc;
        q->worker_done.store(1);
    }

    void admit() {
        std::vector<int> new_slots;
        while (!pending.empty()) {
            Request &q = *requests[pending.front()];
            if (in_use + q.bytes > budget) break;  // first come, first served: no overtaking
            if (q.plain) {
                // at most plain_workers per-system requests admitted at once (first come, first served:
                // the queue waits behind a per-system request until a worker is free)
                if ((int)plain_running.size() >= plain_workers) break;
                in_use += q.bytes;
                q.t_admit = now_s(t0);
                pending.pop_front();
                plain_running.push_back(q.id);
                {
                    std::lock_guard<std::mutex> lock(plain_mutex);
                    plain_queue.push_back(&q);
                }
                plain_cv.notify_one();
                continue;
            }
            const int slot = free_slot();
            if (slot < 0) break;
            void *block = nullptr;
            RDC_CUDA(cudaMallocAsync(&block, q.L.total, stream));
            q.block = block;
            q.slot = slot;
            slot_owner[slot] = q.id;
            in_use += q.bytes;
            q.t_admit = now_s(t0);
            pending.pop_front();
            unsigned char *b = static_cast<unsigned char *>(block);
            RepDesc D{};
            D.geo = q.geo;
            D.pos[0] = reinterpret_cast<float4 *>(b + q.L.pos);
            D.pos[1] = D.pos[0] + q.cap;
            D.force[0] = D.pos[1] + q.cap;
            D.force[1] = D.force[0] + q.cap;
            D.id[0] = reinterpret_cast<uint32_t *>(b + q.L.id);
            D.id[1] = D.id[0] + q.cap;
            int *ints = reinterpret_cast<int *>(b + q.L.ints);
            D.bin = ints; D.rank = ints + q.cap; D.src = ints + 2 * q.cap; D.claim = ints + 3 * q.cap;
            D.taken = ints + 4 * q.cap;
            D.start = reinterpret_cast<int *>(b + q.L.start);
            D.events = reinterpret_cast<EventRec *>(b + q.L.events);
            D.records = q.max_records > 0 ? reinterpret_cast<unsigned long long *>(b + q.L.records) : nullptr;
            D.rx_counts = reinterpret_cast<unsigned long long *>(b + q.L.rx);
            D.seed = q.seed;
            D.n_steps = q.n_steps;
            D.cap = (int)q.cap;
            D.ecap = 64 + (int)(q.cap / 32);
            D.smem_cells = q.smem_cells;
            D.table = slot;
            D.count_stride = (int)q.stride;
            D.max_records = q.max_records;
            Tables tab;
            build_tables(q.ctx, q.ctx.box, q.dt, tab);
            RepState S{(int)q.n, 0, 0, (int)q.n, 0, 0, 0, 0};
            RDC_CUDA(cudaMemcpyAsync(D.pos[0], q.pos.data(), sizeof(float4) * q.n, cudaMemcpyHostToDevice, stream));
            RDC_CUDA(cudaMemsetAsync(D.claim, 0x7f, sizeof(int) * q.cap, stream));
            RDC_CUDA(cudaMemsetAsync(D.taken, 0, sizeof(int) * q.cap, stream));
            RDC_CUDA(cudaMemsetAsync(b + q.L.records, 0, q.L.rx - q.L.records, stream));
            RDC_CUDA(cudaMemsetAsync(D.rx_counts, 0, sizeof(unsigned long long) * MAX_REACTIONS, stream));
            RDC_CUDA(cudaMemcpyAsync(tabs_dev + slot, &tab, sizeof(Tables), cudaMemcpyHostToDevice, stream));
            RDC_CUDA(cudaMemcpyAsync(desc_dev + slot, &D, sizeof(RepDesc), cudaMemcpyHostToDevice, stream));
            RDC_CUDA(cudaMemcpyAsync(state_dev + slot, &S, sizeof(RepState), cudaMemcpyHostToDevice, stream));
            new_slots.push_back(slot);
            std::vector<float4>().swap(q.pos);
        }
        if (!new_slots.empty()) {
            RDC_CUDA(cudaMemcpyAsync(list_dev, new_slots.data(), sizeof(int) * new_slots.size(),
                                     cudaMemcpyHostToDevice, stream));
            launch_engine_admit(e, list_dev, (int)new_slots.size(), true, stream);
            // the pageable sources above must outlive their copies: wait here, once per admission round
            RDC_CUDA(cudaStreamSynchronize(stream));
            set_order();
        }
    }

    // work list: active engine requests, largest first
    // the engine step (k_engine_step + k_engine_reset) with `nb` CTAs, captured once per grid size
    cudaGraphExec_t graph_for(int nb) {
        nb = std::max(nb, 1);
        auto it = graphs.find(nb);
        if (it != graphs.end()) return it->second;
        cudaGraph_t g;
        cudaGraphExec_t x = nullptr;
        RDC_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        launch_engine_step(e, nb, threads, smem, stream);
        RDC_CUDA(cudaStreamEndCapture(stream, &g));
        RDC_CUDA(cudaGraphInstantiate(&x, g, 0));
        cudaGraphDestroy(g);
        graphs[nb] = x;
        return x;
    }

    // Steps per launch: a request takes as many steps as fit into one step of the largest active request
    // (by the cost model above), so that every request advances at the pace its own size allows and the
    // launches stay about one large step long.
    void set_order() {
        std::vector<int> ord;
        for (int k = 0; k < max_active; ++k)
            if (slot_owner[k]) ord.push_back(k);
        std::stable_sort(ord.begin(), ord.end(),
                         [&](int a, int b) { return requests[slot_owner[a]]->n > requests[slot_owner[b]]->n; });
        const int nw = (int)ord.size();
        if (nw > 0) {
            const double big = ENGINE_FIXED_PARTICLES + (double)requests[slot_owner[ord[0]]]->n;
            for (int k : ord) {
                const double own = ENGINE_FIXED_PARTICLES + (double)requests[slot_owner[k]]->n;
                launch_steps[k] = std::max(1, std::min(ENGINE_MAX_LAUNCH_STEPS, (int)(big / own)));
            }
            RDC_CUDA(cudaMemcpyAsync(launch_steps_dev, launch_steps.data(), sizeof(int) * max_active,
                                     cudaMemcpyHostToDevice, stream));
            RDC_CUDA(cudaMemcpyAsync(order_dev, ord.data(), sizeof(int) * nw, cudaMemcpyHostToDevice, stream));
        }
        RDC_CUDA(cudaMemcpyAsync(n_work_dev, &nw, sizeof(int), cudaMemcpyHostToDevice, stream));
        RDC_CUDA(cudaStreamSynchronize(stream));
    }

    void finish(Request &q) {
        q.finished = true;
        q.t_finish = now_s(t0);
        in_use -= q.bytes;
        unpolled.push_back(q.id);
    }

    // advance the engine requests by up to max_steps launches (stopping early when one of them finishes),
    // retire finished requests of both legs; returns the requests finished by this call
    int64_t progress(int64_t max_steps) {
        admit();
        int64_t finished = 0;
        std::vector<int64_t> active;
        for (int k = 0; k < max_active; ++k)
            if (slot_owner[k]) active.push_back(slot_owner[k]);
        if (!active.empty()) {
            // launches until the first request finishes (each launch takes a request launch_steps steps)
            int64_t K = max_steps;
            for (int64_t id : active) {
                const Request &q = *requests[id];
                const int64_t m = launch_steps[q.slot];
                K = std::min(K, (q.n_steps - q.steps_done + m - 1) / m);
            }
            K = std::max<int64_t>(K, 1);
            // as many persistent CTAs as active engine requests (one request takes one CTA at a time): the
            // other SMs stay free for the per-system workers' kernels
            cudaGraphExec_t step_graph = graph_for((int)std::min<size_t>((size_t)blocks, active.size()));
            for (int64_t k = 0; k < K; ++k) RDC_CUDA(cudaGraphLaunch(step_graph, stream));
            std::vector<RepState> st(max_active);
            RDC_CUDA(cudaMemcpyAsync(st.data(), state_dev, sizeof(RepState) * max_active, cudaMemcpyDeviceToHost,
                                     stream));
            RDC_CUDA(cudaStreamSynchronize(stream));
            bool changed = false;
            for (int64_t id : active) {
                Request &q = *requests[id];
                const RepState &s = st[q.slot];
                q.steps_done = s.step;
                if (s.status == 0 && s.step < q.n_steps) continue;
                if (s.status != 0) {
                    q.status = (s.status & (ST_CAPACITY | ST_EVENTS)) ? RDC_ERR_CAPACITY : RDC_ERR_RUNTIME;
                    q.message = "request device status " + std::to_string(s.status);
                }
                const int T = q.ctx.ntypes;
                q.n_records = std::min<int64_t>(s.rec, q.max_records);
                std::vector<unsigned long long> h((size_t)q.n_records * T);
                if (!h.empty())
                    RDC_CUDA(cudaMemcpyAsync(h.data(), static_cast<unsigned char *>(q.block) + q.L.records,
                                             sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost, stream));
                RDC_CUDA(cudaFreeAsync(q.block, stream));
                RDC_CUDA(cudaStreamSynchronize(stream));
                q.block = nullptr;
                q.records.assign(h.begin(), h.end());
                slot_owner[q.slot] = 0;
                q.slot = -1;
                finish(q);
                ++finished;
                changed = true;
            }
            if (changed) set_order();
        }
        if (active.empty() && !plain_running.empty())  // only per-system requests run: do not spin
            std::this_thread::sleep_for(std::chrono::microseconds(500));
        for (auto it = plain_running.begin(); it != plain_running.end();) {
            Request &q = *requests[*it];
            if (q.worker_done.load()) {
                q.status = q.worker_rc;
                q.message = q.worker_err;
                plain_particle_steps += q.particle_steps;  // counted on the device by the integrator
                finish(q);
                ++finished;
                it = plain_running.erase(it);
            } else {
                ++it;
            }
        }
        admit();
        return finished;
    }
};

namespace {
template <typename F>
int sguard(F &&f) {
    try {
        f();
        return RDC_OK;
    } catch (const rdc::CapacityError &e) {
        s_err = e.what();
        return RDC_ERR_CAPACITY;
    } catch (const rdc::CudaError &e) {
        s_err = e.what();
        return RDC_ERR_CUDA;
    } catch (const std::invalid_argument &e) {
        s_err = e.what();
        return RDC_ERR_INVALID_ARGUMENT;
    } catch (const std::logic_error &e) {
        s_err = e.what();
        return RDC_ERR_LOGIC;
    } catch (const std::exception &e) {
        s_err = e.what();
        return RDC_ERR_RUNTIME;
    }
}

// device bytes a request holds while active, and the leg it takes
size_t request_bytes(const ContextData &c, int64_t n, int64_t n_steps, int64_t stride, int64_t plain_threshold,
                     bool &plain, Geo &geo, int &smem_cells, EngineLayout &L, int &max_records) {
    const int64_t cap = request_capacity(n);
    max_records = stride > 0 ? (int)std::min<int64_t>(n_steps / stride + 1, INT_MAX / 64) : 0;
    plain = plain_threshold > 0 && n > plain_threshold;
    geo = replica_geo(c.box, c.pbc, c.max_cutoff(), 1.0, cap, smem_cells);
    if (plain) return plain_bytes(cap, geo.ncells, max_records, c.ntypes);
    L = engine_layout(cap, geo.ncells, 64 + (int)(cap / 32), max_records, c.ntypes);
    return L.total;
}
}  // namespace

#define SERVE_CALL(...)                                   \
    do {                                                  \
        int rc_ = sguard([&] { __VA_ARGS__; });           \
        if (rc_ != RDC_OK) rdc::set_last_error(s_err);    \
        return rc_;                                       \
    } while (0)

extern "C" {

int rdc_server_create(rdc_server **out, uint64_t budget_bytes, int max_active, int handler, int64_t plain_threshold) {
    SERVE_CALL({
        if (!out) throw std::invalid_argument("null argument");
        if (budget_bytes == 0) throw std::invalid_argument("device-memory budget must be > 0");
        if (max_active <= 0 || max_active > (1 << 16)) throw std::invalid_argument("max_active must be in [1, 65536]");
        if (handler != H_UNCONTROLLED_APPROXIMATION && handler != H_GILLESPIE)
            throw std::invalid_argument("unknown reaction handler");
        if (plain_threshold < 0) throw std::invalid_argument("plain_threshold must be >= 0");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            throw rdc::CudaError("no CUDA device available");
        }
        auto s = std::make_unique<rdc_server>();
        s->init(budget_bytes, max_active, handler, plain_threshold);
        *out = s.release();
    });
}

int rdc_server_set_plain_workers(rdc_server *s, int n) {
    SERVE_CALL({
        if (!s) throw std::invalid_argument("null argument");
        if (n < 1 || n > 256) throw std::invalid_argument("plain workers must be in [1, 256]");
        // the pool only grows; a smaller number lowers how many per-system requests are admitted at once
        while ((int)s->workers.size() < n) s->workers.emplace_back([s] { s->worker_loop(); });
        s->plain_workers = n;
    });
}

int rdc_server_destroy(rdc_server *s) {
    delete s;
    return RDC_OK;
}

int rdc_server_request_bytes(const rdc_context *ctx, int64_t n, int64_t n_steps, int64_t count_stride,
                             int64_t plain_threshold, uint64_t *bytes, int *plain) {
    SERVE_CALL({
        if (!ctx || !bytes) throw std::invalid_argument("null argument");
        if (n < 0 || n_steps < 0 || count_stride < 0) throw std::invalid_argument("negative size");
        bool p;
        Geo g;
        int sm, mr;
        EngineLayout L;
        *bytes = request_bytes(context_data(ctx), n, n_steps, count_stride, plain_threshold, p, g, sm, L, mr);
        if (plain) *plain = p ? 1 : 0;
    });
}

int rdc_server_submit(rdc_server *s, const rdc_context *ctx, int64_t n, const double *positions3, const int *types,
                      int64_t n_steps, double dt, int64_t count_stride, uint64_t seed, int64_t *request_id) {
    SERVE_CALL({
        if (!s || !ctx || !request_id || (n > 0 && (!positions3 || !types))) throw std::invalid_argument("null argument");
        if (n < 0 || n > INT_MAX / 4) throw std::invalid_argument("particle count out of range");
        if (n_steps < 0) throw std::invalid_argument("n_steps must be >= 0");
        if (!(dt > 0)) throw std::invalid_argument("time step must be > 0");
        if (count_stride < 0) throw std::invalid_argument("count_stride must be >= 0");
        auto q = std::make_unique<Request>();
        q->ctx = context_data(ctx);
        q->n = n;
        q->n_steps = n_steps;
        q->dt = dt;
        q->stride = count_stride;
        q->seed = seed;
        q->cap = request_capacity(n);
        q->bytes = request_bytes(q->ctx, n, n_steps, count_stride, s->plain_threshold, q->plain, q->geo,
                                 q->smem_cells, q->L, q->max_records);
        if (q->bytes > s->budget)
            throw std::invalid_argument("request needs " + std::to_string(q->bytes) + " device bytes, more than the budget of " +
                                        std::to_string(s->budget));
        q->pos.resize(n);
        for (int64_t i = 0; i < n; ++i) {
            const int t = types[i];
            if (t < 0 || t >= q->ctx.ntypes) throw std::invalid_argument("particle type out of range");
            float4 p;
            p.x = (float)positions3[3 * i]; p.y = (float)positions3[3 * i + 1]; p.z = (float)positions3[3 * i + 2];
            std::memcpy(&p.w, &t, 4);
            q->pos[i] = p;
        }
        q->id = s->next_id++;
        q->t_submit = now_s(s->t0);
        *request_id = q->id;
        s->pending.push_back(q->id);
        s->requests[q->id] = std::move(q);
    });
}

int rdc_server_progress(rdc_server *s, int64_t max_steps, int64_t *n_finished) {
    SERVE_CALL({
        if (!s) throw std::invalid_argument("null argument");
        if (max_steps <= 0) throw std::invalid_argument("max_steps must be > 0");
        const int64_t f = s->progress(max_steps);
        if (n_finished) *n_finished = f;
    });
}

int rdc_server_poll(rdc_server *s, int64_t capacity, int64_t *ids, int64_t *n_out) {
    SERVE_CALL({
        if (!s || !n_out || (capacity > 0 && !ids)) throw std::invalid_argument("null argument");
        const int64_t k = std::min<int64_t>(capacity, (int64_t)s->unpolled.size());
        for (int64_t i = 0; i < k; ++i) ids[i] = s->unpolled[i];
        s->unpolled.erase(s->unpolled.begin(), s->unpolled.begin() + k);
        *n_out = k;
    });
}

int rdc_server_result(rdc_server *s, int64_t id, int64_t capacity, int64_t *counts, int64_t *n_records, int *status,
                      double *times3) {
    SERVE_CALL({
        if (!s) throw std::invalid_argument("null argument");
        auto it = s->requests.find(id);
        if (it == s->requests.end()) throw std::invalid_argument("unknown request id");
        Request &q = *it->second;
        if (times3) { times3[0] = q.t_submit; times3[1] = q.t_admit; times3[2] = q.t_finish; }
        if (status) *status = q.finished ? q.status : -1;
        if (!q.finished) {
            if (n_records) *n_records = 0;
            return;
        }
        const int64_t need = q.n_records * q.ctx.ntypes;
        if (n_records) *n_records = q.n_records;
        if (counts) {
            if (capacity < need) throw rdc::CapacityError("count buffer too small for the request's records");
            for (int64_t k = 0; k < need; ++k) counts[k] = q.records[k];
        }
    });
}

int rdc_server_peek_records(rdc_server *s, int64_t id, int64_t capacity, int64_t *counts, int64_t *n_records) {
    SERVE_CALL({
        if (!s) throw std::invalid_argument("null argument");
        auto it = s->requests.find(id);
        if (it == s->requests.end()) throw std::invalid_argument("unknown request id");
        Request &q = *it->second;
        const int T = q.ctx.ntypes;
        std::vector<int64_t> h;
        int64_t n = 0;
        if (q.finished) {
            n = q.n_records;
            h.assign(q.records.begin(), q.records.begin() + n * T);
        } else if (q.plain) {
            std::lock_guard<std::mutex> g(q.partial_mutex);
            n = q.n_partial;
            h = q.partial;
        } else if (q.slot >= 0) {
            // the engine is idle between rdc_server_progress calls: its records so far, on the server's stream
            RepState st{};
            RDC_CUDA(cudaMemcpyAsync(&st, s->state_dev + q.slot, sizeof(RepState), cudaMemcpyDeviceToHost, s->stream));
            RDC_CUDA(cudaStreamSynchronize(s->stream));
            n = std::min<int64_t>(st.rec, q.max_records);
            std::vector<unsigned long long> u((size_t)n * T);
            if (n > 0)
                RDC_CUDA(cudaMemcpyAsync(u.data(), static_cast<unsigned char *>(q.block) + q.L.records,
                                         sizeof(unsigned long long) * u.size(), cudaMemcpyDeviceToHost, s->stream));
            RDC_CUDA(cudaStreamSynchronize(s->stream));
            h.assign(u.begin(), u.end());
        }
        if (n_records) *n_records = n;
        if (counts) {
            if (capacity < n * T) throw rdc::CapacityError("count buffer too small for the request's records");
            for (int64_t k = 0; k < n * T; ++k) counts[k] = h[k];
        }
    });
}

int rdc_server_release(rdc_server *s, int64_t id) {
    SERVE_CALL({
        if (!s) throw std::invalid_argument("null argument");
        auto it = s->requests.find(id);
        if (it == s->requests.end()) throw std::invalid_argument("unknown request id");
        if (!it->second->finished) throw std::logic_error("request has not finished");
        s->requests.erase(it);
    });
}

int rdc_server_stats(rdc_server *s, uint64_t *particle_steps, uint64_t *bytes_in_use, int64_t *n_active,
                     int64_t *n_pending) {
    SERVE_CALL({
        if (!s) throw std::invalid_argument("null argument");
        if (particle_steps) {
            unsigned long long v = 0;
            RDC_CUDA(cudaMemcpyAsync(&v, s->particle_steps_dev, sizeof(v), cudaMemcpyDeviceToHost, s->stream));
            RDC_CUDA(cudaStreamSynchronize(s->stream));
            *particle_steps = v + s->plain_particle_steps;
        }
        if (bytes_in_use) *bytes_in_use = s->in_use;
        if (n_active) {
            int64_t a = (int64_t)s->plain_running.size();
            for (int64_t o : s->slot_owner) a += o != 0;
            *n_active = a;
        }
        if (n_pending) *n_pending = (int64_t)s->pending.size();
    });
}

}  // extern "C"

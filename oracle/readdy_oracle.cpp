/*
 * TEST INFRASTRUCTURE ONLY -- not part of the product.
 *
 * FP64 CPU restatement of the ReaDDy CPU-kernel hot path.  It is the checker that the CUDA path is
 * compared against (tests/, __graft_entry__.smoke(), and the timed cpu_baseline leg of bench.py).
 * Every function names the reference file:line whose behaviour it restates.  Paths are relative to
 * the readdy/readdy project root.
 *
 * Differences from the reference, all deliberate and limited to what cannot be reproduced:
 *   - random numbers come from seeded std::mt19937_64 streams (one per worker thread) instead of
 *     the unseedable thread_local generators of include/readdy/model/RandomProvider.h:55-97;
 *   - the serial cell-list fill is used (CellLinkedList.cpp:171-184) so that iteration order is
 *     reproducible; the parallel CAS fill (:186-228) builds the same cell membership;
 *   - particle ids come from a per-system counter instead of the process-global one
 *     (include/readdy/model/Particle.h:112-114).
 * Build with -ffp-contract=off so that x86-64 and aarch64 round identically.
 */
#include "readdy_oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <utility>
#include <vector>

namespace {

thread_local std::string g_err;

struct V3 {
    double x = 0, y = 0, z = 0;
    double &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator/(V3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 &operator+=(V3 &a, V3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
inline V3 &operator-=(V3 &a, V3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
/* dot product with the accumulation order of std::inner_product (ReaDDyVec3.h:332-334) */
inline double dot(V3 a, V3 b) { double r = 0; r += a.x * b.x; r += a.y * b.y; r += a.z * b.z; return r; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }

/* include/readdy/common/boundary_condition_operations.h:53-80 */
struct Box {
    double L[3];
    bool pbc[3];
    void fix(V3 &v) const {
        for (int d = 0; d < 3; ++d) {
            if (pbc[d]) {
                while (v[d] >= .5 * L[d]) v[d] -= L[d];
                while (v[d] < -.5 * L[d]) v[d] += L[d];
            }
        }
    }
    V3 apply(V3 v) const { fix(v); return v; }
    V3 shortest(V3 lhs, V3 rhs) const {
        V3 dv = rhs - lhs;
        for (int i = 0; i < 3; ++i) {
            if (pbc[i]) {
                if (dv[i] > L[i] * .5) dv[i] -= L[i];
                else if (dv[i] <= -L[i] * .5) dv[i] += L[i];
            }
        }
        return dv;
    }
    double dist2(V3 lhs, V3 rhs) const { V3 d = shortest(lhs, rhs); return dot(d, d); }
};

enum Pot1Kind { P1_BOX = 0, P1_SPHERE = 1, P1_CAPSULE = 2, P1_SPHERICAL_BARRIER = 3, P1_CYLINDER = 4 };

/* order-1 (external) potentials, include/readdy/model/potentials/PotentialsOrder1.h:60-225 with the
 * geometries of include/readdy/model/geometry.h */
struct Pot1 {
    int kind;
    bool inclusion;
    double k = 0;
    V3 a, b;            // box v0/v1; sphere/capsule/barrier/cylinder centre or origin in a; direction/normal in b
    double radius = 0, length = 0, height = 0, width = 0, r1 = 0, r2 = 0, r3 = 0, r4 = 0, keff = 0;

    /* geometry::Sphere::smallestDifference, geometry.h:25-49 */
    static V3 sphereDiff(V3 center, double radius, V3 position, bool inclusion) {
        V3 delta = position - center;
        double d2 = dot(delta, delta);
        if (inclusion) {
            if (d2 < radius * radius) return {0, 0, 0};
            double d = std::sqrt(d2);
            return delta * (d - radius) / d;
        }
        if (d2 > radius * radius) return {0, 0, 0};
        double nrm = std::sqrt(d2);
        if (nrm < 1e-5) return {-radius, 0, 0};
        return (nrm - radius) * delta / norm(delta);
    }
    /* geometry::Box::smallestDifference, geometry.h:77-116 */
    V3 boxDiff(V3 x) const {
        V3 diff{0, 0, 0};
        if (inclusion) {
            for (int d = 0; d < 3; ++d) {
                if (x[d] < a[d]) diff[d] = x[d] - a[d];
                else if (x[d] > b[d]) diff[d] = x[d] - b[d];
            }
            return diff;
        }
        bool inside = true;
        for (int d = 0; d < 3; ++d) inside = inside && x[d] > a[d] && x[d] < b[d];
        if (!inside) return diff;
        double diffs[6];
        for (int d = 0; d < 3; ++d) { diffs[2 * d] = std::abs(x[d] - a[d]); diffs[2 * d + 1] = std::abs(x[d] - b[d]); }
        int ix = (int)(std::min_element(diffs, diffs + 6) - diffs);
        diff[ix / 2] = (ix % 2 == 0) ? x[ix / 2] - a[ix / 2] : x[ix / 2] - b[ix / 2];
        return diff;
    }
    /* geometry::Capsule::closestCircleCenter, geometry.h:132-150 */
    V3 capsuleCenter(V3 x) const {
        V3 nd = b / norm(b);
        V3 v = dot(x - a, nd) * nd;
        double lambda = norm(v);
        auto differ = [](double t1, double t2) { return (t1 >= 0 && t2 < 0) || (t1 < 0 && t2 >= 0); };
        if (differ(v.x, nd.x) || differ(v.y, nd.y) || differ(v.z, nd.z)) lambda = -lambda;
        lambda = std::clamp(lambda, -length / 2, length / 2);
        return a + lambda * nd;
    }
    V3 geometryDiff(V3 x) const {
        if (kind == P1_BOX) return boxDiff(x);
        if (kind == P1_SPHERE) return sphereDiff(a, radius, x, inclusion);
        return sphereDiff(capsuleCenter(x), radius, x, inclusion);
    }
    /* calculateForceAndEnergy of each class: force += F, energy += E */
    void forceEnergy(V3 x, V3 &force, double &energy) const {
        if (kind == P1_BOX || kind == P1_SPHERE || kind == P1_CAPSULE) {  // HarmonicGeometryPotential, :66-74
            V3 d = geometryDiff(x);
            energy += 0.5 * k * dot(d, d);
            force += -1 * k * d;
            return;
        }
        if (kind == P1_SPHERICAL_BARRIER) {  // SphericalBarrier, :103-146
            V3 diff = x - a;
            double dist = norm(diff);
            if (dist < r1 || r4 <= dist) return;
            if (dist < r2) {
                energy += 0.5 * keff * std::pow(dist - radius + width, 2.);
                force += -keff * (dist - radius + width) * diff / dist;
            } else if (dist < r3) {
                energy += height - 0.5 * keff * std::pow(dist - radius, 2.);
                force += keff * (dist - radius) * diff / dist;
            } else {
                energy += 0.5 * keff * std::pow(dist - radius - width, 2.);
                force += -keff * (dist - radius - width) * diff / dist;
            }
            return;
        }
        // Cylinder, :168-209
        V3 pos = x - a;
        V3 perp = pos - dot(pos, b) * b;
        double dist = norm(perp);
        if ((inclusion && dist > radius) || (!inclusion && dist < radius)) {
            energy += 0.5 * k * std::pow(dist - radius, 2.);
            force += -k * (dist - radius) * perp / dist;
        }
    }
};

enum PotKind { HARMONIC_REPULSION = 0, WEAK_PIECEWISE_HARMONIC = 1, LENNARD_JONES = 2, SCREENED_ELECTROSTATICS = 3 };

struct Pot2 {
    int kind;
    double p[8];
    double cutoff2;

    /* include/readdy/model/potentials/PotentialsOrder2.h, one branch per potential class */
    double energy(V3 x) const {
        switch (kind) {
            case HARMONIC_REPULSION: {  // :73-82
                double k = p[0], d = p[1], d2 = p[2];
                double s = dot(x, x);
                if (s < d2) {
                    s = std::sqrt(s);
                    s -= d;
                    s *= s;
                    return 0.5 * s * k;
                }
                return 0;
            }
            case WEAK_PIECEWISE_HARMONIC: {  // :131-154
                double k = p[0], d0 = p[1], depth = p[2], rc = p[3];
                const double dist = std::sqrt(dot(x, x));
                const double len2 = rc - d0;
                if (dist < d0) return .5 * k * (dist - d0) * (dist - d0) - depth;
                if (dist < d0 + .5 * len2)
                    return .5 * depth * (1. / (.5 * len2)) * (1. / (.5 * len2)) * (dist - d0) * (dist - d0) - depth;
                if (dist < rc) return -.5 * depth * (1. / (.5 * len2)) * (1. / (.5 * len2)) * (dist - rc) * (dist - rc);
                return 0;
            }
            case LENNARD_JONES: {  // :240-244, 262-264
                double m = p[0], n = p[1], rc = p[2], shift = p[3], sigma = p[5], kk = p[6];
                const double r = norm(x);
                if (r > rc) return 0;
                auto e = [&](double rr) { return kk * (std::pow(sigma / rr, m) - std::pow(sigma / rr, n)); };
                return shift != 0 ? e(r) - e(rc) : e(r);
            }
            case SCREENED_ELECTROSTATICS: {  // :291-296
                double C = p[0], kappa = p[1], D = p[2], sigma = p[3], ex = p[4];
                const double r = norm(x);
                double res = C * std::exp(-kappa * r) / r;
                res += D * std::pow(sigma / r, ex);
                return res;
            }
        }
        return 0;
    }

    void force(V3 &f, V3 x) const {
        switch (kind) {
            case HARMONIC_REPULSION: {  // :84-91
                double k = p[0], d = p[1], d2 = p[2];
                double s = dot(x, x);
                if (s < d2 && s > 0) {
                    s = std::sqrt(s);
                    f += ((k * (s - d)) / s) * x;
                }
                return;
            }
            case WEAK_PIECEWISE_HARMONIC: {  // :156-183
                double k = p[0], d0 = p[1], depth = p[2], rc = p[3];
                const double dist = std::sqrt(dot(x, x));
                const double len2 = rc - d0;
                double factor = 0;
                if (dist < d0) {
                    factor = -1 * k * (d0 - dist);
                } else if (dist < d0 + .5 * len2) {
                    factor = -1. * depth * (1. / (.5 * len2)) * (1. / (.5 * len2)) * (d0 - dist);
                } else if (dist < rc) {
                    factor = depth * (1. / (.5 * len2)) * (1. / (.5 * len2)) * (rc - dist);
                }
                if (dist > 0 && factor != 0) f += (factor * x) / dist;
                return;
            }
            case LENNARD_JONES: {  // :246-253
                double m = p[0], n = p[1], rc = p[2], sigma = p[5], kk = p[6];
                const double r = norm(x);
                if (r <= rc) {
                    double s = -1. * kk * (1 / (sigma * sigma)) *
                               (m * std::pow(sigma / r, m + 2) - n * std::pow(sigma / r, n + 2));
                    f += s * x;
                }
                return;
            }
            case SCREENED_ELECTROSTATICS: {  // :298-305
                double C = p[0], kappa = p[1], D = p[2], sigma = p[3], ex = p[4];
                double r = norm(x);
                double ff = C * std::exp(-kappa * r);
                ff *= (kappa / r + 1. / std::pow(r, 2.));
                ff += D * ex / sigma * std::pow(sigma / r, ex + 1.);
                f += ff * ((-1. * x) / r);
                return;
            }
        }
    }
};

enum ReactionKind { CONVERSION = 0, FUSION = 1, FISSION = 2, ENZYMATIC = 3, DECAY = 4 };

struct Reaction {
    int kind, id;
    int educts[2] = {0, 0}, products[2] = {0, 0};
    int nEducts, nProducts;
    double rate, eductDistance = 0, eductDistance2 = 0, productDistance = 0, w1 = .5, w2 = .5;
};

struct Entry {
    V3 pos, force;
    double fscale = 0;  // sum of the magnitudes of the force terms acting on the particle
    uint64_t id = 0;
    int type = 0;
    bool deactivated = false;
};

struct Event {  // kernels/cpu .. reactions/Event.h:51-67
    int nEducts, nProducts;
    size_t idx1, idx2;
    size_t reactionIndex;
    int t1, t2;
    double rate, cumulativeRate;
};

struct Bond { size_t i, j; double k, l0; };
struct Angle { size_t i, j, k; double kf, theta0; };
struct Dihedral { size_t i, j, k, l; double kf, mult, phi0; };

/* a small fork/join pool standing in for ctpl::thread_pool (include/readdy/common/thread/ctpl.h) */
class Pool {
public:
    explicit Pool(int n) : n_(std::max(1, n)) {
        for (int t = 1; t < n_; ++t) workers_.emplace_back([this, t] { loop(t); });
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> g(m_);
            stop_ = true;
            ++gen_;
        }
        cv_.notify_all();
        for (auto &w : workers_) w.join();
    }
    int size() const { return n_; }
    /* runs fn(tid) on every thread, tid 0 on the caller, and joins */
    void run(const std::function<void(int)> &fn) {
        if (n_ == 1) { fn(0); return; }
        {
            std::lock_guard<std::mutex> g(m_);
            job_ = &fn;
            pending_ = n_ - 1;
            ++gen_;
        }
        cv_.notify_all();
        fn(0);
        std::unique_lock<std::mutex> l(m_);
        done_.wait(l, [this] { return pending_ == 0; });
        job_ = nullptr;
    }

private:
    void loop(int tid) {
        uint64_t seen = 0;
        for (;;) {
            const std::function<void(int)> *job;
            {
                std::unique_lock<std::mutex> l(m_);
                cv_.wait(l, [&] { return gen_ != seen; });
                seen = gen_;
                if (stop_) return;
                job = job_;
            }
            (*job)(tid);
            {
                std::lock_guard<std::mutex> g(m_);
                if (--pending_ == 0) done_.notify_one();
            }
        }
    }
    int n_;
    std::vector<std::thread> workers_;
    std::mutex m_;
    std::condition_variable cv_, done_;
    const std::function<void(int)> *job_ = nullptr;
    int pending_ = 0;
    uint64_t gen_ = 0;
    bool stop_ = false;
};

inline std::pair<size_t, size_t> chunk(size_t n, int parts, int t) {
    size_t g = n / parts;
    size_t b = g * t, e = (t == parts - 1) ? n : b + g;
    return {b, e};
}

}  // namespace

struct orc_recipe {
    struct Op {
        int kind;
        int64_t a, b;
        int type;
        std::vector<int64_t> neighbors;
        double pos[3];
    };
    std::vector<Op> ops;
};

struct orc_system {
    Box box;
    double kbt;
    std::vector<double> D;
    int nTypes;
    std::map<std::pair<int, int>, std::vector<Pot2>> pot2;          // symmetric key (min,max)
    std::vector<std::vector<Pot1>> pot1;                           // by type
    bool recordVirial = false;                                      // Context::recordVirial (Context.h:168-174)
    double virial[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};                 // StateModel::virial(), row-major
    std::vector<std::vector<const Reaction *>> o1;                 // by type
    std::map<std::pair<int, int>, std::vector<const Reaction *>> o2;  // symmetric key
    std::vector<Reaction *> reactions;
    std::vector<int64_t> reactionCounts;
    std::vector<Bond> bonds;
    std::vector<Angle> angles;
    std::vector<Dihedral> dihedrals;
    // terms given explicitly (orc_add_harmonic_bonds and friends); configureTopologies keeps them
    std::vector<Bond> fixedBonds;
    std::vector<Angle> fixedAngles;
    std::vector<Dihedral> fixedDihedrals;

    // TopologyRegistry potential configuration (include/readdy/api/PotentialConfiguration.h:136-161) and
    // particle flavors (ParticleTypeRegistry.h:58-63)
    struct BondCfg { int t1, t2; double k, l0; };
    struct AngleCfg { int t1, t2, t3; double k, theta0; };
    struct DihedralCfg { int t1, t2, t3, t4; double k, mult, phi0; };
    std::vector<BondCfg> bondCfg;
    std::vector<AngleCfg> angleCfg;
    std::vector<DihedralCfg> dihedralCfg;
    std::vector<int> flavor;
    // topologies: type, vertices (particle ids, in vertex order) and edges (vertex pairs)
    struct Graph {
        int type = 0;
        std::vector<uint64_t> ids;
        std::vector<std::pair<int, int>> edges;
    };
    std::vector<Graph> graphs;
    uint64_t breakCalls = 0;

    /* spatial topology reactions (SpatialTopologyReaction.h:64-191), STRMode order */
    struct Spatial {
        int mode;
        int t1, tt1, t2, tt2, to1, tto1, to2, tto2;
        double rate, radius;
        int minGraphDistance;
        orc_spatial_rate_fn rateFn = nullptr;  // topology-topology reactions: rate(top1, top2)
        void *rateUser = nullptr;
        bool allowSelf() const { return mode == 2; }
        bool fusion() const { return mode == 1 || mode == 2 || mode == 4; }
        bool tp() const { return tt2 == -1; }
    };
    std::vector<Spatial> spatial;
    bool legacySelfFusion = false;
    std::vector<int64_t> spatialCounts;

    /* structural reactions: functions of the caller (StructuralTopologyReaction.h), rates cached per
     * topology until it changes (GraphTopology::updateReactionRates) */
    struct Structural {
        int topologyType;
        orc_topology_rate_fn rate;
        orc_topology_recipe_fn reaction;
        void *user;
        bool expectConnected;
    };
    std::vector<Structural> structural;
    std::vector<int64_t> structuralCounts;
    std::vector<std::vector<double>> graphRates;  // per graph; empty = to be evaluated

    std::vector<Entry> entries;
    std::vector<size_t> blanks;
    uint64_t nextId = 0;
    double energy = 0;

    // CompactCellLinkedList (CellLinkedList.cpp)
    int radius;
    bool nlSetUp = false;
    double nlCutoff = 0;
    size_t dims[3] = {1, 1, 1};
    double cellSize[3] = {1, 1, 1};
    std::vector<std::vector<size_t>> adjacency;
    std::vector<size_t> head, list;

    Pool pool;
    std::vector<std::mt19937_64> rng;

    orc_system(const double b[3], const int p[3], double kbt_, int nt, const double *diff, uint64_t seed, int nthreads,
               int r)
        : kbt(kbt_), nTypes(nt), radius(r), pool(nthreads) {
        for (int d = 0; d < 3; ++d) { box.L[d] = b[d]; box.pbc[d] = p[d] != 0; }
        D.assign(diff, diff + nt);
        flavor.assign(nt, 0);
        o1.resize(nt);
        pot1.resize(nt);
        std::seed_seq ss{(uint32_t)(seed & 0xffffffffu), (uint32_t)(seed >> 32), 0x5eedu};
        std::vector<uint32_t> seeds(pool.size());
        ss.generate(seeds.begin(), seeds.end());
        for (int t = 0; t < pool.size(); ++t) rng.emplace_back(seeds[t] ^ (uint64_t(t) << 32));
    }
    ~orc_system() { for (auto r : reactions) delete r; }

    using IdMap = std::unordered_map<uint64_t, size_t>;
    IdMap idMap() const {
        IdMap m;
        for (size_t i = 0; i < entries.size(); ++i)
            if (!entries[i].deactivated) m[entries[i].id] = i;
        return m;
    }
    static size_t indexOf(const IdMap &m, uint64_t id) {
        auto it = m.find(id);
        if (it == m.end()) throw std::invalid_argument("no active particle with id " + std::to_string(id));
        return it->second;
    }

    /* GraphTopology::configure (readdy/main/model/topologies/GraphTopology.cpp:59-143) over
     * Graph::findNTuples (include/graphs/bits/Graph_detail.h:39-76); the configuration lookups are
     * reversal-symmetric (PotentialConfiguration.h:136-161) */
    void configureGraph(const Graph &g, const IdMap &ids) {
        const size_t n = g.ids.size();
        std::vector<std::vector<int>> nbrs(n);
        for (auto &e : g.edges) {
            nbrs[e.first].push_back(e.second);
            nbrs[e.second].push_back(e.first);
        }
        std::vector<size_t> pidx(n);
        std::vector<int> ty(n);
        for (size_t v = 0; v < n; ++v) {
            pidx[v] = indexOf(ids, g.ids[v]);
            ty[v] = entries[pidx[v]].type;
        }
        auto pair_cb = [&](int a, int b) {
            bool found = false;
            for (auto &c : bondCfg)
                if ((c.t1 == ty[a] && c.t2 == ty[b]) || (c.t1 == ty[b] && c.t2 == ty[a])) {
                    bonds.push_back(Bond{pidx[a], pidx[b], c.k, c.l0});
                    found = true;
                }
            if (!found) throw std::invalid_argument("an edge has no bond configured");
        };
        auto triple_cb = [&](int a, int b, int c3) {
            for (auto &c : angleCfg)
                if ((c.t1 == ty[a] && c.t2 == ty[b] && c.t3 == ty[c3]) || (c.t1 == ty[c3] && c.t2 == ty[b] && c.t3 == ty[a]))
                    angles.push_back(Angle{pidx[a], pidx[b], pidx[c3], c.k, c.theta0});
        };
        auto quad_cb = [&](int a, int b, int c3, int d4) {
            for (auto &c : dihedralCfg) {
                const bool fwd = c.t1 == ty[a] && c.t2 == ty[b] && c.t3 == ty[c3] && c.t4 == ty[d4];
                const bool bwd = c.t1 == ty[d4] && c.t2 == ty[c3] && c.t3 == ty[b] && c.t4 == ty[a];
                if (fwd || bwd) dihedrals.push_back(Dihedral{pidx[a], pidx[b], pidx[c3], pidx[d4], c.k, c.mult, c.phi0});
            }
        };
        std::vector<char> visited(n, 0);
        for (size_t v1 = 0; v1 < n; ++v1) {
            visited[v1] = 1;
            for (int v2 : nbrs[v1]) {
                if (!visited[v2]) {
                    pair_cb((int)v1, v2);
                    for (int v3 : nbrs[v1])
                        if (v3 != v2)
                            for (int v4 : nbrs[v2])
                                if (v4 != (int)v1 && v4 != v3) quad_cb(v3, (int)v1, v2, v4);
                }
                for (int w : nbrs[v1])
                    if (w != v2 && w < v2) triple_cb(w, (int)v1, v2);
            }
        }
    }
    void configureTopologies() {
        bonds = fixedBonds;
        angles = fixedAngles;
        dihedrals = fixedDihedrals;
        const IdMap ids = idMap();
        for (auto &g : graphs) configureGraph(g, ids);
    }

    /* CPUEvaluateTopologyReactions::perform for the spatial reactions
     * (kernels/cpu/src/actions/CPUEvaluateTopologyReactions.cpp:86-475): gatherEvents over the cells,
     * algo::performEvents (include/readdy/common/algorithm.h:62-136) with eventsDependent, and the
     * handlers handleTopologyParticleReaction / handleTopologyTopologyReaction; bonded terms derived again
     * at the end (each handler configures its topology; configure depends on the graph only). */
    struct TREvent {
        double rate, cumulativeRate;
        long g1, g2;  // topology indices (g2 = -1: topology-particle or structural)
        const Spatial *r;
        size_t idx1, idx2;  // idx1 belongs to a topology
        int structuralIndex;  // >= 0: a structural event
    };
    int64_t evaluateTopologyReactions(double dt) {
        if (spatialCounts.size() != spatial.size()) spatialCounts.assign(spatial.size(), 0);
        if (structuralCounts.size() != structural.size()) structuralCounts.assign(structural.size(), 0);
        if ((spatial.empty() && structural.empty()) || graphs.empty()) return 0;
        if (!spatial.empty() && !nlSetUp) throw std::logic_error("neighbor list not set up");
        graphRates.resize(graphs.size());
        for (size_t gi = 0; gi < graphs.size(); ++gi)
            if (graphRates[gi].empty() && !structural.empty()) {
                graphRates[gi].assign(structural.size(), 0.0);
                for (size_t k = 0; k < structural.size(); ++k)
                    if (structural[k].topologyType == graphs[gi].type)
                        graphRates[gi][k] = structural[k].rate(structural[k].user, this, (int64_t)gi);
            }
        IdMap idx = idMap();
        std::vector<long> topOf(entries.size(), -1);
        std::vector<int> vertexOf(entries.size(), -1);
        for (size_t gi = 0; gi < graphs.size(); ++gi)
            for (size_t v = 0; v < graphs[gi].ids.size(); ++v) {
                const size_t pi = indexOf(idx, graphs[gi].ids[v]);
                topOf[pi] = (long)gi;
                vertexOf[pi] = (int)v;
            }
        std::vector<char> spatialType(nTypes, 0);
        for (auto &r : spatial) spatialType[r.t1] = spatialType[r.t2] = 1;
        auto graphDistance = [&](const Graph &g, int from, int to) {
            std::vector<std::vector<int>> nb(g.ids.size());
            for (auto &e : g.edges) { nb[e.first].push_back(e.second); nb[e.second].push_back(e.first); }
            std::vector<int> dist(g.ids.size(), -1);
            std::vector<int> q{from};
            dist[from] = 0;
            for (size_t k = 0; k < q.size(); ++k)
                for (int w : nb[q[k]]) if (dist[w] < 0) { dist[w] = dist[q[k]] + 1; q.push_back(w); }
            return dist[to];
        };
        std::vector<TREvent> events;
        // gatherEvents, :199-219: the structural events first (second topology -1 and second particle 0, as
        // TREvent's defaults leave them)
        for (size_t gi = 0; gi < graphs.size() && !structural.empty(); ++gi)
            for (size_t k = 0; k < structural.size(); ++k)
                if (graphRates[gi][k] > 0)
                    events.push_back(TREvent{graphRates[gi][k], 0, (long)gi, -1, nullptr, 0, 0, (int)k});
        for (size_t cell = 0; cell < adjacency.size() && !spatial.empty(); ++cell) {
            forEachInCell(cell, [&](size_t ip) {
                const Entry &en = entries[ip];
                if (en.deactivated || !spatialType[en.type]) return;
                const bool hasEntryTop = topOf[ip] >= 0;
                forEachNeighbor(ip, cell, [&](size_t jn) {
                    const Entry &nb = entries[jn];
                    if (nb.deactivated) return;
                    const bool hasNbTop = topOf[jn] >= 0;
                    if ((!hasEntryTop && !hasNbTop) || (hasNbTop && ip > jn)) return;
                    const long tt1 = hasEntryTop ? graphs[topOf[ip]].type : -1;
                    const long tt2 = hasNbTop ? graphs[topOf[jn]].type : -1;
                    const double d2 = box.dist2(en.pos, nb.pos);
                    for (const auto &r : spatial) {
                        // spatialReactionsByType: the key matches in either order (TopologyParticleTypeMap.h:60-92)
                        const bool fwd = r.t1 == en.type && r.tt1 == tt1 && r.t2 == nb.type && r.tt2 == tt2;
                        const bool bwd = r.t1 == nb.type && r.tt1 == tt2 && r.t2 == en.type && r.tt2 == tt1;
                        if (!fwd && !bwd) continue;
                        if (!r.allowSelf() && topOf[ip] == topOf[jn]) continue;
                        if (!(d2 < r.radius * r.radius)) continue;
                        TREvent ev{r.rate, 0, -1, -1, &r, ip, jn, -1};
                        if (hasEntryTop && !hasNbTop) { ev.g1 = topOf[ip]; ev.idx1 = ip; ev.idx2 = jn; }
                        else if (!hasEntryTop && hasNbTop) { ev.g1 = topOf[jn]; ev.idx1 = jn; ev.idx2 = ip; }
                        else {
                            ev.g1 = topOf[ip];
                            ev.g2 = topOf[jn];
                            // SpatialTopologyReaction::rate(top1, top2) (SpatialTopologyReaction.h:179-191)
                            if (r.rateFn) {
                                ev.rate = r.rateFn(r.rateUser, this, (int64_t)ev.g1, (int64_t)ev.g2);
                                if (!(ev.rate >= 0.0))
                                    throw std::runtime_error("a spatial topology reaction's rate function produced "
                                                             "a rate smaller than 0");
                            }
                        }
                        if (r.allowSelf() && topOf[ip] == topOf[jn]) {
                            const int dg = graphDistance(graphs[topOf[ip]], vertexOf[ev.idx1], vertexOf[ev.idx2]);
                            if ((dg != -1 && dg <= r.minGraphDistance) || (!legacySelfFusion && dg == 1)) continue;
                        }
                        events.push_back(ev);
                    }
                });
            });
        }
        auto dependent = [](const TREvent &a, const TREvent &b) {  // eventsDependent, :459-468
            if (a.g1 == b.g1 || a.g1 == b.g2) return true;
            if (a.g2 < 0 && b.g2 < 0 && a.idx2 == b.idx2) return true;
            return a.g2 >= 0 && (a.g2 == b.g1 || a.g2 == b.g2);
        };
        std::vector<char> dead(graphs.size(), 0);
        std::vector<Graph> children;
        std::vector<char> changed(graphs.size(), 0);
        int64_t performed = 0;
        auto evalStructural = [&](const TREvent &ev) {  // executeStructuralReaction, Utils.h:52-81
            const Structural &sr = structural[ev.structuralIndex];
            orc_recipe recipe;
            sr.reaction(sr.user, this, (int64_t)ev.g1, &recipe);
            Graph &g = graphs[ev.g1];
            auto vtx = [&](int64_t v) {
                if (v < 0 || v >= (int64_t)g.ids.size()) throw std::invalid_argument("recipe vertex index out of range");
                return (int)v;
            };
            auto findEdge = [&](int a, int b) {
                for (size_t x = 0; x < g.edges.size(); ++x)
                    if ((g.edges[x].first == a && g.edges[x].second == b) || (g.edges[x].first == b && g.edges[x].second == a))
                        return (long)x;
                return -1L;
            };
            for (const auto &op : recipe.ops) {
                if (op.kind == 0) entries[indexOf(idx, g.ids[vtx(op.a)])].type = op.type;
                else if (op.kind == 1) {
                    const int a = vtx(op.a), b = vtx(op.b);
                    if (findEdge(a, b) < 0) g.edges.push_back({a, b});
                } else if (op.kind == 2) {
                    const long x = findEdge(vtx(op.a), vtx(op.b));
                    if (x < 0) throw std::invalid_argument("recipe: the edge to remove does not exist");
                    g.edges.erase(g.edges.begin() + x);
                } else if (op.kind == 3) {
                    const int v = vtx(op.a);
                    std::vector<std::pair<int, int>> kept;
                    for (auto &e : g.edges) if (e.first != v && e.second != v) kept.push_back(e);
                    g.edges = std::move(kept);
                } else if (op.kind == 4) {
                    g.type = op.type;
                } else if (op.kind == 5) {  // CPUAppendParticle, CPUTopologyActions.h:112-131
                    if (op.neighbors.empty()) throw std::invalid_argument("recipe: a new particle needs a neighbour");
                    std::vector<int> nb;
                    for (int64_t x : op.neighbors) nb.push_back(vtx(x));
                    Entry en;
                    en.pos = {op.pos[0], op.pos[1], op.pos[2]};
                    box.fix(en.pos);
                    en.type = op.type;
                    en.id = nextId++;
                    idx[en.id] = addEntry(en);
                    g.ids.push_back(en.id);
                    const int nvx = (int)g.ids.size() - 1;
                    for (int v : nb)
                        if (findEdge(v, nvx) < 0) g.edges.push_back({v, nvx});
                } else if (op.kind == 6) {
                    V3 p{op.pos[0], op.pos[1], op.pos[2]};
                    box.fix(p);
                    entries[indexOf(idx, g.ids[vtx(op.a)])].pos = p;
                }
            }
            const int nv = (int)g.ids.size();
            changed[ev.g1] = 1;
            std::vector<std::vector<int>> nb(nv);
            for (auto &e : g.edges) { nb[e.first].push_back(e.second); nb[e.second].push_back(e.first); }
            std::vector<int> comp(nv, -1);
            int nc = 0;
            for (int v = 0; v < nv; ++v) {
                if (comp[v] >= 0) continue;
                std::vector<int> todo{v};
                comp[v] = nc;
                while (!todo.empty()) {
                    const int u = todo.back();
                    todo.pop_back();
                    for (int w : nb[u]) if (comp[w] < 0) { comp[w] = nc; todo.push_back(w); }
                }
                ++nc;
            }
            auto normalSingle = [&](const Graph &x) {
                return x.ids.size() == 1 && flavor[entries[indexOf(idx, x.ids[0])].type] == 0;
            };
            if (nc > 1) {
                if (sr.expectConnected)
                    throw std::logic_error("The topology was expected to still be connected after the reaction");
                std::vector<Graph> parts(nc);
                std::vector<int> local(nv);
                for (int v = 0; v < nv; ++v) {
                    local[v] = (int)parts[comp[v]].ids.size();
                    parts[comp[v]].ids.push_back(g.ids[v]);
                    parts[comp[v]].type = g.type;
                }
                for (auto &e : g.edges) parts[comp[e.first]].edges.push_back({local[e.first], local[e.second]});
                for (auto &part : parts) if (!normalSingle(part)) children.push_back(std::move(part));
                dead[ev.g1] = 1;
            } else if (normalSingle(g)) {
                dead[ev.g1] = 1;
            }
            ++structuralCounts[ev.structuralIndex];
            ++performed;
        };
        auto eval = [&](const TREvent &ev) {
            if (ev.structuralIndex >= 0) { evalStructural(ev); return; }
            const Spatial &r = *ev.r;
            Entry &e1 = entries[ev.idx1];
            Entry &e2 = entries[ev.idx2];
            Graph &t1 = graphs[ev.g1];
            if (ev.g2 < 0) {  // handleTopologyParticleReaction, :322-358
                const bool first = e1.type == r.t1;
                const int n1 = first ? r.to1 : r.to2, n2 = first ? r.to2 : r.to1;
                e1.type = n1;
                e2.type = n2;
                if (r.fusion()) {
                    t1.ids.push_back(e2.id);
                    t1.edges.push_back({(int)t1.ids.size() - 1, vertexOf[ev.idx1]});
                    topOf[ev.idx2] = ev.g1;
                    vertexOf[ev.idx2] = (int)t1.ids.size() - 1;
                }
                t1.type = t1.type == r.tt1 ? r.tto1 : r.tto2;
            } else {  // handleTopologyTopologyReaction, :360-457
                Graph &t2 = graphs[ev.g2];
                if (r.fusion() && ev.g1 == ev.g2) {
                    const int a = vertexOf[ev.idx1], b = vertexOf[ev.idx2];
                    bool present = false;
                    for (auto &e : t1.edges) present |= (e.first == a && e.second == b) || (e.first == b && e.second == a);
                    if (!present) t1.edges.push_back({a, b});
                    t1.type = r.tto1;
                    const bool first = e1.type == r.t1;
                    const int n1 = first ? r.to1 : r.to2, n2 = first ? r.to2 : r.to1;
                    e1.type = n1;
                    e2.type = n2;
                } else {
                    int tto1 = r.tto1, tto2 = r.tto2;
                    if (e1.type == r.t1 && t1.type == r.tt1) { e1.type = r.to1; e2.type = r.to2; }
                    else { std::swap(tto1, tto2); e1.type = r.to2; e2.type = r.to1; }
                    if (r.fusion()) {  // GraphTopology::appendTopology: t2 joins t1 with the edge idx1 -- idx2
                        const int off = (int)t1.ids.size();
                        for (size_t v = 0; v < t2.ids.size(); ++v) {
                            t1.ids.push_back(t2.ids[v]);
                            const size_t pi = indexOf(idx, t2.ids[v]);
                            topOf[pi] = ev.g1;
                            vertexOf[pi] = off + (int)v;
                        }
                        for (auto &e : t2.edges) t1.edges.push_back({off + e.first, off + e.second});
                        t1.edges.push_back({vertexOf[ev.idx2], vertexOf[ev.idx1]});
                        t1.type = r.tto1;
                        t2.ids.clear();
                        t2.edges.clear();
                        dead[ev.g2] = 1;
                    } else {
                        t1.type = tto1;
                        t2.type = tto2;
                    }
                }
            }
            changed[ev.g1] = 1;
            if (ev.g2 >= 0) changed[ev.g2] = 1;
            ++spatialCounts[ev.r - spatial.data()];
            ++performed;
        };
        if (!events.empty()) {  // algo::performEvents
            size_t nDeact = 0;
            const size_t nEvents = events.size();
            double cum = 0;
            for (auto &ev : events) { ev.cumulativeRate = ev.rate + cum; cum = ev.cumulativeRate; }
            while (nDeact < nEvents) {
                const double cr = (events.end() - nDeact - 1)->cumulativeRate;
                const double x = uniform(0, 0., cr);
                auto it = std::lower_bound(events.begin(), events.end() - nDeact, x,
                                           [](const TREvent &e, double v) { return e.cumulativeRate < v; });
                if (it == events.end()) throw std::logic_error("performEvents: no event could be selected");
                if (coin(0, it->rate, dt)) {
                    const TREvent done = *it;
                    eval(done);
                    auto j = events.begin();
                    double cs = 0;
                    while (j < events.end() - nDeact) {
                        if (dependent(*j, done)) {
                            ++nDeact;
                            std::iter_swap(j, events.end() - nDeact);
                        } else {
                            cs += j->rate;
                            j->cumulativeRate = cs;
                            ++j;
                        }
                    }
                } else {
                    ++nDeact;
                    std::iter_swap(it, events.end() - nDeact);
                    it->cumulativeRate = it->rate;
                    if (it > events.begin()) it->cumulativeRate += (it - 1)->cumulativeRate;
                    double c2 = it->cumulativeRate;
                    for (auto j = it + 1; j < events.end() - nDeact; ++j) { c2 += j->rate; j->cumulativeRate = c2; }
                }
            }
        }
        if (performed > 0) {
            std::vector<Graph> kept;
            std::vector<std::vector<double>> keptRates;
            for (size_t gi = 0; gi < graphs.size(); ++gi)
                if (!dead[gi]) {
                    kept.push_back(std::move(graphs[gi]));
                    keptRates.push_back(changed[gi] ? std::vector<double>{} : graphRates[gi]);
                }
            for (auto &c : children) {
                kept.push_back(std::move(c));
                keptRates.emplace_back();
            }
            graphs = std::move(kept);
            graphRates = std::move(keptRates);
            configureTopologies();
        }
        return performed;
    }

    /* BreakBonds::genericPerform (include/readdy/model/actions/Actions.h:236-290): per topology and per
     * edge, the energy of the edge's bond configurations (evaluateEdgeEnergy, :292-342; harmonic bond
     * energy of BondedPotential.h) against the type pair's threshold, then a coin
     * u < 1 - exp(-rate dt); the topology without the removed edges splits into its connected
     * components (StructuralTopologyReaction.cpp:70-130), one-particle components of NORMAL flavor
     * leave the topologies (include/readdy/model/actions/Utils.h:52-81, GraphTopology.cpp:161-173) */
    int64_t breakBonds(double dt, int n, const int *t1, const int *t2, const double *thr, const double *rate) {
        std::map<std::pair<int, int>, std::pair<double, double>> cfg;  // unordered pair -> (threshold, rate)
        for (int k = 0; k < n; ++k) cfg[{std::min(t1[k], t2[k]), std::max(t1[k], t2[k])}] = {thr[k], rate[k]};
        ++breakCalls;
        int64_t removed = 0;
        const IdMap idx = idMap();
        std::vector<Graph> result;
        for (auto &g : graphs) {
            std::vector<char> gone(g.edges.size(), 0);
            for (size_t e = 0; e < g.edges.size(); ++e) {
                const Entry &a = entries[indexOf(idx, g.ids[g.edges[e].first])];
                const Entry &b = entries[indexOf(idx, g.ids[g.edges[e].second])];
                double energy = 0;
                const double d = norm(box.shortest(a.pos, b.pos));
                for (auto &c : bondCfg)
                    if ((c.t1 == a.type && c.t2 == b.type) || (c.t1 == b.type && c.t2 == a.type))
                        energy += c.k * (d - c.l0) * (d - c.l0);
                auto it = cfg.find({std::min(a.type, b.type), std::max(a.type, b.type)});
                if (it != cfg.end() && energy > it->second.first && uniform(0) < 1 - std::exp(-it->second.second * dt)) {
                    gone[e] = 1;
                    ++removed;
                }
            }
            Graph kept;
            kept.type = g.type;
            kept.ids = g.ids;
            for (size_t e = 0; e < g.edges.size(); ++e)
                if (!gone[e]) kept.edges.push_back(g.edges[e]);
            // connected components (Graph::connectedComponents), vertices in their graph order
            const size_t nv = kept.ids.size();
            std::vector<int> comp(nv, -1);
            std::vector<std::vector<int>> nb(nv);
            for (auto &e : kept.edges) { nb[e.first].push_back(e.second); nb[e.second].push_back(e.first); }
            int nc = 0;
            for (size_t v = 0; v < nv; ++v) {
                if (comp[v] >= 0) continue;
                std::vector<int> todo{(int)v};
                comp[v] = nc;
                while (!todo.empty()) {
                    int u = todo.back();
                    todo.pop_back();
                    for (int w : nb[u]) if (comp[w] < 0) { comp[w] = nc; todo.push_back(w); }
                }
                ++nc;
            }
            if (nc == 1) { result.push_back(std::move(kept)); continue; }
            std::vector<Graph> parts(nc);
            std::vector<int> local(nv);
            for (size_t v = 0; v < nv; ++v) {
                local[v] = (int)parts[comp[v]].ids.size();
                parts[comp[v]].ids.push_back(kept.ids[v]);
                parts[comp[v]].type = kept.type;
            }
            for (auto &e : kept.edges) parts[comp[e.first]].edges.push_back({local[e.first], local[e.second]});
            for (auto &part : parts) {
                const bool normal = part.ids.size() == 1 && flavor[entries[indexOf(idx, part.ids[0])].type] == 0;
                if (!normal) result.push_back(std::move(part));
            }
        }
        graphs = std::move(result);
        graphRates.clear();  // structural rates of every topology are evaluated again
        configureTopologies();
        return removed;
    }

    static std::pair<int, int> key(int a, int b) { return {std::min(a, b), std::max(a, b)}; }

    const std::vector<Pot2> *pots(int a, int b) const {
        auto it = pot2.find(key(a, b));
        return it == pot2.end() ? nullptr : &it->second;
    }
    const std::vector<const Reaction *> *reac2(int a, int b) const {
        auto it = o2.find(key(a, b));
        return it == o2.end() ? nullptr : &it->second;
    }

    double normal(int tid) { std::normal_distribution<double> nd(0., 1.); return nd(rng[tid]); }
    V3 normal3(int tid) { V3 v; v.x = normal(tid); v.y = normal(tid); v.z = normal(tid); return v; }
    double uniform(int tid, double a = 0., double b = 1.) {
        std::uniform_real_distribution<double> u(a, b);
        return u(rng[tid]);
    }

    /* Context::calculateMaxCutoff, readdy/main/model/Context.cpp:126-144 */
    double maxCutoff() const {
        double c = 0;
        for (auto &e : pot2) for (auto &p : e.second) c = std::max(c, std::sqrt(p.cutoff2));
        for (auto &e : o2) for (auto *r : e.second) c = std::max(c, r->eductDistance);
        for (auto &r : spatial) c = std::max(c, r.radius);  // Context::calculateMaxCutoff
        return c;
    }

    /* DefaultDataContainer::addParticles / addEntry, DefaultDataContainer.h:79-101 */
    size_t addEntry(const Entry &e) {
        if (!blanks.empty()) {
            size_t idx = blanks.back();
            blanks.pop_back();
            entries.at(idx) = e;
            return idx;
        }
        entries.push_back(e);
        return entries.size() - 1;
    }
    void removeEntry(size_t idx) {  // DataContainer.h:149-157
        auto &e = entries.at(idx);
        if (!e.deactivated) { e.deactivated = true; blanks.push_back(idx); }
    }

    /* CellLinkedList::setUp, kernels/cpu/src/nl/CellLinkedList.cpp:52-142 */
    void nlSetup(double cutoff) {
        if (cutoff <= 0) throw std::logic_error("The cutoff distance for setting up a neighbor list must be > 0");
        nlCutoff = cutoff;
        double width = cutoff / static_cast<double>(radius);
        for (int i = 0; i < 3; ++i) {
            dims[i] = static_cast<unsigned int>(std::max(1., std::floor(box.L[i] / width)));
            cellSize[i] = box.L[i] / static_cast<double>(dims[i]);
        }
        size_t nCells = dims[0] * dims[1] * dims[2];
        adjacency.assign(nCells, {});
        int r = radius;
        for (int i = 0; i < (int)dims[0]; ++i)
            for (int j = 0; j < (int)dims[1]; ++j)
                for (int k = 0; k < (int)dims[2]; ++k) {
                    size_t self = cellIndex(i, j, k);
                    std::vector<size_t> adj;
                    for (int ii = i - r; ii <= i + r; ++ii)
                        for (int jj = j - r; jj <= j + r; ++jj)
                            for (int kk = k - r; kk <= k + r; ++kk) {
                                if (ii == i && jj == j && kk == k) continue;
                                int a[3] = {ii, jj, kk};
                                bool ok = true;
                                for (int d = 0; d < 3; ++d) {
                                    int c = (int)dims[d];
                                    if (box.pbc[d]) a[d] = (a[d] % c + c) % c;
                                    if (a[d] < 0 || a[d] >= c) ok = false;
                                }
                                if (ok) adj.push_back(cellIndex(a[0], a[1], a[2]));
                            }
                    std::sort(adj.begin(), adj.end());
                    adj.erase(std::unique(adj.begin(), adj.end()), adj.end());
                    adj.erase(std::remove(adj.begin(), adj.end(), self), adj.end());
                    adjacency[self] = std::move(adj);
                }
        nlSetUp = true;
        nlUpdate();
    }
    /* row-major Index3D, include/readdy/common/Index.h:130-141 */
    size_t cellIndex(size_t i, size_t j, size_t k) const { return k + dims[2] * (j + dims[1] * i); }

    /* CompactCellLinkedList::setUpBins + fillBins<true>, CellLinkedList.cpp:161-184, 230-247 */
    void nlUpdate() {
        if (!nlSetUp) throw std::logic_error("Attempting to fill neighborlist bins, but cell structure is not set up yet");
        head.assign(adjacency.size(), 0);
        list.assign(entries.size() + 1, 0);
        size_t pidx = 1;
        for (const auto &e : entries) {
            const V3 &p = e.pos;
            bool inBox = -.5 * box.L[0] <= p.x && .5 * box.L[0] > p.x && -.5 * box.L[1] <= p.y &&
                         .5 * box.L[1] > p.y && -.5 * box.L[2] <= p.z && .5 * box.L[2] > p.z;
            if (!e.deactivated && inBox) {
                auto i = static_cast<size_t>(std::floor((p.x + .5 * box.L[0]) / cellSize[0]));
                auto j = static_cast<size_t>(std::floor((p.y + .5 * box.L[1]) / cellSize[1]));
                auto k = static_cast<size_t>(std::floor((p.z + .5 * box.L[2]) / cellSize[2]));
                size_t c = cellIndex(i, j, k);
                list[pidx] = head.at(c);
                head[c] = pidx;
            }
            ++pidx;
        }
    }
    template <typename F>
    void forEachInCell(size_t cell, F f) const {
        for (size_t s = head[cell]; s != 0; s = list[s]) f(s - 1);
    }
    /* CompactCellLinkedList::forEachNeighbor, CellLinkedList.h:304-313 */
    template <typename F>
    void forEachNeighbor(size_t particle, size_t cell, F f) const {
        forEachInCell(cell, [&](size_t x) { if (x != particle) f(x); });
        for (size_t nc : adjacency[cell]) forEachInCell(nc, f);
    }

    /* CPUCalculateForces::perform, kernels/cpu/src/actions/CPUCalculateForces.cpp:46-212 */
    double calculateForces() {
        energy = 0;
        bool any1 = false;
        for (auto &v : pot1) any1 = any1 || !v.empty();
        if (!any1 && pot2.empty() && bonds.empty() && angles.empty() && dihedrals.empty()) return 0;
        for (auto &e : entries) { e.force = {0, 0, 0}; e.fscale = 0; }
        if (any1) energy += order1();
        int nt = pool.size();
        std::vector<double> part(nt, 0.);
        if (!bonds.empty() || !angles.empty() || !dihedrals.empty()) energy += bondedForces();
        if (!pot2.empty()) {
            if (!nlSetUp) throw std::logic_error("neighbor list not set up");
            size_t nCells = adjacency.size();
            std::vector<std::array<double, 9>> vpart(nt);
            pool.run([&](int tid) {
                auto [cb, ce] = chunk(nCells, nt, tid);
                vpart[tid].fill(0.);
                part[tid] = order2(cb, ce, vpart[tid].data());
            });
            for (double p : part) energy += p;
            for (int k = 0; k < 9; ++k) {
                virial[k] = 0;
                if (recordVirial)
                    for (auto &v : vpart) virial[k] += v[k];
            }
        }
        return energy;
    }
    /* calculateOrder1, CPUCalculateForces.cpp:295-314 */
    double order1() {
        double eUpd = 0;
        for (auto &e : entries) {
            if (e.deactivated) continue;
            for (const auto &p : pot1[e.type]) {
                V3 upd{0, 0, 0};
                p.forceEnergy(e.pos, upd, eUpd);
                e.force += upd;
                e.fscale += norm(upd);
            }
        }
        return eUpd;
    }
    /* calculateOrder2<false>, CPUCalculateForces.cpp:214-268 */
    double order2(size_t cb, size_t ce, double *vir) {
        double eUpd = 0;
        for (size_t cell = cb; cell < ce; ++cell) {
            forEachInCell(cell, [&](size_t pi) {
                Entry &entry = entries[pi];
                if (entry.deactivated) return;
                forEachNeighbor(pi, cell, [&](size_t ni) {
                    const Entry &nb = entries[ni];
                    if (nb.deactivated) return;
                    double myE = 0;
                    const auto *ps = pots(entry.type, nb.type);
                    if (ps) {
                        V3 xij = box.shortest(entry.pos, nb.pos);
                        double d2 = dot(xij, xij);
                        for (const auto &pot : *ps) {
                            if (d2 < pot.cutoff2) {
                                V3 upd{0, 0, 0};
                                myE += pot.energy(xij);
                                pot.force(upd, xij);
                                entry.force += upd;
                                entry.fscale += norm(upd);
                                // calculateOrder2<true>: each pair once, outer(-x_ij, f_i) (CPUCalculateForces.cpp:247-249)
                                if (recordVirial && pi < ni)
                                    for (int a = 0; a < 3; ++a)
                                        for (int b = 0; b < 3; ++b) vir[3 * a + b] += -xij[a] * upd[b];
                            }
                        }
                    }
                    eUpd += 0.5 * myE;
                });
            });
        }
        return eUpd;
    }

    /* bonded terms, kernels/cpu/src/actions/topologies/CPUTopologyActions.cpp:55-123 */
    double bondedForces() {
        double e = 0;
        for (const auto &b : bonds) {  // :61-74, BondedPotential.h:105-113
            if (b.k == 0) continue;
            Entry &e1 = entries.at(b.i), &e2 = entries.at(b.j);
            V3 xij = box.shortest(e1.pos, e2.pos);
            const double nrm = norm(xij);
            V3 upd = (2. * b.k * (nrm - b.l0) / nrm) * xij;
            e1.force += upd;
            e2.force -= upd;
            e1.fscale += norm(upd);
            e2.fscale += norm(upd);
            const double n2 = std::sqrt(dot(xij, xij));
            e += b.k * (n2 - b.l0) * (n2 - b.l0);
        }
        for (const auto &a : angles) {  // :82-97, AnglePotential.cpp:58-104
            Entry &e1 = entries.at(a.i), &e2 = entries.at(a.j), &e3 = entries.at(a.k);
            V3 xji = box.shortest(e2.pos, e1.pos);
            V3 xjk = box.shortest(e2.pos, e3.pos);
            e += angleEnergy(xji, xjk, a);
            V3 f1{0, 0, 0}, f2{0, 0, 0}, f3{0, 0, 0};
            angleForce(f1, f2, f3, xji, xjk, a);
            e1.force += f1; e2.force += f2; e3.force += f3;
            e1.fscale += norm(f1); e2.fscale += norm(f2); e3.fscale += norm(f3);
        }
        for (const auto &d : dihedrals) {  // :106-123, TorsionPotential.cpp:53-159
            Entry &ei = entries.at(d.i), &ej = entries.at(d.j), &ek = entries.at(d.k), &el = entries.at(d.l);
            V3 xji = box.shortest(ej.pos, ei.pos);
            V3 xkj = box.shortest(ek.pos, ej.pos);
            V3 xkl = box.shortest(ek.pos, el.pos);
            e += dihedralEnergy(xji, xkj, xkl, d);
            V3 f1{0, 0, 0}, f2{0, 0, 0}, f3{0, 0, 0}, f4{0, 0, 0};
            dihedralForce(f1, f2, f3, f4, xji, xkj, xkl, d);
            ei.force += f1; ej.force += f2; ek.force += f3; el.force += f4;
            ei.fscale += norm(f1); ej.fscale += norm(f2); ek.fscale += norm(f3); el.fscale += norm(f4);
        }
        return e;
    }

    static double angleEnergy(V3 xij, V3 xkj, const Angle &a) {  // AnglePotential.cpp:58-65
        const double sp = dot(xij, xkj);
        const double th = std::acos(sp / (norm(xij) * norm(xkj)));
        return a.kf * (th - a.theta0) * (th - a.theta0);
    }
    static void angleForce(V3 &fi, V3 &fj, V3 &fk, V3 xji, V3 xjk, const Angle &a) {  // :67-102
        const double SMALL = 1e-10;
        const double sp = dot(xji, xjk);
        double nji2 = dot(xji, xji);
        if (nji2 < SMALL) nji2 = SMALL;
        const double nji = std::sqrt(nji2);
        double njk2 = dot(xjk, xjk);
        if (njk2 < SMALL) njk2 = SMALL;
        const double njk = std::sqrt(njk2);
        double np = nji * njk;
        if (np < SMALL) np = SMALL;
        const double inp = 1. / np;
        double c = inp * sp;
        c = std::min(1., std::max(-1., c));
        double sinv = std::sqrt(1. - c * c);
        if (sinv < SMALL) sinv = SMALL;
        sinv = 1. / sinv;
        const double cc = 2. * a.kf * (std::acos(c) - a.theta0) * sinv;
        const V3 f_i = cc * c * (1. / nji2) * xji - cc * inp * xjk;
        const V3 f_k = -cc * inp * xji + cc * c * (1. / njk2) * xjk;
        fi -= f_i;
        fj += f_i + f_k;
        fk -= f_k;
    }

    static double dihedralEnergy(V3 xji, V3 xkj, V3 xkl, const Dihedral &d) {  // TorsionPotential.cpp:53-68
        const double SMALL = .0001;
        const V3 xjk = -1. * xkj;
        double xjkn = norm(xjk);
        xjkn = xjkn < SMALL ? SMALL : xjkn;
        const V3 m = cross(xji, xkj);
        const double mn = norm(m);
        const V3 n = cross(xkl, xjk);
        const double nn = norm(n);
        double mnn = mn * nn;
        mnn = mnn < SMALL ? SMALL : mnn;
        const double sinT = dot(cross(m, n), xjk) / (mnn * xjkn);
        const double cosT = dot(m, n) / mnn;
        const double dih = -std::atan2(sinT, cosT);
        return d.kf * (1 + std::cos(d.mult * dih - d.phi0));
    }

    /* 3x3 "tensor" of three column vectors, include/readdy/common/Vec3Tensor.h */
    struct T3 { V3 c[3]; };
    static T3 skew(V3 v) {  // the columns written at TorsionPotential.cpp:111-112
        return T3{{V3{0, -v[2], v[1]}, V3{v[2], 0, -v[0]}, V3{-v[1], v[0], 0}}};
    }
    static T3 add(T3 a, T3 b) { return T3{{a.c[0] + b.c[0], a.c[1] + b.c[1], a.c[2] + b.c[2]}}; }
    static T3 scale(T3 a, double s) { return T3{{a.c[0] * s, a.c[1] * s, a.c[2] * s}}; }
    static V3 vecT(V3 v, T3 t) { return {dot(t.c[0], v), dot(t.c[1], v), dot(t.c[2], v)}; }  // Vec3 * Tensor

    static void dihedralForce(V3 &fi, V3 &fj, V3 &fk, V3 &fl, V3 xji, V3 xkj, V3 xkl,
                              const Dihedral &dh) {  // TorsionPotential.cpp:70-153
        const double SMALL = .0001;
        const V3 xjk = -1. * xkj;
        double xjkn2 = dot(xjk, xjk);
        xjkn2 = xjkn2 < SMALL ? SMALL : xjkn2;
        const double xjkn = std::sqrt(xjkn2);
        const V3 m = cross(xji, xkj);
        double mn2 = dot(m, m);
        mn2 = mn2 < SMALL ? SMALL : mn2;
        const double mn = std::sqrt(mn2);
        const V3 n = cross(xkl, xjk);
        double nn2 = dot(n, n);
        nn2 = nn2 < SMALL ? SMALL : nn2;
        const double nn = std::sqrt(nn2);
        double nmn = mn * nn;
        nmn = nmn < SMALL ? SMALL : nmn;
        const V3 mxn = cross(m, n);
        const double n_m = dot(n, m);
        const double cphi = n_m / nmn;
        if (std::abs(cphi) < SMALL) return;
        const double sphi = dot(cross(m, n), xjk) / (nmn * xjkn);
        const double phi = -std::atan2(sphi, cphi);
        const double dVdphi = -dh.kf * dh.mult * std::sin(dh.mult * phi - dh.phi0);
        const V3 dmn2_dxi = 2 * xjkn2 * xji - 2 * dot(xji, xkj) * xkj;
        const V3 dmn_dxi = dmn2_dxi / (2 * mn);
        const V3 dmn2_dxk = -2 * dot(xji, xji) * xkj + 2 * dot(xji, xkj) * xji;
        const V3 dmn_dxk = dmn2_dxk / (2 * mn);
        const V3 dmn2_dxj = -1. * (dmn2_dxi + dmn2_dxk);
        const V3 dmn_dxj = dmn2_dxj / (2 * mn);
        const V3 dnn2_dxl = 2 * xjkn2 * xkl - 2 * dot(xkl, xjk) * xjk;
        const V3 dnn_dxl = dnn2_dxl / (2 * nn);
        const V3 dnn2_dxj = -2 * dot(xkl, xkl) * xjk + 2 * dot(xkl, xjk) * xkl;
        const V3 dnn_dxj = dnn2_dxj / (2 * nn);
        const V3 dnn2_dxk = -1. * (dnn2_dxl + dnn2_dxj);
        const V3 dnn_dxk = dnn2_dxk / (2 * nn);

        const T3 dm_dxi = skew(xkj);
        const T3 dm_dxk = skew(xji);
        const T3 dm_dxj = scale(add(dm_dxk, dm_dxi), -1.);
        const T3 dn_dxl = scale(dm_dxi, -1);
        const T3 dn_dxj = skew(xkl);
        const T3 dn_dxk = scale(add(dn_dxj, dn_dxl), -1);

        const double cpre = 1. / nmn;
        const V3 dc_dxi = cpre * (vecT(n, dm_dxi) - (cphi * nn) * dmn_dxi);
        const V3 dc_dxj = cpre * (vecT(n, dm_dxj) + vecT(m, dn_dxj) - (cphi * nn) * dmn_dxj - (cphi * mn) * dnn_dxj);
        const V3 dc_dxk = cpre * (vecT(n, dm_dxk) + vecT(m, dn_dxk) - (cphi * nn) * dmn_dxk - (cphi * mn) * dnn_dxk);
        const V3 dc_dxl = cpre * (vecT(m, dn_dxl) - (cphi * mn) * dnn_dxl);

        auto colCross = [](T3 t, V3 v) { return T3{{cross(t.c[0], v), cross(t.c[1], v), cross(t.c[2], v)}}; };
        auto crossCol = [](V3 v, T3 t) { return T3{{cross(v, t.c[0]), cross(v, t.c[1]), cross(v, t.c[2])}}; };
        const T3 dmxn_dxi = colCross(dm_dxi, n);
        const T3 dmxn_dxj = add(colCross(dm_dxj, n), crossCol(m, dn_dxj));
        const T3 dmxn_dxk = add(colCross(dm_dxk, n), crossCol(m, dn_dxk));
        const T3 dmxn_dxl = crossCol(m, dn_dxl);

        const double spre = 1. / (nmn * xjkn);
        const V3 ds_dxi = spre * (vecT(xjk, dmxn_dxi) - (sphi * nn * xjkn) * dmn_dxi);
        const V3 ds_dxj = spre * (vecT(xjk, dmxn_dxj) - 1. * mxn - (sphi * nn * xjkn) * dmn_dxj -
                                  (sphi * mn * xjkn) * dnn_dxj + (sphi * nmn / xjkn) * xjk);
        const V3 ds_dxk = spre * (vecT(xjk, dmxn_dxk) + mxn - (sphi * nn * xjkn) * dmn_dxk -
                                  (sphi * mn * xjkn) * dnn_dxk - (sphi * nmn / xjkn) * xjk);
        const V3 ds_dxl = spre * (vecT(xjk, dmxn_dxl) - (sphi * mn * xjkn) * dnn_dxl);

        const double sbc = sphi / cphi;
        const double ppre = -1. / (cphi * (1. + sbc * sbc));
        const V3 dphi_dxi = ppre * (ds_dxi - sbc * dc_dxi);
        const V3 dphi_dxj = ppre * (ds_dxj - sbc * dc_dxj);
        const V3 dphi_dxk = ppre * (ds_dxk - sbc * dc_dxk);
        const V3 dphi_dxl = ppre * (ds_dxl - sbc * dc_dxl);
        fi += -dVdphi * dphi_dxi;
        fj += -dVdphi * dphi_dxj;
        fk += -dVdphi * dphi_dxk;
        fl += -dVdphi * dphi_dxl;
    }

    /* CPUEulerBDIntegrator::perform, kernels/cpu/src/actions/CPUEulerBDIntegrator.cpp:51-103 */
    void eulerBD(double dt) {
        int nt = pool.size();
        size_t n = entries.size();
        pool.run([&](int tid) {
            auto [b, e] = chunk(n, nt, tid);
            for (size_t i = b; i < e; ++i) {
                Entry &en = entries[i];
                if (en.deactivated) continue;
                const double Dt = D[en.type];
                V3 rnd = normal3(tid);
                V3 det = ((en.force * Dt) * dt) / kbt;
                rnd = rnd * std::sqrt(2. * Dt * dt);
                en.pos += rnd + det;
                box.fix(en.pos);
            }
        });
    }

    /* performReactionEvent<false>, include/readdy/kernel/cpu/actions/reactions/ReactionUtils.h:64-71 */
    bool coin(int tid, double rate, double dt) { return uniform(tid) < 1 - std::exp(-rate * dt); }

    /* performReaction, ReactionUtils.h:146-227 */
    void performReaction(size_t idx1, size_t idx2, const Reaction *r, std::vector<Entry> &newEntries,
                         std::vector<size_t> &decayed) {
        Entry &e1 = entries.at(idx1);
        Entry &e2 = entries.at(idx2);
        switch (r->kind) {
            case DECAY: decayed.push_back(idx1); break;
            case CONVERSION: e1.type = r->products[0]; e1.id = nextId++; break;
            case ENZYMATIC:
                if (e1.type == r->educts[1]) { e2.type = r->products[0]; e2.id = nextId++; }
                else { e1.type = r->products[0]; e1.id = nextId++; }
                break;
            case FISSION: {
                V3 n3 = normal3(0);
                n3 = n3 / std::sqrt(dot(n3, n3));
                Entry ne;
                ne.pos = box.apply(e1.pos - (r->w2 * r->productDistance) * n3);
                ne.type = r->products[1];
                ne.id = nextId++;
                newEntries.push_back(ne);
                e1.type = r->products[0];
                e1.id = nextId++;
                e1.pos += (r->w1 * r->productDistance) * n3;   // DefaultDataContainer::displace :141-146
                box.fix(e1.pos);
                break;
            }
            case FUSION: {
                V3 diff = box.shortest(e1.pos, e2.pos);
                Entry ne;
                ne.pos = box.apply(e1.pos + (r->educts[0] == e1.type ? r->w1 : r->w2) * diff);
                ne.type = r->products[0];
                ne.id = nextId++;
                newEntries.push_back(ne);
                decayed.push_back(idx1);
                decayed.push_back(idx2);
                break;
            }
        }
        reactionCounts[r->id]++;
    }

    /* DefaultDataContainer::update, DefaultDataContainer.h:121-139 */
    void commit(std::vector<Entry> &newEntries, std::vector<size_t> &decayed) {
        auto it = decayed.begin();
        for (auto &ne : newEntries) {
            if (it != decayed.end()) { entries.at(*it) = ne; ++it; }
            else addEntry(ne);
        }
        for (; it != decayed.end(); ++it) removeEntry(*it);
    }

    /* CPUUncontrolledApproximation::perform, kernels/cpu/src/actions/reactions/CPUUncontrolledApproximation.cpp:135-256 */
    void uncontrolledApproximation(double dt) {
        if (!nlSetUp) throw std::logic_error("neighbor list not set up");
        int nt = pool.size();
        std::vector<std::vector<Event>> parts(nt);
        size_t n = entries.size(), nCells = adjacency.size();
        pool.run([&](int tid) {  // findEvents :70-133
            auto &ev = parts[tid];
            auto [b, e] = chunk(n, nt, tid);
            for (size_t i = b; i < e; ++i) {
                const Entry &en = entries[i];
                if (en.deactivated) continue;
                const auto &rs = o1[en.type];
                for (size_t ri = 0; ri < rs.size(); ++ri) {
                    double rate = rs[ri]->rate;
                    if (rate > 0 && coin(tid, rate, dt))
                        ev.push_back(Event{1, rs[ri]->nProducts, i, i, ri, en.type, 0, rate, 0});
                }
            }
            auto [cb, ce] = chunk(nCells, nt, tid);
            for (size_t cell = cb; cell < ce; ++cell) {
                forEachInCell(cell, [&](size_t pi) {
                    const Entry &en = entries[pi];
                    if (en.deactivated) return;
                    forEachNeighbor(pi, cell, [&](size_t ni) {
                        if (!(pi > ni)) return;
                        const Entry &nb = entries[ni];
                        if (nb.deactivated) return;
                        const auto *rs = reac2(en.type, nb.type);
                        if (!rs) return;
                        const double d2 = box.dist2(nb.pos, en.pos);
                        for (size_t ri = 0; ri < rs->size(); ++ri) {
                            const Reaction *r = (*rs)[ri];
                            if (r->rate > 0 && d2 < r->eductDistance2 && coin(tid, r->rate, dt))
                                ev.push_back(Event{2, r->nProducts, pi, ni, ri, en.type, nb.type, r->rate, 0});
                        }
                    });
                });
            }
        });
        std::vector<Event> events;
        for (auto &p : parts) events.insert(events.end(), p.begin(), p.end());
        std::shuffle(events.begin(), events.end(), rng[0]);
        std::vector<Entry> newEntries;
        std::vector<size_t> decayed;
        for (auto it = events.begin(); it != events.end(); ++it) {  // :206-253
            Event &ev = *it;
            if (ev.cumulativeRate != 0) continue;
            size_t e1 = ev.idx1;
            if (ev.nEducts == 1) {
                performReaction(e1, e1, o1[ev.t1][ev.reactionIndex], newEntries, decayed);
                for (auto j = it + 1; j != events.end(); ++j)
                    if (j->idx1 == e1 || j->idx2 == e1) j->cumulativeRate = 1;
            } else {
                performReaction(e1, ev.idx2, (*reac2(ev.t1, ev.t2))[ev.reactionIndex], newEntries, decayed);
                for (auto j = it + 1; j != events.end(); ++j)
                    if (j->idx1 == e1 || j->idx2 == e1 || j->idx1 == ev.idx2 || j->idx2 == ev.idx2)
                        j->cumulativeRate = 1;
            }
        }
        commit(newEntries, decayed);
    }

    /* CPUGillespie::perform + gatherEvents + handleEventsGillespie + algo::performEvents:
     * kernels/cpu/src/actions/reactions/CPUGillespie.cpp:53-93, ReactionUtils.h:83-144,
     * kernels/cpu/src/actions/reactions/ReactionUtils.cpp:55-123, include/readdy/common/algorithm.h:62-136 */
    void gillespie(double dt) {
        if (reactions.empty()) return;
        if (!nlSetUp) throw std::logic_error("neighbor list not set up");
        double alpha = 0;
        std::vector<Event> events;
        for (size_t i = 0; i < entries.size(); ++i) {
            const Entry &en = entries[i];
            if (en.deactivated) continue;
            const auto &rs = o1[en.type];
            for (size_t ri = 0; ri < rs.size(); ++ri) {
                double rate = rs[ri]->rate;
                if (rate > 0) {
                    alpha += rate;
                    events.push_back(Event{1, rs[ri]->nProducts, i, 0, ri, en.type, 0, rate, alpha});
                }
            }
        }
        for (size_t cell = 0; cell < adjacency.size(); ++cell) {
            forEachInCell(cell, [&](size_t i1) {
                const Entry &en = entries[i1];
                if (en.deactivated) return;
                forEachNeighbor(i1, cell, [&](size_t i2) {
                    if (i1 > i2) return;
                    const Entry &nb = entries[i2];
                    if (nb.deactivated) return;
                    const auto *rs = reac2(en.type, nb.type);
                    if (!rs) return;
                    const double d2 = box.dist2(nb.pos, en.pos);
                    for (size_t ri = 0; ri < rs->size(); ++ri) {
                        const Reaction *r = (*rs)[ri];
                        if (r->rate > 0 && d2 < r->eductDistance2) {
                            alpha += r->rate;
                            events.push_back(Event{2, r->nProducts, i1, i2, ri, en.type, nb.type, r->rate, alpha});
                        }
                    }
                });
            });
        }
        std::vector<Entry> newEntries;
        std::vector<size_t> decayed;
        auto depending = [](const Event &a, const Event &b) {  // ReactionUtils.cpp:77-80
            return a.idx1 == b.idx1 || (b.nEducts == 2 && a.idx1 == b.idx2) ||
                   (a.nEducts == 2 && (a.idx2 == b.idx1 || (b.nEducts == 2 && a.idx2 == b.idx2)));
        };
        auto eval = [&](const Event &ev) {
            if (ev.nEducts == 1) performReaction(ev.idx1, ev.idx1, o1[ev.t1][ev.reactionIndex], newEntries, decayed);
            else performReaction(ev.idx1, ev.idx2, (*reac2(ev.t1, ev.t2))[ev.reactionIndex], newEntries, decayed);
        };
        if (!events.empty()) {  // algo::performEvents
            size_t nDeact = 0;
            const size_t nEvents = events.size();
            double cum = 0;
            for (auto &ev : events) { ev.cumulativeRate = ev.rate + cum; cum = ev.cumulativeRate; }
            while (nDeact < nEvents) {
                const double cr = (events.end() - nDeact - 1)->cumulativeRate;
                const double x = uniform(0, 0., cr);
                auto it = std::lower_bound(events.begin(), events.end() - nDeact, x,
                                           [](const Event &e, double v) { return e.cumulativeRate < v; });
                if (it == events.end()) throw std::logic_error("performEvents: no event could be selected");
                if (coin(0, it->rate, dt)) {
                    eval(*it);
                    Event done = *it;
                    auto j = events.begin();
                    double cs = 0;
                    while (j < events.end() - nDeact) {
                        if (depending(*j, done)) {
                            ++nDeact;
                            std::iter_swap(j, events.end() - nDeact);
                        } else {
                            cs += j->rate;
                            j->cumulativeRate = cs;
                            ++j;
                        }
                    }
                } else {
                    ++nDeact;
                    std::iter_swap(it, events.end() - nDeact);
                    it->cumulativeRate = it->rate;
                    if (it > events.begin()) it->cumulativeRate += (it - 1)->cumulativeRate;
                    double cs = it->cumulativeRate;
                    for (auto j = it + 1; j < events.end() - nDeact; ++j) { cs += j->rate; j->cumulativeRate = cs; }
                }
            }
        }
        commit(newEntries, decayed);
    }

    void countTypes(int64_t *out) const {
        for (int t = 0; t < nTypes; ++t) out[t] = 0;
        for (const auto &e : entries) if (!e.deactivated) out[e.type]++;
    }
};

extern "C" {

const char *orc_last_error(void) { return g_err.c_str(); }

orc_system *orc_create(const double box[3], const int periodic[3], double kbt, int n_types, const double *diffusion,
                       uint64_t seed, int n_threads, int cll_radius) {
    try {
        if (n_types <= 0 || cll_radius <= 0) throw std::invalid_argument("bad n_types or cll radius");
        return new orc_system(box, periodic, kbt, n_types, diffusion, seed, n_threads, cll_radius);
    } catch (const std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}
void orc_destroy(orc_system *s) { delete s; }

static int addPot(orc_system *s, int t1, int t2, Pot2 p) {
    if (t1 < 0 || t2 < 0 || t1 >= s->nTypes || t2 >= s->nTypes) { g_err = "bad type"; return -1; }
    s->pot2[orc_system::key(t1, t2)].push_back(p);
    return 0;
}
static int addPot1(orc_system *s, int t, const Pot1 &p) {
    if (t < 0 || t >= s->nTypes) { g_err = "type out of range"; return -1; }
    s->pot1[t].push_back(p);
    return 0;
}
static V3 v3(const double *a) { return V3{a[0], a[1], a[2]}; }
/* PotentialRegistry::addBox / addHarmonicGeometry(Box) (PotentialRegistry.h:99-112, 335-345): v1 = origin + extent */
int orc_add_box(orc_system *s, int t, double k, const double *origin, const double *extent, int inclusion) {
    Pot1 p{P1_BOX, inclusion != 0};
    p.k = k; p.a = v3(origin); p.b = v3(origin) + v3(extent);
    return addPot1(s, t, p);
}
/* PotentialRegistry::addSphere (:253-270) */
int orc_add_sphere(orc_system *s, int t, double k, const double *origin, double radius, int inclusion) {
    Pot1 p{P1_SPHERE, inclusion != 0};
    p.k = k; p.a = v3(origin); p.radius = radius;
    return addPot1(s, t, p);
}
/* PotentialRegistry::addCapsule / addHarmonicGeometry(Capsule) (:274-293) */
int orc_add_capsule(orc_system *s, int t, double k, const double *center, const double *direction, double length,
                    double radius, int inclusion) {
    Pot1 p{P1_CAPSULE, inclusion != 0};
    p.k = k; p.a = v3(center); p.b = v3(direction); p.length = length; p.radius = radius;
    return addPot1(s, t, p);
}
/* PotentialRegistry::addSphericalBarrier (:305-317), SphericalBarrier ctor (Potentials.cpp:86-92) */
int orc_add_spherical_barrier(orc_system *s, int t, double height, double width, const double *origin,
                              double radius) {
    if (width > radius) { g_err = "SphericalBarrier must have a radius larger than its width"; return -1; }
    Pot1 p{P1_SPHERICAL_BARRIER, true};
    p.a = v3(origin); p.radius = radius; p.height = height; p.width = width;
    p.r1 = radius - width; p.r2 = radius - width / 2.; p.r3 = radius + width / 2.; p.r4 = radius + width;
    p.keff = 4. * height / width / width;
    return addPot1(s, t, p);
}
/* PotentialRegistry::addCylinder (:330-...), Cylinder ctor normalises the normal (PotentialsOrder1.h:160-163) */
int orc_add_cylinder(orc_system *s, int t, double k, const double *origin, const double *normal, double radius,
                     int inclusion) {
    Pot1 p{P1_CYLINDER, inclusion != 0};
    V3 n = v3(normal);
    p.k = k; p.a = v3(origin); p.b = n / norm(n); p.radius = radius;
    return addPot1(s, t, p);
}

int orc_add_harmonic_repulsion(orc_system *s, int t1, int t2, double k, double d) {
    Pot2 p{HARMONIC_REPULSION, {k, d, d * d}, d * d};
    return addPot(s, t1, t2, p);
}
int orc_add_weak_interaction_piecewise_harmonic(orc_system *s, int t1, int t2, double k, double d0, double depth,
                                                double rc) {
    Pot2 p{WEAK_PIECEWISE_HARMONIC, {k, d0, depth, rc}, rc * rc};
    return addPot(s, t1, t2, p);
}
int orc_add_lennard_jones(orc_system *s, int t1, int t2, unsigned m, unsigned n, double cutoff, int shift,
                          double epsilon, double sigma) {
    if (m <= n) { g_err = "LJ: m must be greater than n"; return -1; }  // Potentials.cpp:163-166
    double dm = m, dn = n;
    double rmin = sigma * std::pow(dn / dm, 1. / (dn - dm));            // Potentials.cpp:167-170
    double kk = -epsilon / (std::pow(sigma / rmin, dm) - std::pow(sigma / rmin, dn));
    Pot2 p{LENNARD_JONES, {dm, dn, cutoff, shift ? 1. : 0., epsilon, sigma, kk}, cutoff * cutoff};
    return addPot(s, t1, t2, p);
}
int orc_add_screened_electrostatics(orc_system *s, int t1, int t2, double C, double kappa, double D, double sigma,
                                    unsigned exponent, double cutoff) {
    if (kappa < 0 || D < 0 || sigma < 0 || cutoff < 0) { g_err = "screened electrostatics: negative parameter"; return -1; }
    Pot2 p{SCREENED_ELECTROSTATICS, {C, kappa, D, sigma, (double)exponent, cutoff}, cutoff * cutoff};
    return addPot(s, t1, t2, p);
}

static int addReaction(orc_system *s, Reaction *r) {
    r->id = (int)s->reactions.size();
    s->reactions.push_back(r);
    s->reactionCounts.push_back(0);
    if (r->nEducts == 1) s->o1.at(r->educts[0]).push_back(r);
    else s->o2[orc_system::key(r->educts[0], r->educts[1])].push_back(r);
    return r->id;
}
static void normWeights(Reaction *r) {  // Fusion.h:62-68, Fission.h:64-70
    double sum = r->w1 + r->w2;
    if (sum != 1) { r->w1 /= sum; r->w2 /= sum; }
}
int orc_add_conversion(orc_system *s, int from, int to, double rate) {
    auto *r = new Reaction{CONVERSION, 0, {from, 0}, {to, 0}, 1, 1, rate};
    return addReaction(s, r);
}
int orc_add_decay(orc_system *s, int from, double rate) {
    auto *r = new Reaction{DECAY, 0, {from, 0}, {0, 0}, 1, 0, rate};
    return addReaction(s, r);
}
int orc_add_fusion(orc_system *s, int from1, int from2, int to, double rate, double ed, double w1, double w2) {
    auto *r = new Reaction{FUSION, 0, {from1, from2}, {to, 0}, 2, 1, rate, ed, ed * ed, 0, w1, w2};
    normWeights(r);
    return addReaction(s, r);
}
int orc_add_fission(orc_system *s, int from, int to1, int to2, double rate, double pd, double w1, double w2) {
    auto *r = new Reaction{FISSION, 0, {from, 0}, {to1, to2}, 1, 2, rate, 0, 0, pd, w1, w2};
    normWeights(r);
    return addReaction(s, r);
}
int orc_add_enzymatic(orc_system *s, int catalyst, int from, int to, double rate, double ed) {
    auto *r = new Reaction{ENZYMATIC, 0, {from, catalyst}, {to, catalyst}, 2, 2, rate, ed, ed * ed};
    return addReaction(s, r);
}

int orc_add_harmonic_bonds(orc_system *s, int n, const int *idx, const double *k, const double *l0) {
    for (int i = 0; i < n; ++i) {
        s->fixedBonds.push_back(Bond{(size_t)idx[2 * i], (size_t)idx[2 * i + 1], k[i], l0[i]});
        s->bonds.push_back(s->fixedBonds.back());
    }
    return 0;
}
int orc_add_harmonic_angles(orc_system *s, int n, const int *idx, const double *k, const double *th) {
    for (int i = 0; i < n; ++i) {
        s->fixedAngles.push_back(Angle{(size_t)idx[3 * i], (size_t)idx[3 * i + 1], (size_t)idx[3 * i + 2], k[i], th[i]});
        s->angles.push_back(s->fixedAngles.back());
    }
    return 0;
}
int orc_add_cosine_dihedrals(orc_system *s, int n, const int *idx, const double *k, const double *mult,
                             const double *phi0) {
    for (int i = 0; i < n; ++i) {
        s->fixedDihedrals.push_back(Dihedral{(size_t)idx[4 * i], (size_t)idx[4 * i + 1], (size_t)idx[4 * i + 2],
                                             (size_t)idx[4 * i + 3], k[i], mult[i], phi0[i]});
        s->dihedrals.push_back(s->fixedDihedrals.back());
    }
    return 0;
}

/* topology registry, flavors, topologies and BreakBonds */
int orc_set_particle_flavor(orc_system *s, int type, int flavor) {
    if (type < 0 || type >= s->nTypes) { g_err = "particle type out of range"; return -1; }
    s->flavor[type] = flavor;
    return 0;
}
int orc_configure_harmonic_bond(orc_system *s, int t1, int t2, double k, double l0) {
    s->bondCfg.push_back({t1, t2, k, l0});
    return 0;
}
int orc_configure_harmonic_angle(orc_system *s, int t1, int t2, int t3, double k, double theta0) {
    s->angleCfg.push_back({t1, t2, t3, k, theta0});
    return 0;
}
int orc_configure_cosine_dihedral(orc_system *s, int t1, int t2, int t3, int t4, double k, double mult, double phi0) {
    s->dihedralCfg.push_back({t1, t2, t3, t4, k, mult, phi0});
    return 0;
}
/* StateModel::addTopology + the graph's edges + GraphTopology::configure; ids_out receives the ids */
int orc_add_topology(orc_system *s, int type, int n, const double *pos, const int *types, int n_edges,
                     const int *edges, uint64_t *ids_out) {
    try {
        orc_system::Graph g;
        g.type = type;
        orc_system::IdMap ids;
        for (int i = 0; i < n; ++i) {
            Entry e;
            e.pos = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
            e.type = types[i];
            e.id = s->nextId++;
            ids[e.id] = s->addEntry(e);
            g.ids.push_back(e.id);
            if (ids_out) ids_out[i] = e.id;
        }
        for (int k = 0; k < n_edges; ++k) g.edges.push_back({edges[2 * k], edges[2 * k + 1]});
        const size_t nb = s->bonds.size(), na = s->angles.size(), nd = s->dihedrals.size();
        try {
            s->configureGraph(g, ids);
        } catch (...) {
            s->bonds.resize(nb);
            s->angles.resize(na);
            s->dihedrals.resize(nd);
            throw;
        }
        s->graphs.push_back(std::move(g));
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}
int orc_break_bonds(orc_system *s, double dt, int n, const int *t1, const int *t2, const double *thr,
                    const double *rate, int64_t *n_broken) {
    try {
        const int64_t r = s->breakBonds(dt, n, t1, t2, thr, rate);
        if (n_broken) *n_broken = r;
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}
int orc_add_spatial_topology_reaction(orc_system *s, int mode, int t1, int tt1, int t2, int tt2, int to1, int tto1,
                                      int to2, int tto2, double rate, double radius, int min_graph_distance) {
    s->spatial.push_back({mode, t1, tt1, t2, tt2, to1, tto1, to2, tt2 == -1 ? -1 : tto2, rate, radius,
                          min_graph_distance});
    return (int)s->spatial.size() - 1;
}
int orc_set_spatial_topology_rate_function(orc_system *s, int reaction_id, orc_spatial_rate_fn rate, void *user) {
    if (reaction_id < 0 || reaction_id >= (int)s->spatial.size() || s->spatial[reaction_id].tp()) {
        g_err = "rate functions apply to topology-topology spatial reactions";
        return -1;
    }
    s->spatial[reaction_id].rateFn = rate;
    s->spatial[reaction_id].rateUser = user;
    return 0;
}
int orc_set_legacy_topology_self_fusion(orc_system *s, int legacy) {
    s->legacySelfFusion = legacy != 0;
    return 0;
}
int orc_evaluate_topology_reactions(orc_system *s, double dt, int64_t *n_performed) {
    try {
        const int64_t n = s->evaluateTopologyReactions(dt);
        if (n_performed) *n_performed = n;
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}
int orc_add_structural_topology_reaction(orc_system *s, int topology_type, orc_topology_rate_fn rate,
                                         orc_topology_recipe_fn reaction, void *user, int expect_connected) {
    s->structural.push_back({topology_type, rate, reaction, user, expect_connected != 0});
    s->graphRates.clear();
    return (int)s->structural.size() - 1;
}
int orc_structural_reaction_counts(const orc_system *s, int64_t *counts, int n) {
    for (int k = 0; k < n; ++k) counts[k] = k < (int)s->structuralCounts.size() ? s->structuralCounts[k] : 0;
    return 0;
}
int orc_recipe_change_particle_type(orc_recipe *r, int64_t v, int type) { r->ops.push_back({0, v, 0, type}); return 0; }
int orc_recipe_add_edge(orc_recipe *r, int64_t a, int64_t b) { r->ops.push_back({1, a, b, 0}); return 0; }
int orc_recipe_remove_edge(orc_recipe *r, int64_t a, int64_t b) { r->ops.push_back({2, a, b, 0}); return 0; }
int orc_recipe_separate_vertex(orc_recipe *r, int64_t v) { r->ops.push_back({3, v, 0, 0}); return 0; }
int orc_recipe_change_topology_type(orc_recipe *r, int type) { r->ops.push_back({4, 0, 0, type}); return 0; }
int orc_recipe_append_particle(orc_recipe *r, int64_t n, const int64_t *nb, int type, const double *pos3) {
    r->ops.push_back({5, 0, 0, type, std::vector<int64_t>(nb, nb + n), {pos3[0], pos3[1], pos3[2]}});
    return 0;
}
int orc_recipe_change_particle_position(orc_recipe *r, int64_t v, const double *pos3) {
    r->ops.push_back({6, v, 0, 0, {}, {pos3[0], pos3[1], pos3[2]}});
    return 0;
}
int orc_get_topology(const orc_system *s, int64_t k, int *type, uint64_t *ids, int *types, double *pos3,
                     int64_t *n_vertices, int64_t *edges2, int64_t *n_edges) {
    if (k < 0 || k >= (int64_t)s->graphs.size()) { g_err = "topology index out of range"; return -1; }
    const auto &g = s->graphs[k];
    const auto idx = s->idMap();
    if (type) *type = g.type;
    if (n_vertices) *n_vertices = (int64_t)g.ids.size();
    if (n_edges) *n_edges = (int64_t)g.edges.size();
    for (size_t v = 0; v < g.ids.size(); ++v) {
        const auto &e = s->entries[orc_system::indexOf(idx, g.ids[v])];
        if (ids) ids[v] = g.ids[v];
        if (types) types[v] = e.type;
        if (pos3) { pos3[3 * v] = e.pos.x; pos3[3 * v + 1] = e.pos.y; pos3[3 * v + 2] = e.pos.z; }
    }
    if (edges2)
        for (size_t e = 0; e < g.edges.size(); ++e) { edges2[2 * e] = g.edges[e].first; edges2[2 * e + 1] = g.edges[e].second; }
    return 0;
}
int orc_topology_reaction_counts(const orc_system *s, int64_t *counts, int n) {
    for (int k = 0; k < n; ++k) counts[k] = k < (int)s->spatialCounts.size() ? s->spatialCounts[k] : 0;
    return 0;
}
/* topologies as CSR over particle ids (any output may be NULL; sizes first) */
int orc_get_topologies(const orc_system *s, int *types, int64_t *offsets, uint64_t *ids, int64_t *n_top,
                       int64_t *n_ids) {
    int64_t at = 0;
    for (size_t k = 0; k < s->graphs.size(); ++k) {
        if (types) types[k] = s->graphs[k].type;
        if (offsets) offsets[k] = at;
        for (auto id : s->graphs[k].ids) {
            if (ids) ids[at] = id;
            ++at;
        }
    }
    if (offsets) offsets[s->graphs.size()] = at;
    if (n_top) *n_top = (int64_t)s->graphs.size();
    if (n_ids) *n_ids = at;
    return 0;
}
int orc_get_topology_edges(const orc_system *s, int64_t *offsets, uint64_t *edges2, int64_t *n_edges) {
    int64_t at = 0;
    for (size_t k = 0; k < s->graphs.size(); ++k) {
        if (offsets) offsets[k] = at;
        const auto &g = s->graphs[k];
        for (auto &e : g.edges) {
            if (edges2) { edges2[2 * at] = g.ids[e.first]; edges2[2 * at + 1] = g.ids[e.second]; }
            ++at;
        }
    }
    if (offsets) offsets[s->graphs.size()] = at;
    if (n_edges) *n_edges = at;
    return 0;
}

int orc_add_particles(orc_system *s, int n, const double *pos, const int *types) {
    for (int i = 0; i < n; ++i) {
        Entry e;
        e.pos = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        e.type = types[i];
        e.id = s->nextId++;
        s->addEntry(e);
    }
    return 0;
}
int orc_n_particles(const orc_system *s) {
    int n = 0;
    for (auto &e : s->entries) n += !e.deactivated;
    return n;
}
int orc_n_entries(const orc_system *s) { return (int)s->entries.size(); }
int orc_get_force_scales(const orc_system *s, double *out) {
    int k = 0;
    for (const auto &e : s->entries)
        if (!e.deactivated) out[k++] = e.fscale;
    return k;
}
int orc_get_particles(const orc_system *s, double *pos, int *types, uint64_t *ids, double *force, int *sidx) {
    int k = 0;
    for (size_t i = 0; i < s->entries.size(); ++i) {
        const auto &e = s->entries[i];
        if (e.deactivated) continue;
        if (pos) { pos[3 * k] = e.pos.x; pos[3 * k + 1] = e.pos.y; pos[3 * k + 2] = e.pos.z; }
        if (types) types[k] = e.type;
        if (ids) ids[k] = e.id;
        if (force) { force[3 * k] = e.force.x; force[3 * k + 1] = e.force.y; force[3 * k + 2] = e.force.z; }
        if (sidx) sidx[k] = (int)i;
        ++k;
    }
    return k;
}
double orc_calculate_max_cutoff(const orc_system *s) { return s->maxCutoff(); }

int orc_nl_setup(orc_system *s, double cutoff) {
    try { s->nlSetup(cutoff); return 0; } catch (const std::exception &e) { g_err = e.what(); return -1; }
}
int orc_nl_update(orc_system *s) {
    try { s->nlUpdate(); return 0; } catch (const std::exception &e) { g_err = e.what(); return -1; }
}

static int64_t finishPairs(std::vector<std::pair<uint64_t, uint64_t>> &v, int64_t cap, uint64_t *out) {
    std::sort(v.begin(), v.end());
    if ((int64_t)v.size() > cap) return -1;
    for (size_t i = 0; i < v.size(); ++i) { out[2 * i] = v[i].first; out[2 * i + 1] = v[i].second; }
    return (int64_t)v.size();
}
/* the pair-set contract of the consumers: CPUCalculateForces.cpp:240-243 (d^2 < rc^2 on the minimum image) */
int64_t orc_nl_pairs(const orc_system *s, double cutoff, int64_t cap, uint64_t *out) {
    std::vector<std::pair<uint64_t, uint64_t>> v;
    const double c2 = cutoff * cutoff;
    for (size_t cell = 0; cell < s->adjacency.size(); ++cell) {
        s->forEachInCell(cell, [&](size_t i) {
            const auto &a = s->entries[i];
            if (a.deactivated) return;
            s->forEachNeighbor(i, cell, [&](size_t j) {
                if (i > j) return;
                const auto &b = s->entries[j];
                if (b.deactivated) return;
                V3 x = s->box.shortest(a.pos, b.pos);
                if (dot(x, x) < c2) v.push_back({std::min(a.id, b.id), std::max(a.id, b.id)});
            });
        });
    }
    return finishPairs(v, cap, out);
}
/* brute force over all in-box pairs, kernels/cpu/test/TestNeighborList.cpp:277-297 */
int64_t orc_brute_force_pairs(const orc_system *s, double cutoff, int64_t cap, uint64_t *out) {
    std::vector<std::pair<uint64_t, uint64_t>> v;
    const double c2 = cutoff * cutoff;
    auto inBox = [s](const V3 &p) {
        for (int d = 0; d < 3; ++d) if (!(-.5 * s->box.L[d] <= p[d] && .5 * s->box.L[d] > p[d])) return false;
        return true;
    };
    for (size_t i = 0; i < s->entries.size(); ++i) {
        const auto &a = s->entries[i];
        if (a.deactivated || !inBox(a.pos)) continue;
        for (size_t j = i + 1; j < s->entries.size(); ++j) {
            const auto &b = s->entries[j];
            if (b.deactivated || !inBox(b.pos)) continue;
            V3 x = s->box.shortest(a.pos, b.pos);
            if (dot(x, x) < c2) v.push_back({std::min(a.id, b.id), std::max(a.id, b.id)});
        }
    }
    return finishPairs(v, cap, out);
}

int orc_set_record_virial(orc_system *s, int record) { s->recordVirial = record != 0; return 0; }
int orc_get_virial(const orc_system *s, double *out9) {
    for (int k = 0; k < 9; ++k) out9[k] = s->virial[k];
    return 0;
}
double orc_calculate_forces(orc_system *s) {
    try { return s->calculateForces(); } catch (const std::exception &e) { g_err = e.what(); return NAN; }
}
double orc_energy(const orc_system *s) { return s->energy; }
int orc_euler_bd(orc_system *s, double dt) { s->eulerBD(dt); return 0; }
int orc_uncontrolled_approximation(orc_system *s, double dt) {
    try { s->uncontrolledApproximation(dt); return 0; } catch (const std::exception &e) { g_err = e.what(); return -1; }
}
int orc_gillespie(orc_system *s, double dt) {
    try { s->gillespie(dt); return 0; } catch (const std::exception &e) { g_err = e.what(); return -1; }
}

/* SimulationLoop::run, include/readdy/api/SimulationLoop.h:256-306 (no compartments, no topology reactions) */
int orc_run(orc_system *s, int64_t n_steps, double dt, int handler, int stride, int64_t *counts, int64_t maxrec) {
    try {
        double cutoff = s->maxCutoff();
        bool nl = cutoff > 0;
        int64_t rec = 0;
        auto observe = [&](int64_t t) {
            if (counts && stride > 0 && t % stride == 0 && rec < maxrec) s->countTypes(counts + rec++ * s->nTypes);
        };
        if (nl) s->nlSetup(cutoff);
        s->calculateForces();
        observe(0);
        for (int64_t t = 0; t < n_steps; ++t) {
            s->eulerBD(dt);
            if (nl) s->nlUpdate();
            if (!s->reactions.empty()) {
                if (handler == ORC_GILLESPIE) s->gillespie(dt);
                else s->uncontrolledApproximation(dt);
            }
            // runTopologyReactions (SimulationLoop.h:285); the cells are refreshed first so that particles the
            // reactions created take part
            if ((!s->spatial.empty() || !s->structural.empty()) && !s->graphs.empty()) {
                if (nl) s->nlUpdate();
                s->evaluateTopologyReactions(dt);
            }
            if (nl) s->nlUpdate();
            s->calculateForces();
            observe(t + 1);
        }
        return (int)rec;
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}

int orc_reaction_counts(const orc_system *s, int64_t *counts, int cap) {
    int n = std::min<int>(cap, (int)s->reactionCounts.size());
    for (int i = 0; i < n; ++i) counts[i] = s->reactionCounts[i];
    return n;
}

/* kernels/cpu/src/observables/CPUObservables.cpp:85-146: for every active particle of a listed type, the
 * index of std::upper_bound(borders, pos[axis]); index k counts into bin k - 1 when 1 <= k < n_borders - 1
 * (the result has n_borders - 1 bins and the CPU kernel compares the index with that size, so the last
 * bin is never counted) */
int orc_histogram_along_axis(const orc_system *s, int n_borders, const double *borders, int n_types,
                             const int *types, int axis, double *counts) {
    if (n_borders < 2 || axis < 0 || axis > 2) return -1;
    const int size = n_borders - 1;
    std::fill(counts, counts + size, 0.0);
    for (const Entry &e : s->entries) {
        if (e.deactivated || std::find(types, types + n_types, e.type) == types + n_types) continue;
        const double *ub = std::upper_bound(borders, borders + n_borders, e.pos[axis]);
        if (ub == borders + n_borders) continue;
        const long k = ub - borders;
        if (k >= 1 && k < size) counts[k - 1] += 1.0;
    }
    return size;
}

/* readdy/main/model/observables/RadialDistribution.cpp:75-128: every ordered pair (from, to) of active
 * particles with distinct ids, from of a from type and to of a to type, counts into bin k - 1 of
 * k = index of std::upper_bound(borders, |shortestDifference|) when k < n_borders; the distribution
 * divides each count by 4/3 pi (r_hi^3 - r_lo^3) n_from particle_to_density.  A distance below the first
 * border would count into bin -1 there; it is not counted here. */
int orc_radial_distribution(const orc_system *s, int n_borders, const double *borders, int n_from,
                            const int *from_types, int n_to, const int *to_types, double particle_to_density,
                            double *counts, double *distribution) {
    if (n_borders < 2) return -1;
    const int size = n_borders - 1;
    std::fill(counts, counts + size, 0.0);
    auto in = [](int t, const int *set, int n) { return std::find(set, set + n, t) != set + n; };
    long n_from_particles = 0;
    for (const Entry &e : s->entries)
        if (!e.deactivated && in(e.type, from_types, n_from)) ++n_from_particles;
    for (const Entry &a : s->entries) {
        if (a.deactivated || !in(a.type, from_types, n_from)) continue;
        for (const Entry &b : s->entries) {
            if (b.deactivated || !in(b.type, to_types, n_to) || a.id == b.id) continue;
            const double dist = std::sqrt(s->box.dist2(a.pos, b.pos));
            const double *ub = std::upper_bound(borders, borders + n_borders, dist);
            if (ub == borders + n_borders || ub == borders) continue;
            counts[(ub - borders) - 1] += 1.0;
        }
    }
    const double pi = 3.14159265358979323846;
    for (int k = 0; k < size; ++k)
        distribution[k] = counts[k] / (4. / 3. * pi * (std::pow(borders[k + 1], 3.) - std::pow(borders[k], 3.)) *
                                       (double)n_from_particles * particle_to_density);
    return size;
}

}  // extern "C"

// CPU oracle (test infrastructure only) — restatement of the reference's
// PhysicsWorld::step hot path.  See pe_oracle.h for what this is and is not.
//
// Every expression keeps the reference's operation order and association so
// that the float instance is bit-identical to the reference compiled with
// floating-point contraction off.  All citations are paths inside the
// bkuangs/phys-engine project.
#include "pe_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <numeric>
#include <string>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace oracle {

// Persistent worker threads shared by every world, the calling thread joining
// in (the reference keeps a world-owned pool that includes the caller,
// src/world/step_workspace.hpp:24-172).  run() hands out jobs [0, jobs) from
// an atomic counter to `workers` threads and returns when all are done.
class Pool {
  public:
    static Pool &instance() {
        static Pool pool;
        return pool;
    }
    void run(int workers, size_t jobs, const std::function<void(size_t)> &fn) {
        if (workers <= 1 || jobs <= 1) {
            for (size_t j = 0; j < jobs; ++j) fn(j);
            return;
        }
        std::lock_guard<std::mutex> serial(runMutex_);
        const int helpers = workers - 1;
        while ((int)threads_.size() < helpers) {
            const size_t id = threads_.size();
            threads_.emplace_back([this, id] { loop(id); });
        }
        {
            std::lock_guard<std::mutex> l(m_);
            fn_ = &fn;
            jobs_ = jobs;
            next_.store(0);
            participants_ = helpers;
            active_ = helpers;
            ++generation_;
        }
        wake_.notify_all();
        work();
        std::unique_lock<std::mutex> l(m_);
        done_.wait(l, [&] { return active_ == 0; });
        fn_ = nullptr;
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> l(m_);
            stop_ = true;
        }
        wake_.notify_all();
        for (auto &t : threads_) t.join();
    }

  private:
    void work() {
        for (size_t j; (j = next_.fetch_add(1)) < jobs_;) (*fn_)(j);
    }
    void loop(size_t id) {
        uint64_t seen = 0;
        std::unique_lock<std::mutex> l(m_);
        for (;;) {
            wake_.wait(l, [&] { return stop_ || generation_ != seen; });
            if (stop_) return;
            seen = generation_;
            if ((int)id >= participants_) continue;  // not needed this round
            l.unlock();
            work();
            l.lock();
            if (--active_ == 0) done_.notify_one();
        }
    }
    std::mutex runMutex_, m_;
    std::condition_variable wake_, done_;
    std::vector<std::thread> threads_;
    const std::function<void(size_t)> *fn_ = nullptr;
    size_t jobs_ = 0;
    std::atomic<size_t> next_{0};
    int participants_ = 0, active_ = 0;
    uint64_t generation_ = 0;
    bool stop_ = false;
};

// ---------------------------------------------------------------------------
// Math (include/phys/math/vec3.hpp, quaternion.hpp, mat3.hpp, math_utils.hpp,
// src/math/math_utils.cpp)
// ---------------------------------------------------------------------------
template <class T> struct V3 {
    T x{}, y{}, z{};
};
template <class T> inline V3<T> operator+(V3<T> a, const V3<T> &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, const V3<T> &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator-(const V3<T> &a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline V3<T> operator*(const V3<T> &a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator/(const V3<T> &a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline V3<T> &operator+=(V3<T> &a, const V3<T> &b) {
    a.x += b.x; a.y += b.y; a.z += b.z;
    return a;
}
// Math3d::dot (math_utils.cpp:28-31)
template <class T> inline T dot(const V3<T> &a, const V3<T> &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// Math3d::cross (math_utils.hpp:19-26)
template <class T> inline V3<T> cross(const V3<T> &a, const V3<T> &b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// Math3d::length (math_utils.cpp:7-12)
template <class T> inline T length(const V3<T> &v) { return std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
// Math3d::normalize (math_utils.cpp:19-26)
template <class T> inline V3<T> normalize(const V3<T> &v) {
    T len = length(v);
    if (len <= T(1e-8f)) return {T(0), T(0), T(0)};
    return v * (T(1) / len);
}
// std::max / std::min semantics (first argument returned on ties/unordered)
template <class T> inline T smax(T a, T b) { return (a < b) ? b : a; }
template <class T> inline T smin(T a, T b) { return (b < a) ? b : a; }
// Math3d::clamp (math_utils.hpp:31-39); min > max never occurs for box extents.
template <class T> inline T clampv(T v, T lo, T hi) {
    if (lo == hi) return lo;
    if (v < lo) return lo;
    if (v > hi) return hi;
    return v;
}

template <class T> struct Q {
    T x{}, y{}, z{}, w{1};
};
// Quaternion::operator* (quaternion.hpp:24-31)
template <class T> inline Q<T> qmul(const Q<T> &a, const Q<T> &o) {
    return {a.w * o.x + a.x * o.w + a.y * o.z - a.z * o.y,
            a.w * o.y - a.x * o.z + a.y * o.w + a.z * o.x,
            a.w * o.z + a.x * o.y - a.y * o.x + a.z * o.w,
            a.w * o.w - a.x * o.x - a.y * o.y - a.z * o.z};
}
template <class T> inline Q<T> conj(const Q<T> &q) { return {-q.x, -q.y, -q.z, q.w}; }
// Quaternion::normalized (quaternion.hpp:37-45)
template <class T> inline Q<T> qnormalized(const Q<T> &q) {
    T len = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    if (len == T(0)) return {T(0), T(0), T(0), T(1)};
    return {q.x / len, q.y / len, q.z / len, q.w / len};
}
// Quaternion::rotate (quaternion.hpp:47-51): q * (v, 0) * conj(q)
template <class T> inline V3<T> rotate(const Q<T> &q, const V3<T> &v) {
    Q<T> p{v.x, v.y, v.z, T(0)};
    Q<T> r = qmul(qmul(q, p), conj(q));
    return {r.x, r.y, r.z};
}

template <class T> struct M3 {
    T m00{}, m01{}, m02{}, m10{}, m11{}, m12{}, m20{}, m21{}, m22{};
};
// Quaternion::toMat3 (quaternion.hpp:54-64)
template <class T> inline M3<T> toMat3(const Q<T> &q) {
    T xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
    T xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
    T wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    return {T(1) - T(2) * (yy + zz), T(2) * (xy - wz), T(2) * (xz + wy),
            T(2) * (xy + wz), T(1) - T(2) * (xx + zz), T(2) * (yz - wx),
            T(2) * (xz - wy), T(2) * (yz + wx), T(1) - T(2) * (xx + yy)};
}
// Mat3 * Vec3 (mat3.hpp:20-26)
template <class T> inline V3<T> mul(const M3<T> &m, const V3<T> &v) {
    return {m.m00 * v.x + m.m01 * v.y + m.m02 * v.z,
            m.m10 * v.x + m.m11 * v.y + m.m12 * v.z,
            m.m20 * v.x + m.m21 * v.y + m.m22 * v.z};
}
// Mat3 * Mat3 (mat3.hpp:51-63)
template <class T> inline M3<T> mul(const M3<T> &l, const M3<T> &r) {
    return {l.m00 * r.m00 + l.m01 * r.m10 + l.m02 * r.m20,
            l.m00 * r.m01 + l.m01 * r.m11 + l.m02 * r.m21,
            l.m00 * r.m02 + l.m01 * r.m12 + l.m02 * r.m22,
            l.m10 * r.m00 + l.m11 * r.m10 + l.m12 * r.m20,
            l.m10 * r.m01 + l.m11 * r.m11 + l.m12 * r.m21,
            l.m10 * r.m02 + l.m11 * r.m12 + l.m12 * r.m22,
            l.m20 * r.m00 + l.m21 * r.m10 + l.m22 * r.m20,
            l.m20 * r.m01 + l.m21 * r.m11 + l.m22 * r.m21,
            l.m20 * r.m02 + l.m21 * r.m12 + l.m22 * r.m22};
}
template <class T> inline M3<T> transpose(const M3<T> &v) {
    return {v.m00, v.m10, v.m20, v.m01, v.m11, v.m21, v.m02, v.m12, v.m22};
}

template <class T> struct Tf {
    V3<T> p;
    Q<T> q;
};
// toLocalPoint / toWorldPoint (src/collision/narrowphase.cpp:16-25)
template <class T> inline V3<T> toLocal(const V3<T> &w, const Tf<T> &tf) { return rotate(conj(tf.q), w - tf.p); }
template <class T> inline V3<T> toWorld(const V3<T> &l, const Tf<T> &tf) { return tf.p + rotate(tf.q, l); }

// ---------------------------------------------------------------------------
// Data model (include/phys/dynamics/rigid_body.hpp, collision/collider.hpp,
// collision/manifold.hpp, world/physics_world.hpp)
// ---------------------------------------------------------------------------
enum Shape : int { kSphere = 0, kBox = 1, kHull = 2 };
enum FeatureKind : uint32_t { kFeatSphereSphere = 1, kFeatSphereBox = 2, kFeatBoxFace = 3, kFeatBoxFallback = 4, kFeatHull = 5 };

template <class T> struct Body {
    T mass{}, restitution{}, friction{};
    bool isStatic{};
    V3<T> pos, lin, ang, force;
    Q<T> rot;
    M3<T> invInertiaLocal{};
    uint32_t generation = 0;
    bool alive = false;
    // Sleep flags (rigid_body.hpp:53-58, :132-133)
    bool sleeping = false;
    bool wakeRequested = true;
    // RigidBody::getInverseMass (rigid_body.hpp:72-75)
    T inverseMass() const { return isStatic || mass <= T(0) ? T(0) : T(1) / mass; }
    bool isSleeping() const { return !isStatic && sleeping; }
    void wakeUp() {
        sleeping = false;
        wakeRequested = true;
    }
};

template <class T> struct Aabb {
    V3<T> min, max;
    // Aabb::overlaps (include/phys/collision/aabb.hpp:15-19)
    bool overlaps(const Aabb &o) const {
        return min.x <= o.max.x && max.x >= o.min.x && min.y <= o.max.y && max.y >= o.min.y &&
               min.z <= o.max.z && max.z >= o.min.z;
    }
};

template <class T> struct Collider {
    uint32_t bodyIndex = 0, bodyGeneration = 0;
    Tf<T> local{{}, {T(0), T(0), T(0), T(1)}};
    int shape = kSphere;
    T radius{};
    V3<T> halfExtents;
    int hull = -1;
    Aabb<T> bounds;
    uint32_t generation = 0;
    bool alive = false;
};

template <class T> struct Point {
    V3<T> anchorA, anchorB;
    T penetration{}, normalImpulse{}, tangentImpulse1{}, tangentImpulse2{};
    uint32_t feature = 0;
};

template <class T> struct Manifold {
    uint32_t aIdx = 0, aGen = 0, bIdx = 0, bGen = 0;
    V3<T> normal;
    Point<T> points[4];
    uint32_t pointCount = 0;
    T friction{}, restitution{};
};

template <class T> struct Cached {
    uint32_t aIdx, aGen, bIdx, bGen;
    V3<T> anchorA, anchorB;
    T normalImpulse, tangentImpulse1, tangentImpulse2;
};

struct Stats {
    ow_step_stats s{};
};

template <class T> struct HullShape {
    std::vector<V3<T>> vertices;
};

// ---------------------------------------------------------------------------
// AABB (src/collision/aabb.cpp:8-32), hull bounds project-defined
// ---------------------------------------------------------------------------
template <class T> inline Tf<T> colliderWorld(const Collider<T> &c, const Tf<T> &body) {
    // physics_world.cpp:658-667 / aabb.cpp:10-13
    return {body.p + rotate(body.q, c.local.p), qmul(body.q, c.local.q)};
}

template <class T>
Aabb<T> aabbFromCollider(const Collider<T> &c, const Tf<T> &body, const std::vector<HullShape<T>> &hulls) {
    Tf<T> w = colliderWorld(c, body);
    if (c.shape == kSphere) {
        V3<T> r{c.radius, c.radius, c.radius};
        return {w.p - r, w.p + r};
    }
    if (c.shape == kHull) {
        const auto &verts = hulls[c.hull].vertices;
        Aabb<T> b;
        for (size_t i = 0; i < verts.size(); ++i) {
            V3<T> v = toWorld(verts[i], w);
            if (i == 0) {
                b.min = v;
                b.max = v;
            } else {
                b.min = {smin(b.min.x, v.x), smin(b.min.y, v.y), smin(b.min.z, v.z)};
                b.max = {smax(b.max.x, v.x), smax(b.max.y, v.y), smax(b.max.z, v.z)};
            }
        }
        return b;
    }
    V3<T> h = c.halfExtents;
    M3<T> m = toMat3(w.q);
    V3<T> e{std::abs(m.m00) * h.x + std::abs(m.m01) * h.y + std::abs(m.m02) * h.z,
            std::abs(m.m10) * h.x + std::abs(m.m11) * h.y + std::abs(m.m12) * h.z,
            std::abs(m.m20) * h.x + std::abs(m.m21) * h.y + std::abs(m.m22) * h.z};
    return {w.p - e, w.p + e};
}

// ---------------------------------------------------------------------------
// Broadphase (src/collision/broadphase.cpp)
// ---------------------------------------------------------------------------
using Pair = std::pair<uint32_t, uint32_t>;

// sortPairs / sortPairsLinear (broadphase.cpp:18-60): both yield lexicographic
// (first, second) order; a stable sort on the pair reproduces either.
inline void sortPairsLex(std::vector<Pair> &pairs) { std::sort(pairs.begin(), pairs.end()); }

// The sweep's pair sort (broadphase.cpp:27-60): with at least as many pairs
// as boxes, two stable counting passes (by second, then by first) in linear
// time; otherwise a comparison sort.  Either gives the lexicographic order.
inline void sortPairsLinear(std::vector<Pair> &pairs, size_t keyCount) {
    if (pairs.size() < 2) return;
    if (pairs.size() < keyCount) return sortPairsLex(pairs);
    thread_local std::vector<Pair> buffer;
    thread_local std::vector<size_t> counts;
    buffer.resize(pairs.size());
    auto pass = [&](const std::vector<Pair> &in, std::vector<Pair> &out, auto key) {
        counts.assign(keyCount, 0);
        for (const Pair &p : in) ++counts[key(p)];
        size_t offset = 0;
        for (size_t &c : counts) {
            const size_t n = c;
            c = offset;
            offset += n;
        }
        for (const Pair &p : in) out[counts[key(p)]++] = p;
    };
    pass(pairs, buffer, [](const Pair &p) { return p.second; });
    pass(buffer, pairs, [](const Pair &p) { return p.first; });
}

// SAP: detail::findCandidatePairs (broadphase.cpp:205-290)
template <class T>
void sapPairs(const std::vector<Aabb<T>> &bounds, std::vector<Pair> &pairs, ow_step_stats &st, int threads) {
    struct Entry {
        Aabb<T> b;
        uint32_t idx;
    };
    // kept between calls (the reference's workspace); the pool's threads reach
    // the caller's copies through these references
    thread_local std::vector<Entry> entriesStore;
    thread_local std::vector<std::vector<Pair>> outsStore;
    std::vector<Entry> &entries = entriesStore;
    entries.resize(bounds.size());
    for (uint32_t i = 0; i < bounds.size(); ++i) entries[i] = {bounds[i], i};
    std::sort(entries.begin(), entries.end(), [](const Entry &l, const Entry &r) {
        if (l.b.min.x != r.b.min.x) return l.b.min.x < r.b.min.x;
        return l.idx < r.idx;
    });
    auto sweep = [&](size_t begin, size_t end, std::vector<Pair> &out, uint64_t &cmp) {
        for (size_t i = begin; i < end; ++i) {
            const Entry &f = entries[i];
            size_t j = i + 1;
            for (; j < entries.size(); ++j) {
                const Entry &s = entries[j];
                if (s.b.min.x > f.b.max.x) break;
                if (f.b.min.y <= s.b.max.y && f.b.max.y >= s.b.min.y && f.b.min.z <= s.b.max.z &&
                    f.b.max.z >= s.b.min.z)
                    out.push_back({std::min(f.idx, s.idx), std::max(f.idx, s.idx)});
            }
            cmp += j - i - 1;
        }
    };
    pairs.clear();
    uint64_t cmp = 0;
    if (threads > 1 && entries.size() >= 4096) {
        // Parallel sweep over contiguous ranges (broadphase.cpp:244-274).
        size_t ranges = (size_t)threads * 16;
        std::vector<std::vector<Pair>> &outs = outsStore;
        outs.resize(ranges);
        for (auto &o : outs) o.clear();
        std::vector<uint64_t> cmps(ranges, 0);
        Pool::instance().run(threads, ranges, [&](size_t r) {
            sweep(entries.size() * r / ranges, entries.size() * (r + 1) / ranges, outs[r], cmps[r]);
        });
        for (size_t r = 0; r < ranges; ++r) {
            pairs.insert(pairs.end(), outs[r].begin(), outs[r].end());
            cmp += cmps[r];
        }
    } else {
        sweep(0, entries.size(), pairs, cmp);
    }
    sortPairsLinear(pairs, bounds.size());
    st.x_window_comparisons = cmp;
    st.aabb_pairs = pairs.size();
    st.grid_comparisons = st.grid_entries = st.grid_overflow_aabbs = 0;
    st.grid_cell_size = 0.0;
}

// gridRange (broadphase.cpp:62-88)
template <class T>
bool gridRange(const Aabb<T> &b, double cell, int32_t first[3], int counts[3]) {
    const size_t maxCells = 64;
    double lower[] = {std::floor((double)b.min.x / cell), std::floor((double)b.min.y / cell),
                      std::floor((double)b.min.z / cell)};
    double upper[] = {std::floor((double)b.max.x / cell), std::floor((double)b.max.y / cell),
                      std::floor((double)b.max.z / cell)};
    size_t total = 1;
    for (int a = 0; a < 3; ++a) {
        if (!std::isfinite(lower[a]) || !std::isfinite(upper[a]) ||
            lower[a] < (double)std::numeric_limits<int32_t>::min() ||
            upper[a] > (double)std::numeric_limits<int32_t>::max() || lower[a] > upper[a])
            return false;
        int64_t count = (int64_t)upper[a] - (int64_t)lower[a] + 1;
        if (count > (int64_t)(maxCells / total)) return false;
        first[a] = (int32_t)lower[a];
        counts[a] = (int)count;
        total *= (size_t)count;
    }
    return true;
}

// findGridPairs (broadphase.cpp:90-182); cellSize > 0 overrides the median.
template <class T>
void gridPairs(const std::vector<Aabb<T>> &bounds, double fixedCell, std::vector<Pair> &pairs, ow_step_stats &st) {
    double cell = 1.0;
    if (fixedCell > 0.0) {
        cell = fixedCell;
    } else {
        std::vector<double> widths;
        for (const auto &b : bounds) {
            double w = std::max({(double)b.max.x - (double)b.min.x, (double)b.max.y - (double)b.min.y,
                                 (double)b.max.z - (double)b.min.z});
            if (w > 0.0 && std::isfinite(w)) widths.push_back(w);
        }
        if (!widths.empty()) {
            auto med = widths.begin() + widths.size() / 2;
            std::nth_element(widths.begin(), med, widths.end());
            cell = *med;
        }
    }
    struct CellEntry {
        int32_t c[3];
        uint32_t idx;
    };
    std::vector<CellEntry> entries;
    std::vector<uint8_t> inGrid(bounds.size(), 0);
    std::vector<uint32_t> overflow;
    for (uint32_t i = 0; i < bounds.size(); ++i) {
        int32_t f[3];
        int n[3];
        if (!gridRange(bounds[i], cell, f, n)) {
            overflow.push_back(i);
            continue;
        }
        inGrid[i] = 1;
        for (int x = 0; x < n[0]; ++x)
            for (int y = 0; y < n[1]; ++y)
                for (int z = 0; z < n[2]; ++z) entries.push_back({{f[0] + x, f[1] + y, f[2] + z}, i});
    }
    std::sort(entries.begin(), entries.end(), [](const CellEntry &l, const CellEntry &r) {
        if (l.c[0] != r.c[0]) return l.c[0] < r.c[0];
        if (l.c[1] != r.c[1]) return l.c[1] < r.c[1];
        if (l.c[2] != r.c[2]) return l.c[2] < r.c[2];
        return l.idx < r.idx;
    });
    uint64_t comparisons = 0;
    pairs.clear();
    auto check = [&](uint32_t a, uint32_t b) {
        ++comparisons;
        if (bounds[a].overlaps(bounds[b])) pairs.push_back({std::min(a, b), std::max(a, b)});
    };
    for (size_t begin = 0; begin < entries.size();) {
        size_t end = begin + 1;
        while (end < entries.size() && entries[end].c[0] == entries[begin].c[0] &&
               entries[end].c[1] == entries[begin].c[1] && entries[end].c[2] == entries[begin].c[2])
            ++end;
        for (size_t a = begin; a < end; ++a)
            for (size_t b = a + 1; b < end; ++b) check(entries[a].idx, entries[b].idx);
        begin = end;
    }
    for (uint32_t f : overflow)
        for (uint32_t s = 0; s < bounds.size(); ++s)
            if (f != s && (inGrid[s] || f < s)) check(f, s);
    sortPairsLex(pairs);
    pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
    st.x_window_comparisons = 0;
    st.aabb_pairs = pairs.size();
    st.grid_comparisons = comparisons;
    st.grid_entries = entries.size();
    st.grid_overflow_aabbs = overflow.size();
    st.grid_cell_size = cell;
}

// ---------------------------------------------------------------------------
// SAT (src/collision/sat.cpp:10-102)
// ---------------------------------------------------------------------------
template <class T> struct WorldBox {
    V3<T> center, he;
    Q<T> q;
    V3<T> axis(int i) const {
        M3<T> m = toMat3(q);
        if (i == 0) return {m.m00, m.m10, m.m20};
        if (i == 1) return {m.m01, m.m11, m.m21};
        return {m.m02, m.m12, m.m22};
    }
};
template <class T> T satProjectedRadius(const WorldBox<T> &b, const V3<T> &a) {
    return std::abs(dot(b.axis(0), a)) * b.he.x + std::abs(dot(b.axis(1), a)) * b.he.y +
           std::abs(dot(b.axis(2), a)) * b.he.z;
}
template <class T>
bool overlapOnAxis(const WorldBox<T> &a, const WorldBox<T> &b, V3<T> axis, V3<T> &na, T &depth) {
    T lsq = dot(axis, axis);
    if (lsq < T(1e-8f)) {
        depth = std::numeric_limits<T>::max();
        return true;
    }
    na = axis * (T(1) / std::sqrt(lsq));
    T distance = std::abs(dot(b.center - a.center, na));
    T d = (satProjectedRadius(a, na) + satProjectedRadius(b, na)) - distance;
    if (d < T(0)) return false;
    depth = d;
    return true;
}
template <class T>
bool testOBBOBB(const V3<T> &heA, const Tf<T> &tA, const V3<T> &heB, const Tf<T> &tB, V3<T> &outAxis,
                T &outDepth) {
    outDepth = std::numeric_limits<T>::max();
    WorldBox<T> A{tA.p, heA, tA.q}, B{tB.p, heB, tB.q};
    V3<T> axA[3] = {A.axis(0), A.axis(1), A.axis(2)};
    V3<T> axB[3] = {B.axis(0), B.axis(1), B.axis(2)};
    for (auto &ax : axA) {
        V3<T> na;
        T d;
        if (!overlapOnAxis(A, B, ax, na, d)) return false;
        if (d < outDepth) { outDepth = d; outAxis = na; }
    }
    for (auto &ax : axB) {
        V3<T> na;
        T d;
        if (!overlapOnAxis(A, B, ax, na, d)) return false;
        if (d < outDepth) { outDepth = d; outAxis = na; }
    }
    for (auto &ea : axA)
        for (auto &eb : axB) {
            V3<T> na;
            T d;
            if (!overlapOnAxis(A, B, cross(ea, eb), na, d)) return false;
            if (d < outDepth) { outDepth = d; outAxis = na; }
        }
    return true;
}

// ---------------------------------------------------------------------------
// Narrowphase (src/collision/narrowphase.cpp)
// ---------------------------------------------------------------------------
template <class T> V3<T> boxSupport(const V3<T> &he, const Tf<T> &tf, const V3<T> &dir) {
    V3<T> ld = rotate(conj(tf.q), dir);
    V3<T> lp{ld.x >= T(0) ? he.x : -he.x, ld.y >= T(0) ? he.y : -he.y, ld.z >= T(0) ? he.z : -he.z};
    return toWorld(lp, tf);
}
template <class T> T boxProjectedRadius(const V3<T> &he, const Tf<T> &tf, const V3<T> &axis) {
    M3<T> r = toMat3(tf.q);
    V3<T> a0{r.m00, r.m10, r.m20}, a1{r.m01, r.m11, r.m21}, a2{r.m02, r.m12, r.m22};
    return std::abs(dot(a0, axis)) * he.x + std::abs(dot(a1, axis)) * he.y + std::abs(dot(a2, axis)) * he.z;
}
template <class T>
T overlapMidpoint(const V3<T> &heA, const Tf<T> &tA, const V3<T> &heB, const Tf<T> &tB, const V3<T> &axis) {
    T cA = dot(tA.p, axis), cB = dot(tB.p, axis);
    T rA = boxProjectedRadius(heA, tA, axis), rB = boxProjectedRadius(heB, tB, axis);
    T lower = smax(cA - rA, cB - rB);
    T upper = smin(cA + rA, cB + rB);
    return (lower + upper) * T(0.5f);
}
template <class T>
void supportFaceVertices(const V3<T> &he, const Tf<T> &tf, const V3<T> &dir, V3<T> out[4], int &faceAxis,
                         int &faceSignBit) {
    V3<T> ld = rotate(conj(tf.q), dir);
    faceAxis = 0;
    T largest = std::abs(ld.x);
    if (std::abs(ld.y) > largest) { faceAxis = 1; largest = std::abs(ld.y); }
    if (std::abs(ld.z) > largest) faceAxis = 2;
    T comp = faceAxis == 0 ? ld.x : faceAxis == 1 ? ld.y : ld.z;
    T faceSign = comp >= T(0) ? T(1) : T(-1);
    faceSignBit = comp >= T(0) ? 0 : 1;
    T ext[] = {he.x, he.y, he.z};
    int fa = (faceAxis + 1) % 3, sa = (faceAxis + 2) % 3;
    for (int i = 0; i < 4; ++i) {
        T c[3] = {T(0), T(0), T(0)};
        c[faceAxis] = faceSign * ext[faceAxis];
        c[fa] = (i & 1) ? ext[fa] : -ext[fa];
        c[sa] = (i & 2) ? ext[sa] : -ext[sa];
        out[i] = toWorld(V3<T>{c[0], c[1], c[2]}, tf);
    }
}
template <class T> bool pointInsideBox(const V3<T> &p, const V3<T> &he, const Tf<T> &tf) {
    V3<T> l = rotate(conj(tf.q), p - tf.p);
    const T tol = T(1e-4f);
    return std::abs(l.x) <= he.x + tol && std::abs(l.y) <= he.y + tol && std::abs(l.z) <= he.z + tol;
}
template <class T> bool duplicatePoint(const V3<T> pts[4], uint32_t n, const V3<T> &p) {
    const T tolSq = T(1e-6f);
    for (uint32_t i = 0; i < n; ++i) {
        V3<T> d = pts[i] - p;
        if (dot(d, d) <= tolSq) return true;
    }
    return false;
}

// intersectSphereSphere (narrowphase.cpp:132-160)
template <class T>
bool sphereSphere(T rA, const Tf<T> &tA, T rB, const Tf<T> &tB, Manifold<T> &m) {
    V3<T> delta = tB.p - tA.p;
    T distance = length(delta);
    T radii = rA + rB;
    if (distance >= radii) return false;
    m.normal = distance > T(1e-6f) ? delta / distance : V3<T>{T(1), T(0), T(0)};
    m.pointCount = 1;
    Point<T> &pt = m.points[0];
    pt.penetration = radii - distance;
    V3<T> pA = tA.p + m.normal * rA;
    V3<T> pB = tB.p - m.normal * rB;
    V3<T> wc = (pA + pB) * T(0.5f);
    pt.anchorA = toLocal(wc, tA);
    pt.anchorB = toLocal(wc, tB);
    pt.feature = kFeatSphereSphere << 24;
    return true;
}

// intersectSphereBox (narrowphase.cpp:162-248)
template <class T>
bool sphereBox(T r, const Tf<T> &tS, const V3<T> &he, const Tf<T> &tB, Manifold<T> &m) {
    V3<T> c = rotate(conj(tB.q), tS.p - tB.p);
    V3<T> cl{clampv(c.x, -he.x, he.x), clampv(c.y, -he.y, he.y), clampv(c.z, -he.z, he.z)};
    V3<T> dl = cl - c;
    T distance = length(dl);
    V3<T> nl;
    T pen;
    uint32_t region;
    if (distance > T(1e-6f)) {
        if (distance >= r) return false;
        nl = dl / distance;
        pen = r - distance;
        region = 6;
    } else {
        T dpx = he.x - c.x, dnx = he.x + c.x, dpy = he.y - c.y, dny = he.y + c.y, dpz = he.z - c.z,
          dnz = he.z + c.z;
        T nearest = dpx;
        nl = {T(-1), T(0), T(0)};
        region = 0;
        if (dnx < nearest) { nearest = dnx; nl = {T(1), T(0), T(0)}; region = 1; }
        if (dpy < nearest) { nearest = dpy; nl = {T(0), T(-1), T(0)}; region = 2; }
        if (dny < nearest) { nearest = dny; nl = {T(0), T(1), T(0)}; region = 3; }
        if (dpz < nearest) { nearest = dpz; nl = {T(0), T(0), T(-1)}; region = 4; }
        if (dnz < nearest) { nearest = dnz; nl = {T(0), T(0), T(1)}; region = 5; }
        pen = r + nearest;
    }
    m.normal = rotate(tB.q, nl);
    m.pointCount = 1;
    Point<T> &pt = m.points[0];
    pt.penetration = pen;
    V3<T> bp = toWorld(cl, tB);
    V3<T> sp = tS.p + m.normal * r;
    V3<T> wc = (sp + bp) * T(0.5f);
    pt.anchorA = toLocal(wc, tS);
    pt.anchorB = toLocal(wc, tB);
    pt.feature = (kFeatSphereBox << 24) | region;
    return true;
}

// intersectBoxBox (narrowphase.cpp:250-324); feature IDs project-defined:
// (kind << 24) | (source << 16) | (faceAxis << 8) | (faceSign << 4) | vertex.
template <class T>
bool boxBox(const V3<T> &heA, const Tf<T> &tA, const V3<T> &heB, const Tf<T> &tB, Manifold<T> &m) {
    V3<T> normal;
    T penetration;
    if (!testOBBOBB(heA, tA, heB, tB, normal, penetration)) return false;
    V3<T> cd = tB.p - tA.p;
    if (dot(cd, normal) < T(0)) normal = -normal;
    m.normal = normal;
    V3<T> tref = std::abs(normal.x) < T(0.9f) ? V3<T>{T(1), T(0), T(0)} : V3<T>{T(0), T(1), T(0)};
    V3<T> t1 = normalize(cross(normal, tref));
    V3<T> t2 = cross(normal, t1);
    T nc = (dot(tA.p, normal) + boxProjectedRadius(heA, tA, normal) + dot(tB.p, normal) -
            boxProjectedRadius(heB, tB, normal)) *
           T(0.5f);
    V3<T> fallback = normal * nc + t1 * overlapMidpoint(heA, tA, heB, tB, t1) + t2 * overlapMidpoint(heA, tA, heB, tB, t2);
    V3<T> contacts[4];
    T depths[4];
    uint32_t feats[4];
    uint32_t count = 0;
    auto addFace = [&](const V3<T> &srcHe, const Tf<T> &srcTf, const V3<T> &othHe, const Tf<T> &othTf,
                       V3<T> dir, uint32_t source) {
        T otherSurface = dot(boxSupport(othHe, othTf, -dir), dir);
        V3<T> verts[4];
        int faceAxis, signBit;
        supportFaceVertices(srcHe, srcTf, dir, verts, faceAxis, signBit);
        for (uint32_t vi = 0; vi < 4; ++vi) {
            const V3<T> &v = verts[vi];
            if (!pointInsideBox(v, othHe, othTf)) continue;
            T depth = smax(dot(v, dir) - otherSurface, T(0));
            V3<T> cand = v - dir * (depth * T(0.5f));
            if (count < 4 && !duplicatePoint(contacts, count, cand)) {
                depths[count] = depth;
                feats[count] = (kFeatBoxFace << 24) | (source << 16) | ((uint32_t)faceAxis << 8) |
                               ((uint32_t)signBit << 4) | vi;
                contacts[count++] = cand;
            }
        }
    };
    addFace(heA, tA, heB, tB, normal, 0);
    addFace(heB, tB, heA, tA, -normal, 1);
    if (count == 0) {
        depths[count] = penetration;
        feats[count] = kFeatBoxFallback << 24;
        contacts[count++] = fallback;
    }
    m.pointCount = count;
    for (uint32_t i = 0; i < count; ++i) {
        Point<T> &pt = m.points[i];
        pt.penetration = depths[i];
        pt.anchorA = toLocal(contacts[i], tA);
        pt.anchorB = toLocal(contacts[i], tB);
        pt.feature = feats[i];
    }
    return true;
}

// ---------------------------------------------------------------------------
// GJK / EPA (src/collision/gjk.cpp:11-158, src/collision/epa.cpp:29-130) over
// support maps; EPA storage bounded like the GPU path (failure on overflow).
// ---------------------------------------------------------------------------
constexpr int kEpaMaxVertices = 4 + 64;
constexpr int kEpaMaxFaces = 256;
constexpr int kEpaMaxHorizon = 128;

template <class T> struct Simplex {
    V3<T> p[4];
    uint32_t size = 0;
};
template <class T> inline V3<T> tripleCross(const V3<T> &a, const V3<T> &b, const V3<T> &c) {
    return cross(cross(a, b), c);
}
template <class T> inline T lenSq(const V3<T> &v) { return dot(v, v); }

// setLineDirection (gjk.cpp:21-41)
template <class T> bool gjkLine(Simplex<T> &s, V3<T> &dir) {
    V3<T> A = s.p[0], B = s.p[1];
    V3<T> toO = -A;
    V3<T> e = B - A;
    if (dot(e, toO) > T(0)) {
        dir = tripleCross(e, toO, e);
        if (lenSq(dir) < T(1e-12f)) dir = cross(e, V3<T>{T(1), T(0), T(0)});
        if (lenSq(dir) < T(1e-12f)) dir = cross(e, V3<T>{T(0), T(1), T(0)});
    } else {
        s.p[0] = A;
        s.size = 1;
        dir = toO;
    }
    return false;
}
// setTriangleDirection (gjk.cpp:43-74)
template <class T> bool gjkTriangle(Simplex<T> &s, V3<T> &dir) {
    V3<T> A = s.p[0], B = s.p[1], C = s.p[2];
    V3<T> toO = -A;
    V3<T> ab = B - A, ac = C - A;
    V3<T> n = cross(ab, ac);
    if (dot(cross(n, ac), toO) > T(0)) {
        if (dot(ac, toO) > T(0)) {
            s.p[1] = C;
            s.size = 2;
            dir = tripleCross(ac, toO, ac);
            return false;
        }
        return gjkLine(s, dir);
    }
    if (dot(cross(ab, n), toO) > T(0)) return gjkLine(s, dir);
    if (dot(n, toO) > T(0)) {
        dir = n;
    } else {
        std::swap(s.p[1], s.p[2]);
        dir = -n;
    }
    return false;
}
// containsOrigin (gjk.cpp:76-124).  The third face case assigns through
// references into the simplex it is rewriting (points[1] = D, then
// points[2] = pointB, which now aliases D); that behaviour is kept.
template <class T> bool gjkContains(Simplex<T> &s, V3<T> &dir) {
    if (s.size == 1) {
        dir = -s.p[0];
        return false;
    }
    if (s.size == 2) return gjkLine(s, dir);
    if (s.size == 3) return gjkTriangle(s, dir);
    V3<T> A = s.p[0];
    V3<T> toO = -A;
    auto outside = [&](const V3<T> &fb, const V3<T> &fc, const V3<T> &op) {
        V3<T> n = cross(fb - A, fc - A);
        if (dot(n, op - A) > T(0)) n = -n;
        return dot(n, toO) > T(0);
    };
    if (outside(s.p[1], s.p[2], s.p[3])) {
        s.size = 3;
        return gjkTriangle(s, dir);
    }
    if (outside(s.p[2], s.p[3], s.p[1])) {
        s.p[1] = s.p[2];
        s.p[2] = s.p[3];
        s.size = 3;
        return gjkTriangle(s, dir);
    }
    if (outside(s.p[3], s.p[1], s.p[2])) {
        s.p[1] = s.p[3];
        s.p[2] = s.p[1];
        s.size = 3;
        return gjkTriangle(s, dir);
    }
    return true;
}

template <class T, class SA, class SB>
bool gjk(const SA &supA, const SB &supB, Simplex<T> &out, uint32_t maxIt = 32) {
    Simplex<T> s;
    V3<T> dir{T(1), T(0), T(0)};
    for (uint32_t it = 0; it < maxIt; ++it) {
        if (lenSq(dir) < T(1e-12f)) break;
        V3<T> p = supA(dir) - supB(-dir);
        if (dot(p, dir) <= T(0)) break;
        for (uint32_t i = std::min(s.size, 3u); i > 0; --i) s.p[i] = s.p[i - 1];
        s.p[0] = p;
        s.size = std::min(s.size + 1, 4u);
        if (gjkContains(s, dir)) {
            out = s;
            return true;
        }
    }
    out = s;
    return false;
}

template <class T> struct EpaFace {
    uint32_t a, b, c;
    V3<T> n;
    T d;
};
template <class T> EpaFace<T> makeFace(const V3<T> *v, uint32_t a, uint32_t b, uint32_t c) {
    V3<T> n = cross(v[b] - v[a], v[c] - v[a]);
    T len = length(n);
    if (len > T(1e-8f)) n = n * (T(1) / len);
    T d = dot(n, v[a]);
    if (d < T(0)) {
        std::swap(b, c);
        n = -n;
        d = -d;
    }
    return {a, b, c, n, d};
}

// Returns 1 success, 0 failure (degenerate, iteration cap or storage cap).
template <class T, class SA, class SB>
int epa(const SA &supA, const SB &supB, const Simplex<T> &s, V3<T> &normal, T &depth, uint32_t maxIt = 64,
        T tol = T(1e-4f)) {
    normal = {};
    depth = T(0);
    if (s.size < 4 || maxIt == 0) return 0;
    V3<T> v[kEpaMaxVertices];
    uint32_t nv = 0;
    for (uint32_t i = 0; i < s.size; ++i) v[nv++] = s.p[i];
    EpaFace<T> faces[kEpaMaxFaces];
    uint32_t nf = 0;
    faces[nf++] = makeFace(v, 0, 1, 2);
    faces[nf++] = makeFace(v, 0, 3, 1);
    faces[nf++] = makeFace(v, 0, 2, 3);
    faces[nf++] = makeFace(v, 1, 3, 2);
    for (uint32_t it = 0; it < maxIt; ++it) {
        if (nf == 0) return 0;
        uint32_t ci = 0;
        for (uint32_t f = 1; f < nf; ++f)
            if (faces[f].d < faces[ci].d) ci = f;
        EpaFace<T> cf = faces[ci];
        V3<T> sup = supA(cf.n) - supB(-cf.n);
        T sd = dot(sup, cf.n);
        if (sd - cf.d <= tol) {
            normal = cf.n;
            depth = smax(cf.d, T(0));
            return 1;
        }
        if (nv >= (uint32_t)kEpaMaxVertices) return 0;
        uint32_t si = nv;
        v[nv++] = sup;
        uint32_t he[kEpaMaxHorizon][2];
        uint32_t nh = 0;
        bool overflow = false;
        auto addEdge = [&](uint32_t a, uint32_t b) {
            for (uint32_t k = 0; k < nh; ++k)
                if (he[k][0] == b && he[k][1] == a) {
                    for (uint32_t m = k + 1; m < nh; ++m) { he[m - 1][0] = he[m][0]; he[m - 1][1] = he[m][1]; }
                    --nh;
                    return;
                }
            if (nh >= (uint32_t)kEpaMaxHorizon) { overflow = true; return; }
            he[nh][0] = a;
            he[nh][1] = b;
            ++nh;
        };
        uint32_t kept = 0;
        for (uint32_t f = 0; f < nf; ++f) {
            const EpaFace<T> face = faces[f];
            T vis = dot(face.n, sup - v[face.a]);
            if (vis > tol) {
                addEdge(face.a, face.b);
                addEdge(face.b, face.c);
                addEdge(face.c, face.a);
            } else {
                faces[kept++] = face;
            }
        }
        if (overflow) return 0;
        if (nh == 0) return 0;
        nf = kept;
        if (nf + nh > (uint32_t)kEpaMaxFaces) return 0;
        for (uint32_t k = 0; k < nh; ++k) faces[nf++] = makeFace(v, he[k][0], he[k][1], si);
    }
    return 0;
}

// Support maps (project-defined for sphere and hull; box = boxSupportPoint).
template <class T> struct Support {
    int shape;
    T radius;
    V3<T> he;
    const V3<T> *verts;
    uint32_t nverts;
    Tf<T> tf;
    mutable uint32_t lastIndex = 0xFFu;
    V3<T> operator()(const V3<T> &dir) const {
        if (shape == kBox) return boxSupport(he, tf, dir);
        if (shape == kSphere) return tf.p + normalize(dir) * radius;
        V3<T> ld = rotate(conj(tf.q), dir);
        uint32_t best = 0;
        T bd = dot(verts[0], ld);
        for (uint32_t i = 1; i < nverts; ++i) {
            T d = dot(verts[i], ld);
            if (d > bd) { bd = d; best = i; }
        }
        lastIndex = best;
        return toWorld(verts[best], tf);
    }
};

// Hull contact (project-defined): GJK, EPA normal (A toward B) and depth, one
// point midway between A's support along n and B's support along -n.
template <class T>
bool hullContact(const Support<T> &A, const Support<T> &B, Manifold<T> &m, bool &epaFailed) {
    Simplex<T> s;
    epaFailed = false;
    if (!gjk<T>(A, B, s)) return false;
    V3<T> n;
    T depth;
    if (!epa<T>(A, B, s, n, depth)) {
        epaFailed = true;
        return false;
    }
    m.normal = n;
    m.pointCount = 1;
    V3<T> pa = A(n);
    uint32_t ia = A.shape == kHull ? A.lastIndex : 0xFFu;
    V3<T> pb = B(-n);
    uint32_t ib = B.shape == kHull ? B.lastIndex : 0xFFu;
    V3<T> wc = (pa + pb) * T(0.5f);
    Point<T> &pt = m.points[0];
    pt.penetration = depth;
    pt.anchorA = toLocal(wc, A.tf);
    pt.anchorB = toLocal(wc, B.tf);
    pt.feature = (kFeatHull << 24) | ((ia & 0xFFu) << 8) | (ib & 0xFFu);
    return true;
}

// NarrowPhase::generateContact (narrowphase.cpp:326-374) + hulls.
template <class T>
bool generateContact(const Collider<T> &a, const Tf<T> &tA, const Collider<T> &b, const Tf<T> &tB,
                     const std::vector<HullShape<T>> &hulls, Manifold<T> &m) {
    if (a.shape == kHull || b.shape == kHull) {
        auto mk = [&](const Collider<T> &c, const Tf<T> &t) {
            Support<T> s{c.shape, c.radius, c.halfExtents, nullptr, 0, t};
            if (c.shape == kHull) {
                s.verts = hulls[c.hull].vertices.data();
                s.nverts = (uint32_t)hulls[c.hull].vertices.size();
            }
            return s;
        };
        bool failed;
        return hullContact(mk(a, tA), mk(b, tB), m, failed);
    }
    if (a.shape == kSphere && b.shape == kSphere) return sphereSphere(a.radius, tA, b.radius, tB, m);
    if (a.shape == kSphere && b.shape == kBox) return sphereBox(a.radius, tA, b.halfExtents, tB, m);
    if (a.shape == kBox && b.shape == kSphere) {
        bool hit = sphereBox(b.radius, tB, a.halfExtents, tA, m);
        if (hit) {
            m.normal = -m.normal;
            for (uint32_t i = 0; i < m.pointCount; ++i) std::swap(m.points[i].anchorA, m.points[i].anchorB);
        }
        return hit;
    }
    return boxBox(a.halfExtents, tA, b.halfExtents, tB, m);
}

// ---------------------------------------------------------------------------
// Graph colouring of manifolds (project-defined; the GPU solve order).
// Priority is a bijective 32-bit mix of the manifold index; the colouring is
// greedy in decreasing priority: each manifold takes the smallest colour not
// used by a higher-priority manifold sharing one of its non-static bodies.
// Solve order: (colour ascending, manifold index ascending).
// ---------------------------------------------------------------------------
inline uint32_t colorPriority(uint32_t m) {
    uint32_t h = m;
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

// ---------------------------------------------------------------------------
// World
// ---------------------------------------------------------------------------
struct WorldBase {
    virtual ~WorldBase() = default;
    virtual WorldBase *clone() const = 0;
    // wall time of the last step's stages (ms): integrate + bounds, broadphase,
    // narrowphase, colouring / order, solve, pose, total; then the solve's
    // prepare, warm start, velocity iterations and cache update
    double stageMs[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
};
inline double msSince(std::chrono::steady_clock::time_point &t) {
    const auto now = std::chrono::steady_clock::now();
    const double ms = std::chrono::duration<double, std::milli>(now - t).count();
    t = now;
    return ms;
}

template <class T> struct World : WorldBase {
    V3<T> gravity{T(0), T(-9.81f), T(0)};
    int algo = 0;
    double cellSize = 0.0;
    int iterations = 8;
    int orderMode = 0;
    int threads = 1;
    std::vector<Body<T>> bodies;
    std::vector<uint32_t> freeBodies;
    std::vector<Collider<T>> colliders;
    std::vector<uint32_t> freeColliders;
    std::vector<HullShape<T>> hulls;
    std::vector<Manifold<T>> contacts;
    std::vector<Pair> pairs;
    std::vector<Cached<T>> cache;
    std::vector<Cached<T>> wsNextCache;  // the next cache's storage, kept between steps
    std::vector<uint32_t> order, colors;
    ow_step_stats stats{};

    WorldBase *clone() const override { return new World<T>(*this); }

    Body<T> *getBody(uint32_t idx, uint32_t gen) {
        if (idx >= bodies.size()) return nullptr;
        Body<T> &b = bodies[idx];
        if (!b.alive || b.generation != gen) return nullptr;
        return &b;
    }

    // PhysicsWorld::addBody (physics_world.cpp:162-179)
    uint32_t addBody(const Body<T> &b, uint32_t &gen) {
        if (!freeBodies.empty()) {
            uint32_t idx = freeBodies.back();
            freeBodies.pop_back();
            uint32_t g = bodies[idx].generation;
            bodies[idx] = b;
            bodies[idx].generation = g;
            bodies[idx].alive = true;
            bodies[idx].wakeUp();
            gen = g;
            return idx;
        }
        bodies.push_back(b);
        bodies.back().generation = 0;
        bodies.back().alive = true;
        bodies.back().wakeUp();
        gen = 0;
        return (uint32_t)bodies.size() - 1;
    }
    // PhysicsWorld::addCollider (physics_world.cpp:276-298)
    uint32_t addCollider(const Collider<T> &c, uint32_t &gen) {
        if (Body<T> *b = getBody(c.bodyIndex, c.bodyGeneration)) b->wakeUp();
        if (!freeColliders.empty()) {
            uint32_t idx = freeColliders.back();
            freeColliders.pop_back();
            uint32_t g = colliders[idx].generation;
            colliders[idx] = c;
            colliders[idx].generation = g;
            colliders[idx].alive = true;
            if (idx < sleepColliders.size()) sleepColliders[idx] = colliders[idx];
            gen = g;
            return idx;
        }
        colliders.push_back(c);
        colliders.back().generation = 0;
        colliders.back().alive = true;
        gen = 0;
        return (uint32_t)colliders.size() - 1;
    }
    // PhysicsWorld::removeBody (physics_world.cpp:223-250)
    void removeBody(uint32_t idx, uint32_t gen) {
        if (idx >= bodies.size()) return;
        Body<T> &b = bodies[idx];
        if (!b.alive || b.generation != gen) return;
        wakeContacts(idx, gen);
        b.alive = false;
        b.generation++;
        freeBodies.push_back(idx);
        for (uint32_t i = 0; i < colliders.size(); ++i) {
            Collider<T> &c = colliders[i];
            if (c.alive && c.bodyIndex == idx && c.bodyGeneration == gen) {
                c.alive = false;
                c.generation++;
                freeColliders.push_back(i);
            }
        }
    }

    // PhysicsWorld::removeCollider (physics_world.cpp:300-315)
    void removeCollider(uint32_t idx, uint32_t gen) {
        if (idx >= colliders.size()) return;
        Collider<T> &c = colliders[idx];
        if (!c.alive || c.generation != gen) return;
        if (Body<T> *b = getBody(c.bodyIndex, c.bodyGeneration)) b->wakeUp();
        wakeContacts(c.bodyIndex, c.bodyGeneration);
        c.alive = false;
        c.generation++;
        freeColliders.push_back(idx);
    }

    // ---------------- sleeping (physics_world.cpp:341-516) -------------------
    struct SleepState {
        Tf<T> pose{{}, {T(0), T(0), T(0), T(1)}};
        T mass{}, restitution{}, friction{};
        bool isStatic = false;
        bool integratedVelocity = false;
        uint32_t parent = 0;
        bool hasAwake = false, hasSleeping = false, needsWake = false;
        T quietTime{}, islandQuietTime{};
    };
    bool sleepingEnabled = false;
    V3<T> sleepGravity{};
    std::vector<SleepState> sleepStates;
    std::vector<Collider<T>> sleepColliders;

    // PhysicsWorld::setSleepingEnabled (physics_world.cpp:341-351)
    void setSleepingEnabled(bool enabled) {
        if (sleepingEnabled == enabled) return;
        sleepingEnabled = enabled;
        sleepStates.clear();
        sleepColliders.clear();
        for (auto &b : bodies)
            if (b.alive) b.wakeUp();
    }
    // PhysicsWorld::wakeContacts (physics_world.cpp:353-371): the dynamic bodies
    // touching a body in the last step's contacts.
    void wakeContacts(uint32_t idx, uint32_t gen) {
        if (!sleepingEnabled) return;
        for (const Manifold<T> &m : contacts) {
            if (m.aIdx == idx && m.aGen == gen)
                if (Body<T> *o = getBody(m.bIdx, m.bGen); o && !o->isStatic) o->wakeUp();
            if (m.bIdx == idx && m.bGen == gen)
                if (Body<T> *o = getBody(m.aIdx, m.aGen); o && !o->isStatic) o->wakeUp();
        }
    }
    // PhysicsWorld::sleepRoot (physics_world.cpp:373-381), path halving.
    uint32_t sleepRoot(uint32_t i) {
        while (sleepStates[i].parent != i) {
            sleepStates[i].parent = sleepStates[sleepStates[i].parent].parent;
            i = sleepStates[i].parent;
        }
        return i;
    }
    // PhysicsWorld::wakeSleepIslands (physics_world.cpp:383-432): islands are
    // the dynamic bodies joined by contacts (a static body joins nothing); an
    // island with a wake request, or with awake and sleeping bodies, wakes.
    void wakeSleepIslands() {
        for (uint32_t i = 0; i < bodies.size(); ++i) {
            SleepState &st = sleepStates[i];
            st.parent = i;
            st.hasAwake = st.hasSleeping = st.needsWake = false;
        }
        for (const Manifold<T> &m : contacts) {
            Body<T> *A = getBody(m.aIdx, m.aGen), *B = getBody(m.bIdx, m.bGen);
            if (!A || !B || m.pointCount == 0) continue;
            if (!A->isStatic && !B->isStatic) {
                uint32_t ra = sleepRoot(m.aIdx), rb = sleepRoot(m.bIdx);
                sleepStates[std::max(ra, rb)].parent = std::min(ra, rb);
            } else if (A->isStatic && A->wakeRequested && !B->isStatic) {
                B->wakeUp();
            } else if (B->isStatic && B->wakeRequested && !A->isStatic) {
                A->wakeUp();
            }
        }
        for (uint32_t i = 0; i < bodies.size(); ++i) {
            const Body<T> &b = bodies[i];
            if (!b.alive || b.isStatic) continue;
            SleepState &island = sleepStates[sleepRoot(i)];
            island.hasAwake |= !b.isSleeping();
            island.hasSleeping |= b.isSleeping();
            island.needsWake |= b.wakeRequested;
        }
        for (uint32_t i = 0; i < bodies.size(); ++i) {
            Body<T> &b = bodies[i];
            if (!b.alive || b.isStatic) continue;
            const SleepState &island = sleepStates[sleepRoot(i)];
            if (island.needsWake || (island.hasAwake && island.hasSleeping)) {
                b.wakeUp();
                sleepStates[i].quietTime = T(0);
            }
        }
    }
    static bool sameV(const V3<T> &a, const V3<T> &b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
    static bool sameTf(const Tf<T> &a, const Tf<T> &b) {
        return sameV(a.p, b.p) && a.q.x == b.q.x && a.q.y == b.q.y && a.q.z == b.q.z && a.q.w == b.q.w;
    }
    // sameColliderGeometry (physics_world.cpp:38-46)
    static bool sameGeometry(const Collider<T> &a, const Collider<T> &b) {
        if (a.bodyIndex != b.bodyIndex || a.bodyGeneration != b.bodyGeneration || !sameTf(a.local, b.local) ||
            a.shape != b.shape)
            return false;
        if (a.shape == kSphere) return a.radius == b.radius;
        if (a.shape == kBox) return sameV(a.halfExtents, b.halfExtents);
        return a.hull == b.hull;
    }
    // PhysicsWorld::prepareSleeping (physics_world.cpp:434-466): edits since the
    // last step (gravity, mass, material, static flag, pose, collider geometry)
    // wake the bodies they touch.
    void prepareSleeping() {
        sleepStates.resize(bodies.size());
        const size_t previousColliders = sleepColliders.size();
        sleepColliders.resize(colliders.size());
        const bool gravityChanged = !sameV(gravity, sleepGravity);
        for (uint32_t i = 0; i < bodies.size(); ++i) {
            Body<T> &b = bodies[i];
            if (!b.alive) continue;
            const SleepState &prev = sleepStates[i];
            if (gravityChanged || prev.mass != b.mass || prev.isStatic != b.isStatic || prev.friction != b.friction ||
                prev.restitution != b.restitution || !sameTf(prev.pose, Tf<T>{b.pos, b.rot}))
                b.wakeUp();
        }
        for (uint32_t i = 0; i < colliders.size(); ++i) {
            const Collider<T> &c = colliders[i];
            if (!c.alive || sameGeometry(c, sleepColliders[i])) continue;
            if (i < previousColliders)
                if (Body<T> *old = getBody(sleepColliders[i].bodyIndex, sleepColliders[i].bodyGeneration)) old->wakeUp();
            if (Body<T> *b = getBody(c.bodyIndex, c.bodyGeneration)) b->wakeUp();
        }
        wakeSleepIslands();
    }
    // PhysicsWorld::finishSleeping (physics_world.cpp:468-516): half a second of
    // island-wide quiet (|v|^2 and |w|^2 <= 0.05^2, no wake request) puts an
    // island to sleep with zero velocities.
    void finishSleeping(T dt) {
        const T quietSpeedSquared = T(0.05f) * T(0.05f);
        const T timeToSleep = T(0.5f);
        for (SleepState &st : sleepStates) st.islandQuietTime = std::numeric_limits<T>::max();
        for (uint32_t i = 0; i < bodies.size(); ++i) {
            Body<T> &b = bodies[i];
            if (!b.alive || b.isStatic) continue;
            SleepState &st = sleepStates[i];
            if (!b.isSleeping()) {
                if (!b.wakeRequested && dt > T(0) && std::isfinite(dt) && dot(b.lin, b.lin) <= quietSpeedSquared &&
                    dot(b.ang, b.ang) <= quietSpeedSquared)
                    st.quietTime = std::min(st.quietTime + dt, timeToSleep);
                else
                    st.quietTime = T(0);
            }
            SleepState &island = sleepStates[sleepRoot(i)];
            island.islandQuietTime = std::min(island.islandQuietTime, st.quietTime);
        }
        for (uint32_t i = 0; i < bodies.size(); ++i) {
            Body<T> &b = bodies[i];
            if (!b.alive) continue;
            if (!b.isStatic && sleepStates[sleepRoot(i)].islandQuietTime >= timeToSleep) {
                b.sleeping = true;
                b.lin = b.ang = V3<T>{};
            }
            SleepState &st = sleepStates[i];
            st.pose = Tf<T>{b.pos, b.rot};
            st.mass = b.mass;
            st.isStatic = b.isStatic;
            st.friction = b.friction;
            st.restitution = b.restitution;
            b.wakeRequested = false;
        }
        for (uint32_t i = 0; i < colliders.size(); ++i)
            if (colliders[i].alive) sleepColliders[i] = colliders[i];
        sleepGravity = gravity;
    }

    // RigidBody::integrateVelocity (rigid_body.cpp:94-101)
    void integrateVelocity(Body<T> &b, T dt) {
        if (b.isStatic || b.sleeping) return;
        V3<T> acc = gravity + b.force * b.inverseMass();
        b.lin += acc * dt;
    }
    // RigidBody::integratePosition / integrateRotation (rigid_body.cpp:103-125)
    static void integratePose(Body<T> &b, T dt) {
        if (b.isStatic || b.sleeping) return;
        b.pos += b.lin * dt;
        Q<T> spin{b.ang.x, b.ang.y, b.ang.z, T(0)};
        Q<T> d = qmul(spin, b.rot);
        T h = T(0.5f) * dt;
        b.rot.x += h * d.x;
        b.rot.y += h * d.y;
        b.rot.z += h * d.z;
        b.rot.w += h * d.w;
        b.rot = qnormalized(b.rot);
    }

    // ---------------- solver (src/solver/sequential_impulse_solver.cpp) -----
    struct PBody {
        Body<T> *body = nullptr;
        T invMass{};
        M3<T> invI{};
    };
    struct PPoint {
        V3<T> offA, offB, t1, t2, nrA, nrB, trA1, trB1, trA2, trB2;
        T iem{}, itm00{}, itm01{}, itm11{}, ntr1{}, ntr2{}, bias{}, rv{};
    };
    struct PManifold {
        Manifold<T> *m;
        PBody *a, *b;
        PPoint p[4];
    };
    // Per-step work arrays kept between steps (the reference keeps its step
    // workspace the same way, step_workspace.hpp): re-allocating megabytes a
    // step would touch fresh pages every step.
    std::vector<PBody> wsBodies;
    std::vector<uint8_t> wsBodyDone;
    std::vector<PManifold> wsManifolds;
    std::vector<Aabb<T>> wsBounds;
    std::vector<uint32_t> wsSlots;
    std::vector<uint64_t> wsPerBody;
    std::vector<Manifold<T>> wsResults;
    std::vector<int8_t> wsHit;
    std::vector<uint32_t> wsIslandStart, wsIslandItems, wsIslandJobs, wsParent, wsLookup, wsIslandOf, wsCounts,
        wsPoints, wsFill;

    // prepareContactPoints (sequential_impulse_solver.cpp:101-214)
    static size_t preparePoints(PManifold &pm, T inverseDt) {
        const T slop = T(0.005f);
        Manifold<T> &m = *pm.m;
        Body<T> *A = pm.a->body, *B = pm.b->body;
        size_t count = 0;
        for (uint32_t i = 0; i < m.pointCount; ++i) {
            Point<T> &pt = m.points[i];
            PPoint &pp = pm.p[i];
            pp.offA = rotate(A->rot, pt.anchorA);
            pp.offB = rotate(B->rot, pt.anchorB);
            V3<T> tref = std::abs(m.normal.x) < T(0.9f) ? V3<T>{T(1), T(0), T(0)} : V3<T>{T(0), T(1), T(0)};
            pp.t1 = cross(m.normal, tref);
            T tl = std::sqrt(dot(pp.t1, pp.t1));
            if (tl <= T(1e-6f)) continue;
            pp.t1 = pp.t1 / tl;
            pp.t2 = cross(m.normal, pp.t1);
            V3<T> vA = A->lin + cross(A->ang, pp.offA);
            V3<T> vB = B->lin + cross(B->ang, pp.offB);
            T vin = dot(vB - vA, m.normal);
            V3<T> jA = cross(pp.offA, m.normal), jB = cross(pp.offB, m.normal);
            pp.nrA = mul(pm.a->invI, jA);
            pp.nrB = mul(pm.b->invI, jB);
            T ims = pm.a->invMass + pm.b->invMass;
            pp.iem = ims + dot(jA, pp.nrA) + dot(jB, pp.nrB);
            V3<T> tjA = cross(pp.offA, pp.t1), tjB = cross(pp.offB, pp.t1);
            pp.trA1 = mul(pm.a->invI, tjA);
            pp.trB1 = mul(pm.b->invI, tjB);
            T tm00 = ims + dot(tjA, pp.trA1) + dot(tjB, pp.trB1);
            pp.ntr1 = ims * dot(m.normal, pp.t1) + dot(tjA, pp.nrA) + dot(tjB, pp.nrB);
            tjA = cross(pp.offA, pp.t2);
            tjB = cross(pp.offB, pp.t2);
            pp.trA2 = mul(pm.a->invI, tjA);
            pp.trB2 = mul(pm.b->invI, tjB);
            T tm11 = ims + dot(tjA, pp.trA2) + dot(tjB, pp.trB2);
            pp.ntr2 = ims * dot(m.normal, pp.t2) + dot(tjA, pp.nrA) + dot(tjB, pp.nrB);
            T tm01 = dot(tjA, pp.trA1) + dot(tjB, pp.trB1);
            T det = tm00 * tm11 - tm01 * tm01;
            if (det > T(0)) {
                T inv = T(1) / det;
                pp.itm00 = tm11 * inv;
                pp.itm01 = -tm01 * inv;
                pp.itm11 = tm00 * inv;
            } else {
                pp.itm00 = pp.itm01 = pp.itm11 = T(0);
            }
            if (pp.iem <= T(0)) continue;
            ++count;
            pp.bias = smax(pt.penetration - slop, T(0)) * (T(0.2f) * inverseDt);
            pp.rv = vin < T(-1) ? m.restitution * vin : T(0);
        }
        return count;
    }

    static bool cacheLess(uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0, uint32_t b1,
                          uint32_t b2, uint32_t b3) {
        if (a0 != b0) return a0 < b0;
        if (a1 != b1) return a1 < b1;
        if (a2 != b2) return a2 < b2;
        return a3 < b3;
    }

    // SequentialImpulseSolver::solve (sequential_impulse_solver.cpp:226-684),
    // serial path, iteration count and order as parameters.
    void solve(std::vector<Manifold<T>> &cs, T dt, int iters, const uint32_t *ord) {
        auto &ss = stats;
        auto sclk = std::chrono::steady_clock::now();
        ss.prepared_points = ss.warm_start_comparisons = ss.warm_start_matches = ss.velocity_point_visits = 0;
        const T inverseDt = T(1) / smax(dt, T(1e-6f));
        std::vector<PBody> &pbodies = wsBodies;
        std::vector<uint8_t> &pdone = wsBodyDone;
        pbodies.resize(bodies.size());
        pdone.assign(bodies.size(), 0);
        auto prepareBody = [&](Body<T> *b, uint32_t idx) -> PBody * {
            PBody &p = pbodies[idx];
            if (!pdone[idx]) {
                p.body = b;
                p.invMass = b->inverseMass();
                M3<T> R = toMat3(b->rot);
                p.invI = mul(mul(R, b->invInertiaLocal), transpose(R));
                pdone[idx] = 1;
            }
            return &p;
        };
        std::vector<PManifold> &pc = wsManifolds;
        pc.clear();
        pc.reserve(cs.size());
        size_t prepared = 0;
        // With more than one worker and at least 4,096 contacts the reference
        // prepares the contact points on its workers after the bodies
        // (sequential_impulse_solver.cpp:312-350); each manifold's points
        // depend only on it and its two prepared bodies.
        const bool deferPreparation = threads > 1 && cs.size() >= 4096;
        for (size_t k = 0; k < cs.size(); ++k) {
            Manifold<T> &m = cs[ord ? ord[k] : k];
            Body<T> *A = getBody(m.aIdx, m.aGen), *B = getBody(m.bIdx, m.bGen);
            if (!A || !B) continue;
            // contacts among static and sleeping bodies only are not solved (:321-324)
            if (sleepingEnabled && (A->isStatic || A->isSleeping()) && (B->isStatic || B->isSleeping())) continue;
            PManifold p{};
            p.m = &m;
            p.a = prepareBody(A, m.aIdx);
            p.b = prepareBody(B, m.bIdx);
            if (!deferPreparation) prepared += preparePoints(p, inverseDt);
            pc.push_back(p);
        }
        if (deferPreparation) {
            std::vector<size_t> counts((pc.size() + 63) / 64, 0);
            Pool::instance().run(threads, counts.size(), [&](size_t chunk) {
                for (size_t k = 64 * chunk, e = std::min(pc.size(), k + 64); k < e; ++k)
                    counts[chunk] += preparePoints(pc[k], inverseDt);
            });
            for (size_t c : counts) prepared += c;
        }
        ss.solved_contact_count = pc.size();
        ss.prepared_points = prepared;
        stageMs[7] = msSince(sclk);

        auto applyCached = [](const PBody &p, const V3<T> &imp, const V3<T> &off) {
            Body<T> *b = p.body;
            if (b->isStatic) return;
            b->lin += imp * p.invMass;
            b->ang += mul(p.invI, cross(off, imp));
        };
        auto applyAxis = [](const PBody &p, const V3<T> &imp, const V3<T> &resp, T mag) {
            Body<T> *b = p.body;
            if (b->isStatic) return;
            b->lin += imp * p.invMass;
            b->ang += resp * mag;
        };
        auto applyTangent = [](const PBody &p, const V3<T> &imp, const V3<T> &resp) {
            Body<T> *b = p.body;
            if (b->isStatic) return;
            b->lin += imp * p.invMass;
            b->ang += resp;
        };

        // Islands (sequential_impulse_solver.cpp:366-442): with more than one
        // worker and at least 4,096 solved contacts the reference solves the
        // islands (contacts joined by shared non-static bodies) in parallel,
        // each in solve order; islands share no moving body, so the result is
        // the serial one.
        std::vector<uint32_t> &islandStart = wsIslandStart, &islandItems = wsIslandItems, &islandJobs = wsIslandJobs;
        const bool parallelIslands = threads > 1 && pc.size() >= 4096;
        if (parallelIslands) {
            std::vector<uint32_t> &parent = wsParent;
            parent.resize(bodies.size());
            std::iota(parent.begin(), parent.end(), 0u);
            auto root = [&](uint32_t i) {
                while (parent[i] != i) i = parent[i] = parent[parent[i]];
                return i;
            };
            for (const PManifold &p : pc) {
                if (p.a->body->isStatic || p.b->body->isStatic) continue;
                const uint32_t ra = root(p.m->aIdx), rb = root(p.m->bIdx);
                if (ra != rb) parent[std::max(ra, rb)] = std::min(ra, rb);
            }
            const uint32_t none = 0xFFFFFFFFu;
            std::vector<uint32_t> &lookup = wsLookup, &islandOf = wsIslandOf, &counts = wsCounts, &points = wsPoints;
            lookup.assign(bodies.size(), none);
            islandOf.resize(pc.size());
            counts.clear();
            points.clear();
            for (size_t k = 0; k < pc.size(); ++k) {
                const PManifold &p = pc[k];
                const uint32_t r = root(p.a->body->isStatic ? p.m->bIdx : p.m->aIdx);
                if (lookup[r] == none) {
                    lookup[r] = (uint32_t)counts.size();
                    counts.push_back(0);
                    points.push_back(0);
                }
                islandOf[k] = lookup[r];
                ++counts[lookup[r]];
                points[lookup[r]] += p.m->pointCount;
            }
            islandStart.assign(counts.size() + 1, 0);
            for (size_t i = 0; i < counts.size(); ++i) islandStart[i + 1] = islandStart[i] + counts[i];
            std::vector<uint32_t> &fill = wsFill;
            fill.assign(islandStart.begin(), islandStart.end() - 1);
            islandItems.resize(pc.size());
            for (size_t k = 0; k < pc.size(); ++k) islandItems[fill[islandOf[k]]++] = (uint32_t)k;
            // largest islands first (load balance only)
            islandJobs.resize(counts.size());
            std::iota(islandJobs.begin(), islandJobs.end(), 0u);
            std::stable_sort(islandJobs.begin(), islandJobs.end(),
                             [&](uint32_t x, uint32_t y) { return points[x] > points[y]; });
        }

        // warmStartPrepared (sequential_impulse_solver.cpp:448-490)
        const T matchSq = T(0.05f) * T(0.05f);
        auto warmStartOne = [&](PManifold &p, uint64_t &cmp, uint64_t &matches) {
            Manifold<T> &m = *p.m;
            // the pair's entries (std::equal_range, as the reference searches)
            struct PairOrder {
                bool operator()(const Cached<T> &c, const Manifold<T> &k) const {
                    return cacheLess(c.aIdx, c.aGen, c.bIdx, c.bGen, k.aIdx, k.aGen, k.bIdx, k.bGen);
                }
                bool operator()(const Manifold<T> &k, const Cached<T> &c) const {
                    return cacheLess(k.aIdx, k.aGen, k.bIdx, k.bGen, c.aIdx, c.aGen, c.bIdx, c.bGen);
                }
            };
            const auto range = std::equal_range(cache.begin(), cache.end(), m, PairOrder{});
            const auto lo = range.first, hi = range.second;
            for (uint32_t i = 0; i < m.pointCount; ++i) {
                Point<T> &pt = m.points[i];
                PPoint &pp = p.p[i];
                if (pp.iem <= T(0)) continue;
                for (auto c = lo; c != hi; ++c) {
                    ++cmp;
                    V3<T> da = c->anchorA - pt.anchorA, db = c->anchorB - pt.anchorB;
                    if (dot(da, da) > matchSq || dot(db, db) > matchSq) continue;
                    pt.normalImpulse = smax(c->normalImpulse, T(0));
                    T limit = smax(m.friction, T(0)) * pt.normalImpulse;
                    T tlsq = c->tangentImpulse1 * c->tangentImpulse1 + c->tangentImpulse2 * c->tangentImpulse2;
                    T scale = tlsq > limit * limit ? limit / std::sqrt(tlsq) : T(1);
                    pt.tangentImpulse1 = c->tangentImpulse1 * scale;
                    pt.tangentImpulse2 = c->tangentImpulse2 * scale;
                    V3<T> w = m.normal * pt.normalImpulse + pp.t1 * pt.tangentImpulse1 + pp.t2 * pt.tangentImpulse2;
                    applyCached(*p.a, -w, pp.offA);
                    applyCached(*p.b, w, pp.offB);
                    ++matches;
                    break;
                }
            }
        };
        uint64_t cmp = 0, matches = 0;
        if (parallelIslands) {
            std::vector<uint64_t> icmp(islandJobs.size(), 0), imatch(islandJobs.size(), 0);
            Pool::instance().run(threads, islandJobs.size(), [&](size_t job) {
                const uint32_t isl = islandJobs[job];
                for (uint32_t o = islandStart[isl]; o < islandStart[isl + 1]; ++o)
                    warmStartOne(pc[islandItems[o]], icmp[job], imatch[job]);
            });
            for (size_t j = 0; j < islandJobs.size(); ++j) {
                cmp += icmp[j];
                matches += imatch[j];
            }
        } else {
            for (PManifold &p : pc) warmStartOne(p, cmp, matches);
        }
        ss.warm_start_comparisons = cmp;
        ss.warm_start_matches = matches;
        stageMs[8] = msSince(sclk);

        // solvePrepared (sequential_impulse_solver.cpp:520-603)
        auto solveOne = [&](PManifold &p) {
            Manifold<T> &m = *p.m;
            Body<T> *A = p.a->body, *B = p.b->body;
            for (uint32_t i = 0; i < m.pointCount; ++i) {
                Point<T> &pt = m.points[i];
                PPoint &pp = p.p[i];
                if (pp.iem <= T(0)) continue;
                const V3<T> vA = A->lin + cross(A->ang, pp.offA);
                const V3<T> vB = B->lin + cross(B->ang, pp.offB);
                const V3<T> rel = vB - vA;
                T vn = dot(rel, m.normal);
                T delta = -(vn + pp.rv - pp.bias) / pp.iem;
                T prev = pt.normalImpulse;
                pt.normalImpulse = smax(prev + delta, T(0));
                T applied = pt.normalImpulse - prev;
                V3<T> imp = m.normal * applied;
                applyAxis(*p.a, -imp, pp.nrA, -applied);
                applyAxis(*p.b, imp, pp.nrB, applied);
                if (pp.itm00 <= T(0) || pp.itm11 <= T(0)) continue;
                T limit = smax(m.friction, T(0)) * pt.normalImpulse;
                T tv1 = dot(rel, pp.t1) + pp.ntr1 * applied;
                T tv2 = dot(rel, pp.t2) + pp.ntr2 * applied;
                T d1 = -(pp.itm00 * tv1 + pp.itm01 * tv2);
                T d2 = -(pp.itm01 * tv1 + pp.itm11 * tv2);
                T p1 = pt.tangentImpulse1, p2 = pt.tangentImpulse2;
                pt.tangentImpulse1 += d1;
                pt.tangentImpulse2 += d2;
                T lsq = pt.tangentImpulse1 * pt.tangentImpulse1 + pt.tangentImpulse2 * pt.tangentImpulse2;
                if (lsq > limit * limit) {
                    T s = limit / std::sqrt(lsq);
                    pt.tangentImpulse1 *= s;
                    pt.tangentImpulse2 *= s;
                }
                T a1 = pt.tangentImpulse1 - p1;
                T a2 = pt.tangentImpulse2 - p2;
                V3<T> ti = pp.t1 * a1 + pp.t2 * a2;
                V3<T> rA = pp.trA1 * a1 + pp.trA2 * a2;
                V3<T> rB = pp.trB1 * a1 + pp.trB2 * a2;
                applyTangent(*p.a, -ti, -rA);
                applyTangent(*p.b, ti, rB);
            }
        };
        if (parallelIslands) {
            Pool::instance().run(threads, islandJobs.size(), [&](size_t job) {
                const uint32_t isl = islandJobs[job];
                for (int it = 0; it < iters; ++it)
                    for (uint32_t o = islandStart[isl]; o < islandStart[isl + 1]; ++o) solveOne(pc[islandItems[o]]);
            });
        } else {
            for (int it = 0; it < iters; ++it)
                for (PManifold &p : pc) solveOne(p);
        }
        ss.velocity_point_visits = prepared * (uint64_t)iters;
        stageMs[9] = msSince(sclk);

        // Cache update (sequential_impulse_solver.cpp:623-681): with sleeping
        // on, the entries of sleeping contacts are carried over first.  The
        // next cache's storage is kept between steps, and a cache that comes
        // out already in pair order (manifolds in pair order) needs no sort,
        // as in the reference.
        std::vector<Cached<T>> &next = wsNextCache;
        next.clear();
        if (sleepingEnabled)
            for (const Cached<T> &c : cache) {
                const Body<T> *A = getBody(c.aIdx, c.aGen), *B = getBody(c.bIdx, c.bGen);
                if (A && B && (A->isSleeping() || B->isSleeping()) && (A->isStatic || A->isSleeping()) &&
                    (B->isStatic || B->isSleeping()))
                    next.push_back(c);
            }
        for (const PManifold &p : pc) {
            const Manifold<T> &m = *p.m;
            for (uint32_t i = 0; i < m.pointCount; ++i) {
                const Point<T> &pt = m.points[i];
                next.push_back({m.aIdx, m.aGen, m.bIdx, m.bGen, pt.anchorA, pt.anchorB, pt.normalImpulse,
                                pt.tangentImpulse1, pt.tangentImpulse2});
            }
        }
        auto pairLess = [](const Cached<T> &l, const Cached<T> &r) {
            return cacheLess(l.aIdx, l.aGen, l.bIdx, l.bGen, r.aIdx, r.aGen, r.bIdx, r.bGen);
        };
        if (!std::is_sorted(next.begin(), next.end(), pairLess)) std::stable_sort(next.begin(), next.end(), pairLess);
        cache.swap(next);
        stageMs[10] = msSince(sclk);
    }

    uint32_t colorManifolds(const std::vector<Manifold<T>> &cs, std::vector<uint32_t> &ord,
                            std::vector<uint32_t> &col) {
        const uint32_t M = (uint32_t)cs.size();
        col.assign(M, 0);
        std::vector<uint32_t> byPrio(M);
        std::iota(byPrio.begin(), byPrio.end(), 0u);
        std::sort(byPrio.begin(), byPrio.end(),
                  [](uint32_t a, uint32_t b) { return colorPriority(a) > colorPriority(b); });
        // Per dynamic body, the colours already taken by coloured manifolds.
        std::vector<std::vector<uint32_t>> used(bodies.size());
        // (a sleeping body is not dynamic here: its contacts are not solved)
        auto dynamicBody = [&](uint32_t idx, uint32_t gen) {
            if (idx >= bodies.size()) return false;
            const Body<T> &b = bodies[idx];
            return b.alive && b.generation == gen && !b.isStatic && !(sleepingEnabled && b.sleeping);
        };
        uint32_t ncol = 0;
        for (uint32_t m : byPrio) {
            const Manifold<T> &c = cs[m];
            bool da = dynamicBody(c.aIdx, c.aGen), db = dynamicBody(c.bIdx, c.bGen);
            uint32_t color = 0;
            for (;; ++color) {
                bool taken = false;
                if (da) taken |= std::find(used[c.aIdx].begin(), used[c.aIdx].end(), color) != used[c.aIdx].end();
                if (db) taken |= std::find(used[c.bIdx].begin(), used[c.bIdx].end(), color) != used[c.bIdx].end();
                if (!taken) break;
            }
            col[m] = color;
            if (da) used[c.aIdx].push_back(color);
            if (db) used[c.bIdx].push_back(color);
            ncol = std::max(ncol, color + 1);
        }
        ord.resize(M);
        std::iota(ord.begin(), ord.end(), 0u);
        std::stable_sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) { return col[a] < col[b]; });
        return ncol;
    }

    // PhysicsWorld::step (physics_world.cpp:518-782)
    void step(T dt) {
        auto clk = std::chrono::steady_clock::now();
        const auto start = clk;
        if (sleepingEnabled) prepareSleeping();
        for (uint32_t i = 0; i < bodies.size(); ++i) {
            Body<T> &b = bodies[i];
            if (!b.alive) continue;
            if (sleepingEnabled) sleepStates[i].integratedVelocity = !b.isSleeping();
            integrateVelocity(b, dt);
        }
        for (auto &c : colliders) {
            if (!c.alive) continue;
            Body<T> *b = getBody(c.bodyIndex, c.bodyGeneration);
            if (!b) continue;
            c.bounds = aabbFromCollider(c, Tf<T>{b->pos, b->rot}, hulls);
        }
        stageMs[0] = msSince(clk);
        std::vector<Aabb<T>> &bounds = wsBounds;
        std::vector<uint32_t> &slots = wsSlots;
        std::vector<uint64_t> &perBody = wsPerBody;
        bounds.clear();
        slots.clear();
        perBody.assign(bodies.size(), 0);
        uint64_t possible = 0;
        for (uint32_t i = 0; i < colliders.size(); ++i) {
            const Collider<T> &c = colliders[i];
            if (!c.alive || !getBody(c.bodyIndex, c.bodyGeneration)) continue;
            possible += bounds.size() - perBody[c.bodyIndex];
            ++perBody[c.bodyIndex];
            bounds.push_back(c.bounds);
            slots.push_back(i);
        }
        ow_step_stats bp{};
        if (algo == 1) {
            gridPairs(bounds, cellSize, pairs, bp);
        } else {
            sapPairs(bounds, pairs, bp, threads);
            // DynamicTree: the same sorted pair set (dynamic_aabb_tree.cpp:306-327)
            // and no sweep counters
            if (algo == 2) bp.x_window_comparisons = 0;
        }
        stats = ow_step_stats{};
        stats.x_window_comparisons = bp.x_window_comparisons;
        stats.aabb_pairs = bp.aabb_pairs;
        stats.grid_comparisons = bp.grid_comparisons;
        stats.grid_entries = bp.grid_entries;
        stats.grid_overflow_aabbs = bp.grid_overflow_aabbs;
        stats.grid_cell_size = bp.grid_cell_size;
        for (auto &p : pairs) {
            p.first = slots[p.first];
            p.second = slots[p.second];
        }
        pairs.erase(std::remove_if(pairs.begin(), pairs.end(),
                                   [&](const Pair &p) {
                                       const auto &a = colliders[p.first], &b = colliders[p.second];
                                       return a.bodyIndex == b.bodyIndex && a.bodyGeneration == b.bodyGeneration;
                                   }),
                    pairs.end());
        stats.possible_pairs = possible;
        stats.candidate_pairs = pairs.size();
        stageMs[1] = msSince(clk);

        // Narrowphase driver (physics_world.cpp:645-736); results kept in pair order.
        contacts.clear();
        std::vector<Manifold<T>> &results = wsResults;
        std::vector<int8_t> &hit = wsHit;
        results.resize(pairs.size());
        hit.assign(pairs.size(), -1);
        // pair k's manifold into m; -1: a body is gone, 0: no contact, 1: contact
        auto gen = [&](size_t k, Manifold<T> &m) -> int8_t {
            const Collider<T> &ca = colliders[pairs[k].first], &cb = colliders[pairs[k].second];
            Body<T> *A = getBody(ca.bodyIndex, ca.bodyGeneration), *B = getBody(cb.bodyIndex, cb.bodyGeneration);
            if (!A || !B) return -1;
            Tf<T> tA = colliderWorld(ca, Tf<T>{A->pos, A->rot});
            Tf<T> tB = colliderWorld(cb, Tf<T>{B->pos, B->rot});
            m = Manifold<T>{};
            m.aIdx = ca.bodyIndex;
            m.aGen = ca.bodyGeneration;
            m.bIdx = cb.bodyIndex;
            m.bGen = cb.bodyGeneration;
            if (!generateContact(ca, tA, cb, tB, hulls, m)) return 0;
            for (uint32_t i = 0; i < m.pointCount; ++i) {
                Point<T> &pt = m.points[i];
                pt.anchorA = ca.local.p + rotate(ca.local.q, pt.anchorA);
                pt.anchorB = cb.local.p + rotate(cb.local.q, pt.anchorB);
            }
            m.restitution = smax(A->restitution, B->restitution);
            m.friction = std::sqrt(smax(A->friction, T(0)) * smax(B->friction, T(0)));
            return 1;
        };
        auto category = [&](size_t k) {
            const Collider<T> &ca = colliders[pairs[k].first], &cb = colliders[pairs[k].second];
            return (ca.shape == kHull || cb.shape == kHull) ? 3 : ca.shape + cb.shape;
        };
        if (threads > 1 && pairs.size() >= 4096) {
            Pool::instance().run(threads, (pairs.size() + 63) / 64, [&](size_t chunk) {
                for (size_t k = 64 * chunk, e = std::min(pairs.size(), k + 64); k < e; ++k) hit[k] = gen(k, results[k]);
            });
            for (size_t k = 0; k < pairs.size(); ++k) {
                if (hit[k] < 0) continue;
                const int cat = category(k);
                ++stats.np_candidates[cat];
                if (!hit[k]) continue;
                ++stats.np_contacts[cat];
                contacts.push_back(results[k]);
            }
        } else {
            // one pass in pair order, each manifold built in place
            contacts.reserve(pairs.size());
            for (size_t k = 0; k < pairs.size(); ++k) {
                contacts.emplace_back();
                const int8_t h = gen(k, contacts.back());
                if (h != 1) contacts.pop_back();
                if (h < 0) continue;
                const int cat = category(k);
                ++stats.np_candidates[cat];
                if (h) ++stats.np_contacts[cat];
            }
        }
        stats.contact_count = contacts.size();
        if (sleepingEnabled) {
            // contacts can wake an island after gravity integration (:741-748)
            wakeSleepIslands();
            for (uint32_t i = 0; i < bodies.size(); ++i)
                if (bodies[i].alive && !sleepStates[i].integratedVelocity && !bodies[i].isSleeping())
                    integrateVelocity(bodies[i], dt);
        }

        stageMs[2] = msSince(clk);
        if (orderMode == 1) {
            stats.color_count = colorManifolds(contacts, order, colors);
        } else {
            order.resize(contacts.size());
            std::iota(order.begin(), order.end(), 0u);
            colors.assign(contacts.size(), 0);
            for (uint32_t i = 0; i < colors.size(); ++i) colors[i] = i;
            stats.color_count = contacts.size();
        }
        stageMs[3] = msSince(clk);
        solve(contacts, dt, iterations, order.data());
        stageMs[4] = msSince(clk);

        for (auto &b : bodies) {
            if (!b.alive) continue;
            integratePose(b, dt);
            b.force = {};
        }
        stageMs[5] = msSince(clk);
        if (sleepingEnabled) finishSleeping(dt);
        stats.awake_body_count = stats.sleeping_body_count = 0;
        for (auto &b : bodies)
            if (b.alive && !b.isStatic) ++(b.isSleeping() ? stats.sleeping_body_count : stats.awake_body_count);
        stageMs[6] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - start).count();
    }
};

} // namespace oracle

using namespace oracle;

struct ow_world {
    bool fp64;
    std::unique_ptr<WorldBase> w;
};

template <class F> static auto dispatch(const ow_world *ow, F &&f) {
    if (ow->fp64) return f(*static_cast<World<double> *>(ow->w.get()));
    return f(*static_cast<World<float> *>(ow->w.get()));
}

template <class T> static void toRecord(const Manifold<T> &m, ow_manifold &r) {
    std::memset(&r, 0, sizeof(r));
    r.body_a_index = m.aIdx;
    r.body_a_generation = m.aGen;
    r.body_b_index = m.bIdx;
    r.body_b_generation = m.bGen;
    r.normal[0] = (float)m.normal.x;
    r.normal[1] = (float)m.normal.y;
    r.normal[2] = (float)m.normal.z;
    r.point_count = m.pointCount;
    r.friction = (float)m.friction;
    r.restitution = (float)m.restitution;
    for (int i = 0; i < 4; ++i) {
        const Point<T> &p = m.points[i];
        r.anchor_a[i][0] = (float)p.anchorA.x;
        r.anchor_a[i][1] = (float)p.anchorA.y;
        r.anchor_a[i][2] = (float)p.anchorA.z;
        r.anchor_b[i][0] = (float)p.anchorB.x;
        r.anchor_b[i][1] = (float)p.anchorB.y;
        r.anchor_b[i][2] = (float)p.anchorB.z;
        r.penetration[i] = (float)p.penetration;
        r.normal_impulse[i] = (float)p.normalImpulse;
        r.tangent_impulse1[i] = (float)p.tangentImpulse1;
        r.tangent_impulse2[i] = (float)p.tangentImpulse2;
        r.feature[i] = p.feature;
    }
}
template <class T> static Manifold<T> fromRecord(const ow_manifold &r) {
    Manifold<T> m;
    m.aIdx = r.body_a_index;
    m.aGen = r.body_a_generation;
    m.bIdx = r.body_b_index;
    m.bGen = r.body_b_generation;
    m.normal = {T(r.normal[0]), T(r.normal[1]), T(r.normal[2])};
    m.pointCount = r.point_count;
    m.friction = T(r.friction);
    m.restitution = T(r.restitution);
    for (int i = 0; i < 4; ++i) {
        Point<T> &p = m.points[i];
        p.anchorA = {T(r.anchor_a[i][0]), T(r.anchor_a[i][1]), T(r.anchor_a[i][2])};
        p.anchorB = {T(r.anchor_b[i][0]), T(r.anchor_b[i][1]), T(r.anchor_b[i][2])};
        p.penetration = T(r.penetration[i]);
        p.normalImpulse = T(r.normal_impulse[i]);
        p.tangentImpulse1 = T(r.tangent_impulse1[i]);
        p.tangentImpulse2 = T(r.tangent_impulse2[i]);
        p.feature = r.feature[i];
    }
    return m;
}

template <class O, class W> static void getBodiesT(W &w, O *pos, O *quat, O *lin, O *ang) {
    for (size_t i = 0; i < w.bodies.size(); ++i) {
        const auto &b = w.bodies[i];
        if (pos) { pos[3 * i] = (O)b.pos.x; pos[3 * i + 1] = (O)b.pos.y; pos[3 * i + 2] = (O)b.pos.z; }
        if (quat) {
            quat[4 * i] = (O)b.rot.x; quat[4 * i + 1] = (O)b.rot.y;
            quat[4 * i + 2] = (O)b.rot.z; quat[4 * i + 3] = (O)b.rot.w;
        }
        if (lin) { lin[3 * i] = (O)b.lin.x; lin[3 * i + 1] = (O)b.lin.y; lin[3 * i + 2] = (O)b.lin.z; }
        if (ang) { ang[3 * i] = (O)b.ang.x; ang[3 * i + 1] = (O)b.ang.y; ang[3 * i + 2] = (O)b.ang.z; }
    }
}
extern "C" {

ow_world *ow_create(int fp64) {
    auto *ow = new ow_world;
    ow->fp64 = fp64 != 0;
    if (ow->fp64)
        ow->w.reset(new World<double>());
    else
        ow->w.reset(new World<float>());
    return ow;
}
ow_world *ow_clone(const ow_world *world) {
    auto *ow = new ow_world;
    ow->fp64 = world->fp64;
    ow->w.reset(world->w->clone());
    return ow;
}
void ow_destroy(ow_world *world) { delete world; }
void ow_set_gravity(ow_world *world, double gx, double gy, double gz) {
    // The float instance rounds the request to float like the reference's Vec3.
    dispatch(world, [&](auto &w) {
        using T = decltype(w.gravity.x);
        if (world->fp64)
            w.gravity = {T(gx), T(gy), T(gz)};
        else
            w.gravity = {T((float)gx), T((float)gy), T((float)gz)};
    });
}
void ow_set_broadphase(ow_world *world, int algo, double cell) {
    dispatch(world, [&](auto &w) { w.algo = algo; w.cellSize = cell; });
}
void ow_set_solver(ow_world *world, int iterations, int order_mode) {
    dispatch(world, [&](auto &w) { w.iterations = iterations; w.orderMode = order_mode; });
}
void ow_set_threads(ow_world *world, int threads) {
    dispatch(world, [&](auto &w) { w.threads = threads < 1 ? 1 : threads; });
}

// RigidBody::createSphere / createBox (rigid_body.cpp:25-91) and
// PhysicsWorld::createSphere / createBox (physics_world.cpp:181-221).
int ow_create_body(ow_world *world, int shape, const float *dims, const float *pos, float density,
                   int is_static, float restitution, float friction, uint32_t *handles, char *err,
                   int err_len) {
    auto fail = [&](const char *msg) {
        if (err && err_len > 0) {
            std::strncpy(err, msg, (size_t)err_len - 1);
            err[err_len - 1] = 0;
        }
        return 1;
    };
    const float pi = 3.14159265358979323846f;
    const float minSize = 0.01f * 0.01f, maxSize = 64.0f * 64.0f;
    float volume;
    if (shape == kSphere) {
        float r = dims[0];
        volume = (4.0f / 3.0f) * pi * r * r * r;
        if (volume < minSize) return fail("Sphere is too small");
        if (volume > maxSize) return fail("Sphere is too large");
    } else {
        if (dims[0] <= 0.0f || dims[1] <= 0.0f || dims[2] <= 0.0f) return fail("Box dimensions must be positive");
        volume = dims[0] * dims[1] * dims[2];
        if (volume < minSize) return fail("Box is too small");
        if (volume > maxSize) return fail("Box is too large");
    }
    if (!(density >= 0.2f && density <= 21.4f)) return fail("Density is out of range");
    float rest = restitution;
    if (rest < 0.0f) rest = 0.0f;
    if (rest > 1.0f) rest = 1.0f;
    float fr = friction < 0.0f ? 0.0f : friction;
    const float mass = volume * density;
    M3<float> iil{};
    if (!is_static) {
        if (shape == kSphere) {
            float r = dims[0];
            if (mass > 0.0f && r > 0.0f) {
                float ii = 1.0f / (0.4f * mass * r * r);
                iil = {ii, 0, 0, 0, ii, 0, 0, 0, ii};
            }
        } else {
            float w = dims[0], h = dims[1], d = dims[2];
            if (mass > 0.0f) {
                float factor = 12.0f / mass;
                iil = {factor / (h * h + d * d), 0, 0, 0, factor / (w * w + d * d), 0, 0, 0, factor / (w * w + h * h)};
            }
        }
    }
    dispatch(world, [&](auto &w) {
        using T = decltype(w.gravity.x);
        Body<T> b;
        b.mass = T(mass);
        b.restitution = T(rest);
        b.friction = T(fr);
        b.isStatic = is_static != 0;
        b.pos = {T(pos[0]), T(pos[1]), T(pos[2])};
        b.rot = {T(0), T(0), T(0), T(1)};
        b.invInertiaLocal = {T(iil.m00), T(iil.m01), T(iil.m02), T(iil.m10), T(iil.m11),
                             T(iil.m12), T(iil.m20), T(iil.m21), T(iil.m22)};
        uint32_t bg, cg;
        uint32_t bi = w.addBody(b, bg);
        Collider<T> c;
        c.bodyIndex = bi;
        c.bodyGeneration = bg;
        c.shape = shape;
        if (shape == kSphere)
            c.radius = T(dims[0]);
        else
            c.halfExtents = {T(dims[0] * 0.5f), T(dims[1] * 0.5f), T(dims[2] * 0.5f)};
        uint32_t ci = w.addCollider(c, cg);
        handles[0] = bi;
        handles[1] = bg;
        handles[2] = ci;
        handles[3] = cg;
    });
    return 0;
}

// PhysicsWorld::addCollider (physics_world.cpp:276-298) with a local transform.
int ow_add_collider(ow_world *world, uint32_t body_index, uint32_t body_generation, int shape, const float *dims,
                    const float *local_pos, const float *local_rot, uint32_t *handle) {
    return dispatch(world, [&](auto &w) {
        using T = decltype(w.gravity.x);
        if (!w.getBody(body_index, body_generation)) {
            handle[0] = handle[1] = 0;
            return 1;
        }
        Collider<T> c;
        c.bodyIndex = body_index;
        c.bodyGeneration = body_generation;
        c.shape = shape;
        if (shape == kSphere)
            c.radius = T(dims[0]);
        else
            c.halfExtents = {T(dims[0]), T(dims[1]), T(dims[2])};
        c.local.p = {T(local_pos[0]), T(local_pos[1]), T(local_pos[2])};
        c.local.q = {T(local_rot[0]), T(local_rot[1]), T(local_rot[2]), T(local_rot[3])};
        uint32_t g;
        handle[0] = w.addCollider(c, g);
        handle[1] = g;
        return 0;
    });
}

int ow_add_hull_shape(ow_world *world, uint32_t n, const float *v) {
    return dispatch(world, [&](auto &w) {
        using T = decltype(w.gravity.x);
        HullShape<T> h;
        for (uint32_t i = 0; i < n; ++i) h.vertices.push_back({T(v[3 * i]), T(v[3 * i + 1]), T(v[3 * i + 2])});
        w.hulls.push_back(h);
        return (int)w.hulls.size() - 1;
    });
}

int ow_create_hull_body(ow_world *world, int hull_id, const float *pos, float mass, const float *iid,
                        int is_static, float restitution, float friction, uint32_t *handles) {
    dispatch(world, [&](auto &w) {
        using T = decltype(w.gravity.x);
        Body<T> b;
        b.mass = T(mass);
        b.restitution = T(restitution);
        b.friction = T(friction);
        b.isStatic = is_static != 0;
        b.pos = {T(pos[0]), T(pos[1]), T(pos[2])};
        if (!is_static) b.invInertiaLocal = {T(iid[0]), T(0), T(0), T(0), T(iid[1]), T(0), T(0), T(0), T(iid[2])};
        uint32_t bg, cg;
        uint32_t bi = w.addBody(b, bg);
        Collider<T> c;
        c.bodyIndex = bi;
        c.bodyGeneration = bg;
        c.shape = kHull;
        c.hull = hull_id;
        uint32_t ci = w.addCollider(c, cg);
        handles[0] = bi;
        handles[1] = bg;
        handles[2] = ci;
        handles[3] = cg;
    });
    return 0;
}

void ow_remove_body(ow_world *world, uint32_t index, uint32_t generation) {
    dispatch(world, [&](auto &w) { w.removeBody(index, generation); });
}
void ow_remove_collider(ow_world *world, uint32_t index, uint32_t generation) {
    dispatch(world, [&](auto &w) { w.removeCollider(index, generation); });
}
void ow_set_sleeping_enabled(ow_world *world, int enabled) {
    dispatch(world, [&](auto &w) { w.setSleepingEnabled(enabled != 0); });
}
void ow_get_sleeping(const ow_world *world, uint8_t *sleeping) {
    dispatch(world, [&](auto &w) {
        for (size_t i = 0; i < w.bodies.size(); ++i) sleeping[i] = w.bodies[i].isSleeping() ? 1 : 0;
    });
}
void ow_wake_body(ow_world *world, uint32_t i) {
    dispatch(world, [&](auto &w) { w.bodies[i].wakeUp(); });
}
// RigidBody::applyForce (rigid_body.hpp:77-85)
void ow_apply_force(ow_world *world, uint32_t i, const float *f) {
    dispatch(world, [&](auto &w) {
        using T = decltype(w.gravity.x);
        auto &b = w.bodies[i];
        if (b.isStatic) return;
        if (f[0] != 0.0f || f[1] != 0.0f || f[2] != 0.0f) b.wakeUp();
        b.force += V3<T>{T(f[0]), T(f[1]), T(f[2])};
    });
}
uint32_t ow_body_slot_count(const ow_world *world) {
    return dispatch(world, [&](auto &w) { return (uint32_t)w.bodies.size(); });
}

void ow_get_bodies(const ow_world *world, float *pos, float *quat, float *lin, float *ang) {
    dispatch(world, [&](auto &w) { getBodiesT(w, pos, quat, lin, ang); });
}
void ow_get_bodies_f64(const ow_world *world, double *pos, double *quat, double *lin, double *ang) {
    dispatch(world, [&](auto &w) { getBodiesT(w, pos, quat, lin, ang); });
}
// setLinearVelocity / setAngularVelocity wake the body (rigid_body.hpp:59-63, :91-95)
void ow_set_velocity(ow_world *world, uint32_t i, const float *lin, const float *ang) {
    dispatch(world, [&](auto &w) {
        using T = decltype(w.gravity.x);
        if (lin || ang) w.bodies[i].wakeUp();
        if (lin) w.bodies[i].lin = {T(lin[0]), T(lin[1]), T(lin[2])};
        if (ang) w.bodies[i].ang = {T(ang[0]), T(ang[1]), T(ang[2])};
    });
}
void ow_set_velocity_f64(ow_world *world, uint32_t i, const double *lin, const double *ang) {
    dispatch(world, [&](auto &w) {
        using T = decltype(w.gravity.x);
        if (lin || ang) w.bodies[i].wakeUp();
        if (lin) w.bodies[i].lin = {T(lin[0]), T(lin[1]), T(lin[2])};
        if (ang) w.bodies[i].ang = {T(ang[0]), T(ang[1]), T(ang[2])};
    });
}
void ow_set_position_f64(ow_world *world, uint32_t i, const double *pos) {
    dispatch(world, [&](auto &w) {
        using T = decltype(w.gravity.x);
        w.bodies[i].pos = {T(pos[0]), T(pos[1]), T(pos[2])};
    });
}
// RigidBody::setAngularVelocity + integrateRotation(1) + setAngularVelocity(0)
// (rigid_body.hpp:95-99, rigid_body.cpp:110-125); integrateRotation returns early
// for static bodies (rigid_body.cpp:112-113), so their orientation stays identity.
void ow_apply_spin(ow_world *world, uint32_t i, const float *spin) {
    dispatch(world, [&](auto &w) {
        using T = decltype(w.gravity.x);
        auto &b = w.bodies[i];
        b.wakeUp();
        if (b.isStatic) return;
        b.ang = {T(spin[0]), T(spin[1]), T(spin[2])};
        Q<T> s{b.ang.x, b.ang.y, b.ang.z, T(0)};
        Q<T> d = qmul(s, b.rot);
        T h = T(0.5f) * T(1);
        b.rot.x += h * d.x;
        b.rot.y += h * d.y;
        b.rot.z += h * d.z;
        b.rot.w += h * d.w;
        b.rot = qnormalized(b.rot);
        b.ang = {T(0), T(0), T(0)};
    });
}
void ow_set_material(ow_world *world, uint32_t i, double mass, double friction, double restitution) {
    dispatch(world, [&](auto &w) {
        using T = decltype(w.gravity.x);
        auto &b = w.bodies[i];
        b.mass = world->fp64 ? T(mass) : T((float)mass);
        b.friction = world->fp64 ? T(friction) : T((float)friction);
        b.restitution = world->fp64 ? T(restitution) : T((float)restitution);
    });
}
void ow_get_material(const ow_world *world, uint32_t i, double *mass, double *friction, double *restitution) {
    dispatch(world, [&](auto &w) {
        const auto &b = w.bodies[i];
        *mass = (double)b.mass;
        *friction = (double)b.friction;
        *restitution = (double)b.restitution;
    });
}

int ow_step(ow_world *world, float dt) {
    dispatch(world, [&](auto &w) {
        using T = decltype(w.gravity.x);
        w.step(T(dt));
    });
    return 0;
}
void ow_get_stage_ms(const ow_world *world, double *ms) {
    for (int i = 0; i < 11; ++i) ms[i] = world->w->stageMs[i];
}

void ow_get_stats(const ow_world *world, ow_step_stats *s) {
    dispatch(world, [&](auto &w) { *s = w.stats; });
}
uint32_t ow_pair_count(const ow_world *world) {
    return dispatch(world, [&](auto &w) { return (uint32_t)w.pairs.size(); });
}
void ow_get_pairs(const ow_world *world, uint32_t *pairs) {
    dispatch(world, [&](auto &w) {
        for (size_t i = 0; i < w.pairs.size(); ++i) {
            pairs[2 * i] = w.pairs[i].first;
            pairs[2 * i + 1] = w.pairs[i].second;
        }
    });
}
uint32_t ow_contact_count(const ow_world *world) {
    return dispatch(world, [&](auto &w) { return (uint32_t)w.contacts.size(); });
}
void ow_get_contacts(const ow_world *world, ow_manifold *out) {
    dispatch(world, [&](auto &w) {
        for (size_t i = 0; i < w.contacts.size(); ++i) toRecord(w.contacts[i], out[i]);
    });
}
void ow_get_solve_order(const ow_world *world, uint32_t *order, uint32_t *colors) {
    dispatch(world, [&](auto &w) {
        for (size_t i = 0; i < w.order.size(); ++i) {
            if (order) order[i] = w.order[i];
            if (colors) colors[i] = w.colors[i];
        }
    });
}

uint64_t ow_broadphase(const float *mins, const float *maxs, uint32_t n, int algo, double cell, uint32_t *pairs,
                       uint64_t capacity, ow_step_stats *stats) {
    std::vector<Aabb<float>> bounds(n);
    for (uint32_t i = 0; i < n; ++i) {
        bounds[i].min = {mins[3 * i], mins[3 * i + 1], mins[3 * i + 2]};
        bounds[i].max = {maxs[3 * i], maxs[3 * i + 1], maxs[3 * i + 2]};
    }
    std::vector<Pair> out;
    ow_step_stats st{};
    if (algo == 1)
        gridPairs(bounds, cell, out, st);
    else
        sapPairs(bounds, out, st, 1);
    if (stats) *stats = st;
    if (pairs && out.size() <= capacity)
        for (size_t i = 0; i < out.size(); ++i) {
            pairs[2 * i] = out[i].first;
            pairs[2 * i + 1] = out[i].second;
        }
    return out.size();
}

int ow_generate_contact(int sa, const float *da, const float *pa, const float *qa, int sb, const float *db,
                        const float *pb, const float *qb, ow_manifold *out) {
    Collider<float> a, b;
    a.shape = sa;
    b.shape = sb;
    if (sa == kSphere) a.radius = da[0]; else a.halfExtents = {da[0], da[1], da[2]};
    if (sb == kSphere) b.radius = db[0]; else b.halfExtents = {db[0], db[1], db[2]};
    Tf<float> tA{{pa[0], pa[1], pa[2]}, {qa[0], qa[1], qa[2], qa[3]}};
    Tf<float> tB{{pb[0], pb[1], pb[2]}, {qb[0], qb[1], qb[2], qb[3]}};
    Manifold<float> m{};
    std::vector<HullShape<float>> none;
    bool hit = generateContact(a, tA, b, tB, none, m);
    toRecord(m, *out);
    return hit ? 1 : 0;
}

void ow_solve(ow_world *world, ow_manifold *contacts, uint32_t count, float dt, int iterations,
              const uint32_t *order, ow_step_stats *stats) {
    dispatch(world, [&](auto &w) {
        using T = decltype(w.gravity.x);
        std::vector<Manifold<T>> cs;
        for (uint32_t i = 0; i < count; ++i) cs.push_back(fromRecord<T>(contacts[i]));
        w.solve(cs, T(dt), iterations, order);
        for (uint32_t i = 0; i < count; ++i) toRecord(cs[i], contacts[i]);
        if (stats) *stats = w.stats;
    });
}

uint32_t ow_color_manifolds(const ow_world *world, const ow_manifold *contacts, uint32_t count, uint32_t *order,
                            uint32_t *colors) {
    return dispatch(world, [&](auto &w) {
        using T = decltype(w.gravity.x);
        std::vector<Manifold<T>> cs;
        for (uint32_t i = 0; i < count; ++i) cs.push_back(fromRecord<T>(contacts[i]));
        std::vector<uint32_t> ord, col;
        uint32_t n = w.colorManifolds(cs, ord, col);
        for (uint32_t i = 0; i < count; ++i) {
            order[i] = ord[i];
            colors[i] = col[i];
        }
        return n;
    });
}

int ow_gjk_epa(const float *points_a, uint32_t count_a, const float *points_b, uint32_t count_b, float *normal,
               float *depth, uint32_t *simplex_size) {
    std::vector<V3<float>> A(count_a), B(count_b);
    for (uint32_t i = 0; i < count_a; ++i) A[i] = {points_a[3 * i], points_a[3 * i + 1], points_a[3 * i + 2]};
    for (uint32_t i = 0; i < count_b; ++i) B[i] = {points_b[3 * i], points_b[3 * i + 1], points_b[3 * i + 2]};
    Tf<float> id{{0, 0, 0}, {0, 0, 0, 1}};
    Support<float> sa{kHull, 0.f, {}, A.data(), count_a, id};
    Support<float> sb{kHull, 0.f, {}, B.data(), count_b, id};
    Simplex<float> s;
    bool hit = gjk<float>(sa, sb, s);
    if (simplex_size) *simplex_size = s.size;
    if (!hit) return -1;
    V3<float> n;
    float d;
    int ok = epa<float>(sa, sb, s, n, d);
    if (normal) { normal[0] = n.x; normal[1] = n.y; normal[2] = n.z; }
    if (depth) *depth = d;
    return ok;
}

} // extern "C"

// Host side of the batched worlds: device layout (per-world slices of shared
// arrays), size buckets, the per-step CUDA graph (one persistent launch per
// bucket on forked streams), capacity growth with step re-run, the autotuner,
// and read-back.
#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <string>

#include "batch.h"

namespace pe {
namespace {

template <class T> void uploadVec(DeviceArray<T> &d, const std::vector<T> &h, cudaStream_t s) {
    d.reserve(h.size());
    if (!h.empty()) PE_CHECK(cudaMemcpyAsync(d.ptr, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

uint32_t pow2ceil(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    if (p > 0x80000000ull) throw std::runtime_error("batch buffer size beyond 2^31 entries");
    return (uint32_t)p;
}

// Moves each world's live warm-start entries from an old layout to a new one.
__global__ void k_cache_relayout(const WorldDesc *oldD, const WorldDesc *newD, const uint32_t *counts, uint32_t W,
                                 CacheView from, CacheView to) {
    for (uint32_t w = blockIdx.x; w < W; w += gridDim.x) {
        const uint32_t n = min(counts[w], newD[w].cacheCap);
        const uint32_t a = oldD[w].cacheBase, b = newD[w].cacheBase;
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            to.key[b + i] = from.key[a + i];
            to.gens[b + i] = from.gens[a + i];
            to.anchorA[b + i] = from.anchorA[a + i];
            to.anchorB[b + i] = from.anchorB[a + i];
            to.tangent2[b + i] = from.tangent2[a + i];
        }
    }
}

constexpr uint32_t kBucketEdges[] = {64, 256, 1024, 0xFFFFFFFFu};
constexpr uint32_t kBatchMaxWorldBodies = 8192;

} // namespace

Batch::Batch(int device) : device_(device) {
    PE_CHECK(cudaSetDevice(device_));
    PE_CHECK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    for (int i = 0; i < 3; ++i) {
        cudaStream_t s;
        cudaEvent_t e;
        PE_CHECK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        PE_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        side_.push_back(s);
        joins_.push_back(e);
    }
    PE_CHECK(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
    PE_CHECK(cudaEventCreate(&t0_));
    PE_CHECK(cudaEventCreate(&t1_));
    PE_CHECK(cudaMallocHost(&hostErr_, sizeof(uint32_t)));
    *hostErr_ = 0;
    batchErr_.reserve(1);
}

Batch::~Batch() {
    if (stream_) cudaStreamSynchronize(stream_);
    dropGraphs();
    if (hostErr_) cudaFreeHost(hostErr_);
    for (auto s : side_) cudaStreamDestroy(s);
    for (auto e : joins_) cudaEventDestroy(e);
    if (fork_) cudaEventDestroy(fork_);
    if (t0_) cudaEventDestroy(t0_);
    if (t1_) cudaEventDestroy(t1_);
    if (stream_) cudaStreamDestroy(stream_);
}

void Batch::dropGraphs() {
    for (auto &row : graph_)
        for (auto &g : row) {
            if (g) cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

void Batch::create(const std::vector<uint32_t> &worldBodies, const std::vector<HostBody> &bodies,
                   const std::vector<HostCollider> &colliders) {
    PE_CHECK(cudaSetDevice(device_));
    uint64_t total = 0;
    for (uint32_t n : worldBodies) {
        if (n == 0) throw std::invalid_argument("every batched world needs at least one body");
        if (n > kBatchMaxWorldBodies)
            throw std::invalid_argument("a batched world holds at most " + std::to_string(kBatchMaxWorldBodies) +
                                        " bodies");
        total += n;
    }
    if (worldBodies.empty()) throw std::invalid_argument("a batch needs at least one world");
    if (total != bodies.size() || total != colliders.size())
        throw std::invalid_argument("body and collider arrays must hold the sum of the world body counts");
    if (total >= (1ull << 31)) throw std::invalid_argument("too many bodies for one batch");
    dropGraphs();
    worldBodies_ = worldBodies;
    nb_ = total;
    const uint32_t W = (uint32_t)worldBodies.size();
    desc_.assign(W, WorldDesc{});
    uint32_t start = 0;
    for (uint32_t w = 0; w < W; ++w) {
        desc_[w].bodyStart = start;
        desc_[w].bodyCount = worldBodies[w];
        start += worldBodies[w];
    }
    std::vector<float4> p(nb_), q(nb_), l(nb_), a(nb_), mat(nb_), ii(nb_), cs(nb_);
    std::vector<uint32_t> flags(nb_), gen(nb_), cb(nb_), cg(nb_), cf(nb_);
    for (uint64_t i = 0; i < nb_; ++i) {
        const HostBody &b = bodies[i];
        const HostCollider &c = colliders[i];
        const uint32_t w = (uint32_t)(std::upper_bound(desc_.begin(), desc_.end(), (uint32_t)i,
                                                       [](uint32_t v, const WorldDesc &d) { return v < d.bodyStart; }) -
                                      desc_.begin() - 1);
        if (c.body != i - desc_[w].bodyStart)
            throw std::invalid_argument("batched worlds need collider i on body i of the same world");
        if (c.shape != kShapeSphere && c.shape != kShapeBox)
            throw std::invalid_argument("batched worlds hold sphere and box colliders");
        p[i] = make_float4(b.pos[0], b.pos[1], b.pos[2], 0.0f);
        q[i] = make_float4(b.rot[0], b.rot[1], b.rot[2], b.rot[3]);
        l[i] = make_float4(b.lin[0], b.lin[1], b.lin[2], 0.0f);
        a[i] = make_float4(b.ang[0], b.ang[1], b.ang[2], 0.0f);
        // RigidBody::getInverseMass (rigid_body.hpp:72-75)
        const float invMass = b.isStatic || b.mass <= 0.0f ? 0.0f : 1.0f / b.mass;
        mat[i] = make_float4(invMass, b.restitution, b.friction, b.mass);
        ii[i] = make_float4(b.iinv[0], b.iinv[1], b.iinv[2], 0.0f);
        flags[i] = kBodyAlive | (b.isStatic ? kBodyStatic : 0u);
        gen[i] = 0;
        cb[i] = c.body;
        cg[i] = 0;
        cf[i] = kColliderAlive | (c.shape << 8);
        cs[i] = make_float4(c.dims[0], c.dims[1], c.dims[2], 0.0f);
    }
    parity_ = 0;
    steps_ = 0;
    uploadVec(pos_[0], p, stream_);
    uploadVec(rot_[0], q, stream_);
    uploadVec(lin_[0], l, stream_);
    uploadVec(ang_[0], a, stream_);
    pos_[1].reserve(nb_);
    rot_[1].reserve(nb_);
    lin_[1].reserve(nb_);
    ang_[1].reserve(nb_);
    uploadVec(mat_, mat, stream_);
    uploadVec(iinv_, ii, stream_);
    uploadVec(bflags_, flags, stream_);
    uploadVec(bgen_, gen, stream_);
    uploadVec(cbody_, cb, stream_);
    uploadVec(cbgen_, cg, stream_);
    uploadVec(cflags_, cf, stream_);
    uploadVec(cshape_, cs, stream_);
    force_.reserve(nb_);
    forces_ = false;
    aabbMin_.reserve(nb_);
    aabbMax_.reserve(nb_);
    bodyBest_.reserve(nb_);
    bodyUsed_.reserve(2 * nb_);
    epoch_.reserve(W);
    colorCount_.reserve((size_t)W * kMaxColors);
    stats_.reserve(W);
    cacheCount_.reserve(2ull * W);
    PE_CHECK(cudaMemsetAsync(cacheCount_.ptr, 0, 2ull * W * sizeof(uint32_t), stream_));
    std::vector<uint32_t> pairCap(W), mCap(W);
    for (uint32_t w = 0; w < W; ++w) {
        const uint32_t n = worldBodies[w];
        pairCap[w] = pow2ceil(std::max<uint64_t>(64, 4ull * n));
        mCap[w] = std::min<uint32_t>(kBlockMaxManifolds, pow2ceil(std::max<uint64_t>(32, 2ull * n)));
    }
    layout(pairCap, mCap, false);
    makeBuckets();
    PE_CHECK(cudaStreamSynchronize(stream_));
}

void Batch::layout(const std::vector<uint32_t> &pairCap, const std::vector<uint32_t> &mCap, bool keepCaches) {
    const uint32_t W = (uint32_t)desc_.size();
    std::vector<WorldDesc> nd = desc_;
    uint64_t pb = 0, mb = 0, cb = 0;
    for (uint32_t w = 0; w < W; ++w) {
        nd[w].pairBase = (uint32_t)pb;
        nd[w].pairCap = pairCap[w];
        nd[w].mBase = (uint32_t)mb;
        nd[w].mCap = mCap[w];
        nd[w].cacheBase = (uint32_t)cb;
        nd[w].cacheCap = 4 * mCap[w];
        pb += pairCap[w];
        mb += mCap[w];
        cb += 4ull * mCap[w];
    }
    if (pb >= (1ull << 32) || 40 * mb >= (1ull << 40) || cb >= (1ull << 32))
        throw std::runtime_error("batch buffers beyond 32-bit offsets");
    pairTotal_ = pb;
    mTotal_ = mb;
    cacheTotal_ = cb;
    pairKeys_.reserve(pb);
    mBodyA_.reserve(mb);
    mGenA_.reserve(mb);
    mBodyB_.reserve(mb);
    mGenB_.reserve(mb);
    mCount_.reserve(mb);
    mRest_.reserve(mb);
    mNormal_.reserve(mb);
    mFeature_.reserve(4 * mb);
    mAnchorA_.reserve(4 * mb);
    mAnchorB_.reserve(4 * mb);
    mImpulse_.reserve(4 * mb);
    color_.reserve(mb);
    dyn_.reserve(mb);
    order_.reserve(mb);
    colorStart_.reserve(mb);
    pm_.reserve(mb);
    pmInertia_.reserve(6 * mb);
    pp_.reserve((size_t)kPreparedVec4 * 4 * mb);
    pimp_.reserve(4 * mb);
    pn_.reserve(mb);
    pbody_.reserve(mb);
    pcount_.reserve(mb);
    if (keepCaches) {
        // Move the current parity's cache into freshly sized arrays.
        DeviceArray<unsigned long long> key, gens;
        DeviceArray<float4> ca, cbv;
        DeviceArray<float> t2;
        key.reserve(cb);
        gens.reserve(cb);
        ca.reserve(cb);
        cbv.reserve(cb);
        t2.reserve(cb);
        DeviceArray<WorldDesc> newDesc;
        uploadVec(newDesc, nd, stream_);
        const int c = (int)parity_;
        k_cache_relayout<<<std::min<uint32_t>(W, 1024), 128, 0, stream_>>>(
            descDev_.ptr, newDesc.ptr, cacheCount_.ptr + (size_t)parity_ * W, W,
            CacheView{cacheKey_[c].ptr, cacheGens_[c].ptr, cacheA_[c].ptr, cacheB_[c].ptr, cacheT2_[c].ptr},
            CacheView{key.ptr, gens.ptr, ca.ptr, cbv.ptr, t2.ptr});
        PE_LAUNCHED();
        PE_CHECK(cudaStreamSynchronize(stream_));
        cacheKey_[c].swap(key);
        cacheGens_[c].swap(gens);
        cacheA_[c].swap(ca);
        cacheB_[c].swap(cbv);
        cacheT2_[c].swap(t2);
        const int o = 1 - c;
        cacheKey_[o].reserve(cb);
        cacheGens_[o].reserve(cb);
        cacheA_[o].reserve(cb);
        cacheB_[o].reserve(cb);
        cacheT2_[o].reserve(cb);
    } else {
        for (int c = 0; c < 2; ++c) {
            cacheKey_[c].reserve(cb);
            cacheGens_[c].reserve(cb);
            cacheA_[c].reserve(cb);
            cacheB_[c].reserve(cb);
            cacheT2_[c].reserve(cb);
        }
    }
    desc_ = nd;
    uploadVec(descDev_, desc_, stream_);
    PE_CHECK(cudaStreamSynchronize(stream_));
    deviceBytes_ = nb_ * (8 * 16 + 7 * 16 + 5 * 4 + 3 * 8) + pb * 8 + mb * (6 * 4 + 16 + 4 * (4 + 3 * 16)) +
                   mb * (3 * 4 + 16 + 6 * 16 + 40 * 16 + 4 * 16 + 16 + 8 + 4) + cb * 2 * (8 + 8 + 16 + 16 + 4);
}

void Batch::makeBuckets() {
    std::vector<BatchBucket> old = buckets_;
    buckets_.clear();
    uint32_t lo = 1;
    for (uint32_t hi : kBucketEdges) {
        BatchBucket b;
        b.lo = lo;
        b.hi = hi;
        for (uint32_t w = 0; w < desc_.size(); ++w)
            if (desc_[w].bodyCount >= lo && desc_[w].bodyCount <= hi) b.worlds.push_back(w);
        lo = hi + 1;
        if (b.worlds.empty()) continue;
        std::stable_sort(b.worlds.begin(), b.worlds.end(),
                         [&](uint32_t x, uint32_t y) { return desc_[x].bodyCount > desc_[y].bodyCount; });
        for (uint32_t w : b.worlds) {
            b.maxN = std::max(b.maxN, desc_[w].bodyCount);
            b.maxM = std::max(b.maxM, desc_[w].mCap);
        }
        b.maxM = pow2ceil(b.maxM);
        for (const BatchBucket &o : old)
            if (o.lo == b.lo) {
                b.variant = o.variant;
                b.tunedMs = o.tunedMs;
                b.candidateMs = o.candidateMs;
            }
        buckets_.push_back(b);
    }
    std::vector<uint32_t> q;
    for (BatchBucket &b : buckets_) {
        b.queueOff = (uint32_t)q.size();
        q.insert(q.end(), b.worlds.begin(), b.worlds.end());
        const size_t smem = batchSharedBytes(b.maxN, b.maxM);
        b.blocks = std::min<uint32_t>((uint32_t)b.worlds.size(), batchMaxBlocks(b.variant, smem));
    }
    uploadVec(queue_, q, stream_);
    queueHead_.reserve(buckets_.size());
    PE_CHECK(cudaStreamSynchronize(stream_));
}

BatchView Batch::view(const BatchBucket &bk, float dt, uint32_t parity) const {
    BatchView v{};
    for (int c = 0; c < 2; ++c) v.state[c] = BodyState{pos_[c].ptr, rot_[c].ptr, lin_[c].ptr, ang_[c].ptr};
    v.force = forces_ ? force_.ptr : nullptr;
    v.mat = mat_.ptr;
    v.iinv = iinv_.ptr;
    v.bflags = bflags_.ptr;
    v.bgen = bgen_.ptr;
    v.cbody = cbody_.ptr;
    v.cbgen = cbgen_.ptr;
    v.cflags = cflags_.ptr;
    v.cshape = cshape_.ptr;
    v.aabbMin = aabbMin_.ptr;
    v.aabbMax = aabbMax_.ptr;
    v.pairKeys = pairKeys_.ptr;
    v.mv = ManifoldView{mBodyA_.ptr, mGenA_.ptr,     mBodyB_.ptr,   mGenB_.ptr,    mNormal_.ptr, mRest_.ptr,
                        mCount_.ptr, mAnchorA_.ptr, mAnchorB_.ptr, mImpulse_.ptr, mFeature_.ptr};
    v.sb = SolverBuffers{};
    v.sb.bodyBest = bodyBest_.ptr;
    v.sb.bodyUsed = bodyUsed_.ptr;
    v.sb.color = color_.ptr;
    v.sb.dyn = dyn_.ptr;
    v.sb.order = order_.ptr;
    v.sb.colorStart = colorStart_.ptr;
    v.sb.pm = pm_.ptr;
    v.sb.pmInertia = pmInertia_.ptr;
    v.sb.pp = pp_.ptr;
    v.sb.pimp = pimp_.ptr;
    v.sb.pn = pn_.ptr;
    v.sb.pbody = pbody_.ptr;
    v.sb.pcount = pcount_.ptr;
    for (int c = 0; c < 2; ++c)
        v.cache[c] = CacheView{cacheKey_[c].ptr, cacheGens_[c].ptr, cacheA_[c].ptr, cacheB_[c].ptr, cacheT2_[c].ptr};
    v.cacheCount = cacheCount_.ptr;
    v.epoch = epoch_.ptr;
    v.colorCount = colorCount_.ptr;
    v.stats = stats_.ptr;
    v.worlds = descDev_.ptr;
    v.queue = queue_.ptr + bk.queueOff;
    v.queueLen = (uint32_t)bk.worlds.size();
    v.queueHead = queueHead_.ptr + (&bk - buckets_.data());
    v.batchErr = batchErr_.ptr;
    v.worldCount = (uint32_t)desc_.size();
    v.maxM = bk.maxM;
    v.maxN = bk.maxN;
    v.iterations = iterations;
    v.parity = parity;
    v.gx = gravity[0];
    v.gy = gravity[1];
    v.gz = gravity[2];
    v.dt = dt;
    return v;
}

void Batch::launchAll(float dt, uint32_t parity) {
    PE_CHECK(cudaMemsetAsync(queueHead_.ptr, 0, buckets_.size() * sizeof(uint32_t), stream_));
    PE_CHECK(cudaMemsetAsync(batchErr_.ptr, 0, sizeof(uint32_t), stream_));
    const size_t nbk = buckets_.size();
    if (nbk > 1) {
        PE_CHECK(cudaEventRecord(fork_, stream_));
        for (size_t i = 1; i < nbk; ++i) PE_CHECK(cudaStreamWaitEvent(side_[i - 1], fork_, 0));
    }
    for (size_t i = 0; i < nbk; ++i) {
        cudaStream_t s = i == 0 ? stream_ : side_[i - 1];
        launchBatchBucket(view(buckets_[i], dt, parity), buckets_[i].variant, buckets_[i].blocks, s);
    }
    for (size_t i = 1; i < nbk; ++i) {
        PE_CHECK(cudaEventRecord(joins_[i - 1], side_[i - 1]));
        PE_CHECK(cudaStreamWaitEvent(stream_, joins_[i - 1], 0));
    }
    PE_CHECK(cudaMemcpyAsync(hostErr_, batchErr_.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_));
}

void Batch::step(float dt) {
    PE_CHECK(cudaSetDevice(device_));
    if (buckets_.empty()) throw std::runtime_error("batch has no worlds");
    if (graphDt_ != dt) {
        dropGraphs();
        graphDt_ = dt;
    }
    for (int attempt = 0; attempt < 8; ++attempt) {
        PE_CHECK(cudaEventRecord(t0_, stream_));
        bool graphed = false;
        if (!graphsDisabled_) {
            cudaGraphExec_t &g = graph_[parity_][forces_ ? 1 : 0];
            if (!g) {
                cudaGraph_t graph = nullptr;
                cudaError_t e = cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal);
                if (e == cudaSuccess) {
                    try {
                        launchAll(dt, parity_);
                    } catch (...) {
                        cudaStreamEndCapture(stream_, &graph);
                        if (graph) cudaGraphDestroy(graph);
                        throw;
                    }
                    e = cudaStreamEndCapture(stream_, &graph);
                }
                if (e == cudaSuccess) e = cudaGraphInstantiate(&g, graph, 0);
                if (graph) cudaGraphDestroy(graph);
                if (e != cudaSuccess) {
                    graphError_ = cudaGetErrorString(e);
                    cudaGetLastError();
                    g = nullptr;
                    graphsDisabled_ = true;
                }
            }
            if (g) {
                PE_CHECK(cudaGraphLaunch(g, stream_));
                graphed = true;
            }
        }
        if (!graphed) launchAll(dt, parity_);
        PE_CHECK(cudaEventRecord(t1_, stream_));
        PE_CHECK(cudaStreamSynchronize(stream_));
        if (*hostErr_ == 0) {
            float ms = 0.0f;
            PE_CHECK(cudaEventElapsedTime(&ms, t0_, t1_));
            lastMs_ = ms;
            lastGraphed_ = graphed;
            lastLaunches_ = buckets_.size();
            parity_ ^= 1u;
            ++steps_;
            forces_ = false;  // PhysicsWorld::step clears forces (physics_world.cpp:766)
            return;
        }
        if (!finishStep()) continue;
    }
    throw std::runtime_error("batched step still overflowed its buffers after growing them");
}

// Grows what overflowed; returns false so that step() re-runs from the
// untouched state copy.
bool Batch::finishStep() {
    const uint32_t err = *hostErr_;
    const uint32_t W = (uint32_t)desc_.size();
    std::vector<DevStats> h(W);
    PE_CHECK(cudaMemcpy(h.data(), stats_.ptr, W * sizeof(DevStats), cudaMemcpyDeviceToHost));
    for (uint32_t w = 0; w < W; ++w) {
        if (h[w].err & kErrTimeout) throw std::runtime_error("world " + std::to_string(w) + ": a bounded wait timed out");
        if (h[w].err & kErrColors)
            throw std::runtime_error("world " + std::to_string(w) + ": the solver colouring exceeded its round limit");
    }
    if (!(err & (kErrPairCapacity | kErrManifoldCapacity | kErrSmallPath)))
        throw std::runtime_error("batched step failed on the device (error bits " + std::to_string(err) + ")");
    std::vector<uint32_t> pairCap(W), mCap(W);
    for (uint32_t w = 0; w < W; ++w) {
        pairCap[w] = desc_[w].pairCap;
        mCap[w] = desc_[w].mCap;
        if (h[w].err & kErrPairCapacity) pairCap[w] = pow2ceil((uint64_t)h[w].rawPairs + h[w].rawPairs / 2 + 64);
        if (h[w].err & kErrManifoldCapacity) {
            if (h[w].manifolds > kBlockMaxManifolds)
                throw std::runtime_error("world " + std::to_string(w) + " has " + std::to_string(h[w].manifolds) +
                                         " contact manifolds; a batched world holds at most " +
                                         std::to_string(kBlockMaxManifolds));
            mCap[w] = std::min<uint32_t>(kBlockMaxManifolds, pow2ceil((uint64_t)h[w].manifolds + h[w].manifolds / 2));
        }
    }
    dropGraphs();
    layout(pairCap, mCap, true);
    makeBuckets();
    return false;
}

void Batch::autotune(float dt, int reps) {
    PE_CHECK(cudaSetDevice(device_));
    if (reps < 1) reps = 1;
    // Run the step once without advancing (the state copy it reads stays
    // current) so that overflowing capacities grow before anything is timed.
    for (int attempt = 0;; ++attempt) {
        if (attempt == 8) throw std::runtime_error("batched step still overflowed its buffers after growing them");
        launchAll(dt, parity_);
        PE_CHECK(cudaStreamSynchronize(stream_));
        if (*hostErr_ == 0) break;
        finishStep();
    }
    for (size_t bi = 0; bi < buckets_.size(); ++bi) {
        BatchBucket &bk = buckets_[bi];
        bk.candidateMs.assign(kBatchVariantCount, 0.0);
        double best = 1e30;
        int bestV = bk.variant;
        for (int v = 0; v < kBatchVariantCount; ++v) {
            const size_t smem = batchSharedBytes(bk.maxN, bk.maxM);
            uint32_t blocks;
            try {
                blocks = std::min<uint32_t>((uint32_t)bk.worlds.size(), batchMaxBlocks(v, smem));
            } catch (const std::runtime_error &) {
                bk.candidateMs[v] = -1.0;
                continue;
            }
            BatchView view = this->view(bk, dt, parity_);
            float total = 0.0f;
            for (int r = 0; r < reps + 1; ++r) {
                PE_CHECK(cudaMemsetAsync(queueHead_.ptr + bi, 0, sizeof(uint32_t), stream_));
                PE_CHECK(cudaMemsetAsync(batchErr_.ptr, 0, sizeof(uint32_t), stream_));
                PE_CHECK(cudaEventRecord(t0_, stream_));
                launchBatchBucket(view, v, blocks, stream_);
                PE_CHECK(cudaEventRecord(t1_, stream_));
                PE_CHECK(cudaStreamSynchronize(stream_));
                float ms = 0.0f;
                PE_CHECK(cudaEventElapsedTime(&ms, t0_, t1_));
                if (r > 0) total += ms;  // the first launch warms up
            }
            const double avg = total / reps;
            bk.candidateMs[v] = avg;
            if (avg < best) {
                best = avg;
                bestV = v;
            }
        }
        bk.variant = bestV;
        bk.tunedMs = best;
        bk.blocks = std::min<uint32_t>((uint32_t)bk.worlds.size(),
                                       batchMaxBlocks(bestV, batchSharedBytes(bk.maxN, bk.maxM)));
    }
    dropGraphs();
}

void Batch::readBodies(float *pos, float *rot, float *lin, float *ang) {
    PE_CHECK(cudaSetDevice(device_));
    std::vector<float4> h(nb_);
    DeviceArray<float4> *src[4] = {&pos_[parity_], &rot_[parity_], &lin_[parity_], &ang_[parity_]};
    float *dst[4] = {pos, rot, lin, ang};
    const int width[4] = {3, 4, 3, 3};
    for (int k = 0; k < 4; ++k) {
        if (!dst[k]) continue;
        PE_CHECK(cudaMemcpy(h.data(), src[k]->ptr, nb_ * sizeof(float4), cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < nb_; ++i) {
            const float v[4] = {h[i].x, h[i].y, h[i].z, h[i].w};
            for (int c = 0; c < width[k]; ++c) dst[k][width[k] * i + c] = v[c];
        }
    }
}

void Batch::writeBodies(const float *pos, const float *rot, const float *lin, const float *ang) {
    PE_CHECK(cudaSetDevice(device_));
    std::vector<float4> h(nb_);
    DeviceArray<float4> *dst[4] = {&pos_[parity_], &rot_[parity_], &lin_[parity_], &ang_[parity_]};
    const float *src[4] = {pos, rot, lin, ang};
    const int width[4] = {3, 4, 3, 3};
    for (int k = 0; k < 4; ++k) {
        if (!src[k]) continue;
        for (uint64_t i = 0; i < nb_; ++i) {
            const float *v = src[k] + width[k] * i;
            h[i] = make_float4(v[0], v[1], v[2], width[k] == 4 ? v[3] : 0.0f);
        }
        PE_CHECK(cudaMemcpy(dst[k]->ptr, h.data(), nb_ * sizeof(float4), cudaMemcpyHostToDevice));
    }
}

// Forces in and poses out are repacked on the device (xyz per body <-> the
// engine's float4 arrays), reading and writing the caller's arrays in place
// when they are device-addressable (pinned host memory: over NVLink-C2C on
// GB300), through one plain copy each way otherwise.
__global__ void k_batch_forces_in(const float *f3, float4 *force, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        force[i] = make_float4(f3[3 * i], f3[3 * i + 1], f3[3 * i + 2], 0.0f);
}

__global__ void k_batch_poses_out(const float4 *pos, const float4 *rot, float *p3, float *q4, bool q4Vector,
                                  uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float4 p = pos[i], q = rot[i];
        p3[3 * i] = p.x;
        p3[3 * i + 1] = p.y;
        p3[3 * i + 2] = p.z;
        if (q4Vector) {
            reinterpret_cast<float4 *>(q4)[i] = q;
        } else {
            q4[4 * i] = q.x;
            q4[4 * i + 1] = q.y;
            q4[4 * i + 2] = q.z;
            q4[4 * i + 3] = q.w;
        }
    }
}

void Batch::writeForces(const float *forces) {
    PE_CHECK(cudaSetDevice(device_));
    const float *src = static_cast<const float *>(deviceAddress(forces, 4, device_));
    if (!src) {
        xfer_.reserve(4 * (size_t)nb_);
        PE_CHECK(cudaMemcpyAsync(xfer_.ptr, forces, 3 * (size_t)nb_ * sizeof(float), cudaMemcpyHostToDevice, stream_));
        src = xfer_.ptr;
    }
    const uint32_t grid = (uint32_t)std::min<uint64_t>((nb_ + 255) / 256, 8ull * smCount());
    k_batch_forces_in<<<std::max(grid, 1u), 256, 0, stream_>>>(src, force_.ptr, nb_);
    PE_LAUNCHED();
    // read in place: the caller's array is free again when this returns
    if (src != xfer_.ptr) PE_CHECK(cudaStreamSynchronize(stream_));
    forces_ = true;
}

void Batch::readPoses(float *pos, float *rot) {
    PE_CHECK(cudaSetDevice(device_));
    float *p = static_cast<float *>(deviceAddress(pos, 4, device_));
    float *q = static_cast<float *>(deviceAddress(rot, 4, device_));
    float *pd = p, *qd = q;
    if (!p || !q) xfer_.reserve(7 * (size_t)nb_);
    if (!p) pd = xfer_.ptr;
    if (!q) qd = xfer_.ptr + 3 * (size_t)nb_;
    const uint32_t grid = (uint32_t)std::min<uint64_t>((nb_ + 255) / 256, 8ull * smCount());
    k_batch_poses_out<<<std::max(grid, 1u), 256, 0, stream_>>>(pos_[parity_].ptr, rot_[parity_].ptr, pd, qd,
                                                                reinterpret_cast<uintptr_t>(qd) % 16 == 0, nb_);
    PE_LAUNCHED();
    if (!p) PE_CHECK(cudaMemcpyAsync(pos, pd, 3 * (size_t)nb_ * sizeof(float), cudaMemcpyDeviceToHost, stream_));
    if (!q) PE_CHECK(cudaMemcpyAsync(rot, qd, 4 * (size_t)nb_ * sizeof(float), cudaMemcpyDeviceToHost, stream_));
    PE_CHECK(cudaStreamSynchronize(stream_));
}

void Batch::worldCounters(uint32_t w, StepCounters &c) {
    if (w >= desc_.size()) throw std::invalid_argument("world index out of range");
    DevStats h;
    PE_CHECK(cudaMemcpy(&h, stats_.ptr + w, sizeof(DevStats), cudaMemcpyDeviceToHost));
    const uint64_t n = desc_[w].bodyCount;
    c = StepCounters{};
    c.possiblePairs = n * (n - 1) / 2;
    c.candidatePairs = h.pairs;
    c.contactCount = h.manifolds;
    c.solvedContactCount = h.solved;
    c.xWindow = h.xWindow;
    c.aabbPairs = h.uniquePairs;
    for (int k = 0; k < 4; ++k) {
        c.npCandidates[k] = h.npCandidates[k];
        c.npContacts[k] = h.npContacts[k];
    }
    c.preparedPoints = h.preparedPoints;
    c.warmComparisons = h.warmComparisons;
    c.warmMatches = h.warmMatches;
    c.velocityPointVisits = h.preparedPoints * (uint64_t)iterations;
    c.colors = h.colors;
    c.colorRounds = h.colorRounds;
    c.epaFailures = h.epaFailures;
    c.points = h.points;
    c.gpuMs = lastMs_;
    c.kernelLaunches = lastLaunches_;
    c.graphed = lastGraphed_;
    std::vector<uint32_t> flags(n);
    PE_CHECK(cudaMemcpy(flags.data(), bflags_.ptr + desc_[w].bodyStart, n * 4, cudaMemcpyDeviceToHost));
    for (uint32_t f : flags) c.awakeBodyCount += (f & kBodyStatic) ? 0 : 1;
}

uint32_t Batch::worldPairs(uint32_t w, uint32_t *pairs, uint32_t capacity) {
    if (w >= desc_.size()) throw std::invalid_argument("world index out of range");
    DevStats h;
    PE_CHECK(cudaMemcpy(&h, stats_.ptr + w, sizeof(DevStats), cudaMemcpyDeviceToHost));
    const uint32_t P = std::min(h.pairs, desc_[w].pairCap);
    if (pairs && capacity >= P && P) {
        std::vector<unsigned long long> k(P);
        PE_CHECK(cudaMemcpy(k.data(), pairKeys_.ptr + desc_[w].pairBase, P * 8ull, cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < P; ++i) {
            pairs[2 * i] = (uint32_t)(k[i] >> 32);
            pairs[2 * i + 1] = (uint32_t)k[i];
        }
    }
    return P;
}

uint32_t Batch::worldManifolds(uint32_t w, void *records, uint32_t capacity) {
    if (w >= desc_.size()) throw std::invalid_argument("world index out of range");
    DevStats h;
    PE_CHECK(cudaMemcpy(&h, stats_.ptr + w, sizeof(DevStats), cudaMemcpyDeviceToHost));
    const uint32_t M = std::min(h.manifolds, desc_[w].mCap);
    if (records && capacity >= M) {
        const uint32_t b = desc_[w].mBase;
        const size_t p = 4ull * b;
        ManifoldView mv{mBodyA_.ptr + b,  mGenA_.ptr + b,     mBodyB_.ptr + b,   mGenB_.ptr + b,
                        mNormal_.ptr + b, mRest_.ptr + b,     mCount_.ptr + b,   mAnchorA_.ptr + p,
                        mAnchorB_.ptr + p, mImpulse_.ptr + p, mFeature_.ptr + p};
        downloadManifoldRecords(mv, M, records);
    }
    return M;
}

} // namespace pe

// Seeded synthetic scene generators for the benchmark workloads and the parity
// tests.  Host-only C++ with its own sampling code on top of std::mt19937 (whose
// output sequence the C++ standard fixes), so a seed gives the same scene with
// any standard library.  Box-Muller and Shoemake use libm's log/sin/cos/sqrt in
// double; scenes are generated once per process and fed to every engine from
// the same arrays, so last-bit libm differences between hosts never enter a
// comparison.
//
// A scene is a list of body-creation records in the vocabulary of the
// reference's factories (PhysicsWorld::createSphere / createBox,
// include/phys/world/physics_world.hpp:43-50): shape, full box size or sphere
// radius, position, density in g/cm^3 (the reference's unit, so 1000 kg/m^3 is
// 1.0), static flag, restitution, friction, initial linear velocity, and an
// orientation "spin" vector applied with the reference's own idiom
// setAngularVelocity(spin); integrateRotation(1); setAngularVelocity(0).
// Convex hulls (not a reference shape) carry a hull index, mass and diagonal
// inverse inertia.
#include "phys_gb300_scenes.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <unordered_map>
#include <vector>

namespace {

struct Rng {
    std::mt19937 g;
    explicit Rng(uint32_t seed) : g(seed) {}
    // Exact float in [0, 1): the top 24 bits of one draw.
    float uniform() { return (float)(g() >> 8) * (1.0f / 16777216.0f); }
    float uniform(float a, float b) { return a + (b - a) * uniform(); }
    // (0, 1] in double from two draws.
    double uniform53() {
        uint64_t hi = g() >> 5, lo = g() >> 6;
        return ((double)(hi * 67108864ull + lo) + 1.0) * (1.0 / 9007199254740992.0);
    }
    double normal() {
        double u1 = uniform53(), u2 = uniform53();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
    uint32_t below(uint32_t n) { return (uint32_t)(((uint64_t)g() * n) >> 32); }
};

struct Builder {
    std::vector<uint8_t> shape, is_static;
    std::vector<float> dims, pos, density, restitution, friction, linvel, spin, mass, inv_inertia;
    std::vector<int32_t> hull_id;
    std::vector<float> hull_vertices;
    std::vector<uint32_t> hull_offsets{0};

    void add(uint8_t s, float d0, float d1, float d2, float px, float py, float pz, float dens, bool st,
             float rest, float fric, float vx = 0, float vy = 0, float vz = 0, float sx = 0, float sy = 0,
             float sz = 0, int32_t hid = -1, float m = 0, float i0 = 0, float i1 = 0, float i2 = 0) {
        shape.push_back(s);
        is_static.push_back(st ? 1 : 0);
        dims.insert(dims.end(), {d0, d1, d2});
        pos.insert(pos.end(), {px, py, pz});
        density.push_back(dens);
        restitution.push_back(rest);
        friction.push_back(fric);
        linvel.insert(linvel.end(), {vx, vy, vz});
        spin.insert(spin.end(), {sx, sy, sz});
        hull_id.push_back(hid);
        mass.push_back(m);
        inv_inertia.insert(inv_inertia.end(), {i0, i1, i2});
    }

    void emit(pe_scene *out) const {
        std::memset(out, 0, sizeof(*out));
        out->count = (uint32_t)shape.size();
        auto dup = [](const auto &v) {
            using E = typename std::decay_t<decltype(v)>::value_type;
            E *p = (E *)std::malloc(std::max<size_t>(1, v.size()) * sizeof(E));
            if (!v.empty()) std::memcpy(p, v.data(), v.size() * sizeof(E));
            return p;
        };
        out->shape = dup(shape);
        out->is_static = dup(is_static);
        out->dims = dup(dims);
        out->pos = dup(pos);
        out->density = dup(density);
        out->restitution = dup(restitution);
        out->friction = dup(friction);
        out->linvel = dup(linvel);
        out->spin = dup(spin);
        out->hull_id = dup(hull_id);
        out->mass = dup(mass);
        out->inv_inertia = dup(inv_inertia);
        out->hull_count = (uint32_t)hull_offsets.size() - 1;
        out->hull_offsets = dup(hull_offsets);
        out->hull_vertices = dup(hull_vertices);
    }
};

// Uniform unit quaternion (Shoemake's subgroup algorithm), returned as the
// spin vector of the reference's orientation idiom: the idiom yields
// normalize(0.5*spin, 1), so spin = 2*v/w with w > 0.
bool randomSpin(Rng &r, float &sx, float &sy, float &sz) {
    double u1 = r.uniform53(), u2 = r.uniform53(), u3 = r.uniform53();
    double a = std::sqrt(1.0 - u1), b = std::sqrt(u1);
    double qx = a * std::sin(6.283185307179586 * u2), qy = a * std::cos(6.283185307179586 * u2);
    double qz = b * std::sin(6.283185307179586 * u3), qw = b * std::cos(6.283185307179586 * u3);
    if (qw < 0) { qx = -qx; qy = -qy; qz = -qz; qw = -qw; }
    if (qw < 1e-2) return false;
    sx = (float)(2.0 * qx / qw);
    sy = (float)(2.0 * qy / qw);
    sz = (float)(2.0 * qz / qw);
    return true;
}

// Spatial hash of bounding spheres for rejection sampling without overlap.
struct SphereHash {
    double cell;
    std::unordered_map<uint64_t, std::vector<uint32_t>> cells;
    std::vector<float> cx, cy, cz, cr;
    explicit SphereHash(double c) : cell(c) {}
    static uint64_t key(int64_t x, int64_t y, int64_t z) {
        return ((uint64_t)(x & 0x1FFFFF) << 42) | ((uint64_t)(y & 0x1FFFFF) << 21) | (uint64_t)(z & 0x1FFFFF);
    }
    bool free(float x, float y, float z, float r) const {
        int64_t ix = (int64_t)std::floor(x / cell), iy = (int64_t)std::floor(y / cell), iz = (int64_t)std::floor(z / cell);
        for (int64_t a = ix - 1; a <= ix + 1; ++a)
            for (int64_t b = iy - 1; b <= iy + 1; ++b)
                for (int64_t c = iz - 1; c <= iz + 1; ++c) {
                    auto it = cells.find(key(a, b, c));
                    if (it == cells.end()) continue;
                    for (uint32_t k : it->second) {
                        double dx = x - cx[k], dy = y - cy[k], dz = z - cz[k], rr = r + cr[k];
                        if (dx * dx + dy * dy + dz * dz < rr * rr) return false;
                    }
                }
        return true;
    }
    void insert(float x, float y, float z, float r) {
        uint32_t k = (uint32_t)cx.size();
        cx.push_back(x); cy.push_back(y); cz.push_back(z); cr.push_back(r);
        cells[key((int64_t)std::floor(x / cell), (int64_t)std::floor(y / cell), (int64_t)std::floor(z / cell))].push_back(k);
    }
};

// 1,000 spheres (radius U[0.25,0.5]) rejection-sampled in a 20x40x20 m box above
// a static 40x1x40 m floor slab; friction 0.5, restitution 0, at rest.
void spheresOnFloor(uint32_t n, uint32_t seed, Builder &b) {
    Rng r(seed);
    b.add(1, 40.0f, 1.0f, 40.0f, 0.0f, -0.5f, 0.0f, 1.0f, true, 0.0f, 0.5f);
    SphereHash h(1.0);
    for (uint32_t i = 0; i < n;) {
        float rad = r.uniform(0.25f, 0.5f);
        float x = r.uniform(-10.0f, 10.0f), y = r.uniform(0.5f, 40.5f), z = r.uniform(-10.0f, 10.0f);
        if (!h.free(x, y, z, rad)) continue;
        h.insert(x, y, z, rad);
        b.add(0, rad, 0, 0, x, y, z, 1.0f, false, 0.0f, 0.5f);
        ++i;
    }
}

// Mixed spheres/oriented boxes in a volume with N(0,1) velocities (no floor).
void mixedVolume(uint32_t n, uint32_t seed, float sx, float sy, float sz, Builder &b) {
    Rng r(seed);
    std::vector<uint8_t> isSphere(n, 0);
    std::fill(isSphere.begin(), isSphere.begin() + (n + 1) / 2, 1);
    for (uint32_t i = n; i > 1; --i) std::swap(isSphere[i - 1], isSphere[r.below(i)]);
    SphereHash h(2.2);
    for (uint32_t i = 0; i < n;) {
        float d0, d1, d2, bound;
        if (isSphere[i]) {
            d0 = r.uniform(0.2f, 0.6f);
            d1 = d2 = 0.0f;
            bound = d0;
        } else {
            float hx = r.uniform(0.2f, 0.6f), hy = r.uniform(0.2f, 0.6f), hz = r.uniform(0.2f, 0.6f);
            d0 = 2.0f * hx; d1 = 2.0f * hy; d2 = 2.0f * hz;
            bound = std::sqrt(hx * hx + hy * hy + hz * hz);
        }
        float x = r.uniform(-0.5f * sx, 0.5f * sx), y = r.uniform(-0.5f * sy, 0.5f * sy),
              z = r.uniform(-0.5f * sz, 0.5f * sz);
        if (!h.free(x, y, z, bound)) continue;
        float s0 = 0, s1 = 0, s2 = 0;
        if (!isSphere[i])
            while (!randomSpin(r, s0, s1, s2)) {}
        float vx = (float)r.normal(), vy = (float)r.normal(), vz = (float)r.normal();
        h.insert(x, y, z, bound);
        b.add(isSphere[i] ? 0 : 1, d0, d1, d2, x, y, z, 1.0f, false, 0.1f, 0.5f, vx, vy, vz, s0, s1, s2);
        ++i;
    }
}

// Planar box pyramids on a tiled static floor, plus convex hulls (24 points on
// an ellipsoid, semi-axes U[0.3,0.8]) dropped from 30 m and above.
void pyramids(uint32_t grid, uint32_t base, uint32_t hullCount, uint32_t seed, Builder &b) {
    Rng r(seed);
    const float pitchX = (float)base + 3.0f, pitchZ = 1.0f + 3.0f;
    const float extentX = grid * pitchX, extentZ = grid * pitchZ;
    // Floor tiles 64 x 1 x 64 m (4096 m^3, the reference's static-volume cap),
    // top face at y = 0.
    int tilesX = (int)std::ceil(extentX / 64.0f), tilesZ = (int)std::ceil(extentZ / 64.0f);
    for (int tx = 0; tx < tilesX; ++tx)
        for (int tz = 0; tz < tilesZ; ++tz)
            b.add(1, 64.0f, 1.0f, 64.0f, -0.5f * tilesX * 64.0f + 32.0f + 64.0f * tx, -0.5f,
                  -0.5f * tilesZ * 64.0f + 32.0f + 64.0f * tz, 1.0f, true, 0.0f, 0.6f);
    for (uint32_t gx = 0; gx < grid; ++gx)
        for (uint32_t gz = 0; gz < grid; ++gz) {
            float cx = -0.5f * extentX + pitchX * (gx + 0.5f), cz = -0.5f * extentZ + pitchZ * (gz + 0.5f);
            for (uint32_t row = 0; row < base; ++row) {
                uint32_t count = base - row;
                for (uint32_t i = 0; i < count; ++i) {
                    float x = cx + ((float)i - 0.5f * (float)(count - 1));
                    b.add(1, 1.0f, 1.0f, 1.0f, x, 0.5f + (float)row, cz, 1.0f, false, 0.0f, 0.6f);
                }
            }
        }
    if (hullCount == 0) return;
    // 24 unit-sphere directions (Fibonacci lattice), scaled per hull.
    float dirs[24][3];
    for (int k = 0; k < 24; ++k) {
        double y = 1.0 - (k + 0.5) * 2.0 / 24.0, rad = std::sqrt(1.0 - y * y);
        double phi = k * 2.399963229728653;
        dirs[k][0] = (float)(rad * std::cos(phi));
        dirs[k][1] = (float)y;
        dirs[k][2] = (float)(rad * std::sin(phi));
    }
    SphereHash h(1.8);
    const float pi = 3.14159265358979323846f;
    for (uint32_t i = 0; i < hullCount;) {
        float a = r.uniform(0.3f, 0.8f), bb = r.uniform(0.3f, 0.8f), c = r.uniform(0.3f, 0.8f);
        float bound = std::max(a, std::max(bb, c));
        float x = r.uniform(-0.5f * extentX + 1.0f, 0.5f * extentX - 1.0f);
        float y = r.uniform(30.0f, 60.0f);
        float z = r.uniform(-0.5f * extentZ + 1.0f, 0.5f * extentZ - 1.0f);
        if (!h.free(x, y, z, bound)) continue;
        float s0, s1, s2;
        while (!randomSpin(r, s0, s1, s2)) {}
        h.insert(x, y, z, bound);
        int32_t hid = (int32_t)b.hull_offsets.size() - 1;
        for (int k = 0; k < 24; ++k)
            b.hull_vertices.insert(b.hull_vertices.end(), {dirs[k][0] * a, dirs[k][1] * bb, dirs[k][2] * c});
        b.hull_offsets.push_back((uint32_t)(b.hull_vertices.size() / 3));
        float m = (4.0f / 3.0f) * pi * a * bb * c;
        float i0 = 5.0f / (m * (bb * bb + c * c)), i1 = 5.0f / (m * (a * a + c * c)), i2 = 5.0f / (m * (a * a + bb * bb));
        b.add(2, a, bb, c, x, y, z, 1.0f, false, 0.0f, 0.6f, 0, 0, 0, s0, s1, s2, hid, m, i0, i1, i2);
        ++i;
    }
}

// Boxes (half-extents U[0.2,0.5]) resting on a static floor slab, materials
// friction U[0.2,0.8], restitution U[0,0.3].
void boxesOnPlane(uint32_t n, uint32_t seed, Builder &b) {
    Rng r(seed);
    b.add(1, 40.0f, 1.0f, 40.0f, 0.0f, -0.5f, 0.0f, 1.0f, true, 0.0f, 0.5f);
    uint32_t side = (uint32_t)std::ceil(std::sqrt((double)n));
    for (uint32_t i = 0; i < n; ++i) {
        float hx = r.uniform(0.2f, 0.5f), hy = r.uniform(0.2f, 0.5f), hz = r.uniform(0.2f, 0.5f);
        float fr = r.uniform(0.2f, 0.8f), re = r.uniform(0.0f, 0.3f);
        float x = 1.2f * ((float)(i % side) - 0.5f * (float)(side - 1));
        float z = 1.2f * ((float)(i / side) - 0.5f * (float)(side - 1));
        b.add(1, 2.0f * hx, 2.0f * hy, 2.0f * hz, x, hy, z, 1.0f, false, re, fr);
    }
}

} // namespace

extern "C" {

int pe_scene_generate(int kind, uint32_t n, uint32_t seed, pe_scene *out) {
    if (!out) return 1;
    Builder b;
    switch (kind) {
    case PE_SCENE_SPHERES_ON_FLOOR: spheresOnFloor(n, seed, b); break;
    case PE_SCENE_MIXED_VOLUME: {
        // 200 x 100 x 200 m for 100,000 bodies; other counts keep the density.
        float s = (float)std::cbrt((double)n / 100000.0);
        mixedVolume(n, seed, 200.0f * s, 100.0f * s, 200.0f * s, b);
        break;
    }
    case PE_SCENE_PYRAMIDS: {
        // n = pyramids per side; hulls scale with the pyramid count (20,000 at 16).
        uint32_t hulls = (uint32_t)((uint64_t)20000 * n * n / 256);
        pyramids(n, 20, hulls, seed, b);
        break;
    }
    case PE_SCENE_PYRAMIDS_BOXES_ONLY: pyramids(n, 20, 0, seed, b); break;
    case PE_SCENE_BOXES_ON_PLANE: boxesOnPlane(n, seed, b); break;
    default: return 2;
    }
    b.emit(out);
    return 0;
}

void pe_scene_free(pe_scene *s) {
    if (!s) return;
    void *ptrs[] = {s->shape, s->is_static, s->dims, s->pos, s->density, s->restitution, s->friction,
                    s->linvel, s->spin, s->hull_id, s->mass, s->inv_inertia, s->hull_offsets, s->hull_vertices};
    for (void *p : ptrs) std::free(p);
    std::memset(s, 0, sizeof(*s));
}

} // extern "C"

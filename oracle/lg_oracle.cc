// CPU oracle of the LightGraph path -- TEST INFRASTRUCTURE (see lg_oracle.h).
// FP64 restatement of the reference loops; compiled with -ffp-contract=off so
// x86-64 and aarch64 give the same numbers. PARITY UNPINNED (no reference tests
// or fixtures exist; the reference cannot be built here).
#include "lg_oracle.h"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>
#include <climits>
#include <random>
#include <set>
#include <tuple>

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kDelta = 1e-9;  // openvdb::math::Delta<double>::value()
const double kInfD = std::numeric_limits<double>::infinity();

struct V3 {
    double x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(double a, double b, double c) : x(a), y(b), z(c) {}
    explicit V3(double a) : x(a), y(a), z(a) {}
    double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    V3 operator+(const V3& o) const { return V3(x + o.x, y + o.y, z + o.z); }
    V3 operator-(const V3& o) const { return V3(x - o.x, y - o.y, z - o.z); }
    V3 operator*(const V3& o) const { return V3(x * o.x, y * o.y, z * o.z); }
    V3 operator*(double s) const { return V3(x * s, y * s, z * s); }
    V3 operator/(double s) const { return V3(x / s, y / s, z / s); }
    V3& operator+=(const V3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    V3& operator*=(const V3& o) { x *= o.x; y *= o.y; z *= o.z; return *this; }
    double lengthSqr() const { return x * x + y * y + z * z; }
    double dot(const V3& o) const { return x * o.x + y * o.y + z * o.z; }
};

V3 vexp(const V3& v) { return V3(std::exp(v.x), std::exp(v.y), std::exp(v.z)); }

// ---------------------------------------------------------------------------
// counter-based random streams (same formulas as the GPU path)
// ---------------------------------------------------------------------------
uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}
float u01(uint32_t h) { return (float)(h >> 8) * (1.0f / 16777216.0f); }
struct Stream { uint32_t a, b; };
Stream make_stream(uint64_t seed, uint64_t id) {
    const uint64_t k = mix64(seed ^ mix64(id));
    return Stream{(uint32_t)k, (uint32_t)(k >> 32)};
}
float draw(Stream s, uint32_t key) { return u01(hash32(s.a ^ (s.b + key * 0x9E3779B9u))); }
uint32_t shadow_key(Stream s, uint32_t n, uint32_t k, uint32_t ls) {
    return hash32(s.a ^ hash32(s.b ^ (0x30000000u | (n & 0x0FFFFFFFu))) + k * 0x9E3779B9u + ls * 0x85EBCA6Bu);
}
float draw_sub(uint32_t sub, uint32_t key) { return u01(hash32(sub ^ (key * 0x9E3779B9u))); }
// Step-jitter streams: a full-period 32-bit LCG advanced once per loop
// iteration, seeded by a hash of the march's key; u = (x >> 9) / 2^23.
uint32_t step_next(uint32_t x) { return x * 1664525u + 1013904223u; }
double step_u(uint32_t x) { return (double)(x >> 9) * (1.0 / 8388608.0); }
constexpr uint64_t kDomainPixel = 0x01ull << 56, kDomainVertex = 0x02ull << 56;
constexpr uint32_t kTagJitterX = 0x00000000u, kTagJitterY = 0x00000001u, kTagPrimarySpan = 0x10000000u,
                   kTagPrimaryStep = 0x20000000u, kTagShadowSpan = 0x40000000u, kTagShadowStep = 0x50000000u,
                   kTagEnvU = 0x60000000u, kTagEnvV = 0x60000001u;

// ---------------------------------------------------------------------------
// grid: dense values + leaf table (OpenVDB FloatGrid restated)
// ---------------------------------------------------------------------------
struct Grid {
    const float* v = nullptr;
    int dims[3] = {0, 0, 0}, origin[3] = {0, 0, 0};
    double h = 1.0, wo[3] = {0, 0, 0};
    int lnx = 0, lny = 0, lnz = 0;  // leaves over the box
    std::vector<uint8_t> leaf;
    bool has_leaves = false;
    double bbmin[3] = {0, 0, 0}, bbmax[3] = {0, 0, 0};  // leaf bbox padded by one voxel

    void init(const lgo_grid* g) {
        v = g->values;
        for (int a = 0; a < 3; ++a) {
            dims[a] = g->desc.dims[a];
            origin[a] = g->desc.origin[a];
            wo[a] = g->desc.world_origin[a];
        }
        h = g->desc.voxel_size;
        lnx = (dims[0] + 7) / 8;
        lny = (dims[1] + 7) / 8;
        lnz = (dims[2] + 7) / 8;
        leaf.assign((size_t)lnx * lny * lnz, 0);
        for (int lz = 0; lz < lnz; ++lz)
            for (int ly = 0; ly < lny; ++ly)
                for (int lx = 0; lx < lnx; ++lx) {
                    const size_t li = ((size_t)lz * lny + ly) * lnx + lx;
                    if (g->desc.leaf_mask) {
                        leaf[li] = g->desc.leaf_mask[li] ? 1 : 0;
                        continue;
                    }
                    bool any = false;
                    for (int z = lz * 8; z < std::min(lz * 8 + 8, dims[2]) && !any; ++z)
                        for (int y = ly * 8; y < std::min(ly * 8 + 8, dims[1]) && !any; ++y)
                            for (int x = lx * 8; x < std::min(lx * 8 + 8, dims[0]); ++x)
                                if (v[((size_t)z * dims[1] + y) * dims[0] + x] != 0.0f) { any = true; break; }
                    leaf[li] = any;
                }
        int mn[3] = {1 << 30, 1 << 30, 1 << 30}, mx[3] = {-(1 << 30), -(1 << 30), -(1 << 30)};
        for (int lz = 0; lz < lnz; ++lz)
            for (int ly = 0; ly < lny; ++ly)
                for (int lx = 0; lx < lnx; ++lx)
                    if (leaf[((size_t)lz * lny + ly) * lnx + lx]) {
                        const int c[3] = {lx, ly, lz};
                        for (int a = 0; a < 3; ++a) {
                            mn[a] = std::min(mn[a], c[a]);
                            mx[a] = std::max(mx[a], c[a]);
                        }
                    }
        has_leaves = mn[0] <= mx[0];
        // evalActiveBoundingBox at node granularity, then max.offset(1)
        for (int a = 0; a < 3; ++a) {
            bbmin[a] = has_leaves ? (double)(origin[a] + 8 * mn[a]) : 0.0;
            bbmax[a] = has_leaves ? (double)(origin[a] + 8 * mx[a] + 7 + 1) : 0.0;
        }
    }
    float voxel(int x, int y, int z) const {
        x -= origin[0];
        y -= origin[1];
        z -= origin[2];
        if (x < 0 || y < 0 || z < 0 || x >= dims[0] || y >= dims[1] || z >= dims[2]) return 0.0f;
        return v[((size_t)z * dims[1] + y) * dims[0] + x];
    }
    bool is_leaf_cell(int cx, int cy, int cz) const {  // cell = index >> 3
        const int lx = cx - (origin[0] >> 3), ly = cy - (origin[1] >> 3), lz = cz - (origin[2] >> 3);
        if (lx < 0 || ly < 0 || lz < 0 || lx >= lnx || ly >= lny || lz >= lnz) return false;
        return leaf[((size_t)lz * lny + ly) * lnx + lx] != 0;
    }
    // BoxSampler::sample at an index position: float voxel values, double
    // weights, interpolated along z, then y, then x; result float.
    float sample_index(double px, double py, double pz) const {
        const double fx = std::floor(px), fy = std::floor(py), fz = std::floor(pz);
        const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
        const double u = px - fx, w = py - fy, t = pz - fz;
        float d[2][2][2];
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int c = 0; c < 2; ++c) d[a][b][c] = voxel(ix + a, iy + b, iz + c);
        auto lerp = [](float a, float b, double wt) {
            const double temp = (double)(b - a) * wt;
            return (float)(a + (float)temp);
        };
        return lerp(lerp(lerp(d[0][0][0], d[0][0][1], t), lerp(d[0][1][0], d[0][1][1], t), w),
                    lerp(lerp(d[1][0][0], d[1][0][1], t), lerp(d[1][1][0], d[1][1][1], t), w), u);
    }
    // GridSampler::wsSample
    float sample_world(const V3& p) const {
        return sample_index((p.x - wo[0]) / h, (p.y - wo[1]) / h, (p.z - wo[2]) / h);
    }
    V3 world_to_index(const V3& p) const { return V3((p.x - wo[0]) / h, (p.y - wo[1]) / h, (p.z - wo[2]) / h); }
    V3 index_to_world(const V3& p) const { return V3(p.x * h + wo[0], p.y * h + wo[1], p.z * h + wo[2]); }
};

// ---------------------------------------------------------------------------
// VolumeRayIntersector restated: index ray, bbox clip, leaf-span march
// ---------------------------------------------------------------------------
struct IndexRay {
    V3 e, d, inv;
    double t0, t1;
    V3 at(double t) const { return V3(e.x + t * d.x, e.y + t * d.y, e.z + t * d.z); }
};

// Ray::worldToIndex for a uniform linear map: unit direction, times / voxel.
IndexRay world_to_index(const Grid& g, const V3& eye, const V3& dir_unit, double t0, double t1) {
    IndexRay r;
    r.e = g.world_to_index(eye);
    const V3 di = dir_unit / g.h;
    const double len = std::sqrt(di.lengthSqr());
    r.d = di / len;
    r.t0 = len * t0;
    r.t1 = len * t1;
    r.inv = V3(1.0 / r.d.x, 1.0 / r.d.y, 1.0 / r.d.z);
    return r;
}

bool clip(const Grid& g, IndexRay& r) {
    if (!g.has_leaves) return false;
    double t0 = r.t0, t1 = r.t1;
    for (int i = 0; i < 3; ++i) {
        double a = (g.bbmin[i] - r.e[i]) * r.inv[i];
        double b = (g.bbmax[i] - r.e[i]) * r.inv[i];
        if (a > b) std::swap(a, b);
        if (a > t0) t0 = a;
        if (b < t1) t1 = b;
        if (t0 > t1) return false;
    }
    r.t0 = t0;
    r.t1 = t1;
    return true;
}

// Maximal runs of leaf cells along the ray, from a DDA over 8^3 cells.
struct SpanMarch {
    const Grid* g;
    double t, tmax;
    double next[3], delta[3];
    int cell[3], step[3];
    bool open = false, done = false;
    double start = 0;
    SpanMarch(const Grid& grid, const IndexRay& r) : g(&grid), t(r.t0), tmax(r.t1) {
        const V3 p = r.at(r.t0);
        for (int i = 0; i < 3; ++i) {
            const int vox = (int)std::floor(p[i]);
            const int c = vox >> 3;  // floor division by 8
            cell[i] = c;
            if (r.d[i] == 0.0) {
                step[i] = 0;
                next[i] = std::numeric_limits<double>::max();
                delta[i] = std::numeric_limits<double>::max();
            } else if (r.inv[i] > 0) {
                step[i] = 1;
                next[i] = r.t0 + ((double)(c * 8 + 8) - p[i]) * r.inv[i];
                delta[i] = 8.0 * r.inv[i];
            } else {
                step[i] = -1;
                next[i] = r.t0 + ((double)(c * 8) - p[i]) * r.inv[i];
                delta[i] = -8.0 * r.inv[i];
            }
        }
    }
    bool next_span(double& ta, double& tb) {
        while (!done) {
            const bool leaf = g->is_leaf_cell(cell[0], cell[1], cell[2]);
            if (leaf) {
                if (!open) { open = true; start = t; }
            } else if (open) {
                open = false;
                if (t - start > kDelta) { ta = start; tb = t; return true; }
            }
            int a;
            if (next[0] < next[1]) a = (next[0] < next[2]) ? 0 : 2;
            else a = (next[1] < next[2]) ? 1 : 2;
            t = next[a];
            next[a] += delta[a];
            cell[a] += step[a];
            if (!(t <= tmax)) {
                done = true;
                if (open && tmax - start > kDelta) { ta = start; tb = tmax; return true; }
            }
        }
        return false;
    }
};

V3 ext_of(const lg_shader* sh) { return V3(sh->extinction[0], sh->extinction[1], sh->extinction[2]); }
V3 albedo_of(const lg_shader* sh) { return V3(sh->albedo[0], sh->albedo[1], sh->albedo[2]); }

// ColorRamp::getColor (src/Shader.h:63-92)
V3 ramp(const lg_shader* sh, double t) {
    const int n = sh->ramp_n;
    if (n == 0) return V3(0.0);
    double x = (t - sh->ramp_in) / (sh->ramp_out - sh->ramp_in);
    x = std::min(std::max(x, 0.0), 1.0);
    auto col = [&](int k) { return V3(sh->ramp_color[k][0], sh->ramp_color[k][1], sh->ramp_color[k][2]); };
    if (n == 1) return col(0);
    int prev = 0, next = 0;
    for (int i = 0; i < n; ++i) {
        if (sh->ramp_pos[i] <= x) prev = i;
        else { next = i; break; }
    }
    const double range = sh->ramp_pos[next] - sh->ramp_pos[prev];
    const double blend = (x - sh->ramp_pos[prev]) / range;
    return col(prev) * (1.0 - blend) + col(next) * blend;
}

// ---------------------------------------------------------------------------
// environment light
// ---------------------------------------------------------------------------
struct Dist1D {
    std::vector<float> func, cdf;
    float funcInt = 0;
    void build(const float* f, int n) {
        func.assign(f, f + n);
        cdf.assign(n + 1, 0.f);
        double acc = 0.0;
        for (int i = 1; i <= n; ++i) acc += (double)f[i - 1] / (double)n;
        const double total = acc;
        if (total == 0.0) {
            for (int i = 1; i <= n; ++i) cdf[i] = (float)((double)i / (double)n);
        } else {
            double run = 0.0;
            for (int i = 1; i <= n; ++i) {
                run += (double)f[i - 1] / (double)n;
                cdf[i] = (float)(run / total);
            }
        }
        funcInt = (float)total;
    }
    // SampleContinuous with FindInterval (src/Sampling.h:59-72,102-119)
    float sample(float u, int* off_out) const {
        const int size = (int)cdf.size();
        int first = 0, len = size;
        while (len > 0) {
            const int half = len >> 1, middle = first + half;
            if (cdf[middle] <= u) { first = middle + 1; len -= half + 1; }
            else len = half;
        }
        int off = std::min(std::max(first - 1, 0), size - 2);
        float du = u - cdf[off];
        if ((cdf[off + 1] - cdf[off]) > 0) du /= (cdf[off + 1] - cdf[off]);
        if (off_out) *off_out = off;
        return ((float)off + du) / (float)func.size();
    }
};

struct EnvDist {
    int w = 0, h = 0;
    const float* rgb = nullptr;
    std::vector<Dist1D> cond;
    Dist1D marg;
    void build(const lgo_env* env) {
        w = env->w;
        h = env->h;
        rgb = env->rgb;
        std::vector<float> Y((size_t)w * h);
        for (int i = 0; i < h; ++i) {
            const float sin_theta = (float)std::sin(kPi * (double)((float)i / (float)(h - 1)));
            for (int j = 0; j < w; ++j) {
                const float* p = rgb + ((size_t)i * w + j) * 3;
                const float y = (float)(0.2126 * (double)p[0] + 0.7152 * (double)p[1] + 0.0722 * (double)p[2]);
                Y[(size_t)i * w + j] = y * sin_theta;
            }
        }
        cond.resize(h);
        std::vector<float> mf(h);
        for (int v = 0; v < h; ++v) {
            cond[v].build(&Y[(size_t)v * w], w);
            mf[v] = cond[v].funcInt;
        }
        marg.build(mf.data(), h);
    }
    // EnvLight::illuminate (src/Light.h:185-233); the column index wraps and
    // the row clamps where the reference reads one texel past the map.
    void illuminate(const lg_light& L, float u, float v, V3& ldir, V3& I) const {
        int row;
        const float d1 = marg.sample(v, &row);
        const float d0 = cond[row].sample(u, nullptr);
        const float xs = d0 * (float)w, ys = d1 * (float)h;
        int col_lo = (int)std::floor(xs), row_lo = (int)std::floor(ys);
        int col_hi = (int)std::ceil(xs), row_hi = (int)std::ceil(ys);
        const float col_ratio = xs - (float)col_lo, row_ratio = ys - (float)row_lo;
        if (col_lo >= w) col_lo = w - 1;
        if (row_lo >= h) row_lo = h - 1;
        if (col_hi >= w) col_hi -= w;
        if (col_hi >= w) col_hi = w - 1;
        if (row_hi >= h) row_hi = h - 1;
        const float theta = d0 * (float)kPi * 2.0f;
        const float phi = d1 * (float)kPi;
        const double sphi = (double)std::sin(phi);
        V3 sd((double)std::cos(theta) * sphi, (double)std::cos(phi), (double)std::sin(theta) * sphi);
        V3 t;
        for (int c = 0; c < 3; ++c) t[c] = sd[0] * L.rot[0 * 3 + c] + sd[1] * L.rot[1 * 3 + c] + sd[2] * L.rot[2 * 3 + c];
        const double len = std::sqrt(t.lengthSqr());
        t = t / len;
        auto texel = [&](int r, int c) {
            const float* p = rgb + ((size_t)r * w + c) * 3;
            return V3(p[0], p[1], p[2]);
        };
        const V3 img = texel(row_lo, col_lo) * (double)((1.0f - row_ratio) * (1.0f - col_ratio)) +
                       texel(row_lo, col_hi) * (double)((1.0f - row_ratio) * col_ratio) +
                       texel(row_hi, col_lo) * (double)(row_ratio * (1.0f - col_ratio)) +
                       texel(row_hi, col_hi) * (double)(row_ratio * col_ratio);
        ldir = V3(-t.x, -t.y, -t.z);
        I = img * V3(L.color[0], L.color[1], L.color[2]) * (double)(float)L.intensity;
    }
};

// Light::illuminate for distant and point lights (src/Light.h:79-89,118-126)
void illuminate(const lg_light& L, const V3& p, V3& ldir, V3& I, double& dist) {
    const V3 color(L.color[0], L.color[1], L.color[2]);
    const double inten = (double)(float)L.intensity;
    if (L.type == LG_LIGHT_POINT) {
        V3 d = p - V3(L.pos[0], L.pos[1], L.pos[2]);
        const float r2 = (float)d.lengthSqr();
        dist = std::sqrt(r2);
        ldir = d / dist;
        I = color * inten / (1.0 + 4.0 * kPi * r2);
    } else {
        ldir = V3(L.dir[0], L.dir[1], L.dir[2]);
        I = color * inten;
        dist = std::numeric_limits<double>::max();
    }
}

}  // namespace

extern "C" int lgo_threads(void) { return omp_get_max_threads(); }

// ---------------------------------------------------------------------------
// scatterPoints (src/LightGraph.h:206-274) with RandGen (src/RandGen.h:16-44):
// the same std::mt19937 engines (seeded seed_base + iteration) read through
// std::uniform_real_distribution<float>(0, 1) of this host's C++ library, the
// active-voxel bbox of the grid (src/main.cc:512-518) and float / double types
// as the reference declares them.
// ---------------------------------------------------------------------------
extern "C" void lgo_randgen_draws(uint32_t seed, int64_t n, float* out, uint32_t* raw) {
    std::mt19937 eng(seed), eng2(seed);
    std::uniform_real_distribution<float> uni(0.0f, 1.0f);
    for (int64_t k = 0; k < n; ++k) {
        if (raw) raw[k] = (uint32_t)eng2();
        if (out) out[k] = uni(eng);
    }
}

extern "C" void lgo_scatter_points(const lgo_grid* dens, const lg_scatter_opts* o, int first_iter, int n_iter,
                                   float* points, int32_t* counts, float* last_min_dist_sq) {
    Grid g;
    g.init(dens);
    int vmin[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, vmax[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
    for (int z = 0; z < g.dims[2]; ++z)
        for (int y = 0; y < g.dims[1]; ++y)
            for (int x = 0; x < g.dims[0]; ++x)
                if (g.v[((size_t)z * g.dims[1] + y) * g.dims[0] + x] != 0.0f) {
                    const int c[3] = {x, y, z};
                    for (int a = 0; a < 3; ++a) {
                        vmin[a] = std::min(vmin[a], c[a] + g.origin[a]);
                        vmax[a] = std::max(vmax[a], c[a] + g.origin[a]);
                    }
                }
    double bbmin[3];
    float bbsize[3];
    for (int a = 0; a < 3; ++a) {
        bbmin[a] = g.wo[a] + (double)vmin[a] * g.h;
        bbsize[a] = (float)((g.wo[a] + (double)vmax[a] * g.h) - bbmin[a]);
    }
    const float avg = (bbsize[0] + bbsize[1] + bbsize[2]) / 3.0f;
    const float min_dist = o->min_dist_mult * avg;
    const uint32_t batch = o->scatter_count / o->n_estimates;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < n_iter; ++i) {
        std::mt19937 eng(o->seed_base + (uint32_t)(first_iter + i));
        std::uniform_real_distribution<float> uni(0.0f, 1.0f);
        std::vector<V3> pc;
        float m2 = min_dist * min_dist, last = m2;
        uint32_t pc_size = 0;
        for (uint32_t n = 0; n < o->scatter_count; ++n) {
            float np[3];
            for (int a = 0; a < 3; ++a) np[a] = uni(eng) * bbsize[a] + bbmin[a];
            if (pc_size > o->target_size) break;
            if ((n + 1) % batch == 0) {
                const uint32_t expected =
                    o->target_size * std::pow((double)n / (double)o->scatter_count, (double)o->growth_power);
                const double ratio = pc_size / (double)expected;
                m2 *= ratio;
            }
            const V3 pt(np[0], np[1], np[2]);
            if (g.sample_world(pt) < o->density_cutoff) continue;
            bool collision = false;
            for (size_t k = 0; k < pc.size(); ++k)
                if ((pt - pc[k]).lengthSqr() < m2) { collision = true; break; }
            if (!collision) {
                pc.push_back(pt);
                last = m2;
                ++pc_size;
            }
        }
        float* dst = points + (size_t)i * o->hard_limit * 3;
        for (size_t k = 0; k < pc.size() && k < o->hard_limit; ++k) {
            dst[3 * k] = (float)pc[k].x;
            dst[3 * k + 1] = (float)pc[k].y;
            dst[3 * k + 2] = (float)pc[k].z;
        }
        counts[i] = (int32_t)pc.size();
        last_min_dist_sq[i] = last;
    }
}

// ---------------------------------------------------------------------------
// buildGraph (src/LightGraph.h:287-318)
// ---------------------------------------------------------------------------
extern "C" int64_t lgo_build_graph(int n, const float* pts, float radius_sq, int max_connect, uint8_t* adj) {
    std::vector<uint32_t> cnt(n, 0);
    std::memset(adj, 0, (size_t)n * n);
    int64_t connect = 0;
    const double r2 = (double)radius_sq;
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) {
            if (cnt[i] >= (uint32_t)max_connect) break;
            if (cnt[j] >= (uint32_t)max_connect) continue;
            if (i < j) {
                const double dx = (double)pts[3 * i] - (double)pts[3 * j];
                const double dy = (double)pts[3 * i + 1] - (double)pts[3 * j + 1];
                const double dz = (double)pts[3 * i + 2] - (double)pts[3 * j + 2];
                if (dx * dx + dy * dy + dz * dz < r2) {
                    adj[(size_t)i * n + j] = 1;
                    adj[(size_t)j * n + i] = 1;
                    ++cnt[i];
                    ++cnt[j];
                    ++connect;
                }
            }
        }
    }
    return connect;
}

// ---------------------------------------------------------------------------
// raymarchConnection (src/LightGraph.h:347-418)
// ---------------------------------------------------------------------------
extern "C" void lgo_march_edges(const lgo_grid* dens, const lg_shader* sh, const lg_settings* st, int n,
                                const float* pts, const uint8_t* adj, double* T, double* S) {
    Grid g;
    g.init(dens);
    const V3 ext = ext_of(sh);
    const double step = st->step[1], cutoff = st->cutoff;
    const double scale = sh->density_scale * sh->shadow_density_scale * sh->scatter_density_scale;
    if (T) std::fill(T, T + (size_t)n * n * 3, 0.0);
    if (S) std::fill(S, S + (size_t)n * n, kInfD);
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < n; ++i) {
        for (int j = i + 1; j < n; ++j) {
            if (!adj[(size_t)i * n + j]) continue;
            const V3 start(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
            V3 dir = V3(pts[3 * j], pts[3 * j + 1], pts[3 * j + 2]) - start;
            const float dist = (float)std::sqrt(dir.lengthSqr());
            dir = dir / std::sqrt(dir.lengthSqr());
            IndexRay r = world_to_index(g, start, dir, kDelta, (double)dist);
            if (!clip(g, r)) continue;  // pathGraph stays 0
            V3 trans(1.0);
            double s_sum = 0.0;
            bool dropped = false;
            SpanMarch m(g, r);
            double t0, t1;
            while (!dropped && m.next_span(t0, t1)) {
                for (double t = step * std::ceil(t0 / step); t <= t1; t += step) {
                    const V3 wp = g.index_to_world(r.at(t));
                    const double rho = std::min((double)g.sample_world(wp) * scale, sh->density_max);
                    if (rho < cutoff && sh->scatter_density_min < cutoff) continue;
                    const double x = std::max(rho, sh->scatter_density_min);
                    trans *= vexp(ext * (x * step));
                    s_sum += x * step;
                    if (trans.lengthSqr() < cutoff) {
                        trans = V3(0.0);
                        dropped = true;
                        break;
                    }
                }
            }
            if (T) {
                for (int c = 0; c < 3; ++c) {
                    T[((size_t)i * n + j) * 3 + c] = trans[c];
                    T[((size_t)j * n + i) * 3 + c] = trans[c];
                }
            }
            if (S) {
                const double v = dropped ? kInfD : s_sum;
                S[(size_t)i * n + j] = v;
                S[(size_t)j * n + i] = v;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// floydAlgo (src/LightGraph.h:512-542) and the min-plus forms
// ---------------------------------------------------------------------------
extern "C" void lgo_fw_maxtimes_rounds(int n, double* T, int k0, int k1) {
    for (int k = k0; k < k1 && k < n; ++k) {
        // row k and column k are not changed in round k (T_kk <= 1), so the
        // i loop can run in parallel without changing the result
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            const double* tik = T + ((size_t)i * n + k) * 3;
            if (!(tik[0] * tik[0] + tik[1] * tik[1] + tik[2] * tik[2] > 0)) continue;
            double* ti = T + (size_t)i * n * 3;
            const double* tk = T + (size_t)k * n * 3;
            const double a0 = tik[0], a1 = tik[1], a2 = tik[2];
            for (int j = 0; j < n; ++j) {
                const double* tkj = tk + 3 * j;
                if (!(tkj[0] * tkj[0] + tkj[1] * tkj[1] + tkj[2] * tkj[2] > 0)) continue;
                double* tij = ti + 3 * j;
                tij[0] = std::max(tij[0], a0 * tkj[0]);
                tij[1] = std::max(tij[1], a1 * tkj[1]);
                tij[2] = std::max(tij[2], a2 * tkj[2]);
            }
        }
    }
}

extern "C" void lgo_fw_maxtimes(int n, double* T) {
    lgo_fw_maxtimes_rounds(n, T, 0, n);
    for (int i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) T[((size_t)i * n + i) * 3 + c] = 1.0;
}

extern "C" void lgo_fw_minplus_f32(int n, float* S) {
    for (int k = 0; k < n; ++k) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            const float sik = S[(size_t)i * n + k];
            float* si = S + (size_t)i * n;
            const float* sk = S + (size_t)k * n;
            for (int j = 0; j < n; ++j) {
                const float v = sik + sk[j];
                if (v < si[j]) si[j] = v;
            }
        }
    }
}

extern "C" void lgo_fw_minplus_f64(int n, double* S) {
    for (int k = 0; k < n; ++k) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            const double sik = S[(size_t)i * n + k];
            double* si = S + (size_t)i * n;
            const double* sk = S + (size_t)k * n;
            for (int j = 0; j < n; ++j) {
                const double v = sik + sk[j];
                if (v < si[j]) si[j] = v;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// computeLighting (src/LightGraph.h:427-505)
// ---------------------------------------------------------------------------
extern "C" void lgo_vertex_light(const lgo_grid* dens, const lgo_grid* temp, const lg_shader* sh,
                                 const lg_settings* st, const lg_light* lights, int n_lights, const lgo_env* env,
                                 int n, const float* pts, int graph_id, double* L) {
    Grid g, tg;
    g.init(dens);
    if (temp) tg.init(temp);
    EnvDist ed;
    if (env && env->rgb) ed.build(env);
    const V3 ext = ext_of(sh), albedo = albedo_of(sh);
    const double step = st->step[1], cutoff = st->cutoff;
    const double scale = sh->density_scale * sh->shadow_density_scale * sh->scatter_density_scale;
#pragma omp parallel for schedule(dynamic, 8)
    for (int i = 0; i < n; ++i) {
        const V3 p(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
        V3 acc(0.0);
        const double ptemp = temp ? (double)tg.sample_world(p) : 0.0;
        const V3 emission = ramp(sh, ptemp) * sh->emission_scale;
        const Stream stream = make_stream(st->seed, kDomainVertex | ((uint64_t)graph_id << 32) | (uint32_t)i);
        for (int k = 0; k < n_lights; ++k) {
            const lg_light& Lk = lights[k];
            V3 lumi(0.0);
            uint64_t ns = (uint64_t)Lk.samples;
            if (ns > 1) ns *= 10;
            for (uint64_t s = 0; s < ns; ++s) {
                V3 ldir, I;
                double dist;
                if (Lk.type == LG_LIGHT_ENV) {
                    const uint32_t sub = shadow_key(stream, 0, (uint32_t)k, (uint32_t)s);
                    ed.illuminate(Lk, draw_sub(sub, kTagEnvU), draw_sub(sub, kTagEnvV), ldir, I);
                    dist = std::numeric_limits<double>::max();
                } else {
                    illuminate(Lk, p, ldir, I, dist);
                }
                IndexRay r = world_to_index(g, p, V3(-ldir.x, -ldir.y, -ldir.z), kDelta, dist);
                V3 trans(1.0);
                if (!clip(g, r)) continue;
                SpanMarch m(g, r);
                double t0, t1;
                bool dropped = false;
                while (!dropped && m.next_span(t0, t1)) {
                    for (double t = step * std::ceil(t0 / step); t <= t1; t += step) {
                        const double rho = std::min((double)g.sample_world(g.index_to_world(r.at(t))) * scale,
                                                    sh->density_max);
                        if (rho < cutoff) continue;
                        trans *= vexp(ext * (rho * step));
                        if (trans.lengthSqr() < cutoff) {
                            trans = V3(0.0);
                            dropped = true;
                            break;
                        }
                    }
                }
                lumi += I * trans;
            }
            acc += albedo * (lumi / (double)ns);
        }
        acc += emission;
        L[3 * i] = acc.x;
        L[3 * i + 1] = acc.y;
        L[3 * i + 2] = acc.z;
    }
}

// ---------------------------------------------------------------------------
// diffuseLight (src/LightGraph.h:554-587)
// ---------------------------------------------------------------------------
extern "C" void lgo_diffuse(int n, const double* T, const double* L, double* D) {
    std::vector<double> accum((size_t)n * 3);
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; ++j) {
        double a[3] = {0, 0, 0};
        for (int i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c) a[c] += T[((size_t)i * n + j) * 3 + c];
        for (int c = 0; c < 3; ++c) accum[3 * j + c] = std::max(a[c], 1.0);
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double d[3] = {0, 0, 0};
        for (int j = 0; j < n; ++j)
            for (int c = 0; c < 3; ++c) d[c] += L[3 * j + c] * (T[((size_t)i * n + j) * 3 + c] / accum[3 * j + c]);
        for (int c = 0; c < 3; ++c) D[3 * i + c] = d[c];
    }
}

// ---------------------------------------------------------------------------
// ScatterGrid (src/ScatterGrid.h:61-144)
// ---------------------------------------------------------------------------
static int floor_div(int a, int b) { return (a >= 0) ? a / b : -((-a + b - 1) / b); }

// points::computeVoxelSize(positions, pointsPerVoxel) as LightGraph::
// buildVdbPointGrid calls it (src/LightGraph.h:713-714; identity transform,
// five decimal places). OpenVDB is not under the reference tree and no version
// is pinned; this restates its documented procedure (OpenVDB 7/8,
// openvdb/points/PointConversion.h):
//  * 0.1 for fewer than two points or coincident points;
//  * target = max(1, n / pointsPerVoxel) voxels (integer division);
//  * start from the points' bounding box: voxel = float(pow(volume / target,
//    1/3)); a flat box uses maxExtent * nextExtent^2, a line maxExtent^3;
//  * refine: count the distinct voxels the points fall in (cell-centred index
//    round(p / voxel)), volume = float(voxel^3) * count; stop when the volume
//    does not shrink, when the count stops growing, or when the new voxel is
//    more than 0.9 of the last;
//  * round the result to five decimal places (six, seven, ... if that gives
//    zero): floor(v * 10^d + 0.5) / 10^d, stored as float.
// Returned as the double the point grid's transform reports.
namespace {
bool voxel_from_volume(double volume, size_t target, float& voxel) {
    const double vmin = 3e-15;  // ScaleMap's smallest voxel volume
    const double fmax = (double)std::numeric_limits<float>::max();
    const double vmax = fmax * fmax * fmax;
    double vv = volume / (double)target;
    bool ok = true;
    if (vv < vmin) {
        vv = vmin;
        ok = false;
    } else if (vv > vmax) {
        vv = vmax;
        ok = false;
    }
    voxel = (float)std::pow(vv, 1.0 / 3.0);
    return ok;
}
}  // namespace

extern "C" double lgo_point_voxel_size(int64_t n, const float* pts, int points_per_voxel) {
    float voxel = 0.1f;
    if (n <= 1 || points_per_voxel <= 0) return voxel;
    size_t target = (size_t)n / (size_t)points_per_voxel;
    if (target == 0) target = 1;
    double lo[3], hi[3];
    for (int a = 0; a < 3; ++a) lo[a] = hi[a] = (double)pts[a];
    for (int64_t i = 1; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], (double)pts[3 * i + a]);
            hi[a] = std::max(hi[a], (double)pts[3 * i + a]);
        }
    if (lo[0] == hi[0] && lo[1] == hi[1] && lo[2] == hi[2]) return voxel;
    double ext[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    double volume = ext[0] * ext[1] * ext[2];
    if (std::fabs(volume) <= 1e-15) {
        std::sort(ext, ext + 3);  // ascending: ext[2] largest
        if (std::fabs(ext[1]) <= 1e-15)
            volume = ext[2] * ext[2] * ext[2];
        else
            volume = ext[2] * ext[1] * ext[1];
    }
    double prev_volume = volume;
    if (!voxel_from_volume(volume, target, voxel)) return voxel;
    size_t prev_count = 0, count = 1;
    while (count > prev_count) {
        const double inv = 1.0 / (double)voxel;
        std::set<std::tuple<int, int, int>> cells;
        for (int64_t i = 0; i < n; ++i) {
            int c[3];
            for (int a = 0; a < 3; ++a) c[a] = (int)std::floor((double)pts[3 * i + a] * inv + 0.5);
            cells.insert(std::make_tuple(c[0], c[1], c[2]));
        }
        prev_count = count;
        count = cells.size();
        const float cube = voxel * voxel * voxel;
        volume = (double)(cube * (float)count);
        if (volume >= prev_volume) break;
        prev_volume = volume;
        const float prev_voxel = voxel;
        if (!voxel_from_volume(volume, target, voxel)) {
            voxel = prev_voxel;
            break;
        }
        if (voxel / prev_voxel > 0.9f) break;
    }
    float out = voxel;
    for (int d = 5; d < 11; ++d) {
        double tenth = 1.0;
        for (int k = 0; k < d; ++k) tenth *= 10.0;
        out = (float)(std::floor((double)voxel * tenth + 0.5) / tenth);
        if (out != 0.0f) break;
    }
    return (double)out;
}

extern "C" double lgo_splat(const lgo_grid* dens, int f, int64_t np, const float* pts, const double* D,
                            double hp, double K, int32_t out_lo[3], int32_t out_dims[3], double* out) {
    Grid g;
    g.init(dens);
    int lo[3], dims[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = floor_div(g.origin[a], f) - 1;
        const int hi = floor_div(g.origin[a] + g.dims[a] - 1, f) + 1;
        dims[a] = hi - lo[a] + 1;
        if (out_lo) out_lo[a] = lo[a];
        if (out_dims) out_dims[a] = dims[a];
    }
    const size_t total = (size_t)dims[0] * dims[1] * dims[2];
    // topology: coarse voxel c covers fine voxels f*c .. f*c+f-1; then dilate
    std::vector<uint8_t> act0(total, 0), act(total, 0);
#pragma omp parallel for schedule(static)
    for (int cz = 0; cz < dims[2]; ++cz)
        for (int cy = 0; cy < dims[1]; ++cy)
            for (int cx = 0; cx < dims[0]; ++cx) {
                bool any = false;
                for (int z = 0; z < f && !any; ++z)
                    for (int y = 0; y < f && !any; ++y)
                        for (int x = 0; x < f; ++x)
                            if (g.voxel((lo[0] + cx) * f + x, (lo[1] + cy) * f + y, (lo[2] + cz) * f + z) != 0.0f) {
                                any = true;
                                break;
                            }
                act0[((size_t)cz * dims[1] + cy) * dims[0] + cx] = any;
            }
#pragma omp parallel for schedule(static)
    for (int cz = 0; cz < dims[2]; ++cz)
        for (int cy = 0; cy < dims[1]; ++cy)
            for (int cx = 0; cx < dims[0]; ++cx) {
                bool any = false;
                for (int dz = -1; dz <= 1; ++dz)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dx = -1; dx <= 1; ++dx) {
                            const int x = cx + dx, y = cy + dy, z = cz + dz;
                            if (x < 0 || y < 0 || z < 0 || x >= dims[0] || y >= dims[1] || z >= dims[2]) continue;
                            any |= act0[((size_t)z * dims[1] + y) * dims[0] + x] != 0;
                        }
                act[((size_t)cz * dims[1] + cy) * dims[0] + cx] = any;
            }
    const double H = g.h * f;
    // src/ScatterGrid.h:69-75: voxelSizeCubed first, then the cube root by pow
    const double hp3 = hp * hp * hp;
    const double radius = std::pow((3.0 * K * hp3) / (32.0 * kPi), 1.0 / 3.0);
    const double sigma2 = -(radius * radius) / (2.0 * std::log(0.1));
    // uniform cells of edge `radius` over the points' bbox for the search
    double plo[3] = {0, 0, 0}, phi[3] = {0, 0, 0};
    if (np > 0) {
        for (int a = 0; a < 3; ++a) { plo[a] = 1e300; phi[a] = -1e300; }
        for (int64_t i = 0; i < np; ++i)
            for (int a = 0; a < 3; ++a) {
                plo[a] = std::min(plo[a], (double)pts[3 * i + a]);
                phi[a] = std::max(phi[a], (double)pts[3 * i + a]);
            }
    }
    double cell = std::max(radius, 1e-12), ext = 0;
    for (int a = 0; a < 3; ++a) ext = std::max(ext, phi[a] - plo[a]);
    if (ext / cell > 255.0) cell = ext / 255.0;
    int cd[3];
    for (int a = 0; a < 3; ++a) cd[a] = (int)std::floor((phi[a] - plo[a]) / cell) + 1;
    std::vector<std::vector<int64_t>> cells((size_t)cd[0] * cd[1] * cd[2]);
    auto cell_of = [&](double x, int a) {
        int c = (int)std::floor((x - plo[a]) / cell);
        return std::min(std::max(c, 0), cd[a] - 1);
    };
    for (int64_t i = 0; i < np; ++i) {
        const size_t c = ((size_t)cell_of(pts[3 * i + 2], 2) * cd[1] + cell_of(pts[3 * i + 1], 1)) * cd[0] +
                         cell_of(pts[3 * i], 0);
        cells[c].push_back(i);
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t idx = 0; idx < (int64_t)total; ++idx) {
        double* o = out + 3 * idx;
        o[0] = o[1] = o[2] = 0.0;
        if (!act[idx]) continue;
        const int cx = (int)(idx % dims[0]), cy = (int)((idx / dims[0]) % dims[1]),
                  cz = (int)(idx / ((int64_t)dims[0] * dims[1]));
        const V3 wpos((lo[0] + cx) * H, (lo[1] + cy) * H, (lo[2] + cz) * H);
        const int qx = (int)std::floor((wpos.x - plo[0]) / cell), qy = (int)std::floor((wpos.y - plo[1]) / cell),
                  qz = (int)std::floor((wpos.z - plo[2]) / cell);
        V3 sc(0.0);
        double tw = 0.0;
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int x = qx + dx, y = qy + dy, z = qz + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= cd[0] || y >= cd[1] || z >= cd[2]) continue;
                    for (int64_t p : cells[((size_t)z * cd[1] + y) * cd[0] + x]) {
                        // Vec3s diff = worldPos - point (float), lengthSqr in float
                        const float ex = (float)(wpos.x - pts[3 * p]), ey = (float)(wpos.y - pts[3 * p + 1]),
                                    ez = (float)(wpos.z - pts[3 * p + 2]);
                        const float d2 = ex * ex + ey * ey + ez * ez;
                        if (!((double)d2 < radius * radius)) continue;
                        const double w = std::exp(-(1.0 / (2.0 * sigma2)) * (double)d2);
                        tw += w;
                        sc += V3(D[3 * p], D[3 * p + 1], D[3 * p + 2]) * w;
                    }
                }
        if (tw > 0.0) sc = sc / tw;
        o[0] = sc.x;
        o[1] = sc.y;
        o[2] = sc.z;
    }
    return radius;
}

// ---------------------------------------------------------------------------
// VolumeRender::operator() (src/Renderer.h:505-693)
// ---------------------------------------------------------------------------
namespace {

void rotation3(int axis, double ang, double R[3][3]) {
    const double c = std::cos(ang), s = std::sin(ang);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R[i][j] = (i == j) ? 1.0 : 0.0;
    if (axis == 0) { R[1][1] = c; R[1][2] = s; R[2][1] = -s; R[2][2] = c; }
    else if (axis == 1) { R[0][0] = c; R[0][2] = -s; R[2][0] = s; R[2][2] = c; }
    else { R[0][0] = c; R[0][1] = s; R[1][0] = -s; R[1][1] = c; }
}

struct Camera {
    double M[3][3];
    V3 eye, cdir;
    double sw, sh, znear, zfar;
    int w, h;
    void init(const lg_camera& c) {
        const double d2r = kPi / 180.0;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) M[i][j] = (i == j);
        const double ang[3] = {c.rotate[0] * d2r, (c.rotate[1] + c.y_rotate) * d2r, c.rotate[2] * d2r};
        for (int a = 0; a < 3; ++a) {  // accumPostRotation: M <- M * rotation(axis, -angle)
            double R[3][3], T[3][3];
            rotation3(a, -ang[a], R);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) T[i][j] = M[i][0] * R[0][j] + M[i][1] * R[1][j] + M[i][2] * R[2][j];
            std::memcpy(M, T, sizeof T);
        }
        double Ry[3][3];
        rotation3(1, c.y_rotate * d2r, Ry);
        for (int j = 0; j < 3; ++j)
            eye[j] = c.translate[0] * Ry[0][j] + c.translate[1] * Ry[1][j] + c.translate[2] * Ry[2][j];
        for (int j = 0; j < 3; ++j) cdir[j] = -M[2][j];
        sw = 0.5 * c.aperture / c.focal;
        sh = sw * (double)c.height / (double)c.width;
        znear = c.znear;
        zfar = c.zfar;
        w = c.width;
        h = c.height;
    }
    V3 jac(const V3& v) const {
        V3 o;
        for (int j = 0; j < 3; ++j) o[j] = v[0] * M[0][j] + v[1] * M[1][j] + v[2] * M[2][j];
        return o;
    }
};

struct ScatterLookup {
    const float* v = nullptr;
    int lo[3] = {0, 0, 0}, dims[3] = {0, 0, 0};
    double H = 1.0;
    // trilinear Vec3f sample (GridSampler<Vec3fGrid, BoxSampler>)
    V3 sample(const V3& wp) const {
        V3 out(0.0);
        if (!v) return out;
        const double px = wp.x / H, py = wp.y / H, pz = wp.z / H;
        const double fx = std::floor(px), fy = std::floor(py), fz = std::floor(pz);
        const int ix = (int)fx - lo[0], iy = (int)fy - lo[1], iz = (int)fz - lo[2];
        const double u = px - fx, w = py - fy, t = pz - fz;
        for (int c = 0; c < 3; ++c) {
            float d[2][2][2];
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b)
                    for (int e = 0; e < 2; ++e) {
                        const int x = ix + a, y = iy + b, z = iz + e;
                        d[a][b][e] = (x < 0 || y < 0 || z < 0 || x >= dims[0] || y >= dims[1] || z >= dims[2])
                                         ? 0.0f
                                         : v[(((size_t)z * dims[1] + y) * dims[0] + x) * 3 + c];
                    }
            auto lerp = [](float a, float b, double wt) { return (float)(a + (float)((double)(b - a) * wt)); };
            out[c] = lerp(lerp(lerp(d[0][0][0], d[0][0][1], t), lerp(d[0][1][0], d[0][1][1], t), w),
                          lerp(lerp(d[1][0][0], d[1][0][1], t), lerp(d[1][1][0], d[1][1][1], t), w), u);
        }
        return out;
    }
};

}  // namespace

// VolumeRender::operator() over the pixels of the listed image rows, in
// parallel over pixels (the reference's TBB body runs over rows of a full
// frame; a pixel-level schedule keeps every thread busy when only a few rows
// are rendered). Results do not depend on the schedule: every random draw is
// keyed by pixel and sample.
static void render_rows(const lgo_grid* dens, const lgo_grid* temp, const lg_shader* sh, const lg_settings* st,
                        const lg_light* lights, int n_lights, const lgo_env* env, const lg_camera* cam_in,
                        const int32_t sg_lo[3], const int32_t sg_dims[3], double sg_h, const float* sg_values,
                        const int32_t* rows, int n_rows, float* rgba, float* direct, float* scatter,
                        float* emission, uint64_t* counters) {
    Grid g, tg;
    g.init(dens);
    if (temp) tg.init(temp);
    EnvDist ed;
    if (env && env->rgb) ed.build(env);
    Camera cam;
    cam.init(*cam_in);
    ScatterLookup sl;
    if (sg_values) {
        sl.v = sg_values;
        for (int a = 0; a < 3; ++a) { sl.lo[a] = sg_lo[a]; sl.dims[a] = sg_dims[a]; }
        sl.H = sg_h;
    }
    const V3 ext = ext_of(sh), albedo = albedo_of(sh), One(1.0);
    const V3 inv_scatter(1.0 / sh->scattering[0], 1.0 / sh->scattering[1], 1.0 / sh->scattering[2]);
    const double step0 = st->step[0], step1 = st->step[1], cutoff = st->cutoff, jit = 0.5;
    const int spp = cam_in->samples;
    uint64_t cnt_p = 0, cnt_s = 0;
    const int64_t n_pix = (int64_t)n_rows * cam.w;
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : cnt_p, cnt_s)
    for (int64_t q = 0; q < n_pix; ++q) {
        {
            const int j = rows[q / cam.w], i = (int)(q % cam.w);
            const int64_t pix = (int64_t)j * cam.w + i;
            V3 pTransAA(0.0), pLumiAA(0.0), dirAA(0.0), scatAA(0.0), emitAA(0.0);
            const double ratioAA = 1.0 / (double)spp;
            for (int s = 0; s < spp; ++s) {
                const Stream stream = make_stream(st->seed, kDomainPixel | (uint64_t)(pix * spp + s));
                // PerspectiveCamera::getRay with offset 0.5 + (u - 0.5)
                const double jx = (double)draw(stream, kTagJitterX), jy = (double)draw(stream, kTagJitterY);
                V3 dir((2.0 * ((double)i + jx) / (double)cam.w - 1.0) * cam.sw,
                       (1.0 - 2.0 * ((double)j + jy) / (double)cam.h) * cam.sh, -1.0);
                dir = cam.jac(dir);
                dir = dir / std::sqrt(dir.lengthSqr());
                const double tscale = 1.0 / dir.dot(cam.cdir);
                IndexRay pr = world_to_index(g, cam.eye, dir, cam.znear * tscale, cam.zfar * tscale);
                V3 pTrans(1.0);
                if (!clip(g, pr)) {
                    pTransAA += pTrans * ratioAA;
                    continue;
                }
                V3 pLumi(0.0), directLumi(0.0), scatterLumi(0.0), emitLumi(0.0);
                SpanMarch pm(g, pr);
                double pT0, pT1;
                uint32_t span_ord = 0, n_iter = 0;
                uint32_t pj = hash32(stream.a ^ (stream.b + kTagPrimaryStep * 0x9E3779B9u));
                bool pDropout = false;
                while (!pDropout && pm.next_span(pT0, pT1)) {
                    double pStep = step0 * (1.0 + ((double)draw(stream, kTagPrimarySpan | span_ord) - 0.5) * jit);
                    ++span_ord;
                    for (double pT = step0 * std::ceil(pT0 / step0); pT <= pT1; pT += pStep) {
                        const uint32_t n = n_iter++;
                        pj = step_next(pj);
                        ++cnt_p;
                        const V3 pPos = g.index_to_world(pr.at(pT));
                        const double pDensity = std::min((double)g.sample_world(pPos) * sh->density_scale,
                                                         sh->density_max);
                        if (pDensity < cutoff) continue;
                        const V3 pScatter = sl.sample(pPos);
                        const V3 scat = pScatter * inv_scatter *
                                        (std::pow(std::min(std::max(pDensity, 0.0), 1.0), sh->scatter_density_mask_power) *
                                         sh->scatter_scale);
                        const double pTemp = temp ? (double)tg.sample_world(pPos) : 0.0;
                        const V3 emis = ramp(sh, pTemp) * sh->emission_scale;
                        const V3 dT = vexp(ext * (pDensity * pStep));
                        for (int k = 0; k < n_lights; ++k) {
                            const lg_light& Lk = lights[k];
                            V3 tmpLumi(0.0);
                            for (int ls = 0; ls < Lk.samples; ++ls) {
                                const uint32_t sub = shadow_key(stream, n, (uint32_t)k, (uint32_t)ls);
                                V3 sTrans(1.0), ldir, I;
                                double dist;
                                if (Lk.type == LG_LIGHT_ENV) {
                                    ed.illuminate(Lk, draw_sub(sub, kTagEnvU), draw_sub(sub, kTagEnvV), ldir, I);
                                    dist = std::numeric_limits<double>::max();
                                } else {
                                    illuminate(Lk, pPos, ldir, I, dist);
                                }
                                IndexRay sr = world_to_index(g, pPos, V3(-ldir.x, -ldir.y, -ldir.z), kDelta, dist);
                                if (!clip(g, sr)) continue;
                                SpanMarch sm(g, sr);
                                double sT0, sT1;
                                uint32_t sspan = 0, siter = 0;
                                uint32_t sj = hash32(sub ^ kTagShadowStep);
                                bool sDropout = false;
                                while (!sDropout && sm.next_span(sT0, sT1)) {
                                    double sStep = step1 * (1.0 + ((double)draw_sub(sub, kTagShadowSpan | sspan) - 0.5) * jit);
                                    ++sspan;
                                    for (double sT = step1 * std::ceil(sT0 / step1); sT <= sT1; sT += sStep) {
                                        ++siter;
                                        sj = step_next(sj);
                                        const double sDensity =
                                            std::min((double)g.sample_world(g.index_to_world(sr.at(sT))) *
                                                         sh->density_scale * sh->shadow_density_scale,
                                                     sh->density_max);
                                        if (sDensity < cutoff) continue;
                                        sTrans *= vexp(ext * (sDensity * sStep));
                                        if (sTrans.lengthSqr() < cutoff) {
                                            sTrans = V3(0.0);
                                            sDropout = true;
                                            break;
                                        }
                                        sStep = step1 * (1.0 + (step_u(sj) - 0.5) * jit);
                                    }
                                }
                                cnt_s += siter;
                                tmpLumi += I * sTrans;
                            }
                            const V3 tmpDirect = albedo * (tmpLumi / (double)Lk.samples) * pTrans * (One - dT);
                            pLumi += tmpDirect;
                            directLumi += tmpDirect;
                        }
                        const V3 tmpScatter = scat * pTrans * (One - dT);
                        const V3 tmpEmit = emis * pTrans * (One - dT);
                        scatterLumi += tmpScatter;
                        emitLumi += tmpEmit;
                        pLumi += tmpScatter + tmpEmit;
                        pTrans *= dT;
                        if (pTrans.lengthSqr() < cutoff) {
                            pDropout = true;
                            break;
                        }
                        pStep = step0 * (1.0 + (step_u(pj) - 0.5) * jit);
                    }
                }
                pLumiAA += pLumi * ratioAA;
                dirAA += directLumi * ratioAA;
                scatAA += scatterLumi * ratioAA;
                emitAA += emitLumi * ratioAA;
                pTransAA += pTrans * ratioAA;
            }
            const size_t o = (size_t)pix * 4;
            if (rgba) {
                rgba[o] = (float)pLumiAA.x;
                rgba[o + 1] = (float)pLumiAA.y;
                rgba[o + 2] = (float)pLumiAA.z;
                rgba[o + 3] = (float)(1.0f - (pTransAA.x + pTransAA.y + pTransAA.z) / 3.0f);
            }
            if (direct) { direct[o] = (float)dirAA.x; direct[o + 1] = (float)dirAA.y; direct[o + 2] = (float)dirAA.z; direct[o + 3] = 0.f; }
            if (scatter) { scatter[o] = (float)scatAA.x; scatter[o + 1] = (float)scatAA.y; scatter[o + 2] = (float)scatAA.z; scatter[o + 3] = 0.f; }
            if (emission) { emission[o] = (float)emitAA.x; emission[o + 1] = (float)emitAA.y; emission[o + 2] = (float)emitAA.z; emission[o + 3] = 0.f; }
        }
    }
    if (counters) {
        counters[0] = cnt_p;
        counters[1] = cnt_s;
    }
}

extern "C" void lgo_render(const lgo_grid* dens, const lgo_grid* temp, const lg_shader* sh, const lg_settings* st,
                           const lg_light* lights, int n_lights, const lgo_env* env, const lg_camera* cam,
                           const int32_t sg_lo[3], const int32_t sg_dims[3], double sg_h, const float* sg_values,
                           int row0, int row1, float* rgba, float* direct, float* scatter, float* emission,
                           uint64_t* counters) {
    std::vector<int32_t> rows;
    for (int j = std::max(row0, 0); j < row1 && j < cam->height; ++j) rows.push_back(j);
    render_rows(dens, temp, sh, st, lights, n_lights, env, cam, sg_lo, sg_dims, sg_h, sg_values, rows.data(),
                (int)rows.size(), rgba, direct, scatter, emission, counters);
}

extern "C" void lgo_render_rows(const lgo_grid* dens, const lgo_grid* temp, const lg_shader* sh,
                                const lg_settings* st, const lg_light* lights, int n_lights, const lgo_env* env,
                                const lg_camera* cam, const int32_t sg_lo[3], const int32_t sg_dims[3], double sg_h,
                                const float* sg_values, const int32_t* rows, int n_rows, float* rgba, float* direct,
                                float* scatter, float* emission, uint64_t* counters) {
    render_rows(dens, temp, sh, st, lights, n_lights, env, cam, sg_lo, sg_dims, sg_h, sg_values, rows, n_rows, rgba,
                direct, scatter, emission, counters);
}

extern "C" void lgo_fw_minplus_f32_rounds(int n, float* S, int k0, int k1) {
    for (int k = k0; k < k1 && k < n; ++k) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            const float sik = S[(size_t)i * n + k];
            if (!(sik < std::numeric_limits<float>::infinity())) continue;
            float* si = S + (size_t)i * n;
            const float* sk = S + (size_t)k * n;
            for (int j = 0; j < n; ++j) {
                const float v = sik + sk[j];
                if (v < si[j]) si[j] = v;
            }
        }
    }
}

extern "C" void lgo_transmittance_of(int64_t count, const double* S, const double ext[3], double* T) {
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < count; ++e) {
        const double v = S[e];
        for (int c = 0; c < 3; ++c) T[3 * e + c] = v < std::numeric_limits<double>::infinity() ? std::exp(ext[c] * v) : 0.0;
    }
}

extern "C" void lgo_env_cdf(const lgo_env* env, float* cond_func, float* cond_cdf, float* cond_int, float* marg_func,
                            float* marg_cdf, float* marg_int) {
    EnvDist ed;
    ed.build(env);
    for (int v = 0; v < ed.h; ++v) {
        std::copy(ed.cond[v].func.begin(), ed.cond[v].func.end(), cond_func + (size_t)v * ed.w);
        std::copy(ed.cond[v].cdf.begin(), ed.cond[v].cdf.end(), cond_cdf + (size_t)v * (ed.w + 1));
        cond_int[v] = ed.cond[v].funcInt;
    }
    std::copy(ed.marg.func.begin(), ed.marg.func.end(), marg_func);
    std::copy(ed.marg.cdf.begin(), ed.marg.cdf.end(), marg_cdf);
    *marg_int = ed.marg.funcInt;
}

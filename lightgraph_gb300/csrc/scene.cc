// Seeded synthetic scene inputs (volumes, point sets, environment map).
// See include/lightgraph_scene.h. Compiled with -ffp-contract=off so that the
// x86-64 container and the aarch64 GPU host generate bit-identical inputs.
#include "lightgraph_scene.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Lattice value in [-1, 1] for integer point (x, y, z) of octave o.
inline double lattice(int64_t x, int64_t y, int64_t z, int o, uint64_t seed) {
    uint64_t h = splitmix64(seed ^ 0xA5A5A5A5ull);
    h = splitmix64(h ^ (uint64_t)(x * 73856093ll));
    h = splitmix64(h ^ (uint64_t)(y * 19349663ll));
    h = splitmix64(h ^ (uint64_t)(z * 83492791ll));
    h = splitmix64(h ^ (uint64_t)o);
    return (double)(h >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

inline double fade(double t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); }

// Value noise with quintic fade, range about [-1, 1].
double vnoise(double px, double py, double pz, int o, uint64_t seed) {
    double fx = std::floor(px), fy = std::floor(py), fz = std::floor(pz);
    int64_t ix = (int64_t)fx, iy = (int64_t)fy, iz = (int64_t)fz;
    double ux = fade(px - fx), uy = fade(py - fy), uz = fade(pz - fz);
    double c[2][2][2];
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx)
                c[dz][dy][dx] = lattice(ix + dx, iy + dy, iz + dz, o, seed);
    double x00 = c[0][0][0] + (c[0][0][1] - c[0][0][0]) * ux;
    double x10 = c[0][1][0] + (c[0][1][1] - c[0][1][0]) * ux;
    double x01 = c[1][0][0] + (c[1][0][1] - c[1][0][0]) * ux;
    double x11 = c[1][1][0] + (c[1][1][1] - c[1][1][0]) * ux;
    double y0 = x00 + (x10 - x00) * uy;
    double y1 = x01 + (x11 - x01) * uy;
    return y0 + (y1 - y0) * uz;
}

// Normalised fBm: sum of octaves with gain 1/2 and lacunarity 2, divided by
// the amplitude sum so the result stays in about [-1, 1].
double fbm(double x, double y, double z, int octaves, uint64_t seed) {
    double sum = 0.0, amp = 1.0, norm = 0.0, f = 1.0;
    for (int o = 0; o < octaves; ++o) {
        sum += amp * vnoise(x * f, y * f, z * f, o, seed);
        norm += amp;
        amp *= 0.5;
        f *= 2.0;
    }
    return sum / norm;
}

inline double clamp01(double v) { return v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v); }

inline double smoothstep(double a, double b, double x) {
    double t = clamp01((x - a) / (b - a));
    return t * t * (3.0 - 2.0 * t);
}

struct Puff { double cx, cy, cz, r; };

// Cumulus puffs: a base row of wide puffs and a crown of smaller ones, placed
// from the seed around the centre of the unit box.
std::vector<Puff> make_puffs(uint64_t seed) {
    std::vector<Puff> p;
    uint64_t s = splitmix64(seed ^ 0xC0FFEEull);
    auto u01 = [&]() { s = splitmix64(s); return (double)(s >> 11) / 9007199254740992.0; };
    auto sym = [&]() { return 2.0 * u01() - 1.0; };
    p.push_back({0.50, 0.46, 0.50, 0.20});
    for (int k = 0; k < 6; ++k) {
        p.push_back({0.5 + 0.20 * sym(), 0.40 + 0.05 * u01(), 0.5 + 0.20 * sym(),
                     0.12 + 0.05 * u01()});
    }
    for (int k = 0; k < 4; ++k) {
        p.push_back({0.5 + 0.09 * sym(), 0.58 + 0.06 * u01(), 0.5 + 0.09 * sym(),
                     0.10 + 0.04 * u01()});
    }
    return p;
}

}  // namespace

extern "C" int64_t lgs_volume(int kind, int res, int octaves, uint64_t seed, double scale,
                              const float* mask, float* out) {
    if (res <= 0 || !out) return -1;
    const int64_t n = (int64_t)res * res * res;
    std::vector<Puff> puffs;
    if (kind == LGS_VOLUME_CUMULUS) puffs = make_puffs(seed);
    int64_t nonzero = 0;
#pragma omp parallel for schedule(static) reduction(+ : nonzero)
    for (int z = 0; z < res; ++z) {
        for (int y = 0; y < res; ++y) {
            for (int x = 0; x < res; ++x) {
                const int64_t idx = ((int64_t)z * res + y) * res + x;
                // unit-box coordinates of the voxel centre
                const double ux = (x + 0.5) / res, uy = (y + 0.5) / res, uz = (z + 0.5) / res;
                double v = 0.0;
                if (kind == LGS_VOLUME_SPHERE_FBM) {
                    const double dx = ux - 0.5, dy = uy - 0.5, dz = uz - 0.5;
                    if (dx * dx + dy * dy + dz * dz < 0.4 * 0.4) {
                        v = clamp01(0.5 + fbm(ux * 4.0, uy * 4.0, uz * 4.0, octaves, seed));
                    }
                } else if (kind == LGS_VOLUME_CUMULUS) {
                    double f = -1.0;
                    for (const Puff& p : puffs) {
                        const double dx = ux - p.cx, dy = (uy - p.cy) * 1.3, dz = uz - p.cz;
                        const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
                        const double g = 1.0 - d / (p.r * 1.45);
                        if (g > f) f = g;
                    }
                    if (f > -0.6) {
                        const double base = smoothstep(0.27, 0.31, uy);
                        const double n6 = fbm(ux * 6.0, uy * 6.0, uz * 6.0, octaves, seed);
                        v = clamp01((f + 0.45 * n6) * 3.0) * base;
                        if (v < 1e-3) v = 0.0;
                    }
                } else if (kind == LGS_VOLUME_TEMPERATURE) {
                    if (!mask || mask[idx] > 0.0f) {
                        v = clamp01(0.5 + 0.8 * fbm(ux * 3.0, uy * 3.0, uz * 3.0, octaves, seed));
                    }
                }
                const float fv = (float)(v * scale);
                out[idx] = fv;
                if (fv != 0.0f) ++nonzero;
            }
        }
    }
    return nonzero;
}

namespace {

// Trilinear density at an index-space position of the res^3 box whose first
// voxel has index -res/2 (background 0 outside), in the order z, y, x of the
// reference's BoxSampler.
double sample_box(const float* v, int res, double ix, double iy, double iz) {
    const int lo = -res / 2;
    double fx = std::floor(ix), fy = std::floor(iy), fz = std::floor(iz);
    int x0 = (int)fx - lo, y0 = (int)fy - lo, z0 = (int)fz - lo;
    double wx = ix - fx, wy = iy - fy, wz = iz - fz;
    auto at = [&](int x, int y, int z) -> double {
        if (x < 0 || y < 0 || z < 0 || x >= res || y >= res || z >= res) return 0.0;
        return v[((int64_t)z * res + y) * res + x];
    };
    double d[2][2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 2; ++c) d[a][b][c] = at(x0 + a, y0 + b, z0 + c);
    auto lerp = [](double a, double b, double w) { return a + (b - a) * w; };
    return lerp(lerp(lerp(d[0][0][0], d[0][0][1], wz), lerp(d[0][1][0], d[0][1][1], wz), wy),
                lerp(lerp(d[1][0][0], d[1][0][1], wz), lerp(d[1][1][0], d[1][1][1], wz), wy), wx);
}

}  // namespace

extern "C" int64_t lgs_points(const float* density, int res, double voxel_size, int64_t n,
                              uint64_t seed, double min_density, int64_t max_tries, float* out) {
    if (!density || !out || res <= 0 || n < 0 || voxel_size <= 0) return -1;
    const int lo = -res / 2;
    // active voxel bbox (evalActiveVoxelBoundingBox, src/main.cc:512)
    int bmin[3] = {res, res, res}, bmax[3] = {-1, -1, -1};
    for (int z = 0; z < res; ++z)
        for (int y = 0; y < res; ++y)
            for (int x = 0; x < res; ++x) {
                if (density[((int64_t)z * res + y) * res + x] != 0.0f) {
                    if (x < bmin[0]) bmin[0] = x;
                    if (y < bmin[1]) bmin[1] = y;
                    if (z < bmin[2]) bmin[2] = z;
                    if (x > bmax[0]) bmax[0] = x;
                    if (y > bmax[1]) bmax[1] = y;
                    if (z > bmax[2]) bmax[2] = z;
                }
            }
    if (bmax[0] < 0) return 0;
    double wmin[3], wsize[3];
    for (int a = 0; a < 3; ++a) {
        wmin[a] = (bmin[a] + lo) * voxel_size;
        wsize[a] = (bmax[a] - bmin[a]) * voxel_size;
    }
    uint64_t s = splitmix64(seed ^ 0x5EED5EEDull);
    int64_t got = 0;
    for (int64_t t = 0; t < max_tries && got < n; ++t) {
        float p[3];
        for (int a = 0; a < 3; ++a) {
            s = splitmix64(s);
            const float u = (float)(s >> 40) * (1.0f / 16777216.0f);
            p[a] = (float)(u * wsize[a] + wmin[a]);
        }
        const double rho = sample_box(density, res, p[0] / voxel_size, p[1] / voxel_size,
                                      p[2] / voxel_size);
        if (rho < min_density) continue;
        out[3 * got + 0] = p[0];
        out[3 * got + 1] = p[1];
        out[3 * got + 2] = p[2];
        ++got;
    }
    return got;
}

namespace {

// Round to the nearest half-precision value (round-to-nearest-even), keeping
// the result in float. Values beyond the half range saturate to 65504.
float round_half(float f) {
    if (!(f == f)) return f;
    float a = std::fabs(f);
    if (a >= 65520.0f) return f < 0 ? -65504.0f : 65504.0f;
    if (a < 6.103515625e-05f) {  // subnormal half: spacing 2^-24
        const float q = 5.9604644775390625e-08f;
        return std::nearbyint(f / q) * q;
    }
    int e;
    std::frexp(a, &e);                 // a = m * 2^e, m in [0.5, 1)
    const float q = std::ldexp(1.0f, e - 11);  // 11 significant bits
    return std::nearbyint(f / q) * q;
}

}  // namespace

extern "C" void lgs_envmap(int w, int h, double sun_elev_deg, double sun_azim_deg,
                           double sun_sigma_deg, double sun_intensity, float* out) {
    if (!out || w <= 0 || h <= 0) return;
    const double pi = 3.14159265358979323846;
    const double se = sun_elev_deg * pi / 180.0, sa = sun_azim_deg * pi / 180.0;
    // direction convention of EnvLight::illuminate (src/Light.h:201-209):
    // theta = u * 2pi around y, phi = v * pi from +y
    const double sphi = pi / 2 - se;
    const double sun[3] = {std::cos(sa) * std::sin(sphi), std::cos(sphi), std::sin(sa) * std::sin(sphi)};
    const double sig = sun_sigma_deg * pi / 180.0;
    for (int r = 0; r < h; ++r) {
        const double phi = (r + 0.5) / h * pi;
        for (int c = 0; c < w; ++c) {
            const double theta = (c + 0.5) / w * 2.0 * pi;
            const double d[3] = {std::cos(theta) * std::sin(phi), std::cos(phi), std::sin(theta) * std::sin(phi)};
            const double elev = pi / 2 - phi;
            double rgb[3];
            if (elev >= 0) {
                const double t = elev / (pi / 2);  // 0 at horizon, 1 at zenith
                rgb[0] = 0.85 - 0.55 * t;
                rgb[1] = 0.90 - 0.40 * t;
                rgb[2] = 1.00 - 0.10 * t;
            } else {
                rgb[0] = 0.12;
                rgb[1] = 0.11;
                rgb[2] = 0.10;
            }
            double cosang = d[0] * sun[0] + d[1] * sun[1] + d[2] * sun[2];
            if (cosang > 1.0) cosang = 1.0;
            if (cosang < -1.0) cosang = -1.0;
            const double ang = std::acos(cosang);
            const double lobe = sun_intensity * std::exp(-(ang * ang) / (2.0 * sig * sig));
            const double sunc[3] = {1.0, 0.92, 0.80};
            for (int k = 0; k < 3; ++k) {
                out[((int64_t)r * w + c) * 3 + k] = round_half((float)(rgb[k] + lobe * sunc[k]));
            }
        }
    }
}

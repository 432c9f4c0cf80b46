// Camera ray march writing the beauty and AOV films:
// VolumeRender::operator() (src/Renderer.h:505-693) with
// PerspectiveCamera::getRay (src/Renderer.h:216-229).
//
// The reference marches, per pixel and antialiasing sample, a jittered primary
// ray at step[0] (+-25% jittered step) through the density's leaf spans and, at
// every sample with density >= cutoff, one jittered shadow march per light
// sample. The primary march never depends on the shadow results (only the
// accumulated radiance does), so the work is split into waves:
//   k_primary<false> : march the primary rays, count the samples that shade;
//   (exclusive scan of the counts)
//   k_primary<true>  : march again, accumulate the scatter and emission AOVs
//                      and write one shadow task per shading sample
//                      (position, pTrans * (1 - dT), stream words), and the
//                      light-space order key of each pair of tasks per light
//                      with a count per key;
//   (exclusive scan of the key counts)
//   k_ray_scatter    : order each light's shadow rays by their keys (the
//                      counting sort's scatter), so the rays in flight are
//                      neighbouring, parallel rays;
//   k_shadow         : one thread per (light, ordered pair of tasks) marches
//                      that light's shadow rays (all its samples) and writes
//                      the light's contribution to the task's slot;
//   k_resolve        : per pixel, sums the tasks and lights in order and
//                      writes the films.
// Shadow rays accumulate a scalar optical depth (every channel of the
// reference's product of exponentials is exp(-a_c * tau)) and stop when tau
// passes the dropout depth. Random numbers come from counter-based streams
// keyed by (seed, pixel, sample, loop iteration), so results do not depend on
// the launch shape; the reference's render RNG depends on TBB's row split.
#include <atomic>

#include <cooperative_groups.h>

#include "lg_kernels.h"

namespace lg {

namespace cg = cooperative_groups;

// Trilinear Vec3 sample of the coarse scatter grid (0 outside the box). A
// footprint wholly inside the box (the common case) loads its eight corners
// from one base index; one that reaches past a face tests every corner. The
// lerps run the R and G channels as one packed pair (the same rounding per
// channel as fmaf(b - a, w, a)).
__device__ __forceinline__ void sample_scatter(const DevScatterGrid& sg, float wx, float wy, float wz,
                                               float out[3]) {
    const float px = wx * sg.inv_H, py = wy * sg.inv_H, pz = wz * sg.inv_H;
    const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    const int ix = (int)fx - sg.lo[0], iy = (int)fy - sg.lo[1], iz = (int)fz - sg.lo[2];
    const float u = px - fx, v = py - fy, w = pz - fz;
    float4 c[2][2][2];
    if ((unsigned)ix < (unsigned)max(sg.dims[0] - 1, 0) && (unsigned)iy < (unsigned)max(sg.dims[1] - 1, 0) &&
        (unsigned)iz < (unsigned)max(sg.dims[2] - 1, 0)) {
        const int64_t sy = sg.dims[0], sz = (int64_t)sg.dims[0] * sg.dims[1];
        const float4* b = sg.v + ((int64_t)iz * sz + (int64_t)iy * sy + ix);
#pragma unroll
        for (int d = 0; d < 2; ++d)
#pragma unroll
            for (int bb = 0; bb < 2; ++bb) {
                const float4* row = b + d * sz + bb * sy;
                c[0][bb][d] = __ldg(row);
                c[1][bb][d] = __ldg(row + 1);
            }
    } else {
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int bb = 0; bb < 2; ++bb)
#pragma unroll
                for (int d = 0; d < 2; ++d) {
                    const int x = ix + a, y = iy + bb, z = iz + d;
                    if ((unsigned)x < (unsigned)sg.dims[0] && (unsigned)y < (unsigned)sg.dims[1] &&
                        (unsigned)z < (unsigned)sg.dims[2])
                        c[a][bb][d] = __ldg(sg.v + ((int64_t)z * sg.dims[1] + y) * sg.dims[0] + x);
                    else
                        c[a][bb][d] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
    }
    auto l = [](float4 p, float4 q, float t) {
        const float2 rg = __ffma2_rn(__fadd2_rn(make_float2(q.x, q.y), make_float2(-p.x, -p.y)), make_float2(t, t),
                                     make_float2(p.x, p.y));
        return make_float4(rg.x, rg.y, lerpf(p.z, q.z, t), 0.f);
    };
    const float4 r = l(l(l(c[0][0][0], c[0][0][1], w), l(c[0][1][0], c[0][1][1], w), v),
                       l(l(c[1][0][0], c[1][0][1], w), l(c[1][1][0], c[1][1][1], w), v), u);
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
}

__device__ __forceinline__ float jitter_step(float step, float u) { return step * (1.f + (u - 0.5f) * 0.5f); }

// jitter_step with u = (x >> 9) / 2^23 from a step-jitter stream state:
// 1 + u is built from the bits directly, so (u - 0.5) = (1 + u) - 1.5 exactly.
__device__ __forceinline__ float jitter_step_bits(float step, uint32_t x) {
    const float f = __uint_as_float(0x3F800000u | (x >> 9));
    // rounding spelled out (no contraction into the caller's additions): the
    // two primary passes must step identically
    return __fmul_rn(step, __fmaf_rn(__fsub_rn(f, 1.5f), 0.5f, 1.f));
}

// The same jittered step for the shadow rays in one rounding:
// step * (0.75 + 0.5 u) = fma(1 + u, step / 2, step / 4), half = step / 2 and
// quarter = step / 4 (both exact).
__device__ __forceinline__ float jitter_step_fma(float half, float quarter, uint32_t x) {
    return __fmaf_rn(__uint_as_float(0x3F800000u | (x >> 9)), half, quarter);
}

// Light::illuminate for the shadow rays: the point light's distance and
// direction from one approximate reciprocal square root and its falloff from
// one approximate reciprocal (within a few ulp of illuminate's IEEE forms).
__device__ __forceinline__ void illuminate_shadow(const DevLight& L, const float p[3], float dir[3], float I[3],
                                                  float& dist) {
    if (L.type == 1) {
        const float d[3] = {p[0] - L.pos[0], p[1] - L.pos[1], p[2] - L.pos[2]};
        const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const float ri = rsqrtf(r2);
        dist = r2 > 0.f ? r2 * ri : 0.f;
        const float fall = __fdividef(1.f, 1.f + 4.f * 3.14159265358979323846f * r2);
#pragma unroll
        for (int c = 0; c < 3; ++c) { dir[c] = d[c] * ri; I[c] = L.I[c] * fall; }
    } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) { dir[c] = L.dir[c]; I[c] = L.I[c]; }
        dist = kInf;
    }
}

// make_iray with approximate reciprocals of the direction (exact at +-0,
// where they give +-inf like the IEEE quotient).
__device__ __forceinline__ void make_iray_approx(IRay& r, float ex, float ey, float ez, float dx, float dy, float dz,
                                                 float t0, float t1) {
    r.e[0] = ex; r.e[1] = ey; r.e[2] = ez;
    r.d[0] = dx; r.d[1] = dy; r.d[2] = dz;
    r.inv[0] = __fdividef(1.f, dx); r.inv[1] = __fdividef(1.f, dy); r.inv[2] = __fdividef(1.f, dz);
    r.t0 = t0; r.t1 = t1;
}

// clip_to_bbox without branches: the same slab times per axis, t0 raised to
// the near one and t1 lowered to the far one, the test once at the end (t0
// only grows and t1 only shrinks, so it fails there exactly when it fails
// after some axis). A NaN slab time (a zero direction component starting on
// a slab plane) leaves its bound alone, as the slab test's comparisons do.
__device__ __forceinline__ bool clip_to_bbox_flat(const DevGrid& g, IRay& r) {
    float t0 = r.t0, t1 = r.t1;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float a = (g.bbmin[i] - r.e[i]) * r.inv[i];
        const float b = (g.bbmax[i] - r.e[i]) * r.inv[i];
        const bool sw = a > b;
        t0 = fmaxf(t0, sw ? b : a);
        t1 = fminf(t1, sw ? a : b);
    }
    r.t0 = t0;
    r.t1 = t1;
    return g.has_leaves && t0 <= t1;
}

// dda_axis from the floor bits of the start coordinate (|p| < 2^22, which
// the grid upload guarantees): the same cell and first crossing, since the
// bits with their low three cleared are ca * 8 (plus the bias). bias =
// 0x4B400000 / 8 + blo - 1 turns bits >> 3 into the bitmap coordinate.
__device__ __forceinline__ int dda_axis_bits(float e, float d, float inv, float t0, uint32_t bias, int& step,
                                             float& next, float& delta) {
    const float p = __fmaf_rn(t0, d, e);
    float fl;
    const uint32_t bits = floor_bits(p, fl);
    const float c8 = __fsub_rn(__uint_as_float(bits & ~7u), 12582912.0f);  // ca * 8
    const bool up = inv > 0.f;
    const float plane = up ? __fadd_rn(c8, 8.f) : c8;
    step = d == 0.f ? 0 : (up ? 1 : -1);
    next = d == 0.f ? kInf : __fmaf_rn(__fsub_rn(plane, p), inv, t0);
    delta = d == 0.f ? kInf : 8.f * fabsf(inv);
    return (int)((bits >> 3) - bias);
}

// dda_init over dda_axis_bits.
__device__ __forceinline__ void dda_init_bits(LeafDDA& s, const IRay& r, const DevGrid& g) {
    s.t = r.t0;
    s.tmax = r.t1;
    s.done = false;
    s.open = false;
    s.start = 0.f;
    constexpr uint32_t b8 = 0x4B400000u >> 3;
    int sx, sy, sz;
    const int cx = dda_axis_bits(r.e[0], r.d[0], r.inv[0], r.t0, b8 + (uint32_t)g.blo[0] - 1u, sx, s.nx, s.dx);
    const int cy = dda_axis_bits(r.e[1], r.d[1], r.inv[1], r.t0, b8 + (uint32_t)g.blo[1] - 1u, sy, s.ny, s.dy);
    const int cz = dda_axis_bits(r.e[2], r.d[2], r.inv[2], r.t0, b8 + (uint32_t)g.blo[2] - 1u, sz, s.nz, s.dz);
    const bool in = (unsigned)cx < (unsigned)g.lbx && (unsigned)cy < (unsigned)g.lby &&
                    (unsigned)cz < (unsigned)(g.nb[2] + 2);
    s.lin = in ? cz * g.lbxy + cy * g.lbx + cx : (int)g.nbits;
    s.ix = sx;
    s.iy = sy * g.lbx;
    s.iz = sz * g.lbxy;
}

// e^x - 1 for the primary wave's transmittance steps: for |x| < 1/16 the
// Taylor series x + x^2/2! + ... + x^6/6! (the next term is below 2^-30 of
// the result), beyond it __expf(x) - 1 (a few ulp of e^x, which at |x| = 1/16
// is a relative error of about 2e-6 of the result). lg_expm1_check measures
// it against the library's expm1f.
__device__ __forceinline__ float expm1_approx(float x) {
    if (fabsf(x) < 0.0625f) {
        float q = __fmaf_rn(x, 1.f / 720.f, 1.f / 120.f);
        q = __fmaf_rn(x, q, 1.f / 24.f);
        q = __fmaf_rn(x, q, 1.f / 6.f);
        q = __fmaf_rn(x, q, 0.5f);
        return __fmaf_rn(__fmul_rn(x, x), q, x);
    }
    return __fsub_rn(__expf(x), 1.f);
}

__global__ void k_expm1_check(const float* __restrict__ x, float* __restrict__ approx, float* __restrict__ ref,
                              int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        approx[i] = expm1_approx(x[i]);
        ref[i] = expm1f(x[i]);
    }
}

cudaError_t launch_expm1_check(const float* x, float* approx, float* ref, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_expm1_check<<<(n + 255) / 256, 256, 0, st>>>(x, approx, ref, n);
    ++g_launch_counter;
    return cudaGetLastError();
}

// Primary ray of pixel (i, j), sample s: PerspectiveCamera::getRay with the
// offset 0.5 + (u - 0.5) in each axis, mapped to the density's index space.
__device__ __forceinline__ bool primary_ray(const DevScene& sc, const DevCamera& cam, int i, int j, Stream stream,
                                            IRay& pr) {
    const DevGrid& G = sc.dens;
    const float jx = draw(stream, kTagJitterX), jy = draw(stream, kTagJitterY);
    const float sx = (2.f * ((float)i + jx) / (float)cam.width - 1.f) * cam.sw;
    const float sy = (1.f - 2.f * ((float)j + jy) / (float)cam.height) * cam.sh;
    // rounding spelled out: the count and shading passes must trace the same
    // rays
    float d[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) d[c] = __fsub_rn(__fmaf_rn(sx, cam.m[c], __fmul_rn(sy, cam.m[3 + c])), cam.m[6 + c]);
    const float invl = rsqrtf(__fmaf_rn(d[0], d[0], __fmaf_rn(d[1], d[1], __fmul_rn(d[2], d[2]))));
    d[0] *= invl; d[1] *= invl; d[2] *= invl;
    const float tscale =
        1.f / __fmaf_rn(d[0], cam.cdir[0], __fmaf_rn(d[1], cam.cdir[1], __fmul_rn(d[2], cam.cdir[2])));
    make_iray(pr, (cam.eye[0] - G.wo[0]) * G.inv_h, (cam.eye[1] - G.wo[1]) * G.inv_h,
              (cam.eye[2] - G.wo[2]) * G.inv_h, d[0], d[1], d[2], cam.znear * tscale * G.inv_h,
              cam.zfar * tscale * G.inv_h);
    return clip_to_bbox_flat(G, pr);
}

// The low 16 bits of v spread to the even bits (Morton order of two bin
// indices).
__device__ __forceinline__ uint32_t spread_bits16(uint32_t v) {
    v &= 0xFFFFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}
__device__ __forceinline__ int clamp_bin(float x, int n) { return min(max((int)x, 0), n - 1); }

// Key of the shadow ray of light b for the task at index-space position p:
// its light-space bin (Morton order of the (u, v) or cube-map bins) and its
// depth bin, after the keys of the lights before it. The host keeps every
// key below 2^31, so the arithmetic is 32-bit; the point light's cube-map
// coordinates and distance come from approximate reciprocals (the key only
// decides the order in which rays are marched).
__device__ __forceinline__ uint32_t ray_key(const RayBin& b, const float p[3], int64_t t) {
    if (b.kind == 2) return (uint32_t)(b.key_off + (t >> b.shift));
    uint32_t uv;
    float depth;
    if (b.kind == 0) {
        const float u = p[0] * b.U[0] + p[1] * b.U[1] + p[2] * b.U[2] - b.u0;
        const float v = p[0] * b.V[0] + p[1] * b.V[1] + p[2] * b.V[2] - b.v0;
        uv = spread_bits16((uint32_t)clamp_bin(u * b.inv_bs, b.ns)) |
             (spread_bits16((uint32_t)clamp_bin(v * b.inv_bs, b.ns)) << 1);
        depth = p[0] * b.D[0] + p[1] * b.D[1] + p[2] * b.D[2] - b.d0;
    } else {
        const float w0 = p[0] - b.O[0], w1 = p[1] - b.O[1], w2 = p[2] - b.O[2];
        const float a0 = fabsf(w0), a1 = fabsf(w1), a2 = fabsf(w2);
        uint32_t face;
        float m, x, y;
        if (a0 >= a1 && a0 >= a2) { face = w0 < 0.f; m = a0; x = w1; y = w2; }
        else if (a1 >= a2) { face = 2 + (w1 < 0.f); m = a1; x = w0; y = w2; }
        else { face = 4 + (w2 < 0.f); m = a2; x = w0; y = w1; }
        const float inv = m > 0.f ? __fdividef(0.5f, m) : 0.f;
        uv = face * (uint32_t)b.ns * (uint32_t)b.ns +
             (spread_bits16((uint32_t)clamp_bin((x * inv + 0.5f) * (float)b.ns, b.ns)) |
              (spread_bits16((uint32_t)clamp_bin((y * inv + 0.5f) * (float)b.ns, b.ns)) << 1));
        const float r2 = w0 * w0 + w1 * w1 + w2 * w2;
        depth = (r2 > 0.f ? r2 * rsqrtf(r2) : 0.f) - b.d0;
    }
    return (uint32_t)b.key_off + uv * (uint32_t)b.nd + (uint32_t)clamp_bin(depth * b.inv_ds, b.nd);
}

// Per pixel-sample results of the primary wave.
struct PixelSample {
    float scat[3], emis[3], trans[3];
};

// One pixel sample ps = pixel * spp + s of the primary wave. kWrite = false
// only counts the shading samples (counts[ps]); kWrite = true accumulates the
// scatter and emission AOVs and writes the shadow tasks at offsets[ps]. The
// two passes must agree on every sample, so the arithmetic that decides
// which samples shade (positions, transmittance, termination, step jitter)
// is spelled out rounding by rounding (no contraction left to the compiler).
// Returns the primary samples taken.
template <bool kWrite, int DT>
__device__ __forceinline__ uint32_t primary_sample(const DevScene& sc, const DevCamera& cam, const DevScatterGrid& sg,
                                                   int64_t ps, int32_t* __restrict__ counts,
                                                   const int32_t* __restrict__ offsets, ShadowTask* __restrict__ tasks,
                                                   int64_t task_cap, PixelSample* __restrict__ out,
                                                   const RayOrder& ko) {
    uint32_t n_primary = 0;
    const int64_t pix = ps / cam.spp;
    const int i = (int)(pix % cam.width), j = (int)(pix / cam.width);
    const DevGrid& G = sc.dens;
    const DevShader& sh = sc.sh;
    const Stream stream = make_stream(sc.seed, kDomainPixel | (uint64_t)ps);
    const float step0 = sc.step0, cutoff = sc.cutoff;
    float pT3[3] = {1.f, 1.f, 1.f}, sL[3] = {0.f, 0.f, 0.f}, eL[3] = {0.f, 0.f, 0.f};
    int32_t shading = 0;
    IRay pr;
    if (primary_ray(sc, cam, i, j, stream, pr)) {
        LeafDDA dda;
        dda_init_bits(dda, pr, G);
        float ta, tb;
        uint32_t span_ord = 0, n_iter = 0;
        uint32_t jit = step_seed_primary(stream);
        bool pdrop = false;
        int64_t base = kWrite ? offsets[ps] : 0;
        while (!pdrop && next_span(G, dda, ta, tb)) {
            float pStep = jitter_step(step0, draw(stream, kTagPrimarySpan | span_ord));
            ++span_ord;
            // (pT + pStep > pT stops a march whose step underflows against pT)
            for (float pT = step0 * ceilf(ta / step0); pT <= tb && pT + pStep > pT;) {
                const uint32_t n = n_iter++;
                jit = step_next(jit);
                ++n_primary;
                const float p[3] = {__fmaf_rn(pT, pr.d[0], pr.e[0]), __fmaf_rn(pT, pr.d[1], pr.e[1]),
                                    __fmaf_rn(pT, pr.d[2], pr.e[2])};
                const float rho = fminf(sample_span_t<DT>(G, p[0], p[1], p[2]) * sh.dS, sh.dMax);
                if (rho < cutoff) { pT += pStep; continue; }
                float omdT[3], dT[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float e1 = expm1_approx(-sh.a[c] * rho * pStep);
                    dT[c] = 1.f + e1;
                    omdT[c] = -e1;
                }
                if (kWrite) {
                    const float pw[3] = {p[0] * G.h + G.wo[0], p[1] * G.h + G.wo[1], p[2] * G.h + G.wo[2]};
                    float sgv[3], em[3];
                    sample_scatter(sg, pw[0], pw[1], pw[2], sgv);
                    // clamp(rho, 0, 1)^maskPower (src/Renderer.h:584-588) as 2^(p log2 x);
                    // x = 0 gives what pow gives: 1 for p = 0, 0 for p > 0, inf for p < 0
                    const float rc = fminf(fmaxf(rho, 0.f), 1.f), mp = sh.mask_power;
                    const float mask = (rc > 0.f ? exp2f(mp * __log2f(rc)) : (mp == 0.f ? 1.f : mp > 0.f ? 0.f : kInf)) *
                                       sh.scatter_scale;
                    const float temp = sc.has_temp ? sample_world(sc.temp, pw[0], pw[1], pw[2]) : 0.f;
                    ramp_color(sh, temp, em);
                    const int64_t t = base + shading;
                    if (t < task_cap) {
                        ShadowTask tk;
                        tk.p[0] = p[0]; tk.p[1] = p[1]; tk.p[2] = p[2];
#pragma unroll
                        for (int c = 0; c < 3; ++c) tk.w[c] = pT3[c] * omdT[c];
                        tk.sa = stream.a;
                        tk.iw = shadow_iter_word(stream, n);
                        tasks[t] = tk;
                        // the first task of a unit files the unit under each
                        // light's order key (the shadow-ray ordering's count)
                        if ((t & (kRayUnit - 1)) == 0) {
                            const int64_t u = t / kRayUnit;
                            // unrolled over the light slots, so each light's
                            // bin parameters are read as constants
#pragma unroll
                            for (int k = 0; k < kMaxLights; ++k) {
                                if (k >= ko.rb.n) break;
                                const uint32_t key = ray_key(ko.rb.b[k], p, t);
                                ko.keys[k * ko.unit_cap + u] = key;
                                // lanes filing under the same key share one atomic
                                const cg::coalesced_group grp = cg::labeled_partition(cg::coalesced_threads(), key);
                                if (grp.thread_rank() == 0) atomicAdd(ko.key_counts + key, (int)grp.size());
                            }
                        }
                    }
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        sL[c] += sgv[c] * sh.inv_scatter[c] * mask * pT3[c] * omdT[c];
                        eL[c] += em[c] * sh.emission_scale * pT3[c] * omdT[c];
                    }
                }
                ++shading;
#pragma unroll
                for (int c = 0; c < 3; ++c) pT3[c] *= dT[c];
                if (__fmaf_rn(pT3[0], pT3[0], __fmaf_rn(pT3[1], pT3[1], __fmul_rn(pT3[2], pT3[2]))) < cutoff) {
                    pdrop = true;
                    break;
                }
                pStep = jitter_step_bits(step0, jit);
                pT += pStep;
            }
        }
    }
    if (!kWrite) counts[ps] = shading;
    if (kWrite) {
        PixelSample o;
#pragma unroll
        for (int c = 0; c < 3; ++c) { o.scat[c] = sL[c]; o.emis[c] = eL[c]; o.trans[c] = pT3[c]; }
        out[ps] = o;
    }
    return n_primary;
}

// Warps claim 32 consecutive pixel samples at a time from *claim (zero at
// launch) until none are left: a persistent grid in which no warp slot waits
// on another warp's long ray. The shading pass runs 5 CTAs per SM so that
// its registers do not spill; the count pass, lighter, runs 6.
template <bool kWrite, int DT>
__global__ void __launch_bounds__(128, kWrite ? 5 : 6) k_primary(DevScene sc, DevCamera cam, DevScatterGrid sg,
                                                 int32_t* __restrict__ counts, const int32_t* __restrict__ offsets,
                                                 ShadowTask* __restrict__ tasks, int64_t task_cap,
                                                 PixelSample* __restrict__ out, unsigned long long* __restrict__ ctr,
                                                 unsigned long long* __restrict__ claim, RayOrder ko,
                                                 int max_claims) {
    const int64_t n_ps = (int64_t)cam.width * cam.height * cam.spp;
    const int lane = threadIdx.x & 31;
    uint32_t n_primary = 0;
    // max_claims > 0: a warp takes at most that many claims (short-lived
    // CTAs, whose slots free up for kernels of other streams)
    for (int claims = 0; max_claims <= 0 || claims < max_claims; ++claims) {
        unsigned long long claimed = 0;
        if (lane == 0) claimed = atomicAdd(claim, 32ull);
        claimed = __shfl_sync(0xffffffffu, claimed, 0);
        if ((int64_t)claimed >= n_ps) break;
        const int64_t ps = (int64_t)claimed + lane;
        if (ps < n_ps)
            n_primary += primary_sample<kWrite, DT>(sc, cam, sg, ps, counts, offsets, tasks, task_cap, out, ko);
    }
    if (kWrite && ctr) {
        unsigned long long q = n_primary;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(ctr, q);
    }
}

// --- shadow-ray ordering ---------------------------------------------------

// Scatter pass of the warp-aggregated counting sort over units of kRayUnit
// consecutive tasks (neighbouring shading samples of one primary ray, keyed
// by the first one): the shading pass has filed every unit under each
// light's key and counted the keys, the counts have been scanned into
// offsets, and here each run of equal keys in neighbouring lanes takes one
// atomic. Within a key the order is whatever the atomics give; every ray's
// result goes to its own slot, so results do not depend on it.
__global__ void __launch_bounds__(256) k_ray_scatter(const uint32_t* __restrict__ keys, int64_t unit_cap,
                                                     int n_lights, const int32_t* __restrict__ total_ptr,
                                                     int64_t task_cap, int32_t* __restrict__ offsets,
                                                     int32_t* __restrict__ order) {
    const int64_t total = min((int64_t)*total_ptr, task_cap);
    const int64_t n_units = (total + kRayUnit - 1) / kRayUnit;
    const int lane = threadIdx.x & 31;
    // each CTA takes one contiguous chunk of the units, so within a key the
    // units of one chunk (one band of the image) lie next to each other in
    // the order; measured on the production frame: this pass 0.90 -> 0.97 ms,
    // the shadow wave that reads the order 14.32 -> 14.18 ms, against CTAs
    // striding over the units side by side
    const int64_t chunk = (n_units + gridDim.x - 1) / gridDim.x;
    const int64_t u0 = (int64_t)blockIdx.x * chunk, u1 = min(u0 + chunk, n_units);
    for (int k = 0; k < n_lights; ++k) {
        const uint32_t* kk = keys + (int64_t)k * unit_cap;
        for (int64_t base = u0; base < u1; base += blockDim.x) {
            const int64_t u = base + threadIdx.x;
            const bool valid = u < u1;
            // keys index the counts array (fewer than 2^31 of them, checked by
            // the host), so no valid key equals the end marker
            const uint32_t key = valid ? kk[u] : 0xFFFFFFFFu;
            // runs of equal keys in neighbouring lanes (a primary ray's units
            // are neighbours) take one atomic each: the run's first lane adds
            // the run's length and hands the position on (a shuffle and a
            // ballot instead of a 32-lane match: ordering 1.12 -> 0.87 ms on
            // the production frame)
            const uint32_t left = __shfl_up_sync(0xffffffffu, key, 1);
            const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || left != key);
            const unsigned upto = (2u << lane) - 1u;  // lanes 0..lane (all 32 for lane 31)
            const int head = 31 - __clz(heads & upto);
            const unsigned after = heads & ~upto;
            int32_t pos = 0;
            if (valid && head == lane) pos = atomicAdd(offsets + key, (after ? __ffs(after) - 1 : 32) - lane);
            pos = __shfl_sync(0xffffffffu, pos, head);
            if (valid) order[pos + (lane - head)] = (int32_t)u;
        }
    }
}

// --- occupancy bounds of the light-space bins -----------------------------

// Cube-map face of direction w and its two face coordinates in [-1, 1]
// (the same face choice and axis order as ray_key).
__device__ __forceinline__ int cube_face(const float w[3], float& x, float& y) {
    const float a0 = fabsf(w[0]), a1 = fabsf(w[1]), a2 = fabsf(w[2]);
    int face;
    float m;
    if (a0 >= a1 && a0 >= a2) { face = w[0] < 0.f; m = a0; x = w[1]; y = w[2]; }
    else if (a1 >= a2) { face = 2 + (w[1] < 0.f); m = a1; x = w[0]; y = w[2]; }
    else { face = 4 + (w[2] < 0.f); m = a2; x = w[0]; y = w[1]; }
    // an approximate reciprocal: the bound tables' bins are widened by 1e-3
    // of a bin, far more than its error
    const float inv = m > 0.f ? __fdividef(1.f, m) : 0.f;
    x *= inv;
    y *= inv;
    return face;
}

// One thread per leaf-bitmap cell; a leaf cell (an 8^3 index-space box)
// raises the bound of every bin it overlaps, widened by a margin that covers
// the rounding of the rays' own bin computation.
__global__ void __launch_bounds__(256) k_ray_bounds(DevGrid g, RayBins rb) {
    const uint32_t lin = blockIdx.x * blockDim.x + threadIdx.x;
    if (lin >= g.nbits) return;
    if (!((__ldg(g.leafbits + (lin >> 5)) >> (lin & 31u)) & 1u)) return;
    const int cx = (int)(lin % (uint32_t)g.lbx), cy = (int)((lin / (uint32_t)g.lbx) % (uint32_t)g.lby),
              cz = (int)(lin / ((uint32_t)g.lbx * (uint32_t)g.lby));
    const float lo[3] = {(float)((g.blo[0] + cx - 1) * 8), (float)((g.blo[1] + cy - 1) * 8),
                         (float)((g.blo[2] + cz - 1) * 8)};
    for (int k = 0; k < rb.n; ++k) {
        const RayBin& b = rb.b[k];
        if (b.bound == nullptr) continue;
        if (b.kind == 0) {
            float umin = kInf, umax = -kInf, vmin = kInf, vmax = -kInf, dmax = -kInf;
            for (int c = 0; c < 8; ++c) {
                const float q[3] = {lo[0] + 8.f * (c & 1), lo[1] + 4.f * (c & 2), lo[2] + 2.f * (c & 4)};
                const float u = q[0] * b.U[0] + q[1] * b.U[1] + q[2] * b.U[2] - b.u0;
                const float v = q[0] * b.V[0] + q[1] * b.V[1] + q[2] * b.V[2] - b.v0;
                const float d = q[0] * b.D[0] + q[1] * b.D[1] + q[2] * b.D[2] - b.d0;
                umin = fminf(umin, u); umax = fmaxf(umax, u);
                vmin = fminf(vmin, v); vmax = fmaxf(vmax, v);
                dmax = fmaxf(dmax, d);
            }
            const float eps = 0.05f;  // index-space voxels
            const int u0 = clamp_bin((umin - eps) * b.inv_bs, b.ns), u1 = clamp_bin((umax + eps) * b.inv_bs, b.ns);
            const int v0 = clamp_bin((vmin - eps) * b.inv_bs, b.ns), v1 = clamp_bin((vmax + eps) * b.inv_bs, b.ns);
            const int bits = __float_as_int(fmaxf(dmax, 0.f));
            for (int v = v0; v <= v1; ++v)
                for (int u = u0; u <= u1; ++u) atomicMax(reinterpret_cast<int*>(b.bound) + v * b.ns + u, bits);
        } else if (b.kind == 1) {
            // the box's distance from the light
            float d2 = 0.f;
            for (int a = 0; a < 3; ++a) {
                const float e = fmaxf(fmaxf(lo[a] - b.O[a], b.O[a] - (lo[a] + 8.f)), 0.f);
                d2 = fmaf(e, e, d2);
            }
            const int bits = __float_as_int(sqrtf(d2));
            for (int f = 0; f < 6; ++f) {
                const int a = f >> 1;
                const float sg = (f & 1) ? -1.f : 1.f;
                const int ax = a == 0 ? 1 : 0, ay = a == 2 ? 1 : 2;
                int npos = 0;
                float smin = kInf, smax = -kInf, tmin = kInf, tmax = -kInf;
                for (int c = 0; c < 8; ++c) {
                    const float q[3] = {lo[0] + 8.f * (c & 1), lo[1] + 4.f * (c & 2), lo[2] + 2.f * (c & 4)};
                    const float w[3] = {q[0] - b.O[0], q[1] - b.O[1], q[2] - b.O[2]};
                    const float m = sg * w[a];
                    if (!(m > 0.f)) continue;
                    ++npos;
                    const float x = w[ax] / m, y = w[ay] / m;
                    smin = fminf(smin, x); smax = fmaxf(smax, x);
                    tmin = fminf(tmin, y); tmax = fmaxf(tmax, y);
                }
                if (npos == 0) continue;
                int s0 = 0, s1 = b.ns - 1, t0 = 0, t1 = b.ns - 1;
                if (npos == 8) {
                    // the face's bins as ray_key computes them, widened by 1e-3 bin
                    const float eps = 2e-3f / (float)b.ns;
                    s0 = clamp_bin(((smin - eps) * 0.5f + 0.5f) * (float)b.ns, b.ns);
                    s1 = clamp_bin(((smax + eps) * 0.5f + 0.5f) * (float)b.ns, b.ns);
                    t0 = clamp_bin(((tmin - eps) * 0.5f + 0.5f) * (float)b.ns, b.ns);
                    t1 = clamp_bin(((tmax + eps) * 0.5f + 0.5f) * (float)b.ns, b.ns);
                }  // else the box straddles the plane through the light: every bin of the face
                int* tb = reinterpret_cast<int*>(b.bound) + (int64_t)f * b.ns * b.ns;
                for (int t = t0; t <= t1; ++t)
                    for (int s = s0; s <= s1; ++s) atomicMin(tb + t * b.ns + s, bits);
            }
        }
    }
}

cudaError_t launch_ray_bounds(const DevGrid& g, const RayBins& rb, cudaStream_t st) {
    if (g.nbits == 0) return cudaSuccess;
    k_ray_bounds<<<(g.nbits + 255) / 256, 256, 0, st>>>(g, rb);
    ++g_launch_counter;
    return cudaGetLastError();
}

// End time of a shadow ray from index-space position p past which no leaf of
// its light-space bin lies (kInf without a bound table), plus a margin of two
// voxels for the rounding of the bin and depth computations.
__device__ __forceinline__ float shadow_ray_end(const RayBin& b, const float p[3]) {
    if (b.bound == nullptr) return kInf;
    if (b.kind == 0) {
        const float u = p[0] * b.U[0] + p[1] * b.U[1] + p[2] * b.U[2] - b.u0;
        const float v = p[0] * b.V[0] + p[1] * b.V[1] + p[2] * b.V[2] - b.v0;
        const float d = p[0] * b.D[0] + p[1] * b.D[1] + p[2] * b.D[2] - b.d0;
        const int ui = clamp_bin(u * b.inv_bs, b.ns), vi = clamp_bin(v * b.inv_bs, b.ns);
        return __ldg(b.bound + vi * b.ns + ui) - d + 2.f;
    }
    const float w[3] = {p[0] - b.O[0], p[1] - b.O[1], p[2] - b.O[2]};
    float x, y;
    const int f = cube_face(w, x, y);
    const int si = clamp_bin((x * 0.5f + 0.5f) * (float)b.ns, b.ns), ti = clamp_bin((y * 0.5f + 0.5f) * (float)b.ns, b.ns);
    const float dmin = __ldg(b.bound + ((int64_t)f * b.ns + ti) * b.ns + si);
    // the distance from one approximate reciprocal square root (well inside
    // the two-voxel margin)
    const float r2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
    return (r2 > 0.f ? r2 * rsqrtf(r2) : 0.f) - dmin + 2.f;
}

cudaError_t launch_ray_scatter(const uint32_t* keys, int64_t unit_cap, int n_lights, const int32_t* total,
                               int64_t task_cap, int32_t* offsets, int32_t* order, int sms, cudaStream_t st) {
    k_ray_scatter<<<(unsigned)sms * 8u, 256, 0, st>>>(keys, unit_cap, n_lights, total, task_cap, offsets, order);
    ++g_launch_counter;
    return cudaGetLastError();
}

// --- shadow rays -------------------------------------------------------------

// The samples of one leaf span of a shadow ray, from t0 (a multiple of the
// step) while they stay at or before sb and tau at or below the dropout
// depth: tau += rho * step for each sample with rho at or above the cutoff,
// rho = min(raw * scale, dmax) (kUnit: min(raw, dmax / scale), tau then in
// units of 1 / scale; ShadowMarch). A sample below the cutoff adds nothing
// and keeps its step (no re-jitter); the loop is branch-free, so the warp
// stays converged. The step that the last sample still advances is not used.
template <int DT, bool kUnit>
__device__ __forceinline__ void shadow_span_samples(const DevGrid& G, const IRay& r, float t0, float sb, float half_step,
                                                    float quarter_step, const ShadowMarch& sm, float& sStep,
                                                    uint32_t& jit, uint32_t& siter, float& tau) {
    for (float sT = t0; sT <= sb && tau <= sm.drop;) {
        ++siter;
        jit = step_next(jit);
        const float raw = sample_span_t<DT>(G, r.e[0] + sT * r.d[0], r.e[1] + sT * r.d[1], r.e[2] + sT * r.d[2]);
        const float rs = fminf(kUnit ? raw : raw * sm.scale, sm.dmax);
        const bool take = rs >= sm.cut;
        const float next = jitter_step_fma(half_step, quarter_step, jit);
        tau = take ? fmaf(rs, sStep, tau) : tau;
        sStep = take ? next : sStep;
        sT += sStep;
    }
}

// One thread per (light k, ordered slot r): the shadow rays of light k (all
// its samples) from task kRayUnit * order[k * n_units + r / kRayUnit] +
// r % kRayUnit; warps claim 32 consecutive (light, slot) pairs at a time from
// ctr[2] (zero at launch), so the lanes of a warp march neighbouring rays.
// ctr[1] accumulates the shadow samples.
// direct[k * task_cap + t] = albedo * (sum_ls I * T / ns) * w.
// kEnv = false leaves the environment-light branch out (no light of the
// scene is an environment light), which frees registers for occupancy.
// kUnit = sc.smarch.unit: the density scale folded into the march constants
// (ShadowMarch), one multiply per ray instead of one per sample.
template <int DT, bool kEnv, bool kUnit>
__global__ void __launch_bounds__(128, 8) k_shadow(DevScene sc, RayBins rb, const ShadowTask* __restrict__ tasks,
                                                const int32_t* __restrict__ total_ptr, int64_t task_cap,
                                                const int32_t* __restrict__ order, float4* __restrict__ direct,
                                                unsigned long long* __restrict__ ctr) {
    const int64_t total = min((int64_t)*total_ptr, task_cap);
    const uint64_t n_units = (uint64_t)(total + kRayUnit - 1) / kRayUnit;
    const uint64_t per_light = n_units * kRayUnit;
    const DevGrid& G = sc.dens;
    const DevShader& sh = sc.sh;
    const float step1 = sc.step1;
    const float inv_step1 = 1.f / step1, half_step1 = 0.5f * step1, quarter_step1 = 0.25f * step1;
    const ShadowMarch& sm = sc.smarch;
    uint32_t n_shadow = 0;
    // each warp claims the next 32 (light, ordered slot) pairs, lights in
    // order, until none are left: the warps stay busy to the end whatever
    // the rays cost (every ray's result goes to its own slot)
    const uint64_t n_slots = (uint64_t)sc.n_lights * per_light;
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(ctr + 2, 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n_slots) break;
        if (base + lane >= n_slots) continue;
        int k = 0;
        uint64_t rr = base + lane;
        while (rr >= per_light) {
            rr -= per_light;
            ++k;
        }
        const int64_t t = (int64_t)order[k * n_units + rr / kRayUnit] * kRayUnit + (int64_t)(rr % kRayUnit);
        if (t >= total) continue;
        // the task's start point and stream words now, its weights after the
        // march (not held in registers across it)
        const float4 tk0 = __ldg(reinterpret_cast<const float4*>(tasks + t));
        const uint2 tkw = __ldg(reinterpret_cast<const uint2*>(tasks + t) + 3);
        const float tp[3] = {tk0.x, tk0.y, tk0.z};
        const DevLight& Lk = sc.lights[k];
        float lum[3] = {0.f, 0.f, 0.f};
        for (int ls = 0; ls < Lk.samples; ++ls) {
            const uint32_t sub = shadow_key_from(tkw.x, tkw.y, (uint32_t)k, (uint32_t)ls);
            float ldir[3], I[3], dist;
            if (kEnv && Lk.type == 2) {
                env_illuminate(sc.env, Lk, draw_sub(sub, kTagEnvU), draw_sub(sub, kTagEnvV), ldir, I);
                dist = kInf;
            } else {
                const float pw[3] = {tp[0] * G.h + G.wo[0], tp[1] * G.h + G.wo[1], tp[2] * G.h + G.wo[2]};
                illuminate_shadow(Lk, pw, ldir, I, dist);
            }
            IRay srr;
            make_iray_approx(srr, tp[0], tp[1], tp[2], -ldir[0], -ldir[1], -ldir[2], kDelta * G.inv_h,
                             dist * G.inv_h);
            if (!clip_to_bbox_flat(G, srr)) continue;  // the reference skips the light sample
            // past the last leaf of the ray's light-space bin the walk finds no
            // span: stop it there (spans and samples are unchanged)
            srr.t1 = fminf(srr.t1, fmaxf(shadow_ray_end(rb.b[k], tp), srr.t0));
            LeafDDA sd;
            dda_init_bits(sd, srr, G);
            float sa, sb, tau = 0.f;
            uint32_t sspan = 0, siter = 0;
            uint32_t jit = step_seed_shadow(sub);
            bool sdrop = false;
            while (!sdrop && next_span(G, sd, sa, sb)) {
                float sStep = jitter_step(step1, draw_sub(sub, kTagShadowSpan | sspan));
                ++sspan;
                // every jittered step is >= 0.75 step1: if that is not
                // absorbed at sb, sT grows on every iteration up to sb
                if (!(sb + 0.75f * step1 > sb)) continue;
                shadow_span_samples<DT, kUnit>(G, srr, step1 * ceilf(sa * inv_step1), sb, half_step1, quarter_step1, sm,
                                               sStep, jit, siter, tau);
                sdrop = tau > sm.drop;
            }
            n_shadow += siter;
            if (sdrop) continue;
            if (kUnit) tau *= sm.scale;
#pragma unroll
            for (int c = 0; c < 3; ++c) lum[c] += I[c] * __expf(-sh.a[c] * tau);
        }
        const float inv_ns = __fdividef(1.f, (float)Lk.samples);
        const float2 w12 = __ldg(reinterpret_cast<const float2*>(tasks + t) + 2);
        const float tw[3] = {tk0.w, w12.x, w12.y};
        float o[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) o[c] = sh.albedo[c] * (lum[c] * inv_ns) * tw[c];
        direct[(int64_t)k * task_cap + t] = make_float4(o[0], o[1], o[2], 0.f);
    }
    {
        unsigned long long q = n_shadow;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(ctr + 1, q);
    }
}

// One warp per pixel. Its samples run side by side, G lanes each (G a power
// of two, spp * G <= 32, so 32 / G samples per pass): lane l of a sample's
// group sums the sample's tasks l, l + G, ... (a task's direct light is the
// sum of its lights' contributions in light order; two tasks' loads are
// issued before either is added), a butterfly inside the group combines the
// lanes, and lane 0 (whose summation order is fixed) takes the samples in
// order to form the antialiasing averages. Each group's first lane loads its
// sample's primary-wave results up front, in parallel with the task loads,
// and hands them to lane 0 by shuffles. 8 CTAs per SM (64 registers, a few
// bytes spilled) hide the loads' latency better than 7 without spills.
__global__ void __launch_bounds__(128, 8) k_resolve(DevCamera cam, const int32_t* __restrict__ offsets,
                                                 const int32_t* __restrict__ counts,
                                                 const PixelSample* __restrict__ pss,
                                                 const float4* __restrict__ direct, int n_lights, int64_t task_cap,
                                                 float4* __restrict__ rgba, float4* __restrict__ dfilm,
                                                 float4* __restrict__ sfilm, float4* __restrict__ efilm) {
    const int64_t pix = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (pix >= (int64_t)cam.width * cam.height) return;  // uniform across the warp
    const int spp = cam.spp;
    int G = 32;
    while (G > 1 && G * spp > 32) G >>= 1;
    const int per_pass = 32 / G, gl = lane & (G - 1);
    const float ratio = 1.f / (float)spp;
    float tAA[3] = {0.f, 0.f, 0.f}, lAA[3] = {0.f, 0.f, 0.f}, dAA[3] = {0.f, 0.f, 0.f};
    float sAA[3] = {0.f, 0.f, 0.f}, eAA[3] = {0.f, 0.f, 0.f};
    for (int s0 = 0; s0 < spp; s0 += per_pass) {
        const int s = s0 + lane / G;
        float d[3] = {0.f, 0.f, 0.f};
        float o[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // scat, emis, trans
        if (s < spp) {
            const int64_t ps = pix * spp + s;
            if (gl == 0) {
                const PixelSample q = pss[ps];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    o[c] = q.scat[c];
                    o[3 + c] = q.emis[c];
                    o[6 + c] = q.trans[c];
                }
            }
            const int64_t b = offsets[ps], e = min((int64_t)b + counts[ps], task_cap);
            for (int64_t t = b + gl; t < e; t += 2 * G) {
                const bool two = t + G < e;
                float acc0[3] = {0.f, 0.f, 0.f}, acc1[3] = {0.f, 0.f, 0.f};
                for (int k = 0; k < n_lights; ++k) {
                    const float4 v0 = direct[(int64_t)k * task_cap + t];
                    const float4 v1 = two ? direct[(int64_t)k * task_cap + t + G] : make_float4(0.f, 0.f, 0.f, 0.f);
                    acc0[0] += v0.x;
                    acc0[1] += v0.y;
                    acc0[2] += v0.z;
                    acc1[0] += v1.x;
                    acc1[1] += v1.y;
                    acc1[2] += v1.z;
                }
                d[0] += acc0[0];
                d[1] += acc0[1];
                d[2] += acc0[2];
                if (two) {
                    d[0] += acc1[0];
                    d[1] += acc1[1];
                    d[2] += acc1[2];
                }
            }
        }
        for (int off = G >> 1; off > 0; off >>= 1)
#pragma unroll
            for (int c = 0; c < 3; ++c) d[c] += __shfl_xor_sync(0xffffffffu, d[c], off);
        const int ns = min(per_pass, spp - s0);
        for (int jj = 0; jj < ns; ++jj) {
            float dj[3], oj[9];
#pragma unroll
            for (int c = 0; c < 3; ++c) dj[c] = __shfl_sync(0xffffffffu, d[c], jj * G);
#pragma unroll
            for (int c = 0; c < 9; ++c) oj[c] = __shfl_sync(0xffffffffu, o[c], jj * G);
            if (lane == 0) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    lAA[c] += (dj[c] + oj[c] + oj[3 + c]) * ratio;
                    dAA[c] += dj[c] * ratio;
                    sAA[c] += oj[c] * ratio;
                    eAA[c] += oj[3 + c] * ratio;
                    tAA[c] += oj[6 + c] * ratio;
                }
            }
        }
    }
    if (lane != 0) return;
    if (rgba) rgba[pix] = make_float4(lAA[0], lAA[1], lAA[2], 1.f - (tAA[0] + tAA[1] + tAA[2]) / 3.f);
    if (dfilm) dfilm[pix] = make_float4(dAA[0], dAA[1], dAA[2], 0.f);
    if (sfilm) sfilm[pix] = make_float4(sAA[0], sAA[1], sAA[2], 0.f);
    if (efilm) efilm[pix] = make_float4(eAA[0], eAA[1], eAA[2], 0.f);
}

// Resident 128-thread CTAs per SM of the k_primary instance (kWrite, dtype).
// Server slots render from several host threads at once: the value is
// computed into a local and published through an atomic slot.
static int primary_ctas_per_sm(bool write, int dtype) {
    static std::atomic<int> cache[2][3];
    if (dtype < 0 || dtype > 2) dtype = 0;
    std::atomic<int>& c = cache[write ? 1 : 0][dtype];
    if (c.load() == 0) {
        int n = 0;
        cudaError_t e;
        if (write)
            e = dtype == 1   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_primary<true, 1>, 128, 0)
                : dtype == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_primary<true, 2>, 128, 0)
                             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_primary<true, 0>, 128, 0);
        else
            e = dtype == 1   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_primary<false, 1>, 128, 0)
                : dtype == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_primary<false, 2>, 128, 0)
                             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_primary<false, 0>, 128, 0);
        if (e != cudaSuccess || n < 1) n = 1;
        c.store(n);
    }
    return c.load();
}

cudaError_t launch_render_count(const DevScene& sc, const DevCamera& cam, const DevScatterGrid& sg, int32_t* counts,
                                unsigned long long* claim, int sms, cudaStream_t st, bool short_ctas) {
    const int64_t n_ps = (int64_t)cam.width * cam.height * cam.spp;
    if (n_ps == 0) return cudaSuccess;
    // one resident wave, at most one warp per 32 pixel samples; or (short
    // CTAs) one CTA per 128 pixel samples whose warps claim once each
    const unsigned blocks =
        short_ctas ? (unsigned)((n_ps + 127) / 128)
                   : (unsigned)std::min<int64_t>((n_ps + 127) / 128,
                                                 (int64_t)sms * primary_ctas_per_sm(false, sc.dens.dtype));
    const int max_claims = short_ctas ? 1 : 0;
    if (sc.dens.dtype == 1)
        k_primary<false, 1><<<blocks, 128, 0, st>>>(sc, cam, sg, counts, nullptr, nullptr, 0, nullptr, nullptr, claim, RayOrder{}, max_claims);
    else if (sc.dens.dtype == 2)
        k_primary<false, 2><<<blocks, 128, 0, st>>>(sc, cam, sg, counts, nullptr, nullptr, 0, nullptr, nullptr, claim, RayOrder{}, max_claims);
    else
        k_primary<false, 0><<<blocks, 128, 0, st>>>(sc, cam, sg, counts, nullptr, nullptr, 0, nullptr, nullptr, claim, RayOrder{}, max_claims);
    ++g_launch_counter;
    return cudaGetLastError();
}

// The k_shadow instance for (dtype, env, unit).
template <int DT>
static const void* shadow_kernel_dt(bool env, bool unit) {
    if (env) return unit ? (const void*)k_shadow<DT, true, true> : (const void*)k_shadow<DT, true, false>;
    return unit ? (const void*)k_shadow<DT, false, true> : (const void*)k_shadow<DT, false, false>;
}
static const void* shadow_kernel(int dtype, bool env, bool unit) {
    return dtype == 1 ? shadow_kernel_dt<1>(env, unit) : dtype == 2 ? shadow_kernel_dt<2>(env, unit)
                                                                    : shadow_kernel_dt<0>(env, unit);
}

// Resident CTAs per SM of the k_shadow instance for (dtype, env, unit), from
// the occupancy calculator (once per instance; it enqueues no work, so it
// may run while a stream is being captured).
static int shadow_ctas_per_sm(int dtype, bool env, bool unit) {
    static std::atomic<int> cache[3][2][2];
    if (dtype < 0 || dtype > 2) dtype = 0;
    std::atomic<int>& c = cache[dtype][env ? 1 : 0][unit ? 1 : 0];
    if (c.load() == 0) {
        int n = 0;
        const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, shadow_kernel(dtype, env, unit), 128, 0);
        c.store((e == cudaSuccess && n > 0) ? n : 8);
    }
    return c.load();
}

cudaError_t launch_render_shade(const DevScene& sc, const DevCamera& cam, const DevScatterGrid& sg,
                                const int32_t* counts, const int32_t* offsets, const int32_t* total,
                                ShadowTask* tasks, int64_t task_cap, void* pixel_samples, const RayOrder& ro,
                                float4* direct, float4* rgba, float4* dfilm, float4* sfilm, float4* efilm,
                                unsigned long long* counters, int sms, cudaStream_t st, cudaEvent_t* marks) {
    const int64_t n_ps = (int64_t)cam.width * cam.height * cam.spp;
    const int64_t n_pix = (int64_t)cam.width * cam.height;
    if (n_ps == 0) return cudaSuccess;
    PixelSample* pss = reinterpret_cast<PixelSample*>(pixel_samples);
    const unsigned blocks = (unsigned)std::min<int64_t>((n_ps + 127) / 128,
                                                        (int64_t)sms * primary_ctas_per_sm(true, sc.dens.dtype));
    auto mark = [&](int k) {
        if (marks && marks[k]) cudaEventRecord(marks[k], st);
    };
    cudaError_t e;
    // the shading pass also files every unit of shadow rays under its order
    // keys and counts them (the counts zeroed first)
    if (ro.rb.n > 0 && (e = cudaMemsetAsync(ro.key_counts, 0, sizeof(int32_t) * ro.n_keys, st)) != cudaSuccess)
        return e;
    if (sc.dens.dtype == 1)
        k_primary<true, 1><<<blocks, 128, 0, st>>>(sc, cam, sg, nullptr, offsets, tasks, task_cap, pss, counters,
                                                   counters + 4, ro, 0);
    else if (sc.dens.dtype == 2)
        k_primary<true, 2><<<blocks, 128, 0, st>>>(sc, cam, sg, nullptr, offsets, tasks, task_cap, pss, counters,
                                                   counters + 4, ro, 0);
    else
        k_primary<true, 0><<<blocks, 128, 0, st>>>(sc, cam, sg, nullptr, offsets, tasks, task_cap, pss, counters,
                                                   counters + 4, ro, 0);
    ++g_launch_counter;
    mark(0);
    // order the shadow rays: scan the key counts, scatter the units
    if (ro.rb.n > 0) {
        if ((e = launch_exclusive_scan(ro.key_counts, ro.n_keys, ro.key_offsets, ro.key_scan, ro.key_total, st)) !=
            cudaSuccess)
            return e;
        if ((e = launch_ray_scatter(ro.keys, ro.unit_cap, ro.rb.n, total, task_cap, ro.key_offsets, ro.order, sms,
                                    st)) != cudaSuccess)
            return e;
    }
    mark(1);
    bool env = false;
    for (int k = 0; k < sc.n_lights; ++k) env = env || sc.lights[k].type == 2;
    // one resident wave of CTAs; the threads stride over the rays
    const bool unit = sc.smarch.unit != 0;
    const unsigned sblocks = (unsigned)sms * (unsigned)shadow_ctas_per_sm(sc.dens.dtype, env, unit);
    {
        DevScene scv = sc;
        RayBins rbv = ro.rb;
        const ShadowTask* tasks_c = tasks;
        const int32_t* order_c = ro.order;
        void* args[] = {&scv, &rbv, &tasks_c, (void*)&total, &task_cap, &order_c, &direct, &counters};
        if ((e = cudaLaunchKernel(shadow_kernel(sc.dens.dtype, env, unit), dim3(sblocks), dim3(128), args, 0, st)) !=
            cudaSuccess)
            return e;
    }
    ++g_launch_counter;
    mark(2);
    k_resolve<<<(unsigned)((n_pix * 32 + 127) / 128), 128, 0, st>>>(cam, offsets, counts, pss, direct, sc.n_lights,
                                                                   task_cap, rgba, dfilm, sfilm, efilm);
    ++g_launch_counter;
    mark(3);
    return cudaGetLastError();
}

size_t pixel_sample_bytes() { return sizeof(PixelSample); }

}  // namespace lg

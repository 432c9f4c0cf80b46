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
//                      (position, pTrans * (1 - dT), loop iteration);
//   k_shadow         : one thread per task marches its shadow rays (all light
//                      samples); consecutive threads are consecutive samples of
//                      one primary ray, so their shadow rays are coherent;
//   k_resolve        : per pixel, sums the tasks in order and writes the films.
// Shadow rays accumulate a scalar optical depth (every channel of the
// reference's product of exponentials is exp(-a_c * tau)) and stop when tau
// passes the dropout depth. Random numbers come from counter-based streams
// keyed by (seed, pixel, sample, loop iteration), so results do not depend on
// the launch shape; the reference's render RNG depends on TBB's row split.
#include <atomic>

#include "lg_kernels.h"

namespace lg {

// Trilinear Vec3 sample of the coarse scatter grid (0 outside the box).
__device__ __forceinline__ void sample_scatter(const DevScatterGrid& sg, float wx, float wy, float wz,
                                               float out[3]) {
    const float px = wx * sg.inv_H, py = wy * sg.inv_H, pz = wz * sg.inv_H;
    const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    const int ix = (int)fx - sg.lo[0], iy = (int)fy - sg.lo[1], iz = (int)fz - sg.lo[2];
    const float u = px - fx, v = py - fy, w = pz - fz;
    float4 c[2][2][2];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                const int x = ix + a, y = iy + b, z = iz + d;
                if ((unsigned)x < (unsigned)sg.dims[0] && (unsigned)y < (unsigned)sg.dims[1] &&
                    (unsigned)z < (unsigned)sg.dims[2])
                    c[a][b][d] = __ldg(sg.v + ((int64_t)z * sg.dims[1] + y) * sg.dims[0] + x);
                else
                    c[a][b][d] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
    auto l = [](float4 p, float4 q, float t) {
        return make_float4(lerpf(p.x, q.x, t), lerpf(p.y, q.y, t), lerpf(p.z, q.z, t), 0.f);
    };
    const float4 r = l(l(l(c[0][0][0], c[0][0][1], w), l(c[0][1][0], c[0][1][1], w), v),
                       l(l(c[1][0][0], c[1][0][1], w), l(c[1][1][0], c[1][1][1], w), v), u);
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
}

__device__ __forceinline__ float jitter_step(float step, float u) { return step * (1.f + (u - 0.5f) * 0.5f); }

// Primary ray of pixel (i, j), sample s: PerspectiveCamera::getRay with the
// offset 0.5 + (u - 0.5) in each axis, mapped to the density's index space.
__device__ __forceinline__ bool primary_ray(const DevScene& sc, const DevCamera& cam, int i, int j, Stream stream,
                                            IRay& pr) {
    const DevGrid& G = sc.dens;
    const float jx = draw(stream, kTagJitterX), jy = draw(stream, kTagJitterY);
    const float sx = (2.f * ((float)i + jx) / (float)cam.width - 1.f) * cam.sw;
    const float sy = (1.f - 2.f * ((float)j + jy) / (float)cam.height) * cam.sh;
    float d[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) d[c] = sx * cam.m[c] + sy * cam.m[3 + c] - cam.m[6 + c];
    const float invl = rsqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    d[0] *= invl; d[1] *= invl; d[2] *= invl;
    const float tscale = 1.f / (d[0] * cam.cdir[0] + d[1] * cam.cdir[1] + d[2] * cam.cdir[2]);
    make_iray(pr, (cam.eye[0] - G.wo[0]) * G.inv_h, (cam.eye[1] - G.wo[1]) * G.inv_h,
              (cam.eye[2] - G.wo[2]) * G.inv_h, d[0], d[1], d[2], cam.znear * tscale * G.inv_h,
              cam.zfar * tscale * G.inv_h);
    return clip_to_bbox(G, pr);
}

// Per pixel-sample results of the primary wave.
struct PixelSample {
    float scat[3], emis[3], trans[3];
};

// One thread per pixel-sample ps = pixel * spp + s. kWrite = false only
// counts the shading samples; kWrite = true accumulates the scatter and
// emission AOVs and writes the shadow tasks at offsets[ps].
template <bool kWrite, int DT>
__global__ void __launch_bounds__(128, 4) k_primary(DevScene sc, DevCamera cam, DevScatterGrid sg,
                                                 int32_t* __restrict__ counts, const int32_t* __restrict__ offsets,
                                                 ShadowTask* __restrict__ tasks, int64_t task_cap,
                                                 PixelSample* __restrict__ out, unsigned long long* __restrict__ ctr) {
    const int64_t ps = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n_ps = (int64_t)cam.width * cam.height * cam.spp;
    uint32_t n_primary = 0;
    if (ps < n_ps) {
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
            dda_init(dda, pr, G);
            float ta, tb;
            uint32_t span_ord = 0, n_iter = 0;
            bool pdrop = false;
            int64_t base = kWrite ? offsets[ps] : 0;
            while (!pdrop && next_span(G, dda, ta, tb)) {
                float pStep = jitter_step(step0, draw(stream, kTagPrimarySpan | span_ord));
                ++span_ord;
                // (pT + pStep > pT stops a march whose step underflows against pT)
                for (float pT = step0 * ceilf(ta / step0); pT <= tb && pT + pStep > pT;) {
                    const uint32_t n = n_iter++;
                    ++n_primary;
                    const float p[3] = {pr.e[0] + pT * pr.d[0], pr.e[1] + pT * pr.d[1], pr.e[2] + pT * pr.d[2]};
                    const float rho = fminf(sample_index_t<DT>(G, p[0], p[1], p[2]) * sh.dS, sh.dMax);
                    if (rho < cutoff) { pT += pStep; continue; }
                    float omdT[3], dT[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float e1 = expm1f(-sh.a[c] * rho * pStep);
                        dT[c] = 1.f + e1;
                        omdT[c] = -e1;
                    }
                    if (kWrite) {
                        const float pw[3] = {p[0] * G.h + G.wo[0], p[1] * G.h + G.wo[1], p[2] * G.h + G.wo[2]};
                        float sgv[3], em[3];
                        sample_scatter(sg, pw[0], pw[1], pw[2], sgv);
                        const float mask = powf(fminf(fmaxf(rho, 0.f), 1.f), sh.mask_power) * sh.scatter_scale;
                        const float temp = sc.has_temp ? sample_world(sc.temp, pw[0], pw[1], pw[2]) : 0.f;
                        ramp_color(sh, temp, em);
                        const int64_t t = base + shading;
                        if (t < task_cap) {
                            ShadowTask tk;
                            tk.p[0] = p[0]; tk.p[1] = p[1]; tk.p[2] = p[2];
#pragma unroll
                            for (int c = 0; c < 3; ++c) tk.w[c] = pT3[c] * omdT[c];
                            tk.n = n;
                            tk.ps = (uint32_t)ps;
                            tasks[t] = tk;
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
                    if (pT3[0] * pT3[0] + pT3[1] * pT3[1] + pT3[2] * pT3[2] < cutoff) { pdrop = true; break; }
                    pStep = jitter_step(step0, draw(stream, kTagPrimaryStep | n));
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
    }
    if (kWrite && ctr) {
        unsigned long long q = n_primary;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(ctr, q);
    }
}

// One thread per shadow task (grid-stride over the device-side total).
// direct[t] = sum over lights of albedo * (sum_ls I * T_shadow / ns) * w.
// kEnv = false leaves the environment-light branch out (no light of the
// scene is an environment light), which frees registers for occupancy.
template <int DT, bool kEnv>
__global__ void __launch_bounds__(128, 8) k_shadow(DevScene sc, const ShadowTask* __restrict__ tasks,
                                                const int32_t* __restrict__ total_ptr, int64_t task_cap,
                                                float4* __restrict__ direct, unsigned long long* __restrict__ ctr) {
    const int64_t total = min((int64_t)*total_ptr, task_cap);
    const DevGrid& G = sc.dens;
    const DevShader& sh = sc.sh;
    const float step1 = sc.step1, cutoff = sc.cutoff;
    const float scale = sh.dS * sh.shadowDS;
    uint32_t n_shadow = 0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const ShadowTask tk = tasks[t];
        const Stream stream = make_stream(sc.seed, kDomainPixel | (uint64_t)tk.ps);
        const float pw[3] = {tk.p[0] * G.h + G.wo[0], tk.p[1] * G.h + G.wo[1], tk.p[2] * G.h + G.wo[2]};
        float acc[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < sc.n_lights; ++k) {
            const DevLight& Lk = sc.lights[k];
            float lum[3] = {0.f, 0.f, 0.f};
            for (int ls = 0; ls < Lk.samples; ++ls) {
                const uint32_t sub = shadow_key(stream, tk.n, (uint32_t)k, (uint32_t)ls);
                float ldir[3], I[3], dist;
                if (kEnv && Lk.type == 2) {
                    env_illuminate(sc.env, Lk, draw_sub(sub, kTagEnvU), draw_sub(sub, kTagEnvV), ldir, I);
                    dist = kInf;
                } else {
                    illuminate(Lk, pw, ldir, I, dist);
                }
                IRay srr;
                make_iray(srr, tk.p[0], tk.p[1], tk.p[2], -ldir[0], -ldir[1], -ldir[2], kDelta * G.inv_h,
                          dist * G.inv_h);
                if (!clip_to_bbox(G, srr)) continue;
                LeafDDA sd;
                dda_init(sd, srr, G);
                float sa, sb, tau = 0.f;
                uint32_t sspan = 0, siter = 0;
                bool sdrop = false;
                while (!sdrop && next_span(G, sd, sa, sb)) {
                    float sStep = jitter_step(step1, draw_sub(sub, kTagShadowSpan | sspan));
                    ++sspan;
                    for (float sT = step1 * ceilf(sa / step1); sT <= sb && sT + sStep > sT;) {
                        const uint32_t q = siter++;
                        const float rs = fminf(sample_index_t<DT>(G, srr.e[0] + sT * srr.d[0], srr.e[1] + sT * srr.d[1],
                                                            srr.e[2] + sT * srr.d[2]) * scale,
                                               sh.dMax);
                        if (rs < cutoff) { sT += sStep; continue; }
                        tau += rs * sStep;
                        if (tau > sh.tau_drop) { sdrop = true; break; }
                        sStep = jitter_step(step1, draw_sub(sub, kTagShadowStep | q));
                        sT += sStep;
                    }
                }
                n_shadow += siter;
                if (sdrop) continue;
#pragma unroll
                for (int c = 0; c < 3; ++c) lum[c] += I[c] * __expf(-sh.a[c] * tau);
            }
            const float inv_ns = 1.f / (float)Lk.samples;
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[c] += sh.albedo[c] * (lum[c] * inv_ns) * tk.w[c];
        }
        direct[t] = make_float4(acc[0], acc[1], acc[2], 0.f);
    }
    if (ctr) {
        unsigned long long q = n_shadow;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(ctr + 1, q);
    }
}

// One thread per pixel: the antialiasing average in sample order.
__global__ void __launch_bounds__(128) k_resolve(DevCamera cam, const int32_t* __restrict__ offsets,
                                                 const int32_t* __restrict__ counts,
                                                 const PixelSample* __restrict__ pss,
                                                 const float4* __restrict__ direct, int64_t task_cap,
                                                 float4* __restrict__ rgba, float4* __restrict__ dfilm,
                                                 float4* __restrict__ sfilm, float4* __restrict__ efilm) {
    const int64_t pix = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= (int64_t)cam.width * cam.height) return;
    const float ratio = 1.f / (float)cam.spp;
    float tAA[3] = {0.f, 0.f, 0.f}, lAA[3] = {0.f, 0.f, 0.f}, dAA[3] = {0.f, 0.f, 0.f};
    float sAA[3] = {0.f, 0.f, 0.f}, eAA[3] = {0.f, 0.f, 0.f};
    for (int s = 0; s < cam.spp; ++s) {
        const int64_t ps = pix * cam.spp + s;
        const PixelSample o = pss[ps];
        float d[3] = {0.f, 0.f, 0.f};
        const int64_t b = offsets[ps], e = min((int64_t)b + counts[ps], task_cap);
        for (int64_t t = b; t < e; ++t) {
            const float4 v = direct[t];
            d[0] += v.x;
            d[1] += v.y;
            d[2] += v.z;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            lAA[c] += (d[c] + o.scat[c] + o.emis[c]) * ratio;
            dAA[c] += d[c] * ratio;
            sAA[c] += o.scat[c] * ratio;
            eAA[c] += o.emis[c] * ratio;
            tAA[c] += o.trans[c] * ratio;
        }
    }
    if (rgba) rgba[pix] = make_float4(lAA[0], lAA[1], lAA[2], 1.f - (tAA[0] + tAA[1] + tAA[2]) / 3.f);
    if (dfilm) dfilm[pix] = make_float4(dAA[0], dAA[1], dAA[2], 0.f);
    if (sfilm) sfilm[pix] = make_float4(sAA[0], sAA[1], sAA[2], 0.f);
    if (efilm) efilm[pix] = make_float4(eAA[0], eAA[1], eAA[2], 0.f);
}

cudaError_t launch_render_count(const DevScene& sc, const DevCamera& cam, const DevScatterGrid& sg, int32_t* counts,
                                cudaStream_t st) {
    const int64_t n_ps = (int64_t)cam.width * cam.height * cam.spp;
    if (n_ps == 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((n_ps + 127) / 128);
    if (sc.dens.dtype == 1)
        k_primary<false, 1><<<blocks, 128, 0, st>>>(sc, cam, sg, counts, nullptr, nullptr, 0, nullptr, nullptr);
    else if (sc.dens.dtype == 2)
        k_primary<false, 2><<<blocks, 128, 0, st>>>(sc, cam, sg, counts, nullptr, nullptr, 0, nullptr, nullptr);
    else
        k_primary<false, 0><<<blocks, 128, 0, st>>>(sc, cam, sg, counts, nullptr, nullptr, 0, nullptr, nullptr);
    ++g_launch_counter;
    return cudaGetLastError();
}

// Resident CTAs per SM of the k_shadow instance for (dtype, env), from the
// occupancy calculator (once per instance; it enqueues no work, so it may run
// while a stream is being captured).
static int shadow_ctas_per_sm(int dtype, bool env) {
    static std::atomic<int> cache[3][2];
    std::atomic<int>& c = cache[dtype < 0 || dtype > 2 ? 0 : dtype][env ? 1 : 0];
    if (c.load() == 0) {
        int n = 0;
        cudaError_t e;
        if (env) {
            e = dtype == 1   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shadow<1, true>, 128, 0)
                : dtype == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shadow<2, true>, 128, 0)
                             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shadow<0, true>, 128, 0);
        } else {
            e = dtype == 1   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shadow<1, false>, 128, 0)
                : dtype == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shadow<2, false>, 128, 0)
                             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shadow<0, false>, 128, 0);
        }
        c.store((e == cudaSuccess && n > 0) ? n : 8);
    }
    return c.load();
}

cudaError_t launch_render_shade(const DevScene& sc, const DevCamera& cam, const DevScatterGrid& sg,
                                const int32_t* counts, const int32_t* offsets, const int32_t* total,
                                ShadowTask* tasks, int64_t task_cap, void* pixel_samples, float4* direct,
                                float4* rgba, float4* dfilm, float4* sfilm, float4* efilm,
                                unsigned long long* counters, int sms, cudaStream_t st, cudaEvent_t* marks) {
    const int64_t n_ps = (int64_t)cam.width * cam.height * cam.spp;
    const int64_t n_pix = (int64_t)cam.width * cam.height;
    if (n_ps == 0) return cudaSuccess;
    PixelSample* pss = reinterpret_cast<PixelSample*>(pixel_samples);
    const unsigned blocks = (unsigned)((n_ps + 127) / 128);
    auto mark = [&](int k) {
        if (marks && marks[k]) cudaEventRecord(marks[k], st);
    };
    if (sc.dens.dtype == 1)
        k_primary<true, 1><<<blocks, 128, 0, st>>>(sc, cam, sg, nullptr, offsets, tasks, task_cap, pss, counters);
    else if (sc.dens.dtype == 2)
        k_primary<true, 2><<<blocks, 128, 0, st>>>(sc, cam, sg, nullptr, offsets, tasks, task_cap, pss, counters);
    else
        k_primary<true, 0><<<blocks, 128, 0, st>>>(sc, cam, sg, nullptr, offsets, tasks, task_cap, pss, counters);
    mark(0);
    bool env = false;
    for (int k = 0; k < sc.n_lights; ++k) env = env || sc.lights[k].type == 2;
    // one resident wave of CTAs; the threads stride over the tasks
    const unsigned sblocks = (unsigned)sms * (unsigned)shadow_ctas_per_sm(sc.dens.dtype, env);
    if (env) {
        if (sc.dens.dtype == 1) k_shadow<1, true><<<sblocks, 128, 0, st>>>(sc, tasks, total, task_cap, direct, counters);
        else if (sc.dens.dtype == 2) k_shadow<2, true><<<sblocks, 128, 0, st>>>(sc, tasks, total, task_cap, direct, counters);
        else k_shadow<0, true><<<sblocks, 128, 0, st>>>(sc, tasks, total, task_cap, direct, counters);
    } else {
        if (sc.dens.dtype == 1) k_shadow<1, false><<<sblocks, 128, 0, st>>>(sc, tasks, total, task_cap, direct, counters);
        else if (sc.dens.dtype == 2) k_shadow<2, false><<<sblocks, 128, 0, st>>>(sc, tasks, total, task_cap, direct, counters);
        else k_shadow<0, false><<<sblocks, 128, 0, st>>>(sc, tasks, total, task_cap, direct, counters);
    }
    mark(1);
    k_resolve<<<(unsigned)((n_pix + 127) / 128), 128, 0, st>>>(cam, offsets, counts, pss, direct, task_cap, rgba,
                                                              dfilm, sfilm, efilm);
    mark(2);
    g_launch_counter += 3;
    return cudaGetLastError();
}

size_t pixel_sample_bytes() { return sizeof(PixelSample); }

}  // namespace lg

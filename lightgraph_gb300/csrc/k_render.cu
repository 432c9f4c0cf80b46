// Camera ray march writing the beauty and AOV films:
// VolumeRender::operator() (src/Renderer.h:505-693) with
// PerspectiveCamera::getRay (src/Renderer.h:216-229).
//
// One thread per pixel, its antialiasing samples in order, like the
// reference's per-pixel loop. Per sample: a jittered primary ray marched at
// step[0] with a +-25% jittered step through the density's leaf spans; at each
// sample with density >= cutoff it reads the scatter grid and the temperature
// ramp, and casts one jittered shadow march per light sample. Shadow rays
// accumulate a scalar optical depth (every channel of the reference's
// product of exponentials is exp(-a_c * tau)) and stop when tau passes the
// dropout depth. Random numbers come from counter-based streams keyed by
// (seed, pixel, sample, loop iteration), so a result does not depend on the
// launch shape; the reference's render RNG depends on TBB's row split.
#include "lg_kernels.h"

namespace lg {

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

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
                    c[a][b][d] = ldg4(sg.v + ((int64_t)z * sg.dims[1] + y) * sg.dims[0] + x);
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

__global__ void __launch_bounds__(128) k_render(DevScene sc, DevCamera cam, DevScatterGrid sg,
                                                float4* __restrict__ rgba, float4* __restrict__ direct,
                                                float4* __restrict__ scatter, float4* __restrict__ emission,
                                                unsigned long long* __restrict__ counters) {
    const int i = blockIdx.x * 16 + (threadIdx.x & 15);
    const int j = blockIdx.y * 8 + (threadIdx.x >> 4);
    const bool live = i < cam.width && j < cam.height;
    uint32_t n_primary = 0, n_shadow = 0;
    if (live) {
        const DevGrid& G = sc.dens;
        const DevShader& sh = sc.sh;
        const int64_t pix = (int64_t)j * cam.width + i;
        const float ratio = 1.f / (float)cam.spp;
        float tAA[3] = {0.f, 0.f, 0.f}, lAA[3] = {0.f, 0.f, 0.f}, dAA[3] = {0.f, 0.f, 0.f};
        float sAA[3] = {0.f, 0.f, 0.f}, eAA[3] = {0.f, 0.f, 0.f};
        const float step0 = sc.step0, step1 = sc.step1, cutoff = sc.cutoff;
        for (int s = 0; s < cam.spp; ++s) {
            const Stream stream = make_stream(sc.seed, kDomainPixel | (uint64_t)(pix * cam.spp + s));
            const float jx = draw(stream, kTagJitterX), jy = draw(stream, kTagJitterY);
            // rasterToScreen(i + 0.5 + (u - 0.5), j + 0.5 + (v - 0.5), -1)
            const float sx = (2.f * ((float)i + jx) / (float)cam.width - 1.f) * cam.sw;
            const float sy = (1.f - 2.f * ((float)j + jy) / (float)cam.height) * cam.sh;
            float d[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) d[c] = sx * cam.m[c] + sy * cam.m[3 + c] - cam.m[6 + c];
            const float invl = rsqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            d[0] *= invl; d[1] *= invl; d[2] *= invl;
            const float tscale = 1.f / (d[0] * cam.cdir[0] + d[1] * cam.cdir[1] + d[2] * cam.cdir[2]);
            IRay pr;
            make_iray(pr, (cam.eye[0] - G.wo[0]) * G.inv_h, (cam.eye[1] - G.wo[1]) * G.inv_h,
                      (cam.eye[2] - G.wo[2]) * G.inv_h, d[0], d[1], d[2], cam.znear * tscale * G.inv_h,
                      cam.zfar * tscale * G.inv_h);
            if (!clip_to_bbox(G, pr)) {
                tAA[0] += ratio; tAA[1] += ratio; tAA[2] += ratio;
                continue;
            }
            float pT3[3] = {1.f, 1.f, 1.f};
            float pL[3] = {0.f, 0.f, 0.f}, dL[3] = {0.f, 0.f, 0.f}, sL[3] = {0.f, 0.f, 0.f},
                  eL[3] = {0.f, 0.f, 0.f};
            LeafDDA dda;
            dda_init(dda, pr);
            float ta, tb;
            uint32_t span_ord = 0, n_iter = 0;
            bool pdrop = false;
            while (!pdrop && next_span(G, dda, ta, tb)) {
                float pStep = jitter_step(step0, draw(stream, kTagPrimarySpan | span_ord));
                ++span_ord;
                // (pT + pStep > pT stops a march whose step underflows against pT)
                for (float pT = step0 * ceilf(ta / step0); pT <= tb && pT + pStep > pT;) {
                    const uint32_t n = n_iter++;
                    ++n_primary;
                    const float pi3[3] = {pr.e[0] + pT * pr.d[0], pr.e[1] + pT * pr.d[1], pr.e[2] + pT * pr.d[2]};
                    const float rho = fminf(sample_index(G, pi3[0], pi3[1], pi3[2]) * sh.dS, sh.dMax);
                    if (rho < cutoff) { pT += pStep; continue; }
                    const float pw[3] = {pi3[0] * G.h + G.wo[0], pi3[1] * G.h + G.wo[1], pi3[2] * G.h + G.wo[2]};
                    float sgv[3];
                    sample_scatter(sg, pw[0], pw[1], pw[2], sgv);
                    const float mask = powf(fminf(fmaxf(rho, 0.f), 1.f), sh.mask_power) * sh.scatter_scale;
                    float em[3];
                    const float temp = sc.has_temp ? sample_world(sc.temp, pw[0], pw[1], pw[2]) : 0.f;
                    ramp_color(sh, temp, em);
                    float omdT[3], dT[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float e1 = expm1f(-sh.a[c] * rho * pStep);
                        dT[c] = 1.f + e1;
                        omdT[c] = -e1;
                    }
                    for (int k = 0; k < sc.n_lights; ++k) {
                        const DevLight& Lk = sc.lights[k];
                        float lum[3] = {0.f, 0.f, 0.f};
                        for (int ls = 0; ls < Lk.samples; ++ls) {
                            const uint32_t sub = shadow_key(stream, n, (uint32_t)k, (uint32_t)ls);
                            float ldir[3], I[3], dist;
                            if (Lk.type == 2) {
                                env_illuminate(sc.env, Lk, draw_sub(sub, kTagEnvU), draw_sub(sub, kTagEnvV), ldir, I);
                                dist = kInf;
                            } else {
                                illuminate(Lk, pw, ldir, I, dist);
                            }
                            IRay srr;
                            make_iray(srr, pi3[0], pi3[1], pi3[2], -ldir[0], -ldir[1], -ldir[2], kDelta * G.inv_h,
                                      dist * G.inv_h);
                            if (!clip_to_bbox(G, srr)) continue;
                            LeafDDA sd;
                            dda_init(sd, srr);
                            float sa, sb, tau = 0.f;
                            uint32_t sspan = 0, siter = 0;
                            bool sdrop = false;
                            while (!sdrop && next_span(G, sd, sa, sb)) {
                                float sStep = jitter_step(step1, draw_sub(sub, kTagShadowSpan | sspan));
                                ++sspan;
                                for (float sT = step1 * ceilf(sa / step1); sT <= sb && sT + sStep > sT;) {
                                    const uint32_t q = siter++;
                                    const float rs = fminf(sample_index(G, srr.e[0] + sT * srr.d[0],
                                                                        srr.e[1] + sT * srr.d[1],
                                                                        srr.e[2] + sT * srr.d[2]) *
                                                               sh.dS * sh.shadowDS,
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
                        for (int c = 0; c < 3; ++c) {
                            const float v = sh.albedo[c] * (lum[c] * inv_ns) * pT3[c] * omdT[c];
                            pL[c] += v;
                            dL[c] += v;
                        }
                    }
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float ts = sgv[c] * sh.inv_scatter[c] * mask * pT3[c] * omdT[c];
                        const float te = em[c] * sh.emission_scale * pT3[c] * omdT[c];
                        sL[c] += ts;
                        eL[c] += te;
                        pL[c] += ts + te;
                        pT3[c] *= dT[c];
                    }
                    if (pT3[0] * pT3[0] + pT3[1] * pT3[1] + pT3[2] * pT3[2] < cutoff) { pdrop = true; break; }
                    pStep = jitter_step(step0, draw(stream, kTagPrimaryStep | n));
                    pT += pStep;
                }
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                lAA[c] += pL[c] * ratio;
                dAA[c] += dL[c] * ratio;
                sAA[c] += sL[c] * ratio;
                eAA[c] += eL[c] * ratio;
                tAA[c] += pT3[c] * ratio;
            }
        }
        if (rgba) rgba[pix] = make_float4(lAA[0], lAA[1], lAA[2], 1.f - (tAA[0] + tAA[1] + tAA[2]) / 3.f);
        if (direct) direct[pix] = make_float4(dAA[0], dAA[1], dAA[2], 0.f);
        if (scatter) scatter[pix] = make_float4(sAA[0], sAA[1], sAA[2], 0.f);
        if (emission) emission[pix] = make_float4(eAA[0], eAA[1], eAA[2], 0.f);
    }
    if (counters) {
        // one atomic per warp
        unsigned long long p = n_primary, q = n_shadow;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            p += __shfl_xor_sync(0xffffffffu, p, o);
            q += __shfl_xor_sync(0xffffffffu, q, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(counters, p);
            atomicAdd(counters + 1, q);
        }
    }
}

cudaError_t launch_render(const DevScene& sc, const DevCamera& cam, const DevScatterGrid& sg,
                          float4* rgba, float4* direct, float4* scatter, float4* emission,
                          unsigned long long* counters, cudaStream_t st) {
    if (cam.width <= 0 || cam.height <= 0) return cudaSuccess;
    dim3 grid((cam.width + 15) / 16, (cam.height + 7) / 8);
    k_render<<<grid, 128, 0, st>>>(sc, cam, sg, rgba, direct, scatter, emission, counters);
    ++g_launch_counter;
    return cudaGetLastError();
}

}  // namespace lg

// Edge optical depths (LightGraph::raymarchConnection, src/LightGraph.h:347-418)
// and vertex lighting (LightGraph::computeLighting, src/LightGraph.h:427-505).
//
// The reference accumulates an RGB transmittance sTrans *= exp(ext * x * step)
// per sample. Every channel shares the same x, so the product equals
// exp(ext_c * S) with the scalar S = sum(x * step): these kernels accumulate S
// (FP32) and test the dropout |T|^2 < cutoff as S > tau_drop, the optical depth
// where sum_c exp(2 ext_c S) first falls below the cutoff.
#include "lg_kernels.h"

namespace lg {

// One thread per edge; grid.y = graph.
template <int DT>
__global__ void __launch_bounds__(128) k_edge_march(DevScene sc, const float* __restrict__ pts,
                                                    const GraphInfo* __restrict__ graphs,
                                                    const int2* __restrict__ edges,
                                                    const int32_t* __restrict__ edge_cnt,
                                                    float* __restrict__ S) {
    const GraphInfo g = graphs[blockIdx.y];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= edge_cnt[blockIdx.y]) return;
    const int2 ij = edges[g.e_off + e];
    const float* P = pts + 3 * g.pt_off;
    const float pi[3] = {P[3 * ij.x], P[3 * ij.x + 1], P[3 * ij.x + 2]};
    const float pj[3] = {P[3 * ij.y], P[3 * ij.y + 1], P[3 * ij.y + 2]};
    float d[3] = {pj[0] - pi[0], pj[1] - pi[1], pj[2] - pi[2]};
    const float dist = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    float value = kInf;
    if (dist > 0.f) {
        const float inv = 1.f / dist;
        d[0] *= inv; d[1] *= inv; d[2] *= inv;
        const DevGrid& G = sc.dens;
        IRay r;
        // world ray [Delta, dist] -> index ray (unit direction, times / voxel)
        make_iray(r, (pi[0] - G.wo[0]) * G.inv_h, (pi[1] - G.wo[1]) * G.inv_h,
                  (pi[2] - G.wo[2]) * G.inv_h, d[0], d[1], d[2], kDelta * G.inv_h, dist * G.inv_h);
        const DevShader& sh = sc.sh;
        const float scale = sh.dS * sh.shadowDS * sh.scatterDS;
        const float dmin = sh.scatterDMin, cutoff = sc.cutoff;
        const bool skip_low = dmin < cutoff;
        auto contrib = [&](float rho, float& c) {
            if (rho < cutoff && skip_low) return false;
            c = fmaxf(rho, dmin);
            return true;
        };
        float tau;
        bool dropped;
        uint32_t ns = 0;
        if (march_fixed<DT>(G, r, sc.step1, scale, sh.dMax, sh.tau_drop, contrib, tau, dropped, ns)) {
            value = dropped ? kInf : tau;
        }
    }
    float* M = S + g.s_off;
    M[(int64_t)ij.x * g.ld + ij.y] = value;
    M[(int64_t)ij.y * g.ld + ij.x] = value;
}

// One thread per vertex; grid.y = graph. Output L: 3 floats per vertex.
// Vertex lighting: a group of G lanes per vertex (G a power of two <= 32,
// 32 / G vertices per warp) shares the vertex's R shadow rays (light k's
// samples in order, k = 0, 1, ...): lane l of the group marches rays l,
// l + G, ... and the group's first lane adds their contributions in ray order,
// lum = fmaf(I, T, lum) as a single thread walking the rays in order forms
// it (a missed or dropped ray adds 0 x 0, which leaves a non-negative sum as
// it is). Spreading the rays keeps the warps short: one thread per vertex
// left ~1.2 waves of long, divergent warps at 31 rays per vertex.
template <int DT>
__global__ void __launch_bounds__(128) k_vertex_light(DevScene sc, const float* __restrict__ pts,
                                                      const GraphInfo* __restrict__ graphs,
                                                      float* __restrict__ L, int G, int R) {
    const GraphInfo g = graphs[blockIdx.y];
    const int lane = threadIdx.x & 31, gl = lane & (G - 1);
    const int i = (int)(((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * (32 / G) + lane / G);
    const bool active = i < g.n;  // inactive lanes stay for the shuffles
    float p[3] = {0.f, 0.f, 0.f};
    if (active) {
        const float* P = pts + 3 * (g.pt_off + i);
        p[0] = P[0];
        p[1] = P[1];
        p[2] = P[2];
    }
    const DevGrid& G0 = sc.dens;
    const DevShader& sh = sc.sh;
    const float scale = sh.dS * sh.shadowDS * sh.scatterDS;
    const float cutoff = sc.cutoff;
    auto contrib = [&](float rho, float& c) {
        if (rho < cutoff) return false;
        c = rho;
        return true;
    };
    const Stream stream = make_stream(sc.seed, kDomainVertex | ((uint64_t)blockIdx.y << 32) | (uint32_t)i);
    const float ie[3] = {(p[0] - G0.wo[0]) * G0.inv_h, (p[1] - G0.wo[1]) * G0.inv_h,
                         (p[2] - G0.wo[2]) * G0.inv_h};
    // leader's running sums: light lk's samples so far (lum), lights done (acc)
    float acc[3] = {0.f, 0.f, 0.f}, lum[3] = {0.f, 0.f, 0.f};
    int lk = 0, ls = 0;
    for (int r0 = 0; r0 < R; r0 += G) {
        float rI[3] = {0.f, 0.f, 0.f}, rT[3] = {0.f, 0.f, 0.f};  // intensity, transmittance
        const int r = r0 + gl;
        if (active && r < R) {
            // ray r -> light k, sample s
            int k = 0, s = r;
            for (;;) {
                int nk = sc.lights[k].samples;
                if (nk > 1) nk *= 10;  // env lights are oversampled (src/LightGraph.h:450-452)
                if (s < nk) break;
                s -= nk;
                ++k;
            }
            const DevLight& Lk = sc.lights[k];
            float ldir[3], I[3], dist;
            if (Lk.type == 2) {
                const uint32_t sub = shadow_key(stream, 0, (uint32_t)k, (uint32_t)s);
                env_illuminate(sc.env, Lk, draw_sub(sub, kTagEnvU), draw_sub(sub, kTagEnvV), ldir, I);
                dist = kInf;
            } else {
                illuminate(Lk, p, ldir, I, dist);
            }
            IRay ray;
            make_iray(ray, ie[0], ie[1], ie[2], -ldir[0], -ldir[1], -ldir[2], kDelta * G0.inv_h,
                      dist * G0.inv_h);
            float tau;
            bool dropped;
            uint32_t nsmp = 0;
            // a ray that misses the grid bbox or drops out adds nothing
            if (march_fixed<DT>(G0, ray, sc.step1, scale, sh.dMax, sh.tau_drop, contrib, tau, dropped, nsmp) &&
                !dropped) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    rI[c] = I[c];
                    rT[c] = expf(-sh.a[c] * tau);
                }
            }
        }
        // the leader takes the round's rays in order
        const int nr = min(G, R - r0);
        for (int j = 0; j < nr; ++j) {
            float vI[3], vT[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                vI[c] = __shfl_sync(0xffffffffu, rI[c], j, G);
                vT[c] = __shfl_sync(0xffffffffu, rT[c], j, G);
            }
            if (gl == 0) {
#pragma unroll
                for (int c = 0; c < 3; ++c) lum[c] = fmaf(vI[c], vT[c], lum[c]);
                int nk = sc.lights[lk].samples;
                if (nk > 1) nk *= 10;
                if (++ls == nk) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        acc[c] += sh.albedo[c] * (lum[c] / (float)nk);
                        lum[c] = 0.f;
                    }
                    ++lk;
                    ls = 0;
                }
            }
        }
    }
    if (!active || gl != 0) return;
    float emis[3];
    const float temp = sc.has_temp ? sample_world(sc.temp, p[0], p[1], p[2]) : 0.f;
    ramp_color(sh, temp, emis);
    float* out = L + 3 * (g.pt_off + i);
#pragma unroll
    for (int c = 0; c < 3; ++c) out[c] = acc[c] + emis[c] * sh.emission_scale;
}

cudaError_t launch_edge_march(const DevScene& sc, const float* pts, const GraphInfo* graphs,
                              int n_graphs, int max_edges, const int2* edges,
                              const int32_t* edge_cnt, float* S, cudaStream_t st) {
    if (n_graphs == 0 || max_edges == 0) return cudaSuccess;
    dim3 grid((max_edges + 127) / 128, n_graphs);
    if (sc.dens.dtype == 1) k_edge_march<1><<<grid, 128, 0, st>>>(sc, pts, graphs, edges, edge_cnt, S);
    else if (sc.dens.dtype == 2) k_edge_march<2><<<grid, 128, 0, st>>>(sc, pts, graphs, edges, edge_cnt, S);
    else k_edge_march<0><<<grid, 128, 0, st>>>(sc, pts, graphs, edges, edge_cnt, S);
    ++g_launch_counter;
    return cudaGetLastError();
}

cudaError_t launch_vertex_light(const DevScene& sc, const float* pts, const GraphInfo* graphs,
                                int n_graphs, int max_n, float* L, cudaStream_t st) {
    if (n_graphs == 0 || max_n == 0) return cudaSuccess;
    // rays per vertex, and the lanes per vertex: the power of two >= R, <= 32
    int R = 0;
    for (int k = 0; k < sc.n_lights; ++k) R += sc.lights[k].samples > 1 ? 10 * sc.lights[k].samples : sc.lights[k].samples;
    int G = 1;
    while (G < R && G < 32) G *= 2;
    const int per_block = 128 / 32 * (32 / G);  // vertices per 128-thread block
    dim3 grid((max_n + per_block - 1) / per_block, n_graphs);
    if (sc.dens.dtype == 1) k_vertex_light<1><<<grid, 128, 0, st>>>(sc, pts, graphs, L, G, R);
    else if (sc.dens.dtype == 2) k_vertex_light<2><<<grid, 128, 0, st>>>(sc, pts, graphs, L, G, R);
    else k_vertex_light<0><<<grid, 128, 0, st>>>(sc, pts, graphs, L, G, R);
    ++g_launch_counter;
    return cudaGetLastError();
}

}  // namespace lg

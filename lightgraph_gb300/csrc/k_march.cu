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
template <int DT>
__global__ void __launch_bounds__(128) k_vertex_light(DevScene sc, const float* __restrict__ pts,
                                                      const GraphInfo* __restrict__ graphs,
                                                      float* __restrict__ L) {
    const GraphInfo g = graphs[blockIdx.y];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    const float* P = pts + 3 * (g.pt_off + i);
    const float p[3] = {P[0], P[1], P[2]};
    const DevGrid& G = sc.dens;
    const DevShader& sh = sc.sh;
    float emis[3];
    const float temp = sc.has_temp ? sample_world(sc.temp, p[0], p[1], p[2]) : 0.f;
    ramp_color(sh, temp, emis);
    float acc[3] = {0.f, 0.f, 0.f};
    const float scale = sh.dS * sh.shadowDS * sh.scatterDS;
    const float cutoff = sc.cutoff;
    auto contrib = [&](float rho, float& c) {
        if (rho < cutoff) return false;
        c = rho;
        return true;
    };
    const Stream stream = make_stream(sc.seed, kDomainVertex | ((uint64_t)blockIdx.y << 32) | (uint32_t)i);
    const float ie[3] = {(p[0] - G.wo[0]) * G.inv_h, (p[1] - G.wo[1]) * G.inv_h,
                         (p[2] - G.wo[2]) * G.inv_h};
    for (int k = 0; k < sc.n_lights; ++k) {
        const DevLight& Lk = sc.lights[k];
        int ns = Lk.samples;
        if (ns > 1) ns *= 10;  // env lights are oversampled (src/LightGraph.h:450-452)
        float lum[3] = {0.f, 0.f, 0.f};
        for (int s = 0; s < ns; ++s) {
            float ldir[3], I[3], dist;
            if (Lk.type == 2) {
                const uint32_t sub = shadow_key(stream, 0, (uint32_t)k, (uint32_t)s);
                env_illuminate(sc.env, Lk, draw_sub(sub, kTagEnvU), draw_sub(sub, kTagEnvV), ldir, I);
                dist = kInf;
            } else {
                illuminate(Lk, p, ldir, I, dist);
            }
            IRay r;
            make_iray(r, ie[0], ie[1], ie[2], -ldir[0], -ldir[1], -ldir[2], kDelta * G.inv_h,
                      dist * G.inv_h);
            float tau;
            bool dropped;
            uint32_t nsmp = 0;
            if (!march_fixed<DT>(G, r, sc.step1, scale, sh.dMax, sh.tau_drop, contrib, tau, dropped, nsmp))
                continue;  // shadow ray misses the grid bbox: no contribution
            if (dropped) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) lum[c] += I[c] * expf(-sh.a[c] * tau);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) acc[c] += sh.albedo[c] * (lum[c] / (float)ns);
    }
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
    dim3 grid((max_n + 127) / 128, n_graphs);
    if (sc.dens.dtype == 1) k_vertex_light<1><<<grid, 128, 0, st>>>(sc, pts, graphs, L);
    else if (sc.dens.dtype == 2) k_vertex_light<2><<<grid, 128, 0, st>>>(sc, pts, graphs, L);
    else k_vertex_light<0><<<grid, 128, 0, st>>>(sc, pts, graphs, L);
    ++g_launch_counter;
    return cudaGetLastError();
}

}  // namespace lg

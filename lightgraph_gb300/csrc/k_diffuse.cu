// Radiance diffusion: LightGraph::diffuseLight (src/LightGraph.h:554-587).
//
// After the path solve, P_ij,c = exp(-a_c * S_ij) (the reference's pathGraph
// with its diagonal set to 1, src/LightGraph.h:530-534). The reference makes
// every column energy conserving, c_j = max(sum_i P_ij, 1) per channel, then
// D_i = sum_j L_j * P_ij / c_j. P is never stored: both passes recompute it
// from the FP32 S matrix.
//   k_colsum_partial : column sums over one of kRowChunks row chunks (a
//                      thread per column, so a warp reads a contiguous row
//                      segment);
//   k_colweight      : adds the chunks in a fixed order, w_j = L_j / c_j;
//   k_diffuse_rows   : a warp per row, D_i = sum_j P_ij * w_j.
// Every reduction runs in a fixed order, so results are deterministic.
#include "lg_kernels.h"

namespace lg {

__global__ void __launch_bounds__(128) k_colsum_partial(DevShader sh, const float* __restrict__ S,
                                                        const GraphInfo* __restrict__ graphs,
                                                        float* __restrict__ part) {
    const GraphInfo g = graphs[blockIdx.z];
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.n) return;
    const int rows_per = (g.n + kRowChunks - 1) / kRowChunks;
    const int r0 = blockIdx.y * rows_per, r1 = min(g.n, r0 + rows_per);
    const float* M = S + g.s_off;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    for (int i = r0; i < r1; ++i) {
        const float v = M[(int64_t)i * g.ld + j];
        s0 += __expf(-sh.a[0] * v);
        s1 += __expf(-sh.a[1] * v);
        s2 += __expf(-sh.a[2] * v);
    }
    float* p = part + 3 * ((g.pt_off + j) * kRowChunks + blockIdx.y);
    p[0] = s0;
    p[1] = s1;
    p[2] = s2;
}

__global__ void k_colweight(const GraphInfo* __restrict__ graphs, const float* __restrict__ part,
                            const float* __restrict__ L, float* __restrict__ colw) {
    const GraphInfo g = graphs[blockIdx.y];
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.n) return;
    const int64_t gp = g.pt_off + j;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float s = 0.f;
        for (int k = 0; k < kRowChunks; ++k) s += part[3 * (gp * kRowChunks + k) + c];
        colw[3 * gp + c] = L[3 * gp + c] / fmaxf(s, 1.f);
    }
}

__global__ void __launch_bounds__(256) k_diffuse_rows(DevShader sh, const float* __restrict__ S,
                                                      const GraphInfo* __restrict__ graphs,
                                                      const float* __restrict__ colw,
                                                      float* __restrict__ D) {
    const GraphInfo g = graphs[blockIdx.y];
    const int i = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (i >= g.n) return;
    const float* row = S + g.s_off + (int64_t)i * g.ld;
    const float* w = colw + 3 * g.pt_off;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    for (int j = lane; j < g.n; j += 32) {
        const float v = row[j];
        s0 += __expf(-sh.a[0] * v) * w[3 * j + 0];
        s1 += __expf(-sh.a[1] * v) * w[3 * j + 1];
        s2 += __expf(-sh.a[2] * v) * w[3 * j + 2];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if (lane == 0) {
        float* out = D + 3 * (g.pt_off + i);
        out[0] = s0;
        out[1] = s1;
        out[2] = s2;
    }
}

cudaError_t launch_diffuse(const DevShader& sh, const float* S, const GraphInfo* graphs,
                           int n_graphs, int max_n, const float* L, float* part, float* colw,
                           float* D, cudaStream_t st) {
    if (n_graphs == 0 || max_n == 0) return cudaSuccess;
    k_colsum_partial<<<dim3((max_n + 127) / 128, kRowChunks, n_graphs), 128, 0, st>>>(sh, S, graphs, part);
    ++g_launch_counter;
    k_colweight<<<dim3((max_n + 127) / 128, n_graphs), 128, 0, st>>>(graphs, part, L, colw);
    ++g_launch_counter;
    k_diffuse_rows<<<dim3((max_n + 7) / 8, n_graphs), 256, 0, st>>>(sh, S, graphs, colw, D);
    ++g_launch_counter;
    return cudaGetLastError();
}

}  // namespace lg

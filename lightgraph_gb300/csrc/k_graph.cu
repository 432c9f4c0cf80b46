// Graph construction: LightGraph::buildGraph (src/LightGraph.h:287-318).
//
// The reference loops i = 0..N-1, j = 0..N-1 and connects i < j when
// |p_i - p_j|^2 < r^2 (FP64 on float-valued points) unless either endpoint
// already has max_connect edges. The decision for row i depends only on the
// edge counts left by rows < i, and inside one row every partner j is
// independent, so:
//   1. k_candidates (parallel over rows): the ascending list of j > i with
//      |p_i - p_j|^2 < r^2. The test runs in FP32; only pairs inside a
//      2^-17 relative band of r^2 (where FP32 rounding could disagree with the
//      reference's FP64) are re-tested with FP64 arithmetic.
//   2. k_greedy (one CTA per graph, rows in order): a warp takes the first
//      (max_connect - cnt[i]) candidates whose partner count is below the cap.
#include <algorithm>
#include <mutex>
#include <utility>
#include <vector>

#include "lg_kernels.h"

namespace lg {

__device__ __forceinline__ bool pair_close(const float* pi, const float* pj, float r2, float lo,
                                           float hi) {
    const float dx = pi[0] - pj[0], dy = pi[1] - pj[1], dz = pi[2] - pj[2];
    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    if (d2 < lo) return true;
    if (d2 > hi) return false;
    // near the radius: evaluate exactly as the reference does, in FP64
    // without contraction (Vec3::lengthSqr, x*x + y*y + z*z left to right)
    const double ex = __dsub_rn((double)pi[0], (double)pj[0]);
    const double ey = __dsub_rn((double)pi[1], (double)pj[1]);
    const double ez = __dsub_rn((double)pi[2], (double)pj[2]);
    const double e2 = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
    return e2 < (double)r2;
}

// One warp per row; rows of all graphs in one launch.
__global__ void __launch_bounds__(256) k_candidates(const float* __restrict__ pts,
                                                    const GraphInfo* __restrict__ graphs,
                                                    const int32_t* __restrict__ pt_graph,
                                                    int64_t n_points, uint16_t* __restrict__ cand,
                                                    int32_t* __restrict__ cand_cnt) {
    const int64_t row = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (row >= n_points) return;
    const GraphInfo g = graphs[pt_graph[row]];
    const int i = (int)(row - g.pt_off);
    const float* P = pts + 3 * g.pt_off;
    const float pi[3] = {P[3 * i], P[3 * i + 1], P[3 * i + 2]};
    const float lo = g.r2 * (1.f - 7.62939453125e-06f), hi = g.r2 * (1.f + 7.62939453125e-06f);
    int cnt = 0;
    uint16_t* out = cand + row * kCandCap;
    for (int j0 = i + 1; j0 < g.n; j0 += 32) {
        const int j = j0 + lane;
        bool close = false;
        if (j < g.n) {
            const float pj[3] = {P[3 * j], P[3 * j + 1], P[3 * j + 2]};
            close = pair_close(pi, pj, g.r2, lo, hi);
        }
        const unsigned m = __ballot_sync(0xffffffffu, close);
        const int pos = cnt + __popc(m & ((1u << lane) - 1u));
        if (close && pos < kCandCap) out[pos] = (uint16_t)j;
        cnt += __popc(m);
    }
    if (lane == 0) cand_cnt[row] = cnt;
}

// One CTA per graph. Candidate rows are staged into shared memory in chunks
// of 64 rows, double buffered: warp 0 resolves the rows of one chunk in order
// while warps 1-7 stage the next.
constexpr int kGreedyChunk = 64;
static_assert((kCandCap * sizeof(uint16_t)) % sizeof(uint4) == 0, "candidate rows are copied as 16-byte words");

// A chunk's candidate rows are one contiguous block of rows * kCandCap
// entries whose start, (pt_off + r0) * 192 bytes into the array, is 16-byte
// aligned: it is copied as 16-byte words, every load independent of the
// others (entries past a row's count are copied too and never read).
__device__ __forceinline__ void greedy_stage(const GraphInfo& g, const uint16_t* __restrict__ cand,
                                             const int32_t* __restrict__ cand_cnt, int r0, int rows, uint16_t* cs,
                                             int32_t* cc, int t, int nt) {
    constexpr int kWordsPerRow = kCandCap * (int)sizeof(uint16_t) / (int)sizeof(uint4);
    const uint4* __restrict__ src = reinterpret_cast<const uint4*>(cand + (g.pt_off + r0) * kCandCap);
    uint4* dst = reinterpret_cast<uint4*>(cs);
    const int words = rows * kWordsPerRow;
#pragma unroll 4
    for (int k = t; k < words; k += nt) dst[k] = __ldg(src + k);
    for (int k = t; k < rows; k += nt) cc[k] = cand_cnt[g.pt_off + r0 + k];
}

__global__ void __launch_bounds__(256) k_greedy(const float* __restrict__ pts,
                                                const GraphInfo* __restrict__ graphs,
                                                const uint16_t* __restrict__ cand,
                                                const int32_t* __restrict__ cand_cnt,
                                                int max_connect, int2* __restrict__ edges,
                                                int32_t* __restrict__ edge_cnt) {
    extern __shared__ __align__(16) uint8_t smem[];
    const GraphInfo g = graphs[blockIdx.x];
    const int n = g.n;
    uint16_t* cs2 = reinterpret_cast<uint16_t*>(smem);                       // 2 x chunk x cap
    int32_t* cc2 = reinterpret_cast<int32_t*>(cs2 + 2 * kGreedyChunk * kCandCap);  // 2 x chunk
    uint8_t* cnt = reinterpret_cast<uint8_t*>(cc2 + 2 * kGreedyChunk);        // n
    for (int k = threadIdx.x; k < n; k += blockDim.x) cnt[k] = 0;
    if (n > 0) greedy_stage(g, cand, cand_cnt, 0, min(kGreedyChunk, n), cs2, cc2, threadIdx.x, blockDim.x);
    const int lane = threadIdx.x & 31;
    const float* P = pts + 3 * g.pt_off;
    const float lo = g.r2 * (1.f - 7.62939453125e-06f), hi = g.r2 * (1.f + 7.62939453125e-06f);
    int ecount = 0;  // valid in warp 0
    int2* E = edges + g.e_off;
    for (int r0 = 0, buf = 0; r0 < n; r0 += kGreedyChunk, buf ^= 1) {
        const int rows = min(kGreedyChunk, n - r0);
        __syncthreads();  // chunk r0 staged; the other buffer is free
        const uint16_t* cs = cs2 + buf * kGreedyChunk * kCandCap;
        const int32_t* cc = cc2 + buf * kGreedyChunk;
        if (threadIdx.x >= 32) {
            const int r1 = r0 + kGreedyChunk;
            if (r1 < n)
                greedy_stage(g, cand, cand_cnt, r1, min(kGreedyChunk, n - r1), cs2 + (buf ^ 1) * kGreedyChunk * kCandCap,
                             cc2 + (buf ^ 1) * kGreedyChunk, threadIdx.x - 32, blockDim.x - 32);
        } else {
            for (int r = 0; r < rows; ++r) {
                const int i = r0 + r;
                // the row's candidate count and first 32 candidates do not
                // depend on the edge counts: loaded beside cnt[i]
                const int total = cc[r];
                const int jfirst = cs[r * kCandCap + lane];
                int need = max_connect - (int)cnt[i];
                if (need <= 0) continue;
                const int stored = min(total, kCandCap);
                for (int b = 0; b < stored && need > 0; b += 32) {
                    const int c = b + lane;
                    int j = -1;
                    if (c < stored) j = b == 0 ? jfirst : cs[r * kCandCap + c];
                    const bool elig = j >= 0 && (int)cnt[j] < max_connect;
                    const unsigned m = __ballot_sync(0xffffffffu, elig);
                    const int rank = __popc(m & ((1u << lane) - 1u));
                    if (elig && rank < need) {
                        cnt[j] = cnt[j] + 1;
                        E[ecount + rank] = make_int2(i, j);
                    }
                    const int acc = min(__popc(m), need);
                    need -= acc;
                    ecount += acc;
                    __syncwarp();
                }
                if (need > 0 && total > kCandCap) {
                    // more partners than stored: continue the scan past the last stored one
                    const int jstart = cs[r * kCandCap + kCandCap - 1] + 1;
                    const float pi[3] = {P[3 * i], P[3 * i + 1], P[3 * i + 2]};
                    for (int j0 = jstart; j0 < n && need > 0; j0 += 32) {
                        const int j = j0 + lane;
                        bool elig = false;
                        if (j < n) {
                            const float pj[3] = {P[3 * j], P[3 * j + 1], P[3 * j + 2]};
                            elig = pair_close(pi, pj, g.r2, lo, hi) && (int)cnt[j] < max_connect;
                        }
                        const unsigned m = __ballot_sync(0xffffffffu, elig);
                        const int rank = __popc(m & ((1u << lane) - 1u));
                        if (elig && rank < need) {
                            cnt[j] = cnt[j] + 1;
                            E[ecount + rank] = make_int2(i, j);
                        }
                        const int acc = min(__popc(m), need);
                        need -= acc;
                        ecount += acc;
                        __syncwarp();
                    }
                }
                // cnt[i] is not written back: later rows read only the
                // counts of partners j > their own row, never row i's
            }
        }
    }
    if (threadIdx.x == 0) edge_cnt[blockIdx.x] = ecount;
}

__global__ void k_adjacency(const GraphInfo* __restrict__ graphs, const int2* __restrict__ edges,
                            const int32_t* __restrict__ edge_cnt, uint8_t* __restrict__ adj,
                            const int64_t* __restrict__ adj_off) {
    const GraphInfo g = graphs[blockIdx.y];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= edge_cnt[blockIdx.y]) return;
    const int2 ij = edges[g.e_off + e];
    uint8_t* A = adj + adj_off[blockIdx.y];
    A[(int64_t)ij.x * g.n + ij.y] = 1;
    A[(int64_t)ij.y * g.n + ij.x] = 1;
}

__global__ void k_fill(float* p, int64_t n, float v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = i; k < n; k += stride) p[k] = v;
}

cudaError_t launch_candidates(const float* pts, const GraphInfo* graphs, const int32_t* pt_graph,
                              int64_t n_points, uint16_t* cand, int32_t* cand_cnt,
                              cudaStream_t st) {
    if (n_points == 0) return cudaSuccess;
    const int warps = 8;
    const unsigned blocks = (unsigned)((n_points + warps - 1) / warps);
    k_candidates<<<blocks, warps * 32, 0, st>>>(pts, graphs, pt_graph, n_points, cand, cand_cnt);
    ++g_launch_counter;
    return cudaGetLastError();
}

cudaError_t raise_smem_limit(const void* func) {
    // the limit belongs to the current device's context: one entry per
    // (device, kernel)
    static std::mutex mu;
    static std::vector<std::pair<int, const void*>> done;
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    if (std::find(done.begin(), done.end(), std::make_pair(dev, func)) != done.end()) return cudaSuccess;
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, func);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    if (e == cudaSuccess) done.push_back(std::make_pair(dev, func));
    return e;
}

cudaError_t launch_greedy(const float* pts, const GraphInfo* graphs, int n_graphs, int max_n,
                          const uint16_t* cand, const int32_t* cand_cnt, int max_connect,
                          int2* edges, int32_t* edge_cnt, cudaStream_t st) {
    if (n_graphs == 0) return cudaSuccess;
    const size_t smem = 2 * kGreedyChunk * kCandCap * sizeof(uint16_t) + 2 * kGreedyChunk * sizeof(int32_t) +
                        (size_t)max_n;
    const cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(k_greedy));
    if (e != cudaSuccess) return e;
    k_greedy<<<n_graphs, 256, smem, st>>>(pts, graphs, cand, cand_cnt, max_connect, edges, edge_cnt);
    ++g_launch_counter;
    return cudaGetLastError();
}

cudaError_t launch_adjacency(const GraphInfo* graphs, int n_graphs, int max_edges,
                             const int2* edges, const int32_t* edge_cnt, uint8_t* adj,
                             const int64_t* adj_off, cudaStream_t st) {
    if (n_graphs == 0 || max_edges == 0) return cudaSuccess;
    dim3 grid((max_edges + 127) / 128, n_graphs);
    k_adjacency<<<grid, 128, 0, st>>>(graphs, edges, edge_cnt, adj, adj_off);
    ++g_launch_counter;
    return cudaGetLastError();
}

cudaError_t launch_fill(float* p, int64_t n, float v, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_fill<<<(unsigned)blocks, 256, 0, st>>>(p, n, v);
    ++g_launch_counter;
    return cudaGetLastError();
}

}  // namespace lg

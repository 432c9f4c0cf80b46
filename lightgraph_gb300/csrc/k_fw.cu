// Blocked min-plus Floyd-Warshall: LightGraph::floydAlgo (src/LightGraph.h:512-542).
//
// The reference runs a max-times FW on RGB transmittance T (FP64):
//   T_ij = maxComponent(T_ij, T_ik * T_kj), skipping zero T_ik / T_kj.
// Every channel is T_c = exp(-a_c * S) for one scalar optical depth S (see
// k_march.cu), so the per-channel max-times recurrences are all the same
// min-plus recurrence on S (zero T <-> S = +inf):
//   S_ij = min(S_ij, S_ik + S_kj).
// This file solves that recurrence in FP32 with the 3-phase blocked schedule,
// k-blocks of 64:
//   panel tiles : the diagonal tile is closed in shared memory, then one tile
//                 of the k-block row or column panel (every panel CTA
//                 recomputes the diagonal tile, which saves a launch and a
//                 dependency per round);
//   update tiles: every other element, S_ij = min(S_ij, min_k A_ik + B_kj),
//                 a min-plus product on the CUDA cores. Each thread owns an
//                 8x8 register tile and consumes k in pairs:
//                   s = add.rn.f32x2({A_ik, A_ik+1}, {B_kj, B_k+1,j})
//                   C_ij = min.f32(C_ij, s.x, s.y)        (3-input min)
//                 i.e. 4 FP32 ops in 2 instructions.
// It is not a dense contraction, so tensor cores do not apply.
// All values must be >= 0 (or +inf); then row and column k do not change in
// round k, which makes each round's updates independent of their order.
//
// Two drivers share the tile code:
//   fw_solve         : one matrix, two launches per round (k_fw_panels,
//                      k_fw_update);
//   fw_solve_batched : many matrices of different sizes in ONE persistent
//                      launch (k_fw_persistent). CTAs claim work items from a
//                      queue ordered round by round with a one-round
//                      look-ahead; an item waits (bounded) on the version
//                      counters of the 64 x 64 blocks it reads, whose writers
//                      always come earlier in the queue, so the schedule
//                      cannot deadlock whatever the residency.
#include <algorithm>

#include "lg_kernels.h"

namespace lg {

constexpr int kKB = 64;      // k-block
constexpr int kTile = 128;   // update tile (rows and cols)
constexpr int kApad = 2;     // float2 padding per k-pair row of the A stage

__device__ __forceinline__ float min3f(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Loads of the matrix. The persistent kernel reads data other CTAs wrote
// during the same launch, so it reads through L2 (ld.global.cg), never a
// possibly stale L1 line.
template <bool kL2>
__device__ __forceinline__ float ldm(const float* p) {
    if (kL2) return __ldcg(p);
    return *p;
}
template <bool kL2>
__device__ __forceinline__ float2 ldm2(const float* p) {
    if (kL2) return __ldcg(reinterpret_cast<const float2*>(p));
    return *reinterpret_cast<const float2*>(p);
}
template <bool kL2>
__device__ __forceinline__ float4 ldm4(const float* p) {
    if (kL2) return __ldcg(reinterpret_cast<const float4*>(p));
    return *reinterpret_cast<const float4*>(p);
}

template <bool kL2>
__device__ __forceinline__ float ld_or_inf(const float* d, int n, int ld, int i, int j) {
    return (i < n && j < n) ? ldm<kL2>(d + (int64_t)i * ld + j) : kInf;
}

struct PanelSmem {
    float Dg[kKB][kKB + 1];
    float T[kKB][kKB + 1];
    float rowk[2][kKB];  // row k / column k of the diagonal tile, double buffered
    float colk[2][kKB];
};

// Panel tile b of round kb: 0 = diagonal, 1..nt-1 = row panel, nt..2nt-2 =
// column panel (the diagonal's index skipped). 256 threads, each owning the
// 4x4 elements (ty + 16r, tx + 16c).
//   1. The diagonal tile Dg is closed by 64 FW steps held in registers; step k
//      only needs row k and column k, which do not change in step k, so their
//      owners publish them to shared memory (double buffered, one barrier per
//      step).
//   2. With Dg* closed, the row panel is min(T, Dg* (x) T) and the column panel
//      min(T, T (x) Dg*): every path that leaves the k-block for the last time
//      at k' costs Dg*[k][k'] + T[k'][j], so one min-plus product (no per-k
//      barrier) replaces the 64 sequential panel steps.
template <bool kL2>
// closed_diag: the diagonal block of round kb is already closed in d (the
// persistent schedule closes it once, in its own item), so row and column
// panel tiles load it instead of closing it again.
__device__ __forceinline__ void fw_panel_tile(float* __restrict__ d, int n, int ld, int kb, int b, PanelSmem& sm,
                                              bool closed_diag = false) {
    const int nt = (n + kKB - 1) / kKB;
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    const int K0 = kb * kKB;
    int kind = 0, other = kb;  // 0 diag, 1 row tile (K0, other), 2 col tile (other, K0)
    if (b > 0) {
        int q = b - 1;
        kind = 1;
        if (q >= nt - 1) { kind = 2; q -= nt - 1; }
        other = q < kb ? q : q + 1;
    }
    const int O0 = other * kKB;
    float g[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) g[r][c] = ld_or_inf<kL2>(d, n, ld, K0 + ty + 16 * r, K0 + tx + 16 * c);
    if (kind != 0) {
        for (int e = tid; e < kKB * kKB; e += 256) {
            const int r = e >> 6, c = e & 63;
            sm.T[r][c] = kind == 1 ? ld_or_inf<kL2>(d, n, ld, K0 + r, O0 + c) : ld_or_inf<kL2>(d, n, ld, O0 + r, K0 + c);
        }
    }
    if (kind != 0 && closed_diag) {
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) sm.Dg[ty + 16 * r][tx + 16 * c] = g[r][c];
        __syncthreads();
    } else {
    // publish row 0 and column 0 (owners: ty == 0 row, tx == 0 column)
#pragma unroll
    for (int c = 0; c < 4; ++c)
        if (ty == 0) sm.rowk[0][tx + 16 * c] = g[0][c];
#pragma unroll
    for (int r = 0; r < 4; ++r)
        if (tx == 0) sm.colk[0][ty + 16 * r] = g[r][0];
    __syncthreads();
    // 1. close the diagonal tile in registers
    for (int k = 0; k < kKB; ++k) {
        const int buf = k & 1;
        float rk[4], ck[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) rk[c] = sm.rowk[buf][tx + 16 * c];
#pragma unroll
        for (int r = 0; r < 4; ++r) ck[r] = sm.colk[buf][ty + 16 * r];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) g[r][c] = fminf(g[r][c], ck[r] + rk[c]);
        const int k1 = k + 1;
        if (k1 < kKB) {
            // owners of row k+1 and column k+1 publish them for the next step
            if ((k1 & 15) == ty) {
#pragma unroll
                for (int r = 0; r < 4; ++r)
                    if (ty + 16 * r == k1) {
#pragma unroll
                        for (int c = 0; c < 4; ++c) sm.rowk[buf ^ 1][tx + 16 * c] = g[r][c];
                    }
            }
            if ((k1 & 15) == tx) {
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    if (tx + 16 * c == k1) {
#pragma unroll
                        for (int r = 0; r < 4; ++r) sm.colk[buf ^ 1][ty + 16 * r] = g[r][c];
                    }
            }
        }
        __syncthreads();
    }
    if (kind == 0) {
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int gi = K0 + ty + 16 * r, gj = K0 + tx + 16 * c;
                if (gi < n && gj < n) d[(int64_t)gi * ld + gj] = g[r][c];
            }
        return;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) sm.Dg[ty + 16 * r][tx + 16 * c] = g[r][c];
    __syncthreads();
    }
    // 2. one min-plus product against the closed diagonal tile
    float acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = sm.T[ty + 16 * r][tx + 16 * c];
    if (kind == 1) {
#pragma unroll 4
        for (int k = 0; k < kKB; ++k) {
            float a[4], bb[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) a[r] = sm.Dg[ty + 16 * r][k];
#pragma unroll
            for (int c = 0; c < 4; ++c) bb[c] = sm.T[k][tx + 16 * c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[r][c] = fminf(acc[r][c], a[r] + bb[c]);
        }
    } else {
#pragma unroll 4
        for (int k = 0; k < kKB; ++k) {
            float a[4], bb[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) a[r] = sm.T[ty + 16 * r][k];
#pragma unroll
            for (int c = 0; c < 4; ++c) bb[c] = sm.Dg[k][tx + 16 * c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[r][c] = fminf(acc[r][c], a[r] + bb[c]);
        }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int i = ty + 16 * r, j = tx + 16 * c;
            const int gi = kind == 1 ? K0 + i : O0 + i;
            const int gj = kind == 1 ? O0 + j : K0 + j;
            if (gi < n && gj < n) d[(int64_t)gi * ld + gj] = acc[r][c];
        }
}

// Update tile (ti, tj) of round kb, 128x128. 256 threads = 8 warps (4 x 2),
// each warp 32 x 64, each thread 8 x 8 (rows/cols interleaved so the
// shared-memory fragment loads are conflict-free 128-bit reads).
template <bool kL2>
__device__ __forceinline__ void fw_update_tile(float* __restrict__ d, int n, int ld, int kb, int ti, int tj,
                                               float2* __restrict__ As, float2* __restrict__ Bs) {
    const int I0 = ti * kTile, J0 = tj * kTile, K0 = kb * kKB;
    const int tid = threadIdx.x;
    const bool full = (I0 + kTile <= n) && (J0 + kTile <= n) && (K0 + kKB <= n);

    // stage A = S[I0:I0+128, K0:K0+64] as k-pairs: As[kp][i] = {S[i][2kp], S[i][2kp+1]}
    {
        const int i = tid & 127, h = tid >> 7;
        const int gi = I0 + i;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int kp = h * 16 + 2 * q;
            const int gk = K0 + 2 * kp;
            float4 v;
            if (full) {
                v = ldm4<kL2>(d + (int64_t)gi * ld + gk);
            } else {
                v.x = ld_or_inf<kL2>(d, n, ld, gi, gk);
                v.y = ld_or_inf<kL2>(d, n, ld, gi, gk + 1);
                v.z = ld_or_inf<kL2>(d, n, ld, gi, gk + 2);
                v.w = ld_or_inf<kL2>(d, n, ld, gi, gk + 3);
            }
            As[kp * (kTile + kApad) + i] = make_float2(v.x, v.y);
            As[(kp + 1) * (kTile + kApad) + i] = make_float2(v.z, v.w);
        }
    }
    // stage B = S[K0:K0+64, J0:J0+128] as k-pairs: Bs[kp][j] = {S[2kp][j], S[2kp+1][j]}
    {
        const int j4 = tid & 31;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int kp = (tid >> 5) + 8 * q;
            const int gk = K0 + 2 * kp, gj = J0 + 4 * j4;
            float4 r0, r1;
            if (full) {
                r0 = ldm4<kL2>(d + (int64_t)gk * ld + gj);
                r1 = ldm4<kL2>(d + (int64_t)(gk + 1) * ld + gj);
            } else {
                r0.x = ld_or_inf<kL2>(d, n, ld, gk, gj); r0.y = ld_or_inf<kL2>(d, n, ld, gk, gj + 1);
                r0.z = ld_or_inf<kL2>(d, n, ld, gk, gj + 2); r0.w = ld_or_inf<kL2>(d, n, ld, gk, gj + 3);
                r1.x = ld_or_inf<kL2>(d, n, ld, gk + 1, gj); r1.y = ld_or_inf<kL2>(d, n, ld, gk + 1, gj + 1);
                r1.z = ld_or_inf<kL2>(d, n, ld, gk + 1, gj + 2); r1.w = ld_or_inf<kL2>(d, n, ld, gk + 1, gj + 3);
            }
            float4* dst = reinterpret_cast<float4*>(Bs + kp * kTile + 4 * j4);
            dst[0] = make_float4(r0.x, r1.x, r0.y, r1.y);
            dst[1] = make_float4(r0.z, r1.z, r0.w, r1.w);
        }
    }

    const int warp = tid >> 5, lane = tid & 31;
    const int wy = warp >> 1, wx = warp & 1, ty = lane >> 3, tx = lane & 7;
    const int rbase = wy * 32 + ty * 2;  // rows rbase + 8q + {0,1}
    const int cbase = wx * 64 + tx * 2;  // cols cbase + 16p + {0,1}

    float acc[8][8];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const int gi = I0 + rbase + 8 * q + s;
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                const int gj = J0 + cbase + 16 * p;
                float2 v;
                if (full) {
                    v = ldm2<kL2>(d + (int64_t)gi * ld + gj);
                } else {
                    v.x = ld_or_inf<kL2>(d, n, ld, gi, gj);
                    v.y = ld_or_inf<kL2>(d, n, ld, gi, gj + 1);
                }
                acc[2 * q + s][2 * p] = v.x;
                acc[2 * q + s][2 * p + 1] = v.y;
            }
        }
    }
    __syncthreads();

#pragma unroll 1
    for (int kp = 0; kp < 32; ++kp) {
        float2 a[8], b[8];
        const float4* ap = reinterpret_cast<const float4*>(As + kp * (kTile + kApad) + rbase);
        const float4* bp = reinterpret_cast<const float4*>(Bs + kp * kTile + cbase);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float4 va = ap[4 * q];   // rows rbase + 8q, +1
            a[2 * q] = make_float2(va.x, va.y);
            a[2 * q + 1] = make_float2(va.z, va.w);
            const float4 vb = bp[8 * q];   // cols cbase + 16q, +1
            b[2 * q] = make_float2(vb.x, vb.y);
            b[2 * q + 1] = make_float2(vb.z, vb.w);
        }
#pragma unroll
        for (int r = 0; r < 8; ++r) {
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const float2 s = __fadd2_rn(a[r], b[c]);
                acc[r][c] = min3f(acc[r][c], s.x, s.y);
            }
        }
    }

    // store everything outside the k-block's row and column panels
#pragma unroll
    for (int q = 0; q < 4; ++q) {
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const int gi = I0 + rbase + 8 * q + s;
            if (gi >= n || (gi >= K0 && gi < K0 + kKB)) continue;
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                const int gj = J0 + cbase + 16 * p;
                const bool okx = gj < n && !(gj >= K0 && gj < K0 + kKB);
                const bool oky = gj + 1 < n && !(gj + 1 >= K0 && gj + 1 < K0 + kKB);
                float* dst = d + (int64_t)gi * ld + gj;
                if (okx && oky) {
                    *reinterpret_cast<float2*>(dst) = make_float2(acc[2 * q + s][2 * p], acc[2 * q + s][2 * p + 1]);
                } else {
                    if (okx) dst[0] = acc[2 * q + s][2 * p];
                    if (oky) dst[1] = acc[2 * q + s][2 * p + 1];
                }
            }
        }
    }
}

constexpr size_t kUpdateSmem = sizeof(float2) * 32 * (kTile + kApad) + sizeof(float2) * 32 * kTile;
static_assert(sizeof(PanelSmem) <= kUpdateSmem, "panel tiles reuse the update stage");

__global__ void __launch_bounds__(256) k_fw_panels(float* __restrict__ d, int n, int ld, int kb) {
    __shared__ PanelSmem sm;
    fw_panel_tile<false>(d, n, ld, kb, blockIdx.x, sm);
}

__global__ void __launch_bounds__(256, 2) k_fw_update(float* __restrict__ d, int n, int ld, int kb) {
    extern __shared__ float4 fw_smem[];
    float2* As = reinterpret_cast<float2*>(fw_smem);
    float2* Bs = As + 32 * (kTile + kApad);
    fw_update_tile<false>(d, n, ld, kb, blockIdx.y, blockIdx.x, As, Bs);
}

cudaError_t fw_solve(float* d, int n, int ld, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_fw_update, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kUpdateSmem);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const int nt = (n + kKB - 1) / kKB;
    const int nu = (n + kTile - 1) / kTile;
    for (int kb = 0; kb < nt; ++kb) {
        k_fw_panels<<<2 * nt - 1, 256, 0, st>>>(d, n, ld, kb);
        ++g_launch_counter;
        if (nt > 1) {
            k_fw_update<<<dim3(nu, nu), 256, kUpdateSmem, st>>>(d, n, ld, kb);
            ++g_launch_counter;
        }
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// persistent batched solve
// ---------------------------------------------------------------------------

// Each CTA claims items until the queue is empty. An item is
// {graph, round, kind (0 panel, 1 update), tile}. Every 64 x 64 block of a
// graph has a version counter: the number of rounds whose writes to it are
// done (round r writes each block once, by its panel tile when the block is
// in row or column block r, else by the update tile holding it). An item of
// round r waits for exactly the blocks it reads:
//   panel  (r, X)    : X at version >= r, and block (r, r) at version >= r
//                      for the diagonal item (which closes it) or >= r + 1
//                      for the row and column items (which read it closed);
//   update (r, tile) : its A and B panel blocks (column / row block r) at
//                      version >= r + 1 and its own blocks outside row and
//                      column block r at version >= r.
// The queue is ordered with a one-round look-ahead: the update tiles of round
// r that hold row or column block r + 1 come first, then the panel tiles of
// round r + 1, then the rest of round r's update tiles. Every item's
// dependencies come earlier in the queue, so the holder of the earliest
// unfinished item can always proceed: the schedule cannot deadlock whatever
// the residency, and panels overlap the bulk of the previous round's update.
// Waits spin at most kSpinLimit polls (with nanosleep) and then raise
// err[0] = 1; every CTA checks err[0] before each item, so a stalled queue
// ends the launch instead of hanging the GPU.
constexpr uint32_t kSpinLimit = 1u << 24;  // x ~100-200 ns sleeps: seconds

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Bounded wait for *v >= target; false (and err set) when it gives up.
__device__ __forceinline__ bool wait_version(const uint32_t* v, uint32_t target, uint32_t* err) {
    uint32_t spins = 0;
    while (ld_acquire(v) < target) {
        if (++spins > kSpinLimit || ld_acquire(err) != 0) {
            atomicExch(err, 1u);
            return false;
        }
        __nanosleep(100);
    }
    return true;
}

__global__ void __launch_bounds__(256, 2) k_fw_persistent(float* __restrict__ base, const FwGraph* __restrict__ gs,
                                                          const int4* __restrict__ items, int n_items,
                                                          uint32_t* __restrict__ sync) {
    // sync layout: [0] queue head, [1] error flag, then per graph g the nt^2
    // block versions at sync + 2 + gs[g].vofs (row-major blocks)
    extern __shared__ float4 fw_smem[];
    float2* As = reinterpret_cast<float2*>(fw_smem);
    float2* Bs = As + 32 * (kTile + kApad);
    PanelSmem& psm = *reinterpret_cast<PanelSmem*>(fw_smem);
    __shared__ int s_item;
    __shared__ int s_abort;
    uint32_t* head = sync;
    uint32_t* err = sync + 1;
    for (;;) {
        if (threadIdx.x == 0) {
            s_item = (int)atomicAdd(head, 1u);
            s_abort = ld_acquire(err) != 0;
        }
        __syncthreads();
        const int it = s_item;
        if (it >= n_items || s_abort) break;
        const int4 w = items[it];
        const FwGraph g = gs[w.x];
        uint32_t* ver = sync + 2 + g.vofs;
        const int r = w.y, nt = g.nt;
        if (threadIdx.x == 0) {
            bool ok = true;
            if (w.z == 0) {
                int bi = r, bj = r;  // the block this panel tile writes
                if (w.w > 0) {
                    int q = w.w - 1;
                    const bool col = q >= nt - 1;
                    if (col) q -= nt - 1;
                    const int other = q < r ? q : q + 1;
                    bi = col ? other : r;
                    bj = col ? r : other;
                }
                // the diagonal item waits for its block's round r - 1; row
                // and column panels for the diagonal closed in round r
                ok = wait_version(ver + r * nt + r, (uint32_t)r + (w.w > 0 ? 1u : 0u), err) &&
                     wait_version(ver + bi * nt + bj, (uint32_t)r, err);
            } else {
                const int ti = w.w / g.nu, tj = w.w % g.nu;
                for (int a = 0; a < 2 && ok; ++a) {
                    const int bi = 2 * ti + a, bj = 2 * tj + a;
                    if (bi < nt) ok = wait_version(ver + bi * nt + r, (uint32_t)r + 1u, err);
                    if (ok && bj < nt) ok = wait_version(ver + r * nt + bj, (uint32_t)r + 1u, err);
                }
                for (int a = 0; a < 2 && ok; ++a)
                    for (int c = 0; c < 2 && ok; ++c) {
                        const int bi = 2 * ti + a, bj = 2 * tj + c;
                        if (bi < nt && bj < nt && bi != r && bj != r)
                            ok = wait_version(ver + bi * nt + bj, (uint32_t)r, err);
                    }
            }
            if (!ok) s_abort = 1;
        }
        __syncthreads();
        if (s_abort) break;
        float* d = base + g.off;
        if (w.z == 0) {
            fw_panel_tile<true>(d, g.n, g.ld, r, w.w, psm, /*closed_diag=*/true);
        } else {
            fw_update_tile<true>(d, g.n, g.ld, r, w.w / g.nu, w.w % g.nu, As, Bs);
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) {
            if (w.z == 0) {
                int bi = r, bj = r;
                if (w.w > 0) {
                    int q = w.w - 1;
                    const bool col = q >= nt - 1;
                    if (col) q -= nt - 1;
                    const int other = q < r ? q : q + 1;
                    bi = col ? other : r;
                    bj = col ? r : other;
                }
                atomicAdd(ver + bi * nt + bj, 1u);
            } else {
                const int ti = w.w / g.nu, tj = w.w % g.nu;
                for (int a = 0; a < 2; ++a)
                    for (int c = 0; c < 2; ++c) {
                        const int bi = 2 * ti + a, bj = 2 * tj + c;
                        if (bi < nt && bj < nt && bi != r && bj != r) atomicAdd(ver + bi * nt + bj, 1u);
                    }
            }
        }
    }
}

size_t fw_batched_items(const FwGraph* graphs, int n_graphs, int4* items) {
    int max_nt = 0;
    for (int g = 0; g < n_graphs; ++g) max_nt = std::max(max_nt, graphs[g].nt);
    size_t k = 0;
    auto emit = [&](int g, int r, int kind, int t) {
        if (items) items[k] = make_int4(g, r, kind, t);
        ++k;
    };
    auto panels = [&](int r) {
        for (int g = 0; g < n_graphs; ++g)
            if (r < graphs[g].nt)
                for (int b = 0; b < 2 * graphs[g].nt - 1; ++b) emit(g, r, 0, b);
    };
    // prio: the update tiles of round r holding row or column block r + 1
    auto updates = [&](int r, bool prio) {
        for (int g = 0; g < n_graphs; ++g) {
            const FwGraph& G = graphs[g];
            if (r >= G.nt || G.nt < 2) continue;
            const int tn = (r + 1) / 2;
            for (int t = 0; t < G.nu * G.nu; ++t) {
                const int ti = t / G.nu, tj = t % G.nu;
                const bool p = r + 1 < G.nt && (ti == tn || tj == tn);
                if (p == prio) emit(g, r, 1, t);
            }
        }
    };
    panels(0);
    for (int r = 0; r < max_nt; ++r) {
        updates(r, true);
        panels(r + 1);
        updates(r, false);
    }
    return k;
}

size_t fw_sync_words(const FwGraph* graphs, int n_graphs) {
    size_t w = 2;
    for (int g = 0; g < n_graphs; ++g) w += (size_t)graphs[g].nt * graphs[g].nt;
    return w;
}

cudaError_t fw_solve_batched(float* base, const FwGraph* graphs, const int4* items, int n_items, uint32_t* sync,
                             size_t sync_words, int ctas, cudaStream_t st) {
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_fw_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kUpdateSmem);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    cudaError_t e = cudaMemsetAsync(sync, 0, sizeof(uint32_t) * sync_words, st);
    if (e != cudaSuccess) return e;
    if (n_items == 0) return cudaSuccess;
    k_fw_persistent<<<ctas, 256, kUpdateSmem, st>>>(base, graphs, items, n_items, sync);
    ++g_launch_counter;
    return cudaGetLastError();
}

int fw_persistent_ctas_per_sm() {
    int blocks = 0;
    cudaFuncSetAttribute(k_fw_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kUpdateSmem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_fw_persistent, 256, kUpdateSmem) != cudaSuccess)
        return 1;
    return std::max(blocks, 1);
}

__global__ void k_set_diag(float* __restrict__ S, const GraphInfo* __restrict__ graphs) {
    const GraphInfo g = graphs[blockIdx.y];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g.n) S[g.s_off + (int64_t)i * g.ld + i] = 0.f;
}

cudaError_t launch_set_diag(float* S, const GraphInfo* graphs, int n_graphs, int max_n,
                            cudaStream_t st) {
    if (n_graphs == 0 || max_n == 0) return cudaSuccess;
    k_set_diag<<<dim3((max_n + 255) / 256, n_graphs), 256, 0, st>>>(S, graphs);
    ++g_launch_counter;
    return cudaGetLastError();
}

}  // namespace lg

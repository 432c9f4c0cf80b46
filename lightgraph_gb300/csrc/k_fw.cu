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
//   k_fw_panels : the diagonal tile is closed in shared memory, then each
//                 CTA closes one tile of the k-block row or column panel
//                 (every CTA recomputes the diagonal tile, which saves a
//                 launch and a grid-wide dependency per round);
//   k_fw_update : every other element, S_ij = min(S_ij, min_k A_ik + B_kj),
//                 a min-plus product on the CUDA cores. Each thread owns an
//                 8x8 register tile and consumes k in pairs:
//                   s = add.rn.f32x2({A_ik, A_ik+1}, {B_kj, B_k+1,j})
//                   C_ij = min.f32(C_ij, s.x, s.y)        (3-input min)
//                 i.e. 4 FP32 ops in 2 instructions.
// It is not a dense contraction, so tensor cores do not apply.
// All values must be >= 0 (or +inf); then row and column k do not change in
// round k, which makes each round's updates independent of their order.
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

__device__ __forceinline__ float ld_or_inf(const float* d, int n, int ld, int i, int j) {
    return (i < n && j < n) ? d[(int64_t)i * ld + j] : kInf;
}

// Phases 1 and 2 of round kb. blockIdx.x: 0 = diagonal tile, 1..nt-1 = row
// panel tiles, nt..2nt-2 = column panel tiles (the diagonal's index skipped).
__global__ void __launch_bounds__(256) k_fw_panels(float* __restrict__ d, int n, int ld, int kb) {
    __shared__ float Dg[kKB][kKB + 1];
    __shared__ float T[kKB][kKB + 1];
    const int nt = (n + kKB - 1) / kKB;
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    const int K0 = kb * kKB;
    int kind = 0, other = kb;  // 0 diag, 1 row tile (K0, other), 2 col tile (other, K0)
    if (blockIdx.x > 0) {
        int b = blockIdx.x - 1;
        kind = 1;
        if (b >= nt - 1) { kind = 2; b -= nt - 1; }
        other = b < kb ? b : b + 1;
    }
    const int O0 = other * kKB;
    for (int e = tid; e < kKB * kKB; e += 256) {
        const int r = e >> 6, c = e & 63;
        Dg[r][c] = ld_or_inf(d, n, ld, K0 + r, K0 + c);
        if (kind == 1) T[r][c] = ld_or_inf(d, n, ld, K0 + r, O0 + c);
        if (kind == 2) T[r][c] = ld_or_inf(d, n, ld, O0 + r, K0 + c);
    }
    __syncthreads();
    // phase 1: close the diagonal tile
    for (int k = 0; k < kKB; ++k) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int i = ty + 16 * r;
            const float dik = Dg[i][k];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int j = tx + 16 * c;
                const float v = dik + Dg[k][j];
                if (v < Dg[i][j]) Dg[i][j] = v;
            }
        }
        __syncthreads();
    }
    if (kind == 0) {
        for (int e = tid; e < kKB * kKB; e += 256) {
            const int r = e >> 6, c = e & 63;
            if (K0 + r < n && K0 + c < n) d[(int64_t)(K0 + r) * ld + K0 + c] = Dg[r][c];
        }
        return;
    }
    // phase 2: close one panel tile through the k-block
    for (int k = 0; k < kKB; ++k) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int i = ty + 16 * r;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int j = tx + 16 * c;
                const float v = (kind == 1) ? Dg[i][k] + T[k][j] : T[i][k] + Dg[k][j];
                if (v < T[i][j]) T[i][j] = v;
            }
        }
        __syncthreads();
    }
    for (int e = tid; e < kKB * kKB; e += 256) {
        const int r = e >> 6, c = e & 63;
        const int gi = kind == 1 ? K0 + r : O0 + r;
        const int gj = kind == 1 ? O0 + c : K0 + c;
        if (gi < n && gj < n) d[(int64_t)gi * ld + gj] = T[r][c];
    }
}

// Phase 3 of round kb on a 128x128 tile. 256 threads = 8 warps (4 x 2), each
// warp 32 x 64, each thread 8 x 8 (rows/cols interleaved so the shared-memory
// fragment loads are conflict-free 128-bit reads).
__global__ void __launch_bounds__(256, 2) k_fw_update(float* __restrict__ d, int n, int ld, int kb) {
    extern __shared__ float4 fw_smem[];
    float2* As = reinterpret_cast<float2*>(fw_smem);         // [32][kTile + kApad]
    float2* Bs = As + 32 * (kTile + kApad);                   // [32][kTile]
    const int I0 = blockIdx.y * kTile, J0 = blockIdx.x * kTile, K0 = kb * kKB;
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
                v = *reinterpret_cast<const float4*>(d + (int64_t)gi * ld + gk);
            } else {
                v.x = ld_or_inf(d, n, ld, gi, gk);
                v.y = ld_or_inf(d, n, ld, gi, gk + 1);
                v.z = ld_or_inf(d, n, ld, gi, gk + 2);
                v.w = ld_or_inf(d, n, ld, gi, gk + 3);
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
                r0 = *reinterpret_cast<const float4*>(d + (int64_t)gk * ld + gj);
                r1 = *reinterpret_cast<const float4*>(d + (int64_t)(gk + 1) * ld + gj);
            } else {
                r0.x = ld_or_inf(d, n, ld, gk, gj); r0.y = ld_or_inf(d, n, ld, gk, gj + 1);
                r0.z = ld_or_inf(d, n, ld, gk, gj + 2); r0.w = ld_or_inf(d, n, ld, gk, gj + 3);
                r1.x = ld_or_inf(d, n, ld, gk + 1, gj); r1.y = ld_or_inf(d, n, ld, gk + 1, gj + 1);
                r1.z = ld_or_inf(d, n, ld, gk + 1, gj + 2); r1.w = ld_or_inf(d, n, ld, gk + 1, gj + 3);
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
                    v = *reinterpret_cast<const float2*>(d + (int64_t)gi * ld + gj);
                } else {
                    v.x = ld_or_inf(d, n, ld, gi, gj);
                    v.y = ld_or_inf(d, n, ld, gi, gj + 1);
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

cudaError_t fw_solve_batched(float* base, const int64_t* offs, const int32_t* ns, const int32_t* lds,
                             int n_graphs, int max_n, cudaStream_t st) {
    (void)base; (void)offs; (void)ns; (void)lds; (void)n_graphs; (void)max_n; (void)st;
    return cudaErrorNotSupported;
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

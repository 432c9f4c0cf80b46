// Dart throwing of the LightGraph points: LightGraph::scatterPoints
// (src/LightGraph.h:206-274), the caller-side step that feeds buildGraph.
//
// The reference throws, per iteration, up to scatterCount candidates in
// sequence: three draws of the iteration's mt19937 give a position in the
// active-voxel bbox; every scatterCount / nEstimates candidates the squared
// minimum distance is rescaled by pcSize / expectedSize (the expected sizes
// are computed on the host with the C library's pow, as the reference does);
// a candidate whose trilinear density is below the cutoff is skipped, one
// closer than the minimum distance to an accepted point is rejected, and the
// loop stops once more than targetSize points are accepted.
//
// Here one CTA runs one iteration and reproduces that sequence exactly. It
// takes the candidates a block of 208 at a time (208 x 3 = 624 draws: one
// MT19937 state block; word i >= 227 depends only on word i - 227, so 227
// threads each compute a chain of up to three words, while warp 0 walks the
// previous block), with three barriers per block:
//   1. every thread of a candidate computes its position and its density in
//      FP32, re-tested with the reference's sampler arithmetic (float voxel
//      values, double weights, a float result per interpolation step) when
//      the FP32 value is within its error bound of the cutoff;
//   2. between two radius updates, every density-passing candidate is tested
//      in parallel (a warp per candidate, lanes over the accepted points)
//      against the points accepted before the segment;
//   3. one lane walks the survivors in candidate order, testing each against
//      the points accepted earlier in the same segment, and accepts.
// Distances are compared in FP32 and re-tested in FP64 (the reference's
// arithmetic) when within 2^-18 of the squared radius, so the accepted set
// is the reference's. The accepted points live in shared memory.
#include <algorithm>

#include "lg_kernels.h"
#include "lg_mt.h"

namespace lg {

namespace {

constexpr int kDartThreads = 512;  // >= 227 (the twist chains); 4 CTAs per SM
constexpr int kDartBlock = 208;    // candidates per MT block (3 draws each)
constexpr int kDartWarps = kDartThreads / 32;

// BoxSampler::sample restated as the reference evaluates it: float voxel
// values, double weights, each interpolation rounded to float (z, then y,
// then x). p is the index-space position.
__device__ float sample_exact(const DevGrid& g, double px, double py, double pz) {
    const double fx = floor(px), fy = floor(py), fz = floor(pz);
    const double u = px - fx, w = py - fy, t = pz - fz;
    float v[8];
    const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    if (g.dtype == 0) {
        // FP32 records hold the polynomial: each corner is the first entry
        // (the voxel itself) of its own cell's record
#pragma unroll
        for (int c = 0; c < 8; ++c) v[c] = voxel(g, ix + (c & 1), iy + ((c >> 1) & 1), iz + (c >> 2));
    } else {
        const uint32_t rec = cell_record(g, ix, iy, iz);
        if (g.dtype == 1) ld_cell<1>(g.data, rec, v);
        else ld_cell<2>(g.data, rec, v);
    }
    auto lerp = [](float a, float b, double wt) {
        const double tmp = __dmul_rn((double)__fsub_rn(b, a), wt);
        return __fadd_rn(a, __double2float_rn(tmp));
    };
    // v[a + 2b + 4c] = voxel (x + a, y + b, z + c)
    const float x0 = lerp(lerp(v[0], v[4], t), lerp(v[2], v[6], t), w);
    const float x1 = lerp(lerp(v[1], v[5], t), lerp(v[3], v[7], t), w);
    return lerp(x0, x1, u);
}

// The density test without FP64 in the common case: an FP32 sample, and the
// exact sample_exact when the FP32 value lies within its error bound of the
// cutoff or the FP32 position lies within twice its error of a cell face
// (where the exact position may sit in the neighbouring cell). Inside one
// cell the trilinear sample moves by at most 3 * (max tap - min tap) per voxel
// of position error index_err (FP32 rounding of wo, of 1 / h and of the
// subtraction and product); the seven FP32 interpolations add under 2^-19 of
// the largest tap. For an FP32 record (the polynomial k0 + ...) S = sum of
// |k| over the non-constant terms stands in for the taps' spread: every
// partial derivative is at most S and every tap lies within S of k0, so
// |k0| + S bounds every tap; the coefficients' FP32 differences (54 * 2^-24
// of the largest tap), their four evaluation steps and the exact sample's own
// roundings stay under 4e-6 of |k0| + S, and the bound takes twice that.
__device__ __forceinline__ bool density_passes(const DevGrid& g, const float p[3], const DartParams& prm) {
    const float ix = (p[0] - prm.wo_f[0]) * prm.inv_h_f, iy = (p[1] - prm.wo_f[1]) * prm.inv_h_f,
                iz = (p[2] - prm.wo_f[2]) * prm.inv_h_f;
    const float fx = floorf(ix), fy = floorf(iy), fz = floorf(iz);
    const float u = ix - fx, w = iy - fy, t = iz - fz;
    float v[8];
    const uint32_t rec = cell_record(g, (int)fx, (int)fy, (int)fz);
    float val, spread, mag, rel = 2e-6f;
    if (g.dtype == 0) {
        rel = 8e-6f;
        ld_cell<0>(g.data, rec, v);
        val = trilinear_coefs(v, u, w, t);
        float sum = 0.f;
#pragma unroll
        for (int k = 1; k < 8; ++k) sum += fabsf(v[k]);
        spread = sum * (1.f + 1e-6f);
        mag = fabsf(v[0]) + spread;
    } else {
        if (g.dtype == 1) ld_cell<1>(g.data, rec, v);
        else ld_cell<2>(g.data, rec, v);
        float lo = v[0], hi = v[0];
#pragma unroll
        for (int k = 1; k < 8; ++k) { lo = fminf(lo, v[k]); hi = fmaxf(hi, v[k]); }
        auto lerp = [](float a, float b, float wt) { return fmaf(b - a, wt, a); };
        const float x0 = lerp(lerp(v[0], v[4], t), lerp(v[2], v[6], t), w);
        const float x1 = lerp(lerp(v[1], v[5], t), lerp(v[3], v[7], t), w);
        val = lerp(x0, x1, u);
        spread = hi - lo;
        mag = fmaxf(fabsf(hi), fabsf(lo));
    }
    const float e2 = 2.f * prm.index_err;
    const bool near_face = u < e2 || u > 1.f - e2 || w < e2 || w > 1.f - e2 || t < e2 || t > 1.f - e2;
    const float bound = 3.f * spread * prm.index_err + mag * rel + 1e-30f;
    if (!near_face) {
        if (val < prm.cutoff - bound) return false;
        if (val > prm.cutoff + bound) return true;
    }
    const double dx = ((double)p[0] - prm.wo[0]) / prm.h;
    const double dy = ((double)p[1] - prm.wo[1]) / prm.h;
    const double dz = ((double)p[2] - prm.wo[2]) / prm.h;
    return !(sample_exact(g, dx, dy, dz) < prm.cutoff);
}

// |a - b|^2 < m2 as the reference decides it (double arithmetic on float
// coordinates), with an FP32 fast path outside a 2^-18 relative band.
__device__ __forceinline__ bool closer(const float* a, const float* b, float m2) {
    const float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    const float d2 = dx * dx + dy * dy + dz * dz;
    if (d2 < m2 * (1.f - 3.814697265625e-6f)) return true;
    if (d2 > m2 * (1.f + 3.814697265625e-6f)) return false;
    const double ex = __dsub_rn((double)a[0], (double)b[0]);
    const double ey = __dsub_rn((double)a[1], (double)b[1]);
    const double ez = __dsub_rn((double)a[2], (double)b[2]);
    const double e2 = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
    return e2 < (double)m2;
}

// One MT19937 state block: new[i] = f(old[i], old[i+1], x) with x =
// old[i+397] for i < 227 and new[i-227] after, i = 623 taking new[0] as its
// next. Word i >= 227 depends only on word i - 227, so thread t < 227
// computes the chain t, t + 227, t + 454 alone; word 623 (from new[0] and
// new[396]) is left to the one thread that uses it. t >= 227 does nothing.
__device__ __forceinline__ void mt_twist_block(const uint32_t* cur, uint32_t* nxt, int t) {
    if (t < 0 || t >= 227) return;
    uint32_t x = mt_twist_word(cur[t], cur[t + 1], cur[t + kMtM]);
    nxt[t] = x;
    x = mt_twist_word(cur[t + 227], cur[t + 228], x);
    nxt[t + 227] = x;
    if (t < 169) nxt[t + 454] = mt_twist_word(cur[t + 454], cur[t + 455], x);
}

// The reference's radius update: minDist^2 *= pcSize / expectedSize, in
// double, rounded back to float.
__device__ __forceinline__ void radius_update(float& m2, int pc, uint32_t expected) {
    const double ratio = (double)pc / (double)expected;
    m2 = __double2float_rn(__dmul_rn((double)m2, ratio));
}

__global__ void __launch_bounds__(kDartThreads, 4) k_dart(DevGrid g, DartParams prm, const uint32_t* __restrict__ expected,
                                                          float* __restrict__ out_pts, int32_t* __restrict__ out_count,
                                                          float* __restrict__ out_last_m2) {
    __shared__ uint32_t mt_a[kMtN], mt_b[kMtN];
    __shared__ float cand[kDartBlock][3];
    __shared__ uint8_t dens_ok[kDartBlock], hit[kDartBlock];
    extern __shared__ float acc_pts[];  // hard_limit x 3
    __shared__ int s_pc, s_done;
    __shared__ float s_m2, s_last;

    const int it = prm.first_iter + (int)blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        uint32_t x = prm.seed_base + (uint32_t)it;
        mt_a[0] = x;
        for (int k = 1; k < kMtN; ++k) {
            x = mt_init_word(x, (uint32_t)k);
            mt_a[k] = x;
        }
        s_pc = 0;
        s_done = 0;
        s_m2 = prm.min_dist_sq0;
        s_last = prm.min_dist_sq0;
    }
    __syncthreads();
    uint32_t* cur = mt_a;
    uint32_t* nxt = mt_b;
    mt_twist_block(cur, nxt, tid);
    __syncthreads();
    for (uint32_t base = 0; base < prm.scatter_count; base += kDartBlock) {
        if (s_done) break;
        // the block's words (twisted during the previous walk) become current
        {
            uint32_t* t = cur;
            cur = nxt;
            nxt = t;
        }
        // 1. positions and densities of this block's candidates; a radius
        // update at the block's first candidate is applied alongside by an
        // idle thread (the accepted count is final: the last walk is done)
        if (tid < kDartBlock) {
            // the last word of the block (read only by this candidate, and by
            // the next twist after a barrier)
            if (tid == kDartBlock - 1) cur[kMtN - 1] = mt_twist_word(nxt[kMtN - 1], cur[0], cur[396]);
            const uint32_t n = base + (uint32_t)tid;
            bool ok = false;
            if (n < prm.scatter_count) {
                float p[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const float u = mt_canonical_float(mt_temper(cur[3 * tid + a]));
                    // newPos = float(double(float(u * size)) + bbox.min)
                    p[a] = __double2float_rn(__dadd_rn((double)__fmul_rn(u, prm.bbsize[a]), prm.bbmin[a]));
                    cand[tid][a] = p[a];
                }
                ok = density_passes(g, p, prm);
            }
            dens_ok[tid] = ok;
        } else if (tid == kDartThreads - 1 && (base + 1u) % prm.batch == 0u) {
            radius_update(s_m2, s_pc, expected[base / prm.batch]);
        }
        __syncthreads();
        // 2-3. segments between radius updates (candidate n updates before
        // its tests when (n + 1) % batch == 0): one per block but for the
        // blocks that hold a radius update past their first candidate
        int j0 = 0;
        const int jend = (int)min((uint32_t)kDartBlock, prm.scatter_count - base);
        while (j0 < jend && !s_done) {
            // next boundary after j0: the smallest n > base + j0 with
            // (n + 1) % batch == 0
            const uint32_t m = base + (uint32_t)j0 + 1u;
            const uint64_t nb = ((uint64_t)(m + 1u) + prm.batch - 1u) / prm.batch * prm.batch - 1u;
            const int j1 = (int)min((uint64_t)jend, nb - base);
            if (j0 > 0) {
                // the update belongs to candidate j0, a boundary
                if (tid == 0) radius_update(s_m2, s_pc, expected[(base + j0) / prm.batch]);
                __syncthreads();
            }
            const int p0 = s_pc;
            const float m2 = s_m2;
            // 2. survivors of the points accepted before the segment
            for (int j = j0 + warp; j < j1; j += kDartWarps) {
                bool h = false;
                if (dens_ok[j]) {
                    for (int q0 = 0; q0 < p0 && !h; q0 += 32) {
                        const int q = q0 + lane;
                        const bool c = q < p0 && closer(cand[j], acc_pts + 3 * q, m2);
                        h = __any_sync(0xffffffffu, c);
                    }
                }
                if (lane == 0) hit[j] = h;
            }
            __syncthreads();
            // 3. walk the survivors in order (warp 0; lane 0 accepts); after
            // the block's last segment, warps 1-8 twist the next block's
            // words meanwhile (they read this block's words, which the walk
            // does not touch, and overwrite the previous block's)
            if (warp == 0) {
                for (int c0 = j0; c0 < j1; c0 += 32) {
                    const int j = c0 + lane;
                    const unsigned live = __ballot_sync(0xffffffffu, j < j1 && dens_ok[j] && !hit[j]);
                    if (lane == 0) {
                        unsigned mk = live;
                        while (mk && !s_done) {
                            const int jj = c0 + __ffs(mk) - 1;
                            mk &= mk - 1;
                            bool h = false;
                            for (int q = p0; q < s_pc && !h; ++q) h = closer(cand[jj], acc_pts + 3 * q, m2);
                            if (h) continue;
                            const int k = s_pc;
                            acc_pts[3 * k] = cand[jj][0];
                            acc_pts[3 * k + 1] = cand[jj][1];
                            acc_pts[3 * k + 2] = cand[jj][2];
                            s_pc = k + 1;
                            s_last = m2;
                            // the reference stops at the next candidate once
                            // more than target points are accepted
                            if (s_pc > (int)prm.target || s_pc >= (int)prm.hard_limit) s_done = 1;
                        }
                    }
                    __syncwarp();
                }
            } else if (j1 == jend) {
                mt_twist_block(cur, nxt, tid - 32);
            }
            __syncthreads();
            j0 = j1;
        }
    }
    __syncthreads();
    const int pc = s_pc;
    float* dst = out_pts + (size_t)blockIdx.x * prm.hard_limit * 3;
    for (int k = tid; k < 3 * pc; k += kDartThreads) dst[k] = acc_pts[k];
    if (tid == 0) {
        out_count[blockIdx.x] = pc;
        out_last_m2[blockIdx.x] = s_last;
    }
}

}  // namespace

cudaError_t launch_dart(const DevGrid& g, const DartParams& prm, int n_iter, const uint32_t* expected, float* out_pts,
                        int32_t* out_count, float* out_last_m2, cudaStream_t st) {
    if (n_iter <= 0) return cudaSuccess;
    const size_t smem = sizeof(float) * 3 * prm.hard_limit;
    if (smem > 32 * 1024) {  // with the static arrays, past the default 48 KB
        const cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(k_dart));
        if (e != cudaSuccess) return e;
    }
    k_dart<<<n_iter, kDartThreads, smem, st>>>(g, prm, expected, out_pts, out_count, out_last_m2);
    ++g_launch_counter;
    return cudaGetLastError();
}

}  // namespace lg

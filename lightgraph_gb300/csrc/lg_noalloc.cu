// Radiance diffusion for callers that cannot allocate device memory.
//
// Some callers of this library run where cudaMalloc is off limits: a host
// process that hands the GPU to a memory pool it does not own (the device
// memory is already carved up by a framework's caching allocator or a
// fixed-size arena), a render-farm plugin that must not change the device's
// memory footprint between frames, or code that runs while another component
// holds the allocator. They own their inputs and outputs but cannot get
// scratch space. lg_diffuse_noalloc runs the same diffusion kernels as
// lg_diffuse (k_diffuse.cu) with the scratch in a fixed file-scope __device__
// array instead of context buffers, and calls no allocating routine.
//
// The array holds the partial column sums and column weights for up to
// LG_NOALLOC_MAX_POINTS points (about 1.7 MB) plus one GraphInfo record. Every
// GPU that loads this library keeps it until the process exits. All calls
// share it: calls whose work overlaps on the GPU race on it. The work is
// asynchronous, so a host-side lock around the calls does not order them;
// the caller orders them on the device (one stream, or an event or a
// synchronisation between calls on different streams). Every scratch
// element is written before it is read in each call, so the previous call's
// contents never leak into a result and nothing needs clearing.
#include <mutex>

#include "lg_kernels.h"
#include "lightgraph_c.h"

namespace lg {
namespace {

constexpr int kMaxDevices = 64;

// partial sums [point][chunk][3], then the column weights [point][3]
__device__ __align__(256) float g_noalloc_scratch[(size_t)(kRowChunks + 1) * 3 * LG_NOALLOC_MAX_POINTS];
__device__ __align__(256) GraphInfo g_noalloc_graph;

struct DevicePtrs {
    float* scratch = nullptr;
    GraphInfo* graph = nullptr;
    bool ready = false;
};
DevicePtrs g_ptrs[kMaxDevices];
std::mutex g_ptrs_mu;

// Device addresses of the arrays on the current device. Host code cannot use
// the arrays' names as device pointers (they are host-side stand-ins), so the
// addresses are looked up once per device with that device current.
lg_status device_ptrs(DevicePtrs& out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return LG_ERR_CUDA;
    std::lock_guard<std::mutex> lk(g_ptrs_mu);
    DevicePtrs& p = g_ptrs[dev];
    if (!p.ready) {
        if (cudaGetSymbolAddress(reinterpret_cast<void**>(&p.scratch), g_noalloc_scratch) != cudaSuccess) return LG_ERR_CUDA;
        if (cudaGetSymbolAddress(reinterpret_cast<void**>(&p.graph), g_noalloc_graph) != cudaSuccess) return LG_ERR_CUDA;
        p.ready = true;
    }
    out = p;
    return LG_OK;
}

// One record: a single graph of n points whose matrix starts at the caller's
// pointer, with its points and vectors at row 0.
__global__ void k_noalloc_record(int n, int ld) {
    GraphInfo gi{};
    gi.n = n;
    gi.ld = ld;
    g_noalloc_graph = gi;
}

}  // namespace
}  // namespace lg

using namespace lg;

extern "C" lg_status lg_diffuse_noalloc(const float* dist_device, int n, int ld, const float* light_device,
                                        float* diffuse_device, const double extinction[3], void* stream) {
    if (n < 0 || n > LG_NOALLOC_MAX_POINTS || ld < n || !extinction) return LG_ERR_INVALID;
    if (n > 0 && (!dist_device || !light_device || !diffuse_device)) return LG_ERR_INVALID;
    for (int c = 0; c < 3; ++c)
        if (!(extinction[c] <= 0.0)) return LG_ERR_INVALID;
    if (n == 0) return LG_OK;
    DevicePtrs p;
    const lg_status s = device_ptrs(p);
    if (s != LG_OK) return s;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    // the graph record is written on the device, in stream order, from the
    // kernel's arguments: no host buffer has to outlive this call
    k_noalloc_record<<<1, 1, 0, st>>>(n, ld);
    ++g_launch_counter;
    DevShader sh{};
    for (int c = 0; c < 3; ++c) sh.a[c] = (float)(-extinction[c]);
    float* part = p.scratch;
    float* colw = p.scratch + (size_t)kRowChunks * 3 * LG_NOALLOC_MAX_POINTS;
    const cudaError_t e = launch_diffuse(sh, dist_device, p.graph, 1, n, light_device, part, colw, diffuse_device, st);
    return e == cudaSuccess ? LG_OK : LG_ERR_CUDA;
}

// Allocation-free FP64 invariant sums (sph_invariants_noalloc).
//
// For callers that cannot allocate device memory themselves or let a library
// do it: real-time loops that forbid any allocation after start-up (a
// cudaMalloc can block on the device or fail in the middle of a run), and
// host applications whose own allocator reserves all device memory up front
// (an allocation by a library then fails or escapes the host's accounting).
// The variant needs no context: its scratch is the file-scope device array
// below, sized for at most kNoAllocMaxParticles particles.  Each call copies
// the six sums into the caller's host buffer and synchronises the stream
// before it returns.
//
// Every GPU that loads the library holds the scratch until the process
// exits.  All calls share it: two calls that overlap on the GPU (different
// streams, or different host threads) race on it and must be serialised by
// the caller.  Each call writes every scratch slot it later reads, so no
// slot needs clearing between calls.
#include <cuda_runtime.h>

#include <mutex>

#include "sph_internal.cuh"

namespace sphgb {

namespace {

constexpr int kNaThreads = 256;
constexpr int kNaChunk = 4096;                           // particles per block
constexpr int kNaMaxBlocks = 4096;
constexpr int64_t kNoAllocMaxParticles = (int64_t)kNaChunk * kNaMaxBlocks;  // 16,777,216
constexpr int kNaSums = 6;

// partial sums of every block, then the final sums (kNaSums doubles)
__device__ __align__(256) double g_noalloc_scratch[kNaMaxBlocks * kNaSums + kNaSums];

// Block b sums particles [b*kNaChunk, (b+1)*kNaChunk) in a fixed order, so
// the result does not depend on the launch shape.
__global__ void k_inv_chunks(sph_array_view a, double *scratch) {
    double s[kNaSums] = {0, 0, 0, 0, 0, 0};
    const int64_t base = (int64_t)blockIdx.x * kNaChunk;
    for (int k = threadIdx.x; k < kNaChunk; k += blockDim.x) {
        const int64_t i = base + k;
        if (i >= a.n) break;
        if (a.tag != nullptr && a.tag[i] != SPH_TAG_LOCAL_REAL) continue;
        const double m = a.m[i];
        const double u = ld0(a.u, i), v = ld0(a.v, i), w = ld0(a.w, i);
        s[0] += m;
        s[1] += m * u;
        s[2] += m * v;
        s[3] += m * w;
        s[4] += 0.5 * m * (u * u + v * v + w * w);
        s[5] += 1.0;
    }
    __shared__ double sh[kNaSums][kNaThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < kNaSums; ++q) {
        double x = s[q];
        for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
        if (lane == 0) sh[q][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x < kNaSums) {
        double x = 0.0;
        for (int w2 = 0; w2 < kNaThreads / 32; ++w2) x += sh[threadIdx.x][w2];
        scratch[(int64_t)blockIdx.x * kNaSums + threadIdx.x] = x;
    }
}

__global__ void k_inv_final(const double *scratch, int nblocks, double *out) {
    if (threadIdx.x < kNaSums) {
        double x = 0.0;
        for (int b = 0; b < nblocks; ++b) x += scratch[(int64_t)b * kNaSums + threadIdx.x];
        out[threadIdx.x] = x;
    }
}

// Device address of the scratch, looked up once per device with that
// device current (in host code the array's name is only a stand-in).
constexpr int kMaxDevices = 64;
std::mutex g_sym_mutex;
double *g_sym_addr[kMaxDevices] = {nullptr};

int scratch_address(double **out) {
    int dev = 0;
    SPH_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return set_error(SPH_ERR_NOTSUP, "sph_invariants_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_sym_mutex);
    if (!g_sym_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_check(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_sym_addr[dev] = static_cast<double *>(p);
    }
    *out = g_sym_addr[dev];
    return SPH_OK;
}

}  // namespace

}  // namespace sphgb

using namespace sphgb;

extern "C" int sph_invariants_noalloc(const sph_array_view *a, double *out, void *stream) {
    if (!a || !out) return set_error(SPH_ERR_ARG, "sph_invariants_noalloc: null argument");
    if (a->n < 0) return set_error(SPH_ERR_ARG, "sph_invariants_noalloc: negative count");
    if (a->n > kNoAllocMaxParticles)
        return set_error(SPH_ERR_ARG,
                         "sph_invariants_noalloc: at most 16777216 particles (fixed scratch); "
                         "use sph_invariants for larger arrays");
    if (a->n > 0 && !a->m) return set_error(SPH_ERR_ARG, "sph_invariants_noalloc: mass array required");
    double *scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int nblocks = (int)((a->n + kNaChunk - 1) / kNaChunk);
    double *result = scratch + (int64_t)kNaMaxBlocks * kNaSums;
    if (nblocks > 0) {
        k_inv_chunks<<<nblocks, kNaThreads, 0, st>>>(*a, scratch);
        count_launch();
        SPH_LAUNCH_CHECK("k_inv_chunks");
    }
    k_inv_final<<<1, 32, 0, st>>>(scratch, nblocks, result);
    count_launch();
    SPH_LAUNCH_CHECK("k_inv_final");
    SPH_CUDA(cudaMemcpyAsync(out, result, kNaSums * sizeof(double), cudaMemcpyDeviceToHost, st));
    SPH_CUDA(cudaStreamSynchronize(st));
    return SPH_OK;
}

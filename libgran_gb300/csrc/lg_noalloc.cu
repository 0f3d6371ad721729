// lg_noalloc.cu -- observables of a caller-owned particle state without any device allocation.
//
// lg_get_observables reduces through scratch memory that its handle allocated at creation. Some
// callers of this library cannot allocate device memory when they need these numbers: a serving
// loop that admits work against a fixed device-memory budget and must not let a diagnostic grow
// its footprint, a host framework whose own caching allocator holds the device memory the state
// lives in, and code that must not stall other streams (cudaMalloc and cudaFree can synchronise
// the device). lg_observables_noalloc serves them: it reads x, v and omega from device buffers
// the caller owns, writes the results to a device buffer the caller owns, and keeps its
// per-block partial sums in the file-scope array below, which every GPU that loads this library
// holds until the process exits.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "lg_common.cuh"
#include "lg_engine_internal.h"

namespace lg {
namespace {

constexpr int kNaThreads = 256;   // particles per block
constexpr int kNaMaxBlocks = 4096;  // rows of partial sums: one per block, plus one for the totals
constexpr int64_t kNaMaxParticles = (int64_t)(kNaMaxBlocks - 1) * kNaThreads;  // 1,048,320
constexpr int kNaCols = 16;         // sums per row
constexpr int kNaMaxDevices = 64;

// One row of kNaCols partial sums per block (4096 x 16 doubles = 512 KiB per device). Every entry
// that a call reads is written earlier in the same call, so nothing has to be cleared between calls.
__device__ __align__(256) double g_noalloc_partials[kNaMaxBlocks * kNaCols];

// Host-side handle to the array: its device address per device (refreshed by every call made
// outside a stream capture).
std::mutex g_na_mu;
double *g_na_ptr[kNaMaxDevices] = {nullptr};

__device__ __forceinline__ d3 ld3(const double *p, int64_t i) { return mk3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }

// Block tree reduction of one value per thread; thread 0 returns the block's sum.
__device__ __forceinline__ double block_sum(double v, double *sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = kNaThreads / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

// Pass 1: per-block sums of the terms of test/compute_energy.cpp:7-58 and the positions
// (columns 0 e_tot, 1 m|v|^2, 2 I|w|^2, 3-5 v, 6-8 I w, 9-11 x cross m v, 12-14 x).
__global__ void __launch_bounds__(kNaThreads) na_terms(int64_t n, const double *__restrict__ x,
                                                       const double *__restrict__ v, const double *__restrict__ w,
                                                       double m, double I, double *__restrict__ part) {
    __shared__ double sh[kNaThreads];
    const int64_t i = blockIdx.x * (int64_t)kNaThreads + threadIdx.x;
    double t[15];
#pragma unroll
    for (int c = 0; c < 15; ++c) t[c] = 0.0;
    if (i < n) {
        const d3 vi = ld3(v, i), wi = ld3(w, i), xi = ld3(x, i);
        t[0] = m * dot(vi, vi) / 2.0 + I * dot(wi, wi) / 2.0;
        t[1] = m * dot(vi, vi);
        t[2] = I * dot(wi, wi);
        t[3] = vi.x; t[4] = vi.y; t[5] = vi.z;
        const d3 Iw = scl(I, wi);
        t[6] = Iw.x; t[7] = Iw.y; t[8] = Iw.z;
        const d3 L = crs(xi, scl(m, vi));
        t[9] = L.x; t[10] = L.y; t[11] = L.z;
        t[12] = xi.x; t[13] = xi.y; t[14] = xi.z;
    }
    for (int c = 0; c < 15; ++c) {
        const double r = block_sum(t[c], sh);
        if (threadIdx.x == 0) part[blockIdx.x * kNaCols + c] = r;
    }
}

// Pass 2 (one block): fixed-order sums over the block rows; writes the centre of mass to
// out[5..7] and the column sums to res[0..14] (res lives in the partials array, row nblocks).
__global__ void __launch_bounds__(kNaThreads) na_combine(int64_t n, int nblocks, double *__restrict__ part,
                                                         double *__restrict__ out) {
    __shared__ double sh[kNaThreads];
    double *res = part + (int64_t)nblocks * kNaCols;
    for (int c = 0; c < 15; ++c) {
        double acc = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += kNaThreads) acc += part[b * kNaCols + c];
        const double r = block_sum(acc, sh);
        if (threadIdx.x == 0) res[c] = r;
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; ++k) out[5 + k] = res[12 + k] / (double)n;
}

// Pass 3: per-block sums of |x - c|^2 (test/mass_distribution.cpp:17-27) into column 15.
__global__ void __launch_bounds__(kNaThreads) na_gyration(int64_t n, const double *__restrict__ x,
                                                          const double *__restrict__ out, double *__restrict__ part) {
    __shared__ double sh[kNaThreads];
    const int64_t i = blockIdx.x * (int64_t)kNaThreads + threadIdx.x;
    double t = 0.0;
    if (i < n) {
        const d3 q = sub(ld3(x, i), mk3(out[5], out[6], out[7]));
        t = dot(q, q);
    }
    const double r = block_sum(t, sh);
    if (threadIdx.x == 0) part[blockIdx.x * kNaCols + 15] = r;
}

// Pass 4 (one block): final values.
__global__ void __launch_bounds__(kNaThreads) na_finish(int64_t n, int nblocks, double m, double *__restrict__ part,
                                                        double *__restrict__ out) {
    __shared__ double sh[kNaThreads];
    const double *res = part + (int64_t)nblocks * kNaCols;
    double acc = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += kNaThreads) acc += part[b * kNaCols + 15];
    const double rg2 = block_sum(acc, sh);
    if (threadIdx.x != 0) return;
    out[0] = res[1] / 2.0;  // translational kinetic energy
    out[1] = res[2] / 2.0;  // rotational kinetic energy
    out[2] = res[0];        // total kinetic energy
    out[3] = m * sqrt((res[3] * res[3] + res[4] * res[4]) + res[5] * res[5]);
    const double L0 = res[6] + res[9], L1 = res[7] + res[10], L2 = res[8] + res[11];
    out[4] = sqrt((L0 * L0 + L1 * L1) + L2 * L2);
    out[8] = sqrt(rg2 / (double)n);
}

}  // namespace
}  // namespace lg

// Defined here, declared in include/libgran_gb300.h. See the comment at the top of this file.
extern "C" int lg_observables_noalloc(const double *x, const double *v, const double *omega, int64_t n, double mass,
                                      double inertia, double *out, void *stream) {
    using namespace lg;
    if (!x || !v || !omega || !out) return lg_fail(LG_E_INVALID, "lg_observables_noalloc: null pointer");
    if (n < 1 || n > kNaMaxParticles)
        return lg_fail(LG_E_INVALID,
                       "lg_observables_noalloc: n = %lld is outside [1, %lld]; its fixed scratch holds partial sums "
                       "for at most %d blocks of %d particles",
                       (long long)n, (long long)kNaMaxParticles, kNaMaxBlocks - 1, kNaThreads);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return lg_fail(LG_E_CUDA, "lg_observables_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kNaMaxDevices) return lg_fail(LG_E_INVALID, "lg_observables_noalloc: device %d not supported", dev);
    cudaStream_t st = (cudaStream_t)stream;
    double *part = nullptr;
    {
        // set-up with the device current: the device address of the array. The first call on a
        // device looks it up; later calls look it up again unless the stream is being captured, so
        // that an address cached before a cudaDeviceReset (after which the module is loaded anew
        // and the array can move) is not used; a captured call uses the address cached by an
        // earlier call outside the capture.
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
            cudaGetLastError();
            cs = cudaStreamCaptureStatusActive;  // cannot tell: treat as captured, look nothing up
        }
        std::lock_guard<std::mutex> lk(g_na_mu);
        if (cs == cudaStreamCaptureStatusNone || !g_na_ptr[dev]) {
            if (cs != cudaStreamCaptureStatusNone)
                return lg_fail(LG_E_STATE, "lg_observables_noalloc: the first call on device %d must come before any "
                                           "stream capture (it looks up the address of its scratch array)", dev);
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_partials);
            if (e != cudaSuccess)
                return lg_fail(LG_E_CUDA, "lg_observables_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            g_na_ptr[dev] = (double *)p;
        }
        part = g_na_ptr[dev];
    }
    const int nblocks = (int)((n + kNaThreads - 1) / kNaThreads);  // <= kNaMaxBlocks - 1: row nblocks is free
    na_terms<<<nblocks, kNaThreads, 0, st>>>(n, x, v, omega, mass, inertia, part);
    na_combine<<<1, kNaThreads, 0, st>>>(n, nblocks, part, out);
    na_gyration<<<nblocks, kNaThreads, 0, st>>>(n, x, out, part);
    na_finish<<<1, kNaThreads, 0, st>>>(n, nblocks, mass, part, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return lg_fail(LG_E_CUDA, "lg_observables_noalloc: launch: %s", cudaGetErrorString(e));
    return LG_OK;
}

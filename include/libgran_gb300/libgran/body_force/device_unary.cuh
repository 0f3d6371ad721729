// device_unary.cuh (libgran_gb300) -- a user-defined unary force functor evaluated on the GPU.
//
// libgran evaluates user functors (Custom-unary-force-model.md:66-104) on the CPU through their
// operator(). Here the functor is a __device__ callable compiled into the caller's own kernel
// (nvcc), which the engine launches through its unary hook (lg_set_unary_hook) on its stream at
// every force evaluation, after the drift; the terms join the unary fold after the facets, as the
// last functor of the container. F is copied into the kernel's parameters when it is launched or
// captured into a CUDA graph, so a change of its data needs attach() again (which drops the graphs).
//
//   struct my_force {
//       double g;
//       __device__ void operator()(int64_t i, const lg_unary_hook_args &s, double a[3], double alpha[3]) const {
//           a[2] = -g;  // s.x[4*i + k], s.v[...], s.theta[...], s.omega[...]: component k of particle i
//       }
//   };
//   libgran_gb300::device_unary<my_force> f{my_force{9.81}};
//   f.attach(sys);              // or put f into the drop-in unary_force_functor_container
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "../../../libgran_gb300.h"

namespace libgran_gb300 {

template <typename F>
__global__ void device_unary_kernel(F f, lg_unary_hook_args s) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    double a[3] = {0.0, 0.0, 0.0}, alpha[3] = {0.0, 0.0, 0.0};
    f(i, s, a, alpha);
    for (int k = 0; k < 3; ++k) {
        s.a_out[4 * i + k] = a[k];
        s.alpha_out[4 * i + k] = alpha[k];
    }
}

template <typename F>
struct device_unary {
    F f;

    static int launch(const lg_unary_hook_args *s, void *user) {
        const device_unary *self = static_cast<const device_unary *>(user);
        const int threads = 128;
        const int64_t blocks = (s->n + threads - 1) / threads;
        if (blocks > 0)
            device_unary_kernel<F><<<(unsigned)blocks, threads, 0, (cudaStream_t)s->stream>>>(self->f, *s);
        return cudaGetLastError() == cudaSuccess ? 0 : 1;
    }
    int attach(lg_system *sys) { return lg_set_unary_hook(sys, &device_unary::launch, this); }
};

}  // namespace libgran_gb300

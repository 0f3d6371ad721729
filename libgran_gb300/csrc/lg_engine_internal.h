// lg_engine_internal.h -- the handle behind the opaque lg_system pointer of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "lg_kernels.h"

struct lg_system {
    int device = -1;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    lg_system_desc desc{};
    lg::Params P{};
    int precision = LG_PRECISION_FP64;
    bool facet_auto_move = false;

    // state (32-byte slots); v and w ping-pong between the half-step and full-step buffers
    lg::dbl4 *x = nullptr, *th = nullptr, *a = nullptr, *al = nullptr;
    lg::dbl4 *v[2] = {nullptr, nullptr}, *w[2] = {nullptr, nullptr};
    int vcur = 0;
    double *sxi = nullptr;               // surface springs
    double *fv[2] = {nullptr, nullptr};  // facet vertices (current / next)
    int fcur = 0;
    int32_t *err = nullptr;

    // pairs and bonds
    lg::PairView pv[2]{};
    int pcur = 0;
    bool list_built = false;
    int64_t max_cells = 0;
    lg::ListScratch ls{};
    lg::BondView bv{};
    std::vector<int32_t> host_bond_j;
    int64_t n_bonds_initial = 0;

    // observables
    double *obs_scratch = nullptr;
    double *obs_out = nullptr;

    // mixed precision: FP32 position copy for culling
    float4 *x32 = nullptr;
    double origin[3] = {0.0, 0.0, 0.0};
    lg::MixedExtra mx{};

    // force-kernel timing (bench instrumentation)
    bool timing = false;
    std::vector<cudaEvent_t> tev;  // pairs: start, stop
    size_t tev_used = 0;

    int T = 1;  // lanes per row group of the force kernel
    int kernel = LG_FORCE_KERNEL_ROWGROUP;  // resolved force kernel
    int64_t step_index = 0;
    int64_t launches = 0;
    std::vector<void *> allocations;

    template <typename U>
    int alloc(U **p, size_t count);
    void release();
};

int lg_fail(int code, const char *fmt, ...);

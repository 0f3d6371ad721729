// gb300_functor_base.h -- shared pieces of the libgran_gb300 C++ drop-in headers.
//
// These headers keep libgran's class templates, names and constructor signatures (the paths under
// include/libgran_gb300/libgran/ mirror libgran's include/libgran/), but a functor here only records
// its parameters: the pair forces are evaluated by the GPU engine behind the C ABI
// (include/libgran_gb300.h). field_value_t must offer operator[](int) and construction from three
// components, as Eigen::Vector3d does.
#pragma once
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../libgran_gb300.h"

namespace libgran_gb300 {

// Arithmetic of the force kernel used by granular_system objects created after the call.
inline int &default_precision() {
    static int p = LG_PRECISION_FP64;
    return p;
}

inline void check(int status, const char *what) {
    if (status != LG_OK) throw std::runtime_error(std::string(what) + ": " + lg_last_error());
}

template <typename field_value_t>
inline std::vector<double> to_aos(std::vector<field_value_t> const &v) {
    std::vector<double> out(3 * v.size());
    for (size_t i = 0; i < v.size(); ++i)
        for (int c = 0; c < 3; ++c) out[3 * i + c] = v[i][c];
    return out;
}

template <typename field_value_t>
inline void from_aos(std::vector<double> const &a, std::vector<field_value_t> &out) {
    const size_t n = a.size() / 3;
    out.resize(n);
    for (size_t i = 0; i < n; ++i) out[i] = field_value_t(a[3 * i], a[3 * i + 1], a[3 * i + 2]);
}

// The engine handle a functor is bound to once a granular_system has been built from it.
struct binding {
    lg_system *sys = nullptr;
    int32_t facet = -1;
};

}  // namespace libgran_gb300

// unary_force_container.h (libgran_gb300 drop-in) -- unary_force_functor_container, as libgran's
// granular_system/unary_force_container.h:14-35 (triangular facets are its functors here).
#ifndef LIBGRAN_UNARY_FORCE_CONTAINER_H
#define LIBGRAN_UNARY_FORCE_CONTAINER_H
#include <tuple>
#include <vector>

template <typename field_value_t, typename real_t, typename... unary_force_functors_t>
struct unary_force_functor_container {
    typedef std::vector<field_value_t> field_container_t;
    unary_force_functor_container(unary_force_functors_t &...force_functors) : unary_force_functors{force_functors...} {}
    std::tuple<unary_force_functors_t &...> unary_force_functors;
};

#endif

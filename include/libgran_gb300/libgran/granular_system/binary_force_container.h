// binary_force_container.h (libgran_gb300 drop-in) -- binary_force_functor_container holding
// references to the functors, as libgran's granular_system/binary_force_container.h:14-35.
#ifndef LIBGRAN_BINARY_FORCE_CONTAINER_H
#define LIBGRAN_BINARY_FORCE_CONTAINER_H
#include <tuple>
#include <vector>

template <typename field_value_t, typename real_t, typename... binary_force_functors_t>
struct binary_force_functor_container {
    typedef std::vector<field_value_t> field_container_t;
    binary_force_functor_container(binary_force_functors_t &...force_functors)
        : binary_force_functors{force_functors...} {}
    std::tuple<binary_force_functors_t &...> binary_force_functors;
};

#endif

// granular_system_neighbor_list.h (libgran_gb300 drop-in) -- granular_system_neighbor_list with
// libgran's constructor (granular_system/granular_system_neighbor_list.h:54-64): pairs come from a
// GPU Verlet list of radius r_verlet, rebuilt by update_neighbor_list() (test/hamaker_neighbor.cpp:122)
// with spring history carried across rebuilds.
#ifndef LIBGRAN_GRANULAR_SYSTEM_NEIGHBOR_LIST_H
#define LIBGRAN_GRANULAR_SYSTEM_NEIGHBOR_LIST_H
#include "granular_system.h"

template <typename field_value_t, typename real_t,
          template <typename _field_container_t, typename _field_value_t, typename _real_t, typename _functor_t,
                    template <typename __field_container_t, typename __field_value_t> typename _step_handler_t>
          typename integrator_t,
          template <typename _field_container_t, typename _field_value_t> typename step_handler_t,
          typename binary_force_functor_container_t, typename unary_force_functor_container_t>
class granular_system_neighbor_list
    : public granular_system<field_value_t, real_t, integrator_t, step_handler_t, binary_force_functor_container_t,
                             unary_force_functor_container_t> {
    using base = granular_system<field_value_t, real_t, integrator_t, step_handler_t, binary_force_functor_container_t,
                                 unary_force_functor_container_t>;

public:
    typedef std::vector<field_value_t> field_container_t;

    granular_system_neighbor_list(long n_part [[maybe_unused]], real_t r_verlet, field_container_t x0,
                                  field_container_t v0, field_container_t theta0, field_container_t omega0,
                                  real_t t0 [[maybe_unused]], field_value_t field_zero [[maybe_unused]],
                                  real_t real_zero [[maybe_unused]],
                                  step_handler_t<field_container_t, field_value_t> &step_handler,
                                  binary_force_functor_container_t binary_force_functors,
                                  unary_force_functor_container_t unary_force_functors)
        : base(LG_PAIRS_VERLET, (double)r_verlet, std::move(x0), std::move(v0), std::move(theta0), std::move(omega0),
               binary_force_functors, unary_force_functors,
               [&step_handler](size_t n) { return libgran_gb300::hold_of(step_handler, n); }) {}

    void update_neighbor_list() { libgran_gb300::check(lg_update_neighbor_list(this->sys), "update_neighbor_list"); }
};

#endif

// limited_range_hamaker_force.h (libgran_gb300 drop-in) -- limited_range_hamaker_functor, constructor
// as in libgran's hamaker_force/limited_range_hamaker_force.h:20-27.
#ifndef LIBGRAN_LIMITED_RANGE_HAMAKER_FORCE_H
#define LIBGRAN_LIMITED_RANGE_HAMAKER_FORCE_H
#include "../gb300_functor_base.h"

template <typename field_value_t, typename real_t>
struct limited_range_hamaker_functor {
    limited_range_hamaker_functor(real_t A, real_t h0, real_t r_cutoff, real_t r_part, real_t mass,
                                  field_value_t field_zero [[maybe_unused]], real_t real_zero [[maybe_unused]])
        : params{(double)A, (double)h0, (double)r_cutoff, (double)r_part, (double)mass} {}

    static constexpr int mode = LG_HAMAKER_LIMITED;
    lg_hamaker_params params;
};

#endif

// simplified_hamaker_force.h (libgran_gb300 drop-in) -- simplified_hamaker_functor, constructor as in libgran's hamaker_force/simplified_hamaker_force.h:10-16.
#ifndef LIBGRAN_SIMPLIFIED_HAMAKER_FORCE_H
#define LIBGRAN_SIMPLIFIED_HAMAKER_FORCE_H
#include "../gb300_functor_base.h"

template <typename field_value_t, typename real_t>
struct simplified_hamaker_functor {
    simplified_hamaker_functor(real_t A, real_t h0, real_t r_part, real_t mass, field_value_t field_zero [[maybe_unused]],
         real_t real_zero [[maybe_unused]])
        : params{(double)A, (double)h0, 0.0, (double)r_part, (double)mass} {}

    static constexpr int mode = LG_HAMAKER_SIMPLIFIED;
    lg_hamaker_params params;
};

#endif

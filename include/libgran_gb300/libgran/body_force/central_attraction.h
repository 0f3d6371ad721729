// central_attraction.h (libgran_gb300 drop-in) -- the central_attraction_functor of libgran's custom
// unary force tutorial (Custom-unary-force-model.md:108-118, 120-128) with its constructor and
// update_center_of_mass(), evaluated by the engine as the body force LG_BODY_CENTRAL:
// a = k_a / mass * (x0 - x_i), alpha = 0, folded after the facets of the unary container.
// update_center_of_mass(x) computes the centroid as the tutorial does (sum in index order, then
// division by the count) and hands it to the engine; before the first call the centre is the zero
// field.
#ifndef LIBGRAN_GB300_CENTRAL_ATTRACTION_H
#define LIBGRAN_GB300_CENTRAL_ATTRACTION_H
#include <vector>
#include "../gb300_functor_base.h"

template <typename field_value_t, typename real_t>
struct central_attraction_functor {
    central_attraction_functor(central_attraction_functor const &) = delete;

    central_attraction_functor(real_t r [[maybe_unused]], real_t k_a, real_t mass, field_value_t zero_field)
        : zero_field(zero_field) {
        body.model = LG_BODY_CENTRAL;
        body.k_a = (double)k_a;
        body.mass = (double)mass;
        for (int c = 0; c < 3; ++c) body.centre[c] = (double)zero_field[c];
    }

    void update_center_of_mass(std::vector<field_value_t> const &x) {
        field_value_t x0_new = zero_field;
        for (auto const &point : x) x0_new += point;
        field_value_t x0 = x0_new / real_t(x.size());
        for (int c = 0; c < 3; ++c) body.centre[c] = (double)x0[c];
        if (bound.sys) libgran_gb300::check(lg_set_body_centre(bound.sys, body.centre), "update_center_of_mass");
    }

    lg_body_force body{};
    field_value_t zero_field;
    libgran_gb300::binding bound;
};

#endif

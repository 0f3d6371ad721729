// surface_contact_force.h (libgran_gb300 drop-in) -- surface_contact_force_functor, constructor as in
// libgran's contact_force/surface_contact_force.h:10-30.
#ifndef SURFACE_CONTACT_FORCE_H
#define SURFACE_CONTACT_FORCE_H
#include "../gb300_functor_base.h"

template <typename field_value_t, typename real_t>
struct surface_contact_force_functor {
    surface_contact_force_functor(size_t n_part, real_t k, real_t gamma_n, real_t k_t, real_t gamma_t, real_t mu_s,
                                  real_t phi_d, real_t k_r, real_t gamma_r, real_t mu_r, real_t phi_r, real_t k_o,
                                  real_t gamma_o, real_t mu_o, real_t phi_o, real_t r_part, real_t mass,
                                  real_t inertia, real_t dt, field_value_t zero_field [[maybe_unused]],
                                  real_t real_zero [[maybe_unused]])
        : n_part(n_part),
          params{(double)k, (double)gamma_n, (double)k_t, (double)gamma_t, (double)mu_s, (double)phi_d,
                 (double)k_r, (double)gamma_r, (double)mu_r, (double)phi_r, (double)k_o, (double)gamma_o,
                 (double)mu_o, (double)phi_o, (double)r_part, (double)mass, (double)inertia, (double)dt} {}

    size_t n_part;
    lg_contact_params params;
};

#endif

// sinter_bridge.h (libgran_gb300 drop-in) -- sinter_functor and sinter_step_handler with libgran's
// constructor and template signatures (sinter_bridge/sinter_bridge.h:14-21, 100-136, 224-229).
// The constructor finds the bonds and calls the caller's random unit vector generator exactly as
// the reference constructor does (sinter_bridge.h:146-175: pairs i < j with |(|x_j - x_i| - 2r)|
// <= critical_separation, one accepted draw per bond); the engine builds the five connectors of
// every bond from those vectors and moves them with the particles inside its own integrator, so
// the step handler carries no state.
#ifndef LIBGRAN_SINTER_BRIDGE_H
#define LIBGRAN_SINTER_BRIDGE_H
#include <cmath>
#include <functional>
#include "../contact_force/contact_force.h"
#include "alt_sinter_bridge.h"

template <typename field_container_t, typename field_value_t, typename real_t>
struct sinter_step_handler {};

template <typename field_value_t, typename real_t>
struct sinter_functor {
    sinter_functor(size_t n_part, real_t k_d, real_t gamma_d, real_t k, real_t gamma_n, real_t k_t, real_t gamma_t,
                   real_t mu_s, real_t phi_d, real_t k_r, real_t gamma_r, real_t mu_r, real_t phi_r, real_t k_o,
                   real_t gamma_o, real_t mu_o, real_t phi_o, real_t r_part, real_t mass, real_t inertia, real_t dt,
                   field_value_t field_zero [[maybe_unused]], real_t real_zero [[maybe_unused]],
                   typename std::vector<field_value_t>::const_iterator x0_begin_itr,
                   std::function<field_value_t()> random_unit_vector_generator, real_t critical_separation)
        : contact{(double)k, (double)gamma_n, (double)k_t, (double)gamma_t, (double)mu_s, (double)phi_d,
                  (double)k_r, (double)gamma_r, (double)mu_r, (double)phi_r, (double)k_o, (double)gamma_o,
                  (double)mu_o, (double)phi_o, (double)r_part, (double)mass, (double)inertia, (double)dt},
          connector{(double)k_d, (double)gamma_d, (double)critical_separation} {
        for (size_t i = 0; i + 1 < n_part; ++i)
            for (size_t j = i + 1; j < n_part; ++j) {
                field_value_t const &part_i = *(x0_begin_itr + i);
                field_value_t const &part_j = *(x0_begin_itr + j);
                real_t separation = (part_j - part_i).norm() - 2.0 * r_part;
                if (std::abs(separation) > critical_separation) continue;
                field_value_t n_j = -(part_j - part_i).normalized();
                field_value_t v;
                do {
                    v = random_unit_vector_generator();
                } while (v.cross(n_j).norm() == 0.0);
                for (int c = 0; c < 3; ++c) axes.push_back((double)v[c]);
            }
        bonded_contacts.n = n_part;
        bonded_contacts.bound = &bound;
    }

    template <typename field_container_t>
    sinter_step_handler<field_container_t, field_value_t, real_t> get_step_handler() {
        return {};
    }

    static constexpr int model = LG_BINARY_SINTER_CONNECTORS;
    lg_contact_params contact;
    lg_connector_params connector;
    std::vector<double> axes;  // the accepted draw of each bond, in bond order
    libgran_gb300::bonded_view bonded_contacts;
    libgran_gb300::binding bound;
};

#endif

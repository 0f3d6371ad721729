// alt_breaking_sinter_bridge.h (libgran_gb300 drop-in) -- alt_breaking_sinter_functor, constructor
// as in libgran's sinter_bridge/alt_breaking_sinter_bridge.h:17-35. The neck-strength distribution
// is drawn here once per bond, in the reference's bond order (i ascending, then j > i ascending,
// |(|x_i - x_j| - 2r)| < critical_separation, alt_breaking_sinter_bridge.h:65-77); the engine uses
// the drawn value for both directions of the bond.
#ifndef LIBGRAN_ALT_BREAKING_SINTER_BRIDGE_H
#define LIBGRAN_ALT_BREAKING_SINTER_BRIDGE_H
#include "alt_sinter_bridge.h"

template <typename field_value_t, typename real_t, typename neck_strength_distribution_t>
struct alt_breaking_sinter_functor {
    alt_breaking_sinter_functor(size_t n_part, std::vector<field_value_t> x0, real_t k, real_t gamma_n, real_t k_t,
                                real_t gamma_t, real_t k_r, real_t gamma_r, real_t k_o, real_t gamma_o, real_t r_part,
                                real_t mass, real_t inertia, real_t dt, field_value_t field_zero [[maybe_unused]],
                                real_t real_zero [[maybe_unused]], real_t critical_separation,
                                neck_strength_distribution_t neck_strength_distribution,
                                contact_force_functor<field_value_t, real_t> contact_force)
        : params{(double)k, (double)gamma_n, (double)k_t, (double)gamma_t, (double)k_r, (double)gamma_r,
                 (double)k_o, (double)gamma_o, (double)r_part, (double)mass, (double)inertia, (double)dt,
                 (double)critical_separation},
          contact(contact_force.params) {
        bonded_contacts.n = n_part;
        bonded_contacts.bound = &bound;
        for (size_t i = 0; i + 1 < n_part; ++i)
            for (size_t j = i + 1; j < n_part; ++j) {
                double dx = (double)x0[i][0] - (double)x0[j][0], dy = (double)x0[i][1] - (double)x0[j][1],
                       dz = (double)x0[i][2] - (double)x0[j][2];
                double g = std::sqrt((dx * dx + dy * dy) + dz * dz) - 2.0 * (double)r_part;
                if (std::fabs(g) < (double)critical_separation)
                    neck_strengths_drawn.push_back((double)neck_strength_distribution());
            }
    }

    static constexpr int model = LG_BINARY_BREAKING_SINTER;
    lg_sinter_params params;
    lg_contact_params contact;
    libgran_gb300::bonded_view bonded_contacts;
    libgran_gb300::binding bound;
    std::vector<double> neck_strengths_drawn;
};

#endif

// alt_sinter_bridge.h (libgran_gb300 drop-in) -- alt_sinter_functor, constructor as in libgran's
// sinter_bridge/alt_sinter_bridge.h:19-36. Bond detection (with its cycle check) runs in the
// engine when the granular_system is built; bonded_contacts reads the bonds back from it.
#ifndef LIBGRAN_ALT_SINTER_BRIDGE_H
#define LIBGRAN_ALT_SINTER_BRIDGE_H
#include "../contact_force/contact_force.h"

namespace libgran_gb300 {
// Read-only view of bonded_contacts[i * n + j] (alt_sinter_bridge.h:163) backed by the engine.
struct bonded_view {
    size_t n = 0;
    binding *bound = nullptr;
    bool operator[](size_t idx) const {
        if (!bound || !bound->sys) return false;
        int64_t nb = 0;
        check(lg_get_bonds(bound->sys, &nb, nullptr, 0), "lg_get_bonds");
        std::vector<int64_t> pairs(2 * (size_t)nb);
        check(lg_get_bonds(bound->sys, &nb, pairs.data(), nb), "lg_get_bonds");
        const int64_t i = (int64_t)(idx / n), j = (int64_t)(idx % n);
        for (int64_t b = 0; b < nb; ++b)
            if (pairs[2 * b] == i && pairs[2 * b + 1] == j) return true;
        return false;
    }
    size_t size() const { return n * n; }
};
}  // namespace libgran_gb300

template <typename field_value_t, typename real_t>
struct alt_sinter_functor {
    alt_sinter_functor(size_t n_part, std::vector<field_value_t> x0 [[maybe_unused]], real_t k, real_t gamma_n,
                       real_t k_t, real_t gamma_t, real_t k_r, real_t gamma_r, real_t k_o, real_t gamma_o,
                       real_t r_part, real_t mass, real_t inertia, real_t dt, field_value_t field_zero [[maybe_unused]],
                       real_t real_zero [[maybe_unused]], real_t critical_separation,
                       contact_force_functor<field_value_t, real_t> contact_force)
        : params{(double)k, (double)gamma_n, (double)k_t, (double)gamma_t, (double)k_r, (double)gamma_r,
                 (double)k_o, (double)gamma_o, (double)r_part, (double)mass, (double)inertia, (double)dt,
                 (double)critical_separation},
          contact(contact_force.params) {
        bonded_contacts.n = n_part;
        bonded_contacts.bound = &bound;
    }

    static constexpr int model = LG_BINARY_SINTER;
    lg_sinter_params params;
    lg_contact_params contact;
    libgran_gb300::bonded_view bonded_contacts;
    libgran_gb300::binding bound;
    std::vector<double> neck_strengths_drawn;  // unused by the non-breaking functor
};

#endif

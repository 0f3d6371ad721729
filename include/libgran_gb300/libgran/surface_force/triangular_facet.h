// triangular_facet.h (libgran_gb300 drop-in) -- triangular_facet, constructor as in libgran's
// surface_force/triangular_facet.h:18-19, with at most one surface_contact_force_functor and one
// surface_hamaker_functor among its surface functors (folded contact first).
#ifndef TRIANGULAR_FACET_H
#define TRIANGULAR_FACET_H
#include "../contact_force/surface_contact_force.h"
#include "../hamaker_force/surface_hamaker_force.h"

template <typename field_value_t, typename real_t, typename... surface_force_functors_t>
struct triangular_facet {
    explicit triangular_facet(field_value_t v_facet, std::tuple<field_value_t, field_value_t, field_value_t> vertices,
                              surface_force_functors_t &...force_functors)
        : v_facet(v_facet), vertices(vertices) {
        static_assert(sizeof...(surface_force_functors_t) > 0, "at least one surface force functor must be provided");
        desc = lg_facet_desc{};
        for (int c = 0; c < 3; ++c) desc.v_facet[c] = (double)v_facet[c];
        auto put = [&](int k, field_value_t const &p) {
            for (int c = 0; c < 3; ++c) desc.vertices[3 * k + c] = (double)p[c];
        };
        put(0, std::get<0>(vertices));
        put(1, std::get<1>(vertices));
        put(2, std::get<2>(vertices));
        (add(force_functors), ...);
    }

    // Move the facet by v_facet * dt (triangular_facet.h:62-66); after binding, in the engine.
    void update_positions(real_t dt) {
        if (bound.sys) {
            libgran_gb300::check(lg_facet_update_positions(bound.sys, bound.facet, (double)dt), "update_positions");
            return;
        }
        std::get<0>(vertices) = shifted(std::get<0>(vertices), dt);
        std::get<1>(vertices) = shifted(std::get<1>(vertices), dt);
        std::get<2>(vertices) = shifted(std::get<2>(vertices), dt);
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) desc.vertices[3 * k + c] += desc.v_facet[c] * (double)dt;
    }

    std::tuple<field_value_t, field_value_t, field_value_t> const &get_vertices() {
        if (bound.sys) {
            double h[9];
            libgran_gb300::check(lg_facet_get_vertices(bound.sys, bound.facet, h), "get_vertices");
            vertices = std::make_tuple(field_value_t(h[0], h[1], h[2]), field_value_t(h[3], h[4], h[5]),
                                       field_value_t(h[6], h[7], h[8]));
        }
        return vertices;
    }

    field_value_t v_facet;
    lg_facet_desc desc;
    libgran_gb300::binding bound;

private:
    field_value_t shifted(field_value_t p, real_t dt) const {
        return field_value_t(p[0] + v_facet[0] * dt, p[1] + v_facet[1] * dt, p[2] + v_facet[2] * dt);
    }
    template <typename F>
    void add(F &f) {
        if constexpr (std::is_same_v<F, surface_contact_force_functor<field_value_t, real_t>>) {
            desc.has_contact = 1;
            desc.contact = f.params;
        } else if constexpr (std::is_same_v<F, surface_hamaker_functor<field_value_t, real_t>>) {
            desc.has_hamaker = 1;
            desc.hamaker = f.params;
        } else {
            static_assert(sizeof(F) == 0, "triangular_facet: unsupported surface functor for the GPU engine");
        }
    }
    std::tuple<field_value_t, field_value_t, field_value_t> vertices;
};

#endif

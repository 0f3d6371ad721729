// harness_tu.cpp -- compiles libgran's own functor headers (from the libgran source tree, unmodified)
// on lgref_vec3 and wires them into the harness system loop. TEST INFRASTRUCTURE ONLY.
// Compiled six times: LGREF_BREAKING selects alt_breaking_sinter_bridge.h and LGREF_CONNECTORS
// sinter_bridge.h (the 5-connector model with its step handler) instead of alt_sinter_bridge.h;
// LGREF_LIMITED selects limited_range_hamaker_force.h instead of hamaker_force.h +
// simplified_hamaker_force.h.
#include <cmath>
#include <math.h>      // ::abs(double), as in an Eigen build (alt_sinter_bridge.h:69 calls abs unqualified)
#include <iostream>    // alt_sinter_bridge.h:71 uses std::cout without including it
#include <algorithm>
#include <tuple>
#include <vector>
#include <forward_list>
#include <numeric>
#include <limits>
#include "lgref_base.hpp"

#define private public  // expose the functors' spring buffers to the harness
#include <libgran/utility/operator_overloads.h>
#include <libgran/granular_system/binary_force_container.h>
#include <libgran/granular_system/unary_force_container.h>
#include <libgran/contact_force/contact_force.h>
#if LGREF_LIMITED
#include <libgran/hamaker_force/limited_range_hamaker_force.h>
#else
#include <libgran/hamaker_force/hamaker_force.h>
#include <libgran/hamaker_force/simplified_hamaker_force.h>
#endif
#include <libgran/contact_force/surface_contact_force.h>
#include <libgran/hamaker_force/surface_hamaker_force.h>
#include <libgran/surface_force/triangular_facet.h>
#if LGREF_CONNECTORS
#include <libgran/sinter_bridge/sinter_bridge.h>
#elif LGREF_BREAKING
#include <libgran/sinter_bridge/alt_breaking_sinter_bridge.h>
#else
#include <libgran/sinter_bridge/alt_sinter_bridge.h>
#endif
#undef private

namespace {

using CF = contact_force_functor<V, double>;
using SC = surface_contact_force_functor<V, double>;
using SH = surface_hamaker_functor<V, double>;
using FacetT = triangular_facet<V, double, SC, SH>;

struct seq_strength {  // neck strength "distribution": hands out the given values in order
    std::shared_ptr<std::vector<double>> vals;
    size_t k = 0;
    double operator()() { return k < vals->size() ? (*vals)[k++] : std::numeric_limits<double>::infinity(); }
};
#if LGREF_CONNECTORS
using SinterT = sinter_functor<V, double>;
#elif LGREF_BREAKING
using SinterT = alt_breaking_sinter_functor<V, double, seq_strength>;
#else
using SinterT = alt_sinter_functor<V, double>;
#endif
#if LGREF_LIMITED
using HamT = limited_range_hamaker_functor<V, double>;
#else
using HamT = hamaker_functor<V, double>;
using SHamT = simplified_hamaker_functor<V, double>;
#endif

std::shared_ptr<CF> make_contact(const lg_contact_params &p, size_t n) {
    return std::make_shared<CF>(n, p.k, p.gamma_n, p.k_t, p.gamma_t, p.mu_s, p.phi_d, p.k_r, p.gamma_r, p.mu_r,
                                p.phi_r, p.k_o, p.gamma_o, p.mu_o, p.phi_o, p.r_part, p.mass, p.inertia, p.dt,
                                V::Zero(), 0.0);
}

template <typename... F>
BinFn bin_of(RefSys *s, std::shared_ptr<F>... f) {
    auto c = std::make_shared<binary_force_functor_container<V, double, F...>>(*f...);
    (s->keep.push_back(f), ...);
    s->keep.push_back(c);
    return [c](size_t i, size_t j, Field const &x, Field const &v, Field const &th, Field const &om, double t) {
        return (*c)(i, j, x, v, th, om, t);
    };
}

// The tutorial's central_attraction_functor (Custom-unary-force-model.md:108-118): a user-defined
// unary functor, restated here because it exists only as documentation; the container folds it
// after the facets.
struct central_attraction {
    double k_a, mass;
    V x0;
    std::pair<V, V> operator()(size_t i, Field const &x, Field const &, Field const &, Field const &, double) const {
        V a = k_a / mass * (x0 - x[i]);
        return std::make_pair(a, V::Zero());
    }
};

template <size_t> using FacetAt = FacetT;

// libgran's unary container over the facets (in order) and, when `body` is set, the central
// functor after them.
template <size_t... I>
UnFn unary_of(RefSys *s, std::vector<std::shared_ptr<FacetT>> &fs, std::shared_ptr<central_attraction> body,
              std::index_sequence<I...>) {
    if (body) {
        auto c = std::make_shared<unary_force_functor_container<V, double, FacetAt<I>..., central_attraction>>(*fs[I]...,
                                                                                                             *body);
        s->keep.push_back(c);
        return [c](size_t i, Field const &x, Field const &v, Field const &th, Field const &om, double t) {
            return (*c)(i, x, v, th, om, t);
        };
    }
    if constexpr (sizeof...(I) == 0) {
        return UnFn();
    } else {
        auto c = std::make_shared<unary_force_functor_container<V, double, FacetAt<I>...>>(*fs[I]...);
        s->keep.push_back(c);
        return [c](size_t i, Field const &x, Field const &v, Field const &th, Field const &om, double t) {
            return (*c)(i, x, v, th, om, t);
        };
    }
}

void fill9(double *out, std::tuple<V, V, V> const &t) {
    V a = std::get<0>(t), b = std::get<1>(t), c = std::get<2>(t);
    for (int k = 0; k < 3; ++k) { out[k] = a[k]; out[3 + k] = b[k]; out[6 + k] = c[k]; }
}

}  // namespace

#if LGREF_CONNECTORS && LGREF_LIMITED
#define FACTORY lgref_make_conn_limited
#elif LGREF_CONNECTORS
#define FACTORY lgref_make_conn_full
#elif LGREF_BREAKING && LGREF_LIMITED
#define FACTORY lgref_make_brk_limited
#elif LGREF_BREAKING
#define FACTORY lgref_make_brk_full
#elif LGREF_LIMITED
#define FACTORY lgref_make_alt_limited
#else
#define FACTORY lgref_make_alt_full
#endif

RefSys *FACTORY(const lg_system_desc *d, const double *x0, const double *v0, const double *th0, const double *om0,
                const lg_facet_desc *facets, const double *neck, int64_t n_neck) {
    const size_t n = (size_t)d->n_part;
    RefSys *s = new RefSys();
    s->x = to_field(x0, d->n_part); s->v = to_field(v0, d->n_part);
    s->th = to_field(th0, d->n_part); s->om = to_field(om0, d->n_part);
    s->a.assign(n, V::Zero()); s->al.assign(n, V::Zero());
    s->verlet = (d->pairs == LG_PAIRS_VERLET);
    s->rv = d->r_verlet;
    s->facet_auto_move = d->facet_auto_move != 0;

    auto contact = make_contact(d->contact, n);
    std::shared_ptr<SinterT> sinter;
#if LGREF_CONNECTORS
    (void)neck; (void)n_neck;
    if (d->binary_model == LG_BINARY_SINTER_CONNECTORS) {
        const lg_contact_params &p = d->contact;
        // the caller's axes stand in for the reference's random unit vector generator, in order
        auto axes = std::make_shared<std::vector<V>>();
        for (int64_t b = 0; b < d->n_connector_axes; ++b)
            axes->push_back(V(d->connector_axes[3 * b], d->connector_axes[3 * b + 1], d->connector_axes[3 * b + 2]));
        auto next = std::make_shared<size_t>(0);
        std::function<V()> gen = [axes, next]() { return (*next < axes->size()) ? (*axes)[(*next)++] : V(1.0, 0.0, 0.0); };
        sinter = std::make_shared<SinterT>(n, d->connector.k_d, d->connector.gamma_d, p.k, p.gamma_n, p.k_t, p.gamma_t,
                                           p.mu_s, p.phi_d, p.k_r, p.gamma_r, p.mu_r, p.phi_r, p.k_o, p.gamma_o, p.mu_o,
                                           p.phi_o, p.r_part, p.mass, p.inertia, p.dt, V::Zero(), 0.0, s->x.begin(),
                                           gen, d->connector.critical_separation);
        auto handler = std::make_shared<sinter_step_handler<Field, V, double>>(sinter->get_step_handler<Field>());
        s->keep.push_back(handler);
        s->inc_x = [s, handler](size_t i, V const &dx) {
            handler->increment_x(i, dx, s->x.begin(), s->v.begin(), s->a.begin(), s->th.begin(), s->om.begin(), s->al.begin());
        };
        s->inc_theta = [s, handler](size_t i, V const &dth) {
            handler->increment_theta(i, dth, s->x.begin(), s->v.begin(), s->a.begin(), s->th.begin(), s->om.begin(),
                                     s->al.begin());
        };
    }
#else
    if (d->binary_model == LG_BINARY_SINTER || d->binary_model == LG_BINARY_BREAKING_SINTER) {
        const lg_sinter_params &p = d->sinter;
#if LGREF_BREAKING
        seq_strength dist{std::make_shared<std::vector<double>>(neck, neck + (neck ? n_neck : 0))};
        sinter = std::make_shared<SinterT>(n, s->x, p.k, p.gamma_n, p.k_t, p.gamma_t, p.k_r, p.gamma_r, p.k_o,
                                           p.gamma_o, p.r_part, p.mass, p.inertia, p.dt, V::Zero(), 0.0,
                                           p.critical_separation, dist, *contact);
#else
        (void)neck; (void)n_neck;
        sinter = std::make_shared<SinterT>(n, s->x, p.k, p.gamma_n, p.k_t, p.gamma_t, p.k_r, p.gamma_r, p.k_o,
                                           p.gamma_o, p.r_part, p.mass, p.inertia, p.dt, V::Zero(), 0.0,
                                           p.critical_separation, *contact);
#endif
    }
#endif
    const lg_hamaker_params &hp = d->hamaker;
#if LGREF_LIMITED
    std::shared_ptr<HamT> ham;
    if (d->hamaker_model == LG_HAMAKER_LIMITED)
        ham = std::make_shared<HamT>(hp.A, hp.h0, hp.r_cutoff, hp.r_part, hp.mass, V::Zero(), 0.0);
#else
    std::shared_ptr<HamT> ham;
    std::shared_ptr<SHamT> sham;
    if (d->hamaker_model == LG_HAMAKER_FULL) ham = std::make_shared<HamT>(hp.A, hp.h0, hp.r_part, hp.mass, V::Zero(), 0.0);
    if (d->hamaker_model == LG_HAMAKER_SIMPLIFIED) sham = std::make_shared<SHamT>(hp.A, hp.h0, hp.r_part, hp.mass, V::Zero(), 0.0);
#endif
    auto with_primary = [&](auto prim) {
        if (ham) s->bin = bin_of(s, prim, ham);
#if !LGREF_LIMITED
        else if (sham) s->bin = bin_of(s, prim, sham);
#endif
        else s->bin = bin_of(s, prim);
    };
    if (d->binary_model == LG_BINARY_CONTACT) with_primary(contact);
    else if (sinter) with_primary(sinter);
    else {
        if (ham) s->bin = bin_of(s, ham);
#if !LGREF_LIMITED
        else if (sham) s->bin = bin_of(s, sham);
#endif
    }

    // spring and bond read-back
    s->springs = [contact, sinter, n, bm = d->binary_model](size_t i, size_t j, double *out) {
#if LGREF_CONNECTORS
        if (sinter && sinter->bonded_contacts[i * n + j]) {  // the five connectors of i for the bond
            for (int k = 0; k < 9; ++k) out[k] = 0.0;
            return;
        }
#else
        if (sinter && sinter->bonded_contacts[i * n + j]) { fill9(out, sinter->contact_springs[i * n + j]); return; }
#endif
        if (sinter) { fill9(out, sinter->contact_force.contact_springs[i * n + j]); return; }
        if (bm == LG_BINARY_CONTACT) { fill9(out, contact->contact_springs[i * n + j]); return; }
        for (int k = 0; k < 9; ++k) out[k] = 0.0;
    };
    s->bonds = [sinter, n](int64_t *pairs, int64_t cap) -> int64_t {
        if (!sinter) return 0;
        int64_t c = 0;
        for (size_t i = 0; i < n; ++i)
            for (size_t j = 0; j < n; ++j)
                if (sinter->bonded_contacts[i * n + j]) {
                    if (pairs && c < cap) { pairs[2 * c] = (int64_t)i; pairs[2 * c + 1] = (int64_t)j; }
                    ++c;
                }
        return c;
    };

    // facets: each with a surface contact functor and a surface Hamaker functor
    std::vector<std::shared_ptr<FacetT>> fs;
    for (int32_t f = 0; f < d->n_facets; ++f) {
        const lg_facet_desc &fd = facets[f];
        const lg_contact_params &p = fd.contact;
        auto sc = std::make_shared<SC>(n, p.k, p.gamma_n, p.k_t, p.gamma_t, p.mu_s, p.phi_d, p.k_r, p.gamma_r, p.mu_r,
                                       p.phi_r, p.k_o, p.gamma_o, p.mu_o, p.phi_o, p.r_part, p.mass, p.inertia, p.dt,
                                       V::Zero(), 0.0);
        double A = fd.has_hamaker ? fd.hamaker.A : 0.0;
        auto sh = std::make_shared<SH>(A, fd.hamaker.h0, fd.hamaker.r_part, fd.hamaker.mass, V::Zero(), 0.0);
        std::tuple<V, V, V> verts{V(fd.vertices[0], fd.vertices[1], fd.vertices[2]),
                                  V(fd.vertices[3], fd.vertices[4], fd.vertices[5]),
                                  V(fd.vertices[6], fd.vertices[7], fd.vertices[8])};
        auto fc = std::make_shared<FacetT>(V(fd.v_facet[0], fd.v_facet[1], fd.v_facet[2]), verts, *sc, *sh);
        s->keep.push_back(sc); s->keep.push_back(sh); s->keep.push_back(fc);
        fs.push_back(fc);
        s->facet_move.push_back([fc](double dt) { fc->update_positions(dt); });
        s->facet_vertices.push_back([fc](double *out) {
            auto const &vt = fc->get_vertices();
            V a = std::get<0>(vt), b = std::get<1>(vt), c = std::get<2>(vt);
            for (int k = 0; k < 3; ++k) { out[k] = a[k]; out[3 + k] = b[k]; out[6 + k] = c[k]; }
        });
    }
    std::shared_ptr<central_attraction> body;
    if (d->body.model == LG_BODY_CENTRAL) {
        body = std::make_shared<central_attraction>();
        body->k_a = d->body.k_a;
        body->mass = d->body.mass;
        body->x0 = V(d->body.centre[0], d->body.centre[1], d->body.centre[2]);
        s->keep.push_back(body);
        s->set_centre = [body](const double *c) { body->x0 = V(c[0], c[1], c[2]); };
    }
    switch (fs.size()) {
        case 0: s->un = unary_of(s, fs, body, std::make_index_sequence<0>()); break;
        case 1: s->un = unary_of(s, fs, body, std::make_index_sequence<1>()); break;
        case 2: s->un = unary_of(s, fs, body, std::make_index_sequence<2>()); break;
        case 3: s->un = unary_of(s, fs, body, std::make_index_sequence<3>()); break;
        case 4: s->un = unary_of(s, fs, body, std::make_index_sequence<4>()); break;
        default: delete s; return nullptr;
    }
    if (d->hold_mask) s->hold.assign(d->hold_mask, d->hold_mask + n);
    s->build_rows();
    s->forces();
    return s;
}

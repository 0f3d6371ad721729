// granular_system.h (libgran_gb300 drop-in) -- granular_system with libgran's template parameters
// and constructor (granular_system/granular_system.h:25-63) on the GPU engine. The functor
// containers are read at construction: which functors are present and their parameters become one
// lg_system_desc; do_step(dt) is one engine step (rotational velocity Verlet, see the C ABI), and
// get_x/get_v/get_theta/get_omega read the state back (Granular-system.md:65-226).
#ifndef LIBGRAN_GRANULAR_SYSTEM_H
#define LIBGRAN_GRANULAR_SYSTEM_H
#include <functional>
#include "../contact_force/contact_force.h"
#include "../utility/operator_overloads.h"
#include "binary_force_container.h"
#include "unary_force_container.h"

// Integrator and step handler names of libtimestep (the libgran drivers pass them as template
// arguments); the engine's integrator is the rotational velocity Verlet scheme they name.
template <typename field_container_t, typename field_value_t, typename real_t, typename functor_t,
          template <typename, typename> typename step_handler_t>
struct rotational_velocity_verlet_half {};
template <typename field_container_t, typename field_value_t>
struct rotational_step_handler {};

template <typename, typename> struct alt_sinter_functor;
template <typename, typename> struct sinter_functor;
template <typename, typename, typename> struct alt_breaking_sinter_functor;
template <typename, typename> struct hamaker_functor;
template <typename, typename> struct limited_range_hamaker_functor;
template <typename, typename> struct simplified_hamaker_functor;
template <typename, typename, typename...> struct triangular_facet;
template <typename, typename> struct central_attraction_functor;
namespace libgran_gb300 {
template <typename> struct device_unary;
}

namespace libgran_gb300 {

template <typename T> struct is_contact : std::false_type {};
template <typename V, typename R> struct is_contact<contact_force_functor<V, R>> : std::true_type {};
template <typename T> struct is_sinter : std::false_type {};
template <typename V, typename R> struct is_sinter<alt_sinter_functor<V, R>> : std::true_type {};
template <typename V, typename R, typename D> struct is_sinter<alt_breaking_sinter_functor<V, R, D>> : std::true_type {};
template <typename T> struct is_connector_sinter : std::false_type {};
template <typename V, typename R> struct is_connector_sinter<sinter_functor<V, R>> : std::true_type {};
template <typename T> struct is_hamaker : std::false_type {};
template <typename V, typename R> struct is_hamaker<hamaker_functor<V, R>> : std::true_type {};
template <typename V, typename R> struct is_hamaker<limited_range_hamaker_functor<V, R>> : std::true_type {};
template <typename V, typename R> struct is_hamaker<simplified_hamaker_functor<V, R>> : std::true_type {};
template <typename T> struct is_facet : std::false_type {};
template <typename V, typename R, typename... F> struct is_facet<triangular_facet<V, R, F...>> : std::true_type {};
template <typename T> struct is_central : std::false_type {};
template <typename V, typename R> struct is_central<central_attraction_functor<V, R>> : std::true_type {};
template <typename T> struct is_device_unary : std::false_type {};
template <typename F> struct is_device_unary<device_unary<F>> : std::true_type {};
// step handlers that hold increments expose hold_mask(n)
template <typename H, typename = void> struct has_hold_mask : std::false_type {};
template <typename H>
struct has_hold_mask<H, std::void_t<decltype(std::declval<H const &>().hold_mask(size_t{}))>> : std::true_type {};

struct desc_builder {
    lg_system_desc d{};
    std::vector<lg_facet_desc> facets;
    std::vector<double> neck;
    std::vector<binding *> sinter_bindings;
    std::vector<binding *> facet_bindings;
    std::vector<binding *> body_bindings;
    std::vector<uint8_t> hold;
    bool has_binary = false, has_hamaker = false, has_body = false;

    template <typename F>
    void binary(F &f) {
        using T = std::decay_t<F>;
        if constexpr (is_contact<T>::value) {
            if (has_binary) throw std::invalid_argument("one contact or sintered functor per container");
            has_binary = true;
            d.binary_model = LG_BINARY_CONTACT;
            d.contact = f.params;
        } else if constexpr (is_sinter<T>::value) {
            if (has_binary) throw std::invalid_argument("one contact or sintered functor per container");
            has_binary = true;
            d.binary_model = T::model;
            d.sinter = f.params;
            d.contact = f.contact;
            neck = f.neck_strengths_drawn;
            sinter_bindings.push_back(&f.bound);
        } else if constexpr (is_connector_sinter<T>::value) {
            if (has_binary) throw std::invalid_argument("one contact or sintered functor per container");
            has_binary = true;
            d.binary_model = T::model;
            d.contact = f.contact;
            d.connector = f.connector;
            d.connector_axes = f.axes.data();
            d.n_connector_axes = (int64_t)(f.axes.size() / 3);
            sinter_bindings.push_back(&f.bound);
        } else if constexpr (is_hamaker<T>::value) {
            if (has_hamaker) throw std::invalid_argument("one Hamaker functor per container");
            has_hamaker = true;
            d.hamaker_model = T::mode;
            d.hamaker = f.params;
        } else {
            static_assert(sizeof(T) == 0, "binary functor has no GPU implementation in libgran_gb300");
        }
    }
    // Unary functors: the facets, then at most one body force (the container's right fold puts the
    // engine's body term last, so it must be the last functor).
    template <typename F>
    void unary(F &f) {
        using T = std::decay_t<F>;
        if constexpr (is_facet<T>::value) {
            if (has_body) throw std::invalid_argument("the body-force functor must follow the facets in the container");
            facets.push_back(f.desc);
            facet_bindings.push_back(&f.bound);
        } else if constexpr (is_central<T>::value) {
            if (has_body) throw std::invalid_argument("one body-force functor per container");
            has_body = true;
            d.body = f.body;
            body_bindings.push_back(&f.bound);
        } else if constexpr (is_device_unary<T>::value) {
            if (has_body) throw std::invalid_argument("one body-force functor per container");
            has_body = true;
            d.unary_hook = &T::launch;
            d.unary_hook_user = (void *)&f;
        } else {
            static_assert(sizeof(T) == 0, "unary functor has no GPU implementation in libgran_gb300");
        }
    }
};

// The hold mask of a step handler that holds increments (fixed_particle_step_handler,
// held_particles_step_handler); empty for the others.
template <typename H>
std::vector<uint8_t> hold_of(H const &h, size_t n) {
    if constexpr (has_hold_mask<H>::value)
        return h.hold_mask(n);
    else
        return {};
}

}  // namespace libgran_gb300

template <typename field_value_t, typename real_t,
          template <typename _field_container_t, typename _field_value_t, typename _real_t, typename _functor_t,
                    template <typename __field_container_t, typename __field_value_t> typename _step_handler_t>
          typename integrator_t,
          template <typename _field_container_t, typename _field_value_t> typename step_handler_t,
          typename binary_force_functor_container_t, typename unary_force_functor_container_t>
class granular_system {
public:
    typedef std::vector<field_value_t> field_container_t;

    granular_system(granular_system const &) = delete;

    granular_system(field_container_t x0, field_container_t v0, field_container_t theta0, field_container_t omega0,
                    real_t t0 [[maybe_unused]], field_value_t field_zero [[maybe_unused]],
                    real_t real_zero [[maybe_unused]],
                    step_handler_t<field_container_t, field_value_t> &step_handler [[maybe_unused]],
                    binary_force_functor_container_t binary_force_functors,
                    unary_force_functor_container_t unary_force_functors)
        : granular_system(LG_PAIRS_ALL, 0.0, std::move(x0), std::move(v0), std::move(theta0), std::move(omega0),
                          binary_force_functors, unary_force_functors,
                          [&step_handler](size_t n_part) { return libgran_gb300::hold_of(step_handler, n_part); }) {}

    ~granular_system() { lg_destroy(sys); }

    void do_step(real_t dt) { libgran_gb300::check(lg_step(sys, (double)dt, 1, 0), "do_step"); }

    // Extension: n steps in one call (captured as CUDA graphs), Verlet list rebuilt every
    // rebuild_every steps.
    void do_steps(real_t dt, int64_t n, int64_t rebuild_every = 0) {
        libgran_gb300::check(lg_step(sys, (double)dt, n, rebuild_every), "do_steps");
    }

    field_container_t const &get_x() { return fetch(LG_FIELD_X, x); }
    field_container_t const &get_v() { return fetch(LG_FIELD_V, v); }
    field_container_t const &get_theta() { return fetch(LG_FIELD_THETA, theta); }
    field_container_t const &get_omega() { return fetch(LG_FIELD_OMEGA, omega); }
    // Extension: the accelerations of the last force evaluation (libgran's a / alpha buffers).
    field_container_t const &get_a() { return fetch(LG_FIELD_A, a); }
    field_container_t const &get_alpha() { return fetch(LG_FIELD_ALPHA, alpha); }
    void reset_acceleration_buffers() { libgran_gb300::check(lg_reset_acceleration_buffers(sys), "reset"); }
    lg_system *handle() { return sys; }

protected:
    granular_system(int pairs, double r_verlet, field_container_t x0, field_container_t v0, field_container_t theta0,
                    field_container_t omega0, binary_force_functor_container_t &binary,
                    unary_force_functor_container_t &unary,
                    std::function<std::vector<uint8_t>(size_t)> hold_mask_of = nullptr) {
        libgran_gb300::desc_builder b;
        std::apply([&b](auto &...f) { (b.binary(f), ...); }, binary.binary_force_functors);
        std::apply([&b](auto &...f) { (b.unary(f), ...); }, unary.unary_force_functors);
        n = x0.size();
        b.d.n_part = (int64_t)x0.size();
        b.d.pairs = pairs;
        b.d.r_verlet = r_verlet;
        b.d.precision = libgran_gb300::default_precision();
        if (b.d.binary_model == LG_BINARY_SINTER_CONNECTORS) b.d.precision = LG_PRECISION_FP64;  // FP64 only
        b.d.n_facets = (int32_t)b.facets.size();
        std::vector<uint8_t> hold;
        if (hold_mask_of) hold = hold_mask_of(x0.size());
        if (!hold.empty()) b.d.hold_mask = hold.data();
        auto xa = libgran_gb300::to_aos(x0), va = libgran_gb300::to_aos(v0), ta = libgran_gb300::to_aos(theta0),
             wa = libgran_gb300::to_aos(omega0);
        libgran_gb300::check(lg_create(&b.d, xa.data(), va.data(), ta.data(), wa.data(),
                                       b.facets.empty() ? nullptr : b.facets.data(),
                                       b.neck.empty() ? nullptr : b.neck.data(), (int64_t)b.neck.size(), 0, &sys),
                             "granular_system");
        for (auto *p : b.sinter_bindings) p->sys = sys;
        for (auto *p : b.body_bindings) p->sys = sys;
        for (size_t f = 0; f < b.facet_bindings.size(); ++f) {
            b.facet_bindings[f]->sys = sys;
            b.facet_bindings[f]->facet = (int32_t)f;
        }
    }

    lg_system *sys = nullptr;

private:
    field_container_t const &fetch(int field, field_container_t &cache) {
        std::vector<double> h(3 * n);
        libgran_gb300::check(lg_get(sys, field, h.data()), "get");
        libgran_gb300::from_aos(h, cache);
        return cache;
    }
    size_t n = 0;
    field_container_t x, v, theta, omega, a, alpha;
};

#endif

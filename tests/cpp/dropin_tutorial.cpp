// A driver in the shape of libgran's custom step-handler tutorial (Custom-step-handler.md,
// tutorial_04.cpp): contact + Hamaker in the binary container, the tutorial's
// central_attraction_functor in the unary container, fixed_particle_step_handler over
// rotational_step_handler holding one particle's velocity; update_center_of_mass(x0) before every
// do_step, as the tutorial does. Built on the libgran_gb300 drop-in headers. Initial positions and
// velocities come from a file; the end state is written to another.
// Usage: dropin_tutorial <state_in> <state_out> <n_steps> <fixed_particle>
//   state_in: int64 n, then x (3n doubles), v (3n doubles); state_out: x, v, theta, omega (3n each)
#include <libgran/body_force/central_attraction.h>
#include <libgran/contact_force/contact_force.h>
#include <libgran/granular_system/granular_system.h>
#include <libgran/hamaker_force/hamaker_force.h>
#include <libgran/step_handler/fixed_particle_step_handler.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

struct vec3 {
    double c[3];
    vec3() : c{0, 0, 0} {}
    vec3(double x, double y, double z) : c{x, y, z} {}
    double operator[](int k) const { return c[k]; }
    double &operator[](int k) { return c[k]; }
    static vec3 Zero() { return vec3(); }
    vec3 &operator+=(vec3 const &o) {
        for (int k = 0; k < 3; ++k) c[k] += o.c[k];
        return *this;
    }
    vec3 operator/(double s) const { return vec3(c[0] / s, c[1] / s, c[2] / s); }
};

using contact_force_functor_t = contact_force_functor<vec3, double>;
using vdw_force_functor_t = hamaker_functor<vec3, double>;
using central_force_functor_t = central_attraction_functor<vec3, double>;
using binary_force_container_t =
    binary_force_functor_container<vec3, double, contact_force_functor_t, vdw_force_functor_t>;
using unary_force_container_t = unary_force_functor_container<vec3, double, central_force_functor_t>;
template <typename field_container_t, typename field_value_t>
using step_handler_t = fixed_particle_step_handler<field_container_t, field_value_t, rotational_step_handler>;
using granular_system_t = granular_system<vec3, double, rotational_velocity_verlet_half, step_handler_t,
                                          binary_force_container_t, unary_force_container_t>;

int main(int argc, char **argv) {
    if (argc < 5) return 2;
    FILE *fi = std::fopen(argv[1], "rb");
    if (!fi) return 2;
    int64_t n = 0;
    if (std::fread(&n, sizeof(n), 1, fi) != 1 || n < 1) return 2;
    std::vector<double> buf(6 * (size_t)n);
    if (std::fread(buf.data(), sizeof(double), buf.size(), fi) != buf.size()) return 2;
    std::fclose(fi);
    const size_t n_steps = (size_t)std::atoll(argv[3]);
    const size_t fixed_particle = (size_t)std::atoll(argv[4]);

    const double dt = 1e-13, rho = 1700.0, r_part = 1.4e-8;
    const double mass = 4.0 / 3.0 * M_PI * std::pow(r_part, 3.0) * rho;
    const double inertia = 2.0 / 5.0 * mass * std::pow(r_part, 2.0);
    const double k = 10000.0, gamma_n = 5.0e-9, mu = 1.0, phi = 1.0, mu_o = 0.1;
    const double gamma_t = 0.2 * gamma_n, gamma_r = 0.05 * gamma_n, gamma_o = 0.05 * gamma_n;
    const double A = 1.0e-19, h0 = 1.0e-9, k_attr = 8.0e-6;

    std::vector<vec3> x0, v0, theta0((size_t)n), omega0((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        x0.emplace_back(buf[3 * i], buf[3 * i + 1], buf[3 * i + 2]);
        v0.emplace_back(buf[3 * n + 3 * i], buf[3 * n + 3 * i + 1], buf[3 * n + 3 * i + 2]);
    }

    contact_force_functor_t contact_force_model(x0.size(), k, gamma_n, k, gamma_t, mu, phi, k, gamma_r, mu_o, phi, k,
                                                gamma_o, mu_o, phi, r_part, mass, inertia, dt, vec3::Zero(), 0.0);
    vdw_force_functor_t hamaker_model(A, h0, r_part, mass, vec3::Zero(), 0.0);
    central_force_functor_t central_model(r_part, k_attr, mass, vec3::Zero());
    central_model.update_center_of_mass(x0);  // the centre of the construction-time evaluation
    binary_force_container_t binary_force_functors{contact_force_model, hamaker_model};
    unary_force_container_t unary_force_functors{central_model};
    rotational_step_handler<std::vector<vec3>, vec3> base_step_handler_instance;
    step_handler_t<std::vector<vec3>, vec3> step_handler_instance(fixed_particle, base_step_handler_instance);
    granular_system_t system(x0, v0, theta0, omega0, 0.0, vec3::Zero(), 0.0, step_handler_instance,
                             binary_force_functors, unary_force_functors);

    for (size_t s = 0; s < n_steps; ++s) {
        central_model.update_center_of_mass(x0);
        system.do_step(dt);
    }

    FILE *fo = std::fopen(argv[2], "wb");
    if (!fo) return 2;
    for (auto const *f : {&system.get_x(), &system.get_v(), &system.get_theta(), &system.get_omega()})
        for (auto const &p : *f) std::fwrite(p.c, sizeof(double), 3, fo);
    std::fclose(fo);
    return 0;
}

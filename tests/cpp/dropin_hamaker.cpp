// A libgran driver written against the libgran_gb300 drop-in headers: the set-up of libgran's
// test/hamaker.cpp and test/hamaker_neighbor.cpp (18-particle plate + projectile, contact + Hamaker)
// with the same template composition and constructor calls, checked against libgran's 1 % targets.
// Usage: dropin_hamaker [all|neighbor] [steps_per_call] [n_steps]
// With n_steps given the driver prints its end state (momentum, kinetic energy, radius of gyration)
// and skips the 1 % check, which applies to the full 3e6-step run.
#include <libgran/contact_force/contact_force.h>
#include <libgran/granular_system/granular_system.h>
#include <libgran/granular_system/granular_system_neighbor_list.h>
#include <libgran/hamaker_force/hamaker_force.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

struct vec3 {  // a minimal field_value_t (libgran's drivers use Eigen::Vector3d)
    double c[3];
    vec3() : c{0, 0, 0} {}
    vec3(double x, double y, double z) : c{x, y, z} {}
    double operator[](int k) const { return c[k]; }
    double &operator[](int k) { return c[k]; }
    static vec3 Zero() { return vec3(); }
};

template <bool neighbor, typename S>
int run(S &system, double dt, size_t n_steps, size_t per_call, double mass, double inertia, bool check) {
    for (size_t n = 0; n < n_steps;) {
        if constexpr (neighbor) {  // update_neighbor_list() every 20 steps, as test/hamaker_neighbor.cpp:121-122
            system.update_neighbor_list();
            size_t k = std::min<size_t>(20, n_steps - n);
            system.do_steps(dt, (int64_t)k, 0);
            n += k;
        } else if (per_call > 1) {
            size_t k = std::min(per_call, n_steps - n);
            system.do_steps(dt, (int64_t)k, 0);
            n += k;
        } else {
            system.do_step(dt);
            ++n;
        }
    }
    auto const &v = system.get_v();
    auto const &w = system.get_omega();
    auto const &x = system.get_x();
    double ke = 0, px = 0, py = 0, pz = 0, cx = 0, cy = 0, cz = 0;
    for (size_t i = 0; i < v.size(); ++i) {
        ke += mass * ((v[i][0] * v[i][0] + v[i][1] * v[i][1]) + v[i][2] * v[i][2]) / 2.0;
        ke += inertia * ((w[i][0] * w[i][0] + w[i][1] * w[i][1]) + w[i][2] * w[i][2]) / 2.0;
        px += v[i][0]; py += v[i][1]; pz += v[i][2];
        cx += x[i][0]; cy += x[i][1]; cz += x[i][2];
    }
    double p = mass * std::sqrt((px * px + py * py) + pz * pz);
    cx /= x.size(); cy /= x.size(); cz /= x.size();
    double rg = 0;
    for (auto const &q : x) rg += ((q[0] - cx) * (q[0] - cx) + (q[1] - cy) * (q[1] - cy)) + (q[2] - cz) * (q[2] - cz);
    rg = std::sqrt(rg / x.size());
    const double tp = 1.96373e-19, tke = 8.33959e-20, trg = 3.56253e-08;
    std::printf("momentum %.17g ke %.17g rg %.17g\n", p, ke, rg);
    if (!check) return 0;
    std::printf("targets: momentum %.6g ke %.6g rg %.6g\n", tp, tke, trg);
    if (std::fabs(ke - tke) / tke > 0.01 || std::fabs(p - tp) / tp > 0.01 || std::fabs(rg - trg) / trg > 0.01)
        return EXIT_FAILURE;
    return 0;
}

int main(int argc, char **argv) {
    const bool neighbor = argc > 1 && std::strcmp(argv[1], "neighbor") == 0;
    const size_t per_call = argc > 2 ? (size_t)std::atol(argv[2]) : 1000;
    const double dt = 1e-13, t_tot = 3.0e-7;
    const bool full = argc <= 3;
    const auto n_steps = full ? size_t(t_tot / dt) : (size_t)std::atol(argv[3]);
    const double rho = 1700.0, r_part = 1.4e-8;
    const double mass = 4.0 / 3.0 * M_PI * std::pow(r_part, 3.0) * rho;
    const double inertia = 2.0 / 5.0 * mass * std::pow(r_part, 2.0);
    const double k = 10000.0, gamma_n = 5.0e-9, mu = 1.0, phi = 1.0, mu_o = 0.1;
    const double gamma_t = 0.2 * gamma_n, gamma_r = 0.05 * gamma_n, gamma_o = 0.05 * gamma_n;
    const double A = 1.0e-20, h0 = 1.0e-9;

    std::vector<vec3> x0, v0, theta0, omega0;
    for (size_t i = 0; i < 3; i++) {
        auto y = -3.0 * r_part + double(i) * 2.0 * r_part;
        for (size_t j = 0; j < 3; j++) {
            auto x = -3.0 * r_part + double(j) * 2.0 * r_part;
            x0.emplace_back(x, y, 0.0);
            x0.emplace_back(x, y, -2.0 * r_part);
        }
    }
    x0.emplace_back(0, 0, 3.0 * r_part);
    v0.resize(x0.size());
    theta0.resize(x0.size());
    omega0.resize(x0.size());
    v0.back() = vec3(1.0, 0.0, -10.0);

    rotational_step_handler<std::vector<vec3>, vec3> step_handler_instance;
    contact_force_functor<vec3, double> contact_force_model(x0.size(), k, gamma_n, k, gamma_t, mu, phi, k, gamma_r, mu_o,
                                                            phi, k, gamma_o, mu_o, phi, r_part, mass, inertia, dt,
                                                            vec3::Zero(), 0.0);
    hamaker_functor<vec3, double> hamaker_model(A, h0, r_part, mass, vec3::Zero(), 0.0);
    binary_force_functor_container<vec3, double, contact_force_functor<vec3, double>, hamaker_functor<vec3, double>>
        binary_force_functors{contact_force_model, hamaker_model};
    unary_force_functor_container<vec3, double> unary_force_functors;
    using bin_t = binary_force_functor_container<vec3, double, contact_force_functor<vec3, double>, hamaker_functor<vec3, double>>;
    using un_t = unary_force_functor_container<vec3, double>;
    if (neighbor) {
        granular_system_neighbor_list<vec3, double, rotational_velocity_verlet_half, rotational_step_handler, bin_t, un_t>
            system(x0.size(), 5.0 * r_part, x0, v0, theta0, omega0, 0.0, vec3::Zero(), 0.0, step_handler_instance,
                   binary_force_functors, unary_force_functors);
        return run<true>(system, dt, n_steps, per_call, mass, inertia, full);
    }
    granular_system<vec3, double, rotational_velocity_verlet_half, rotational_step_handler, bin_t, un_t> system(
        x0, v0, theta0, omega0, 0.0, vec3::Zero(), 0.0, step_handler_instance, binary_force_functors, unary_force_functors);
    return run<false>(system, dt, n_steps, per_call, mass, inertia, full);
}

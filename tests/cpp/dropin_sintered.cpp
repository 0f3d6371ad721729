// A libgran driver written against the libgran_gb300 drop-in headers: the set-up of libgran's
// test/sintered.cpp (a 3x3x3 cube joined by 5-connector sinter bridges, thrown into rigid motion)
// with the same functor, step handler alias and granular_system composition. Prints the end
// state's radius of gyration and centre displacement. Usage: dropin_sintered [n_steps]
#include <libgran/contact_force/contact_force.h>
#include <libgran/granular_system/granular_system.h>
#include <libgran/sinter_bridge/sinter_bridge.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

struct vec3 {  // a minimal field_value_t (libgran's drivers use Eigen::Vector3d)
    double c[3];
    vec3() : c{0, 0, 0} {}
    vec3(double x, double y, double z) : c{x, y, z} {}
    double operator[](int k) const { return c[k]; }
    double &operator[](int k) { return c[k]; }
    static vec3 Zero() { return vec3(); }
    double norm() const { return std::sqrt((c[0] * c[0] + c[1] * c[1]) + c[2] * c[2]); }
    vec3 normalized() const {
        double z = (c[0] * c[0] + c[1] * c[1]) + c[2] * c[2];
        if (z > 0.0) {
            double s = std::sqrt(z);
            return vec3(c[0] / s, c[1] / s, c[2] / s);
        }
        return *this;
    }
    vec3 cross(vec3 const &o) const {
        return vec3(c[1] * o.c[2] - c[2] * o.c[1], c[2] * o.c[0] - c[0] * o.c[2], c[0] * o.c[1] - c[1] * o.c[0]);
    }
    vec3 operator-(vec3 const &o) const { return vec3(c[0] - o.c[0], c[1] - o.c[1], c[2] - o.c[2]); }
    vec3 operator-() const { return vec3(-c[0], -c[1], -c[2]); }
};

static std::mt19937_64 mt(0);
static std::uniform_real_distribution<double> dist(-1.0, 1.0);

static vec3 generate_random_unit_vector() {
    vec3 v;
    do {
        v = vec3(dist(mt), dist(mt), dist(mt));
    } while (v.norm() == 0);
    return v.normalized();
}

template <typename field_container_t, typename field_value_t>
using sinter_step_handler_double = sinter_step_handler<field_container_t, field_value_t, double>;

static void centre_and_rg(std::vector<vec3> const &x, vec3 &c, double &rg) {
    c = vec3();
    for (auto const &p : x)
        for (int k = 0; k < 3; ++k) c[k] += p[k];
    for (int k = 0; k < 3; ++k) c[k] /= (double)x.size();
    double s = 0;
    for (auto const &p : x) s += (p - c)[0] * (p - c)[0] + (p - c)[1] * (p - c)[1] + (p - c)[2] * (p - c)[2];
    rg = std::sqrt(s / (double)x.size());
}

int main(int argc, char **argv) {
    const double dt = 1e-13;
    const size_t n_steps = argc > 1 ? (size_t)std::atoll(argv[1]) : (size_t)(1.0e-7 / dt);
    const double rho = 1700.0, r_part = 1.4e-8;
    const double mass = 4.0 / 3.0 * M_PI * std::pow(r_part, 3.0) * rho;
    const double inertia = 2.0 / 5.0 * mass * std::pow(r_part, 2.0);
    const double k = 10000.0, gamma_d = 0.0, gamma_n = 5.0e-9, mu = 1.0, phi = 1.0, mu_o = 0.1;
    const double gamma_t = 0.2 * gamma_n, gamma_r = 0.05 * gamma_n, gamma_o = 0.05 * gamma_n;

    std::vector<vec3> x0, v0, theta0, omega0;
    for (size_t i = 0; i < 3; i++) {
        double y = -1.0 * r_part + double(i) * 2.0 * r_part;
        for (size_t j = 0; j < 3; j++) {
            double x = -1.0 * r_part + double(j) * 2.0 * r_part;
            x0.emplace_back(x, y, 0.0);
            x0.emplace_back(x, y, -2.0 * r_part);
            x0.emplace_back(x, y, -4.0 * r_part);
            vec3 vel = j == 0 ? vec3(0.0, 0.0, 5.0) : (j == 2 ? vec3(0.0, 5.0, 0.0) : vec3());
            for (size_t n = 0; n < 3; n++) v0.emplace_back(vel);
        }
    }
    theta0.assign(x0.size(), vec3());
    omega0.assign(x0.size(), vec3());

    sinter_functor<vec3, double> sinter_model(x0.size(), k, gamma_d, k, gamma_n, k, gamma_t, mu, phi, k, gamma_r, mu_o,
                                              phi, k, gamma_o, mu_o, phi, r_part, mass, inertia, dt, vec3::Zero(), 0.0,
                                              x0.begin(), generate_random_unit_vector, 1.0e-9);
    binary_force_functor_container<vec3, double, sinter_functor<vec3, double>> binary_force_functors{sinter_model};
    unary_force_functor_container<vec3, double> unary_force_functors;
    auto step_handler_instance = sinter_model.get_step_handler<std::vector<vec3>>();
    granular_system<vec3, double, rotational_velocity_verlet_half, sinter_step_handler_double,
                    binary_force_functor_container<vec3, double, sinter_functor<vec3, double>>,
                    unary_force_functor_container<vec3, double>>
        system(x0, v0, theta0, omega0, 0.0, vec3::Zero(), 0.0, step_handler_instance, binary_force_functors,
               unary_force_functors);

    vec3 c0, c1;
    double rg0, rg;
    centre_and_rg(system.get_x(), c0, rg0);
    system.do_steps(dt, (int64_t)n_steps, 0);
    if (system.get_a().size() != x0.size() || system.get_alpha().size() != x0.size()) return 3;
    centre_and_rg(system.get_x(), c1, rg);
    const double cd = (c1 - c0).norm();
    std::printf("rg %.9e centre_displacement %.9e\n", rg, cd);
    return 0;
}

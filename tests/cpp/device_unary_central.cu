// libgran_gb300::device_unary (include/libgran_gb300/libgran/body_force/device_unary.cuh): a
// __device__ functor restating the tutorial's central attraction, attached as the unary hook, must
// give the same bits as the engine's built-in LG_BODY_CENTRAL, stepped eagerly and through CUDA
// graphs. Usage: device_unary_central <state_in> (int64 n, x: 3n doubles, v: 3n doubles)
#include <libgran/body_force/device_unary.cuh>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

struct central_dev {
    double kam, c[3];
    __device__ void operator()(int64_t i, const lg_unary_hook_args &s, double a[3], double alpha[3]) const {
        for (int k = 0; k < 3; ++k) a[k] = kam * (c[k] - s.x[4 * i + k]);
    }
};

static lg_system *make(const lg_system_desc &d, std::vector<double> const &x, std::vector<double> const &v) {
    std::vector<double> z(x.size(), 0.0);
    lg_system *s = nullptr;
    if (lg_create(&d, x.data(), v.data(), z.data(), z.data(), nullptr, nullptr, 0, 0, &s) != LG_OK) {
        std::printf("create failed: %s\n", lg_last_error());
        return nullptr;
    }
    return s;
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    FILE *fi = std::fopen(argv[1], "rb");
    int64_t n = 0;
    if (!fi || std::fread(&n, sizeof(n), 1, fi) != 1 || n < 1) return 2;
    std::vector<double> x(3 * (size_t)n), v(3 * (size_t)n);
    if (std::fread(x.data(), sizeof(double), x.size(), fi) != x.size()) return 2;
    if (std::fread(v.data(), sizeof(double), v.size(), fi) != v.size()) return 2;
    std::fclose(fi);

    const double r = 1.4e-8, rho = 1700.0, mass = 4.0 / 3.0 * M_PI * std::pow(r, 3.0) * rho;
    const double inertia = 2.0 / 5.0 * mass * r * r, dt = 1e-13, k_a = 8.0e-6;
    lg_system_desc d;
    std::memset(&d, 0, sizeof(d));
    d.n_part = n;
    d.binary_model = LG_BINARY_CONTACT;
    d.hamaker_model = LG_HAMAKER_FULL;
    d.contact = lg_contact_params{1e4, 5e-9, 1e4, 1e-9, 1.0, 1.0, 1e4, 2.5e-10, 0.1, 1.0, 1e4, 2.5e-10, 0.1, 1.0,
                                  r, mass, inertia, dt};
    d.hamaker = lg_hamaker_params{1e-19, 1e-9, 0.0, r, mass};
    d.pairs = LG_PAIRS_ALL;
    d.precision = LG_PRECISION_FP64;
    d.force_kernel = LG_FORCE_KERNEL_PAIRS;
    double c[3] = {0, 0, 0};
    for (int64_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) c[k] += x[3 * i + k];
    for (int k = 0; k < 3; ++k) c[k] /= (double)n;

    lg_system_desc db = d;
    db.body.model = LG_BODY_CENTRAL;
    db.body.k_a = k_a;
    db.body.mass = mass;
    for (int k = 0; k < 3; ++k) db.body.centre[k] = c[k];
    libgran_gb300::device_unary<central_dev> f{central_dev{k_a / mass, {c[0], c[1], c[2]}}};
    lg_system_desc dh = d;
    dh.unary_hook = &libgran_gb300::device_unary<central_dev>::launch;
    dh.unary_hook_user = &f;

    lg_system *sb = make(db, x, v), *sh = make(dh, x, v);
    if (!sb || !sh) return 1;
    int bad = 0;
    for (int round = 0; round < 3; ++round) {
        // one eager step, then 64 steps replayed from CUDA graphs
        if (lg_step(sb, dt, 1, 0) || lg_step(sh, dt, 1, 0) || lg_step(sb, dt, 64, 0) || lg_step(sh, dt, 64, 0)) {
            std::printf("step failed: %s\n", lg_last_error());
            return 1;
        }
        for (int field = LG_FIELD_X; field <= LG_FIELD_ALPHA; ++field) {
            std::vector<double> ob(3 * (size_t)n), oh(3 * (size_t)n);
            lg_get(sb, field, ob.data());
            lg_get(sh, field, oh.data());
            if (std::memcmp(ob.data(), oh.data(), sizeof(double) * ob.size()) != 0) {
                std::printf("round %d field %d differs\n", round, field);
                bad = 1;
            }
        }
    }
    int64_t launches = 0;
    lg_get_launch_count(sh, &launches);
    lg_destroy(sb);
    lg_destroy(sh);
    std::printf(bad ? "DIFFER\n" : "IDENTICAL launches %lld\n", (long long)launches);
    return bad;
}

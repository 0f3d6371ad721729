// libgran's writer calls (write_particles, write_necks, write_spring_connectors) through the
// drop-in writer.h: reads n, x (3n), theta (3n) from a file and writes into the given directory
// twice each (file counters 1 and 2). Usage: dropin_writer <state_in> <dir> <r_part>
#include <writer.h>

#include <array>
#include <cstdio>
#include <cstdlib>
#include <vector>

struct vec3 {
    double c[3];
    double operator[](int k) const { return c[k]; }
};

int main(int argc, char **argv) {
    if (argc < 4) return 2;
    FILE *f = std::fopen(argv[1], "rb");
    int64_t n = 0;
    if (!f || std::fread(&n, sizeof(n), 1, f) != 1 || n < 2) return 2;
    std::vector<vec3> x((size_t)n), th((size_t)n);
    for (auto *v : {&x, &th})
        for (auto &p : *v)
            if (std::fread(p.c, sizeof(double), 3, f) != 3) return 2;
    std::fclose(f);
    const double r = std::atof(argv[3]);
    std::vector<bool> enabled((size_t)(n * n), true);
    std::vector<std::array<vec3, 5>> conn((size_t)(n * n));
    // necks between consecutive particles; connectors: x_i shifted by q * r / 10 along each axis
    for (int64_t i = 0; i + 1 < n; ++i) {
        enabled[(size_t)(i * n + i + 1)] = enabled[(size_t)((i + 1) * n + i)] = false;
        for (int q = 0; q < 5; ++q) {
            conn[(size_t)(i * n + i + 1)][q] = vec3{{x[i][0] + q * r / 10, x[i][1], x[i][2]}};
            conn[(size_t)((i + 1) * n + i)][q] = vec3{{x[i + 1][0], x[i + 1][1] + q * r / 10, x[i + 1][2]}};
        }
    }
    for (int rep = 0; rep < 2; ++rep) {
        write_particles(argv[2], x, th, r);
        write_necks(argv[2], x, r, enabled);
        write_spring_connectors(argv[2], r, conn, enabled);
    }
    return 0;
}

// lg_writer.cpp -- state dumps in the formats of libgran's writer (writer.cpp:13-170) and of the
// tutorials' CSV dump (Custom-step-handler.md, dump_particle_positions).
//
// The text is what libgran's std::ofstream code produces: numbers through operator<< with the
// default flags and precision (the "%.6g" conversion; here std::to_chars, general format, 6
// digits), coordinates divided by the particle radius, the same headers and separators. The
// orientation fields are the columns of the rotation matrix of the quaternion
// AngleAxis(theta_x, X) * AngleAxis(theta_y, Y) * AngleAxis(theta_z, Z) (writer.cpp:78-115),
// formed with Eigen's published formulas: an axis-angle pair becomes (cos(a/2), sin(a/2) * axis),
// quaternions multiply by the Hamilton product, and the matrix of (w, x, y, z) uses
// t = 2 (x, y, z), e.g. m00 = 1 - (t_y y + t_z z), m10 = t_y x + t_z w.
//
// Large states are formatted in parallel chunks (host threads) into one buffer written with one
// call; the engine-side writers copy the state off the device once.
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "lg_engine_internal.h"

#define LG_TRY(expr)                  \
    do {                              \
        int rc_ = (expr);             \
        if (rc_ != LG_OK) return rc_; \
    } while (0)
#define LG_CUDA(call)                                                                                       \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess) return lg_fail(LG_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_));          \
    } while (0)

namespace {

// operator<<(double) with default flags: "%.6g"
inline char *put_num(char *p, double v) { return std::to_chars(p, p + 40, v, std::chars_format::general, 6).ptr; }

struct quat {
    double w, x, y, z;
};

// Eigen's AngleAxis -> Quaternion about a coordinate axis: w = cos(a/2), vec = sin(a/2) * axis
inline quat axis_angle(double angle, int axis) {
    const double ha = 0.5 * angle, s = std::sin(ha);
    const double e[3] = {axis == 0 ? 1.0 : 0.0, axis == 1 ? 1.0 : 0.0, axis == 2 ? 1.0 : 0.0};
    return quat{std::cos(ha), s * e[0], s * e[1], s * e[2]};
}

inline quat hamilton(quat a, quat b) {
    return quat{a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z, a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
                a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z, a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x};
}

// Columns of the rotation matrix of AngleAxis(t0, X) * AngleAxis(t1, Y) * AngleAxis(t2, Z):
// col[k] = m * unit_k.
inline void orientation(const double *t, double col[3][3]) {
    const quat q = hamilton(hamilton(axis_angle(t[0], 0), axis_angle(t[1], 1)), axis_angle(t[2], 2));
    const double tx = 2.0 * q.x, ty = 2.0 * q.y, tz = 2.0 * q.z;
    const double twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
    const double txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
    const double tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
    const double m[3][3] = {{1.0 - (tyy + tzz), txy - twz, txz + twy},
                            {txy + twz, 1.0 - (txx + tzz), tyz - twx},
                            {txz - twy, tyz + twx, 1.0 - (txx + tyy)}};
    // m * unit_k: ((m(i,0) u0 + m(i,1) u1) + m(i,2) u2)
    for (int k = 0; k < 3; ++k)
        for (int i = 0; i < 3; ++i) {
            const double u0 = k == 0 ? 1.0 : 0.0, u1 = k == 1 ? 1.0 : 0.0, u2 = k == 2 ? 1.0 : 0.0;
            col[k][i] = (m[i][0] * u0 + m[i][1] * u1) + m[i][2] * u2;
        }
}

// Format records [0, count) with fmt(k, p) -> end pointer (at most `per` bytes per record), in
// parallel chunks, appended to out in order.
template <typename F>
void format_records(std::string &out, int64_t count, size_t per, F fmt) {
    if (count <= 0) return;
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (count < 4096) nt = 1;
    const int64_t chunk = (count + nt - 1) / nt;
    std::vector<std::string> parts(nt);
    auto work = [&](unsigned t) {
        const int64_t a = (int64_t)t * chunk, b = std::min<int64_t>(count, a + chunk);
        if (a >= b) return;
        std::string &s = parts[t];
        s.resize((size_t)(b - a) * per);
        char *p = &s[0];
        for (int64_t k = a; k < b; ++k) p = fmt(k, p);
        s.resize((size_t)(p - &s[0]));
    };
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; ++t) th.emplace_back(work, t);
    work(0);
    for (auto &x : th) x.join();
    for (auto &s : parts) out += s;
}

int write_file(const char *path, const std::string &text, const char *what) {
    FILE *f = std::fopen(path, "wb");
    if (!f) return lg_fail(LG_E_INVALID, "%s: unable to create dump file %s", what, path);
    const size_t w = std::fwrite(text.data(), 1, text.size(), f);
    const int c = std::fclose(f);
    if (w != text.size() || c != 0) return lg_fail(LG_E_INVALID, "%s: write to %s failed", what, path);
    return LG_OK;
}

const char *kHeader = "# vtk DataFile Version 4.0\nGenerated by libFractalCommon\nASCII\nDATASET POLYDATA\n";

// Per-value worst case: sign, 6 digits, point, exponent "e-308", separator.
constexpr size_t kNum = 16;

}  // namespace

extern "C" int lg_format_vtk_particles(const double *x, const double *theta, int64_t n, double r_part,
                                       const char *path) {
    if (!path || n < 0 || (n > 0 && (!x || !theta))) return lg_fail(LG_E_INVALID, "lg_format_vtk_particles: bad arguments");
    std::string t = kHeader;
    t += "POINTS " + std::to_string(n) + " FLOAT\n";
    format_records(t, n, 3 * kNum, [&](int64_t i, char *p) {
        for (int c = 0; c < 3; ++c) {
            p = put_num(p, x[3 * i + c] / r_part);
            *p++ = ' ';
        }
        return p;
    });
    t += "\n\nPOINT_DATA " + std::to_string(n) + "\nFIELD FieldData 3\n";
    const char *names[3] = {"thetax", "thetay", "thetaz"};
    for (int k = 0; k < 3; ++k) {
        if (k > 0) t += "\n";
        t += std::string(names[k]) + " 3 " + std::to_string(n) + " double\n";
        format_records(t, n, 3 * kNum, [&](int64_t i, char *p) {
            double col[3][3];
            orientation(theta + 3 * i, col);
            for (int c = 0; c < 3; ++c) {
                p = put_num(p, col[k][c]);
                *p++ = ' ';
            }
            return p;
        });
    }
    t += "\n";
    return write_file(path, t, "lg_format_vtk_particles");
}

extern "C" int lg_format_vtk_necks(const double *x, int64_t n, const int64_t *pairs, int64_t n_pairs, double r_part,
                                   const char *path) {
    if (!path || n < 0 || n_pairs < 0 || (n_pairs > 0 && (!x || !pairs)))
        return lg_fail(LG_E_INVALID, "lg_format_vtk_necks: bad arguments");
    for (int64_t k = 0; k < n_pairs; ++k)
        if (pairs[2 * k] < 0 || pairs[2 * k] >= n || pairs[2 * k + 1] < 0 || pairs[2 * k + 1] >= n)
            return lg_fail(LG_E_INVALID, "lg_format_vtk_necks: pair %lld out of range", (long long)k);
    std::string t = kHeader;
    t += "POINTS " + std::to_string(n_pairs) + " FLOAT\n";
    format_records(t, n_pairs, 3 * kNum, [&](int64_t k, char *p) {
        const double *a = x + 3 * pairs[2 * k], *b = x + 3 * pairs[2 * k + 1];
        for (int c = 0; c < 3; ++c) {
            p = put_num(p, (a[c] + b[c]) / 2.0 / r_part);
            *p++ = ' ';
        }
        return p;
    });
    t += "\n\nPOINT_DATA " + std::to_string(n_pairs) + "\nFIELD FieldData 1\nnormals 3 " + std::to_string(n_pairs) +
         " double\n";
    format_records(t, n_pairs, 3 * kNum, [&](int64_t k, char *p) {
        const double *a = x + 3 * pairs[2 * k], *b = x + 3 * pairs[2 * k + 1];
        double d[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
        const double z = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];  // normalized(): v / norm() when norm > 0
        if (z > 0.0) {
            const double s = std::sqrt(z);
            for (double &c : d) c = c / s;
        }
        for (int c = 0; c < 3; ++c) {
            p = put_num(p, d[c]);
            *p++ = ' ';
        }
        return p;
    });
    return write_file(path, t, "lg_format_vtk_necks");
}

extern "C" int lg_format_vtk_connectors(const double *points, int64_t n_points, double r_part, const char *path) {
    if (!path || n_points < 0 || (n_points > 0 && !points)) return lg_fail(LG_E_INVALID, "lg_format_vtk_connectors: bad arguments");
    std::string t = kHeader;
    t += "POINTS " + std::to_string(n_points) + " FLOAT\n";
    format_records(t, n_points, 3 * kNum, [&](int64_t k, char *p) {
        for (int c = 0; c < 3; ++c) {
            p = put_num(p, points[3 * k + c] / r_part);
            *p++ = ' ';
        }
        return p;
    });
    t += "\n";
    return write_file(path, t, "lg_format_vtk_connectors");
}

extern "C" int lg_format_csv_positions(const double *x, int64_t n, double r_part, const char *path) {
    if (!path || n < 0 || (n > 0 && !x)) return lg_fail(LG_E_INVALID, "lg_format_csv_positions: bad arguments");
    std::string t = "x, y, z\n";
    format_records(t, n, 3 * kNum + 4, [&](int64_t i, char *p) {
        for (int c = 0; c < 3; ++c) {
            p = put_num(p, x[3 * i + c] / r_part);
            if (c < 2) {
                *p++ = ',';
                *p++ = ' ';
            }
        }
        *p++ = '\n';
        return p;
    });
    return write_file(path, t, "lg_format_csv_positions");
}

// ---- engine-side writers: the current state of a handle ---------------------------------------

static int host_field(lg_system *s, int field, std::vector<double> &out) {
    out.resize(3 * (size_t)s->P.n);
    return lg_get(s, field, out.data());
}

extern "C" int lg_write_vtk_particles(lg_system *s, const char *path, double r_part) {
    if (!s) return lg_fail(LG_E_INVALID, "null system handle");
    std::vector<double> x, th;
    LG_TRY(host_field(s, LG_FIELD_X, x));
    LG_TRY(host_field(s, LG_FIELD_THETA, th));
    return lg_format_vtk_particles(x.data(), th.data(), s->P.n, r_part, path);
}

extern "C" int lg_write_csv_positions(lg_system *s, const char *path, double r_part) {
    if (!s) return lg_fail(LG_E_INVALID, "null system handle");
    std::vector<double> x;
    LG_TRY(host_field(s, LG_FIELD_X, x));
    return lg_format_csv_positions(x.data(), s->P.n, r_part, path);
}

extern "C" int lg_write_vtk_necks(lg_system *s, const char *path, double r_part) {
    if (!s) return lg_fail(LG_E_INVALID, "null system handle");
    std::vector<double> x;
    LG_TRY(host_field(s, LG_FIELD_X, x));
    int64_t nb = 0;
    LG_TRY(lg_get_bonds(s, &nb, nullptr, 0));
    std::vector<int64_t> all(2 * (size_t)std::max<int64_t>(nb, 1)), pairs;
    LG_TRY(lg_get_bonds(s, &nb, all.data(), nb));
    for (int64_t k = 0; k < nb; ++k)  // each neck once, i < j, in (i, j) order (writer.cpp:131-136)
        if (all[2 * k] < all[2 * k + 1]) {
            pairs.push_back(all[2 * k]);
            pairs.push_back(all[2 * k + 1]);
        }
    return lg_format_vtk_necks(x.data(), s->P.n, pairs.data(), (int64_t)pairs.size() / 2, r_part, path);
}

extern "C" int lg_get_connectors(lg_system *s, int64_t *n_points, double *out, int64_t capacity) {
    if (!s) return lg_fail(LG_E_INVALID, "null system handle");
    if (!n_points) return lg_fail(LG_E_INVALID, "lg_get_connectors: null count");
    *n_points = 0;
    if (!s->bv.cn) return LG_OK;
    const int64_t n = s->P.n;
    const size_t bs = (size_t)s->bv.bcap * (size_t)n;
    std::vector<double> cn(15 * bs);
    LG_CUDA(cudaStreamSynchronize(s->stream));
    LG_CUDA(cudaMemcpy(cn.data(), s->bv.cn, sizeof(double) * cn.size(), cudaMemcpyDeviceToHost));
    // the bond ends of every particle in ascending partner order, as spring_connectors[i * n + j]
    // (sinter_bridge.h:139, 185-198) is laid out
    std::vector<std::pair<int32_t, size_t>> ends;
    int64_t k = 0;
    for (int64_t i = 0; i < n; ++i) {
        ends.clear();
        for (int b = 0; b < s->bv.bcap; ++b) {
            const size_t e = (size_t)b * (size_t)n + (size_t)i;
            if (s->host_bond_j[e] >= 0) ends.emplace_back(s->host_bond_j[e], e);
        }
        std::sort(ends.begin(), ends.end());
        for (auto &pe : ends)
            for (int q = 0; q < 5; ++q, ++k)
                if (out && k < capacity)
                    for (int c = 0; c < 3; ++c) out[3 * k + c] = cn[(size_t)(3 * q + c) * bs + pe.second];
    }
    *n_points = k;
    return LG_OK;
}

extern "C" int lg_write_vtk_connectors(lg_system *s, const char *path, double r_part) {
    int64_t np = 0;
    LG_TRY(lg_get_connectors(s, &np, nullptr, 0));
    std::vector<double> pts(3 * (size_t)std::max<int64_t>(np, 1));
    LG_TRY(lg_get_connectors(s, &np, pts.data(), np));
    return lg_format_vtk_connectors(pts.data(), np, r_part, path);
}

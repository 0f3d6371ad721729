// lgref_vec3.hpp -- a small 3-vector that satisfies the field_value_t contract of libgran's
// functor templates (the subset of Eigen::Vector3d they call). Evaluation order matches the
// oracle: norm() = sqrt((x*x + y*y) + z*z), dot = (x*x' + y*y') + z*z', normalized() = v / norm().
// TEST INFRASTRUCTURE ONLY: used to compile libgran's own functor headers into the reference
// harness that checks the oracle.
#pragma once
#include <cmath>

struct lgref_vec3 {
    double c[3];
    lgref_vec3() : c{0.0, 0.0, 0.0} {}
    lgref_vec3(double x, double y, double z) : c{x, y, z} {}
    static lgref_vec3 Zero() { return lgref_vec3(0.0, 0.0, 0.0); }
    double &operator[](int k) { return c[k]; }
    double operator[](int k) const { return c[k]; }
    double dot(lgref_vec3 const &o) const { return (c[0] * o.c[0] + c[1] * o.c[1]) + c[2] * o.c[2]; }
    double squaredNorm() const { return (c[0] * c[0] + c[1] * c[1]) + c[2] * c[2]; }
    double norm() const { return std::sqrt(squaredNorm()); }
    lgref_vec3 normalized() const {
        double z = squaredNorm();
        if (z > 0.0) {
            double s = std::sqrt(z);
            return lgref_vec3(c[0] / s, c[1] / s, c[2] / s);
        }
        return *this;
    }
    void normalize() {
        double z = squaredNorm();
        if (z > 0.0) {
            double s = std::sqrt(z);
            c[0] /= s; c[1] /= s; c[2] /= s;
        }
    }
    lgref_vec3 cross(lgref_vec3 const &o) const {
        return lgref_vec3(c[1] * o.c[2] - c[2] * o.c[1], c[2] * o.c[0] - c[0] * o.c[2], c[0] * o.c[1] - c[1] * o.c[0]);
    }
    lgref_vec3 &operator+=(lgref_vec3 const &o) { c[0] += o.c[0]; c[1] += o.c[1]; c[2] += o.c[2]; return *this; }
    lgref_vec3 &operator-=(lgref_vec3 const &o) { c[0] -= o.c[0]; c[1] -= o.c[1]; c[2] -= o.c[2]; return *this; }
    lgref_vec3 &operator*=(double s) { c[0] *= s; c[1] *= s; c[2] *= s; return *this; }
    lgref_vec3 &operator/=(double s) { c[0] /= s; c[1] /= s; c[2] /= s; return *this; }
};
inline lgref_vec3 operator+(lgref_vec3 const &a, lgref_vec3 const &b) { return lgref_vec3(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
inline lgref_vec3 operator-(lgref_vec3 const &a, lgref_vec3 const &b) { return lgref_vec3(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
inline lgref_vec3 operator-(lgref_vec3 const &a) { return lgref_vec3(-a[0], -a[1], -a[2]); }
inline lgref_vec3 operator*(double s, lgref_vec3 const &a) { return lgref_vec3(s * a[0], s * a[1], s * a[2]); }
inline lgref_vec3 operator*(lgref_vec3 const &a, double s) { return lgref_vec3(a[0] * s, a[1] * s, a[2] * s); }
inline lgref_vec3 operator/(lgref_vec3 const &a, double s) { return lgref_vec3(a[0] / s, a[1] / s, a[2] / s); }

// writer.h (libgran_gb300 drop-in) -- libgran's writer (writer.h:15-21, writer.cpp:13-170) with its
// function names, arguments and file naming (dir/particles_<k>.vtk, dir/necks_<k>.vtk,
// dir/spring_connectors_<k>.vtk, k counting from 1 per function) and the same text, formatted by
// the engine library's lg_format_* functions (parallel, no GPU needed). field_value_t is any type
// with operator[](int) (libgran passes Eigen::Vector3d). On a file error the process exits with
// EXIT_FAILURE after printing the reference's message, as libgran's writer does.
#ifndef LIBGRAN_WRITER_H
#define LIBGRAN_WRITER_H
#include <array>
#include <cstdint>
#include <cstdlib>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "../libgran_gb300.h"

namespace libgran_gb300 {
inline size_t &writer_counter(int which) {
    static size_t counters[3] = {1, 1, 1};
    return counters[which];
}
inline std::string next_path(std::string const &dir, const char *stem, int which) {
    std::stringstream path;
    path << dir << "/" << stem << "_" << writer_counter(which) << ".vtk";
    writer_counter(which)++;
    return path.str();
}
inline void writer_check(int status) {
    if (status != LG_OK) {
        std::cerr << "ERROR: Unable to create dump file" << "\n";
        std::exit(EXIT_FAILURE);
    }
}
template <typename field_value_t>
inline std::vector<double> flat(std::vector<field_value_t> const &v) {
    std::vector<double> out(3 * v.size());
    for (size_t i = 0; i < v.size(); ++i)
        for (int c = 0; c < 3; ++c) out[3 * i + c] = v[i][c];
    return out;
}
}  // namespace libgran_gb300

template <typename field_value_t>
void write_particles(const std::string &dir, std::vector<field_value_t> const &x,
                     std::vector<field_value_t> const &theta, double r_part) {
    const std::string path = libgran_gb300::next_path(dir, "particles", 0);
    auto xf = libgran_gb300::flat(x), tf = libgran_gb300::flat(theta);
    libgran_gb300::writer_check(lg_format_vtk_particles(xf.data(), tf.data(), (int64_t)x.size(), r_part, path.c_str()));
}

// enabled_contacts: n*n flags, false where (i, j) is necked (writer.cpp:131-136)
template <typename field_value_t>
void write_necks(std::string const &dir, std::vector<field_value_t> const &x, double r_part,
                 std::vector<bool> const &enabled_contacts) {
    const std::string path = libgran_gb300::next_path(dir, "necks", 2);
    const size_t n = x.size();
    std::vector<int64_t> pairs;
    for (size_t i = 0; i + 1 < n; ++i)
        for (size_t j = i + 1; j < n; ++j)
            if (!enabled_contacts[i * n + j]) {
                pairs.push_back((int64_t)i);
                pairs.push_back((int64_t)j);
            }
    auto xf = libgran_gb300::flat(x);
    libgran_gb300::writer_check(
        lg_format_vtk_necks(xf.data(), (int64_t)n, pairs.data(), (int64_t)pairs.size() / 2, r_part, path.c_str()));
}

// spring_connectors[i * n + j]: the 5 connectors of particle i in bond (i, j); written where
// enabled_contacts[i * n + j] is false (writer.cpp:37-45)
template <typename field_value_t>
void write_spring_connectors(std::string const &dir, double r_part,
                             std::vector<std::array<field_value_t, 5>> const &spring_connectors,
                             std::vector<bool> const &enabled_contacts) {
    const std::string path = libgran_gb300::next_path(dir, "spring_connectors", 1);
    std::vector<double> pts;
    for (size_t k = 0; k < enabled_contacts.size(); ++k)
        if (!enabled_contacts[k])
            for (int q = 0; q < 5; ++q)
                for (int c = 0; c < 3; ++c) pts.push_back(spring_connectors[k][q][c]);
    libgran_gb300::writer_check(
        lg_format_vtk_connectors(pts.data(), (int64_t)pts.size() / 3, r_part, path.c_str()));
}

#endif

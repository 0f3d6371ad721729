// lgref_base.hpp -- the system loop of the reference harness (TEST INFRASTRUCTURE ONLY).
// libgran's functor headers are compiled unmodified; this file supplies what the libgran tree
// lacks (libtimestep's system loop and integrator) with the same definition as the oracle:
// force evaluation at construction, then kick (dt/2), drift, force evaluation, kick (dt/2).
#pragma once
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <utility>
#include <vector>
#include "lgref_vec3.hpp"
#include "../../include/libgran_gb300.h"

using V = lgref_vec3;
using PairT = std::pair<V, V>;
using Field = std::vector<V>;
using BinFn = std::function<PairT(size_t, size_t, Field const &, Field const &, Field const &, Field const &, double)>;
using UnFn = std::function<PairT(size_t, Field const &, Field const &, Field const &, Field const &, double)>;

struct RefSys {
    Field x, v, th, om, a, al;
    BinFn bin;
    UnFn un;  // empty when the unary container is empty
    bool verlet = false;
    double rv = 0.0;
    std::vector<std::vector<size_t>> rows;
    std::vector<std::shared_ptr<void>> keep;  // functor objects the containers refer to
    std::function<void(size_t, size_t, double *)> springs;  // (i, j) -> 9 doubles
    std::function<int64_t(int64_t *, int64_t)> bonds;      // intact ordered bonded pairs
    std::vector<std::function<void(double)>> facet_move;
    std::vector<std::function<void(double *)>> facet_vertices;
    bool facet_auto_move = false;
    // step handler increments of the drift (sinter_step_handler of the 5-connector model); empty:
    // plain x += v*dt, theta += omega*dt
    std::function<void(size_t, V const &)> inc_x, inc_theta;
    // a custom step handler that holds increments (Custom-step-handler.md:82-97): LG_HOLD_* bits per
    // particle; a held increment is not passed on to the base handler
    std::vector<uint8_t> hold;
    std::function<void(const double *)> set_centre;  // central body force: the tutorial's update
    int64_t step_index = 0;
    double t = 0.0;

    void build_rows() {
        size_t n = x.size();
        rows.assign(n, {});
        for (size_t i = 0; i < n; ++i)
            for (size_t j = 0; j < n; ++j) {
                if (j == i) continue;
                if (!verlet || (x[i] - x[j]).squaredNorm() < rv * rv) rows[i].push_back(j);
            }
    }
    void forces() {
        size_t n = x.size();
        for (size_t i = 0; i < n; ++i) {
            PairT acc = std::make_pair(V::Zero(), V::Zero());
            for (size_t j : rows[i]) {  // pair += pair, as libgran's operator_overloads.h:16-20
                PairT p = bin(i, j, x, v, th, om, t);
                acc.first += p.first;
                acc.second += p.second;
            }
            if (un) {
                PairT p = un(i, x, v, th, om, t);
                acc.first += p.first;
                acc.second += p.second;
            }
            a[i] = acc.first;
            al[i] = acc.second;
        }
    }
    unsigned held(size_t i) const { return hold.empty() ? 0u : hold[i]; }
    void kick(double hdt) {
        for (size_t i = 0; i < x.size(); ++i) {
            if (!(held(i) & LG_HOLD_V)) v[i] += a[i] * hdt;
            if (!(held(i) & LG_HOLD_OMEGA)) om[i] += al[i] * hdt;
        }
    }
    void step(double dt, int64_t nsteps, int64_t rebuild_every) {
        size_t n = x.size();
        double hdt = dt / 2.0;
        for (int64_t s = 0; s < nsteps; ++s) {
            if (verlet && rebuild_every > 0 && step_index % rebuild_every == 0) build_rows();
            kick(hdt);
            for (size_t i = 0; i < n; ++i) {
                const unsigned h = held(i);
                if (!(h & LG_HOLD_X)) {
                    if (inc_x) inc_x(i, v[i] * dt); else x[i] += v[i] * dt;
                }
                if (!(h & LG_HOLD_THETA)) {
                    if (inc_theta) inc_theta(i, om[i] * dt); else th[i] += om[i] * dt;
                }
            }
            forces();
            kick(hdt);
            if (facet_auto_move)
                for (auto &mv : facet_move) mv(dt);
            ++step_index;
        }
    }
};

inline Field to_field(const double *p, int64_t n) {
    Field f((size_t)n);
    for (int64_t i = 0; i < n; ++i) f[(size_t)i] = V(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
    return f;
}

// Factories exported by each harness translation unit (the libgran headers cannot all share one
// unit: alt_sinter_bridge.h and alt_breaking_sinter_bridge.h use the same include guard, and
// hamaker_force.h and limited_range_hamaker_force.h both define square() and cube()).
RefSys *lgref_make_alt_full(const lg_system_desc *, const double *, const double *, const double *, const double *,
                            const lg_facet_desc *, const double *, int64_t);
RefSys *lgref_make_alt_limited(const lg_system_desc *, const double *, const double *, const double *, const double *,
                               const lg_facet_desc *, const double *, int64_t);
RefSys *lgref_make_brk_full(const lg_system_desc *, const double *, const double *, const double *, const double *,
                            const lg_facet_desc *, const double *, int64_t);
RefSys *lgref_make_brk_limited(const lg_system_desc *, const double *, const double *, const double *, const double *,
                               const lg_facet_desc *, const double *, int64_t);
RefSys *lgref_make_conn_full(const lg_system_desc *, const double *, const double *, const double *, const double *,
                             const lg_facet_desc *, const double *, int64_t);
RefSys *lgref_make_conn_limited(const lg_system_desc *, const double *, const double *, const double *, const double *,
                                const lg_facet_desc *, const double *, int64_t);

// lg_compact.cuh -- pieces shared by the FP64 (lg_forces_compact.cu) and mixed-precision
// (lg_forces_compact_mixed.cu) warp-compacted force kernels: the slot windows, the slicing of a
// row's windows over several warps, and the per-particle tail of a force evaluation (unary facet
// terms, stores, half kick, finiteness check). Everything here is inline device code, so each
// translation unit compiles it with its own floating-point flags.
#pragma once
#include "lg_common.cuh"

namespace lg {
namespace compact {

constexpr int kWin = 4;           // slots per window (classified per memory round trip)
constexpr int kHCap = 32 * kWin;  // Hamaker queue capacity per window

// Slicing: the windows of a 32-row group may be split over SL warps (window w of a row goes to
// warp w % SL); virtual slot v of slice sl (its windows sl, sl + SL, ...) -> slot of the row.
template <int SL>
__device__ __forceinline__ int64_t slot_of(int64_t v, int sl) {
    return ((v / kWin) * SL + sl) * kWin + (v % kWin);
}

// Facet auto-move: the vertices one step ahead, written once per launch into the second vertex
// buffer; the engine swaps the two buffers after the step.
__device__ __forceinline__ void move_facets(const Params &P, const StateView &S, double dt) {
    for (int f = 0; f < P.n_facets; ++f)
        for (int q = 0; q < 9; ++q) S.facet_vert_next[9 * f + q] = S.facet_vert[9 * f + q] + P.facets[f].v[q % 3] * dt;
}

// Unary terms of particle i: the facets in order, then the body-force term (P.ext_a / P.ext_al),
// folded as the reference's unary container folds its functors, f0 + (f1 + (... + body))
// (unary_force_container.h:27-29): the last term first, each earlier one added in front. Returns
// false when there is no unary term. Kept out of line: the common no-facet path then needs few
// registers; static: each translation unit keeps its own copy, compiled with its own
// floating-point flags.
static __device__ __noinline__ bool unary_terms(const Params &P, const StateView &S, int64_t i, int64_t n, d3 vi,
                                                d3 wi, d3 &ua, d3 &ual) {
    const d3 xi = ld4(S.x, i);
    bool have = false;
    if (P.ext_a) {
        ua = ld4(P.ext_a, i);
        ual = ld4(P.ext_al, i);
        have = true;
    }
    for (int f = P.n_facets - 1; f >= 0; --f) {
        const FacetDev &fd = P.facets[f];
        d3 N = mk3(fd.normal[0], fd.normal[1], fd.normal[2]);
        d3 xf = closest_point_on_triangle(S.facet_vert + 9 * f, fd.area, N, xi);
        d3 vf = mk3(fd.v[0], fd.v[1], fd.v[2]);
        d3 fa = zero3(), fal = zero3();
        bool hv = false;
        if (fd.has_contact) {
            const int64_t base = (int64_t)f * 9 * n;
            d3 s[3];
#pragma unroll
            for (int q = 0; q < 3; ++q)
                s[q] = mk3(S.sxi[base + (3 * q) * n + i], S.sxi[base + (3 * q + 1) * n + i],
                           S.sxi[base + (3 * q + 2) * n + i]);
            surface_contact(fd.contact, xf, vf, xi, vi, wi, s, fa, fal);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                S.sxi[base + (3 * q) * n + i] = s[q].x;
                S.sxi[base + (3 * q + 1) * n + i] = s[q].y;
                S.sxi[base + (3 * q + 2) * n + i] = s[q].z;
            }
            hv = true;
        }
        if (fd.has_hamaker) {
            d3 ha = surface_hamaker(fd.hamaker, xf, xi);
            if (hv) {
                fa = add(fa, ha);
                fal = add(fal, zero3());
            } else {
                fa = ha;
                fal = zero3();
            }
        }
        if (have) {
            ua = add(fa, ua);
            ual = add(fal, ual);
        } else {
            ua = fa;
            ual = fal;
            have = true;
        }
    }
    return have;
}

// Tail of particle i's force evaluation: the unary terms (facets, body force), added after the
// binary sums (accA, accW return the totals); stores a and alpha, the half-kicked velocities (a held
// increment keeps the velocity), and flags non-finite results. FACETS = false: the caller knows
// there is no unary term.
template <bool FACETS = true>
__device__ __forceinline__ void finish_row(const Params &P, const StateView &S, int64_t i, int64_t n, d3 &accA,
                                           d3 &accW, d3 vi, d3 wi, double hdt) {
    if (FACETS && (P.n_facets > 0 || P.ext_a)) {
        d3 ua, ual;
        if (unary_terms(P, S, i, n, vi, wi, ua, ual)) {
            accA = add(accA, ua);
            accW = add(accW, ual);
        }
    }
    const uint32_t h = hold_of(P.hold, i);
    st4(S.a, i, accA);
    st4(S.al, i, accW);
    st4(S.v_out, i, kick_unless(vi, hdt, accA, h & LG_HOLD_V));
    st4(S.w_out, i, kick_unless(wi, hdt, accW, h & LG_HOLD_OMEGA));
    if (!isfinite(accA.x) || !isfinite(accA.y) || !isfinite(accA.z) || !isfinite(accW.x) || !isfinite(accW.y) ||
        !isfinite(accW.z))
        set_error(S.err, LG_DEVERR_NONFINITE);
}

}  // namespace compact
}  // namespace lg

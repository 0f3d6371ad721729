// harness_api.cpp -- C entry points of the reference harness (TEST INFRASTRUCTURE ONLY).
#include "lgref_base.hpp"

extern "C" {

void *lgref_create(const lg_system_desc *d, const double *x0, const double *v0, const double *th0, const double *om0,
                   const lg_facet_desc *facets, const double *neck, int64_t n_neck) {
    bool brk = d->binary_model == LG_BINARY_BREAKING_SINTER;
    bool lim = d->hamaker_model == LG_HAMAKER_LIMITED;
    if (d->binary_model == LG_BINARY_SINTER_CONNECTORS)
        return lim ? lgref_make_conn_limited(d, x0, v0, th0, om0, facets, neck, n_neck)
                   : lgref_make_conn_full(d, x0, v0, th0, om0, facets, neck, n_neck);
    if (brk && lim) return lgref_make_brk_limited(d, x0, v0, th0, om0, facets, neck, n_neck);
    if (brk) return lgref_make_brk_full(d, x0, v0, th0, om0, facets, neck, n_neck);
    if (lim) return lgref_make_alt_limited(d, x0, v0, th0, om0, facets, neck, n_neck);
    return lgref_make_alt_full(d, x0, v0, th0, om0, facets, neck, n_neck);
}

void lgref_destroy(void *h) { delete (RefSys *)h; }

int lgref_step(void *h, double dt, int64_t nsteps, int64_t rebuild_every) {
    ((RefSys *)h)->step(dt, nsteps, rebuild_every);
    return 0;
}

int lgref_update_neighbor_list(void *h) {
    RefSys *s = (RefSys *)h;
    if (s->verlet) s->build_rows();
    return 0;
}

int lgref_get(void *h, int field, double *out) {
    RefSys *s = (RefSys *)h;
    Field *f = nullptr;
    switch (field) {
        case LG_FIELD_X: f = &s->x; break;
        case LG_FIELD_V: f = &s->v; break;
        case LG_FIELD_THETA: f = &s->th; break;
        case LG_FIELD_OMEGA: f = &s->om; break;
        case LG_FIELD_A: f = &s->a; break;
        case LG_FIELD_ALPHA: f = &s->al; break;
        default: return -1;
    }
    for (size_t i = 0; i < f->size(); ++i)
        for (int k = 0; k < 3; ++k) out[3 * i + k] = (*f)[i][k];
    return 0;
}

int lgref_set_body_centre(void *h, const double *c) {
    RefSys *s = (RefSys *)h;
    if (!s->set_centre) return -1;
    s->set_centre(c);
    return 0;
}

int lgref_pair_springs(void *h, int64_t i, int64_t j, double *out9) {
    ((RefSys *)h)->springs((size_t)i, (size_t)j, out9);
    return 0;
}

int64_t lgref_bonds(void *h, int64_t *pairs, int64_t cap) { return ((RefSys *)h)->bonds(pairs, cap); }

int lgref_facet_get_vertices(void *h, int32_t f, double *out9) {
    RefSys *s = (RefSys *)h;
    if (f < 0 || (size_t)f >= s->facet_vertices.size()) return -1;
    s->facet_vertices[(size_t)f](out9);
    return 0;
}

int lgref_facet_update_positions(void *h, int32_t f, double dt) {
    RefSys *s = (RefSys *)h;
    if (f < 0 || (size_t)f >= s->facet_move.size()) return -1;
    s->facet_move[(size_t)f](dt);
    return 0;
}
}

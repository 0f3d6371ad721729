"""The libgran known-answer simulations, restated as system descriptions.

Each entry rebuilds the set-up of one of libgran's own end-to-end tests (parameters, initial state,
step count and the end-state targets it checks at 1 %):
  contact         test/contact.cpp:30-77,111-122
  hamaker         test/hamaker.cpp:30-90,127-142
  hamaker_nbr     test/hamaker_neighbor.cpp (same set-up, Verlet list r=5r rebuilt every 20 steps,
                  :115,121-122,129-144)
  alt_sintered    test/alt_sintered.cpp:37-96,141-149
  sintered        test/sintered.cpp:54-106,137-150 (5-connector sinter_functor with its
                  sinter_step_handler; connector axes drawn from a seeded generator, as the test draws
                  them from its own, test/sintered.cpp:30-39)
  surface         test/surface.cpp:48-90,117-123
"""
import math

import numpy as np

from libgran_gb300 import _abi as A
from libgran_gb300 import configs as K

R = 1.4e-8
RHO = 1700.0
MASS = K.mass_of(R, RHO)
INERTIA = K.inertia_of(MASS, R)


def _contact(dt, mu=1.0):
    k, gamma_n, phi, mu_o = 10000.0, 5.0e-9, 1.0, 0.1
    gamma_t, gamma_r, gamma_o = 0.2 * gamma_n, 0.05 * gamma_n, 0.05 * gamma_n
    # argument pattern of the drivers: (k, gamma_n, k, gamma_t, mu, phi, k, gamma_r, mu_o, phi, k, gamma_o, mu_o, phi)
    return K.contact_params(k, gamma_n, k, gamma_t, mu, phi, k, gamma_r, mu_o, phi, k, gamma_o, mu_o, phi,
                            R, MASS, INERTIA, dt)


def _plate_and_projectile():
    x0 = []
    for i in range(3):
        y = -3.0 * R + float(i) * 2.0 * R
        for j in range(3):
            x = -3.0 * R + float(j) * 2.0 * R
            x0.append((x, y, 0.0))
            x0.append((x, y, -2.0 * R))
    x0.append((0.0, 0.0, 3.0 * R))
    x0 = np.array(x0)
    v0 = np.zeros_like(x0)
    v0[-1] = (1.0, 0.0, -10.0)
    return x0, v0


def contact_case():
    dt = 1e-13
    x0, v0 = _plate_and_projectile()
    desc = K.make_desc(len(x0), A.LG_BINARY_CONTACT, A.LG_HAMAKER_NONE, contact=_contact(dt))
    return dict(name="contact", desc=desc, x0=x0, v0=v0, dt=dt, nsteps=int(3.0e-7 / dt), rebuild=0,
                targets={"linear_momentum": 1.96373e-19, "ke_total": 3.4925e-19})


def hamaker_case(neighbor=False):
    dt = 1e-13
    x0, v0 = _plate_and_projectile()
    desc = K.make_desc(len(x0), A.LG_BINARY_CONTACT, A.LG_HAMAKER_FULL, contact=_contact(dt),
                       hamaker=K.hamaker_params(1.0e-20, 1.0e-9, R, MASS),
                       pairs=A.LG_PAIRS_VERLET if neighbor else A.LG_PAIRS_ALL,
                       r_verlet=5.0 * R if neighbor else 0.0)
    return dict(name="hamaker_nbr" if neighbor else "hamaker", desc=desc, x0=x0, v0=v0, dt=dt,
                nsteps=int(3.0e-7 / dt), rebuild=20 if neighbor else 0,
                targets={"linear_momentum": 1.96373e-19, "ke_total": 8.33959e-20,
                         "radius_of_gyration": 3.56253e-08})


def alt_sintered_case():
    dt = 5e-14
    k_bond = 1000.0
    gamma_n_bond = 2.0 * math.sqrt(2.0 * MASS * k_bond)
    x0, v0 = [], []
    for i in range(3):
        y = -1.0 * R + float(i) * 2.0 * R
        for j in range(3):
            x = -1.0 * R + float(j) * 2.0 * R
            x0 += [(x, y, 0.0), (x, y, -2.0 * R), (x, y, -4.0 * R)]
            vel = (0.0, 0.0, 5.0) if j == 0 else ((0.0, 5.0, 0.0) if j == 2 else (0.0, 0.0, 0.0))
            v0 += [vel] * 3
    x0, v0 = np.array(x0), np.array(v0)
    sinter = K.sinter_params(k_bond, gamma_n_bond, k_bond, 0.2 * gamma_n_bond, k_bond, 0.05 * gamma_n_bond,
                             k_bond, 0.05 * gamma_n_bond, R, MASS, INERTIA, dt, 1.0e-9)
    desc = K.make_desc(len(x0), A.LG_BINARY_SINTER, A.LG_HAMAKER_NONE, contact=_contact(dt), sinter=sinter)
    return dict(name="alt_sintered", desc=desc, x0=x0, v0=v0, dt=dt, nsteps=int(1.0e-7 / dt), rebuild=0,
                targets={"radius_of_gyration": 3.9598e-08, "center_displacement": 2.35702e-07})


def sintered_case():
    dt = 1e-13
    x0, v0 = [], []
    for i in range(3):
        y = -1.0 * R + float(i) * 2.0 * R
        for j in range(3):
            x = -1.0 * R + float(j) * 2.0 * R
            x0 += [(x, y, 0.0), (x, y, -2.0 * R), (x, y, -4.0 * R)]
            vel = (0.0, 0.0, 5.0) if j == 0 else ((0.0, 5.0, 0.0) if j == 2 else (0.0, 0.0, 0.0))
            v0 += [vel] * 3
    x0, v0 = np.array(x0), np.array(v0)
    k, gamma_n, mu, phi, mu_o = 10000.0, 5.0e-9, 1.0, 1.0, 0.1
    # the driver's sinter_functor arguments (test/sintered.cpp:106): k_d = k, gamma_d = 0, then the
    # contact pattern (k, gamma_n, k, gamma_t, mu, phi, k, gamma_r, mu_o, phi, k, gamma_o, mu_o, phi)
    cp = K.contact_params(k, gamma_n, k, 0.2 * gamma_n, mu, phi, k, 0.05 * gamma_n, mu_o, phi, k, 0.05 * gamma_n,
                          mu_o, phi, R, MASS, INERTIA, dt)
    desc = K.make_desc(len(x0), A.LG_BINARY_SINTER_CONNECTORS, A.LG_HAMAKER_NONE, contact=cp)
    nb = len(K.connector_bonds(x0, R, 1.0e-9))
    K.set_connectors(desc, k, 0.0, 1.0e-9, K.random_unit_axes(nb, 0))
    return dict(name="sintered", desc=desc, x0=x0, v0=v0, dt=dt, nsteps=int(1.0e-7 / dt), rebuild=0,
                targets={"radius_of_gyration": 3.95981e-08, "center_displacement": 2.35702e-07})


def surface_facet(dt, A_h=0.0, h0=1.0e-9, mu=0.5):
    a = 50.0 * R
    f = A.lg_facet_desc()
    for c in range(3):
        f.v_facet[c] = 0.0
    verts = [(-a, -a, 0.0), (-a, a, 0.0), (a, -a, 0.0)]
    for k, v in enumerate(verts):
        for c in range(3):
            f.vertices[3 * k + c] = v[c]
    f.has_contact = 1
    f.has_hamaker = 1
    f.contact = _contact(dt, mu=mu)
    f.hamaker = K.hamaker_params(A_h, h0, R, MASS)
    return f


def surface_case():
    dt = 1e-13
    x0 = np.array([(0.5 * R, 0.5 * R, 2.5 * R)])
    v0 = np.array([(0.0, 0.0, -0.5)])
    desc = K.make_desc(1, A.LG_BINARY_CONTACT, A.LG_HAMAKER_NONE, contact=_contact(dt, mu=0.5), n_facets=1)
    return dict(name="surface", desc=desc, x0=x0, v0=v0, dt=dt, nsteps=int(5.0e-7 / dt), rebuild=0,
                facets=[surface_facet(dt)], targets={"ke_total": 1.0922e-21})


def all_cases():
    return [contact_case(), hamaker_case(False), hamaker_case(True), alt_sintered_case(), sintered_case(),
            surface_case()]


def measured(case, obs0, obs1):
    """The quantities the reference tests compare, from observables at start and end."""
    out = {"linear_momentum": obs1["linear_momentum"], "ke_total": obs1["ke_total"],
           "radius_of_gyration": obs1["radius_of_gyration"]}
    c0, c1 = np.array(obs0["center_of_mass"]), np.array(obs1["center_of_mass"])
    out["center_displacement"] = float(np.linalg.norm(c1 - c0))
    return out

"""Small systems whose trajectories are pinned by golden fixtures (tests/golden/*.npz).

Each case is a system description plus initial state; make_golden.py runs it through the reference
harness (libgran's own functors) and stores the states at the checkpoints. The same cases drive
the oracle and GPU parity tests.
"""
import numpy as np

from libgran_gb300 import _abi as A
from libgran_gb300 import configs as K
from libgran_gb300.system import generate_aggregate, generate_velocities

import known_answer as KA


def _neck(nb, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(5e-10, 2e-9, size=nb)


def _bond_count(desc, x0):
    # bonds of the breaking functor: every pair with |(|x_i - x_j| - 2r)| < d_crit (no cycle check)
    r, dc = desc.sinter.r_part, desc.sinter.critical_separation
    n = len(x0)
    d = np.sqrt(((x0[:, None, :] - x0[None, :, :]) ** 2).sum(-1))
    iu = np.triu_indices(n, 1)
    return int((np.abs(d[iu] - 2.0 * r) < dc).sum())


def centroid_seq(x):
    """Centroid as the tutorial's update_center_of_mass forms it: sum in index order, then / count."""
    c = np.zeros(3)
    for p in x:
        c = c + p
    return c / float(len(x))


def cases():
    out = []
    # 1. plate + projectile, contact + full Hamaker (test/hamaker.cpp set-up), short run
    c = KA.hamaker_case(False)
    out.append(dict(name="plate_contact_hamaker", desc=c["desc"], x0=c["x0"], v0=c["v0"], dt=c["dt"],
                    checkpoints=[0, 1, 10, 100, 3000], spring_pairs=[(18, 9), (9, 18), (18, 8), (0, 1)]))
    # 2. same through a Verlet list (test/hamaker_neighbor.cpp set-up)
    c = KA.hamaker_case(True)
    out.append(dict(name="plate_verlet", desc=c["desc"], x0=c["x0"], v0=c["v0"], dt=c["dt"], rebuild=20,
                    checkpoints=[0, 1, 40, 3000], spring_pairs=[(18, 9), (9, 18)]))
    # 3. sintered cube (test/alt_sintered.cpp set-up, cycle-free bonds), short run
    c = KA.alt_sintered_case()
    out.append(dict(name="cube_sinter", desc=c["desc"], x0=c["x0"], v0=c["v0"], dt=c["dt"],
                    checkpoints=[0, 1, 10, 500], spring_pairs=[(0, 1), (1, 0), (0, 3), (13, 14)]))
    # 4. RSA aggregate, sintered bonds + limited Hamaker (aggregate workload constants)
    mat = K.Material()
    x0 = generate_aggregate(11, 48, mat.r)
    v0 = generate_velocities(11, 48, 0.1)
    d = K.make_desc(48, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(), sinter=mat.sinter(),
                    hamaker=mat.hamaker())
    out.append(dict(name="rsa48_sinter_limited", desc=d, x0=x0, v0=v0, dt=mat.dt, checkpoints=[0, 1, 10, 200],
                    spring_pairs=[(0, 1), (1, 0), (2, 5)]))
    # 5. RSA aggregate, breaking bonds (reference neck indexing) + full Hamaker, compressed velocities
    x0 = generate_aggregate(12, 40, mat.r)
    v0 = -2.0e7 * (x0 - x0.mean(0))  # inward motion so that bonds load and break
    d = K.make_desc(40, A.LG_BINARY_BREAKING_SINTER, A.LG_HAMAKER_FULL, contact=mat.contact(), sinter=mat.sinter(),
                    hamaker=mat.hamaker(), neck_mode=A.LG_NECK_REFERENCE_INDEXING)
    nb = _bond_count(d, x0)
    out.append(dict(name="rsa40_breaking_full", desc=d, x0=x0, v0=v0, dt=mat.dt, checkpoints=[0, 1, 10, 300],
                    neck=_neck(nb, 5), spring_pairs=[(0, 1), (1, 0)]))
    # 6. contact + simplified Hamaker on the plate
    c = KA.contact_case()
    d = K.make_desc(19, A.LG_BINARY_CONTACT, A.LG_HAMAKER_SIMPLIFIED, contact=c["desc"].contact,
                    hamaker=K.hamaker_params(1.0e-20, 1.0e-9, KA.R, KA.MASS))
    out.append(dict(name="plate_simplified", desc=d, x0=c["x0"], v0=c["v0"], dt=c["dt"], checkpoints=[0, 10, 2000],
                    spring_pairs=[(18, 9)]))
    # 7. particle on a moving facet with surface contact + surface Hamaker
    c = KA.surface_case()
    f = KA.surface_facet(c["dt"], A_h=1.0e-20, h0=1.0e-9, mu=0.5)
    f.v_facet[2] = 0.2
    d = K.make_desc(1, A.LG_BINARY_CONTACT, A.LG_HAMAKER_NONE, contact=c["desc"].contact, n_facets=1,
                    facet_auto_move=1)
    out.append(dict(name="facet_moving", desc=d, x0=c["x0"], v0=c["v0"] * 0.0 + np.array([0.3, 0.1, -0.5]),
                    dt=c["dt"], checkpoints=[0, 10, 2000, 6000], facets=[f]))
    # 8. 5-connector sintered cube (test/sintered.cpp set-up), short run
    c = KA.sintered_case()
    out.append(dict(name="cube_connectors", desc=c["desc"], x0=c["x0"], v0=c["v0"], dt=c["dt"],
                    checkpoints=[0, 1, 10, 500]))
    # 9. RSA aggregate, 5-connector bonds + limited Hamaker, inward motion (contacts between
    #    non-bonded monomers)
    x0 = generate_aggregate(13, 40, mat.r)
    v0 = -1.5e7 * (x0 - x0.mean(0)) + generate_velocities(13, 40, 0.2)
    d = K.make_desc(40, A.LG_BINARY_SINTER_CONNECTORS, A.LG_HAMAKER_LIMITED, contact=mat.contact(),
                    hamaker=mat.hamaker())
    nb = len(K.connector_bonds(x0, mat.r, mat.d_crit))
    K.set_connectors(d, 0.5 * mat.k_n, 0.5 * mat.g_n, mat.d_crit, K.random_unit_axes(nb, 13))
    out.append(dict(name="rsa40_connectors_limited", desc=d, x0=x0, v0=v0, dt=mat.dt, checkpoints=[0, 1, 10, 300],
                    spring_pairs=[(0, 1), (1, 0), (0, 2)]))
    # 10. the custom step-handler tutorial set-up (Custom-step-handler.md: contact + Hamaker with
    #     A = 1e-19, the central attraction body force k_a = 8e-6 towards the initial centroid, the
    #     velocity of particle 10 held) on a seeded RSA aggregate of 60 monomers
    c = KA.contact_case()
    x0 = generate_aggregate(14, 60, KA.R)
    d = K.make_desc(60, A.LG_BINARY_CONTACT, A.LG_HAMAKER_FULL, contact=c["desc"].contact,
                    hamaker=K.hamaker_params(1.0e-19, 1.0e-9, KA.R, KA.MASS))
    d.body = K.central_body(8.0e-6, KA.MASS, centroid_seq(x0))
    hold = np.zeros(60, dtype=np.uint8)
    hold[10] = A.LG_HOLD_V
    K.set_hold(d, hold)
    out.append(dict(name="tutorial_central_fixed", desc=d, x0=x0, v0=generate_velocities(14, 60, 0.05), dt=c["dt"],
                    checkpoints=[0, 1, 10, 400], spring_pairs=[(0, 1), (10, 11)]))
    # 11. three facets (a floor of two triangles and a tilted wall), a central body force after them,
    #     and held increments (x of one particle, theta of another, v and omega of a third): the unary container's
    #     right fold f0 + (f1 + (f2 + body))
    x0 = generate_aggregate(15, 24, KA.R) + np.array([0.0, 0.0, 9.0 * KA.R])
    x0[:, 2] -= x0[:, 2].min() - 0.995 * KA.R  # the lowest monomer starts touching the floor
    v0 = generate_velocities(15, 24, 0.2) + np.array([0.3, -0.2, -1.0])
    fl = []
    a_ = 40.0 * KA.R
    for verts in ([(-a_, -a_, 0.0), (a_, -a_, 0.0), (-a_, a_, 0.0)], [(a_, a_, 0.0), (-a_, a_, 0.0), (a_, -a_, 0.0)],
                  [(6.0 * KA.R, -a_, -a_), (6.0 * KA.R, a_, -a_), (4.0 * KA.R, -a_, a_)]):
        f = KA.surface_facet(c["dt"], A_h=2.0e-20, h0=1.0e-9, mu=0.5)
        for k, v in enumerate(verts):
            for q in range(3):
                f.vertices[3 * k + q] = v[q]
        fl.append(f)
    d = K.make_desc(24, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED, contact=c["desc"].contact,
                    hamaker=K.hamaker_params(1.0e-20, 1.0e-9, KA.R, KA.MASS, r_cutoff=4.0 * KA.R), n_facets=3)
    d.body = K.central_body(2.0e-6, KA.MASS, x0.mean(0) + np.array([0.0, 0.0, 3.0 * KA.R]))
    hold = np.zeros(24, dtype=np.uint8)
    hold[3] = A.LG_HOLD_X
    hold[7] = A.LG_HOLD_THETA
    hold[12] = A.LG_HOLD_OMEGA | A.LG_HOLD_V
    K.set_hold(d, hold)
    out.append(dict(name="three_facets_body_hold", desc=d, x0=x0, v0=v0, dt=c["dt"], checkpoints=[0, 1, 10, 600],
                    facets=fl, spring_pairs=[(0, 1)]))
    return out

"""Parameter presets: the material constants libgran's drivers use and the seeded synthetic
aggregate workloads (r = 14 nm soot monomers, density 1700 kg/m^3).

Reference: the constants of test/contact.cpp:37-51 (rho, r_part, mass, inertia, k, gamma_n, mu, phi,
mu_o, gamma_t, gamma_r, gamma_o) and the functor argument order of contact_force.h:10-30.
"""
import ctypes as C
import math

import numpy as np

from . import _abi as A

PI = 3.14159265358979323846
RHO = 1700.0
R_PART = 1.4e-8


def mass_of(r=R_PART, rho=RHO):
    """4/3 pi r^3 rho, written as test/contact.cpp:40 computes it."""
    return 4.0 / 3.0 * PI * math.pow(r, 3.0) * rho


def inertia_of(m, r=R_PART):
    """2/5 m r^2 (test/contact.cpp:41)."""
    return 2.0 / 5.0 * m * math.pow(r, 2.0)


def contact_params(k, gamma_n, k_t, gamma_t, mu_s, phi_d, k_r, gamma_r, mu_r, phi_r, k_o, gamma_o, mu_o, phi_o,
                   r_part, mass, inertia, dt):
    """Same argument order as contact_force_functor's constructor (contact_force.h:10-30)."""
    return A.lg_contact_params(k, gamma_n, k_t, gamma_t, mu_s, phi_d, k_r, gamma_r, mu_r, phi_r, k_o, gamma_o,
                               mu_o, phi_o, r_part, mass, inertia, dt)


def sinter_params(k, gamma_n, k_t, gamma_t, k_r, gamma_r, k_o, gamma_o, r_part, mass, inertia, dt,
                  critical_separation):
    """Same argument order as alt_sinter_functor's constructor (alt_sinter_bridge.h:19-36)."""
    return A.lg_sinter_params(k, gamma_n, k_t, gamma_t, k_r, gamma_r, k_o, gamma_o, r_part, mass, inertia, dt,
                              critical_separation)


def hamaker_params(A_, h0, r_part, mass, r_cutoff=0.0):
    return A.lg_hamaker_params(A_, h0, r_cutoff, r_part, mass)


def make_desc(n_part, binary_model=A.LG_BINARY_CONTACT, hamaker_model=A.LG_HAMAKER_NONE, contact=None,
              sinter=None, hamaker=None, neck_mode=A.LG_NECK_PER_BOND, pairs=A.LG_PAIRS_ALL, r_verlet=0.0,
              precision=A.LG_PRECISION_FP64, n_facets=0, facet_auto_move=0, max_neighbors=0, threads_per_row=0,
              force_kernel=A.LG_FORCE_KERNEL_AUTO):
    d = A.lg_system_desc()
    d.n_part = int(n_part)
    d.binary_model = binary_model
    d.hamaker_model = hamaker_model
    if contact is not None:
        d.contact = contact
    if sinter is not None:
        d.sinter = sinter
    if hamaker is not None:
        d.hamaker = hamaker
    d.neck_mode = neck_mode
    d.pairs = pairs
    d.r_verlet = r_verlet
    d.precision = precision
    d.n_facets = n_facets
    d.facet_auto_move = facet_auto_move
    d.max_neighbors = max_neighbors
    d.threads_per_row = threads_per_row
    d.force_kernel = force_kernel
    return d


# --------------------------------------------------------------------------------------------
# Synthetic aggregate workloads (seeded random-sequential-attachment aggregates)
# --------------------------------------------------------------------------------------------
def connector_bonds(x0, r_part, critical_separation):
    """Bonds of the 5-connector sinter model in its detection order (sinter_bridge.h:146-160): every
    pair i < j with |(|x_j - x_i| - 2 r)| <= critical_separation, i ascending, then j ascending.
    Returns an (nb, 2) int64 array."""
    x0 = np.asarray(x0, dtype=np.float64)
    n = len(x0)
    out = []
    for i in range(n - 1):
        d = x0[i + 1:] - x0[i]
        g = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]) - 2.0 * r_part
        for k in np.nonzero(~(np.abs(g) > critical_separation))[0]:
            out.append((i, i + 1 + int(k)))
    return np.array(out, dtype=np.int64).reshape(-1, 2)


def set_connectors(desc, k_d, gamma_d, critical_separation, axes):
    """Configure a descriptor for LG_BINARY_SINTER_CONNECTORS: connector stiffness/damping, bonding
    distance and one unit axis per bond (the vectors the reference draws from its generator). The
    axes array is kept alive on the descriptor."""
    axes = np.ascontiguousarray(np.asarray(axes, dtype=np.float64).reshape(-1, 3))
    desc.binary_model = A.LG_BINARY_SINTER_CONNECTORS
    desc.connector = A.lg_connector_params(k_d, gamma_d, critical_separation)
    desc.connector_axes = axes.ctypes.data_as(C.POINTER(C.c_double))
    desc.n_connector_axes = len(axes)
    desc._axes_keepalive = axes
    return desc


def set_hold(desc, mask):
    """Hold mask from construction on: LG_HOLD_* bits per particle (kept alive on the descriptor)."""
    m = np.ascontiguousarray(np.asarray(mask, dtype=np.uint8).reshape(-1))
    desc.hold_mask = m.ctypes.data_as(C.POINTER(C.c_uint8))
    desc._hold_keepalive = m
    return desc


def central_body(k_a, mass, centre):
    """lg_body_force of the central attraction a = k_a / mass * (centre - x_i)."""
    return A.lg_body_force(A.LG_BODY_CENTRAL, float(k_a), float(mass), (C.c_double * 3)(*[float(c) for c in centre]))


def random_unit_axes(count, seed):
    """Seeded unit vectors (uniform in the cube, normalised), one per bond."""
    rng = np.random.default_rng(seed)
    v = rng.uniform(-1.0, 1.0, size=(count, 3))
    return v / np.linalg.norm(v, axis=1)[:, None]


class Material:
    """Constants of the aggregate workloads: r = 14 nm, rho = 1700 kg/m^3, k_n = 1e4 N/m,
    tangential/rolling/torsion stiffness 0.5 k_n, damping ratio 0.1 on the reduced mass m/2,
    friction coefficient 1, Hamaker constant 1e-19 J with saturation distance 0.4 nm, surface-gap
    cutoff 2r (centre distance 4r), time step 0.01 sqrt(m/k_n)."""

    def __init__(self, r=R_PART, rho=RHO, k_n=1e4, stiff_ratio=0.5, zeta=0.1, mu=1.0, A_h=1e-19, h0=0.4e-9,
                 d_crit=1.0e-9):
        self.r = r
        self.m = mass_of(r, rho)
        self.I = inertia_of(self.m, r)
        self.k_n = k_n
        self.k_s = stiff_ratio * k_n
        damp = lambda k: 2.0 * zeta * math.sqrt(k * self.m / 2.0)
        self.g_n = damp(k_n)
        self.g_s = damp(self.k_s)
        self.mu = mu
        self.A = A_h
        self.h0 = h0
        self.r_cut = 4.0 * r
        self.d_crit = d_crit
        self.dt = 0.01 * math.sqrt(self.m / k_n)

    def contact(self):
        return contact_params(self.k_n, self.g_n, self.k_s, self.g_s, self.mu, 1.0, self.k_s, self.g_s, self.mu,
                              1.0, self.k_s, self.g_s, self.mu, 1.0, self.r, self.m, self.I, self.dt)

    def sinter(self):
        return sinter_params(self.k_n, self.g_n, self.k_s, self.g_s, self.k_s, self.g_s, self.k_s, self.g_s, self.r,
                             self.m, self.I, self.dt, self.d_crit)

    def hamaker(self):
        return hamaker_params(self.A, self.h0, self.r, self.m, r_cutoff=self.r_cut)


def lognormal_sizes(count, median, lo, hi, seed, clip_frac=0.01):
    """Aggregate sizes: log-normal with the given median, sigma chosen so that about clip_frac of the
    draws fall outside [lo, hi] on each side of a symmetric range, clipped to [lo, hi]."""
    import numpy as np
    from math import log
    z = 2.326347874040841  # standard-normal quantile of 0.99
    sigma = log(hi / median) / z
    rng = np.random.default_rng(seed)
    n = np.exp(rng.normal(log(median), sigma, size=count))
    return np.clip(np.rint(n), lo, hi).astype(np.int64)


def loguniform_sizes(count, lo, hi, seed):
    """Aggregate sizes log-uniform in [lo, hi]."""
    import numpy as np
    from math import log
    rng = np.random.default_rng(seed)
    return np.clip(np.rint(np.exp(rng.uniform(log(lo), log(hi), size=count))), lo, hi).astype(np.int64)


def seeded_aggregates(sizes, config_id, r, vmax=0.1):
    """Positions and velocities of a list of aggregates; aggregate a uses seed config_id * 2^32 + a."""
    import numpy as np
    from .system import generate_aggregate, generate_velocities
    xs, vs = [], []
    for a, n in enumerate(sizes):
        seed = (int(config_id) << 32) + a
        xs.append(generate_aggregate(seed, int(n), r))
        vs.append(generate_velocities(seed, int(n), vmax))
    return np.concatenate(xs), np.concatenate(vs)


def wall_facet(mat, extent, v_wall=1.0, k_n=1e4):
    """A rigid plane wall z = 0 moving along +z at v_wall, as one large triangle (side ~ 20 extent)
    carrying a surface contact functor with normal stiffness k_n (the aggregate workload's other
    contact constants) and a surface Hamaker functor."""
    f = A.lg_facet_desc()
    L = 20.0 * extent
    f.v_facet[0], f.v_facet[1], f.v_facet[2] = 0.0, 0.0, v_wall
    verts = [(-L, -L, 0.0), (-L, 3 * L, 0.0), (3 * L, -L, 0.0)]
    for k, v in enumerate(verts):
        for c in range(3):
            f.vertices[3 * k + c] = v[c]
    f.has_contact = 1
    f.has_hamaker = 1
    c = mat.contact()
    c.k = k_n
    f.contact = c
    f.hamaker = mat.hamaker()
    return f


def rest_on_wall(x, sizes, r):
    """Translate every aggregate so that its lowest sphere touches the plane z = 0 from above
    (x, y centred on the aggregate's centroid)."""
    import numpy as np
    out = np.array(x, dtype=np.float64, copy=True)
    off = np.concatenate([[0], np.cumsum(sizes)])
    for a in range(len(sizes)):
        seg = out[off[a]:off[a + 1]]
        c = seg.mean(0)
        seg[:, 0] -= c[0]
        seg[:, 1] -= c[1]
        seg[:, 2] -= seg[:, 2].min() - r
    return out

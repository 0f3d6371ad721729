"""Engine-side state dumps (lg_write_vtk_*, lg_write_csv_positions, lg_get_connectors) of a live
handle: the text equals libgran's writer formats of the handle's own state, and the connector
points equal the oracle's bit for bit."""
import numpy as np
import pytest

from libgran_gb300 import _abi as A
from libgran_gb300 import configs as K
from libgran_gb300.system import System, generate_aggregate, generate_velocities
from oracle import oracle as O

import test_writer_cpu as W

pytestmark = pytest.mark.gpu


def test_particles_necks_csv_of_a_sintered_aggregate(tmp_path):
    mat = K.Material()
    n = 300
    x0 = generate_aggregate(71, n, mat.r)
    v0 = generate_velocities(71, n, 0.5)
    om0 = generate_velocities(72, n, 3.0e8)
    d = K.make_desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(), sinter=mat.sinter(),
                    hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r)
    s = System(d, x0, v0, om0=om0)
    s.step(mat.dt, 200, 20)
    x, th = s.get(A.LG_FIELD_X), s.get(A.LG_FIELD_THETA)
    assert np.abs(th).max() > 0
    s.write_vtk("particles", tmp_path / "p.vtk", mat.r)
    assert (tmp_path / "p.vtk").read_text() == W.particles_text(x, th, mat.r)
    s.write_vtk("csv", tmp_path / "p.csv", mat.r)
    assert (tmp_path / "p.csv").read_text() == W.csv_text(x, mat.r)
    bonds = [(int(i), int(j)) for i, j in s.bonds() if i < j]
    assert bonds
    s.write_vtk("necks", tmp_path / "n.vtk", mat.r)
    assert (tmp_path / "n.vtk").read_text() == W.necks_text(x, bonds, mat.r)


def test_connectors_match_oracle_and_dump(tmp_path):
    mat = K.Material()
    n = 120
    x0 = generate_aggregate(73, n, mat.r)
    v0 = generate_velocities(73, n, 0.5)
    om0 = generate_velocities(74, n, 3.0e8)
    d = K.make_desc(n, A.LG_BINARY_SINTER_CONNECTORS, A.LG_HAMAKER_LIMITED, contact=mat.contact(),
                    hamaker=mat.hamaker())
    K.set_connectors(d, 0.5 * mat.k_n, 0.3 * mat.g_n, mat.d_crit,
                     K.random_unit_axes(len(K.connector_bonds(x0, mat.r, mat.d_crit)), 74))
    s = System(d, x0, v0, om0=om0)
    o = O.OracleSystem(d, x0, v0, om0=om0)
    assert np.array_equal(s.connectors(), o.connectors())
    s.step(mat.dt, 150)
    o.step(mat.dt, 150)
    cg = s.connectors()
    assert len(cg) == 5 * 2 * d.n_connector_axes
    assert np.array_equal(cg, o.connectors())
    s.write_vtk("connectors", tmp_path / "c.vtk", mat.r)
    assert (tmp_path / "c.vtk").read_text() == W.connectors_text(cg, mat.r)

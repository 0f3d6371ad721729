"""State dumps in libgran's writer formats (writer.cpp:13-170) and the tutorials' CSV dump, without
a GPU: the engine library's host formatters against a restatement of libgran's writer in Python
(same headers and separators; numbers as an std::ostream prints doubles by default, "%.6g"; the
orientation fields from Eigen's AngleAxis -> quaternion -> rotation matrix formulas), and the
drop-in writer.h (file naming and counters) through a C++ driver."""
import ctypes as C
import math
import os
import subprocess

import numpy as np
import pytest

from libgran_gb300 import _abi as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEAD = "# vtk DataFile Version 4.0\nGenerated by libFractalCommon\nASCII\nDATASET POLYDATA\n"


def g6(v):
    return "%.6g" % v


def _aa(angle, k):
    ha = 0.5 * angle
    s = math.sin(ha)
    e = [1.0 if k == j else 0.0 for j in range(3)]
    return (math.cos(ha), s * e[0], s * e[1], s * e[2])


def _ham(a, b):
    aw, ax, ay, az = a
    bw, bx, by, bz = b
    return (aw * bw - ax * bx - ay * by - az * bz, aw * bx + ax * bw + ay * bz - az * by,
            aw * by + ay * bw + az * bx - ax * bz, aw * bz + az * bw + ax * by - ay * bx)


def _columns(t):
    w, x, y, z = _ham(_ham(_aa(t[0], 0), _aa(t[1], 1)), _aa(t[2], 2))
    tx, ty, tz = 2.0 * x, 2.0 * y, 2.0 * z
    twx, twy, twz = tx * w, ty * w, tz * w
    txx, txy, txz = tx * x, ty * x, tz * x
    tyy, tyz, tzz = ty * y, tz * y, tz * z
    m = [[1.0 - (tyy + tzz), txy - twz, txz + twy], [txy + twz, 1.0 - (txx + tzz), tyz - twx],
         [txz - twy, tyz + twx, 1.0 - (txx + tyy)]]
    cols = []
    for k in range(3):
        u = [1.0 if k == j else 0.0 for j in range(3)]
        cols.append([(m[i][0] * u[0] + m[i][1] * u[1]) + m[i][2] * u[2] for i in range(3)])
    return cols


def particles_text(x, th, r):
    n = len(x)
    t = HEAD + "POINTS %d FLOAT\n" % n
    t += "".join(g6(p[c] / r) + " " for p in x for c in range(3))
    t += "\n\nPOINT_DATA %d\nFIELD FieldData 3\n" % n
    cols = [_columns(q) for q in th]
    for k, name in enumerate(("thetax", "thetay", "thetaz")):
        t += ("\n" if k else "") + "%s 3 %d double\n" % (name, n)
        t += "".join(g6(cols[i][k][c]) + " " for i in range(n) for c in range(3))
    return t + "\n"


def necks_text(x, pairs, r):
    t = HEAD + "POINTS %d FLOAT\n" % len(pairs)
    t += "".join(g6((x[i][c] + x[j][c]) / 2.0 / r) + " " for i, j in pairs for c in range(3))
    t += "\n\nPOINT_DATA %d\nFIELD FieldData 1\nnormals 3 %d double\n" % (len(pairs), len(pairs))
    for i, j in pairs:
        d = [x[i][c] - x[j][c] for c in range(3)]
        z = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]
        if z > 0.0:
            s = math.sqrt(z)
            d = [c / s for c in d]
        t += "".join(g6(c) + " " for c in d)
    return t


def connectors_text(pts, r):
    return HEAD + "POINTS %d FLOAT\n" % len(pts) + "".join(g6(p[c] / r) + " " for p in pts for c in range(3)) + "\n"


def csv_text(x, r):
    return "x, y, z\n" + "".join("%s, %s, %s\n" % tuple(g6(p[c] / r) for c in range(3)) for p in x)


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _state(n, seed):
    rng = np.random.default_rng(seed)
    r = 1.4e-8
    x = rng.normal(scale=20 * r, size=(n, 3))
    th = rng.uniform(-12.0, 12.0, size=(n, 3))
    th[0] = 0.0
    th[1] = [-0.0, math.pi, -math.pi / 2]
    x[2] = [0.0, -0.0, 1e-30]
    return r, np.ascontiguousarray(x), np.ascontiguousarray(th)


@pytest.mark.parametrize("n", [1, 7, 5000])  # 5000: parallel chunks
def test_particles_vtk_matches_writer_restatement(tmp_path, n):
    r, x, th = _state(max(n, 3), n)
    x, th = x[:n], th[:n]
    p = str(tmp_path / "p.vtk")
    A.check(A.lib().lg_format_vtk_particles(_dp(x), _dp(th), n, r, p.encode()), "format")
    assert open(p).read() == particles_text(x, th, r)


def test_necks_connectors_csv_match_writer_restatement(tmp_path):
    r, x, th = _state(4000, 3)
    pairs = np.array([(i, j) for i in range(0, 3990, 3) for j in (i + 1, i + 5)], dtype=np.int64)
    p = str(tmp_path / "n.vtk")
    A.check(A.lib().lg_format_vtk_necks(_dp(x), len(x), pairs.ctypes.data_as(C.POINTER(C.c_int64)), len(pairs), r,
                                         p.encode()), "format")
    assert open(p).read() == necks_text(x, pairs, r)
    pts = np.ascontiguousarray(x[:2500])
    A.check(A.lib().lg_format_vtk_connectors(_dp(pts), len(pts), r, p.encode()), "format")
    assert open(p).read() == connectors_text(pts, r)
    A.check(A.lib().lg_format_csv_positions(_dp(x), len(x), r, p.encode()), "format")
    assert open(p).read() == csv_text(x, r)


def test_format_errors_are_reported(tmp_path):
    x = np.zeros((2, 3))
    bad = np.array([0, 5], dtype=np.int64)
    with pytest.raises(RuntimeError, match="out of range"):
        A.check(A.lib().lg_format_vtk_necks(_dp(x), 2, bad.ctypes.data_as(C.POINTER(C.c_int64)), 1, 1.0,
                                             str(tmp_path / "n.vtk").encode()), "format")
    with pytest.raises(RuntimeError, match="unable to create"):
        A.check(A.lib().lg_format_csv_positions(_dp(x), 2, 1.0, str(tmp_path / "no" / "such.csv").encode()),
                "format")


def test_dropin_writer_header_names_and_counts_files(tmp_path):
    exe = str(tmp_path / "dropin_writer")
    lib = os.path.join(ROOT, "libgran_gb300", "_lib")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include", "libgran_gb300"),
                           "-I/usr/local/cuda/include", "-o", exe, os.path.join(ROOT, "tests", "cpp", "dropin_writer.cpp"),
                           "-L" + lib, "-llg_gb300", "-Wl,-rpath," + lib])
    r, x, th = _state(40, 9)
    sin = str(tmp_path / "in.bin")
    with open(sin, "wb") as f:
        f.write(np.int64(len(x)).tobytes() + x.tobytes() + th.tobytes())
    out = tmp_path / "run"
    out.mkdir()
    subprocess.check_call([exe, sin, str(out), repr(r)])
    pairs = [(i, i + 1) for i in range(len(x) - 1)]
    conn = []
    for i in range(len(x)):  # the driver's connectors, in (i, j) order
        for j in sorted({i - 1, i + 1} & set(range(len(x)))):
            for q in range(5):
                conn.append([x[i][0] + q * r / 10, x[i][1], x[i][2]] if j == i + 1 else
                            [x[i][0], x[i][1] + q * r / 10, x[i][2]])
    for k in (1, 2):
        assert (out / ("particles_%d.vtk" % k)).read_text() == particles_text(x, th, r)
        assert (out / ("necks_%d.vtk" % k)).read_text() == necks_text(x, pairs, r)
        assert (out / ("spring_connectors_%d.vtk" % k)).read_text() == connectors_text(np.array(conn), r)
    assert not (out / "particles_3.vtk").exists()

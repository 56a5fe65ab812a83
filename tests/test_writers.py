"""Result files in the reference's formats: Tecplot ASCII (fileIO_velocity, C/fileIO.h:69-87),
Tecplot binary #!TDV101 (Output3Dvelocity, C/fileIO.h:502-659) and Monitor.dat (Launch_Monitor,
C/monitor.h:4-26), parsed back and compared with the solver's fields and mesh."""
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def solver(islbm):
    p = islbm.default_params(NX=8, NY=16, NZ=12, Re=60.0, Uref=0.05, precision="fp64", init_mode=1, seed=9)
    s = islbm.Solver(p)
    s.step(6)
    return p, s


def padded_nodes(islbm, p, s):
    """(x, y, z, u, v, w) on the nodes i, j, k = 3 .. N6-4 of the padded layout, k slowest."""
    f = s.fields(layout=islbm.LAYOUT_REFERENCE)
    x = islbm.host_table(p, "x")
    y = islbm.host_table(p, "y")
    z = islbm.host_table(p, "z").reshape(p.NY + 7, p.NZ + 6)
    rows = []
    for k in range(3, p.NZ + 3):
        for j in range(3, p.NY + 4):
            for i in range(3, p.NX + 4):
                rows.append((x[i], y[j], z[j, k], f["u"][j, k, i], f["v"][j, k, i], f["w"][j, k, i]))
    return np.array(rows)


def test_tecplot_ascii(islbm_lib, tmp_path):
    islbm = islbm_lib
    p, s = solver(islbm)
    with s:
        path = tmp_path / "velocity.dat"
        s.write_tecplot_ascii(str(path))
        ref = padded_nodes(islbm, p, s)
    lines = path.read_text().splitlines()
    assert lines[0] == 'VARIABLES = "X", "Y", "Z", "U", "V", "W"'
    assert lines[1] == 'ZONE T = "velocity", F = POINT'
    assert lines[2] == "I = %d, J = %d, K = %d" % (p.NX + 1, p.NY + 1, p.NZ)
    data = np.array([[float(t) for t in ln.split()] for ln in lines[3:]])
    assert data.shape == ref.shape
    np.testing.assert_allclose(data[:, :3], ref[:, :3], atol=5e-5)
    np.testing.assert_allclose(data[:, 3:], ref[:, 3:], atol=5e-16)


def read_str(b, o):
    out = []
    while True:
        c = struct.unpack_from("<i", b, o)[0]
        o += 4
        if c == 0:
            return "".join(out), o
        out.append(chr(c))


def test_tecplot_binary(islbm_lib, tmp_path):
    islbm = islbm_lib
    p, s = solver(islbm)
    with s:
        path = tmp_path / "test_0.plt"
        s.write_tecplot_plt(str(path))
        ref = padded_nodes(islbm, p, s)
        uref = s.constants()["Uref"]
    b = path.read_bytes()
    assert b[:8] == b"#!TDV101"
    o = 8
    assert struct.unpack_from("<i", b, o)[0] == 1
    o += 4
    title, o = read_str(b, o)
    assert title == "Particle intensity"
    nvar = struct.unpack_from("<i", b, o)[0]
    o += 4
    names = []
    for _ in range(nvar):
        n, o = read_str(b, o)
        names.append(n)
    assert names == ["X", "Y", "Z", "U", "V", "W"]
    assert struct.unpack_from("<f", b, o)[0] == 299.0
    o += 4
    zone, o = read_str(b, o)
    assert zone == "Zone 001"
    hdr = struct.unpack_from("<9i", b, o)
    o += 36
    assert hdr == (-1, 0, 1, 0, 0, p.NX + 1, p.NY + 1, p.NZ, 0)
    assert struct.unpack_from("<f", b, o)[0] == 357.0 and struct.unpack_from("<f", b, o + 4)[0] == 299.0
    o += 8
    assert struct.unpack_from("<8i", b, o) == (2, 2, 2, 2, 2, 2, 0, -1)
    o += 32
    data = np.frombuffer(b[o:], dtype="<f8").reshape(-1, 6)
    np.testing.assert_array_equal(data[:, :3], ref[:, :3])
    np.testing.assert_allclose(data[:, 3:], ref[:, 3:] / uref, rtol=1e-15, atol=1e-18)


def test_monitor(islbm_lib, tmp_path):
    islbm = islbm_lib
    p, s = solver(islbm)
    with s:
        path = tmp_path / "Monitor.dat"
        s.write_monitor(str(path), 6)
        s.step(2)
        s.write_monitor(str(path), 8)
        f = s.fields(layout=islbm.LAYOUT_REFERENCE)
        force = s.force
    lines = path.read_text().splitlines()
    assert len(lines) == 2
    vals = [float(t) for t in lines[1].split()]
    i, j, k = (p.NX + 7) // 2, (p.NY + 7) // 2, (p.NZ + 6) // 2
    assert int(vals[0]) == 8
    np.testing.assert_allclose(vals[1:], [f["v"][j, k, i], f["u"][j, k, i], f["w"][j, k, i], force], atol=5e-16)

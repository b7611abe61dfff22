"""CPU: physical properties of the oracle restatement, independent of the
fixtures.  Forces are minus the gradient of the total energy (central finite
differences), torques minus its derivative in the body angle, and Newton's
third law holds (the reference's own check, src/particles/base/particle.cu:96)."""
import numpy as np

from oracle.oracle import BumpyOracle, DiskOracle, bumpy_packing, disk_packing

ALL = 2  # all-pairs lists: positions can move freely without a rebuild


def disk_energy(st, x, y):
    o = DiskOracle(len(x), st["box"])
    o.set_arrays(x=x, y=y, r=st["r"], m=st["m"])
    o.setup_neighbors(ALL, 1.5, 0.2, 8.0, 0.5)
    return o.total_pe(), o.get_arrays()


def test_disk_forces_are_minus_the_energy_gradient():
    st = disk_packing(48, 0.9, 5)
    x, y = st["x"].copy(), st["y"].copy()
    u0, a = disk_energy(st, x, y)
    assert u0 > 0
    np.testing.assert_allclose(a["fx"].sum(), 0.0, atol=1e-12)
    np.testing.assert_allclose(a["fy"].sum(), 0.0, atol=1e-12)
    h = 1e-6
    for i in range(0, 48, 5):
        for arr, f in ((x, a["fx"]), (y, a["fy"])):
            keep = arr[i]
            arr[i] = keep + h
            up, _ = disk_energy(st, x, y)
            arr[i] = keep - h
            um, _ = disk_energy(st, x, y)
            arr[i] = keep
            np.testing.assert_allclose(-(up - um) / (2 * h), f[i], rtol=0, atol=1e-7)


def bumpy_energy(st, px, py, rotation=True):
    b = BumpyOracle(len(st["r"]), st["nv"], st["box"], st["e_c"], 2.0, st["rv"], st["seg"], rotation)
    b.set_bodies(st["x"], st["y"], st["th"], st["r"], st["nvb"])
    b.set_vertices(px, py)
    b.set_mass(1.0)
    b.setup_neighbors(ALL, 1.5, 0.2, 8.0, 0.5)
    return b.total_pe(), b.bodies()


def test_rigid_forces_and_torques_are_minus_the_energy_gradient():
    st = bumpy_packing(24, 0.85, 8)
    b = BumpyOracle(24, st["nv"], st["box"], st["e_c"], 2.0, st["rv"], st["seg"], True)
    b.set_bodies(st["x"], st["y"], st["th"], st["r"], st["nvb"])
    b.init_vertices()
    px, py = b.vertices()
    u0, bd = bumpy_energy(st, px, py)
    assert u0 > 0
    np.testing.assert_allclose(bd["fx"].sum(), 0.0, atol=1e-12)
    np.testing.assert_allclose(bd["fy"].sum(), 0.0, atol=1e-12)
    start = np.concatenate([[0], np.cumsum(st["nvb"])])
    h = 1e-6
    checked = 0
    for k in range(24):
        if bd["fx"][k] == 0.0 and bd["tq"][k] == 0.0:
            continue
        sl = slice(start[k], start[k + 1])
        # translation of body k along x
        qx = px.copy()
        qx[sl] += h
        up, _ = bumpy_energy(st, qx, py)
        qx[sl] -= 2 * h
        um, _ = bumpy_energy(st, qx, py)
        np.testing.assert_allclose(-(up - um) / (2 * h), bd["fx"][k], rtol=0, atol=1e-7)
        # rotation of body k about its centre
        cx, cy = st["x"][k], st["y"][k]
        e = []
        for dth in (h, -h):
            c, s = np.cos(dth), np.sin(dth)
            rx, ry = px[sl] - cx, py[sl] - cy
            qx, qy = px.copy(), py.copy()
            qx[sl], qy[sl] = cx + rx * c - ry * s, cy + rx * s + ry * c
            e.append(bumpy_energy(st, qx, qy)[0])
        np.testing.assert_allclose(-(e[0] - e[1]) / (2 * h), bd["tq"][k], rtol=0, atol=1e-7)
        checked += 1
        if checked == 6:
            break
    assert checked >= 3

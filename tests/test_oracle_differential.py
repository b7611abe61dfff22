"""CPU: the oracle against the reference's own kernels run live (oracle/_ref,
built from the reference sources where they are present; skipped elsewhere),
over a sweep the fixtures do not cover: sizes, densities, the three neighbour
methods, rigid bodies with and without rotation, and every operation the
drop-in offers.  Everything must agree bit for bit."""
import numpy as np
import pytest

from oracle.oracle import (BumpyOracle, DiskOracle, bumpy_packing, disk_packing, fill_normal,
                           reference_available)

pytestmark = pytest.mark.skipif(not reference_available(),
                                reason="reference kernels not built here (oracle/_ref)")

DISK_KEYS = ("x", "y", "vx", "vy", "fx", "fy", "pe")
BODY_KEYS = ("x", "y", "th", "vx", "vy", "w", "fx", "fy", "tq", "pe")


def disk_pair(n, phi, seed, method, vel=True):
    st = disk_packing(n, phi, seed, kind="reference")
    vx = vy = None
    if vel:
        vx = fill_normal(n, 0.0, 1e-2, 1, seed)
        vy = fill_normal(n, 0.0, 1e-2, 1 + n, seed)
    out = []
    for kind in ("oracle", "reference"):
        o = DiskOracle(n, st["box"], kind=kind)
        o.set_arrays(x=st["x"], y=st["y"], vx=vx, vy=vy, r=st["r"], m=st["m"])
        out.append((o, o.setup_neighbors(method, 1.7 / 1.4, 0.2, 8.0, 0.5)))
    assert out[0][1] == out[1][1]
    return out[0][0], out[1][0]


def same_disks(a, b, tag):
    x, y = a.get_arrays(), b.get_arrays()
    for k in DISK_KEYS:
        np.testing.assert_array_equal(x[k], y[k], err_msg=f"{tag} {k}")
    assert a.neighbor_info() == b.neighbor_info(), tag


@pytest.mark.parametrize("n,phi,seed", [(16, 0.5, 1), (100, 0.85, 2), (333, 0.95, 3), (700, 0.7, 4)])
@pytest.mark.parametrize("method", [0, 1, 2])
def test_disk_operations_bit_for_bit(n, phi, seed, method):
    a, b = disk_pair(n, phi, seed, method)
    same_disks(a, b, "setup")
    for o in (a, b):
        o.nve_steps(1e-2, 40)
    same_disks(a, b, "nve")
    for o in (a, b):
        o.fire_init(0.1, 1e-2)
        for _ in range(30):
            o.fire_step()
    same_disks(a, b, "fire")
    for o in (a, b):
        o.init_adam()
        for t in range(15):
            o.zero_force_and_pe()
            o.check_for_neighbor_update()
            o.calculate_forces()
            o.adam_step(t, 1e-3)
    same_disks(a, b, "adam")
    for o in (a, b):
        o.damped_nve_steps(1e-2, 0.3, 20)
    same_disks(a, b, "damped")
    assert a.pressure() == b.pressure() and a.contact_count() == b.contact_count()
    pa, pb = a.pair_dump(), b.pair_dump()
    for k in pa:
        np.testing.assert_array_equal(pa[k], pb[k], err_msg=f"pairs {k}")


def bumpy_pair(nb, phi, seed, rotation, method):
    st = bumpy_packing(nb, phi, seed, kind="reference")
    vx = fill_normal(nb, 0.0, 1e-2, 1, seed)
    vy = fill_normal(nb, 0.0, 1e-2, 1 + nb, seed)
    w = fill_normal(nb, 0.0, 1e-2, 1 + 2 * nb, seed)
    out = []
    for kind in ("oracle", "reference"):
        b = BumpyOracle(nb, st["nv"], st["box"], st["e_c"], 2.0, st["rv"], st["seg"], rotation,
                        kind=kind)
        b.set_bodies(st["x"], st["y"], st["th"], st["r"], st["nvb"], vx, vy, w)
        b.init_vertices()
        b.set_mass(1.0)
        out.append((b, b.setup_neighbors(method, 1.5, 0.2, 8.0, 0.3)))
    assert out[0][1] == out[1][1]
    return out[0][0], out[1][0]


def same_bodies(a, b, tag):
    x, y = a.bodies(), b.bodies()
    for k in BODY_KEYS:
        np.testing.assert_array_equal(x[k], y[k], err_msg=f"{tag} {k}")
    for u, v in zip(a.vertices(), b.vertices()):
        np.testing.assert_array_equal(u, v, err_msg=f"{tag} vertices")
    assert a.neighbor_info() == b.neighbor_info(), tag


@pytest.mark.parametrize("nb,phi,seed", [(8, 0.6, 11), (40, 0.85, 12), (150, 0.75, 13)])
@pytest.mark.parametrize("rotation", [True, False])
@pytest.mark.parametrize("method", [0, 1])
def test_rigid_operations_bit_for_bit(nb, phi, seed, rotation, method):
    a, b = bumpy_pair(nb, phi, seed, rotation, method)
    same_bodies(a, b, "setup")
    ta, pa = a.stress()
    tb, pb = b.stress()
    np.testing.assert_array_equal(pa, pb)
    ca, cb = a.count_contacts(), b.count_contacts()
    assert ca[0] == cb[0] and np.array_equal(ca[1], cb[1]) and np.array_equal(ca[2], cb[2])
    for k, v in a.pair_dump().items():
        np.testing.assert_array_equal(v, b.pair_dump()[k], err_msg=f"pairs {k}")
    for o in (a, b):
        o.nve_steps(5e-3, 30)
    same_bodies(a, b, "nve")
    for o in (a, b):
        o.fire_init(0.1, 1e-2)
        for _ in range(25):
            o.fire_step()
    same_bodies(a, b, "fire")
    for o in (a, b):
        o.damped_nve_steps(5e-3, 0.4, 20)
    same_bodies(a, b, "damped")
    for o in (a, b):
        o.nve_wall_steps(5e-3, 20)
    same_bodies(a, b, "walls")
    for o in (a, b):
        o.adam_steps(20, 2e-3)
    same_bodies(a, b, "adam")
    for o in (a, b):
        o.save_state()
        o.fire_init(0.1, 1e-2)
        for _ in range(15):
            o.fire_step()
        o.restore_state()
    same_bodies(a, b, "revert")

"""GPU: dpg_disk_forces_noalloc, the one entry point that allocates no device
memory, against the allocating path (dpg_setup_neighbors + dpg_compute_forces)
and against the CPU oracle of the reference's force kernel.

It exists for callers that cannot call cudaMalloc: hosts that hand all device
memory to their own fixed pool up front, and real-time loops that cannot wait
on the allocator.  Its cell-list scratch is a fixed array inside the library
that every call shares, so the test makes several calls in a row with
different sizes: a call that found the previous call's counters still in place
would give wrong forces.

Summation order over a particle's contacts differs between the paths (cell
stencil order here, neighbour-list order in the library and the oracle), so
forces and energies agree to 1e-12 of the largest value rather than bit for
bit.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12
MAX_PARTICLES = 65536


def packing(n, phi, seed):
    """Bidisperse disks (radii 0.5 and 0.7) at random positions, box set by phi."""
    rng = np.random.default_rng(seed)
    r = np.where(np.arange(n) % 2 == 0, 0.5, 0.7).astype(np.float64)
    box = float(np.sqrt(np.pi * np.sum(r * r) / phi))
    x = rng.uniform(0.0, box, n)
    y = rng.uniform(0.0, box, n)
    return x, y, r, box


def allocating_path(dpg, x, y, r, box):
    s = dpg.Disk(len(x), box)
    try:
        s.setState(x, y, None, None, r, np.ones_like(r))
        s.setupNeighbors("cell", 1.5, 0.2, 8.0, 0.5)
        s.zeroForceAndPotentialEnergy()
        s.calculateForces()
        st = s.getState()
    finally:
        s.close()
    return st["fx"], st["fy"], st["pe"]


def oracle_path(x, y, r, box):
    from oracle.oracle import DiskOracle
    o = DiskOracle(len(x), box)
    o.set_arrays(x=x, y=y, r=r, m=np.ones_like(r))
    o.setup_neighbors(0, 1.5, 0.2, 8.0, 0.5)
    o.zero_force_and_pe()
    o.calculate_forces()
    a = o.get_arrays()
    o.close()
    return a["fx"], a["fy"], a["pe"]


def noalloc_path(lib, torch, x, y, r, box):
    dev = torch.device("cuda:0")
    tx, ty, tr = (torch.as_tensor(a, dtype=torch.float64, device=dev) for a in (x, y, r))
    out = [torch.full_like(tx, float("nan")) for _ in range(3)]
    stream = torch.cuda.current_stream(dev)
    rc = lib.dpg_disk_forces_noalloc(
        C.c_void_p(tx.data_ptr()), C.c_void_p(ty.data_ptr()), C.c_void_p(tr.data_ptr()),
        len(x), box, box, 1.0, 2.0, float(2.0 * r.max()),
        *[C.c_void_p(o.data_ptr()) for o in out], C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.dpg_last_error()
    torch.cuda.synchronize(dev)
    return [o.cpu().numpy() for o in out]


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import dpcuda_gb300
    return dpcuda_gb300, dpcuda_gb300.load_library(), torch


def test_noalloc_matches_allocating_path_on_calls_in_a_row(env):
    dpg, lib, torch = env
    # large, tiny (all-pairs: fewer than 3 cells a side), large again
    for n, phi, seed in [(4096, 0.86, 11), (16, 0.8, 12), (4096, 0.86, 11), (20000, 0.9, 13)]:
        x, y, r, box = packing(n, phi, seed)
        want = allocating_path(dpg, x, y, r, box)
        oracle = oracle_path(x, y, r, box)
        got = noalloc_path(lib, torch, x, y, r, box)
        for ref_name, ref in (("allocating path", want), ("oracle", oracle)):
            for name, g, w in zip(("fx", "fy", "pe"), got, ref):
                assert np.all(np.isfinite(g)), name
                scale = max(np.abs(w).max(), 1e-300)
                np.testing.assert_allclose(g, w, rtol=0, atol=TOL * scale,
                                           err_msg=f"{name} n={n} against the {ref_name}")
        assert np.abs(want[0]).max() > 0  # the packing has contacts


def test_noalloc_rejects_sizes_beyond_its_scratch(env):
    _, lib, torch = env
    t = torch.zeros(4, dtype=torch.float64, device="cuda:0")
    buf = C.c_void_p(t.data_ptr())
    rc = lib.dpg_disk_forces_noalloc(buf, buf, buf, MAX_PARTICLES + 1, 10.0, 10.0, 1.0, 2.0,
                                     1.0, buf, buf, buf, None)
    assert rc != 0
    assert b"65536" in lib.dpg_last_error()
    rc = lib.dpg_disk_forces_noalloc(buf, buf, buf, 100, 1000.0, 1000.0, 1.0, 2.0,
                                     1.0, buf, buf, buf, None)
    assert rc != 0
    assert b"cells" in lib.dpg_last_error()

"""mpm_volume_setup_noalloc against the allocating path, through the C ABI.

Callers that cannot call cudaMalloc (a JAX/XLA FFI handler given its buffers by
XLA, or an application whose framework owns the device memory pool) use
mpm_volume_setup_noalloc, which keeps its per-element counters in a fixed
device array instead of allocating.  Its element ids, volumes and masses must
equal what a handle computes (mpm_initialize, then mpm_read_field of
ELEMENT_ID / VOLUME / MASS) for the same particles, on two calls in a row (the
second call reuses the array the first one left behind).  The test buffers are
allocated here, by the test; the entry point itself allocates nothing.

This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

import diffmpm_gb300 as D
from diffmpm_gb300 import _lib, workloads

pytestmark = pytest.mark.gpu


def _reference_setup(n_mesh):
    """Element ids, volumes and masses from the allocating path, for the
    scale-up particles plus two on mesh lines that are still inside the mesh
    (one on the left boundary x = 0, one on an interior node corner)."""
    solver, g, info = workloads.plain_scaleup(D, n=n_mesh, sim_steps=1)
    ps = solver.mesh.particles[0]
    loc = np.concatenate([ps.loc.reshape(-1, 2).astype(np.float32),
                          np.array([[0.0, 0.25], [0.5, 0.5]], np.float32)])
    density = np.concatenate([ps.density.reshape(-1).astype(np.float32),
                              np.array([1900.0, 2100.0], np.float32)])
    sim = D.Simulation((n_mesh, n_mesh), (1.0 / n_mesh, 1.0 / n_mesh), 1e-6,
                       materials=list(ps.materials))
    sim.set_particles(loc, np.zeros(len(loc), np.int32))
    sim.write("density", density)
    sim.initialize()
    out = (loc, density, sim.read("element_ids"), sim.read("volume"), sim.read("mass"))
    sim.close()
    return out


def _call_noalloc(torch, n_mesh, loc, density):
    lib = _lib.load()
    dev = torch.device("cuda:0")
    t_loc = torch.from_numpy(loc).to(dev).contiguous()
    t_rho = torch.from_numpy(density).to(dev).contiguous()
    n = loc.shape[0]
    eid = torch.full((n,), -7, dtype=torch.int32, device=dev)
    vol = torch.full((n,), -1.0, dtype=torch.float32, device=dev)
    mass = torch.full((n,), -1.0, dtype=torch.float32, device=dev)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    h = 1.0 / n_mesh
    rc = lib.mpm_volume_setup_noalloc(n_mesh, n_mesh, h, h, n, C.c_void_p(t_loc.data_ptr()),
                                      C.c_void_p(t_rho.data_ptr()), C.c_void_p(eid.data_ptr()),
                                      C.c_void_p(vol.data_ptr()), C.c_void_p(mass.data_ptr()),
                                      stream)
    assert rc == 0, lib.mpm_last_error(None)
    torch.cuda.synchronize()
    return eid.cpu().numpy(), vol.cpu().numpy(), mass.cpu().numpy()


def test_noalloc_matches_allocating_path_twice(built):
    """Bit for bit the allocating path's values (both run the same float32
    formula), on two calls in a row.  Two more particles lie outside the mesh
    -- one beyond it, one exactly on its right edge x = nx * hx, which the
    reference's locate rule puts in the element past the last column -- and
    take element id -1 with zero volume and mass, where mpm_initialize would
    refuse the population with MPM_ERR_OUT_OF_MESH; they do not change the
    counts of the elements inside."""
    torch = pytest.importorskip("torch")
    n_mesh = 64
    loc, density, eid_ref, vol_ref, mass_ref = _reference_setup(n_mesh)
    outside = np.array([[1.5, 0.5], [1.0, 0.25]], np.float32)
    loc_all = np.concatenate([loc, outside])
    rho_all = np.concatenate([density, np.array([1000.0, 1000.0], np.float32)])
    for _ in range(2):
        eid, vol, mass = _call_noalloc(torch, n_mesh, loc_all, rho_all)
        n = len(loc)
        np.testing.assert_array_equal(eid[:n], eid_ref)
        np.testing.assert_array_equal(vol[:n], vol_ref)
        np.testing.assert_array_equal(mass[:n], mass_ref)
        np.testing.assert_array_equal(eid[n:], [-1, -1])
        np.testing.assert_array_equal(vol[n:], [0.0, 0.0])
        np.testing.assert_array_equal(mass[n:], [0.0, 0.0])
    # the two particles on mesh lines inside the mesh: x = 0 is column 0,
    # the node corner (0.5, 0.5) belongs to the element above and right of it
    assert eid_ref[-2] == (n_mesh // 4) * n_mesh + 0
    assert eid_ref[-1] == (n_mesh // 2) * n_mesh + n_mesh // 2


def test_noalloc_rejects_mesh_beyond_limit(built):
    lib = _lib.load()
    limit = 1 << 20
    rc = lib.mpm_volume_setup_noalloc(limit + 1, 1, 1.0, 1.0, 1, None, None, None, None, None, None)
    assert rc == 1
    assert b"no-allocation limit" in lib.mpm_last_error(None)

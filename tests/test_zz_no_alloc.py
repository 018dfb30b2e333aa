"""ipic3d_gpu_project_noalloc: the projection for callers that cannot
allocate device memory (their host owns all device memory through its own
pool, or a per-step loop must not synchronise on a cudaMalloc). The test
owns every buffer, calls the entry point through the C ABI twice in a row
with different particles, and checks each result against the allocating
entry point (ipic3d_gpu_project) at the projection tolerance of the other
parity tests (1e-12 relative). This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import allscale_ipic3d_gb300 as g
from allscale_ipic3d_gb300 import abi
from common import gpu_sim, scenario

pytestmark = pytest.mark.gpu


def reference_projection(props, parts, counts):
    sim = gpu_sim(props, abi.Config.make(projector=abi.PROJECT_CIC, flags=abi.F_J_DIV8))
    sim.upload_particles(parts, counts)
    sim.project()
    _, _, J, rho = sim.download_fields()
    sim.close()
    return J, rho


def test_project_noalloc_matches_project_on_two_calls_in_a_row():
    import torch
    torch.cuda.init()
    lib = g.library()
    for seed, size in ((101, (5, 4, 6)), (102, (8, 8, 8))):
        props, parts, counts = scenario(seed, size, width=(0.5, 1.0, 2.0), origin=(-1.0, 0.5, 2.0), ppc=9,
                                        vscale=0.4, species=((1.0, 1.0), (-0.5, -2.0)), ragged=True)
        J_ref, rho_ref = reference_projection(props, parts, counts)
        # caller-owned device buffers
        d_p = torch.from_numpy(parts.view(np.uint8).copy()).cuda()
        off = np.concatenate([[0], np.cumsum(counts.astype(np.int64))]).astype(np.int64)
        d_off = torch.from_numpy(off).cuda()
        d_J = torch.full(J_ref.shape, float("nan"), dtype=torch.float64, device="cuda")
        d_rho = torch.full(rho_ref.shape, float("nan"), dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        rc = lib.ipic3d_gpu_project_noalloc(C.byref(props), abi.F_J_DIV8, C.c_void_p(d_p.data_ptr()),
                                            C.c_void_p(d_off.data_ptr()), C.c_void_p(d_J.data_ptr()),
                                            C.c_void_p(d_rho.data_ptr()), C.c_void_p(stream))
        torch.cuda.synchronize()
        assert rc == 0
        J, rho = d_J.cpu().numpy(), d_rho.cpu().numpy()
        np.testing.assert_allclose(J, J_ref, rtol=1e-12, atol=1e-14 * np.abs(J_ref).max())
        np.testing.assert_allclose(rho, rho_ref, rtol=1e-12, atol=1e-14 * np.abs(rho_ref).max())


def test_project_noalloc_rejects_grids_beyond_its_scratch():
    import torch
    torch.cuda.init()
    props = abi.Props.make(size=(33, 32, 32))
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    lib = g.library()
    rc = lib.ipic3d_gpu_project_noalloc(C.byref(props), 0, None, C.c_void_p(d.data_ptr()),
                                        C.c_void_p(d.data_ptr()), None, None)
    assert rc == abi.E_CAPACITY
    buf = C.create_string_buffer(256)
    lib.ipic3d_gpu_last_error(buf, 256)
    assert b"too large" in buf.value

"""ipic3d_gpu_project_noalloc: the projection for callers that cannot
allocate device memory (their host owns all device memory through its own
pool, or a per-step loop must not synchronise on a cudaMalloc). The tests own
every buffer and call the entry point through the C ABI:

  * twice in a row with different particles, against the allocating entry
    point (ipic3d_gpu_project), for both normalisations and with and without
    rho, at the projection tolerance of the other parity tests (1e-12);
  * against the golden projections of the compiled reference
    (tests/golden/project_small.npz, projectToDensityField's own output);
  * with no particles after a call that left sums in the shared scratch: the
    result must be all zeros (the scratch is cleared before each call);
  * with a grid beyond its fixed scratch (refused before any work).

The file name sorts last so that pytest collects it after every other test
file: a run that stops at the first failure (-x) has then already run the
rest of the suite. It does not depend on that order and passes on its own in
a fresh process."""
import ctypes as C

import numpy as np
import pytest

import allscale_ipic3d_gb300 as g
from allscale_ipic3d_gb300 import abi
from common import golden_npz, gpu_sim, props_from_vec, scenario

pytestmark = pytest.mark.gpu


def allocating_projection(props, parts, counts, flags):
    sim = gpu_sim(props, abi.Config.make(projector=abi.PROJECT_CIC, flags=flags))
    sim.upload_particles(parts, counts)
    sim.project()
    _, _, J, rho = sim.download_fields()
    sim.close()
    return J, rho


class Buffers:
    """Caller-owned device buffers for one universe (torch allocates them,
    not the entry point)."""

    def __init__(self, props, parts, counts, with_rho):
        import torch
        n = tuple(int(s) + 1 for s in props.size)
        self.d_p = torch.from_numpy(parts.view(np.uint8).copy()).cuda()
        off = np.concatenate([[0], np.cumsum(counts.astype(np.int64))]).astype(np.int64)
        self.d_off = torch.from_numpy(off).cuda()
        self.d_J = torch.full(n + (3,), float("nan"), dtype=torch.float64, device="cuda")
        self.d_rho = torch.full(n, float("nan"), dtype=torch.float64, device="cuda") if with_rho else None

    def call(self, props, flags, particles=True):
        import torch
        lib = g.library()
        stream = torch.cuda.current_stream().cuda_stream
        rc = lib.ipic3d_gpu_project_noalloc(C.byref(props), flags,
                                            C.c_void_p(self.d_p.data_ptr()) if particles else None,
                                            C.c_void_p(self.d_off.data_ptr()), C.c_void_p(self.d_J.data_ptr()),
                                            C.c_void_p(self.d_rho.data_ptr()) if self.d_rho is not None else None,
                                            C.c_void_p(stream))
        torch.cuda.synchronize()
        assert rc == 0, rc
        return self.d_J.cpu().numpy(), (self.d_rho.cpu().numpy() if self.d_rho is not None else None)


def close(a, b):
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-14 * max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("flags", [0, abi.F_J_DIV8])
@pytest.mark.parametrize("with_rho", [True, False])
def test_project_noalloc_matches_project_on_two_calls_in_a_row(flags, with_rho):
    import torch
    torch.cuda.init()
    for seed, size in ((101, (5, 4, 6)), (102, (8, 8, 8))):
        props, parts, counts = scenario(seed, size, width=(0.5, 1.0, 2.0), origin=(-1.0, 0.5, 2.0), ppc=9,
                                        vscale=0.4, species=((1.0, 1.0), (-0.5, -2.0)), ragged=True)
        J_ref, rho_ref = allocating_projection(props, parts, counts, flags)
        J, rho = Buffers(props, parts, counts, with_rho).call(props, flags)
        close(J, J_ref)
        if with_rho:
            close(rho, rho_ref)


@pytest.mark.parametrize("name", ["p3", "p435"])
def test_project_noalloc_matches_the_reference_projection(name):
    """J = projectToDensityField's (cell.h:787-824, with its /8) from the
    compiled reference; without the /8 flag exactly 8 times that."""
    import torch
    torch.cuda.init()
    gold = golden_npz("project_small.npz")
    props = props_from_vec(gold[name + "_props"])
    parts, counts = gold[name + "_in"], gold[name + "_in_counts"]
    buf = Buffers(props, parts, counts, True)
    J, _ = buf.call(props, abi.F_J_DIV8)
    close(J, gold[name + "_J"])
    J, _ = buf.call(props, 0)
    close(J, 8.0 * gold[name + "_J"])


def test_project_noalloc_without_particles_gives_zero_grids():
    import torch
    torch.cuda.init()
    props, parts, counts = scenario(103, (6, 6, 6), ppc=7, vscale=0.3, species=((1.0, 1.0),))
    buf = Buffers(props, parts, counts, True)
    J, rho = buf.call(props, abi.F_J_DIV8)  # leaves non-zero sums in the shared scratch
    assert np.abs(J).max() > 0 and np.abs(rho).max() > 0
    J, rho = buf.call(props, abi.F_J_DIV8, particles=False)
    assert not J.any() and not rho.any()


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

"""ipic3d_gpu_aggregate_contributions (aggregateDensityContributions,
cell.h:835-855, over all nodes) against the reference's own function
(fixture) and the oracle: J bit-identical (the same FP64 additions in the
same order, then / vol / 8)."""
import ctypes as C

import numpy as np
import pytest

import allscale_ipic3d_gb300 as ipg
import oracle
from allscale_ipic3d_gb300 import abi
from common import golden_npz, props_from_vec

pytestmark = pytest.mark.gpu


def gpu_aggregate(props, contrib, J0):
    torch = pytest.importorskip("torch")
    dc = torch.from_numpy(np.ascontiguousarray(contrib)).cuda()
    dj = torch.from_numpy(np.ascontiguousarray(J0).copy()).cuda()
    ipg.aggregate_contributions(props, dc.data_ptr(), dj.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return dj.cpu().numpy()


@pytest.mark.parametrize("name", ["a3", "a425"])
def test_aggregate_matches_reference(name):
    g = golden_npz("aggregate_small.npz")
    props = props_from_vec(g[name + "_props"])
    np.testing.assert_array_equal(gpu_aggregate(props, g[name + "_contrib"], g[name + "_J0"]), g[name + "_J"])


@pytest.mark.parametrize("size,width", [((1, 1, 1), (0.3, 0.7, 1.1)), ((64, 48, 40), (0.5, 0.25, 2.0))])
def test_aggregate_matches_oracle(size, width):
    props = abi.Props.make(size=size, cell_width=width, dt=0.1)
    rng = np.random.default_rng(sum(size))
    contrib = rng.normal(0.0, 1.0, tuple(2 * v for v in size) + (3,))
    J0 = rng.normal(0.0, 1.0, abi.density_shape(props))
    want = J0.copy()
    assert oracle.load().oracle_aggregate_contributions(C.byref(props), abi.vptr(contrib), abi.vptr(want)) == 0
    np.testing.assert_array_equal(gpu_aggregate(props, contrib, J0), want)


def test_aggregate_rejects_bad_arguments():
    props = abi.Props.make(size=(2, 2, 2))
    with pytest.raises(ipg.GpuPathError):
        ipg.aggregate_contributions(props, None, None)

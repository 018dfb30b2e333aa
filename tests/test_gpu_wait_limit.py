"""The FP32 push's bounded waits. Its warps wait only on their own thread
block's shared-memory barriers (bulk-copy completion, stage release), each
wait with a bound; a wait that runs out makes the thread block record a
timeout, let its own copies in flight land and return, and the step returns
IPIC3D_E_TIMEOUT. Here the bound is set to zero polls so that every wait runs
out at once (nothing is broken: the copies are real and complete); the
context must report the timeout with its message, then run normally with the
default bound and match the oracle."""
import numpy as np
import pytest

import allscale_ipic3d_gb300 as g
from allscale_ipic3d_gb300 import abi
from common import OracleSim, gpu_sim, scenario

pytestmark = pytest.mark.gpu


def test_push_wait_runs_out_then_context_recovers():
    props, parts, counts = scenario(4242, (8, 8, 8), dt=0.05, ppc=32, vscale=0.05,
                                    species=((-1.0 / 32, -1.0), (1.0 / 32, 0.01)))
    kw = dict(mover=abi.MOVER_FIELD, solver=abi.SOLVER_LEAPFROG, projector=abi.PROJECT_CIC, bc=abi.BC_PERIODIC,
              flags=abi.F_REFRESH_NODE_B)
    sim = gpu_sim(props, abi.Config.make(precision=abi.FP32, flags=kw.pop("flags") | abi.F_USE_GRAPH, **kw))
    kw["flags"] = abi.F_REFRESH_NODE_B
    sim.set_push_shape(item=256, item_cells=32, blocks_per_sm=2)  # no tuning trials
    sim.upload_particles(parts, counts)
    sim.set_wait_limit(0)
    with pytest.raises(g.GpuPathError) as e:
        sim.step(1)
    assert e.value.status == abi.E_TIMEOUT
    assert "gave up waiting" in str(e.value)
    # the same context, the default bound, the original state again
    sim.set_wait_limit(None)
    f0 = np.zeros(abi.field_shape(props))
    bc0 = np.zeros(abi.bcfield_shape(props))
    j0 = np.zeros(abi.density_shape(props))
    sim.upload_fields(f0, bc0, j0)
    sim.upload_particles(parts, counts)
    sim.step(3)
    orc = OracleSim(props, abi.Config.make(**kw))
    orc.upload_particles(parts, counts)
    orc.step(3)
    c32, co = sim.conserved(), orc.conserved()
    assert c32["particles"] == co["particles"] == len(parts)
    assert abs(c32["kinetic_energy"] - co["kinetic_energy"]) <= 1e-5 * abs(co["kinetic_energy"])
    np.testing.assert_array_equal(sim.cell_counts(), orc.cell_counts())
    assert sim.stats()["steps"] >= 3
    sim.close()

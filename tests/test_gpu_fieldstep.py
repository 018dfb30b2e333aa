"""A run of steps in which the next step's field solve runs beside the
current step's placement (graph steps: the first solve alone, then each move
with the following solve on a second stream), against the one-call-per-phase
sequence of the public API (update_boundaries + solve_fields + move): fields
and particles bit-identical. The projector is off, so J stays as uploaded and
nothing depends on the order of atomic additions."""
import numpy as np
import pytest

from allscale_ipic3d_gb300 import abi
from common import align_by_id, gpu_sim, scenario

pytestmark = pytest.mark.gpu

G = abi.F_USE_GRAPH
CASES = [  # (precision, solver, flags, cells per axis)
    (abi.FP64, abi.SOLVER_LEAPFROG, abi.F_REFRESH_NODE_B | G, 8),
    (abi.FP64, abi.SOLVER_LEAPFROG, G, 7),
    (abi.FP64, abi.SOLVER_FORWARD, G, 6),
    (abi.FP64, abi.SOLVER_LEAPFROG, abi.F_REFRESH_NODE_B, 5),  # eager steps, one stream
    (abi.FP32, abi.SOLVER_LEAPFROG, abi.F_REFRESH_NODE_B | G, 8),
    (abi.FP32, abi.SOLVER_LEAPFROG, abi.F_DIPOLE_IN_GATHER | G, 9),
    (abi.FP32, abi.SOLVER_FORWARD, G, 6),
    # a larger grid: multi-block solver kernels beside a multi-block placement
    (abi.FP32, abi.SOLVER_LEAPFROG, abi.F_REFRESH_NODE_B | G, 48),
]


@pytest.mark.parametrize("prec,solver,flags,n", CASES)
def test_fused_field_step_matches_separate_kernels(prec, solver, flags, n):
    props, parts, counts = scenario(7100 + n, (n, n, n), width=(0.5, 0.5, 0.5), dt=0.05, ppc=4 if n < 20 else 1,
                                    vscale=0.1, species=((-1.0, -1.0), (1.0, 0.1)))
    rng = np.random.default_rng(n)
    f = rng.normal(0.0, 0.02, abi.field_shape(props))
    bc = rng.normal(0.0, 0.02, abi.bcfield_shape(props))
    dens = rng.normal(0.0, 0.01, abi.density_shape(props))
    cfg = abi.Config.make(precision=prec, mover=abi.MOVER_FIELD, solver=solver, projector=abi.PROJECT_NONE,
                          bc=abi.BC_PERIODIC, flags=abi.F_TRACK_IDS | flags)
    run, phases = gpu_sim(props, cfg), gpu_sim(props, cfg)
    for s in (run, phases):
        s.upload_fields(f, bc, dens)
        s.upload_particles(parts, counts)
    steps = 4
    run.step(steps)  # overlapped graph steps where F_USE_GRAPH is set, else one stream
    for _ in range(steps):
        phases.update_boundaries()
        phases.solve_fields()
        phases.move()
    (f1, b1, d1, _), (f2, b2, d2, _) = run.download_fields(), phases.download_fields()
    np.testing.assert_array_equal(f1, f2)
    np.testing.assert_array_equal(b1, b2)
    np.testing.assert_array_equal(d1, d2)
    a, b = align_by_id(run.download_particles(), phases.download_particles())
    np.testing.assert_array_equal(a["position"], b["position"])
    np.testing.assert_array_equal(a["velocity"], b["velocity"])
    run.close()
    phases.close()

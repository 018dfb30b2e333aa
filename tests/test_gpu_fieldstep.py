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


def sparse_particles(props, cells, seed):
    """One particle in each listed cell (x, y, z), grouped by cell, slow
    enough to stay put for a few steps; cells two apart share no node (up to
    the periodic fold), so every node's deposit is one addition."""
    rng = np.random.default_rng(seed)
    s = props.shape
    counts = np.zeros(props.ncells, np.uint64)
    order = sorted(cells, key=lambda c: (c[0] * s[1] + c[1]) * s[2] + c[2])
    p = np.zeros(len(order), abi.PARTICLE_DTYPE)
    w = np.array(props.cell_width)
    for i, c in enumerate(order):
        counts[(c[0] * s[1] + c[1]) * s[2] + c[2]] = 1
        p[i]["position"] = np.array(props.origin) + (np.array(c) + 0.3 + 0.4 * rng.random(3)) * w
        p[i]["velocity"] = rng.normal(0.0, 0.002, 3)
    p["q"] = -0.5
    p["qom"] = -1.0
    return p, counts


@pytest.mark.parametrize("prec,width,flags", [
    (abi.FP64, (0.6, 0.5, 0.7), 0),                    # J finalised by division (vol not a power of two)
    (abi.FP64, (0.5, 0.5, 0.5), abi.F_J_DIV8),         # by one multiplication, with the extra / 8
    (abi.FP32, (0.6, 0.5, 0.7), abi.F_REFRESH_NODE_B),
])
def test_raw_j_read_matches_j_finalisation(prec, width, flags):
    """With the projector on, a graph run reads the deposit's raw node sums in
    the E update (periodic fold and normalisation on the read, no J
    finalisation kernel) except after its last step; eager steps finalise J
    every step. Fields, J, rho and particles agree bit for bit."""
    props, _, _ = scenario(7301, (8, 8, 8), width=width, dt=0.05, ppc=1)
    parts, counts = sparse_particles(props, [(0, 0, 0), (7, 3, 0), (3, 7, 5), (5, 0, 7), (2, 4, 3)], 7302)
    rng = np.random.default_rng(7303)
    f = rng.normal(0.0, 0.02, abi.field_shape(props))
    bc = rng.normal(0.0, 0.02, abi.bcfield_shape(props))
    kw = dict(precision=prec, mover=abi.MOVER_FIELD, solver=abi.SOLVER_LEAPFROG, projector=abi.PROJECT_CIC,
              bc=abi.BC_PERIODIC)
    run = gpu_sim(props, abi.Config.make(flags=abi.F_TRACK_IDS | abi.F_USE_GRAPH | flags, **kw))
    eager = gpu_sim(props, abi.Config.make(flags=abi.F_TRACK_IDS | flags, **kw))
    for s in (run, eager):
        s.upload_fields(f, bc, None)
        s.upload_particles(parts, counts)
    if prec == abi.FP32:  # no autotuner trials: the same steps in both
        for s in (run, eager):
            s.set_push_shape(256, 32, 2)
    run.step(6)
    eager.step(6)
    for a, b in zip(run.download_fields(), eager.download_fields()):
        np.testing.assert_array_equal(a, b)
    a, b = align_by_id(run.download_particles(), eager.download_particles())
    np.testing.assert_array_equal(a["position"], b["position"])
    np.testing.assert_array_equal(a["velocity"], b["velocity"])
    run.close()
    eager.close()


@pytest.mark.parametrize("n", [5, 16])
def test_fp32_node_b_refresh_matches_interp_c2n(n):
    """The FP32 leapfrog solve with the node B refresh: every node B equals
    interpC2N's (field.h:234-247) 1/8 sum of the 8 surrounding Bc, summed in
    the same order, bit for bit, on every node of [1, s+1]^3 (the + faces
    included); the ghost nodes keep the uploaded B."""
    props, parts, counts = scenario(7300 + n, (n, n, n), width=(0.5, 0.5, 0.5), dt=0.05, ppc=2, vscale=0.1,
                                    species=((-1.0, -1.0),))
    rng = np.random.default_rng(73 + n)
    f = rng.normal(0.0, 0.02, abi.field_shape(props))
    bc = rng.normal(0.0, 0.02, abi.bcfield_shape(props))
    dens = rng.normal(0.0, 0.01, abi.density_shape(props))
    cfg = abi.Config.make(precision=abi.FP32, mover=abi.MOVER_FIELD, solver=abi.SOLVER_LEAPFROG,
                          projector=abi.PROJECT_NONE, bc=abi.BC_PERIODIC, flags=abi.F_REFRESH_NODE_B)
    sim = gpu_sim(props, cfg)
    sim.upload_fields(f, bc, dens)
    sim.upload_particles(parts, counts)
    sim.solve_fields()
    field, bcf, _, _ = sim.download_fields()
    sim.close()
    s = n
    a = np.zeros((s + 1, s + 1, s + 1, 3))
    for i in range(2):
        for j in range(2):
            for k in range(2):
                a = a + bcf[1 - i:s + 2 - i, 1 - j:s + 2 - j, 1 - k:s + 2 - k, 0:3]
    np.testing.assert_array_equal(field[1:s + 2, 1:s + 2, 1:s + 2, 3:6], 0.125 * a)
    # nodes outside [1, s+1]^3 keep the uploaded B
    mask = np.ones(field.shape[:3], dtype=bool)
    mask[1:s + 2, 1:s + 2, 1:s + 2] = False
    np.testing.assert_array_equal(field[mask][:, 3:6], f[mask][:, 3:6])

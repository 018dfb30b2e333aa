"""The CPU oracle (oracle/ipic3d_oracle*.cpp) pinned against outputs of the
reference's own code (fixtures in tests/golden/, generated by
tests/golden/make_golden.py) and the reference's unit-test known answers."""
import numpy as np
import pytest

from allscale_ipic3d_gb300 import abi
from common import (OracleSim, golden_json, golden_npz, init_inp, props_from_vec, reference_config, sha)

MOVES = ["walls", "dipole", "ragged", "single", "fast", "strong"]


@pytest.mark.parametrize("name", MOVES)
def test_default_loop_bit_exact(name):
    """simulateSteps with the default policies (simulator.h:127-242): counts,
    the per-cell import order (cell.h:1272-1306) and every particle byte."""
    g = golden_npz("moves_small.npz")
    props = props_from_vec(g[name + "_props"])
    sim = OracleSim(props, reference_config())
    sim.upload_particles(g[name + "_in"], g[name + "_in_counts"])
    sim.step(int(g[name + "_steps"][0]))
    p, c, i = sim.download_particles()
    np.testing.assert_array_equal(c, g[name + "_out_counts"])
    np.testing.assert_array_equal(i, g[name + "_out_ids"])
    assert p.tobytes() == g[name + "_out"].tobytes()


@pytest.mark.parametrize("name", ["p3", "p435"])
def test_projection_bit_exact(name):
    """projectToDensityField over all nodes (cell.h:787-824), J = Js/vol/8."""
    g = golden_npz("project_small.npz")
    props = props_from_vec(g[name + "_props"])
    sim = OracleSim(props, abi.Config.make(projector=abi.PROJECT_CIC, flags=abi.F_J_DIV8))
    sim.upload_particles(g[name + "_in"], g[name + "_in_counts"])
    sim.project()
    _, _, J, _ = sim.download_fields()
    assert J.tobytes() == g[name + "_J"].tobytes()


def test_boundaries_and_leapfrog_bit_exact():
    """updateFieldsOnBoundaries (field.h:407-440) and the two-phase reading of
    solveFieldLeapfrog (field.h:342-372)."""
    g = golden_npz("fields_small.npz")
    props = props_from_vec(g["props"])
    sim = OracleSim(props, abi.Config.make(solver=abi.SOLVER_LEAPFROG))
    sim.upload_fields(g["field"], g["bcfield"], g["J"])
    sim.update_boundaries()
    f, b, _, _ = sim.download_fields()
    assert f.tobytes() == g["bnd_field"].tobytes()
    assert b.tobytes() == g["bnd_bcfield"].tobytes()
    sim.upload_fields(g["field"], g["bcfield"], g["J"])
    sim.solve_fields()
    f, b, _, _ = sim.download_fields()
    assert f.tobytes() == g["lf_field"].tobytes()
    assert b.tobytes() == g["lf_bcfield"].tobytes()


def test_forward_solver_e_update():
    """solveFieldForward's E update at a node (field.h:302-311) from the
    unchanged Bc; the Bc and node-B parts of the per-node reference function
    read a mix of old and new E, so only E is compared."""
    g = golden_npz("fields_small.npz")
    props = props_from_vec(g["props"])
    sim = OracleSim(props, abi.Config.make(solver=abi.SOLVER_FORWARD))
    sim.upload_fields(g["field"], g["bcfield"], g["J"])
    sim.solve_fields()
    f, _, _, _ = sim.download_fields()
    for k, nd in enumerate(g["fw_nodes"]):
        x, y, z = nd
        assert f[x, y, z, 0:3].tobytes() == g["fw_field"][k][x, y, z, 0:3].tobytes()


def test_inp_init_bit_exact():
    """initCells<uniform_pos_normal_speed> of the .inp driver (cell.h:492-636,
    src/ipic3d.cxx:70-83): identical particle bytes."""
    runs = golden_json("inp_runs.json")
    for name in ("test", "tiny"):
        props, parts, counts = init_inp(runs[name])
        assert sha(counts) == runs[name]["initial_counts_sha256"], name
        assert sha(parts) == runs[name]["initial_particles_sha256"], name


@pytest.mark.parametrize("name", ["test", "tiny"])
def test_inp_run_bit_exact(name):
    """The whole .inp driver run: ncycles steps of the default loop."""
    run = golden_json("inp_runs.json")[name]
    props, parts, counts = init_inp(run)
    sim = OracleSim(props, reference_config())
    sim.upload_particles(parts, counts)
    sim.step(run["ncycles"])
    p, c, i = sim.download_particles()
    assert c.tolist() == run["final_counts"]
    assert sha(p) == run["final_particles_sha256"]
    assert sha(i) == run["final_ids_sha256"]


def test_boris_known_answers():
    """particle_test.cc:45-81 (qom=4, E=(1,-1,3), B=(0,1,2), dt=1) and
    particle_test.cc:7-42 (position update)."""
    import ctypes as C
    import oracle
    lib = oracle.load()
    p = np.zeros(1, abi.PARTICLE_DTYPE)
    p["velocity"] = (1.0, 2.0, 3.0)
    p["qom"] = 1.0 / 0.25
    E = np.array([1.0, -1.0, 3.0])
    B = np.array([0.0, 1.0, 2.0])
    lib.oracle_boris(abi.vptr(p), 1, abi.vptr(E), abi.vptr(B), 1.0, 1, 0)
    np.testing.assert_allclose(p["velocity"][0], [-2.42857, 3.71429, 12.14286], atol=1e-4)
    q = np.zeros(1, abi.PARTICLE_DTYPE)
    q["velocity"] = (1.0, 2.0, 3.0)
    z = np.zeros(3)
    lib.oracle_boris(abi.vptr(q), 1, abi.vptr(z), abi.vptr(z), 1.0, 1, 1)
    assert list(q["position"][0]) == [1.0, 2.0, 3.0]
    lib.oracle_boris(abi.vptr(q), 1, abi.vptr(z), abi.vptr(z), 0.5, 1, 1)
    assert list(q["position"][0]) == [1.5, 3.0, 4.5]


def test_trilinear_known_answers():
    """field_test.cc:231-273."""
    import oracle
    lib = oracle.load()
    ones = np.ones(8)
    half = np.array([0.5, 0.5, 0.5])
    assert lib.oracle_trilinear(abi.vptr(ones), abi.vptr(half), 1.0) == 1.0
    c = np.array([i * 1 + j * 2 + k * 3 for i in range(2) for j in range(2) for k in range(2)], np.float64)
    assert lib.oracle_trilinear(abi.vptr(c), abi.vptr(half), 0.75) == 4.0
    assert lib.oracle_trilinear(abi.vptr(c), abi.vptr(np.zeros(3)), 3.0) == 0.0
    assert lib.oracle_trilinear(abi.vptr(c), abi.vptr(np.ones(3)), 1.0) == 6.0


def test_inp_conserved_trace():
    """The conserved quantities before every cycle of the test.inp run (the
    trace of the reference's debug build, simulator.h:65-90): total momentum
    and kinetic energy per cycle equal to 1e-12 relative, and printed alike."""
    run = golden_json("inp_runs.json")["test"]
    props, parts, counts = init_inp(run)
    sim = OracleSim(props, reference_config())
    sim.upload_particles(parts, counts)
    for row in run["trace"]:
        c = sim.conserved()
        for k, col in (("total_momentum", 1), ("kinetic_energy", 4)):
            assert abs(c[k] - row[col]) <= 1e-12 * abs(row[col]), (row[0], k, c[k], row[col])
            assert "%g" % c[k] == "%g" % row[col], (row[0], k)
        sim.step(1)


@pytest.mark.parametrize("name", ["a3", "a425"])
def test_aggregate_contributions_bit_exact(name):
    """aggregateDensityContributions (cell.h:835-855) over all nodes: the
    restatement against the reference's own function (fixture)."""
    import ctypes as C

    import oracle
    g = golden_npz("aggregate_small.npz")
    props = props_from_vec(g[name + "_props"])
    J = np.ascontiguousarray(g[name + "_J0"]).copy()
    contrib = np.ascontiguousarray(g[name + "_contrib"])
    assert oracle.load().oracle_aggregate_contributions(C.byref(props), abi.vptr(contrib), abi.vptr(J)) == 0
    np.testing.assert_array_equal(J, g[name + "_J"])

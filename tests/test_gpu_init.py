"""Device initialisation with the reference's random streams:
ipic3d_gpu_init_uniform (initCells(uniform), cell.h:638-697, the ":U:N"
benchmark's universe) against the oracle's restatement, which draws with the
same std::minstd_rand / std::uniform_real_distribution the reference uses:
per-cell counts and every particle bit-identical (FP64 storage), and the
first steps from there equal to the oracle's."""
import ctypes as C

import numpy as np
import pytest

import oracle
from allscale_ipic3d_gb300 import abi
from common import OracleSim, align_by_id, assert_states_close, gpu_sim, reference_config

pytestmark = pytest.mark.gpu

CASES = [  # (particles, cells, cell width, origin)
    (100003, (8, 8, 8), (10.0, 10.0, 10.0), (0.0, 0.0, 0.0)),  # the :U:N geometry, scaled down
    (77777, (6, 5, 7), (0.5, 1.5, 2.0), (-1.0, 2.0, 0.25)),
    (300, (4, 4, 4), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0)),        # fewer particles than 5 per cell
]


def reference_init(props, n):
    lib = oracle.load()
    out = np.zeros(n, abi.PARTICLE_DTYPE)
    counts = np.zeros(props.ncells, np.uint64)
    assert lib.oracle_init_uniform_bench(C.byref(props), n, abi.vptr(out), abi.vptr(counts)) == 0
    return out, counts


@pytest.mark.parametrize("n,size,width,origin", CASES)
def test_init_uniform_fp64_bit_identical(n, size, width, origin):
    props = abi.Props.make(size=size, cell_width=width, dt=0.15, origin=origin)
    sim = gpu_sim(props, abi.Config.make(precision=abi.FP64, flags=abi.F_TRACK_IDS))
    sim.init_uniform(n)
    parts, counts = reference_init(props, n)
    pg, cg, ig = sim.download_particles()
    np.testing.assert_array_equal(cg, counts)
    np.testing.assert_array_equal(np.sort(ig), np.arange(n))
    pg = pg[np.argsort(ig, kind="stable")]
    for f in ("position", "velocity", "q", "qom"):
        np.testing.assert_array_equal(pg[f], parts[f], err_msg=f)
    # the reference's default policies from here: the same particles as the oracle's
    orc = OracleSim(props, reference_config())
    orc.upload_particles(parts, counts)
    for s in (sim, orc):
        s.step(3)
    a, b = align_by_id(sim.download_particles(), orc.download_particles())
    assert_states_close(a, b, rtol=1e-12, atol=1e-12, what="after init")
    sim.close()


def test_init_uniform_fp32_storage():
    """FP32 contexts store the same particles cell-relative: positions within
    FP32 rounding of the cell width, velocities within FP32 rounding."""
    n, size, width = 50000, (6, 6, 6), (10.0, 10.0, 10.0)
    props = abi.Props.make(size=size, cell_width=width, dt=0.15)
    sim = gpu_sim(props, abi.Config.make(precision=abi.FP32, flags=abi.F_TRACK_IDS))
    sim.init_uniform(n)
    parts, counts = reference_init(props, n)
    pg, cg, ig = sim.download_particles()
    np.testing.assert_array_equal(cg, counts)
    pg = pg[np.argsort(ig, kind="stable")]
    np.testing.assert_allclose(pg["position"], parts["position"], rtol=0, atol=1e-6 * 10.0)
    np.testing.assert_allclose(pg["velocity"], parts["velocity"], rtol=1e-7, atol=0)
    np.testing.assert_array_equal(pg["q"], parts["q"])
    sim.close()


def test_init_uniform_replaces_particles_and_zero():
    props = abi.Props.make(size=(3, 3, 3), cell_width=(2.0, 2.0, 2.0), dt=0.1)
    sim = gpu_sim(props, abi.Config.make(precision=abi.FP64))
    sim.init_uniform(1000)
    assert sim.particle_count() == 1000
    sim.init_uniform(0)
    assert sim.particle_count() == 0
    sim.step(2)
    sim.init_uniform(55)
    assert sim.particle_count() == 55
    assert sim.cell_counts().sum() == 55
    sim.close()


@pytest.mark.parametrize("name", ["test", "tiny"])
def test_init_inp_distribution_bit_identical(name):
    """initCells with the .inp driver's uniform_pos_normal_speed distribution
    (cell.h:492-636) on the device: every particle equals the compiled
    reference's (the fixture's SHA-256 of its initial particles, grouped by
    cell) and the oracle's restatement; FP32 storage holds the same values
    within FP32 rounding."""
    from common import golden_json, init_inp, props_from_dict, sha
    run = golden_json("inp_runs.json")[name]
    props = props_from_dict(run["props"])
    ref_parts, ref_counts = init_inp(run)[1:]
    args = [run["num_particles"], run["low"], run["hig"], run["mean"], run["stddev"]]
    sim = gpu_sim(props, abi.Config.make(precision=abi.FP64, flags=abi.F_TRACK_IDS))
    sim.init_uniform_pos_normal_speed(*args)
    pg, cg, ig = sim.download_particles()
    np.testing.assert_array_equal(cg, ref_counts)
    assert sha(cg.astype(np.uint64)) == run["initial_counts_sha256"]
    pg = pg[np.argsort(ig, kind="stable")]
    assert sha(pg) == run["initial_particles_sha256"]
    for f in ("position", "velocity", "q", "qom"):
        np.testing.assert_array_equal(pg[f], ref_parts[f], err_msg=f)
    sim.close()
    sim = gpu_sim(props, abi.Config.make(precision=abi.FP32, flags=abi.F_TRACK_IDS))
    sim.init_uniform_pos_normal_speed(*args)
    p32, c32, i32 = sim.download_particles()
    np.testing.assert_array_equal(c32, ref_counts)
    p32 = p32[np.argsort(i32, kind="stable")]
    w = np.array(props.cell_width)
    assert (np.abs(p32["position"] - ref_parts["position"]) <= 1e-6 * w).all()
    np.testing.assert_allclose(p32["velocity"], ref_parts["velocity"], rtol=1e-7, atol=0)
    sim.close()


def test_init_inp_distribution_arguments():
    props = abi.Props.make(size=(4, 4, 4), cell_width=(1.0, 1.0, 1.0), dt=0.1)
    sim = gpu_sim(props, abi.Config.make(precision=abi.FP64))
    import allscale_ipic3d_gb300 as g
    with pytest.raises(g.GpuPathError) as e:  # an empty position box
        sim.init_uniform_pos_normal_speed(100, (1, 1, 1), (1, 2, 2), (0, 0, 0), (1, 1, 1))
    assert e.value.status == abi.E_INVALID
    with pytest.raises(g.GpuPathError) as e:  # a box outside the universe
        sim.init_uniform_pos_normal_speed(100, (5, 5, 5), (6, 6, 6), (0, 0, 0), (1, 1, 1))
    assert e.value.status == abi.E_INVALID
    sim.init_uniform_pos_normal_speed(0, (0, 0, 0), (4, 4, 4), (0, 0, 0), (1, 1, 1))
    assert sim.particle_count() == 0
    sim.close()

"""The reference's own unit tests with known answers, run through the GPU
path (C ABI): particle_test.cc, simulation_test.cc, cell_test.cc. Each test
cites the reference test it restates and keeps its tolerances."""
import numpy as np
import pytest

import allscale_ipic3d_gb300 as g
from allscale_ipic3d_gb300 import abi
from common import gpu_sim, reference_config

pytestmark = pytest.mark.gpu


def one_particle(pos, vel, q=1.0, qom=1.0):
    p = np.zeros(1, abi.PARTICLE_DTYPE)
    p["position"] = pos
    p["velocity"] = vel
    p["q"] = q
    p["qom"] = qom
    return p


def test_particle_velocity_update():
    """particle_test.cc:45-81."""
    p = one_particle((0.0, 0.0, 0.0), (1.0, 2.0, 3.0), qom=1.0 / 0.25)
    g.boris(p, (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 1.0, push_position=False)
    assert list(p["velocity"][0]) == [1.0, 2.0, 3.0]
    g.boris(p, (1.0, -1.0, 3.0), (0.0, 1.0, 2.0), 1.0, push_position=False)
    np.testing.assert_allclose(p["velocity"][0], [-2.42857, 3.71429, 12.14286], atol=1e-4)


def test_particle_position_update():
    """particle_test.cc:7-42."""
    p = one_particle((0.0, 0.0, 0.0), (1.0, 2.0, 3.0))
    g.boris(p, (0, 0, 0), (0, 0, 0), 1.0)
    assert list(p["position"][0]) == [1.0, 2.0, 3.0]
    g.boris(p, (0, 0, 0), (0, 0, 0), 0.5)
    assert list(p["position"][0]) == [1.5, 3.0, 4.5]


def test_larmor_radius_direct_boris():
    """simulation_test.cc:187-263: electron in B_z = 0.01, 1000 Boris steps
    after a half step back, against the MATLAB trajectory."""
    q, mass = -1.602e-19, 9.109e-31
    B = (0.0, 0.0, 0.01)
    rL = mass * 1e5 / (abs(q) * B[2])
    assert abs(rL - 5.686e-05) < 1e-6
    p = one_particle((rL, 0.0, 0.0), (0.0, 1e5, 0.0), q=q, qom=q / mass)
    g.boris(p, (0, 0, 0), B, -0.5 * 3e-11, push_position=False)
    g.boris(p, (0, 0, 0), B, 3e-11, nsteps=1000)
    x, y, z = p["position"][0]
    u, v, w = p["velocity"][0]
    assert abs(x - -4.50134e-05) < 1e-10 and abs(y - 3.47983e-05) < 1e-9 and abs(z) < 1e-10
    assert abs(u - -63242.7) < 1e1 and abs(v - -77462.0) < 1e1 and abs(w) < 1e-2


def test_exb_drift_direct_boris():
    """simulation_test.cc:340-407: E = (0.2,0,0), B = (0,0,1), 5000 steps."""
    p = one_particle((0.0, 0.0, 0.0), (0.5, 0.0, 0.0))
    E, B = (0.2, 0.0, 0.0), (0.0, 0.0, 1.0)
    g.boris(p, E, B, -0.5 * 0.01, push_position=False)
    g.boris(p, E, B, 0.01, nsteps=5000)
    x, y, z = p["position"][0]
    u, v, w = p["velocity"][0]
    assert abs(x - -0.1131) < 1e-1 and abs(y - -10.0797) < 1e-2 and abs(z) < 1e-10
    assert abs(u - 0.4203) < 1e-2 and abs(v - 0.1131) < 1e-1 and abs(w) < 1e-10


def test_single_particle_boris_mover_in_loop():
    """simulation_test.cc:135-184: one cell, dt 0.1, 9 steps of the default
    mover (no planet: the dipole B is zero, the particle free-streams)."""
    props = abi.Props.make(size=(1, 1, 1), dt=0.1)
    sim = gpu_sim(props, reference_config())
    sim.upload_particles(one_particle((0.5, 0.5, 0.0), (0.0, 0.0, 1.0)), [1])
    sim.step(9)
    p, c, _ = sim.download_particles()
    assert c[0] == 1
    np.testing.assert_allclose(p["position"][0], [0.5, 0.5, 0.899], atol=0.001)


def test_single_particle_larmor_radius_in_loop():
    """simulation_test.cc:266-337: 10 steps of the default loop; with
    planetRadius 0 the particle free-streams whatever the field grid holds."""
    q, mass = -1.602e-19, 9.109e-31
    props = abi.Props.make(size=(1, 1, 1), cell_width=(1e4, 1e4, 1e4), dt=3e-11, origin=(-10.0, -10.0, -10.0))
    rL = mass * 1e5 / (abs(q) * 0.01)
    p = one_particle((rL, 0.0, 0.0), (0.0, 1e5, 0.0), q=q, qom=q / mass)
    g.boris(p, (0, 0, 0), (0, 0, 0.01), -0.5 * 3e-11, push_position=False)
    sim = gpu_sim(props, reference_config())
    sim.upload_particles(p, [1])
    sim.step(10)
    r, c, _ = sim.download_particles()
    np.testing.assert_allclose(r["position"][0][:2], [5.7651e-05, 2.9990e-05], atol=1e-9)
    assert abs(r["position"][0][2]) < 1e-10


def cell_of(props, pos):
    o, w, s = np.array(props.origin), np.array(props.cell_width), np.array(props.size)
    return tuple(int(v) for v in np.floor((np.asarray(pos) - o) / w))


def placed_correctly(props, parts, counts):
    """verifyCorrectParticlesPositionInCell over all cells (cell.h:1168-1184):
    |position - centre| <= half width on every axis."""
    s = props.shape
    o, w = np.array(props.origin), np.array(props.cell_width)
    k = 0
    for c, n in enumerate(counts):
        idx = np.array([c // (s[1] * s[2]), (c // s[2]) % s[1], c % s[2]])
        centre = o + idx * w + w / 2.0
        for _ in range(int(n)):
            if np.any(np.abs(parts["position"][k] - centre) > w / 2.0):
                return False
            k += 1
    return True


def test_particle_migration_one_direction_one_particle():
    """simulation_test.cc:410-556: cell (0,1,0) -> (1,1,0) in one step, then
    100 steps later back in cell (0,1,0) through the wall reflection rule."""
    props = abi.Props.make(size=(3, 3, 3), cell_width=(.5, .5, .5), dt=0.1)
    counts = np.zeros(27, np.uint64)
    counts[0 * 9 + 1 * 3 + 0] = 1
    sim = gpu_sim(props, reference_config())
    sim.upload_particles(one_particle((0.46, 0.8, 0.0), (1.0, 0.5, 0.5)), counts)
    sim.step(1)
    p, c, _ = sim.download_particles()
    assert c.sum() == 1 and c[1 * 9 + 1 * 3 + 0] == 1
    assert abs(p["position"][0][0] - 0.56) < 1e-3 and abs(p["position"][0][1] - 0.8) < 1e-1
    assert abs(p["velocity"][0][0] - 1.0) < 1e-2
    assert placed_correctly(props, p, c)
    sim.step(100)
    p, c, _ = sim.download_particles()
    assert c.sum() == 1 and c[0 * 9 + 1 * 3 + 0] == 1
    assert abs(p["position"][0][0] - 0.06) < 1e-2 and abs(p["position"][0][1] - 0.8) < 1e-1
    assert abs(p["velocity"][0][0] - -1.0) < 1e-1
    assert placed_correctly(props, p, c)


def test_particle_migration_many_particles():
    """simulation_test.cc:687-777: 8 particles in 8 cells, 20 steps: count
    conserved and every particle in its correct cell."""
    props = abi.Props.make(size=(4, 4, 4), cell_width=(.5, .5, .5), dt=0.1)
    P = []
    p0 = ((0.4, 0.4, 0.4), (0.6, 0.6, 0.6))
    p1 = ((0.8, 0.4, 0.4), (0.3, 0.3, 0.3))
    p2 = ((0.4, 0.8, 0.4), (0.1, 0.1, 0.1))
    p3 = ((0.75, 0.75, 0.4), (0.8, 0.8, 0.8))
    p4 = ((0.4, 0.4, 0.6), p0[1])
    p5 = ((0.8, 0.4, 0.8), p1[1])
    p6 = ((0.25, 0.75, 0.75), p3[1])
    p7 = ((0.75, 0.75, 0.8), p3[1])
    cells = {(0, 0, 0): p0, (1, 0, 0): p1, (0, 1, 0): p2, (1, 1, 0): p3, (0, 0, 1): p4, (1, 0, 1): p5,
             (0, 1, 1): p6, (1, 1, 1): p7}
    counts = np.zeros(64, np.uint64)
    order = sorted(cells, key=lambda c: (c[0] * 4 + c[1]) * 4 + c[2])
    parts = np.zeros(8, abi.PARTICLE_DTYPE)
    for k, cidx in enumerate(order):
        parts[k]["position"], parts[k]["velocity"] = cells[cidx]
        counts[(cidx[0] * 4 + cidx[1]) * 4 + cidx[2]] = 1
    parts["q"] = parts["qom"] = 1.0
    assert placed_correctly(props, parts, counts)
    sim = gpu_sim(props, reference_config())
    sim.upload_particles(parts, counts)
    sim.step(20)
    p, c, _ = sim.download_particles()
    assert c.sum() == 8
    assert placed_correctly(props, p, c)


def test_project_to_density_field_kat():
    """cell_test.cc:211-291: 2^3 cells of width 0.5, 8 particles ->
    J(1,1,1) = (1.0952, 1.0952, 1.0952)."""
    props = abi.Props.make(size=(2, 2, 2), cell_width=(.5, .5, .5), dt=0.1)
    pos = {(0, 0, 0): (0.4, 0.4, 0.4), (1, 0, 0): (0.8, 0.4, 0.4), (0, 1, 0): (0.4, 0.8, 0.4),
           (1, 1, 0): (0.75, 0.75, 0.4), (0, 0, 1): (0.4, 0.4, 0.6), (1, 0, 1): (0.8, 0.4, 0.8),
           (0, 1, 1): (0.25, 0.75, 0.75), (1, 1, 1): (0.75, 0.75, 0.8)}
    vel = {(0, 0, 0): 0.6, (1, 0, 0): 0.3, (0, 1, 0): 0.1, (1, 1, 0): 0.8, (0, 0, 1): 0.6, (1, 0, 1): 0.3,
           (0, 1, 1): 0.8, (1, 1, 1): 0.8}
    order = sorted(pos, key=lambda c: (c[0] * 2 + c[1]) * 2 + c[2])
    parts = np.zeros(8, abi.PARTICLE_DTYPE)
    for k, cidx in enumerate(order):
        parts[k]["position"] = pos[cidx]
        parts[k]["velocity"] = (vel[cidx],) * 3
    parts["q"] = parts["qom"] = 1.0
    sim = gpu_sim(props, abi.Config.make(projector=abi.PROJECT_CIC, flags=abi.F_J_DIV8))
    sim.upload_particles(parts, np.ones(8, np.uint64))
    sim.project()
    _, _, J, _ = sim.download_fields()
    np.testing.assert_allclose(J[1, 1, 1], [1.0952, 1.0952, 1.0952], atol=1e-4)


def test_update_fields_on_boundaries_kat():
    """field_test.cc:316-416 (sums 6527, 7858, 7004; edges untouched)."""
    props = abi.Props.make(size=(10, 10, 10))
    n, nb = 13, 12
    f = np.zeros((n, n, n, 9))
    idx = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).astype(np.float64)
    f[..., 0:3] = idx
    f[..., 3:6] = idx
    b = np.stack(np.meshgrid(np.arange(nb), np.arange(nb), np.arange(nb), indexing="ij"), -1).astype(np.float64)
    f[1:-1, 1:-1, 1:-1, 0:3] = 1.0
    f[1:-1, 1:-1, 1:-1, 3:6] = 2.0
    b[1:-1, 1:-1, 1:-1] = 3.0
    assert list(f[..., 0:3].sum((0, 1, 2))) == [6527.0] * 3
    assert list(f[..., 3:6].sum((0, 1, 2))) == [7858.0] * 3
    assert list(b.sum((0, 1, 2))) == [7004.0] * 3
    sim = gpu_sim(props, abi.Config.make())
    sim.upload_fields(f, b, None)
    sim.update_boundaries()
    f2, b2, _, _ = sim.download_fields()
    for i in (0, n - 1):
        for j in (0, n - 1):
            for k in (0, n - 1):
                assert list(f2[i, j, k, 0:3]) == [i, j, k] and list(f2[i, j, k, 3:6]) == [i, j, k]
    for i in (0, nb - 1):
        for j in (0, nb - 1):
            for k in (0, nb - 1):
                assert list(b2[i, j, k]) == [i, j, k]
    fs = n - 1
    for i in range(1, fs):
        for j in range(1, fs):
            for face in (f2[0, i, j], f2[fs, i, j], f2[i, 0, j], f2[i, fs, j], f2[i, j, 0], f2[i, j, fs]):
                assert list(face[0:3]) == [1.0, 1.0, 1.0]
    # change interior values and check two positions (field_test.cc:405-414)
    f3 = f2.copy()
    f3[1:-1, 1:-1, 1:-1, 0:3] = idx[1:-1, 1:-1, 1:-1]
    f3[1:-1, 1:-1, 1:-1, 3:6] = 2.0 * idx[1:-1, 1:-1, 1:-1]
    sim.upload_fields(f3, b2, None)
    sim.update_boundaries()
    f4, _, _, _ = sim.download_fields()
    assert list(f4[0, 5, 11, 0:3]) == [11.0, 5.0, 11.0]
    assert list(f4[9, 12, 2, 3:6]) == [18.0, 2.0, 4.0]


def test_leapfrog_zero_in_zero_out():
    """field_test.cc:515-557."""
    props = abi.Props.make(size=(5, 5, 5))
    sim = gpu_sim(props, abi.Config.make(solver=abi.SOLVER_LEAPFROG))
    sim.solve_fields()
    f, b, _, _ = sim.download_fields()
    assert not f.any() and not b.any()


def test_forward_solver_kat():
    """field_test.cc:419-463: E = 0.2, B = 0.4, Bc = 0.8, J = 0.6, dt = 1:
    E(2,2,2) = -0.4, Bc(2,2,2) unchanged 0.8."""
    props = abi.Props.make(size=(5, 5, 5), dt=1.0)
    f = np.zeros(abi.field_shape(props))
    f[..., 0:3] = 0.2
    f[..., 3:6] = 0.4
    b = np.full(abi.bcfield_shape(props), 0.8)
    j = np.full(abi.density_shape(props), 0.6)
    sim = gpu_sim(props, abi.Config.make(solver=abi.SOLVER_FORWARD))
    sim.upload_fields(f, b, j)
    sim.solve_fields()
    f2, b2, _, _ = sim.download_fields()
    np.testing.assert_allclose(f2[2, 2, 2, 0:3], [-0.4] * 3, atol=1e-15)
    np.testing.assert_allclose(b2[2, 2, 2], [0.8] * 3, atol=1e-15)

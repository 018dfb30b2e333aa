"""The workload configurations the reference cannot run (periodic particles,
two species, uneven loads, injection), at sizes the oracle finishes in
seconds: the GPU path against the FP64 CPU oracle, plus physical checks."""
import numpy as np
import pytest

from allscale_ipic3d_gb300 import abi
from common import OracleSim, align_by_id, assert_states_close, gpu_sim, scenario

pytestmark = pytest.mark.gpu


def uniform_fields(props, E, B):
    f = np.zeros(abi.field_shape(props))
    f[..., 0:3] = E
    f[..., 3:6] = B
    bc = np.zeros(abi.bcfield_shape(props))
    bc[..., :] = B
    return f, bc


def test_exb_drift_8cube_periodic():
    """8^3 periodic unit cells, one species (q=-1, m=1), 64 particles per cell,
    Maxwellian sigma=0.01, B=(0,0,0.1), E=(0,0.01,0), dt=0.1, 100 steps, FP64,
    Boris + CIC deposit, fields held static: the mean velocity settles on the
    E x B drift v_d = E x B / |B|^2 = (0.1, 0, 0); the GPU matches the oracle
    particle by particle and in the deposited J."""
    props, parts, counts = scenario(1001, (8, 8, 8), dt=0.1, ppc=64, vscale=0.01, species=((-1.0, -1.0),))
    f, bc = uniform_fields(props, (0.0, 0.01, 0.0), (0.0, 0.0, 0.1))
    cfg = abi.Config.make(precision=abi.FP64, mover=abi.MOVER_FIELD, projector=abi.PROJECT_CIC,
                          bc=abi.BC_PERIODIC, flags=abi.F_TRACK_IDS)
    sim, orc = gpu_sim(props, cfg), OracleSim(props, cfg)
    for s in (sim, orc):
        s.upload_fields(f, bc, None)
        s.upload_particles(parts, counts)
        s.step(100)
    a, b = align_by_id(sim.download_particles(), orc.download_particles())
    assert_states_close(a, b, rtol=1e-10, atol=1e-12, what="exb")
    # every particle starts near rest, so all gyrate in phase about the drift:
    # v(t) = v_d (1 - cos wt) x +- v_d sin wt y with w = |q/m| B = 0.1 and
    # t = 100 dt = 10 (Boris turns by 2 atan(w dt / 2) per step)
    wt = 100 * 2 * np.arctan(0.1 * 0.1 / 2)
    vx, vy = a["velocity"][:, 0].mean(), a["velocity"][:, 1].mean()
    assert abs(vx - 0.1 * (1 - np.cos(wt))) < 1e-3, vx
    assert abs(abs(vy) - 0.1 * np.sin(wt)) < 1e-3, vy
    orc.project()
    _, _, J1, _ = sim.download_fields()
    _, _, J2, _ = orc.download_fields()
    np.testing.assert_allclose(J1, J2, rtol=1e-10, atol=1e-12 * np.abs(J2).max())


def test_exb_drift_fp32_against_fp64():
    props, parts, counts = scenario(1002, (8, 8, 8), dt=0.1, ppc=64, vscale=0.01, species=((-1.0, -1.0),))
    f, bc = uniform_fields(props, (0.0, 0.01, 0.0), (0.0, 0.0, 0.1))
    kw = dict(mover=abi.MOVER_FIELD, projector=abi.PROJECT_CIC, bc=abi.BC_PERIODIC, flags=abi.F_TRACK_IDS)
    s32 = gpu_sim(props, abi.Config.make(precision=abi.FP32, **kw))
    s64 = gpu_sim(props, abi.Config.make(precision=abi.FP64, **kw))
    for s in (s32, s64):
        s.upload_fields(f, bc, None)
        s.upload_particles(parts, counts)
        s.step(100)
    c32, c64 = s32.conserved(), s64.conserved()
    assert c32["particles"] == c64["particles"] == len(parts)
    assert abs(c32["kinetic_energy"] - c64["kinetic_energy"]) <= 1e-5 * c64["kinetic_energy"]
    pa, _, ia = s32.download_particles()
    pb, _, ib = s64.download_particles()
    ka, kb = np.argsort(ia), np.argsort(ib)
    # positions: 100 steps of 0.1 at |v| ~ 0.1, in unit cells, FP32 cell-relative
    assert np.abs(pa["position"][ka] - pb["position"][kb]).max() < 2e-5


def blob_scenario(seed, n, ppc_uniform, blob_particles, sigma, centre, species):
    """Half uniform, half a 3-D Gaussian blob: per-cell counts from 0 to
    hundreds (the uneven-load configuration, scaled down)."""
    rng = np.random.default_rng(seed)
    props = abi.Props.make(size=(n, n, n), dt=0.05)
    nc = n ** 3
    pu = np.repeat(np.arange(nc), ppc_uniform)
    cz, cy, cx = pu % n, (pu // n) % n, pu // (n * n)
    pos_u = np.stack([cx, cy, cz], 1) + rng.random((len(pu), 3))
    pos_b = np.clip(rng.normal(centre, sigma, (blob_particles, 3)), 0.0, n - 1e-9)
    pos = np.concatenate([pos_u, pos_b])
    cell = (np.floor(pos[:, 0]).astype(int) * n + np.floor(pos[:, 1]).astype(int)) * n + np.floor(pos[:, 2]).astype(int)
    order = np.argsort(cell, kind="stable")
    pos, cell = pos[order], cell[order]
    N = len(pos)
    p = np.zeros(N, abi.PARTICLE_DTYPE)
    p["position"] = pos
    sp = rng.integers(0, len(species), N)
    q = np.array([s[0] for s in species])[sp]
    qom = np.array([s[1] for s in species])[sp]
    sig = np.array([s[2] for s in species])[sp]
    p["velocity"] = rng.normal(0.0, 1.0, (N, 3)) * sig[:, None]
    p["q"], p["qom"] = q, qom
    counts = np.bincount(cell, minlength=nc).astype(np.uint64)
    return props, p, counts


def test_uneven_load_two_species_fp64_matches_oracle():
    """Uneven loads (0 .. ~700 particles per cell), electrons (q=-1, m=1,
    sigma=0.02) and ions (q=+1, m=100, sigma=0.002), B=(0.05,0,0.1),
    self-consistent E (leapfrog, CIC): GPU FP64 against the oracle."""
    sp = ((-1.0 / 64, -1.0, 0.02), (1.0 / 64, 0.01, 0.002))
    props, parts, counts = blob_scenario(1003, 12, 2, 60000, 1.5, (7.0, 6.0, 5.5), sp)
    assert counts.max() > 400  # 2 .. ~950 particles per cell
    f, bc = uniform_fields(props, (0.0, 0.0, 0.0), (0.05, 0.0, 0.1))
    cfg = abi.Config.make(precision=abi.FP64, mover=abi.MOVER_FIELD, solver=abi.SOLVER_LEAPFROG,
                          projector=abi.PROJECT_CIC, bc=abi.BC_PERIODIC,
                          flags=abi.F_TRACK_IDS | abi.F_REFRESH_NODE_B)
    sim, orc = gpu_sim(props, cfg), OracleSim(props, cfg)
    for s in (sim, orc):
        s.upload_fields(f, bc, None)
        s.upload_particles(parts, counts)
        s.step(10)
    a, b = align_by_id(sim.download_particles(), orc.download_particles())
    assert_states_close(a, b, rtol=1e-9, atol=1e-11, what="uneven")
    (f1, b1, _, _), (f2, b2, _, _) = sim.download_fields(), orc.download_fields()
    np.testing.assert_allclose(f1, f2, rtol=1e-9, atol=1e-13)


def test_uneven_load_fp32_conserved_quantities():
    sp = ((-1.0 / 64, -1.0, 0.02), (1.0 / 64, 0.01, 0.002))
    props, parts, counts = blob_scenario(1004, 16, 2, 120000, 2.0, (9.0, 8.0, 7.0), sp)
    f, bc = uniform_fields(props, (0.0, 0.0, 0.0), (0.05, 0.0, 0.1))
    kw = dict(mover=abi.MOVER_FIELD, solver=abi.SOLVER_LEAPFROG, projector=abi.PROJECT_CIC,
              bc=abi.BC_PERIODIC, flags=abi.F_REFRESH_NODE_B)
    s32 = gpu_sim(props, abi.Config.make(precision=abi.FP32, **kw))
    orc = OracleSim(props, abi.Config.make(**kw))
    for s in (s32, orc):
        s.upload_fields(f, bc, None)
        s.upload_particles(parts, counts)
        s.step(20)
    c1, c2 = s32.conserved(), orc.conserved()
    assert c1["particles"] == c2["particles"]
    tot = lambda c: c["kinetic_energy"] + c["e_energy"] + c["b_energy"]
    assert abs(tot(c1) - tot(c2)) <= 1e-5 * abs(tot(c2))
    np.testing.assert_array_equal(s32.cell_counts().sum(), c2["particles"])

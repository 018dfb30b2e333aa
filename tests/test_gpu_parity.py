"""Parity of the GPU path (through the C ABI) with the reference's own outputs
(tests/golden/) and with the CPU oracle.

Bars: integer work (cell counts, which particle sits in which cell) is
bit-exact; FP64 states agree to 1e-12 relative (the only rounding difference
is pow(r^2, 2.5): the GPU's double-double evaluation is correctly rounded, the
host libm's is in all but rare cases); field updates without particles are
bit-exact; deposits differ only in the summation order of FP64 atomics
(1e-12 relative)."""
import numpy as np
import pytest

from allscale_ipic3d_gb300 import abi
from common import (OracleSim, align_by_id, assert_states_close, golden_json, golden_npz, gpu_sim, init_inp,
                    props_from_vec, reference_config, scenario)

pytestmark = pytest.mark.gpu

MOVES = ["walls", "dipole", "ragged", "single", "fast", "strong"]


@pytest.mark.parametrize("name", MOVES)
def test_default_loop_matches_reference(name):
    g = golden_npz("moves_small.npz")
    props = props_from_vec(g[name + "_props"])
    sim = gpu_sim(props, reference_config(flags=abi.F_TRACK_IDS))
    sim.upload_particles(g[name + "_in"], g[name + "_in_counts"])
    sim.step(int(g[name + "_steps"][0]))
    ref = (g[name + "_out"], g[name + "_out_counts"], g[name + "_out_ids"])
    a, b = align_by_id(sim.download_particles(), ref)
    assert_states_close(a, b, rtol=1e-12, atol=1e-13, what=name)


@pytest.mark.parametrize("name", ["test", "tiny"])
def test_inp_driver_run_counts_bit_exact(name):
    """test.inp / tiny.inp through the GPU: per-cell counts after ncycles
    steps equal the reference's (computed from the same initial particles)."""
    run = golden_json("inp_runs.json")[name]
    props, parts, counts = init_inp(run)
    sim = gpu_sim(props, reference_config())
    sim.upload_particles(parts, counts)
    sim.step(run["ncycles"])
    got = sim.cell_counts()
    assert got.tolist() == run["final_counts"]


@pytest.mark.parametrize("name", ["test", "tiny"])
def test_inp_conserved_trace(name, tmp_path):
    """The trace of the reference's debug build (conserved quantities before
    every cycle, simulator.h:65-90) from the device's reductions: total
    momentum and kinetic energy per cycle against the reference's, to 1e-12
    relative, and the written file in the reference's format."""
    from allscale_ipic3d_gb300 import trace_text
    run = golden_json("inp_runs.json")[name]
    props, parts, counts = init_inp(run)
    sim = gpu_sim(props, reference_config(flags=abi.F_USE_GRAPH))
    sim.upload_particles(parts, counts)
    path = str(tmp_path / (name + "ConservedQuantities.out"))
    rows = sim.conserved_trace(run["ncycles"], path=path)
    assert [r[0] for r in rows] == [r[0] for r in run["trace"]]
    for got, ref in zip(rows, run["trace"]):
        for col in (1, 4):
            assert abs(got[col] - ref[col]) <= 1e-12 * abs(ref[col]), (got[0], col, got[col], ref[col])
            assert "%g" % got[col] == "%g" % ref[col], (got[0], col)
    assert open(path).read() == trace_text(rows)
    assert sim.cell_counts().tolist() == run["final_counts"]


@pytest.mark.parametrize("graph", [False, True])
def test_inp_steps_one_at_a_time_and_graph(graph):
    run = golden_json("inp_runs.json")["test"]
    props, parts, counts = init_inp(run)
    sim = gpu_sim(props, reference_config(flags=abi.F_USE_GRAPH if graph else 0))
    sim.upload_particles(parts, counts)
    for _ in range(run["ncycles"]):
        sim.step(1)
    assert sim.cell_counts().tolist() == run["final_counts"]


@pytest.mark.parametrize("name", ["p3", "p435"])
def test_projection(name):
    g = golden_npz("project_small.npz")
    props = props_from_vec(g[name + "_props"])
    sim = gpu_sim(props, abi.Config.make(projector=abi.PROJECT_CIC, flags=abi.F_J_DIV8))
    sim.upload_particles(g[name + "_in"], g[name + "_in_counts"])
    sim.project()
    _, _, J, _ = sim.download_fields()
    np.testing.assert_allclose(J, g[name + "_J"], rtol=1e-12, atol=1e-14 * np.abs(g[name + "_J"]).max())


def test_boundaries_and_leapfrog_bit_exact():
    g = golden_npz("fields_small.npz")
    props = props_from_vec(g["props"])
    sim = gpu_sim(props, abi.Config.make(solver=abi.SOLVER_LEAPFROG))
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


def test_forward_solver_matches_oracle():
    g = golden_npz("fields_small.npz")
    props = props_from_vec(g["props"])
    cfg = abi.Config.make(solver=abi.SOLVER_FORWARD)
    sim, orc = gpu_sim(props, cfg), OracleSim(props, cfg)
    for s in (sim, orc):
        s.upload_fields(g["field"], g["bcfield"], g["J"])
        s.solve_fields()
    (f1, b1, _, _), (f2, b2, _, _) = sim.download_fields(), orc.download_fields()
    assert f1.tobytes() == f2.tobytes()
    assert b1.tobytes() == b2.tobytes()
    for k, nd in enumerate(g["fw_nodes"]):  # E at a node equals the reference's per-node call
        x, y, z = nd
        assert f1[x, y, z, 0:3].tobytes() == g["fw_field"][k][x, y, z, 0:3].tobytes()


def pic_config(precision, bc=abi.BC_PERIODIC, **kw):
    base = dict(precision=precision, mover=abi.MOVER_FIELD, solver=abi.SOLVER_LEAPFROG, projector=abi.PROJECT_CIC,
                bc=bc, flags=abi.F_REFRESH_NODE_B | abi.F_TRACK_IDS)
    base.update(kw)
    return abi.Config.make(**base)


def uniform_fields(props, E, B):
    f = np.zeros(abi.field_shape(props))
    f[..., 0:3] = E
    f[..., 3:6] = B
    bc = np.zeros(abi.bcfield_shape(props))
    bc[..., :] = B
    return f, bc


@pytest.mark.parametrize("seed,size,bc", [(31, (4, 4, 4), abi.BC_PERIODIC), (32, (6, 6, 6), abi.BC_REFLECT),
                                          (33, (5, 5, 5), abi.BC_OPEN)])
def test_pic_step_fp64_matches_oracle(seed, size, bc):
    """The designed full step (simulator.h:189-223): CIC deposit, ghost copy,
    leapfrog, field-gather mover, export, import."""
    props, parts, counts = scenario(seed, size, dt=0.1, ppc=12, vscale=0.2, species=((-1.0, -1.0), (1.0, 0.01)),
                                    ragged=True)
    f, bcf = uniform_fields(props, (0.0, 0.01, 0.0), (0.0, 0.0, 0.1))
    cfg = pic_config(abi.FP64, bc=bc)
    sim, orc = gpu_sim(props, cfg), OracleSim(props, cfg)
    for s in (sim, orc):
        s.upload_fields(f, bcf, None)
        s.upload_particles(parts, counts)
        s.step(6)
    a, b = align_by_id(sim.download_particles(), orc.download_particles())
    assert_states_close(a, b, rtol=1e-9, atol=1e-11, what="pic fp64")
    (f1, b1, _, _), (f2, b2, _, _) = sim.download_fields(), orc.download_fields()
    np.testing.assert_allclose(f1, f2, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(b1, b2, rtol=1e-9, atol=1e-12)
    # after a step the GPU's J/rho are the projection of the current particles
    # (fused into the push for the next step); the oracle projects on demand
    orc.project()
    _, _, j1, r1 = sim.download_fields()
    _, _, j2, r2 = orc.download_fields()
    np.testing.assert_allclose(j1, j2, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(r1, r2, rtol=1e-9, atol=1e-12)


def test_pic_step_fp32_error_vs_fp64_oracle():
    """FP32 cell-relative push and deposit against the FP64 oracle: conserved
    energy within 1e-5 relative, positions within 1e-4 cell widths."""
    # neutral electron-ion plasma, unit density (omega_p dt = 0.1)
    props, parts, counts = scenario(41, (8, 8, 8), dt=0.1, ppc=64, vscale=0.01,
                                    species=((-1.0 / 32, -1.0), (1.0 / 32, 0.01)))
    f, bcf = uniform_fields(props, (0.0, 0.01, 0.0), (0.0, 0.0, 0.1))
    sim = gpu_sim(props, pic_config(abi.FP32))
    orc = OracleSim(props, pic_config(abi.FP64))
    for s in (sim, orc):
        s.upload_fields(f, bcf, None)
        s.upload_particles(parts, counts)
        s.step(20)
    c1, c2 = sim.conserved(), orc.conserved()
    assert c1["particles"] == c2["particles"]
    assert abs(c1["kinetic_energy"] - c2["kinetic_energy"]) <= 1e-5 * abs(c2["kinetic_energy"])
    assert abs(c1["e_energy"] - c2["e_energy"]) <= 1e-5 * abs(c2["e_energy"]) + 1e-12
    pa, ca, ia = sim.download_particles()
    pb, cb, ib = orc.download_particles()
    ka, kb = np.argsort(ia), np.argsort(ib)
    np.testing.assert_array_equal(ia[ka], ib[kb])
    d = np.abs(pa["position"][ka] - pb["position"][kb]).max()
    assert d < 1e-4, d


def test_injection_and_outflow_fp64_matches_oracle():
    props, parts, counts = scenario(51, (6, 6, 6), dt=0.1, ppc=10, vscale=0.05, species=((-1.0, -1.0),))
    cfg = pic_config(abi.FP64, bc_low=[abi.BC_OPEN, abi.BC_PERIODIC, abi.BC_PERIODIC],
                     bc_high=[abi.BC_OPEN, abi.BC_PERIODIC, abi.BC_PERIODIC],
                     flags=abi.F_REFRESH_NODE_B | abi.F_TRACK_IDS | abi.F_INJECT_LOW_X, inject_per_cell=2.5,
                     inject_q=-1.0, inject_qom=-1.0, inject_drift=(0.3, 0.0, 0.0), inject_vth=(0.05, 0.05, 0.05))
    sim, orc = gpu_sim(props, cfg), OracleSim(props, cfg)
    for s in (sim, orc):
        s.upload_particles(parts, counts)
        s.step(8)
    np.testing.assert_array_equal(sim.cell_counts(), orc.cell_counts())
    c1, c2 = sim.conserved(), orc.conserved()
    assert c1["particles"] == c2["particles"]
    np.testing.assert_allclose(c1["kinetic_energy"], c2["kinetic_energy"], rtol=1e-10)


def test_overflowing_cell_goes_through_pending_and_rebuild():
    """All particles of a 3^3 grid converge on one cell: far more arrivals
    than the cell's slack; the pending path and the re-layout keep every
    particle (counts equal the oracle's)."""
    props = abi.Props.make(size=(3, 3, 3), dt=1.0)
    rng = np.random.default_rng(7)
    n_per = 40
    cells = np.repeat(np.arange(27), n_per)
    cz, cy, cx = cells % 3, (cells // 3) % 3, cells // 9
    pos = np.stack([cx, cy, cz], 1) + 0.5 + rng.uniform(-0.1, 0.1, (len(cells), 3))
    parts = np.zeros(len(cells), abi.PARTICLE_DTYPE)
    parts["position"] = pos
    parts["velocity"] = (1.5 - pos) * 1.0  # every particle aims at the centre cell
    parts["q"] = 1.0
    parts["qom"] = 1.0
    counts = np.full(27, n_per, np.uint64)
    cfg = reference_config(flags=abi.F_TRACK_IDS, slack=0.1, slack_min=4)
    sim, orc = gpu_sim(props, cfg), OracleSim(props, reference_config())
    for s in (sim, orc):
        s.upload_particles(parts, counts)
        s.step(1)
    np.testing.assert_array_equal(sim.cell_counts(), orc.cell_counts())
    assert sim.stats()["rebuilds"] >= 1
    a, b = align_by_id(sim.download_particles(), orc.download_particles())
    assert_states_close(a, b, rtol=1e-12, atol=1e-13)
    for s in (sim, orc):  # and the next step from the re-laid-out storage
        s.step(2)
    a, b = align_by_id(sim.download_particles(), orc.download_particles())
    assert_states_close(a, b, rtol=1e-12, atol=1e-13)


def test_empty_universe_and_empty_cells():
    props = abi.Props.make(size=(3, 2, 4), dt=0.1)
    sim = gpu_sim(props, reference_config())
    sim.step(3)
    assert sim.cell_counts().sum() == 0
    c = sim.conserved()
    assert c["particles"] == 0 and c["kinetic_energy"] == 0.0


def test_particle_at_dipole_centre_with_zero_radius():
    """planetRadius = 0 and a particle exactly at the origin: 0/0 gives a NaN
    field, the reference's x86 build runs no sub-cycle (cell.h:950), and the
    planet rule r^2 <= R^2 (cell.h:1126) then removes the particle. Another
    particle free-streams."""
    props = abi.Props.make(size=(2, 2, 2), origin=(-1.0, -1.0, -1.0), dt=0.1)
    parts = np.zeros(2, abi.PARTICLE_DTYPE)
    parts["position"] = [(0.0, 0.0, 0.0), (0.5, 0.5, 0.5)]
    parts["velocity"] = [(1.0, 1.0, 1.0), (0.2, 0.0, 0.0)]
    parts["q"] = parts["qom"] = 1.0
    counts = np.zeros(8, np.uint64)
    counts[7] = 2  # both in cell (1,1,1) = [0,1)^3
    sim, orc = gpu_sim(props, reference_config(flags=abi.F_TRACK_IDS)), OracleSim(props, reference_config())
    for s in (sim, orc):
        s.upload_particles(parts, counts)
        s.step(1)
    a, b = align_by_id(sim.download_particles(), orc.download_particles())
    assert len(a) == 1
    np.testing.assert_allclose(a["position"][0], [0.52, 0.5, 0.5], rtol=0, atol=1e-15)
    assert_states_close(a, b, rtol=0, atol=0)


def test_conserved_quantities_match_oracle():
    props, parts, counts = scenario(61, (5, 5, 5), dt=0.1, ppc=20, vscale=0.3, species=((1.0, 1.0), (-1.0, -5.0)))
    f = np.random.default_rng(2).normal(0, 1, abi.field_shape(props))
    sim, orc = gpu_sim(props, reference_config()), OracleSim(props, reference_config())
    for s in (sim, orc):
        s.upload_particles(parts, counts)
        s.upload_fields(f, None, None)
    c1, c2 = sim.conserved(), orc.conserved()
    for k in ("total_momentum", "kinetic_energy", "total_charge", "e_energy", "b_energy"):
        np.testing.assert_allclose(c1[k], c2[k], rtol=1e-12, err_msg=k)
    assert c1["particles"] == c2["particles"] == len(parts)


def test_conserved_quantities_count_waiting_particles():
    """Arrivals beyond a cell's slots wait in the pending list (below the
    re-layout threshold of 64 here): the conserved sums and per-cell counts
    still include them, equal to the oracle's."""
    props = abi.Props.make(size=(3, 3, 3), dt=1.0)
    rng = np.random.default_rng(8)
    cells = np.repeat([0, 2, 6, 8], 6)  # 24 particles in 4 corner cells of the x=0 plane
    cz, cy, cx = cells % 3, (cells // 3) % 3, cells // 9
    pos = np.stack([cx, cy, cz], 1) + 0.5 + rng.uniform(-0.1, 0.1, (len(cells), 3))
    parts = np.zeros(len(cells), abi.PARTICLE_DTYPE)
    parts["position"] = pos
    parts["velocity"] = np.array([1.0, 1.5, 1.5]) - pos + np.array([0.0, 0.0, 0.0])  # all aim at cell (0,1,1)
    parts["velocity"][:, 0] = 0.0
    parts["q"] = 1.0
    parts["qom"] = 1.0
    counts = np.bincount(cells, minlength=27).astype(np.uint64)
    cfg = reference_config(flags=abi.F_TRACK_IDS, slack=0.01, slack_min=4)
    sim, orc = gpu_sim(props, cfg), OracleSim(props, reference_config())
    for s in (sim, orc):
        s.upload_particles(parts, counts)
        s.step(1)
    st = sim.stats()
    assert st["pending_last"] > 0 and st["rebuilds"] == 0, st
    np.testing.assert_array_equal(sim.cell_counts(), orc.cell_counts())
    c1, c2 = sim.conserved(), orc.conserved()
    for k in ("total_momentum", "kinetic_energy", "total_charge"):
        np.testing.assert_allclose(c1[k], c2[k], rtol=1e-12, err_msg=k)
    assert c1["particles"] == c2["particles"] == len(parts)


@pytest.mark.parametrize("precision,graph", [(abi.FP64, False), (abi.FP64, True), (abi.FP32, True)])
def test_heavy_migration_placement(precision, graph):
    """Ballistic particles (no field) in a 5^3 periodic grid, 48 per cell
    with velocities up to 0.45 cells per step: about 40 % of the particles
    change cell every step, so cells take dozens of holes and arrivals at
    once (several rounds of the placement's lane groups, tail compaction,
    long hole sorts). Per-cell counts and ids bit-exact against the oracle
    every step; states within the precision's tolerance."""
    props, parts, counts = scenario(9100, (5, 5, 5), dt=1.0, ppc=48, vscale=0.0)
    rng = np.random.default_rng(9101)
    parts["velocity"] = rng.uniform(-0.45, 0.45, (len(parts), 3))
    flags = abi.F_TRACK_IDS | (abi.F_USE_GRAPH if graph else 0)
    kw = dict(mover=abi.MOVER_DIPOLE, bc=abi.BC_PERIODIC)
    sim = gpu_sim(props, abi.Config.make(precision=precision, flags=flags, **kw))
    orc = OracleSim(props, abi.Config.make(**kw))
    for s in (sim, orc):
        s.upload_particles(parts, counts)
    for _ in range(4):
        for s in (sim, orc):
            s.step(1)
        st = sim.stats()
        assert st["migrated_last"] > 0.3 * len(parts), st
        if precision == abi.FP64:
            a, b = align_by_id(sim.download_particles(), orc.download_particles())
            assert_states_close(a, b, rtol=1e-12, atol=1e-12, what="heavy migration")
        else:
            # FP32 may put a particle within rounding of a cell face on the
            # other side: match particles by id, positions modulo the domain
            (pa, ca, ia), (pb, cb, ib) = sim.download_particles(), orc.download_particles()
            assert ca.sum() == cb.sum() == len(parts)
            pa, pb = pa[np.argsort(ia)], pb[np.argsort(ib)]
            np.testing.assert_array_equal(np.sort(ia), np.sort(ib))
            d = (pa["position"] - pb["position"] + 2.5) % 5.0 - 2.5
            assert np.abs(d).max() < 1e-5, np.abs(d).max()
            np.testing.assert_allclose(pa["velocity"], pb["velocity"], rtol=0, atol=1e-6)
    sim.close()


@pytest.mark.parametrize("precision", [abi.FP64, abi.FP32])
def test_dumps_byte_identical_to_reference_writers(tmp_path, precision):
    """outputParticlePositions (cell.h:1400-1429) and outputFieldGrids
    (field.h:464-530) from the device: the positions packed on the device (24
    bytes per particle over the link) and the grids, written in the
    reference's text format, equal the reference's own writers' files
    (fixture from the compiled reference) byte for byte. FP32 storage keeps
    positions cell-relative; printed at 6 significant digits they agree with
    the FP64 ones except where FP32 rounding crosses a printed digit. The
    universe has one species: the device keeps a cell's particles of one
    species in upload order (particles of different species are grouped by
    species within a cell, so the reference's writer on a mixed-species cell
    prints the same lines in another order)."""
    g = golden_npz("dumps_small.npz")
    props = props_from_vec(g["props"])
    sim = gpu_sim(props, abi.Config.make(precision=precision))
    sim.upload_fields(g["field"], g["bcfield"], None)
    sim.upload_particles(g["parts"], g["counts"])
    xyz, c = sim.download_positions()
    np.testing.assert_array_equal(c, g["counts"])
    if precision == abi.FP64:
        np.testing.assert_array_equal(xyz, g["parts"]["position"])
    pos = tmp_path / "positions.txt"
    grids = tmp_path / "fields.txt"
    sim.write_particle_positions(str(pos))
    sim.write_field_grids(str(grids))
    want_pos = bytes(g["positions_txt"])
    got_pos = pos.read_bytes()
    if precision == abi.FP64:
        assert got_pos == want_pos
    else:
        a, b = got_pos.decode().split("\n"), want_pos.decode().split("\n")
        assert len(a) == len(b)
        np.testing.assert_allclose(np.array([list(map(float, l.split())) for l in a if l]),
                                   np.array([list(map(float, l.split())) for l in b if l]), rtol=1e-5)
    assert grids.read_bytes() == bytes(g["field_grids_txt"])
    sim.close()


def test_async_download_overlaps_an_upload():
    """ipic3d_gpu_download_particles_async: the counts at once, the particles
    after ipic3d_gpu_download_wait, equal to the synchronous download of the
    same state even when an upload of other particles runs in between (the
    copies use separate staging buffers and streams)."""
    props, parts, counts = scenario(91, (6, 5, 4), dt=0.1, ppc=20, vscale=0.3, species=((1.0, 1.0), (-1.0, -2.0)),
                                    ragged=True)
    _, parts2, counts2 = scenario(92, (6, 5, 4), dt=0.1, ppc=12, vscale=0.3, species=((1.0, 1.0), (-1.0, -2.0)))
    cfg = abi.Config.make(precision=abi.FP32, mover=abi.MOVER_FIELD, projector=abi.PROJECT_CIC, bc=abi.BC_PERIODIC)
    sim = gpu_sim(props, cfg)
    sim.upload_particles(parts, counts)
    sim.step(3)
    want, want_c, _ = sim.download_particles(ids=False)
    out = np.zeros(len(want) + 10, abi.PARTICLE_DTYPE)
    oc = np.zeros(props.ncells, np.uint64)
    n = sim.download_particles_async((out, oc))
    assert n == len(want)
    np.testing.assert_array_equal(oc, want_c)
    sim.upload_particles(parts2, counts2)  # runs while the copies are in flight
    sim.download_wait()
    assert out[:n].tobytes() == want.tobytes()
    got, got_c, _ = sim.download_particles(ids=False)
    np.testing.assert_array_equal(got_c, counts2)
    sim.step(2)
    sim.download_particles_async((out, oc))
    sim.close()  # waits for the copies in flight

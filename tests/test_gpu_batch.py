"""The batched ensemble (ipic3d_gpu_batch_*): universes of different sizes
advanced by one launch per kernel must give, universe by universe, what the
single-universe path gives (bit-identical particle states where the step has
no floating-point atomics in its data flow) and what the CPU oracle gives."""
import ctypes as C

import numpy as np
import pytest

from allscale_ipic3d_gb300 import Batch, Simulation, abi, library
from common import OracleSim, align_by_id, assert_states_close, scenario

pytestmark = pytest.mark.gpu


def uniform_fields(props, E, B):
    f = np.zeros(abi.field_shape(props))
    f[..., 0:3] = E
    f[..., 3:6] = B
    bc = np.zeros(abi.bcfield_shape(props))
    bc[..., :] = B
    return f, bc


def ensemble(sizes, seed0=500, ppc=12, species=((-1.0, -1.0),), ragged=True, vscale=0.2):
    """Per universe: props, particles, counts and uniform E, B drawn from the
    seed (|B| in [0.02, 0.2] in a random direction, |E| <= 0.02)."""
    out = []
    for i, size in enumerate(sizes):
        props, parts, counts = scenario(seed0 + i, size, dt=0.1, ppc=ppc, vscale=vscale, species=species,
                                        ragged=ragged)
        rng = np.random.default_rng(seed0 + 1000 + i)
        d = rng.normal(size=3)
        B = d / np.linalg.norm(d) * rng.uniform(0.02, 0.2)
        e = rng.normal(size=3)
        E = e / np.linalg.norm(e) * rng.uniform(0.0, 0.02)
        out.append((props, parts, counts, uniform_fields(props, E, B)))
    return out


def load(sim, u):
    props, parts, counts, (f, bc) = u
    sim.upload_fields(f, bc, None)
    sim.upload_particles(parts, counts)


STATIC = dict(mover=abi.MOVER_FIELD, solver=abi.SOLVER_STATIC, projector=abi.PROJECT_CIC, bc=abi.BC_PERIODIC,
              flags=abi.F_TRACK_IDS)
SIZES = [(4, 4, 4), (6, 6, 6), (5, 3, 4), (8, 8, 8), (3, 3, 3)]


@pytest.mark.parametrize("precision", [abi.FP64, abi.FP32])
def test_batch_equals_single_universes(precision):
    """Field mover with static fields: every particle's arithmetic is the
    single-universe kernel's, so states and counts are bit-identical. J/rho
    come from FP64 atomics (summation order free): FP64 agrees to 1e-12; the
    FP32 path first sums the particles of a warp in FP32, and which particles
    share a warp depends on the arrival order of migrants (atomics), so FP32
    agrees to FP32 rounding of the largest node value."""
    us = ensemble(SIZES)
    cfg = abi.Config.make(precision=precision, **STATIC)
    with Batch([u[0] for u in us], cfg) as batch:
        for i, u in enumerate(us):
            load(batch.universe(i), u)
        batch.step(15)
        for i, u in enumerate(us):
            single = Simulation(u[0], cfg)
            load(single, u)
            single.step(15)
            pa, ca, ia = batch.universe(i).download_particles()
            pb, cb, ib = single.download_particles()
            a, b = align_by_id((pa, ca, ia), (pb, cb, ib))
            assert_states_close(a, b, rtol=0, atol=0, what="universe %d" % i)
            _, _, j1, r1 = batch.universe(i).download_fields()
            _, _, j2, r2 = single.download_fields()
            tol = 1e-12 if precision == abi.FP64 else 1e-6
            np.testing.assert_allclose(j1, j2, rtol=tol, atol=tol * max(np.abs(j2).max(), 1e-300))
            np.testing.assert_allclose(r1, r2, rtol=tol, atol=tol * max(np.abs(r2).max(), 1e-300))
            single.close()
        st = batch.stats()
        assert st["steps"] == 15
        assert st["particles"] == sum(int(u[2].sum()) for u in us)


def test_batch_fp64_matches_oracle_static_fields():
    us = ensemble(SIZES[:3], seed0=610)
    cfg = abi.Config.make(precision=abi.FP64, **STATIC)
    with Batch([u[0] for u in us], cfg) as batch:
        for i, u in enumerate(us):
            load(batch.universe(i), u)
        batch.step(10)
        for i, u in enumerate(us):
            orc = OracleSim(u[0], cfg)
            load(orc, u)
            orc.step(10)
            a, b = align_by_id(batch.universe(i).download_particles(), orc.download_particles())
            assert_states_close(a, b, rtol=1e-10, atol=1e-12, what="universe %d" % i)
            orc.project()
            _, _, j1, r1 = batch.universe(i).download_fields()
            _, _, j2, r2 = orc.download_fields()
            np.testing.assert_allclose(j1, j2, rtol=1e-10, atol=1e-12 * max(np.abs(j2).max(), 1e-300))
            np.testing.assert_allclose(r1, r2, rtol=1e-10, atol=1e-12 * max(np.abs(r2).max(), 1e-300))


def test_batch_leapfrog_fp64_matches_oracle():
    """Self-consistent fields (ghost copy + leapfrog + node B refresh) per
    universe, neutral two-species plasma, cubic grids of three sizes."""
    us = ensemble([(4, 4, 4), (6, 6, 6), (5, 5, 5)], seed0=700, species=((-1.0 / 12, -1.0), (1.0 / 12, 0.01)))
    cfg = abi.Config.make(precision=abi.FP64, mover=abi.MOVER_FIELD, solver=abi.SOLVER_LEAPFROG,
                          projector=abi.PROJECT_CIC, bc=abi.BC_PERIODIC,
                          flags=abi.F_REFRESH_NODE_B | abi.F_TRACK_IDS)
    with Batch([u[0] for u in us], cfg) as batch:
        for i, u in enumerate(us):
            load(batch.universe(i), u)
        batch.step(6)
        for i, u in enumerate(us):
            orc = OracleSim(u[0], cfg)
            load(orc, u)
            orc.step(6)
            a, b = align_by_id(batch.universe(i).download_particles(), orc.download_particles())
            assert_states_close(a, b, rtol=1e-9, atol=1e-11, what="universe %d" % i)
            (f1, b1, _, _), (f2, b2, _, _) = batch.universe(i).download_fields(), orc.download_fields()
            np.testing.assert_allclose(f1, f2, rtol=1e-9, atol=1e-12)
            np.testing.assert_allclose(b1, b2, rtol=1e-9, atol=1e-12)


def test_batch_fp32_energy_against_fp64():
    """FP32 batched form against the FP64 batched form: kinetic energy of
    every universe within 1e-5 relative after 100 steps."""
    us = ensemble(SIZES, seed0=800, ragged=False, vscale=0.01)
    kw = dict(STATIC)
    out = {}
    for prec in (abi.FP32, abi.FP64):
        with Batch([u[0] for u in us], abi.Config.make(precision=prec, **kw)) as batch:
            for i, u in enumerate(us):
                load(batch.universe(i), u)
            batch.step(100)
            out[prec] = [batch.universe(i).conserved() for i in range(len(us))]
    for c32, c64 in zip(out[abi.FP32], out[abi.FP64]):
        assert c32["particles"] == c64["particles"]
        assert abs(c32["kinetic_energy"] - c64["kinetic_energy"]) <= 1e-5 * abs(c64["kinetic_energy"])


def test_batch_graph_equals_eager():
    us = ensemble(SIZES[:4], seed0=900)
    res = []
    for flags in (abi.F_TRACK_IDS, abi.F_TRACK_IDS | abi.F_USE_GRAPH):
        cfg = abi.Config.make(precision=abi.FP32, **dict(STATIC, flags=flags))
        with Batch([u[0] for u in us], cfg) as batch:
            for i, u in enumerate(us):
                load(batch.universe(i), u)
            batch.step(7)
            batch.step(5)
            res.append([batch.universe(i).download_particles() for i in range(len(us))])
    for x, y in zip(*res):
        a, b = align_by_id(x, y)
        assert_states_close(a, b, rtol=0, atol=0)


def test_batch_overflow_relayout_matches_single():
    """Universe 1 sends every particle of its x=0 plane into the empty x=1
    plane (far beyond the cells' slack): the pending path and the re-layout
    of that universe inside the batch keep every particle, as the single
    context does; the other universes are untouched by it."""
    us = ensemble([(4, 4, 4), (6, 6, 6)], seed0=950)
    props = abi.Props.make(size=(6, 4, 4), dt=1.0)
    nc = 6 * 4 * 4
    per = np.zeros(nc, np.int64)
    per[:16] = 40  # cells with x = 0
    cells = np.repeat(np.arange(nc), per)
    rng = np.random.default_rng(3)
    pos = np.stack([cells // 16, (cells // 4) % 4, cells % 4], 1) + 0.3 + 0.4 * rng.random((len(cells), 3))
    parts = np.zeros(len(cells), abi.PARTICLE_DTYPE)
    parts["position"] = pos
    parts["velocity"] = [1.0, 0.0, 0.0]
    parts["q"] = -1.0
    parts["qom"] = -1.0
    f, bc = uniform_fields(props, (0.0, 0.0, 0.0), (0.0, 0.0, 0.0))
    us.insert(1, (props, parts, per.astype(np.uint64), (f, bc)))
    cfg = abi.Config.make(precision=abi.FP64, **dict(STATIC, slack=0.1, slack_min=4))
    with Batch([u[0] for u in us], cfg) as batch:
        for i, u in enumerate(us):
            load(batch.universe(i), u)
        batch.step(3)
        assert batch.universe(1).stats()["rebuilds"] >= 1
        for i, u in enumerate(us):
            single = Simulation(u[0], cfg)
            load(single, u)
            single.step(3)
            a, b = align_by_id(batch.universe(i).download_particles(), single.download_particles())
            assert_states_close(a, b, rtol=0, atol=0, what="universe %d" % i)
            single.close()
        assert batch.universe(1).particle_count() == len(parts)


def test_batch_reference_dipole_universes():
    """The reference's own loop (dipole mover, reflecting walls, planet
    removal) for two universes in a batch equals the single path."""
    sizes = [(4, 4, 4), (6, 6, 6)]
    cfg = abi.Config.make(flags=abi.F_TRACK_IDS)
    us = []
    for i, s in enumerate(sizes):
        props, parts, counts = scenario(60 + i, s, width=(10.0, 10.0, 10.0),
                                        origin=tuple(-5.0 * x for x in s), dt=0.15, ppc=10, vscale=0.2,
                                        planet=4.0, bz=1e-4)
        us.append((props, parts, counts))
    with Batch([u[0] for u in us], cfg) as batch:
        for i, (props, parts, counts) in enumerate(us):
            batch.universe(i).upload_particles(parts, counts)
        batch.step(4)
        for i, (props, parts, counts) in enumerate(us):
            single = Simulation(props, cfg)
            single.upload_particles(parts, counts)
            single.step(4)
            a, b = align_by_id(batch.universe(i).download_particles(), single.download_particles())
            assert_states_close(a, b, rtol=0, atol=0, what="universe %d" % i)
            single.close()


def test_batch_empty_universes_and_lent_contexts():
    props = [abi.Props.make(size=(3, 3, 3), dt=0.1), abi.Props.make(size=(2, 5, 3), dt=0.1)]
    cfg = abi.Config.make(precision=abi.FP32, **STATIC)
    with Batch(props, cfg) as batch:
        batch.step(3)
        assert batch.stats()["particles"] == 0
        ctx = C.c_void_p()
        lib = library()
        assert lib.ipic3d_gpu_batch_universe(batch._b, 0, C.byref(ctx)) == 0
        assert lib.ipic3d_gpu_destroy(ctx) == abi.E_STATE
        assert lib.ipic3d_gpu_batch_universe(batch._b, 2, C.byref(ctx)) == abi.E_INVALID
        n = C.c_uint32()
        assert lib.ipic3d_gpu_batch_size(batch._b, C.byref(n)) == 0 and n.value == 2


def test_batch_forward_fp64_matches_oracle():
    """The forward solver (forward E, forward B, node B refresh) per universe
    in the batched form against the oracle."""
    us = ensemble([(4, 4, 4), (6, 6, 6)], seed0=720, species=((-1.0 / 12, -1.0), (1.0 / 12, 0.01)))
    cfg = abi.Config.make(precision=abi.FP64, mover=abi.MOVER_FIELD, solver=abi.SOLVER_FORWARD,
                          projector=abi.PROJECT_CIC, bc=abi.BC_PERIODIC, flags=abi.F_TRACK_IDS)
    with Batch([u[0] for u in us], cfg) as batch:
        for i, u in enumerate(us):
            load(batch.universe(i), u)
        batch.step(5)
        for i, u in enumerate(us):
            orc = OracleSim(u[0], cfg)
            load(orc, u)
            orc.step(5)
            a, b = align_by_id(batch.universe(i).download_particles(), orc.download_particles())
            assert_states_close(a, b, rtol=1e-9, atol=1e-11, what="universe %d" % i)
            (f1, b1, _, _), (f2, b2, _, _) = batch.universe(i).download_fields(), orc.download_fields()
            np.testing.assert_allclose(f1, f2, rtol=1e-9, atol=1e-12)
            np.testing.assert_allclose(b1, b2, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("solver", [abi.SOLVER_LEAPFROG, abi.SOLVER_FORWARD])
def test_batch_fp32_self_consistent_fields_against_oracle(solver):
    """FP32 batched form with self-consistent fields (the cell polynomials
    rebuilt from the solved fields every step) against the FP64 oracle:
    every particle within 1e-4 cell widths, kinetic energy within 1e-5."""
    us = ensemble([(4, 4, 4), (6, 6, 6)], seed0=740, ppc=16, vscale=0.01,
                  species=((-1.0 / 16, -1.0), (1.0 / 16, 0.01)))
    flags = abi.F_TRACK_IDS | (abi.F_REFRESH_NODE_B if solver == abi.SOLVER_LEAPFROG else 0)
    kw = dict(mover=abi.MOVER_FIELD, solver=solver, projector=abi.PROJECT_CIC, bc=abi.BC_PERIODIC, flags=flags)
    with Batch([u[0] for u in us], abi.Config.make(precision=abi.FP32, **kw)) as batch:
        for i, u in enumerate(us):
            load(batch.universe(i), u)
        batch.step(10)
        for i, u in enumerate(us):
            orc = OracleSim(u[0], abi.Config.make(precision=abi.FP64, **kw))
            load(orc, u)
            orc.step(10)
            c1, c2 = batch.universe(i).conserved(), orc.conserved()
            assert c1["particles"] == c2["particles"]
            assert abs(c1["kinetic_energy"] - c2["kinetic_energy"]) <= 1e-5 * abs(c2["kinetic_energy"])
            # matched by id (an FP32 rounding may carry a particle across a face)
            pa, _, ia = batch.universe(i).download_particles()
            pb, _, ib = orc.download_particles()
            ka, kb = np.argsort(ia), np.argsort(ib)
            np.testing.assert_array_equal(ia[ka], ib[kb])
            d = np.abs(pa["position"][ka] - pb["position"][kb]).max()
            assert d < 1e-4, (i, d)

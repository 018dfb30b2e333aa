"""The launch-shape autotuner of the FP32 push: it converges, caches its
choice per workload, and no shape changes a particle's result (every shape
runs the same per-particle arithmetic; only the split of the tiles into
work and the persistent grid differ)."""
import numpy as np
import pytest

from allscale_ipic3d_gb300 import Batch, abi
from common import align_by_id, assert_states_close, gpu_sim, scenario

pytestmark = pytest.mark.gpu

ITEMS = {128, 256, 512, 1024}
ITEM_CELLS = {0, 8, 16, 32}
# warm-up step + item phase (4 shapes) + item-cells phase (4) + blocks-per-SM
# phase (2), each shape timed twice
FULL_PASS_STEPS = 1 + 2 * (4 + 4 + 2)


def dipole_case(seed, n, ppc):
    props, parts, counts = scenario(seed, (n, n, n), width=(0.5, 0.5, 0.5), origin=(-n / 4, -n / 4, -n / 4),
                                    dt=0.05, ppc=ppc, vscale=0.2, planet=0.6, bz=0.5,
                                    species=((-1.0, -1.0), (1.0, 1.0 / 16)))
    return props, parts, counts


def field_case(seed, n, ppc):
    props, parts, counts = scenario(seed, (n, n, n), dt=0.1, ppc=ppc, vscale=0.1, ragged=True,
                                    species=((-1.0, -1.0), (1.0, 0.25)))
    f = np.zeros(abi.field_shape(props))
    f[..., 0:3] = (0.0, 0.01, 0.002)
    f[..., 3:6] = (0.02, 0.0, 0.1)
    bc = np.zeros(abi.bcfield_shape(props))
    bc[..., :] = (0.02, 0.0, 0.1)
    return props, parts, counts, f, bc


def test_autotuned_shape_keeps_particle_results():
    """Dipole mover, two species, reflecting walls and the planet: a context
    that tunes its shape over its first steps and one on the default shape
    end with the same particles in the same cells, state for state."""
    props, parts, counts = dipole_case(5101, 12, 96)
    kw = dict(precision=abi.FP32, flags=abi.F_TRACK_IDS | abi.F_USE_GRAPH)
    tuned = gpu_sim(props, abi.Config.make(block_size=0, **kw))
    fixed = gpu_sim(props, abi.Config.make(block_size=1, **kw))
    steps = FULL_PASS_STEPS + 9
    for s in (tuned, fixed):
        s.upload_particles(parts, counts)
        s.step(steps)
    sh = tuned.push_shape()
    assert sh["tuned"] == 1 and sh["tuning"] == 0, sh
    assert sh["trials"] == FULL_PASS_STEPS - 1, sh
    assert sh["item"] in ITEMS and sh["item_cells"] in ITEM_CELLS and sh["blocks_per_sm"] >= 1, sh
    assert sh["push_ms"] > 0, sh
    d = fixed.push_shape()
    assert (d["item"], d["item_cells"], d["tuned"], d["tuning"]) == (256, 32, 0, 0), d
    a, b = align_by_id(tuned.download_particles(), fixed.download_particles())
    assert_states_close(a, b, rtol=1e-6, atol=1e-6, what="tuned vs default shape")
    # the tuned context replays a graph after its trials, as the fixed one
    st = tuned.stats()
    assert st["steps"] == steps
    # a second context of the same workload takes the cached shape: no trials
    again = gpu_sim(props, abi.Config.make(block_size=0, **kw))
    again.upload_particles(parts, counts)
    again.step(1)
    s2 = again.push_shape()
    assert s2["tuned"] == 1 and s2["trials"] == 0 and s2["tuning"] == 0, s2
    assert (s2["item"], s2["item_cells"], s2["blocks_per_sm"]) == (sh["item"], sh["item_cells"],
                                                                  sh["blocks_per_sm"])
    # a restart runs the trials again
    again.set_push_shape()
    assert again.push_shape()["tuning"] == 1
    again.step(FULL_PASS_STEPS)
    s3 = again.push_shape()
    assert s3["tuned"] == 1 and s3["tuning"] == 0 and s3["trials"] == FULL_PASS_STEPS - 1, s3
    for s in (tuned, fixed, again):
        s.close()


@pytest.mark.parametrize("shape", [(256, 32, 2), (128, 0, 1), (1024, 32, 2), (32, 8, 1), (512, 16, 2)])
def test_fixed_shapes_agree(shape):
    """Field-gather mover with the deposit, periodic, ragged per-cell counts
    (0 to 2 ppc, a fifth of the cells empty) and dense cells: every fixed
    shape, including all tiles slot by slot (item_cells 0) and one-warp
    items (item 32), gives the default shape's particles and J."""
    props, parts, counts, f, bc = field_case(5202, 10, 48)
    kw = dict(precision=abi.FP32, mover=abi.MOVER_FIELD, projector=abi.PROJECT_CIC, bc=abi.BC_PERIODIC,
              flags=abi.F_TRACK_IDS)
    ref = gpu_sim(props, abi.Config.make(block_size=1, **kw))
    sim = gpu_sim(props, abi.Config.make(**kw))
    sim.set_push_shape(*shape)
    got = sim.push_shape()
    assert (got["item"], got["item_cells"], got["blocks_per_sm"], got["tuned"]) == shape + (0,), got
    for s in (ref, sim):
        s.upload_fields(f, bc, None)
        s.upload_particles(parts, counts)
        s.step(12)
    assert sim.push_shape()["tuning"] == 0
    a, b = align_by_id(sim.download_particles(), ref.download_particles())
    assert_states_close(a, b, rtol=1e-6, atol=1e-6, what="shape %s" % (shape,))
    # J and rho: per-item FP32 moment sums group the particles differently
    # under another item size, so they agree to FP32 rounding
    _, _, J1, r1 = sim.download_fields()
    _, _, J2, r2 = ref.download_fields()
    np.testing.assert_allclose(J1, J2, rtol=1e-5, atol=1e-6 * np.abs(J2).max())
    np.testing.assert_allclose(r1, r2, rtol=1e-5, atol=1e-6 * np.abs(r2).max())
    for s in (ref, sim):
        s.close()


def test_bad_shape_is_rejected():
    props, parts, counts = dipole_case(5303, 4, 8)
    sim = gpu_sim(props, abi.Config.make(precision=abi.FP32))
    for bad in ((0, 32, 2), (256, -1, 2), (256, 32, 0)):
        with pytest.raises(Exception):
            sim.set_push_shape(*bad)
    sim.close()


def test_batch_tunes_its_push():
    """A batch of universes of different sizes tunes the batched push's shape
    over its first steps; its particles match a batch on the default shape."""
    sizes = [6, 8, 10, 7]
    props, uploads = [], []
    for i, n in enumerate(sizes):
        p, parts, counts, f, bc = field_case(5400 + i, n, 24 + 8 * i)
        props.append(p)
        uploads.append((parts, counts, f, bc))
    kw = dict(precision=abi.FP32, mover=abi.MOVER_FIELD, projector=abi.PROJECT_CIC, bc=abi.BC_PERIODIC,
              flags=abi.F_TRACK_IDS | abi.F_USE_GRAPH)
    bt = Batch(props, abi.Config.make(block_size=0, **kw))
    bf = Batch(props, abi.Config.make(block_size=1, **kw))
    for b in (bt, bf):
        for i, (parts, counts, f, bc) in enumerate(uploads):
            b.universe(i).upload_fields(f, bc, None)
            b.universe(i).upload_particles(parts, counts)
        b.step(FULL_PASS_STEPS + 4)
    sh = bt.push_shape()
    assert sh["tuned"] == 1 and sh["tuning"] == 0 and sh["trials"] == FULL_PASS_STEPS - 1, sh
    assert bf.push_shape()["tuned"] == 0
    for i in range(len(sizes)):
        a, b = align_by_id(bt.universe(i).download_particles(), bf.universe(i).download_particles())
        assert_states_close(a, b, rtol=1e-6, atol=1e-6, what="universe %d" % i)
    bt.close()
    bf.close()

"""The GPU tracer (ipic3d_gpu_trace / ipic3d_gpu_trace_device,
traceParticle of pic_tracer.cxx:77-148) against the reference's own runs and
the oracle: histograms bit-identical (integer counts), on the reference's
configuration and on small-unit universes that exercise sub-cycling,
periodic wraps, planet hits, particles starting inside the planet or outside
the box and particles on the box's upper faces; at the benchmark's full size
(16M particles, 151 steps, 64^3 cells) through the linearity of the
histogram."""
import numpy as np
import pytest

import allscale_ipic3d_gb300 as ipg
from allscale_ipic3d_gb300 import abi, tracer
from test_tracer_oracle import CASES, oracle_particles, oracle_props, oracle_trace
from common import sha

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", CASES, ids=lambda c: "N%d_T%d_S%d_R%d" % (c["N"], c["T"], c["S"], c["R"]))
def test_trace_matches_reference_runs(case):
    props = tracer.tracer_props(case["R"])
    parts = oracle_particles(oracle_props(case["R"]), case["N"])
    counts = ipg.trace(props, parts, case["T"] + 1, case["S"], case["frames"])
    assert counts.sum(axis=(1, 2, 3)).tolist() == case["frame_totals"]
    assert sha(counts) == case["counts_sha256"]


def unit_universe(seed, size=(8, 9, 7), center=(0.0, 0.0, 0.0), bz=2.0):
    """A universe in units where the dipole is strong: |qom| |B|^2 large
    enough for many sub-cycles near the planet (radius 1, c = 1)."""
    w = (1.0, 0.75, 1.25)
    origin = tuple(center[a] - size[a] * w[a] / 2.0 for a in range(3))
    return abi.Props.make(size=size, cell_width=w, dt=0.05, speed_of_light=1.0, planet_radius=1.0,
                          object_center=center, origin=origin, external_b=(0.0, 0.0, bz))


def unit_particles(props, n, seed):
    """Positions over the box and a margin around it (some start outside or
    inside the planet), speeds up to a box width per few steps, q/m spread
    over two decades and of both signs; a few particles sit exactly on the
    box's upper faces with zero velocity."""
    rng = np.random.default_rng(seed)
    extent = np.array(props.cell_width) * np.array(props.size, dtype=np.float64)
    low = np.array(props.origin)
    p = np.zeros(n, abi.PARTICLE_DTYPE)
    # positions relative to the object centre (traceParticle adds it)
    p["position"] = low - np.array(props.object_center) + rng.uniform(-0.05, 1.05, (n, 3)) * extent
    p["velocity"] = rng.normal(0.0, 1.0, (n, 3)) * rng.choice([0.1, 1.0, 4.0], (n, 1))
    p["q"] = 1.0
    p["qom"] = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-1.0, 1.0, n)
    k = min(24, n // 4)
    for i in range(k):
        a = i % 3
        p["position"][i] = low - np.array(props.object_center) + rng.uniform(0.0, 1.0, 3) * extent
        p["position"][i, a] = (low[a] + extent[a]) - props.object_center[a]
        p["velocity"][i] = 0.0
    return p


UNIT_CASES = [  # (seed, grid, centre, Bz, particles, steps, frame interval)
    (1, (8, 9, 7), (0.0, 0.0, 0.0), 2.0, 20000, 60, 7),
    (2, (6, 6, 6), (0.5, -0.25, 1.0), 5.0, 15000, 41, 10),
    (3, (10, 4, 5), (0.0, 0.0, 0.0), 0.5, 12000, 33, 1),
    (4, (5, 5, 5), (0.0, 0.0, 0.0), 40.0, 5000, 25, 4),   # sub-cycles capped at 100 near the planet
]


@pytest.mark.parametrize("seed,size,center,bz,n,steps,interval", UNIT_CASES)
def test_trace_matches_oracle(seed, size, center, bz, n, steps, interval):
    props = unit_universe(seed, size, center, bz)
    parts = unit_particles(props, n, seed)
    frames = ipg.trace_frames(steps, interval)
    want = oracle_trace(props, parts, steps, interval, frames)
    got = ipg.trace(props, parts, steps, interval, frames)
    assert want.sum() > 0
    np.testing.assert_array_equal(got, want)


def test_trace_upper_face_aliasing_and_extra_frames():
    """Particles resting on the box's upper faces are counted at the
    reference's flat index (the next row, or the next frame); past the
    vector's end they are not counted."""
    props = unit_universe(5, (4, 4, 4), bz=0.0)
    extent = np.array(props.cell_width) * 4
    p = np.zeros(3, abi.PARTICLE_DTYPE)
    p["position"] = np.array(props.origin) + 0.3 * extent
    p["position"][0, 0] = props.origin[0] + extent[0]  # x on the upper face
    p["position"][1, 2] = props.origin[2] + extent[2]  # z on the upper face
    p["qom"] = 1.0
    totals = {}
    for frames in (3, 5):
        want = oracle_trace(props, p, 21, 10, frames)
        got = ipg.trace(props, p, 21, 10, frames)
        np.testing.assert_array_equal(got, want)
        totals[frames] = got.reshape(frames, -1).sum(axis=1).tolist()
    # steps 0, 10, 20 recorded: the x-face particle lands one frame later
    # (its frame-2 count falls off the 3-frame vector), the z-face particle
    # one row later in its own frame
    assert totals[3] == [2, 3, 3]
    assert totals[5] == [2, 3, 3, 1, 0]


def test_trace_device_entry_and_accumulation():
    torch = pytest.importorskip("torch")
    props = unit_universe(6)
    parts = unit_particles(props, 9000, 6)
    steps, interval = 40, 5
    frames = ipg.trace_frames(steps, interval)
    host = ipg.trace(props, parts, steps, interval)
    d_parts = torch.from_numpy(parts.view(np.uint8)).cuda()
    d_counts = torch.zeros(frames * props.ncells, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):  # the histogram accumulates
        ipg.trace_device(props, d_parts.data_ptr(), len(parts), steps, interval, frames, d_counts.data_ptr(), stream)
    torch.cuda.synchronize()
    got = d_counts.cpu().numpy().view(np.uint32).reshape(host.shape)
    np.testing.assert_array_equal(got, 2 * host)
    again = ipg.trace(props, parts, steps, interval, counts=host.copy())
    np.testing.assert_array_equal(again, 2 * host)


def test_trace_empty_and_errors():
    props = unit_universe(7)
    parts = unit_particles(props, 100, 7)
    assert ipg.trace(props, parts[:0], 10, 5).sum() == 0
    assert ipg.trace(props, parts, 0, 5, num_frames=0).size == 0
    with pytest.raises(ipg.GpuPathError) as e:
        ipg.trace(props, parts, 21, 10, num_frames=2)  # frame 2 would not fit
    assert e.value.status == abi.E_INVALID
    with pytest.raises(ipg.GpuPathError):
        ipg.trace(props, parts, 21, 0, num_frames=3)


def test_trace_reference_config_larger_sample():
    """pic_tracer's default configuration (64^3 cells, T = 150, S = 10) on
    200k particles of its stream against the oracle."""
    props = tracer.tracer_props(64)
    parts = oracle_particles(oracle_props(64), 200000, seed=7)
    want = oracle_trace(props, parts, 151, 10, 16)
    got = ipg.trace(props, parts, 151, 10, 16)
    np.testing.assert_array_equal(got, want)


def test_trace_full_size_linearity():
    """16M particles, 151 steps, 64^3 cells, 16 frames: the histogram of the
    whole set equals the sum of its halves' (each a separate launch), and
    every frame holds at most the particles."""
    torch = pytest.importorskip("torch")
    props = tracer.tracer_props(64)
    n = 16 * 1000 * 1000
    rng = np.random.default_rng(11)
    low, hig = tracer.particle_box(props)
    parts = np.zeros(n, abi.PARTICLE_DTYPE)
    parts["position"] = rng.uniform(low, hig, (n, 3))
    parts["velocity"] = rng.standard_normal((n, 3), dtype=np.float32) * tracer.speed_scale(props)
    parts["q"] = tracer.ELEMENTARY_CHARGE
    parts["qom"] = tracer.ELEMENTARY_CHARGE / tracer.PROTON_MASS
    d = torch.from_numpy(parts.view(np.uint8)).cuda()
    del parts
    cells, frames = props.ncells, 16
    whole = torch.zeros(frames * cells, dtype=torch.int32, device="cuda")
    halves = torch.zeros_like(whole)
    stream = torch.cuda.current_stream().cuda_stream
    ipg.trace_device(props, d.data_ptr(), n, 151, 10, frames, whole.data_ptr(), stream)
    h = n // 2
    ipg.trace_device(props, d.data_ptr(), h, 151, 10, frames, halves.data_ptr(), stream)
    ipg.trace_device(props, d.data_ptr() + h * 64, n - h, 151, 10, frames, halves.data_ptr(), stream)
    torch.cuda.synchronize()
    assert torch.equal(whole, halves)
    totals = whole.view(frames, cells).sum(dim=1).cpu().numpy()
    assert totals[0] > 0.99 * n and (totals <= n).all() and (np.diff(totals) <= 0).all()

"""The standalone tracer's oracle and host side against the reference's own
pic_tracer runs (tests/golden/tracer_runs.json, made by running
src/pic_tracer.cxx compiled from the reference sources): the configuration,
the particle stream, traceParticle's histograms and the result files."""
import ctypes as C
import hashlib

import numpy as np
import pytest

import oracle
from allscale_ipic3d_gb300 import abi
from allscale_ipic3d_gb300 import tracer
from common import golden_json, sha

CASES = golden_json("tracer_runs.json")


def oracle_props(R):
    p = abi.Props()
    assert oracle.load().oracle_tracer_config(R, C.byref(p)) == 0
    return p


def oracle_particles(props, n, seed=0):
    out = np.zeros(n, abi.PARTICLE_DTYPE)
    assert oracle.load().oracle_tracer_particles(C.byref(props), n, seed, abi.vptr(out)) == 0
    return out


def oracle_trace(props, parts, steps, interval, frames, counts=None):
    if counts is None:
        counts = np.zeros((frames,) + props.shape, np.uint32)
    assert oracle.load().oracle_trace(C.byref(props), abi.vptr(parts), len(parts), steps, interval, frames,
                                      abi.vptr(counts)) == 0
    return counts


@pytest.mark.parametrize("R", [8, 12, 32, 64])
def test_tracer_config(R):
    a, b = tracer.tracer_props(R), oracle_props(R)
    for f, _ in abi.Props._fields_:
        va, vb = getattr(a, f), getattr(b, f)
        if isinstance(va, (int, float)):
            assert va == vb, f
        else:
            assert list(va) == list(vb), f


def test_particle_stream():
    """Positions in the middle three quarters of the box, normal speeds of
    width v_mod, protons."""
    props = oracle_props(16)
    p = oracle_particles(props, 20000)
    low, hig = tracer.particle_box(props)
    assert (p["position"] >= low).all() and (p["position"] < hig).all()
    sd = p["velocity"].std(axis=0) / tracer.speed_scale(props)
    assert np.all(np.abs(sd - 1.0) < 0.03)
    assert (p["q"] == tracer.ELEMENTARY_CHARGE).all()
    assert (p["qom"] == tracer.ELEMENTARY_CHARGE / tracer.PROTON_MASS).all()


@pytest.mark.parametrize("case", CASES, ids=lambda c: "N%d_T%d_S%d_R%d" % (c["N"], c["T"], c["S"], c["R"]))
def test_oracle_trace_matches_reference_runs(case):
    """pic_tracer N T S R: seed 0 stream (one range), traceParticle(p, T + 1)
    into T / S + 1 frames; every count equal."""
    props = oracle_props(case["R"])
    parts = oracle_particles(props, case["N"])
    counts = oracle_trace(props, parts, case["T"] + 1, case["S"], case["frames"])
    assert counts.sum(axis=(1, 2, 3)).tolist() == case["frame_totals"]
    if "counts" in case:
        np.testing.assert_array_equal(counts.ravel(), np.array(case["counts"], np.uint32))
    assert sha(counts) == case["counts_sha256"]


@pytest.mark.parametrize("case", CASES[:2], ids=lambda c: "R%d" % c["R"])
def test_result_files_match_reference(case, tmp_path):
    """The frame files written from the histogram are byte-identical to the
    reference's."""
    props = tracer.tracer_props(case["R"])
    counts = np.array(case["counts"], np.uint32).reshape((case["frames"],) + props.shape)
    paths = tracer.write_frames(counts, props, 12345, tmp_path)
    assert [p.rsplit(".", 1)[1] for p in paths] == ["%06d" % t for t in range(case["frames"])]
    for path, want in zip(paths, case["file_sha256"]):
        assert hashlib.sha256(open(path, "rb").read()).hexdigest() == want


def test_oracle_trace_accumulates_and_checks_arguments():
    props = oracle_props(8)
    parts = oracle_particles(props, 500)
    once = oracle_trace(props, parts, 21, 10, 3)
    twice = oracle_trace(props, parts, 21, 10, 3, counts=once.copy())
    np.testing.assert_array_equal(twice, 2 * once)
    lib = oracle.load()
    c = np.zeros(8 ** 3 * 2, np.uint32)
    assert lib.oracle_trace(C.byref(props), abi.vptr(parts), 500, 21, 10, 2, abi.vptr(c)) != 0  # frames too few
    assert lib.oracle_trace(C.byref(props), abi.vptr(parts), 500, 21, 0, 3, abi.vptr(c)) != 0   # interval 0


def test_oracle_trace_upper_face_semantics():
    """A particle resting exactly on the box's upper x face has cell
    coordinate `size`: the reference's flat index puts its count into the
    next frame's x = 0 row, and past the vector's end (last frame) it is not
    counted; on the upper z face it lands in the next row of its own frame."""
    props = abi.Props.make(size=(4, 4, 4), cell_width=(1.0, 0.75, 1.25), dt=0.05, speed_of_light=1.0,
                           planet_radius=1.0, origin=(-2.0, -1.5, -2.5))
    extent = np.array(props.cell_width) * 4
    p = np.zeros(3, abi.PARTICLE_DTYPE)
    p["position"] = np.array(props.origin) + 0.3 * extent
    p["position"][0, 0] = props.origin[0] + extent[0]
    p["position"][1, 2] = props.origin[2] + extent[2]
    p["qom"] = 1.0  # no field (Bz = 0): the particles rest
    three = oracle_trace(props, p, 21, 10, 3)
    five = oracle_trace(props, p, 21, 10, 5)
    assert three.reshape(3, -1).sum(axis=1).tolist() == [2, 3, 3]
    assert five.reshape(5, -1).sum(axis=1).tolist() == [2, 3, 3, 1, 0]
    assert five[1, 0].sum() == 1 and five[3, 0].sum() == 1   # x = size -> next frame, x = 0

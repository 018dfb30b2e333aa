"""The C++ drop-in (include/ipic3d_gpu_simulator.hpp, ipic3d_gpu_reference.hpp):
simulateSteps with GPU policy tags over the reference's own Universe type
(compiled here against the reference headers) and over a stand-in Universe
with the same members (compiled and run on the GPU, compared with the C ABI
path)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from allscale_ipic3d_gb300 import abi, library_path

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
CPP = os.path.join(ROOT, "tests", "cpp")
sys.path.insert(0, ROOT)
import oracle  # noqa: E402  (test infrastructure: where the reference sources are, if anywhere)

REFERENCE = oracle.reference_root() or ""


def compile_cpp(src, out, std="c++14", extra=()):
    lib = os.path.dirname(library_path())
    cmd = ["g++", "-std=" + std, "-O2", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), *extra,
           os.path.join(CPP, src), "-L" + lib, "-lipic3d_gb300", "-Wl,-rpath," + lib, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def gpu_present():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


@pytest.mark.reference
def test_adapter_over_reference_universe(tmp_path):
    """pack/unpack of a reference Universe is lossless and in the C ABI's
    layout; the tags select the GPU specialization of ipic3d::simulateSteps."""
    if not os.path.isdir(os.path.join(REFERENCE, "code", "app", "include")):
        pytest.skip("reference sources not present")
    from allscale_ipic3d_gb300 import library
    library(build_if_missing=True)
    exe = compile_cpp("adapter_reference.cpp", str(tmp_path / "adapter_ref"), std="c++17",
                      extra=("-w", "-Wno-error", "-I" + os.path.join(ROOT, "oracle", "allscale_shim"),
                             "-I" + os.path.join(REFERENCE, "code", "app", "include")))
    r = subprocess.run([exe], capture_output=True, text=True)
    assert "roundtrip mismatches 0" in r.stdout, r.stdout + r.stderr
    assert r.returncode == 0
    if not gpu_present():
        assert "status %d" % abi.E_NODEVICE in r.stdout
        assert "trace status %d" % abi.E_NODEVICE in r.stdout


def test_adapter_standin_builds_and_fails_loudly_without_gpu(tmp_path):
    from allscale_ipic3d_gb300 import library
    library(build_if_missing=True)
    exe = compile_cpp("adapter_standin.cpp", str(tmp_path / "standin"))
    if gpu_present():
        pytest.skip("a GPU is present")
    r = subprocess.run([exe, "0", "0", "2", str(tmp_path / "x")], capture_output=True, text=True)
    assert r.returncode == 1 and ("status %d" % abi.E_NODEVICE) in r.stdout


def read_dump(path):
    with open(path, "rb") as f:
        n, nc = np.frombuffer(f.read(16), np.uint64)
        counts = np.frombuffer(f.read(8 * int(nc)), np.uint64).copy()
        parts = np.frombuffer(f.read(64 * int(n)), abi.PARTICLE_DTYPE).copy()
    return parts, counts


def sorted_by_cell(parts, counts):
    cell = np.repeat(np.arange(len(counts)), counts.astype(np.int64))
    keys = [parts["qom"], parts["q"]] + [parts[f][:, k] for f in ("velocity", "position") for k in (2, 1, 0)]
    order = np.lexsort(keys + [cell])
    return parts[order]


@pytest.mark.gpu
@pytest.mark.parametrize("policy", [0, 1])
@pytest.mark.parametrize("fp32", [0, 1])
def test_adapter_standin_matches_c_abi(tmp_path, policy, fp32):
    from allscale_ipic3d_gb300 import Simulation, library
    library(build_if_missing=True)
    exe = compile_cpp("adapter_standin.cpp", str(tmp_path / "standin"))
    pre = str(tmp_path / "run")
    steps = 5
    trace = str(tmp_path / "ConservedQuantities.out")
    r = subprocess.run([exe, str(policy), str(fp32), str(steps), pre, trace], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    parts, counts = read_dump(pre + "_in.bin")
    out, out_counts = read_dump(pre + "_out.bin")
    prec = abi.FP32 if fp32 else abi.FP64
    if policy == 0:
        props = abi.Props.make(size=(6, 6, 6), cell_width=(10.0, 10.0, 10.0), dt=0.15, planet_radius=8.0,
                               origin=(-30.0, -30.0, -30.0), external_b=(0.0, 0.0, 1e-4))
        cfg = abi.Config.make(precision=prec, flags=abi.F_USE_GRAPH)
        f = np.zeros(abi.field_shape(props))
        bc = np.zeros(abi.bcfield_shape(props))
    else:
        props = abi.Props.make(size=(6, 6, 6), dt=0.1)
        cfg = abi.Config.make(precision=prec, mover=abi.MOVER_FIELD, solver=abi.SOLVER_LEAPFROG,
                              projector=abi.PROJECT_CIC, bc=abi.BC_PERIODIC,
                              flags=abi.F_USE_GRAPH | abi.F_REFRESH_NODE_B)
        f = np.zeros(abi.field_shape(props))
        f[..., 1] = 0.01
        f[..., 5] = 0.1
        bc = np.zeros(abi.bcfield_shape(props))
        bc[..., 2] = 0.1
    sim = Simulation(props, cfg)
    sim.upload_fields(f, bc, np.zeros(abi.density_shape(props)))
    sim.upload_particles(parts, counts)
    rows = sim.conserved_trace(steps)  # one step per call, the conserved quantities before each
    p2, c2, _ = sim.download_particles()
    if policy == 0:  # the trace the drop-in wrote equals the C ABI's, in the reference's format
        from allscale_ipic3d_gb300 import trace_text
        assert open(trace).read() == trace_text(rows)
    # density files before cycle 0 (t = 0) and cycles 1 and 3 (t = 1, 2): t,x,y,z,density per cell
    lines = open(trace + ".csv.000000").read().splitlines()
    assert lines[0] == "t,x,y,z,density" and len(lines) == 1 + props.ncells
    assert [int(l.split(",")[4]) for l in lines[1:]] == counts.astype(int).tolist()
    w = props.cell_width[0]
    assert lines[2] == "0,0,0,%g,%d" % (w, counts[1])
    for t in (1, 2):
        assert os.path.exists(trace + ".csv.%06d" % t)
    np.testing.assert_array_equal(out_counts, c2)
    a, b = sorted_by_cell(out, out_counts), sorted_by_cell(p2, c2)
    if policy == 0:  # no floating-point atomics on the particles' data path
        assert a.tobytes() == b.tobytes()
    else:  # the fields evolve from atomic sums (order free): FP64 rounding,
        # or FP32 rounding where the FP32 deposit sums a warp's particles first
        rtol, atol = (1e-5, 1e-7) if fp32 else (1e-9, 1e-12)
        for k in ("position", "velocity"):
            np.testing.assert_allclose(a[k], b[k], rtol=rtol, atol=atol)


@pytest.mark.gpu
def test_tracer_standin_matches_c_abi(tmp_path):
    """ipic3d_gpu::trace_particles over stand-in Particle / properties types
    equals the Python binding's trace on the same particles."""
    import allscale_ipic3d_gb300 as ipg
    from allscale_ipic3d_gb300 import library, tracer
    library(build_if_missing=True)
    exe = compile_cpp("tracer_standin.cpp", str(tmp_path / "tracer_standin"))
    R, steps, S = 16, 31, 10
    props = tracer.tracer_props(R)
    rng = np.random.default_rng(5)
    low, hig = tracer.particle_box(props)
    parts = np.zeros(20000, abi.PARTICLE_DTYPE)
    parts["position"] = rng.uniform(low, hig, (len(parts), 3))
    parts["velocity"] = rng.normal(0.0, tracer.speed_scale(props), (len(parts), 3))
    parts["q"] = tracer.ELEMENTARY_CHARGE
    parts["qom"] = tracer.ELEMENTARY_CHARGE / tracer.PROTON_MASS
    src, dst = str(tmp_path / "p.bin"), str(tmp_path / "c.bin")
    parts.tofile(src)
    frames = ipg.trace_frames(steps, S)
    r = subprocess.run([exe, str(R), str(steps), str(S), str(frames), src, dst], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.fromfile(dst, np.uint32).reshape((frames,) + props.shape)
    np.testing.assert_array_equal(got, ipg.trace(props, parts, steps, S))

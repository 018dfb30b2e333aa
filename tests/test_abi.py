"""The C ABI library: it builds for sm_103a, loads, and exports every entry
point that include/*.h declares (no GPU needed)."""
import ctypes as C
import os
import re

import allscale_ipic3d_gb300 as pkg
from allscale_ipic3d_gb300 import abi

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def declared_entry_points():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(ipic3d_gpu_\w+)\s*\(", text))
    return names


def test_library_builds_and_exports_every_declared_symbol():
    from allscale_ipic3d_gb300.build import build
    path = build()
    assert os.path.exists(path)
    lib = C.CDLL(path)
    declared = declared_entry_points()
    assert len(declared) >= 20
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    assert declared == set(pkg.EXPORTED_SYMBOLS), declared ^ set(pkg.EXPORTED_SYMBOLS)


def test_struct_layouts_match_header():
    assert C.sizeof(abi.Props) == 3 * 8 + 3 * 8 + 3 * 8 + 9 * 8
    assert abi.PARTICLE_DTYPE.itemsize == 64
    assert C.sizeof(abi.Conserved) == 6 * 8
    assert C.sizeof(abi.Stats) == 10 * 8


def test_config_default_matches_reference_policies():
    lib = pkg.library(build_if_missing=True)
    cfg = abi.Config()
    lib.ipic3d_gpu_config_default(C.byref(cfg))
    assert cfg.precision == abi.FP64 and cfg.mover == abi.MOVER_DIPOLE
    assert cfg.solver == abi.SOLVER_STATIC and cfg.projector == abi.PROJECT_NONE
    assert list(cfg.bc_low) == [abi.BC_REFLECT] * 3 and list(cfg.bc_high) == [abi.BC_REFLECT] * 3


def test_create_without_gpu_fails_loudly():
    """On a machine without an sm_103 GPU the library refuses with a status
    (there is no CPU fallback)."""
    try:
        import torch
        if torch.cuda.is_available():
            import pytest
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    lib = pkg.library(build_if_missing=True)
    ctx = C.c_void_p()
    p = abi.Props.make(size=(2, 2, 2))
    cfg = abi.Config.make()
    rc = lib.ipic3d_gpu_create(C.byref(p), C.byref(cfg), C.byref(ctx))
    assert rc == abi.E_NODEVICE
    buf = C.create_string_buffer(256)
    assert lib.ipic3d_gpu_last_error(buf, 256) == abi.E_NODEVICE
    assert buf.value


def test_batch_create_without_gpu_fails_loudly():
    try:
        import torch
        if torch.cuda.is_available():
            import pytest
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    lib = pkg.library(build_if_missing=True)
    b = C.c_void_p()
    props = (abi.Props * 2)(abi.Props.make(size=(2, 2, 2)), abi.Props.make(size=(3, 3, 3)))
    cfg = abi.Config.make()
    assert lib.ipic3d_gpu_batch_create(2, props, C.byref(cfg), C.byref(b)) == abi.E_NODEVICE
    assert lib.ipic3d_gpu_batch_create(0, props, C.byref(cfg), C.byref(b)) == abi.E_INVALID
    assert not b.value


def test_tracer_arguments_and_no_gpu():
    """ipic3d_gpu_trace checks its arguments before any device work, does
    nothing for an empty set, and refuses without an sm_103 GPU."""
    import numpy as np
    import pytest
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from allscale_ipic3d_gb300 import tracer
    props = tracer.tracer_props(8)
    parts = np.zeros(4, abi.PARTICLE_DTYPE)
    with pytest.raises(pkg.GpuPathError) as e:
        pkg.trace(props, parts, 21, 10, num_frames=2)   # frame 2 does not fit
    assert e.value.status == abi.E_INVALID
    with pytest.raises(pkg.GpuPathError) as e:
        pkg.trace(props, parts, 21, 0, num_frames=3)    # frame interval 0
    assert e.value.status == abi.E_INVALID
    assert pkg.trace(props, parts[:0], 21, 10).sum() == 0   # nothing to trace
    assert pkg.trace(props, parts, 0, 10, num_frames=0).size == 0
    with pytest.raises(pkg.GpuPathError) as e:
        pkg.trace(props, parts, 21, 10)
    assert e.value.status == abi.E_NODEVICE
    with pytest.raises(pkg.GpuPathError) as e:
        pkg.aggregate_contributions(props, None, None)
    assert e.value.status == abi.E_INVALID


def test_project_noalloc_rejects_sizes_before_any_device_work():
    """The allocation-free projection checks the grid against its fixed
    scratch axis by axis before it multiplies (no overflow for huge sizes)
    and before it touches a device; the pointers are never dereferenced."""
    import pytest
    lib = pkg.library(build_if_missing=True)
    fake = C.c_void_p(256)
    buf = C.create_string_buffer(256)
    for size in ((1 << 21,) * 3, (1 << 62, 1, 1), (40000, 1, 1), (33, 32, 32), (2, 2, 1 << 40)):
        props = abi.Props.make(size=(1, 1, 1))
        props.size[0], props.size[1], props.size[2] = size
        rc = lib.ipic3d_gpu_project_noalloc(C.byref(props), 0, fake, fake, fake, None, None)
        assert rc == abi.E_CAPACITY, size
        lib.ipic3d_gpu_last_error(buf, 256)
        assert b"too large" in buf.value
    props = abi.Props.make(size=(1, 1, 1))
    props.size[1] = 0
    assert lib.ipic3d_gpu_project_noalloc(C.byref(props), 0, fake, fake, fake, None, None) == abi.E_INVALID
    assert lib.ipic3d_gpu_project_noalloc(None, 0, fake, fake, fake, None, None) == abi.E_INVALID
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    props = abi.Props.make(size=(32, 32, 32))  # fits: refused only for want of a device
    assert lib.ipic3d_gpu_project_noalloc(C.byref(props), 0, fake, fake, fake, None, None) == abi.E_NODEVICE


def test_plain_c_consumer(tmp_path):
    """The header is C99 and the library links from C (the form cgo, JNI or
    N-API bindings use)."""
    import subprocess
    import pytest
    lib = os.path.dirname(pkg.library_path())
    pkg.library(build_if_missing=True)
    exe = str(tmp_path / "c_consumer")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "c_consumer.c"), "-L" + lib, "-lipic3d_gb300",
                        "-Wl,-rpath," + lib, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120).stdout
    assert "defaults 0 0 0 0" in out
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    assert "create %d " % abi.E_NODEVICE in out

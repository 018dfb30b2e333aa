"""CPU oracle of the GB300 particle path (test infrastructure only).

``build()`` compiles the C++ restatement (ipic3d_oracle.cpp) into
``oracle/liboracle.so`` and, where the reference sources are present, the
reference's own code into ``oracle/_ref/`` (see ref/Makefile). ``load()`` and
``load_reference()`` return ctypes handles. Only tests/, the smoke check and
bench.py's CPU-baseline leg use this package.
"""
import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(REF_DIR, "libipic3d_ref.so")
ROOT_RECORD = os.path.join(REF_DIR, "reference_root.txt")


def reference_root():
    """The reference source tree to compile: $IPIC3D_REFERENCE_ROOT, else the
    tree the last build_reference() used (recorded in oracle/_ref/), else
    None (no reference sources: the reference-based tests skip)."""
    root = os.environ.get("IPIC3D_REFERENCE_ROOT")
    if not root and os.path.exists(ROOT_RECORD):
        root = open(ROOT_RECORD).read().strip()
    if root and os.path.isdir(os.path.join(root, "code", "app", "include")):
        return root
    return None


def build(force=False):
    srcs = [os.path.join(HERE, "ipic3d_oracle.cpp"), os.path.join(HERE, "ipic3d_oracle_init.cpp"),
            os.path.join(HERE, "ipic3d_oracle_tracer.cpp")]
    hdrs = [os.path.join(HERE, "ipic3d_oracle.h"), os.path.join(HERE, "..", "include", "ipic3d_gpu.h"),
            os.path.join(HERE, "..", "include", "ipic3d_types.h")]
    newest = max(os.path.getmtime(p) for p in srcs + hdrs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp"
        # -ffp-contract=off: no fused multiply-add, the reference's rounding
        subprocess.check_call(["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                               "-o", tmp] + srcs)
        os.replace(tmp, LIB)
    return LIB


def build_reference(root=None):
    """Compiles the reference's sources in place from `root` (default:
    reference_root()), only where they exist, and records the tree used."""
    root = root or reference_root()
    if not root or not os.path.isdir(os.path.join(root, "code", "app", "include")):
        return None
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"), "-j8", "REF=" + root])
    with open(ROOT_RECORD, "w") as f:
        f.write(root + "\n")
    return REF_LIB


_oracle = None


def load():
    global _oracle
    if _oracle is None:
        build()
        lib = C.CDLL(LIB)
        vp = C.c_void_p
        P = C.POINTER
        lib.oracle_create.argtypes = [vp, vp, P(vp)]
        lib.oracle_destroy.argtypes = [vp]
        lib.oracle_destroy.restype = None
        lib.oracle_set_threads.argtypes = [C.c_int]
        lib.oracle_set_threads.restype = None
        lib.oracle_upload_particles.argtypes = [vp, vp, vp, vp]
        lib.oracle_upload_fields.argtypes = [vp, vp, vp, vp]
        lib.oracle_download_fields.argtypes = [vp, vp, vp, vp, vp]
        lib.oracle_particle_count.argtypes = [vp]
        lib.oracle_particle_count.restype = C.c_uint64
        lib.oracle_download_particles.argtypes = [vp, vp, C.c_uint64, vp, vp]
        lib.oracle_step.argtypes = [vp, C.c_uint64]
        for f in ("oracle_project", "oracle_update_boundaries", "oracle_solve_fields", "oracle_move"):
            getattr(lib, f).argtypes = [vp]
        lib.oracle_conserved.argtypes = [vp, vp]
        lib.oracle_last_counts.argtypes = [vp, vp, vp, vp]
        lib.oracle_boris.argtypes = [vp, C.c_uint64, vp, vp, C.c_double, C.c_uint64, C.c_int]
        lib.oracle_trilinear.argtypes = [vp, vp, C.c_double]
        lib.oracle_trilinear.restype = C.c_double
        lib.oracle_init_uniform_pos_normal_speed.argtypes = [vp, C.c_uint64, vp, vp, vp, vp, vp, vp, vp]
        lib.oracle_init_uniform_bench.argtypes = [vp, C.c_uint64, vp, vp]
        lib.oracle_aggregate_contributions.argtypes = [vp, vp, vp]
        lib.oracle_tracer_config.argtypes = [C.c_int32, vp]
        lib.oracle_tracer_particles.argtypes = [vp, C.c_uint64, C.c_uint32, vp]
        lib.oracle_trace.argtypes = [vp, vp, C.c_uint64, C.c_int32, C.c_int32, C.c_int32, vp]
        _oracle = lib
    return _oracle


_ref = None


def load_reference():
    """The reference's own functions (oracle/_ref/libipic3d_ref.so), or None
    where the reference sources are absent and nothing was built."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB):
            try:
                build_reference()
            except Exception:
                return None
        if not os.path.exists(REF_LIB):
            return None
        lib = C.CDLL(REF_LIB)
        vp = C.c_void_p
        lib.ref_simulate_default.argtypes = [vp, vp, vp, C.c_uint64, vp, C.c_uint64, vp, vp]
        lib.ref_move_particles.argtypes = [vp, vp, vp, C.c_uint64]
        lib.ref_boris.argtypes = [vp, vp, vp, C.c_double, C.c_uint64, C.c_int]
        lib.ref_project_current.argtypes = [vp, vp, vp, vp]
        lib.ref_aggregate_contributions.argtypes = [vp, vp, vp]
        lib.ref_update_boundaries.argtypes = [vp, vp, vp]
        lib.ref_leapfrog_two_phase.argtypes = [vp, vp, vp, vp]
        lib.ref_solve_forward_at.argtypes = [vp, vp, vp, vp, vp]
        lib.ref_trilinear.argtypes = [vp, vp, C.c_double]
        lib.ref_trilinear.restype = C.c_double
        lib.ref_conserved.argtypes = [vp, vp, vp, vp, vp]
        lib.ref_init_from_inp.argtypes = [C.c_char_p, vp, vp, vp, C.c_uint64, vp, vp, vp]
        lib.ref_write_particle_positions.argtypes = [vp, vp, vp, C.c_char_p]
        lib.ref_write_field_grids.argtypes = [vp, vp, vp, C.c_char_p]
        _ref = lib
    return _ref

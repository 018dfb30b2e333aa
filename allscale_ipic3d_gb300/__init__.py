"""GB300 (sm_103a) implementation of the AllScale iPIC3D per-timestep particle
path: the Boris mover, cloud-in-cell projection of charge and current,
particle migration between cells and the field update.

The compute path is the CUDA library ``_lib/libipic3d_gb300.so`` behind the
C ABI of ``include/ipic3d_gpu.h``; this module binds it with ctypes and offers
``Simulation``, a host-side mirror of the reference's ``Universe`` plus
``simulateSteps`` (code/app/include/ipic3d/app/universe.h:12-51,
simulator.h:127-242). There is no CPU fallback: without the library (or
without an sm_103 GPU) every call raises ``GpuPathError``.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .abi import (BC_OPEN, BC_PERIODIC, BC_REFLECT, FP32, FP64, MOVER_DIPOLE, MOVER_FIELD, PARTICLE_DTYPE,
                  PROJECT_CIC, PROJECT_NONE, SOLVER_FORWARD, SOLVER_LEAPFROG, SOLVER_STATIC, Config, Conserved,
                  Props, Stats)

__all__ = ["Simulation", "Batch", "Props", "Config", "Conserved", "Stats", "PARTICLE_DTYPE", "GpuPathError",
           "library", "library_path", "boris", "aggregate_contributions", "trace", "trace_device", "trace_frames", "EXPORTED_SYMBOLS"]

HERE = os.path.dirname(os.path.abspath(__file__))


def library_path():
    return os.path.join(HERE, "_lib", "libipic3d_gb300.so")


class GpuPathError(RuntimeError):
    """A failed call of the CUDA path (status code and the library's message)."""

    def __init__(self, status, message):
        super().__init__("ipic3d_gpu status %d: %s" % (status, message))
        self.status = status


# every entry point of include/ipic3d_gpu.h: (name, restype, argtypes)
_vp = C.c_void_p
_SIGNATURES = [
    ("ipic3d_gpu_config_default", None, [_vp]),
    ("ipic3d_gpu_create", C.c_int, [_vp, _vp, C.POINTER(_vp)]),
    ("ipic3d_gpu_destroy", C.c_int, [_vp]),
    ("ipic3d_gpu_upload_particles", C.c_int, [_vp, _vp, _vp, _vp]),
    ("ipic3d_gpu_reserve", C.c_int, [_vp, C.c_uint64]),
    ("ipic3d_gpu_init_uniform", C.c_int, [_vp, C.c_uint64]),
    ("ipic3d_gpu_init_uniform_pos_normal_speed", C.c_int, [_vp, C.c_uint64, _vp, _vp, _vp, _vp]),
    ("ipic3d_gpu_particle_count", C.c_int, [_vp, C.POINTER(C.c_uint64)]),
    ("ipic3d_gpu_download_particles", C.c_int, [_vp, _vp, C.c_uint64, _vp, _vp]),
    ("ipic3d_gpu_download_positions", C.c_int, [_vp, _vp, C.c_uint64, _vp]),
    ("ipic3d_gpu_download_particles_async", C.c_int, [_vp, _vp, C.c_uint64, _vp, _vp]),
    ("ipic3d_gpu_download_wait", C.c_int, [_vp]),
    ("ipic3d_gpu_cell_counts", C.c_int, [_vp, _vp]),
    ("ipic3d_gpu_upload_fields", C.c_int, [_vp, _vp, _vp, _vp]),
    ("ipic3d_gpu_download_fields", C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    ("ipic3d_gpu_step", C.c_int, [_vp, C.c_uint64]),
    ("ipic3d_gpu_project", C.c_int, [_vp]),
    ("ipic3d_gpu_update_boundaries", C.c_int, [_vp]),
    ("ipic3d_gpu_solve_fields", C.c_int, [_vp]),
    ("ipic3d_gpu_move", C.c_int, [_vp]),
    ("ipic3d_gpu_conserved", C.c_int, [_vp, _vp]),
    ("ipic3d_gpu_synchronize", C.c_int, [_vp]),
    ("ipic3d_gpu_stream", _vp, [_vp]),
    ("ipic3d_gpu_stats", C.c_int, [_vp, _vp]),
    ("ipic3d_gpu_profile", C.c_int, [_vp, C.c_int]),
    ("ipic3d_gpu_profile_read", C.c_int, [_vp, _vp, C.c_int]),
    ("ipic3d_gpu_get_push_shape", C.c_int, [_vp, _vp]),
    ("ipic3d_gpu_set_push_shape", C.c_int, [_vp, _vp]),
    ("ipic3d_gpu_set_wait_limit", C.c_int, [_vp, C.c_int64]),
    ("ipic3d_gpu_project_noalloc", C.c_int, [_vp, C.c_uint32, _vp, _vp, _vp, _vp, _vp]),
    ("ipic3d_gpu_aggregate_contributions", C.c_int, [_vp, _vp, _vp, _vp]),
    ("ipic3d_gpu_trace", C.c_int, [_vp, _vp, C.c_uint64, C.c_int32, C.c_int32, C.c_int32, _vp]),
    ("ipic3d_gpu_trace_device", C.c_int, [_vp, _vp, C.c_uint64, C.c_int32, C.c_int32, C.c_int32, _vp, _vp]),
    ("ipic3d_gpu_boris", C.c_int, [_vp, C.c_uint64, _vp, _vp, C.c_double, C.c_uint64, C.c_int]),
    ("ipic3d_gpu_batch_create", C.c_int, [C.c_uint32, _vp, _vp, C.POINTER(_vp)]),
    ("ipic3d_gpu_batch_destroy", C.c_int, [_vp]),
    ("ipic3d_gpu_batch_size", C.c_int, [_vp, C.POINTER(C.c_uint32)]),
    ("ipic3d_gpu_batch_universe", C.c_int, [_vp, C.c_uint32, C.POINTER(_vp)]),
    ("ipic3d_gpu_batch_step", C.c_int, [_vp, C.c_uint64]),
    ("ipic3d_gpu_batch_synchronize", C.c_int, [_vp]),
    ("ipic3d_gpu_batch_stream", _vp, [_vp]),
    ("ipic3d_gpu_batch_stats", C.c_int, [_vp, _vp]),
    ("ipic3d_gpu_batch_get_push_shape", C.c_int, [_vp, _vp]),
    ("ipic3d_gpu_last_error", C.c_int, [C.c_char_p, C.c_size_t]),
]
EXPORTED_SYMBOLS = [s[0] for s in _SIGNATURES]

_lib = None


def library(build_if_missing=False):
    """The loaded CUDA library (ctypes.CDLL). Raises GpuPathError if absent."""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            if build_if_missing:
                from .build import build
                build()
            else:
                raise GpuPathError(-5, "CUDA library %s is not built (run __graft_entry__.build())" % path)
        lib = C.CDLL(path)
        for name, res, args in _SIGNATURES:
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def _check(rc):
    if rc != 0:
        buf = C.create_string_buffer(512)
        library().ipic3d_gpu_last_error(buf, 512)
        raise GpuPathError(rc, buf.value.decode(errors="replace"))


def trace_text(rows):
    """The reference's ConservedQuantities.out text for trace rows: its
    header, then per row the cycle and four doubles in the default C++ stream
    format (6 significant digits), tab separated (simulator.h:65-90)."""
    lines = ["Cycle \t Total Moment \t E energy \t B energy \t Total KE "]
    lines += ["\t".join([str(int(r[0]))] + ["%g" % v for v in r[1:]]) for r in rows]
    return "\n".join(lines) + "\n"


def boris(particles, E, B, dt, nsteps=1, push_position=True):
    """Particle::updateVelocity (+ updatePosition) applied nsteps times on the
    GPU (particle.h:24-49); `particles` is a PARTICLE_DTYPE array, modified in
    place."""
    p = np.ascontiguousarray(particles, dtype=PARTICLE_DTYPE)
    e = np.asarray(E, dtype=np.float64)
    b = np.asarray(B, dtype=np.float64)
    _check(library().ipic3d_gpu_boris(abi.vptr(p), len(p), abi.vptr(e), abi.vptr(b), float(dt), int(nsteps),
                                      1 if push_position else 0))
    if p is not particles:
        particles[...] = p
    return particles


def project_noalloc(props, flags, d_particles, d_cell_offsets, d_J, d_rho=None, stream=None):
    """ipic3d_gpu_project_noalloc on caller-owned device buffers (integer
    device addresses): the current projection without any allocation."""
    _check(library().ipic3d_gpu_project_noalloc(C.byref(props), int(flags), d_particles, d_cell_offsets, d_J,
                                                d_rho, stream))


def aggregate_contributions(props, d_contributions, d_J, stream=None):
    """aggregateDensityContributions (cell.h:835-855) over all nodes on
    caller-owned device buffers (integer device addresses): the (2 size)^3 x 3
    contribution grid into the (size+1)^3 x 3 J grid, in place."""
    _check(library().ipic3d_gpu_aggregate_contributions(C.byref(props), d_contributions, d_J, stream))


def trace_frames(steps, frame_interval):
    """Frames of a trace of `steps` steps: (steps - 1) // frame_interval + 1
    (pic_tracer's main traces T + 1 steps into T // S + 1 frames)."""
    return (int(steps) - 1) // int(frame_interval) + 1 if steps > 0 else 0


def trace(props, particles, steps, frame_interval, num_frames=None, counts=None):
    """traceParticle (pic_tracer.cxx:77-148) for every particle of a
    PARTICLE_DTYPE array on the GPU. Returns the ParticleCount histogram,
    uint32 of shape (num_frames, *props.shape); `counts`, if given, is added
    to in place (pic_tracer.cxx:282)."""
    p = np.ascontiguousarray(particles, dtype=PARTICLE_DTYPE)
    frames = trace_frames(steps, frame_interval) if num_frames is None else int(num_frames)
    if counts is None:
        counts = np.zeros((frames,) + props.shape, np.uint32)
    if counts.dtype != np.uint32 or not counts.flags.c_contiguous or counts.size != frames * props.ncells:
        raise ValueError("counts must be a C-contiguous uint32 array of num_frames x cells entries")
    _check(library().ipic3d_gpu_trace(C.byref(props), abi.vptr(p), len(p), int(steps), int(frame_interval), frames,
                                      abi.vptr(counts)))
    return counts


def trace_device(props, d_particles, n, steps, frame_interval, num_frames, d_counts, stream=None):
    """ipic3d_gpu_trace_device on caller-owned device buffers (integer device
    addresses): enqueued on `stream`, not synchronised."""
    _check(library().ipic3d_gpu_trace_device(C.byref(props), d_particles, int(n), int(steps), int(frame_interval),
                                             int(num_frames), d_counts, stream))


class Simulation:
    """One Universe resident on the GPU.

    ``props`` mirrors UniverseProperties (universe_properties.h:52-123) and
    ``config`` the simulateSteps policies (simulator.h:42-47,244-276).
    """

    def __init__(self, props, config=None, _lent=None):
        self.props = props
        self.config = config if config is not None else Config.make()
        self.ncells = props.ncells
        if _lent is not None:  # a universe of a Batch (freed with the batch)
            self._ctx = _lent
            self._owner = False
            return
        lib = library()
        ctx = C.c_void_p()
        _check(lib.ipic3d_gpu_create(C.byref(self.props), C.byref(self.config), C.byref(ctx)))
        self._ctx = ctx
        self._owner = True

    # -- lifetime --
    def close(self):
        if getattr(self, "_ctx", None):
            if getattr(self, "_owner", False):
                library().ipic3d_gpu_destroy(self._ctx)
            self._ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- particles --
    def upload_particles(self, particles, cell_counts, ids=None):
        """Universe::cells: particles grouped by cell (row-major), with the
        number per cell."""
        p = np.ascontiguousarray(particles, dtype=PARTICLE_DTYPE)
        c = np.ascontiguousarray(cell_counts, dtype=np.uint64).reshape(-1)
        if c.size != self.ncells:
            raise ValueError("cell_counts has %d entries, grid has %d cells" % (c.size, self.ncells))
        if int(c.sum()) != len(p):
            raise ValueError("cell_counts sum to %d but %d particles given" % (int(c.sum()), len(p)))
        i = None if ids is None else np.ascontiguousarray(ids, dtype=np.uint32)
        _check(library().ipic3d_gpu_upload_particles(self._ctx, abi.vptr(p), abi.vptr(c), abi.vptr(i)))

    def init_uniform(self, num_particles):
        """initCells(uniform) of the reference's :U:N benchmark mode, made on
        the device with the reference's random streams (cell.h:638-697)."""
        _check(library().ipic3d_gpu_init_uniform(self._ctx, int(num_particles)))

    def init_uniform_pos_normal_speed(self, num_particles, low, hig, mean, stddev):
        """initCells with the .inp driver's distribution (cell.h:492-636):
        per-cell counts on the host, the particles made on the device with
        the reference's random streams (src/ipic3d.cxx:69-82 builds low, hig
        as the middle 3/4 of the box, mean 0 and stddev v_mod)."""
        arr = [np.ascontiguousarray(v, np.float64).reshape(3) for v in (low, hig, mean, stddev)]
        _check(library().ipic3d_gpu_init_uniform_pos_normal_speed(self._ctx, int(num_particles),
                                                                  *[abi.vptr(a) for a in arr]))

    def particle_count(self):
        n = C.c_uint64()
        _check(library().ipic3d_gpu_particle_count(self._ctx, C.byref(n)))
        return n.value

    def download_particles(self, out=None, ids=True):
        """(particles, cell_counts, ids) grouped by cell; order inside a cell
        is unspecified. `out` = (particles, cell_counts): caller-owned host
        arrays to fill (for example pinned memory); the result is then views
        of them (particles[:n]) and ids is None unless `ids` is an array."""
        if out is not None:
            p, c = out
            i = ids if isinstance(ids, np.ndarray) else None
            _check(library().ipic3d_gpu_download_particles(self._ctx, abi.vptr(p), len(p), abi.vptr(c),
                                                           abi.vptr(i)))
            n = int(c.sum())
            return p[:n], c, (i[:n] if i is not None else None)
        n = self.particle_count()
        p = np.zeros(n, PARTICLE_DTYPE)
        c = np.zeros(self.ncells, np.uint64)
        i = np.zeros(n, np.uint32) if ids else None
        _check(library().ipic3d_gpu_download_particles(self._ctx, abi.vptr(p), n, abi.vptr(c), abi.vptr(i)))
        return p, c, i

    def download_particles_async(self, out, ids=None):
        """Starts a download into caller-owned host arrays `out` =
        (particles, cell_counts) (pinned memory for full speed): the counts
        are filled at once, the particles (and `ids`, an array or None) once
        download_wait() returns. Meanwhile other calls may run, an upload
        among them (its copies use the link's other direction)."""
        p, c = out
        _check(library().ipic3d_gpu_download_particles_async(self._ctx, abi.vptr(p), len(p), abi.vptr(c),
                                                             abi.vptr(ids)))
        return int(c.sum())

    def download_wait(self):
        _check(library().ipic3d_gpu_download_wait(self._ctx))

    def download_positions(self):
        """(positions (n, 3), cell_counts): every particle's position in the
        download order, packed on the device (24 bytes per particle cross
        the host link)."""
        c = self.cell_counts()
        n = int(c.sum())
        xyz = np.zeros((n, 3))
        _check(library().ipic3d_gpu_download_positions(self._ctx, abi.vptr(xyz), n, abi.vptr(c)))
        return xyz, c

    def write_particle_positions(self, path):
        """outputParticlePositions (cell.h:1400-1429): "x y z" per particle,
        grouped by cell in row-major order, each number as the reference's
        output stream prints a double (6 significant digits)."""
        xyz, _ = self.download_positions()
        with open(path, "w") as f:
            f.write("".join("%g %g %g\n" % (x, y, z) for x, y, z in xyz.tolist()))

    def write_field_grids(self, path):
        """outputFieldGrids (field.h:464-530): the field grid ("i,j,k:[E]|[B]|
        [Bext]" per node), then the BcField grid ("i,j,k:[Bc]" per cell),
        each after its "[nx,ny,nz]" size line and followed by an empty line.
        The reference writes both to the same file entry, one after the
        other, so the second replaces the first; this writer does the same."""
        f, b, _, _ = self.download_fields()

        def vec(v):
            return "[%g,%g,%g]" % tuple(v)

        def grid(a, per_node):
            nx, ny, nz = a.shape[:3]
            lines = ["[%d,%d,%d]\n" % (nx, ny, nz)]
            for i in range(nx):
                for j in range(ny):
                    for k in range(nz):
                        lines.append("%d,%d,%d:%s\n" % (i, j, k, per_node(a[i, j, k].tolist())))
            lines.append("\n")
            return "".join(lines)

        with open(path, "w") as out:
            out.write(grid(f, lambda v: "%s|%s|%s" % (vec(v[0:3]), vec(v[3:6]), vec(v[6:9]))))
        with open(path, "w") as out:
            out.write(grid(b, vec))

    def cell_counts(self):
        c = np.zeros(self.ncells, np.uint64)
        _check(library().ipic3d_gpu_cell_counts(self._ctx, abi.vptr(c)))
        return c

    # -- fields --
    def upload_fields(self, field=None, bcfield=None, density=None):
        f = None if field is None else np.ascontiguousarray(field, np.float64)
        b = None if bcfield is None else np.ascontiguousarray(bcfield, np.float64)
        d = None if density is None else np.ascontiguousarray(density, np.float64)
        if f is not None:
            assert f.size == np.prod(abi.field_shape(self.props))
        if b is not None:
            assert b.size == np.prod(abi.bcfield_shape(self.props))
        if d is not None:
            assert d.size == np.prod(abi.density_shape(self.props))
        _check(library().ipic3d_gpu_upload_fields(self._ctx, abi.vptr(f), abi.vptr(b), abi.vptr(d)))

    def download_fields(self):
        f = np.zeros(abi.field_shape(self.props))
        b = np.zeros(abi.bcfield_shape(self.props))
        d = np.zeros(abi.density_shape(self.props))
        r = np.zeros(abi.density_shape(self.props)[:3])
        _check(library().ipic3d_gpu_download_fields(self._ctx, abi.vptr(f), abi.vptr(b), abi.vptr(d), abi.vptr(r)))
        return f, b, d, r

    # -- the timestep --
    def step(self, n=1):
        """simulateSteps(n, universe) (simulator.h:127-242)."""
        _check(library().ipic3d_gpu_step(self._ctx, int(n)))

    def project(self):
        _check(library().ipic3d_gpu_project(self._ctx))

    def update_boundaries(self):
        _check(library().ipic3d_gpu_update_boundaries(self._ctx))

    def solve_fields(self):
        _check(library().ipic3d_gpu_solve_fields(self._ctx))

    def move(self):
        _check(library().ipic3d_gpu_move(self._ctx))

    def synchronize(self):
        _check(library().ipic3d_gpu_synchronize(self._ctx))

    def conserved(self):
        out = Conserved()
        _check(library().ipic3d_gpu_conserved(self._ctx, C.byref(out)))
        return out.as_dict()

    def stats(self):
        out = Stats()
        _check(library().ipic3d_gpu_stats(self._ctx, C.byref(out)))
        return out.as_dict()

    def conserved_trace(self, steps, every=1, path=None):
        """Runs `steps` steps, one call per cycle, and returns the rows the
        reference's debug build writes (writeOutputData, simulator.h:65-90):
        [cycle, total momentum, E energy, B energy, kinetic energy] before
        every `every`-th cycle and before the last, from the device's
        reductions. With `path`, also writes them in the reference's
        ConservedQuantities.out format."""
        rows = []
        for i in range(int(steps)):
            if every > 0 and (i % every == 0 or i + 1 == steps):
                c = self.conserved()
                rows.append([i, c["total_momentum"], c["e_energy"], c["b_energy"], c["kinetic_energy"]])
            self.step(1)
        if path is not None:
            with open(path, "w") as f:
                f.write(trace_text(rows))
        return rows

    def profile(self, enable=True):
        """Per-phase CUDA-event timing of the following steps (no graph)."""
        _check(library().ipic3d_gpu_profile(self._ctx, 1 if enable else 0))

    def profile_read(self, reset=True):
        out = abi.Profile()
        _check(library().ipic3d_gpu_profile_read(self._ctx, C.byref(out), 1 if reset else 0))
        return out.as_dict()

    def push_shape(self):
        """Launch shape of the FP32 push (autotuned unless fixed)."""
        out = abi.PushShape()
        _check(library().ipic3d_gpu_get_push_shape(self._ctx, C.byref(out)))
        return out.as_dict()

    def set_push_shape(self, item=None, item_cells=None, blocks_per_sm=None):
        """Fixes the push shape (no autotuning); with no argument, restarts
        the autotuner (its trials run in the next steps)."""
        if item is None and item_cells is None and blocks_per_sm is None:
            _check(library().ipic3d_gpu_set_push_shape(self._ctx, None))
            return
        cur = self.push_shape()
        s = abi.PushShape(item=cur["item"] if item is None else int(item),
                          item_cells=cur["item_cells"] if item_cells is None else int(item_cells),
                          blocks_per_sm=cur["blocks_per_sm"] if blocks_per_sm is None else int(blocks_per_sm))
        _check(library().ipic3d_gpu_set_push_shape(self._ctx, C.byref(s)))

    def set_wait_limit(self, polls=None):
        """Bound of the FP32 push's waits on its shared-memory barriers, in
        polls of about 20 us (None: the default, about 1 s; 0: every wait
        gives up at once). A wait that gives up makes the step raise
        GpuPathError with status E_TIMEOUT."""
        _check(library().ipic3d_gpu_set_wait_limit(self._ctx, -1 if polls is None else int(polls)))

    @property
    def stream(self):
        return library().ipic3d_gpu_stream(self._ctx)


class Batch:
    """Independent universes advanced together, one launch per kernel of the
    timestep (ipic3d_gpu_batch_*). ``props`` is a sequence of Props (one per
    universe, sizes may differ); ``config`` is shared. ``universe(i)`` is a
    Simulation view of universe i for uploads, downloads and diagnostics; it
    stays valid until the batch is closed."""

    def __init__(self, props, config=None):
        self.props = list(props)
        self.config = config if config is not None else Config.make()
        arr = (Props * len(self.props))(*self.props)
        b = C.c_void_p()
        _check(library().ipic3d_gpu_batch_create(len(self.props), arr, C.byref(self.config), C.byref(b)))
        self._b = b
        self._views = {}

    def __len__(self):
        return len(self.props)

    def close(self):
        if getattr(self, "_b", None):
            for v in self._views.values():
                v._ctx = None
            self._views = {}
            library().ipic3d_gpu_batch_destroy(self._b)
            self._b = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def universe(self, i):
        if i not in self._views:
            ctx = C.c_void_p()
            _check(library().ipic3d_gpu_batch_universe(self._b, int(i), C.byref(ctx)))
            self._views[i] = Simulation(self.props[i], self.config, _lent=ctx)
        return self._views[i]

    def step(self, n=1):
        _check(library().ipic3d_gpu_batch_step(self._b, int(n)))

    def synchronize(self):
        _check(library().ipic3d_gpu_batch_synchronize(self._b))

    def stats(self):
        out = Stats()
        _check(library().ipic3d_gpu_batch_stats(self._b, C.byref(out)))
        return out.as_dict()

    def push_shape(self):
        out = abi.PushShape()
        _check(library().ipic3d_gpu_batch_get_push_shape(self._b, C.byref(out)))
        return out.as_dict()

    @property
    def stream(self):
        return library().ipic3d_gpu_batch_stream(self._b)

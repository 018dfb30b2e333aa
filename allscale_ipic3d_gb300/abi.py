"""ctypes mirror of the plain-C types in include/ipic3d_types.h and
include/ipic3d_gpu.h.

The structures follow the AllScale iPIC3D reference one to one:
``Props`` is ``UniverseProperties`` (universe_properties.h:52-123),
``PARTICLE_DTYPE`` is ``Particle`` (particle.h:9-60, 64 bytes) and the field
arrays are ``Field`` / ``BcField`` / ``CurrentDensity`` (field.h:14-38).
"""
import ctypes as C

import numpy as np

# ---- status codes (ipic3d_gpu.h) ------------------------------------------
OK = 0
E_INVALID = -1
E_NOMEM = -2
E_CUDA = -3
E_CAPACITY = -4
E_NODEVICE = -5
E_STATE = -6
E_TIMEOUT = -7

# ---- enums -----------------------------------------------------------------
FP64, FP32 = 0, 1
MOVER_DIPOLE, MOVER_FIELD = 0, 1
SOLVER_STATIC, SOLVER_LEAPFROG, SOLVER_FORWARD = 0, 1, 2
PROJECT_NONE, PROJECT_CIC = 0, 1
BC_REFLECT, BC_PERIODIC, BC_OPEN = 0, 1, 2

F_J_DIV8 = 1 << 0
F_GATHER_DIV_VOL = 1 << 1
F_DIPOLE_IN_GATHER = 1 << 2
F_REFRESH_NODE_B = 1 << 3
F_TRACK_IDS = 1 << 4
F_INJECT_LOW_X = 1 << 5
F_USE_GRAPH = 1 << 6

FIELD_NODE_DOUBLES = 9
BC_CELL_DOUBLES = 3
DENSITY_NODE_DOUBLES = 3


class Props(C.Structure):
    """UniverseProperties (universe_properties.h:52-123)."""

    _fields_ = [
        ("size", C.c_int64 * 3),
        ("cell_width", C.c_double * 3),
        ("dt", C.c_double),
        ("speed_of_light", C.c_double),
        ("planet_radius", C.c_double),
        ("object_center", C.c_double * 3),
        ("origin", C.c_double * 3),
        ("external_b", C.c_double * 3),
    ]

    @classmethod
    def make(cls, size=(1, 1, 1), cell_width=(1.0, 1.0, 1.0), dt=1.0, speed_of_light=1.0, planet_radius=0.0,
             object_center=(0.0, 0.0, 0.0), origin=(0.0, 0.0, 0.0), external_b=(0.0, 0.0, 0.0)):
        """Defaults are those of UniverseProperties' constructor
        (universe_properties.h:79)."""
        p = cls()
        p.size[:] = [int(v) for v in size]
        p.cell_width[:] = [float(v) for v in cell_width]
        p.dt = float(dt)
        p.speed_of_light = float(speed_of_light)
        p.planet_radius = float(planet_radius)
        p.object_center[:] = [float(v) for v in object_center]
        p.origin[:] = [float(v) for v in origin]
        p.external_b[:] = [float(v) for v in external_b]
        return p

    @property
    def shape(self):
        return tuple(int(v) for v in self.size)

    @property
    def ncells(self):
        s = self.shape
        return s[0] * s[1] * s[2]


class Config(C.Structure):
    """ipic3d_config: the simulateSteps policy arguments (simulator.h:42-47)."""

    _fields_ = [
        ("precision", C.c_int32),
        ("mover", C.c_int32),
        ("solver", C.c_int32),
        ("projector", C.c_int32),
        ("bc_low", C.c_int32 * 3),
        ("bc_high", C.c_int32 * 3),
        ("flags", C.c_uint32),
        ("slack", C.c_double),
        ("slack_min", C.c_int32),
        ("block_size", C.c_int32),
        ("inject_per_cell", C.c_double),
        ("inject_q", C.c_double),
        ("inject_qom", C.c_double),
        ("inject_drift", C.c_double * 3),
        ("inject_vth", C.c_double * 3),
        ("seed", C.c_uint64),
        ("reserved", C.c_uint64 * 8),
    ]

    @classmethod
    def make(cls, precision=FP64, mover=MOVER_DIPOLE, solver=SOLVER_STATIC, projector=PROJECT_NONE,
             bc=BC_REFLECT, bc_low=None, bc_high=None, flags=0, slack=0.0, slack_min=0, block_size=0,
             inject_per_cell=0.0, inject_q=0.0, inject_qom=0.0, inject_drift=(0.0, 0.0, 0.0),
             inject_vth=(0.0, 0.0, 0.0), seed=12345):
        c = cls()
        c.precision, c.mover, c.solver, c.projector = precision, mover, solver, projector
        c.bc_low[:] = list(bc_low) if bc_low is not None else [bc] * 3
        c.bc_high[:] = list(bc_high) if bc_high is not None else [bc] * 3
        c.flags = flags
        c.slack, c.slack_min, c.block_size = slack, slack_min, block_size
        c.inject_per_cell, c.inject_q, c.inject_qom = inject_per_cell, inject_q, inject_qom
        c.inject_drift[:] = list(inject_drift)
        c.inject_vth[:] = list(inject_vth)
        c.seed = seed
        return c


class Conserved(C.Structure):
    _fields_ = [
        ("total_momentum", C.c_double),
        ("e_energy", C.c_double),
        ("b_energy", C.c_double),
        ("kinetic_energy", C.c_double),
        ("total_charge", C.c_double),
        ("particles", C.c_uint64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("steps", "particles", "capacity", "migrated_last", "removed_last",
                                            "injected_last", "rebuilds", "kernel_launches", "pending_last",
                                            "relayout_steps")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PushShape(C.Structure):
    _fields_ = [("item", C.c_int32), ("item_cells", C.c_int32), ("blocks_per_sm", C.c_int32), ("tuned", C.c_int32),
                ("tuning", C.c_int32), ("trials", C.c_int32), ("push_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


PHASES = ["push", "pending", "inject", "place", "fields", "moments", "unused6", "unused7"]


class Profile(C.Structure):
    _fields_ = [("ms", C.c_double * 8), ("launches", C.c_uint64 * 8), ("particles", C.c_uint64 * 8)]

    def as_dict(self):
        return {PHASES[i]: {"ms": self.ms[i], "launches": self.launches[i], "particles": self.particles[i]}
                for i in range(6)}


# Particle (particle.h:9-60): 8 doubles, 64 bytes
PARTICLE_DTYPE = np.dtype([("position", "<f8", (3,)), ("velocity", "<f8", (3,)), ("q", "<f8"), ("qom", "<f8")])
assert PARTICLE_DTYPE.itemsize == 64


def field_shape(props):
    s = props.shape
    return (s[0] + 3, s[1] + 3, s[2] + 3, FIELD_NODE_DOUBLES)


def bcfield_shape(props):
    s = props.shape
    return (s[0] + 2, s[1] + 2, s[2] + 2, BC_CELL_DOUBLES)


def density_shape(props):
    s = props.shape
    return (s[0] + 1, s[1] + 1, s[2] + 1, DENSITY_NODE_DOUBLES)


def ptr(a, ctype=C.c_double):
    """Pointer to a contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(ctype))


def vptr(a):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)

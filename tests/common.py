"""Shared helpers of the test suite: scenario builders, runners for the GPU
library and the CPU oracle, and comparisons by particle id."""
import ctypes as C
import json
import os

import numpy as np

import oracle
from allscale_ipic3d_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_npz(name):
    return np.load(os.path.join(GOLDEN, name))


def golden_json(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def props_from_vec(v):
    v = [float(x) for x in v]
    return abi.Props.make(size=[int(x) for x in v[0:3]], cell_width=v[3:6], dt=v[6], speed_of_light=v[7],
                          planet_radius=v[8], object_center=v[9:12], origin=v[12:15], external_b=v[15:18])


def props_from_dict(d):
    return abi.Props.make(**d)


def reference_config(**kw):
    """The reference's default simulateSteps policies (simulator.h:42-47)."""
    return abi.Config.make(**kw)


def scenario(seed, size, width=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0), dt=0.1, ppc=8, vscale=0.3, planet=0.0,
             bz=0.0, c=1.0, species=((1.0, 1.0),), ragged=False):
    """Seeded particles, uniform inside their cells, grouped by cell."""
    rng = np.random.default_rng(seed)
    props = abi.Props.make(size=size, cell_width=width, dt=dt, speed_of_light=c, planet_radius=planet,
                           origin=origin, external_b=(0.0, 0.0, bz))
    s = np.array(size)
    nc = int(np.prod(s))
    if ragged:
        per = rng.integers(0, 2 * ppc + 1, nc)
        per[rng.random(nc) < 0.2] = 0
    else:
        per = np.full(nc, ppc)
    n = int(per.sum())
    cell = np.repeat(np.arange(nc), per)
    cz, cy, cx = cell % s[2], (cell // s[2]) % s[1], cell // (s[1] * s[2])
    pos = np.array(origin) + (np.stack([cx, cy, cz], 1) + rng.random((n, 3))) * np.array(width)
    p = np.zeros(n, abi.PARTICLE_DTYPE)
    p["position"] = pos
    p["velocity"] = rng.normal(0.0, vscale, (n, 3))
    sp = rng.integers(0, len(species), n)
    p["q"] = np.array([q for q, _ in species])[sp]
    p["qom"] = np.array([m for _, m in species])[sp]
    return props, p, per.astype(np.uint64)


class OracleSim:
    """ctypes wrapper of the CPU oracle with the GPU Simulation's methods."""

    def __init__(self, props, cfg):
        self.lib = oracle.load()
        self.props = props
        self.s = C.c_void_p()
        assert self.lib.oracle_create(C.byref(props), C.byref(cfg), C.byref(self.s)) == 0

    def close(self):
        if self.s:
            self.lib.oracle_destroy(self.s)
            self.s = None

    __del__ = close

    def upload_particles(self, p, counts, ids=None):
        p = np.ascontiguousarray(p, abi.PARTICLE_DTYPE)
        counts = np.ascontiguousarray(counts, np.uint64)
        i = None if ids is None else np.ascontiguousarray(ids, np.uint32)
        self.lib.oracle_upload_particles(self.s, abi.vptr(p), abi.vptr(counts), abi.vptr(i))

    def upload_fields(self, field=None, bcfield=None, density=None):
        a = [None if x is None else np.ascontiguousarray(x, np.float64) for x in (field, bcfield, density)]
        self.lib.oracle_upload_fields(self.s, *[abi.vptr(x) for x in a])

    def download_fields(self):
        f = np.zeros(abi.field_shape(self.props))
        b = np.zeros(abi.bcfield_shape(self.props))
        d = np.zeros(abi.density_shape(self.props))
        r = np.zeros(abi.density_shape(self.props)[:3])
        self.lib.oracle_download_fields(self.s, abi.vptr(f), abi.vptr(b), abi.vptr(d), abi.vptr(r))
        return f, b, d, r

    def step(self, n=1):
        assert self.lib.oracle_step(self.s, int(n)) == 0

    def project(self):
        self.lib.oracle_project(self.s)

    def update_boundaries(self):
        self.lib.oracle_update_boundaries(self.s)

    def solve_fields(self):
        self.lib.oracle_solve_fields(self.s)

    def move(self):
        self.lib.oracle_move(self.s)

    def download_particles(self):
        n = self.lib.oracle_particle_count(self.s)
        p = np.zeros(n, abi.PARTICLE_DTYPE)
        c = np.zeros(self.props.ncells, np.uint64)
        i = np.zeros(n, np.uint32)
        self.lib.oracle_download_particles(self.s, abi.vptr(p), n, abi.vptr(c), abi.vptr(i))
        return p, c, i

    def cell_counts(self):
        return self.download_particles()[1]

    def conserved(self):
        out = abi.Conserved()
        self.lib.oracle_conserved(self.s, C.byref(out))
        return out.as_dict()


def gpu_sim(props, cfg):
    from allscale_ipic3d_gb300 import Simulation
    return Simulation(props, cfg)


def cell_of_each(counts):
    return np.repeat(np.arange(len(counts)), counts.astype(np.int64))


def align_by_id(a, b):
    """Matches two (particles, counts, ids) triples particle by particle.
    Asserts that every cell holds the same set of ids (integer parity) and
    returns the two particle arrays in a common order."""
    pa, ca, ia = a
    pb, cb, ib = b
    np.testing.assert_array_equal(ca, cb, err_msg="per-cell counts differ")
    cella = cell_of_each(ca)
    cellb = cell_of_each(cb)
    ka = np.lexsort((ia, cella))
    kb = np.lexsort((ib, cellb))
    np.testing.assert_array_equal(ia[ka], ib[kb], err_msg="particle ids per cell differ")
    return pa[ka], pb[kb]


def assert_states_close(pa, pb, rtol, atol, what=""):
    for f in ("position", "velocity"):
        np.testing.assert_allclose(pa[f], pb[f], rtol=rtol, atol=atol, err_msg="%s %s" % (what, f))
    np.testing.assert_array_equal(pa["q"], pb["q"])
    np.testing.assert_array_equal(pa["qom"], pb["qom"])


def init_inp(run):
    """The initial universe of an .inp driver run (fixture inp_runs.json),
    rebuilt by the oracle's restatement of the reference's initCells."""
    props = props_from_dict(run["props"])
    lib = oracle.load()
    n = C.c_uint64()
    arr = [np.ascontiguousarray(run[k], np.float64) for k in ("low", "hig", "mean", "stddev")]
    lib.oracle_init_uniform_pos_normal_speed(C.byref(props), run["num_particles"], *[abi.vptr(a) for a in arr],
                                             None, None, C.byref(n))
    parts = np.zeros(n.value, abi.PARTICLE_DTYPE)
    counts = np.zeros(props.ncells, np.uint64)
    lib.oracle_init_uniform_pos_normal_speed(C.byref(props), run["num_particles"], *[abi.vptr(a) for a in arr],
                                             abi.vptr(parts), abi.vptr(counts), C.byref(n))
    return props, parts, counts


def sha(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()

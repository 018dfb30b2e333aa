"""Generates the golden fixtures in this folder by running the reference's own
code: the AllScale iPIC3D headers compiled against the AllScale shim into
oracle/_ref/libipic3d_ref.so (oracle/ref/Makefile; needs the reference
sources, so this script runs on the build machine only).

    python tests/golden/make_golden.py

Fixtures (all small):
  inp_runs.json      test.inp / tiny.inp driver runs (src/ipic3d.cxx): the
                     distribution parameters, sha256 of the initial and final
                     particle bytes, per-cell counts after ncycles steps and
                     the conserved quantities; `trace`: the conserved
                     quantities before every cycle, as the reference's debug
                     build writes them (simulator.h:65-90). The shipped
                     outputs/<name>ConservedQuantities.out come from an older
                     initialisation; only their field-energy columns agree
                     with the current sources, and those are checked here.
  moves_small.npz    seeded scenarios through simulateSteps with the default
                     policies (mover + export + import): inputs and outputs.
  project_small.npz  projectToDensityField over all nodes.
  dumps_small.npz    outputParticlePositions and outputFieldGrids text of a
                     small universe (the reference's writers).
  fields_small.npz   updateFieldsOnBoundaries, two-phase leapfrog, forward
                     solver at single nodes.
  aggregate_small.npz  aggregateDensityContributions over all nodes of two
                     grids from seeded contribution grids and starting J.
  tracer_runs.json   the standalone tracer (src/pic_tracer.cxx, built as
                     oracle/_ref/pic_tracer_ref) run as `pic_tracer N T S R`:
                     the per-frame histograms it writes (result_*.csv.NNNNNN),
                     in full for the small cases, as sha256 of the uint32
                     counts plus per-frame totals for the larger one, and the
                     sha256 of each frame file's text.
"""
import ctypes as C
import glob
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from allscale_ipic3d_gb300 import abi  # noqa: E402

ref = oracle.load_reference()
if ref is None:
    sys.exit("the reference library could not be built (reference sources missing?)")


def props_to_dict(p):
    return {"size": list(p.size), "cell_width": list(p.cell_width), "dt": p.dt, "speed_of_light": p.speed_of_light,
            "planet_radius": p.planet_radius, "object_center": list(p.object_center), "origin": list(p.origin),
            "external_b": list(p.external_b)}


def props_vec(p):
    """props as a flat float64 vector (size, width, dt, c, R, center, origin, Bext)."""
    return np.array(list(p.size) + list(p.cell_width) + [p.dt, p.speed_of_light, p.planet_radius] +
                    list(p.object_center) + list(p.origin) + list(p.external_b), np.float64)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()


def ref_simulate(props, parts, counts, steps):
    n = len(parts)
    out = np.zeros(n, abi.PARTICLE_DTYPE)
    oc = np.zeros(props.ncells, np.uint64)
    ids = np.zeros(n, np.uint32)
    rc = ref.ref_simulate_default(C.byref(props), abi.vptr(parts), abi.vptr(counts), steps, abi.vptr(out), n,
                                  abi.vptr(oc), abi.vptr(ids))
    assert rc == 0
    m = int(oc.sum())
    return out[:m].copy(), oc, ids[:m].copy()


def trace_line(row):
    """One line of the reference's ConservedQuantities.out: the cycle and four
    doubles in the default C++ stream format (6 significant digits), tab
    separated (simulator.h:83-89)."""
    return "\t".join([str(int(row[0]))] + ["%g" % v for v in row[1:]])


def inp_runs():
    res = {}
    for name in ("test", "tiny"):
        path = os.path.join(oracle.reference_root(), "inputs", name + ".inp").encode()
        props = abi.Props()
        ncyc = C.c_uint64()
        n = C.c_uint64()
        ref.ref_init_from_inp(path, C.byref(props), C.byref(ncyc), None, 0, None, C.byref(n), None)
        N = n.value
        parts = np.zeros(N, abi.PARTICLE_DTYPE)
        counts = np.zeros(props.ncells, np.uint64)
        field = np.zeros(abi.field_shape(props))
        ref.ref_init_from_inp(path, C.byref(props), C.byref(ncyc), abi.vptr(parts), N, abi.vptr(counts),
                              C.byref(n), abi.vptr(field))
        usize = np.array(props.cell_width) * np.array(props.size)
        low = np.array(props.origin) + 0.125 * usize
        hig = low + 0.75 * usize
        c, e, m = 299792458.0, 1.602176565e-19, 1.672621777e-27
        vmod = c / np.sqrt(1.0 + (m * c * c) / (1e7 * e))
        steps = ncyc.value
        # the conserved quantities before every cycle (writeOutputData with
        # FieldOutputCycle 1): one step at a time
        trace = []
        cur, cur_counts = parts, counts
        for i in range(steps):
            cq = abi.Conserved()
            ref.ref_conserved(C.byref(props), abi.vptr(cur), abi.vptr(cur_counts), abi.vptr(field), C.byref(cq))
            trace.append([i, cq.total_momentum, cq.e_energy, cq.b_energy, cq.kinetic_energy])
            cur, cur_counts, _ = ref_simulate(props, cur, cur_counts, 1)
        ref_lines = open(os.path.join(oracle.reference_root(), "outputs", name + "ConservedQuantities.out")).read()
        ref_cols = {int(c[0]): c for c in (l.split("\t") for l in ref_lines.strip().splitlines()[1:])}
        for row in trace:  # the file's cycles (its own output cycle): E energy, B energy
            line = trace_line(row).split("\t")
            if row[0] in ref_cols:
                assert [line[2], line[3]] == ref_cols[row[0]][2:4], (name, line, ref_cols[row[0]])
        out, oc, ids = ref_simulate(props, parts, counts, steps)
        cons = abi.Conserved()
        ref.ref_conserved(C.byref(props), abi.vptr(out), abi.vptr(oc), abi.vptr(field), C.byref(cons))
        res[name] = {
            "props": props_to_dict(props), "num_particles": N, "ncycles": steps,
            "low": low.tolist(), "hig": hig.tolist(), "mean": [0.0, 0.0, 0.0], "stddev": [vmod] * 3,
            "initial_counts_sha256": sha(counts), "initial_particles_sha256": sha(parts),
            "final_counts": oc.tolist(), "final_total": int(oc.sum()),
            "final_particles_sha256": sha(out), "final_ids_sha256": sha(ids),
            "conserved": cons.as_dict(), "trace": trace,
        }
        print(name, N, "->", int(oc.sum()))
    with open(os.path.join(HERE, "inp_runs.json"), "w") as f:
        json.dump(res, f, indent=1)


def tracer_runs():
    exe = os.path.join(oracle.REF_DIR, "pic_tracer_ref")
    res = []
    for N, T, S, R, full in ((4000, 40, 10, 8, True), (3000, 23, 7, 12, True), (5000, 150, 10, 32, False)):
        frames = T // S + 1
        with tempfile.TemporaryDirectory() as d:
            subprocess.check_call([exe, str(N), str(T), str(S), str(R)], cwd=d, stdout=subprocess.DEVNULL)
            counts = np.zeros((frames, R, R, R), np.uint32)
            texts = []
            for t in range(frames):
                (path,) = glob.glob(os.path.join(d, "result_*.csv.%06d" % t))
                text = open(path, "rb").read()
                texts.append(hashlib.sha256(text).hexdigest())
                rows = [l.split(b",") for l in text.splitlines()[1:]]
                counts[t] = np.array([int(r[4]) for r in rows], np.uint32).reshape(R, R, R)
        case = {"N": N, "T": T, "S": S, "R": R, "frames": frames, "frame_totals": counts.sum(axis=(1, 2, 3)).tolist(),
                "counts_sha256": sha(counts), "file_sha256": texts}
        if full:
            case["counts"] = counts.ravel().tolist()
        res.append(case)
        print("tracer", N, T, S, R, case["frame_totals"])
    with open(os.path.join(HERE, "tracer_runs.json"), "w") as f:
        json.dump(res, f)


def scatter_into_cells(props, pos, rng_order=None):
    """Groups particles by the cell their position falls in (row-major)."""
    s = np.array(props.size)
    w = np.array(props.cell_width)
    o = np.array(props.origin)
    c = np.floor((pos - o) / w).astype(np.int64)
    c = np.clip(c, 0, s - 1)
    flat = (c[:, 0] * s[1] + c[:, 1]) * s[2] + c[:, 2]
    order = np.argsort(flat, kind="stable")
    counts = np.bincount(flat, minlength=props.ncells).astype(np.uint64)
    return order, counts


def make_scenario(seed, size, width, origin, dt, ppc, vscale, planet=0.0, bz=0.0, qom=1.0, q=1.0, ragged=False):
    rng = np.random.default_rng(seed)
    props = abi.Props.make(size=size, cell_width=width, dt=dt, speed_of_light=1.0, planet_radius=planet,
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
    cz = cell % s[2]
    cy = (cell // s[2]) % s[1]
    cx = cell // (s[1] * s[2])
    frac = rng.random((n, 3))
    pos = np.array(origin) + (np.stack([cx, cy, cz], 1) + frac) * np.array(width)
    parts = np.zeros(n, abi.PARTICLE_DTYPE)
    parts["position"] = pos
    parts["velocity"] = rng.normal(0.0, vscale, (n, 3))
    parts["q"] = q
    parts["qom"] = qom
    # two species in some scenarios
    if seed % 2 == 1 and n:
        sel = rng.random(n) < 0.3
        parts["q"][sel] = -q
        parts["qom"][sel] = -qom * 0.5
    counts = per.astype(np.uint64)
    return props, parts, counts


SCENARIOS = {
    # name: (kwargs, steps)
    "walls": (dict(seed=1, size=(4, 4, 4), width=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0), dt=0.5, ppc=8,
                   vscale=0.6), 12),
    "dipole": (dict(seed=2, size=(6, 6, 6), width=(1.0, 1.0, 1.0), origin=(-3.0, -3.0, -3.0), dt=0.1, ppc=8,
                    vscale=0.3, planet=1.0, bz=2.0, qom=-1.0), 10),
    "ragged": (dict(seed=3, size=(5, 3, 2), width=(0.5, 1.0, 2.0), origin=(-1.0, 0.5, -2.0), dt=0.2, ppc=10,
                    vscale=0.8, planet=0.3, bz=1.5, qom=2.0, ragged=True), 8),
    "single": (dict(seed=4, size=(1, 1, 1), width=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0), dt=0.3, ppc=16,
                    vscale=1.0), 5),
    "fast": (dict(seed=5, size=(4, 4, 4), width=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0), dt=1.0, ppc=4,
                  vscale=1.5), 6),
    "strong": (dict(seed=7, size=(8, 8, 8), width=(0.5, 0.5, 0.5), origin=(-2.0, -2.0, -2.0), dt=0.05, ppc=6,
                    vscale=0.5, planet=0.4, bz=40.0, qom=-3.0), 6),
}


def moves_small():
    out = {}
    for name, (kw, steps) in SCENARIOS.items():
        props, parts, counts = make_scenario(**kw)
        res, rc, ids = ref_simulate(props, parts, counts, steps)
        out[name + "_props"] = props_vec(props)
        out[name + "_in"] = parts
        out[name + "_in_counts"] = counts
        out[name + "_steps"] = np.array([steps])
        out[name + "_out"] = res
        out[name + "_out_counts"] = rc
        out[name + "_out_ids"] = ids
        print(name, len(parts), "->", len(res))
    np.savez_compressed(os.path.join(HERE, "moves_small.npz"), **out)


def project_small():
    out = {}
    for name, kw in {"p3": dict(seed=11, size=(3, 3, 3), width=(0.5, 0.5, 0.5), origin=(0.0, 0.0, 0.0), dt=0.1,
                                ppc=6, vscale=1.0),
                     "p435": dict(seed=12, size=(4, 3, 5), width=(1.0, 2.0, 0.5), origin=(-1.0, 0.0, 1.0), dt=0.1,
                                  ppc=5, vscale=1.0, ragged=True)}.items():
        props, parts, counts = make_scenario(**kw)
        J = np.zeros(abi.density_shape(props))
        ref.ref_project_current(C.byref(props), abi.vptr(parts), abi.vptr(counts), abi.vptr(J))
        out[name + "_props"] = props_vec(props)
        out[name + "_in"] = parts
        out[name + "_in_counts"] = counts
        out[name + "_J"] = J
    np.savez_compressed(os.path.join(HERE, "project_small.npz"), **out)


def aggregate_small():
    out = {}
    for name, seed, size, width in (("a3", 21, (3, 3, 3), (0.5, 0.5, 0.5)), ("a425", 22, (4, 2, 5), (1.0, 2.0, 0.75))):
        props = abi.Props.make(size=size, cell_width=width, dt=0.1)
        rng = np.random.default_rng(seed)
        contrib = rng.normal(0.0, 1.0, tuple(2 * v for v in size) + (3,))
        J0 = rng.normal(0.0, 1.0, abi.density_shape(props))
        J = J0.copy()
        ref.ref_aggregate_contributions(C.byref(props), abi.vptr(contrib), abi.vptr(J))
        out[name + "_props"] = props_vec(props)
        out[name + "_contrib"] = contrib
        out[name + "_J0"] = J0
        out[name + "_J"] = J
    np.savez_compressed(os.path.join(HERE, "aggregate_small.npz"), **out)


def dumps_small():
    """The reference's text dumps -- outputParticlePositions (cell.h:1400-1429)
    and outputFieldGrids (field.h:464-530) -- of a small universe with
    particles over several orders of magnitude and random fields."""
    import tempfile
    ref = oracle.load_reference()
    # one species (even seed): the GPU keeps a cell's particles in upload
    # order within a species
    props, parts, counts = make_scenario(70, (4, 3, 5), (0.5, 2.0, 1e-3), (-1.0, 3.0, 1e4), 0.1, 6, 0.3,
                                         ragged=True)
    rng = np.random.default_rng(72)
    f = rng.normal(0.0, 1.0, abi.field_shape(props)) * 10.0 ** rng.integers(-8, 8, abi.field_shape(props))
    bc = rng.normal(0.0, 1.0, abi.bcfield_shape(props))
    with tempfile.TemporaryDirectory() as d:
        pp, pf = os.path.join(d, "positions.txt"), os.path.join(d, "fields.txt")
        ref.ref_write_particle_positions(C.byref(props), abi.vptr(parts), abi.vptr(counts), pp.encode())
        ref.ref_write_field_grids(C.byref(props), abi.vptr(f), abi.vptr(bc), pf.encode())
        pos_text, field_text = open(pp, "rb").read(), open(pf, "rb").read()
    np.savez_compressed(os.path.join(HERE, "dumps_small.npz"), props=props_vec(props), parts=parts, counts=counts,
                        field=f, bcfield=bc, positions_txt=np.frombuffer(pos_text, np.uint8),
                        field_grids_txt=np.frombuffer(field_text, np.uint8))


def fields_small():
    rng = np.random.default_rng(21)
    out = {}
    props = abi.Props.make(size=(4, 4, 4), cell_width=(1.0, 0.5, 2.0), dt=0.05, speed_of_light=1.3)
    f0 = rng.normal(0, 1, abi.field_shape(props))
    b0 = rng.normal(0, 1, abi.bcfield_shape(props))
    j0 = rng.normal(0, 1, abi.density_shape(props))
    f1, b1 = f0.copy(), b0.copy()
    ref.ref_update_boundaries(C.byref(props), abi.vptr(f1), abi.vptr(b1))
    f2, b2 = f0.copy(), b0.copy()
    ref.ref_leapfrog_two_phase(C.byref(props), abi.vptr(f2), abi.vptr(b2), abi.vptr(j0))
    out.update(props=props_vec(props), field=f0, bcfield=b0, J=j0, bnd_field=f1, bnd_bcfield=b1, lf_field=f2,
               lf_bcfield=b2)
    # forward solver at three interior nodes, each on the initial fields
    nodes = np.array([[2, 2, 2], [1, 3, 2], [4, 4, 1]], np.int64)
    ff, fb = [], []
    for nd in nodes:
        f3, b3 = f0.copy(), b0.copy()
        ref.ref_solve_forward_at(C.byref(props), abi.vptr(np.ascontiguousarray(nd)), abi.vptr(f3), abi.vptr(b3),
                                 abi.vptr(j0))
        ff.append(f3)
        fb.append(b3)
    out.update(fw_nodes=nodes, fw_field=np.stack(ff), fw_bcfield=np.stack(fb))
    np.savez_compressed(os.path.join(HERE, "fields_small.npz"), **out)


if __name__ == "__main__":
    moves_small()
    project_small()
    fields_small()
    inp_runs()
    tracer_runs()
    aggregate_small()
    dumps_small()

"""Parity at the benchmark sizes (the other parity tests use small grids):
the FP64 GPU path against the CPU oracle on the dipole magnetosphere
workload (32^3 cells, 8,388,608 particles, injection at -x, outflow at +x,
leapfrog fields, CIC deposit) and on the uneven-load (64^3, 134M particles)
and large (128^3, 268M particles) configurations. Integer results (per-cell
counts, which particle ends where) are compared bit for bit; particle states
and fields at the FP64 path's tolerance (FP64 atomics make the deposit's
summation order free)."""
import os
import sys

import numpy as np
import pytest

from allscale_ipic3d_gb300 import abi
from common import OracleSim, gpu_sim

sys.path.insert(0, os.path.abspath(os.path.join(os.path.dirname(__file__), "..")))
import bench  # noqa: E402  (the benchmark's workload generators)

pytestmark = pytest.mark.gpu


def run_pair(props, parts, counts, cfg_gpu, cfg_cpu, steps, fields=None):
    ids = np.arange(len(parts), dtype=np.uint32)
    sim = gpu_sim(props, cfg_gpu)
    orc = OracleSim(props, cfg_cpu)
    for s in (sim, orc):
        if fields is not None:
            s.upload_fields(fields[0], fields[1], None)
        s.upload_particles(parts, counts, ids)
        s.step(steps)
    a, b = bench.state_of(sim), bench.state_of(orc)
    sim.close()
    orc.close()
    return a, b


def check_particles(a, b, props, tol):
    err = bench.particle_error(a[0], b[0], props)
    assert err["cell_counts"]["cells_differing"] == 0, err
    assert err["only_first"] == 0 and err["only_second"] == 0, err
    assert err["injected"][0] == err["injected"][1], err
    assert err["position_cells"]["max"] <= tol and err["velocity_rel"]["max"] <= tol, err
    return err


def test_headline_fp64_matches_oracle():
    props, parts, counts = bench.make_workload(12345)
    cg = bench.make_config(abi.FP64, graph=True)
    cc = bench.make_config(abi.FP64, graph=False)
    for c in (cg, cc):
        c.flags |= abi.F_TRACK_IDS
    a, b = run_pair(props, parts, counts, cg, cc, 5)
    check_particles(a, b, props, 1e-12)
    for k, (x, y) in {"E": (a[1][0][..., 0:3], b[1][0][..., 0:3]), "Bc": (a[1][1], b[1][1])}.items():
        e = bench.array_error(x, y)
        assert e["max_rel_to_peak"] <= 1e-12, (k, e)
    assert a[2]["particles"] == b[2]["particles"]
    assert abs(a[2]["kinetic_energy"] - b[2]["kinetic_energy"]) <= 1e-12 * abs(b[2]["kinetic_energy"])


def test_headline_fp32_against_oracle():
    """FP32 cell-relative path against the FP64 CPU oracle after 5 steps:
    energy at the FP32 bar, positions within 1e-4 cells, counts: every
    difference is a particle within FP32 rounding of a cell face."""
    props, parts, counts = bench.make_workload(12345)
    cg = bench.make_config(abi.FP32, graph=True)
    cc = bench.make_config(abi.FP64, graph=False)
    for c in (cg, cc):
        c.flags |= abi.F_TRACK_IDS
    a, b = run_pair(props, parts, counts, cg, cc, 5)
    err = bench.particle_error(a[0], b[0], props)
    assert err["position_cells"]["max"] < 1e-4, err
    assert err["only_first"] + err["only_second"] <= 2, err
    assert err["cell_counts"]["sum_abs_difference"] <= 4, err
    ke = abs(a[2]["kinetic_energy"] - b[2]["kinetic_energy"]) / abs(b[2]["kinetic_energy"])
    assert ke <= 1e-5, ke


@pytest.mark.parametrize("name", ["c3", "c5"])
def test_large_configs_fp64_counts_match_oracle(name):
    desc, props, parts, counts, fields, kw, _ = {"c3": bench.config_c3, "c5": bench.config_c5}[name]()
    flags = kw.pop("flags") & ~abi.F_USE_GRAPH
    cg = abi.Config.make(precision=abi.FP64, flags=flags | abi.F_TRACK_IDS | abi.F_USE_GRAPH, **kw)
    cc = abi.Config.make(precision=abi.FP64, flags=flags | abi.F_TRACK_IDS, **kw)
    a, b = run_pair(props, parts, counts, cg, cc, 1, fields)
    check_particles(a, b, props, 1e-12)

"""The FP64 kernels' r^2.5 (pow25_core, particle_kernels.cuh) equals the
correctly rounded a^2.5 -- what the reference's libm pow returns -- when run
on the host with the device's reciprocal square root anywhere within its 1
ulp error bound (tests/cpp/pow25_emulation.c), on log-uniform arguments over
the dipole's range, on squares (exact midpoints round to even) and on
integers; the reference values are 300-bit evaluations."""
import os
import shutil
import subprocess

import numpy as np
import pytest

mpmath = pytest.importorskip("mpmath")
HERE = os.path.dirname(os.path.abspath(__file__))


def test_pow25_correctly_rounded(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "pow25")
    subprocess.check_call([cc, "-O2", "-ffp-contract=off", "-o", exe, os.path.join(HERE, "cpp", "pow25_emulation.c"),
                           "-lm"])
    rng = np.random.default_rng(2025)
    a = np.concatenate([10.0 ** rng.uniform(-100, 120, 20000), rng.uniform(1e13, 1e16, 10000),
                        np.floor(rng.uniform(1, 1e6, 10000)) ** 2, rng.integers(1, 10 ** 6, 5000).astype(float)])
    src = tmp_path / "in.bin"
    a.tofile(src)
    out = np.frombuffer(subprocess.run([exe, str(src)], capture_output=True, check=True).stdout,
                        np.float64).reshape(-1, 3)
    mpmath.mp.prec = 300
    want = np.array([float(mpmath.mpf(float(x)) ** mpmath.mpf(2.5)) for x in a])
    bad = np.nonzero((out != want[:, None]).any(axis=1))[0]
    assert len(bad) == 0, [(a[i], out[i], want[i]) for i in bad[:5]]

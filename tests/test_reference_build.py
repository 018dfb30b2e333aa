"""Builds the reference's own code against the AllScale shim (oracle/ref) and
runs the reference's unit tests: this pins the shim on which the fixtures in
tests/golden/ rest. Needs the reference sources (build machine only)."""
import os
import subprocess

import pytest

import oracle

REFERENCE = oracle.reference_root()
HAVE_REF = REFERENCE is not None


@pytest.mark.reference
@pytest.mark.skipif(not HAVE_REF, reason="reference sources not present on this machine")
def test_reference_unit_tests_pass_against_shim():
    r = subprocess.run(["make", "-s", "-C", os.path.join(oracle.HERE, "ref"), "check", "REF=" + REFERENCE],
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith(("PASS", "FAIL"))]
    assert len(lines) == 8, r.stdout
    assert all(l.startswith("PASS") for l in lines), r.stdout

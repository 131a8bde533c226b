"""The preconditioner's dependency waits are bounded: with one tile's flag
never published (ZS_TEST_STALL_TILE_TASK names that task), every wait on it
runs out, the launch gives up, and the call returns ZS_ERR_TIMEOUT instead of
hanging; the context stays usable (an FP64 solve and a mixed solve of
another size in the same process then succeed). Run in a child process so
that the setting stays out of the other tests."""

import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import time
import numpy as np
from zeroslam_gb300 import ba
rng = np.random.default_rng(0)
n = 200
G = rng.normal(size=(n, n)); A = G @ G.T / n + np.eye(n); b = rng.normal(size=n)
st = ba.dense_cholesky_status(A, b, precision=ba.MIXED)
assert st == ba.ZS_ERR_TIMEOUT, st
ok, _, x = ba.dense_cholesky_solve(A, b)
assert ok and np.max(np.abs(x - np.linalg.solve(A, b))) < 1e-9 * np.max(np.abs(x))
print("timeout reported, context usable")
"""


def test_stalled_dependency_times_out(zs_lib):
    env = dict(os.environ, ZS_TEST_STALL_TILE_TASK="0")
    r = subprocess.run([sys.executable, "-c", CHILD], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "timeout reported" in r.stdout

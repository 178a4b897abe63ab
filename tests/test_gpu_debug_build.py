"""The debug build (BBDG_DEBUG=1: every table-derived and neighbour index of the stage kernels
checked, a violation reported as a status bit instead of a trap) builds on the GPU machine,
gives the same results as the oracle on tiny cases and reports no violation. It runs in a
child process so that this process keeps the normal library."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys
sys.path[:0] = [ROOT, os.path.join(ROOT, "bernsteinbasis.jl_gb300")]
import numpy as np, torch, bbdg
from bbdg import _build
from oracle import cpu, meshdata
assert _build.DEBUG and _build.LIB.endswith(os.path.join("_build_debug", "libbbdg.so"))
_build.build()
worst = 0.0
m = bbdg.uniform_tet_mesh(4)
for physics, N, dtype, kind, tol in (("wave", 9, torch.float32, "specialised", 1e-5),
                                      ("maxwell", 5, torch.float32, "specialised", 1e-5),
                                      ("maxwell", 3, torch.float64, "generic", 1e-12)):
    md = meshdata.build(m, N)
    s = bbdg.DGSolver(m, N, physics, dtype=dtype, tau=1.0)
    s.set_kernel(kind)
    assert s.kernel == kind
    q = np.random.default_rng(N).uniform(-1, 1, (s.nf, m.K, s.Np))
    qd = torch.tensor(q, dtype=dtype, device="cuda")
    rd = torch.zeros_like(qd)
    dt = 0.1 * m.h / (N + 1) ** 2
    s.run(qd, rd, dt, 2)
    s.check()                                   # no debug index violation
    want, _ = cpu.lsrk(0 if physics == "wave" else 1, N, q, md, dt, 2, tau=1.0)
    got = qd.cpu().numpy()
    err = max(np.linalg.norm(got[f] - want[f]) / np.linalg.norm(want[f]) for f in range(s.nf))
    assert err < tol, (physics, N, kind, err)
    worst = max(worst, err)
print("debug build ok", worst)
"""


def test_debug_build_runs_clean_and_matches_the_oracle(cuda):
    env = dict(os.environ, BBDG_DEBUG="1")
    code = "ROOT = %r\n" % ROOT + CHILD
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-4000:])
    assert "debug build ok" in r.stdout

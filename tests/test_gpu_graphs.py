"""The optional CUDA-graph replay of the Nystrom factorisation and solve (KM_GRAPHS=1) gives the
same bits as direct launches, on first capture and on replays, in both precision forms."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
SCRIPT = r"""
import sys, hashlib, numpy as np
sys.path.insert(0, "kernelmatrices.jl_gb300")
import kmhodlr as K
from kmhodlr.data import uniform_points
n = 4096
pts = uniform_points(n, 5)
b = np.random.default_rng(6).standard_normal((n, 3))
out = []
for prec in (K.KM_PREC_FP64, K.KM_PREC_MIXED):
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, [1.0, 0.1, 1e-3], K.Matern32()), 0.0, 32, K.FixedLevel(4),
                       nystrom=True, precision=prec)
    for it in range(3):  # first call captures, the next ones replay
        K.symmetricfactorize(hk)
        x = hk.ldiv(b)
        out.append(hashlib.sha256(x.tobytes() + np.float64(hk.logdet()).tobytes()).hexdigest())
print(" ".join(out))
"""


def run(env_extra):
    env = dict(os.environ)
    env.pop("KM_GRAPHS", None)
    env.update(env_extra)
    r = subprocess.run([sys.executable, "-c", SCRIPT], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout.split()


def test_graph_replay_matches_direct_launches(lib):
    direct = run({})
    graphed = run({"KM_GRAPHS": "1"})
    assert graphed == direct
    assert direct[0] == direct[1] == direct[2] and direct[3] == direct[4] == direct[5]

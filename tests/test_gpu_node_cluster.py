"""The cluster form of the float-pair node kernel (the product phases of a node split over 2, 4 or
8 CTAs that exchange columns through distributed shared memory) gives the same bits as the
one-CTA form: every entry is the same sum in the same order, only the CTA that forms it
differs.  KM_NODE_CLUSTER caps the cluster size (1 = one CTA per node)."""
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
out = []
for n, rank, lvl, kern in ((16384, 72, 6, K.Matern32()), (8192, 40, 5, K.RatQuad())):
    pts = uniform_points(n, 11)
    b = np.random.default_rng(12).standard_normal((n, 4))
    params = [1.0, 0.1, 1e-3] if isinstance(kern, K.Matern32) else [1.0, 0.15, 1e-2]
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, params, kern), 0.0, rank, K.FixedLevel(lvl),
                       nystrom=True, precision=K.KM_PREC_MIXED)
    for it in range(2):
        K.symmetricfactorize(hk)
        x = hk.ldiv(b)
        out.append(hashlib.sha256(x.tobytes() + np.float64(hk.logdet()).tobytes()).hexdigest())
print(" ".join(out))
"""


def run(env_extra):
    env = dict(os.environ)
    env.pop("KM_GRAPHS", None)
    env.pop("KM_NODE_CLUSTER", None)
    env.update(env_extra)
    r = subprocess.run([sys.executable, "-c", SCRIPT], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout.split()


def test_node_cluster_forms_bit_identical(lib):
    one = run({"KM_NODE_CLUSTER": "1"})
    assert one[0] == one[1] and one[2] == one[3]
    for cap in ("2", "4", "8"):
        assert run({"KM_NODE_CLUSTER": cap}) == one, cap
    assert run({"KM_GRAPHS": "1"}) == one

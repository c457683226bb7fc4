"""The comparison switches select other kernels for the same algorithm; each is
read once per process, so every variant solves in a child process.  Launching
without programmatic dependent launch (SKILLS_PDL=0) must not change a single
bit; the other variants (the Householder panel instead of CholeskyQR2, the
CUDA-core products instead of the tensor cores, the shared-memory sample QRP,
the barrier-based candidate exchange) must reach the same least-squares
solution: x to 1e-8 relative (the four problems are full rank, condition
numbers ~1e3)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

_CHILD = r"""
import json, sys
import numpy as np
import scipy.sparse as sp
sys.path.insert(0, sys.argv[1])
import skills_gb300 as skl
rng = np.random.default_rng(7)
out = {}
# sparse, full rank, column scales 10^U[0,3]: the randomized CPQR path
A = sp.random(20000, 600, density=0.01, random_state=3, format="csc")
A = (A + sp.eye(20000, 600, format="csc")) @ sp.diags(10.0 ** rng.uniform(0, 3, 600))
b = rng.standard_normal(20000)
r = skl.ls_sparse_spqr(A.tocsc(), b, 1.7, 2, it_tol=1e-12, seed=5)
out["sparse"] = [float(v) for v in r.x]
# dense: the hashing solver with CPQR, without it, and Blendenpik (unpivoted QR)
U, _ = np.linalg.qr(rng.standard_normal((4000, 300)))
V, _ = np.linalg.qr(rng.standard_normal((300, 300)))
D = np.asfortranarray((U * np.logspace(0, -3, 300)) @ V.T)
bd = D @ rng.standard_normal(300) + 1e-4 * rng.standard_normal(4000)
out["dense"] = [float(v) for v in skl.ls_dense_hashing_blendenpik(D, bd, 1.7, 1, it_tol=1e-12, seed=4).x]
out["nocpqr"] = [float(v) for v in skl.ls_dense_hashing_blendenpik_noCPQR(D, bd, 1.7, 1, it_tol=1e-12, seed=4).x]
out["blendenpik"] = [float(v) for v in skl.ls_dense_blendenpik(D, bd, 2.2, it_tol=1e-12, seed=4).x]
print(json.dumps(out))
"""

VARIANTS = {
    "default": {},
    "no_pdl": {"SKILLS_PDL": "0"},
    "householder_panel": {"SKILLS_QR_PANEL": "pivoted"},
    "cuda_core_products": {"SKILLS_QR_TC": "0"},
    "smem_sample_qrp": {"SKILLS_YQRP_REG": "0"},
    "barrier_exchange": {"SKILLS_YQRP_ASYNC": "0"},
}


@pytest.fixture(scope="module")
def runs():
    res = {}
    pkg = os.path.join(ROOT, "ski-lls_gb300")
    for name, env in VARIANTS.items():
        e = dict(os.environ, **env)
        p = subprocess.run([sys.executable, "-c", _CHILD, pkg], env=e, capture_output=True, text=True,
                           timeout=600)
        assert p.returncode == 0, (name, p.stderr[-2000:])
        res[name] = {k: np.array(v) for k, v in json.loads(p.stdout.strip().splitlines()[-1]).items()}
    return res


def test_pdl_off_is_bit_identical(runs):
    for k in runs["default"]:
        assert np.array_equal(runs["default"][k], runs["no_pdl"][k]), k


@pytest.mark.parametrize("variant", ["householder_panel", "cuda_core_products", "smem_sample_qrp",
                                     "barrier_exchange"])
def test_variant_reaches_the_same_solution(runs, variant):
    for k, x0 in runs["default"].items():
        x = runs[variant][k]
        assert np.linalg.norm(x - x0) <= 1e-8 * np.linalg.norm(x0), (variant, k)

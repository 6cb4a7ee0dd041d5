"""The configuration-size reference fixture (tests/golden/config_golden.npz,
written by tests/golden/make_config_golden.py from the reference bcbcg_v1)
against the generators and the restated Lanczos interval, on the CPU: the
GPU parity tests read it as the reference's answer, so its inputs must be
the ones the GPU tests rebuild."""
import os
import sys

import numpy as np
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_config_golden as MG  # noqa: E402

D = np.load(os.path.join(HERE, "golden", "config_golden.npz"))


@pytest.mark.parametrize("key", ["cfg2", "cfg3", "k256lap", "k256vc", "cfg4s4it1"])
def test_fixture_inputs_match_generators(key):
    c = MG.CASES[key]
    kw = c.get("vc", dict(shift=1e-6, sigma=1.5, seed=3)) if c["kind"] == "varcoef2d" else {}
    rp, ci, v = O.gen_matrix(c["kind"], c["N"], **kw)
    n = len(rp) - 1
    B = O.gen_rhs(c["rhs"], n, c["m"], c["seed"], c["a"], c["b"])
    eps = float(D[key + "_eps"][0])
    assert eps == 1e-8 * float(np.linalg.norm(B[:, 0]))
    st = int(D[key + "_stride"][0])
    assert D[key + "_X_rows"].shape == ((n + st - 1) // st, c["m"])


def test_fixture_converged_cases():
    """The reference met its own test (||R(:,0)|| < eps) in the solves the
    parity tests pin, within MAXITER = 100."""
    for key in ("cfg2", "cfg3", "k256lap", "k256vc"):
        it = int(D[key + "_iters"][0])
        assert it < 100
        assert D[key + "_hist"][-1] < D[key + "_eps"][0]
    assert int(D["cfg2_iters"][0]) == 22 and int(D["cfg3_iters"][0]) == 28


def test_config4_lanczos_restatement_reproducible():
    c = MG.CASES["cfg4s4"]
    _, _, _, _, bnd = MG.inputs(c)
    np.testing.assert_allclose(bnd, D["cfg4s4_bounds"], rtol=1e-12)

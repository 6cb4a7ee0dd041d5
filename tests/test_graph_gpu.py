"""CUDA-graph replay of the outer iteration (use_graph on a non-default
stream): the same kernels in the same order, so results are bit-identical
to launching them one by one."""
import numpy as np
import pytest
import torch

import cacg_gb300 as cg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,N,m,s,prec", [("st3d27", 16, 16, 6, "mixed"),
                                             ("lap3d7", 20, 8, 4, "fp64"),
                                             ("lap2d", 40, 3, 5, "mixed"),
                                             ("lap2d", 33, 1, 4, "fp64")])
def test_graph_replay_bit_identical(lib, kind, N, m, s, prec):
    rp, ci, v = cg.gen_matrix(kind, N, shift=1e-3)
    n = len(rp) - 1
    B = cg.gen_rhs("normal", n, m, 5)
    M = cg.Matrix(rp, ci, v, want_fp32=True)
    stream = torch.cuda.Stream()
    out = {}
    for g in (False, True):
        dB = torch.from_numpy(B).cuda()
        dX = torch.zeros_like(dB)
        torch.cuda.synchronize()
        p = cg.Params(s=s, bounds="gerschgorin", tol=1e-8, maxit=500, precision=prec,
                      stream=stream.cuda_stream, use_graph=g)
        info = M.solve_device(dB.data_ptr(), dX.data_ptr(), m, p)
        stream.synchronize()
        out[g] = (dX.cpu().numpy(), info)
    M.close()
    (X0, i0), (X1, i1) = out[False], out[True]
    assert i0["status"] == 0 and i1["status"] == 0
    assert i0["iterations"] == i1["iterations"] and i0["iterations"] > 3
    assert np.array_equal(X0, X1)

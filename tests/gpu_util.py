"""Helpers for the GPU parity tests: device copies through torch (plumbing
only -- every computation under test runs in libcacg.so)."""
import numpy as np


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch

    torch.cuda.synchronize()
    return t.cpu().numpy()


def ptr(t):
    return t.data_ptr() if t is not None else None


def relerr(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm((a - b).ravel())
    s = np.linalg.norm(b.ravel())
    return d / s if s > 0 else d

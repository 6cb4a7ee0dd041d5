"""Serving workload generator (host logic, no GPU)."""
import math

import numpy as np

from cacg_gb300 import serving as SV


def test_request_specs_follow_the_workload_distribution():
    specs = SV.request_specs(2000, seed=4)
    assert len(specs) == 2000
    kinds = [s["kind"] for s in specs]
    frac2d = kinds.count("lap2d") / len(kinds)
    assert 0.45 < frac2d < 0.55
    n = np.array([s["N"] ** (2 if s["kind"] == "lap2d" else 3) for s in specs], float)
    assert n.min() >= 0.5e3 and n.max() <= 1.1e6
    # log-uniform: the median of log10(n) sits near 4.5
    assert abs(np.median(np.log10(n)) - 4.5) < 0.15
    m = np.array([s["m"] for s in specs])
    assert m.min() == 1 and m.max() == 16
    sh = np.array([s["shift"] for s in specs])
    assert sh.min() >= 0.0 and sh.max() < 0.1
    # seeded: identical on a second draw
    assert SV.request_specs(50, seed=4) == specs[:50]


def test_build_request_shapes():
    sp = {"kind": "lap3d7", "N": 6, "shift": 0.05, "m": 3, "seed": 9}
    rp, ci, v, B = SV.build_request(sp)
    assert len(rp) == 6 ** 3 + 1 and B.shape == (216, 3)
    assert math.isclose(v[rp[0]:rp[1]].max(), 6.05)


def test_command_line_help_and_size_cap():
    import pytest

    with pytest.raises(SystemExit) as e:
        SV.main(["--help"])
    assert e.value.code == 0
    # --max-rows caps the stream's sizes (the batched engine's default limit)
    specs = SV.request_specs(500, seed=4, nmax=65536)
    n = np.array([s["N"] ** (2 if s["kind"] == "lap2d" else 3) for s in specs], float)
    assert n.max() <= 65536 * 1.05

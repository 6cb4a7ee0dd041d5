"""The C ABI (include/*.h): libcacg.so loads without a GPU, exports every
function the headers declare, and the ctypes mirror of each struct has the
C layout (checked against the header with the host C compiler)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from cacg_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


def declared_functions():
    names = set()
    for h in os.listdir(INC):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(INC, h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M):
            if not m.group(0).startswith(("typedef", "#")):
                names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_function(lib):
    decl = declared_functions()
    assert "cacg_solve" in decl and "bcbcg_v1" in decl and "cbcg_v1" in decl
    missing = [n for n in decl if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python bindings cover them all
    assert set(decl) <= set(L.exported_symbols())


def _c_layout(structs):
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "cacg.h"', "int main(void){"]
    for s, fields in structs.items():
        src.append('printf("%s %%zu\\n", sizeof(%s));' % (s, s))
        for f in fields:
            src.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (s, f, s, f))
    src.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        open(c, "w").write("\n".join(src))
        exe = os.path.join(d, "l")
        subprocess.check_call(["gcc", "-I", INC, c, "-o", exe])
        out = subprocess.check_output([exe], text=True)
    return dict(line.split() for line in out.splitlines())


def test_python_constants_match_header_defines():
    """Every integer #define CACG_<NAME> of include/cacg.h that the ctypes
    mirror also names (<NAME>) has the same value there."""
    text = open(os.path.join(INC, "cacg.h")).read()
    defines = {m.group(1): int(m.group(2))
               for m in re.finditer(r"^#define\s+CACG_(\w+)\s+(-?\d+)", text, flags=re.M)}
    shared = [k for k in defines if hasattr(L, k)]
    for k in ("VAL_F64", "VAL_F32", "XR_EXACT", "VAL_TC5", "VAL_TC5_CPASYNC", "XR_FFSTATE",
              "SPMM_AUTO", "SPMM_CSR", "SPMM_DIA_UNSTAGED", "ALG_CACG", "ALG_BCG", "GRAM_TC5",
              "MIXED", "FP64"):
        assert k in shared, k
    for k in shared:
        assert getattr(L, k) == defines[k], (k, getattr(L, k), defines[k])


def test_struct_layouts_match_header():
    py = {"cacg_params": L.CacgParams, "cacg_result": L.CacgResult, "cacg_csr": L.CacgCsr,
          "csrType_local": L.CsrTypeLocal, "denseType": L.DenseType,
          "cacg_server_config": L.CacgServerConfig}
    lay = _c_layout({k: [f[0] for f in v._fields_] for k, v in py.items()})
    for name, cls in py.items():
        assert int(lay[name]) == C.sizeof(cls), name
        for f in cls._fields_:
            assert int(lay["%s.%s" % (name, f[0])]) == getattr(cls, f[0]).offset, (name, f[0])


def test_reference_struct_header_is_guard_compatible():
    """cacg_ref_types.h uses the reference's DATATYPES_H guard, so a driver
    including the reference's DataTypes.h and cacg.h compiles."""
    src = '#include "cacg_ref_types.h"\n#include "cacg.h"\nint main(void){csrType_local a; denseType b; (void)a; (void)b; return 0;}\n'
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "g.c")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-Wall", "-Werror", "-I", INC, c, "-o", os.path.join(d, "g")])


def _has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_calls_without_device_fail_loudly(lib):
    import numpy as np

    import cacg_gb300 as cg

    rp, ci, v = cg.gen_matrix("lap2d", 8)
    with pytest.raises(cg.CacgError) as e:
        cg.solve(rp, ci, v, np.ones((64, 1)))
    assert e.value.code == L.ERR_NODEV
    X = np.zeros((64, 1))
    cg.cbcg_v1(rp.astype(np.int64), ci.astype(np.int64), v, np.ones((64, 1)), X, 4, 1e-8)
    assert cg.last_status() == L.ERR_NODEV
    assert not X.any()


def test_params_default_and_status_strings(lib):
    p = L.CacgParams()
    lib.cacg_params_default(C.byref(p))
    assert p.s == 4 and p.maxit == 1000 and p.tol == 1e-8 and p.rr_period == 5
    assert p.tol_mode == L.TOL_REL_ALL and p.precision == L.FP64
    for code in (0, 1, -1, -2, -4, -5, -6, -7, -8):
        assert lib.cacg_status_string(code)
    assert lib.cacg_workspace_bytes(2097152, 16, 6, L.MIXED) > 3 * 2097152 * 96 * 4


def test_overwrite_x0_argument_checks():
    import numpy as np

    import cacg_gb300 as cg

    rp, ci, v = cg.gen_matrix("lap2d", 8)
    B = np.ones((64, 2))
    for X0 in (None, np.zeros((64, 2), np.float32), np.zeros((64, 3)),
               np.zeros((2, 64)).T, np.zeros((64, 2))[:, :1]):
        with pytest.raises(ValueError):
            cg.solve(rp, ci, v, B, X0, overwrite_x0=True)

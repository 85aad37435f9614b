"""The C-ABI library: builds, loads and exports every declared entry point,
and rejects bad parameters on the host (CPU only, no compute calls)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "marbles_gb300.h")).read()
    return sorted(set(re.findall(r"\b(mbg_[a-z0-9_]+)\s*\(", hdr)))


def test_library_builds_and_exports_all_declarations():
    from marbles_gb300 import build
    lib = build.build(verbose=False)
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (mbg_[a-z0-9_]+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing


def test_library_loads_with_ctypes():
    import marbles_gb300 as M
    L = M.lib()
    for s in declared_symbols():
        assert hasattr(L, s)
    assert set(M.EXPORTS) <= set(declared_symbols())


@pytest.mark.parametrize("field,value", [("nu", -1.0), ("adiabatic_exponent", 1.0), ("precision", 7)])
def test_create_rejects_bad_parameters(field, value):
    import marbles_gb300 as M
    p = M.default_params()
    setattr(p, field, value)
    with pytest.raises(M.MbgError, match="MBG_EINVAL"):
        M.Context(p)


def test_create_rejects_inconsistent_periodicity():
    import marbles_gb300 as M
    p = M.default_params()
    p.is_periodic[:] = [0, 1, 1]   # x not periodic but bc code 0
    with pytest.raises(M.MbgError, match="not periodic"):
        M.Context(p)
    p = M.default_params()
    p.bc_lo[:] = [1, 0, 0]          # periodic but wall code
    with pytest.raises(M.MbgError, match="periodic"):
        M.Context(p)


def test_create_rejects_pressure_bc_beside_walls():
    """A pressure face needs periodic tangential directions (the reference's
    functor result depends on its visiting order next to other walls)."""
    import marbles_gb300 as M
    p = M.default_params()
    p.is_periodic[:] = [0, 0, 1]
    p.bc_lo[:] = [3, 1, 0]
    p.bc_hi[:] = [5, 1, 0]
    with pytest.raises(M.MbgError, match="periodic tangential"):
        M.Context(p)


def test_batch_and_adjoint_reject_bad_parameters():
    """Host-side validation of the batch and adjoint entry points (no GPU
    work happens before these checks)."""
    import math
    import marbles_gb300 as M
    p = M.default_params()
    p.precision = 0            # the batch is a 16-bit form only
    with pytest.raises(M.MbgError, match="16-bit"):
        M.Batch(p, [([8, 8, 8], [0.0] * 3, [2 * math.pi] * 3, 0.1, 0.1)])
    p.precision = 1
    with pytest.raises(M.MbgError, match="invalid extent"):
        M.Batch(p, [([1, 8, 8], [0.0] * 3, [2 * math.pi] * 3, 0.1, 0.1)])
    q = M.default_params()
    q.is_periodic[:] = [0, 1, 1]
    with pytest.raises(M.MbgError, match="periodic"):
        M.Adjoint(q)
    q = M.default_params()
    q.precision = 1
    with pytest.raises(M.MbgError, match="FP64"):
        M.Adjoint(q)

"""C-ABI library checks that need no GPU: it builds, loads, and exports every entry point
declared in include/impec2d.h; context creation without a device fails with a status."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "impec2d.h")).read()
    return sorted(set(re.findall(r"\b(impec_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def so():
    from impec2d_gb300 import build as B
    path = B.build()
    return C.CDLL(path)


def test_every_declared_symbol_is_exported(so):
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(so, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    import impec2d_gb300 as E
    missing = [n for n in _declared() if n not in E._SIGS]
    assert not missing, missing


def test_default_params_follow_reference_examples():
    import impec2d_gb300 as E
    P = E.default_params(141, 141)
    assert (P.N1, P.N2) == (141, 141)
    assert P.mu_res == 41.0 and P.mu_inj == 1.0 and P.avgproc == E.HARMONIC
    assert P.dim_splitting == E.SYMMETRIC_PARALLEL and P.hmtype == E.MUSCL
    assert P.peaceman_guard == 1 and P.cfl_porosity == 0 and P.warm_start == 0


def test_invalid_params_are_rejected_without_exiting():
    import impec2d_gb300 as E
    for bad in (dict(nu=1.5), dict(N2=1), dict(hmtype=2), dict(porosity=0.0)):
        P = E.default_params(16, 16)
        for k, v in bad.items():
            setattr(P, k, v)
        h = C.c_void_p()
        st = E.lib().impec_ctx_create(C.byref(P), None, C.byref(h))
        assert st != 0 and not h.value


def test_no_device_is_reported_as_status():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import impec2d_gb300 as E
    P = E.default_params(16, 16)
    with pytest.raises(E.ImpecError) as ei:
        E.Context(P)
    assert ei.value.status == 5

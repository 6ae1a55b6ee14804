"""CPU-side checks of the C ABI: the library loads and exports every symbol
the public headers declare; host-only helpers agree with the oracle."""
import ctypes
import os
import re

import pytest

import oracle
from masterthesislucas_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(tc_\w+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def L():
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libtreecode.so not built")
    return _lib.lib()


def test_every_declared_symbol_is_exported(L):
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"


def test_get_depth_matches_reference_rule(L):
    for leaf, n in [(16, 70000), (16, 65536), (64, 4194304), (16, 3000), (16, 17), (16, 15), (8, 3000), (1, 1)]:
        d = ctypes.c_uint32()
        assert L.tc_get_depth(leaf, n, ctypes.byref(d)) == 0
        expect = oracle.get_depth(leaf, n) if n // leaf >= 1 else 0
        assert d.value == expect, (leaf, n)


def test_node_count(L):
    c = ctypes.c_int64()
    for d in range(0, 10):
        assert L.tc_node_count(d, ctypes.byref(c)) == 0
        assert c.value == oracle.node_count(d)


def test_invalid_config_rejected_without_gpu(L):
    cfg = _lib.TcConfig()
    L.tc_config_init(ctypes.byref(cfg))
    cfg.theta = -1.0
    h = ctypes.c_void_p()
    assert L.tc_create(ctypes.byref(cfg), ctypes.byref(h)) == _lib.TC_ERR_INVALID
    assert b"invalid" in L.tc_last_error()


def test_dropin_adaptor_builds_against_reference_interface(L):
    """GpuTreeSolver<TsnePoint2D> compiles and links as an NBodySolver<TsnePoint2D>
    next to the reference's own solver headers (runs only where a GPU exists)."""
    import subprocess
    if not os.path.isdir("/root/reference/src"):
        pytest.skip("reference sources not present")
    r = subprocess.run(["make", "-s", "-B", "-f", "oracle/Makefile.ref", "dropin"], cwd=ROOT, capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.exists(os.path.join(ROOT, "oracle", "_ref", "dropin_check"))


@pytest.mark.parametrize("fn", ["tc_direct_device", "tc_direct_device_noalloc"])
def test_direct_rejects_more_rows_than_points_without_a_row_list(L, fn):
    """Without a row list the sinks are points 0..m-1: m > n must be rejected
    before anything is launched (the pointers are never dereferenced)."""
    fake = ctypes.c_void_p(256)
    f = getattr(L, fn)
    assert f(1, 1e-3, 1, fake, 100, None, 101, fake, None, None) == -1
    assert b"invalid" in L.tc_last_error()
    # an unknown precision code is rejected the same way
    assert f(1, 1e-3, 7, fake, 100, None, 10, fake, None, None) == -1


def test_stage_names_match_the_header():
    """tc_get_stage_times writes TC_NSTAGES doubles; the Python mirror names each of them."""
    from masterthesislucas_gb300 import NBodySolverFMM_SYM_MORTON
    src = open(os.path.join(ROOT, "include", "treecode.h")).read()
    n = int(re.search(r"#define\s+TC_NSTAGES\s+(\d+)", src).group(1))
    assert len(NBodySolverFMM_SYM_MORTON.STAGES) == n
    assert NBodySolverFMM_SYM_MORTON.STAGES[-1] == "reduce" and "l2p" in NBodySolverFMM_SYM_MORTON.STAGES


def test_near_overlap_switch_needs_no_gpu(L):
    """Setting the near/far overlap is host state only (a null handle is rejected)."""
    assert L.tc_set_near_overlap(None, 0) == _lib.TC_ERR_INVALID

"""The C-ABI library builds for sm_103a, loads, and exports every declared symbol."""
import ctypes
import glob
import os
import re
import subprocess

from gravhopper_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(gh_[A-Za-z0-9_]+)\s*\(",
                            text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("gh_direct_summation", "gh_direct_summation_position", "gh_run_dkd", "gh_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", _capi.lib_path()], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (gh_\w+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    for n in declared_functions():
        assert hasattr(lib, n)


def test_ctypes_signatures_cover_header(lib):
    assert set(declared_functions()) <= set(_capi.SIGNATURES)


def test_version_and_launch_counter_without_gpu(lib):
    assert lib.gh_version() == 100
    assert lib.gh_launch_count() >= 0


def test_library_targets_sm_103a():
    from gravhopper_gb300 import _build
    assert "arch=compute_103a,code=sm_103a" in " ".join(_build.ARCH)
    assert os.path.exists(_build.LIB)


def test_fault_injection_arguments_without_gpu(lib):
    """The test-only fault hooks validate their arguments on the host (no device use)."""
    assert lib.gh_debug_inject(99, 1) == _capi.GH_ERR_ARG
    assert lib.gh_debug_inject(_capi.GH_INJECT_ALLOC, -1) == _capi.GH_ERR_ARG
    assert lib.gh_debug_inject(_capi.GH_INJECT_ALLOC, 0) == _capi.GH_OK
    assert lib.gh_debug_inject(_capi.GH_INJECT_TREE_WAIT, 0) == _capi.GH_OK
    assert lib.gh_debug_sort_stall(-1, None) == _capi.GH_ERR_ARG


def test_direct_tune_rules_without_gpu(lib):
    """Autotuned shape rules: the rule with the largest n_min <= N applies per kind,
    below every rule the built-in table does, and -1 clears the kind's rules."""
    nshape = lib.gh_direct_num_shapes()
    base_force = [lib.gh_direct_shape_for(n, 0) for n in (1000, 50000, 2000000)]
    base_step = [lib.gh_direct_shape_for(n, 1) for n in (1000, 50000, 2000000)]
    try:
        assert lib.gh_direct_tune(10000, 0, 2) == _capi.GH_OK
        assert lib.gh_direct_tune(100000, 0, 5) == _capi.GH_OK
        assert lib.gh_direct_shape_for(1000, 0) == base_force[0]
        assert lib.gh_direct_shape_for(10000, 0) == 2
        assert lib.gh_direct_shape_for(99999, 0) == 2
        assert lib.gh_direct_shape_for(2000000, 0) == 5
        assert [lib.gh_direct_shape_for(n, 1) for n in (1000, 50000, 2000000)] == base_step
        assert lib.gh_direct_tune(100000, 0, 6) == _capi.GH_OK  # replaces the rule
        assert lib.gh_direct_shape_for(2000000, 0) == 6
        assert lib.gh_direct_tune(0, 0, nshape) == _capi.GH_ERR_ARG
        assert lib.gh_direct_tune(0, 2, 1) == _capi.GH_ERR_ARG
        assert lib.gh_direct_shape_for(-1, 0) == -1
    finally:
        assert lib.gh_direct_tune(0, 0, -1) == _capi.GH_OK
    assert [lib.gh_direct_shape_for(n, 0) for n in (1000, 50000, 2000000)] == base_force

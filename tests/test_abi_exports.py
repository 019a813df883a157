"""The C ABI library loads without a GPU and exports every function include/dpcull.h declares."""
import ctypes
import re
import subprocess

import pytest

from conftest import ROOT


def declared_functions() -> list[str]:
    text = (ROOT / "include" / "dpcull.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\*\s]+?\b(dpcull_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib_path():
    from pipeline_gb300 import build

    return build.build_cuda()


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("dpcull_ctx_create", "dpcull_group_set_objects", "dpcull_group_set_matrices",
                 "dpcull_cull", "dpcull_result_changed", "dpcull_cull_batched",
                 "dpcull_plan_create", "dpcull_tree_compute", "dpcull_group_bounding_box",
                 "dpcull_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(str(lib_path))  # loads without a GPU (no device call at load time)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from pipeline_gb300 import native

    assert set(declared_functions()) == set(native.exported_symbols())


def test_no_gpu_means_error_not_fallback(lib_path):
    """Without a GPU the context cannot be created: an error code, never a CPU path."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from pipeline_gb300 import native

    with pytest.raises(native.DpcullError) as e:
        native.Context(0)
    assert e.value.code == native.ERR_CUDA


def test_symbols_are_c_linkage(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib_path)], capture_output=True,
                         text=True).stdout
    syms = {line.split()[-1] for line in out.splitlines() if line.strip()}
    for n in declared_functions():
        assert n in syms, n  # unmangled

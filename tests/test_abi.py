"""The C-ABI library loads and exports every function include/graphaligner_gb300.h declares."""
import ctypes
import os
import re

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "graphaligner_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(ga_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("ga_graph_upload", "ga_extend_batch", "ga_extender_create", "ga_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(cuda_lib):
    missing = [n for n in declared_functions() if not hasattr(cuda_lib, n)]
    assert not missing, f"missing exports: {missing}"


def test_version_string(cuda_lib):
    cuda_lib.ga_version.restype = ctypes.c_char_p
    assert b"sm_103a" in cuda_lib.ga_version()

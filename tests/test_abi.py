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


GA_OK = 0
GA_ERR_ARGUMENT = -1


def test_null_arguments_are_rejected_before_any_device_call(cuda_lib):
    """Every entry point answers a missing argument with GA_ERR_ARGUMENT (and frees of NULL
    with GA_OK) without touching CUDA, so a host-only process can rely on it."""
    L = cuda_lib
    n = None
    calls = {
        "ga_graph_upload": (n, 0, n),
        "ga_extender_create": (n, ctypes.c_uint64(0), n),
        "ga_extender_create_like": (n, n),
        "ga_extend_batch": (n, n, n, n),
        "ga_extend_batch_device": (n, n, n, n, n),
        "ga_extend_batch_noalloc": (n, n, n, n, n),
        "ga_extender_last_kernel_ms": (n, n),
        "ga_extender_last_times": (n, n, n),
        "ga_extender_last_launches": (n, n),
        "ga_extender_last_copy_ms": (n, n, n),
        "ga_extender_set_launch_shape": (n, n),
        "ga_extender_get_launch_shape": (n, n),
        "ga_extender_autotune": (n, n, n, n, 0, 0, n),
        "ga_extender_last_arena_bytes": (n, n),
        "ga_extender_last_layout_counts": (n, n),
        "ga_extender_last_multiseed_counts": (n, n, n, n, n),
        "ga_aligner_create": (n, n, n, n),
        "ga_align_reads": (n, 0, n, n, n, n),
        "ga_aligner_gaf": (n, n, n),
        "ga_aligner_get_seeds": (n, 0, n, n, n, n, n),
        "ga_aligner_read_bp": (n, n),
        "ga_aligner_stats": (n, n),
        "ga_aligner_index": (n, n, n, n, n),
        "ga_multiseed_batch": (n, n, n, n),
        "ga_multiseed_batch_exact": (n, n, n, n),
        "ga_aligner_format_gaf": (n, 0, n, ctypes.c_uint64(0), n, 0, n, n, 0, n, n, n, n),
        "ga_aligner_select_alignments": (n, 0, n, n, n, n, 0, ctypes.c_double(0.9), n),
        "ga_server_create": (n, n, n),
        "ga_server_submit": (n, n, n, 0, n),
        "ga_server_poll": (n, n, 0, n, 0),
        "ga_server_release": (n, ctypes.c_uint64(1)),
        "ga_server_stats_get": (n, n),
    }
    wrong = {name: getattr(L, name)(*args) for name, args in calls.items()}
    wrong = {k: v for k, v in wrong.items() if v != GA_ERR_ARGUMENT}
    assert not wrong, f"not GA_ERR_ARGUMENT: {wrong}"
    for name in ("ga_graph_free", "ga_extender_free", "ga_aligner_free", "ga_server_free"):
        assert getattr(L, name)(n) == GA_OK, name


def test_host_graph_desc_points_at_every_node_name():
    """ga_host_graph_desc.names, as align.HostGraphDesc lays it out (one NUL-separated buffer
    and a pointer per name), reads back as the graph's names, in nodeLookup order."""
    import gzip
    import tempfile
    from graphaligner_gb300 import graph as gg
    from graphaligner_gb300.align import HostGraphDesc
    with tempfile.NamedTemporaryFile(suffix=".gag") as f:
        f.write(gzip.open(os.path.join(ROOT, "tests", "golden", "vg50k_graph.gag.gz")).read())
        f.flush()
        g = gg.load_gag(f.name)
    d = HostGraphDesc.from_graph(g)
    assert d.num_lookup == len(g.names) > 1000
    assert [d.names[i].decode() for i in range(d.num_lookup)] == list(g.names)
    g.names = ["a", "", "node 3"] + list(g.names[3:])
    d = HostGraphDesc.from_graph(g)
    assert [d.names[i].decode() for i in range(3)] == ["a", "", "node 3"]


def test_noalloc_rejects_null_arrays_before_any_device_call(cuda_lib):
    """ga_extend_batch_noalloc with descriptions whose arrays are NULL (num > 0) answers
    GA_ERR_ARGUMENT with a message instead of handing NULL to the kernel."""
    from graphaligner_gb300 import _abi
    L = cuda_lib
    L.ga_last_error.restype = ctypes.c_char_p
    g = _abi.GraphDesc()
    g.num_nodes = 4
    b = _abi.BatchDesc()
    b.num = 3
    r = _abi.Results()
    p = _abi.ExtendParams(10, 14705, 2**64 - 1, 294)
    rc = L.ga_extend_batch_noalloc(ctypes.byref(g), ctypes.byref(p), ctypes.byref(b), ctypes.byref(r), None)
    assert rc == GA_ERR_ARGUMENT
    assert b"null array" in L.ga_last_error()

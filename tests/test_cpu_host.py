"""CPU checks of the host side: the C ABI library's exports, argument
validation and degenerate paths that must not touch the GPU, and the
multi-process timing reduction of bench.py (world size 2, gloo)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from fast_hdbscan_gb300 import _native


def _declared_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"\b(fhg_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    from fast_hdbscan_gb300 import build, _native

    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    declared = _declared_functions()
    assert len(declared) >= 15
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing
    # every declared function is also bound by the Python layer or documented
    # as a direct C entry point
    bound = set(_native.SIGNATURES)
    direct = {"fhg_launch_count", "fhg_profile_enable", "fhg_profile_report",
              "fhg_mst_to_linkage_tree_noalloc"}
    assert set(declared) <= bound | direct
    assert lib.fhg_abi_version() == 2


def test_library_error_reporting_without_gpu():
    """Argument errors are reported before any CUDA call."""
    from fast_hdbscan_gb300 import build

    lib = ctypes.CDLL(build.build())
    lib.fhg_last_error.restype = ctypes.c_char_p
    lib.fhg_index_build.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
                                    ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
    out = ctypes.c_void_p()
    rc = lib.fhg_index_build(None, 10, 3, None, ctypes.byref(out))
    assert rc == 1 and b"null" in lib.fhg_last_error()
    lib.fhg_mst_to_linkage_tree_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int64,
                                                    ctypes.c_void_p, ctypes.c_void_p]
    rc = lib.fhg_mst_to_linkage_tree_noalloc(None, 65537, None, None)
    assert rc == 1 and b"FHG_NOALLOC_MAX_EDGES" in lib.fhg_last_error()


# entry points that take no data (status, switches, sizes, the last call's
# fallback count) or for which a null argument is a valid request (freeing no
# index, switching the radius off)
_NO_DATA = {"fhg_last_error", "fhg_abi_version", "fhg_set_tie_rule", "fhg_set_highd_kernel",
            "fhg_release_cached_memory", "fhg_reference_kdtree_levels", "fhg_index_free",
            "fhg_radius_param_count", "fhg_radius_use", "fhg_radius_fallbacks"}


@pytest.mark.parametrize("name", [n for n in _native.SIGNATURES if n not in _NO_DATA])
def test_entry_point_rejects_null_and_negative_arguments(name):
    """Every data entry point answers null pointers and negative sizes with
    FHG_ERR_INVALID and a message, before any CUDA call (a negative size is
    never taken for an empty input).  Host out-parameters are given, so that
    the checks after them are reached too."""
    from fast_hdbscan_gb300 import build

    lib = ctypes.CDLL(build.build())
    lib.fhg_last_error.restype = ctypes.c_char_p
    restype, argtypes = _native.SIGNATURES[name]
    fn = getattr(lib, name)
    fn.restype, fn.argtypes = restype, argtypes
    keep, args = [], []
    for a in argtypes:
        if isinstance(a, type) and issubclass(a, ctypes._Pointer):
            keep.append(a._type_(0))
            args.append(ctypes.pointer(keep[-1]))
        elif a in (ctypes.c_void_p,):
            args.append(None)
        elif a in (ctypes.c_double, ctypes.c_float):
            args.append(0.0)
        elif a is ctypes.c_uint64:
            args.append(0)
        else:
            args.append(-1)
    assert fn(*args) == _native.FHG_ERR_INVALID
    assert lib.fhg_last_error()


def test_badargs_raise_before_the_engine():
    """fast_hdbscan/tests/test_hdbscan.py:138-166."""
    from fast_hdbscan_gb300 import fast_hdbscan

    X = np.random.default_rng(0).random((50, 2))
    with pytest.raises(ValueError):
        fast_hdbscan("fail")
    with pytest.raises(ValueError):
        fast_hdbscan(None)
    for kw in (dict(min_cluster_size="fail"), dict(min_samples="fail"), dict(min_samples=-1),
               dict(cluster_selection_epsilon="fail"), dict(cluster_selection_epsilon=-1),
               dict(cluster_selection_epsilon=-0.1), dict(cluster_selection_persistence="fail"),
               dict(cluster_selection_persistence=1),
               dict(cluster_selection_persistence=-0.1),
               dict(cluster_selection_method="fail"),
               dict(semi_supervised=True, ss_algorithm="fail"),
               dict(semi_supervised=True, data_labels=None)):
        with pytest.raises(ValueError):
            fast_hdbscan(X, **kw)


def test_degenerate_inputs_need_no_engine():
    """hdbscan.py:278-304: fewer than two points."""
    from fast_hdbscan_gb300 import fast_hdbscan

    labels, probs, slt, ct, mst, nbrs, core = fast_hdbscan(np.zeros((1, 2)), return_trees=True)
    assert labels.shape == (1,) and np.all(labels == -1)
    assert probs.shape == (1,) and slt.shape == (0, 4) and mst.shape == (0, 3)
    assert np.all(np.isinf(core))
    with pytest.raises(ValueError):  # check_array: at least one sample
        fast_hdbscan(np.zeros((0, 2)))


def test_out_of_scope_routes_raise_not_implemented():
    from fast_hdbscan_gb300 import fast_hdbscan
    from fast_hdbscan_gb300.hdbscan import compute_minimum_spanning_tree

    X = np.random.default_rng(1).random((20, 2))
    with pytest.raises(NotImplementedError):
        fast_hdbscan(X, metric="cosine")
    with pytest.raises(NotImplementedError):  # exact full-pairwise Kruskal (knn_k=None)
        fast_hdbscan(X, algorithm="kruskal")
    with pytest.raises(NotImplementedError):  # cannot-link constraints
        fast_hdbscan(X, algorithm="kruskal", knn_k=5, cannot_link_groups=np.zeros(20, np.int32))
    with pytest.raises(ValueError):  # hdbscan.py:420: constraints need algorithm="kruskal"
        fast_hdbscan(X, cannot_link_groups=np.zeros(20, np.int32))
    with pytest.raises(ValueError):
        compute_minimum_spanning_tree(X, algorithm="prim")
    with pytest.raises(NotImplementedError):  # hdbscan.py:447's kNN-graph route: up to 96 dims
        fast_hdbscan(np.random.default_rng(2).random((20, 97)))
    with pytest.raises(NotImplementedError):
        fast_hdbscan(np.random.default_rng(2).random((20, 40)),
                     sample_weights=np.ones(20, np.float32))


def test_knn_graph_route_and_k():
    """hdbscan.py:446-449 routes Euclidean data above 30 dimensions without
    sample weights to the kNN-graph back-end; nndescent.py:214-217 resolves
    its k."""
    from fast_hdbscan_gb300.hdbscan import _knn_graph_route, resolve_knn_graph_k

    X31, X30 = np.zeros((5, 31)), np.zeros((5, 30))
    assert _knn_graph_route("euclidean", X31, None)
    assert not _knn_graph_route("euclidean", X30, None)
    assert not _knn_graph_route("euclidean", X31, np.ones(5))
    assert resolve_knn_graph_k(10, None) == 30 and resolve_knn_graph_k(3, None) == 15
    assert resolve_knn_graph_k(10, 5) == 10 and resolve_knn_graph_k(2, 40) == 40


def test_estimator_params_roundtrip():
    from fast_hdbscan_gb300 import HDBSCAN

    est = HDBSCAN(min_cluster_size=7, min_samples=3, cluster_selection_method="leaf")
    p = est.get_params()
    assert p["min_cluster_size"] == 7 and p["min_samples"] == 3
    assert p["cluster_selection_method"] == "leaf"
    est.set_params(min_cluster_size=11)
    assert est.min_cluster_size == 11


def _gloo_worker(rank, world, port, queue):
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from bench import max_over_ranks

    queue.put((rank, max_over_ranks(10.0 * (rank + 1), torch.device("cpu"))))
    dist.destroy_process_group()


def test_bench_max_over_ranks_gloo():
    """bench.py reports the slowest rank's step time (world size 2, gloo)."""
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_gloo_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 20.0, 1: 20.0}


def _c_kind(decl):
    """Kind of one C parameter or return declaration: 'ptr' or its integer /
    floating type ('int' is int32 on every supported platform)."""
    decl = decl.strip()
    if "*" in decl:
        return "ptr"
    base = decl.replace("const", " ").split()[0]
    return {"int32_t": "i32", "int": "i32", "int64_t": "i64", "uint64_t": "u64", "double": "f64",
            "float": "f32"}.get(base, "?" + base)


def _ctypes_kind(t):
    if t is ctypes.c_void_p or t is ctypes.c_char_p or (
            isinstance(t, type) and issubclass(t, ctypes._Pointer)):
        return "ptr"
    for ct, kind in ((ctypes.c_int32, "i32"), (ctypes.c_int, "i32"), (ctypes.c_int64, "i64"),
                     (ctypes.c_uint64, "u64"), (ctypes.c_double, "f64"), (ctypes.c_float, "f32")):
        if t is ct:
            return kind
    return "?"


def test_ctypes_signatures_match_the_header():
    """Every entry point's ctypes argtypes and restype (fast_hdbscan_gb300/_native.py)
    have the count and kinds (pointer, int32, int64, uint64, float, double) of
    its prototype in include/fhg.h, so no argument is passed with the wrong width."""
    text = open(os.path.join(ROOT, "include", "fhg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    protos = re.findall(r"([A-Za-z_][\w \*]*?)\b(fhg_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text,
                        flags=re.S)
    checked = 0
    for ret, name, params in protos:
        if name not in _native.SIGNATURES:
            continue
        restype, argtypes = _native.SIGNATURES[name]
        decls = [p for p in params.split(",") if p.strip() not in ("", "void")]
        assert [_c_kind(p) for p in decls] == [_ctypes_kind(a) for a in argtypes], name
        assert _c_kind(ret + " x") == _ctypes_kind(restype), name
        checked += 1
    assert checked == len(_native.SIGNATURES)

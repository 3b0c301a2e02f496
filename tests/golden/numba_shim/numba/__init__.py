"""No-op stand-in for numba, used only to run the fast_hdbscan reference as
plain Python when generating golden fixtures (numba itself is not installed
in the build container).

`njit`/`jit` return the function unchanged, `prange` is `range`, and the
type objects cast scalars through numpy so that calls such as
`numba.int32(x)` behave like the compiled code's casts.  Parallel loops run
sequentially, which makes the reference's racy per-component pruning bound
deterministic (the lowest point index is always processed first).
"""
import numpy as _np

from . import types  # noqa: F401
from . import typed  # noqa: F401
from .types import _NbType, void, int8, int16, int32, int64, intp, uint8, uint16, \
    uint32, uint64, float32, float64, boolean, bool_  # noqa: F401

prange = range
config = type("config", (), {"NUMBA_NUM_THREADS": 1})()


def _decorator_factory(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not isinstance(args[0], _NbType) \
            and not kwargs:
        return args[0]

    def deco(fn):
        return fn

    return deco


njit = _decorator_factory
jit = _decorator_factory
generated_jit = _decorator_factory


def get_num_threads():
    return 1


def set_num_threads(n):
    return None


def get_thread_id():
    return 0

"""Permissive numba type objects for the golden-fixture shim."""
import numpy as _np


class _NbType:
    """Callable (casts a scalar), subscriptable (array type) placeholder."""

    def __init__(self, name, np_type=None):
        self._name = name
        self._np = np_type

    def __call__(self, *args, **kwargs):
        if self._np is not None and len(args) == 1 and not kwargs \
                and not isinstance(args[0], _NbType):
            return self._np(args[0])
        return _NbType(self._name + "(...)")

    def __getitem__(self, item):
        return _NbType(self._name + "[]")

    def __repr__(self):
        return "shim:" + self._name


void = _NbType("void")
int8 = _NbType("int8", _np.int8)
int16 = _NbType("int16", _np.int16)
int32 = _NbType("int32", _np.int32)
int64 = _NbType("int64", _np.int64)
intp = _NbType("intp", _np.intp)
uint8 = _NbType("uint8", _np.uint8)
uint16 = _NbType("uint16", _np.uint16)
uint32 = _NbType("uint32", _np.uint32)
uint64 = _NbType("uint64", _np.uint64)
float32 = _NbType("float32", _np.float32)
float64 = _NbType("float64", _np.float64)
boolean = _NbType("boolean", _np.bool_)
bool_ = boolean
NamedTuple = _NbType("NamedTuple")
Tuple = _NbType("Tuple")
UniTuple = _NbType("UniTuple")
Array = _NbType("Array")
ListType = _NbType("ListType")
DictType = _NbType("DictType")


def __getattr__(name):
    return _NbType(name)

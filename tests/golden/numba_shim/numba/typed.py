"""dict/list stand-ins for numba.typed in the golden-fixture shim."""


class Dict(dict):
    @classmethod
    def empty(cls, *args, **kwargs):
        return cls()


class List(list):
    @classmethod
    def empty_list(cls, *args, **kwargs):
        return cls()

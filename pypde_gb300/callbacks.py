"""Callbacks F/B/S -> a compiled device callback system.

Stands in for pypde/cfuncs.py:30-75, which compiles the user's Python
callbacks into host cfuncs with numba.  Here the callbacks must become
device code: built-in systems (pypde_gb300.systems) map to kernels
compiled ahead of time into libpypde_gb300.so.
"""
import ctypes

from . import _lib

_cache = {}


class CompiledSystem:
    """A pypde_system handle (see include/pypde_gb300.h)."""

    def __init__(self, handle, name):
        self.handle = handle
        self.name = name
        V, nd, f, b, s, so = (ctypes.c_int() for _ in range(6))
        _lib.check(_lib.lib().pypde_system_info(handle, V, nd, f, b, s, so))
        self.V, self.ndim = V.value, nd.value
        self.has_F, self.has_B, self.has_S = bool(f.value), bool(b.value), bool(s.value)
        self.second_order = bool(so.value)


def builtin_system(name, ndim):
    key = ("builtin", name, ndim)
    if key not in _cache:
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().pypde_system_builtin(name.encode(), ndim, ctypes.byref(h)))
        _cache[key] = CompiledSystem(h, name)
    return _cache[key]


def resolve_system(F, B, S, ndim, V, secondOrder):
    """Find the device system behind the given callbacks."""
    tags = {getattr(f, "_pypde_builtin", None) for f in (F, B, S) if f is not None}
    if not tags:
        raise ValueError("at least one of F, B, S is required")
    if None in tags:
        raise NotImplementedError(
            "this callback has no device implementation; use the systems of "
            "pypde_gb300.systems")
    if len(tags) != 1:
        raise ValueError("F, B and S must come from one system")
    name, nd = tags.pop()
    if nd != ndim:
        raise ValueError(f"callbacks were built for ndim={nd}, Q0 has ndim={ndim}")
    sysobj = builtin_system(name, ndim)
    if sysobj.V != V:
        raise ValueError(f"system {name} has V={sysobj.V}, Q0 has V={V}")
    if sysobj.second_order != secondOrder:
        raise ValueError("second-order form does not match the callback signature")
    return sysobj

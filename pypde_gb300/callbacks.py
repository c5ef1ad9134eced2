"""Callbacks F/B/S -> a compiled device callback system.

Stands in for pypde/cfuncs.py:30-75, which compiles the user's Python
callbacks into host cfuncs with numba.  Here the callbacks must become
device code:
  * built-in systems (pypde_gb300.systems) map to kernels compiled ahead of
    time into libpypde_gb300.so;
  * any other Python callbacks are translated to CUDA C++ by
    pypde_gb300.translate and compiled at run time with NVRTC
    (pypde_system_compile), once per order N, cached on disk.
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


def compiled_system(F, B, S, ndim, V, name="user"):
    """Translate Python callbacks and register them as a run-time system."""
    from .translate import translate
    src = translate(F, B, S, ndim, V)
    key = ("jit", src, ndim, V)
    if key not in _cache:
        second = F is not None and len(__import__("inspect").signature(F).parameters) == 3
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().pypde_system_compile(src.encode(), name.encode(), ndim, V,
                                                   F is not None, B is not None, S is not None,
                                                   second, ctypes.byref(h)))
        cs = CompiledSystem(h, name)
        cs.source = src
        _cache[key] = cs
    return _cache[key]


def resolve_system(F, B, S, ndim, V, secondOrder, jit=False):
    """Find the device system behind the given callbacks: the built-in
    kernels when all callbacks come from one built-in system (unless jit),
    else run-time compiled device code."""
    tags = {getattr(f, "_pypde_builtin", None) for f in (F, B, S) if f is not None}
    if not tags:
        raise ValueError("at least one of F, B, S is required")
    if None in tags or jit:
        return compiled_system(F, B, S, ndim, V)
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

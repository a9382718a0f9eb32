"""FIESTA's Lua input deck run by the Lua 5.3 VM (libfst_deck.so,
include/fst_deck.h), for hosts that want the reference's own interpreter:
the same keys and conversions as the reference's luaReader, and
fiesta.initial_conditions / fiesta.initialize_grid called per cell / node.

    d = LuaDeck("fiesta.lua")
    cfg = d.config()                 # abi.FstConfig
    X = d.grid_nodes(cfg)            # generalized grids only
    U0 = d.initial_conditions(cfg, X)

The library is built by fiesta_gb300.build.build_deck() against the Lua
sources of a FIESTA tree; deck.py reads the same decks without it.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .build import DECK_LIB, build_deck

_lib = None


def available():
    """Whether libfst_deck.so exists or can be built here."""
    return os.path.exists(DECK_LIB) or build_deck() is not None


def lib():
    global _lib
    if _lib is None:
        if build_deck() is None and not os.path.exists(DECK_LIB):
            raise RuntimeError("libfst_deck.so needs Lua 5.3 sources (FST_LUA_SRC or a FIESTA "
                               "tree's tpls/lua/src)")
        L = C.CDLL(DECK_LIB)
        L.fst_deck_load.restype = C.c_int
        L.fst_deck_load.argtypes = [C.c_char_p, C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t]
        L.fst_deck_destroy.argtypes = [C.c_void_p]
        L.fst_deck_last_error.restype = C.c_char_p
        L.fst_deck_last_error.argtypes = [C.c_void_p]
        L.fst_deck_config.argtypes = [C.c_void_p, C.POINTER(abi.FstConfig)]
        L.fst_deck_noise.argtypes = [C.c_void_p, C.POINTER(abi.FstNoiseParams), C.POINTER(C.c_int)]
        L.fst_deck_grid_nodes.argtypes = [C.c_void_p, C.POINTER(abi.FstConfig),
                                          C.POINTER(C.c_double), C.c_size_t]
        L.fst_deck_initial_conditions.argtypes = [C.c_void_p, C.POINTER(abi.FstConfig),
                                                  C.POINTER(C.c_double), C.POINTER(C.c_double),
                                                  C.c_size_t]
        _lib = L
    return _lib


class LuaDeckError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


class LuaDeck:
    def __init__(self, path):
        self._h = C.c_void_p()
        err = C.create_string_buffer(1024)
        rc = lib().fst_deck_load(os.fsencode(path), C.byref(self._h), err, len(err))
        if rc != 0:
            raise LuaDeckError(rc, err.value.decode())

    def _check(self, rc):
        if rc != 0:
            raise LuaDeckError(rc, lib().fst_deck_last_error(self._h).decode())

    def config(self):
        cfg = abi.FstConfig()
        self._check(lib().fst_deck_config(self._h, C.byref(cfg)))
        return cfg

    def noise_params(self):
        np_, on = abi.FstNoiseParams(), C.c_int()
        self._check(lib().fst_deck_noise(self._h, C.byref(np_), C.byref(on)))
        return np_ if on.value else None

    def grid_nodes(self, cfg):
        ni, nj, nk, _ = abi.grid_dims(cfg)
        X = np.zeros((ni, nj, nk, 3), order="F")
        self._check(lib().fst_deck_grid_nodes(self._h, C.byref(cfg), _dp(X), X.size))
        return X

    def initial_conditions(self, cfg, nodes=None):
        U = np.zeros(abi.dims(cfg), order="F")
        X = None if nodes is None else np.asfortranarray(nodes)
        self._check(lib().fst_deck_initial_conditions(self._h, C.byref(cfg), _dp(X), _dp(U),
                                                      U.size))
        return U

    def close(self):
        if self._h:
            lib().fst_deck_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

"""ctypes binding of the engine's C ABI (include/pysic_gb300.h).

This module is the Python side of the drop-in boundary: it takes the place of
the f2py extension ``pysic.pysic_fortran`` (pysic/calculator.py:16).  There is
no fallback: if the compiled library is missing, importing the engine fails
with an error that says how to build it.
"""
import ctypes
import os
import weakref

import numpy as np

from .error import EngineError

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpysic_gb300.so")

PG_OK = 0
PG_ERR_INVALID = 1
PG_ERR_CUDA = 2
PG_ERR_NOT_READY = 3
PG_ERR_UNSUPPORTED = 4
PG_ERR_NOT_CONVERGED = 5
PG_ERR_TIMEOUT = 6
PG_ERR_SMALL_CELL = 7

PREC_FP64 = 0
PREC_MIXED = 1
WANT_ENERGY = 1
WANT_FORCES = 2
WANT_ENEGS = 4
LANES_TRIPLET = 64  # bond-order tile: 16 lanes per atom, one (bond, neighbour) pair per lane

_c_double_p = ctypes.POINTER(ctypes.c_double)
_c_int_p = ctypes.POINTER(ctypes.c_int32)
_c_u64_p = ctypes.POINTER(ctypes.c_uint64)
_c_i64_p = ctypes.POINTER(ctypes.c_int64)
_c_float_p = ctypes.POINTER(ctypes.c_float)
_ctx = ctypes.c_void_p

_SIGNATURES = {
    "pg_last_error": (ctypes.c_char_p, []),
    "pg_version": (ctypes.c_char_p, []),
    "pg_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p)]),
    "pg_destroy": (ctypes.c_int, [_ctx]),
    "pg_create_on": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32]),
    "pg_create_cell": (ctypes.c_int, [_ctx, _c_double_p, _c_double_p, _c_int_p]),
    "pg_create_atoms": (ctypes.c_int, [_ctx, ctypes.c_int32, _c_double_p, _c_double_p, _c_int_p]),
    "pg_update_atom_coordinates": (ctypes.c_int, [_ctx, _c_double_p]),
    "pg_update_atom_charges": (ctypes.c_int, [_ctx, _c_double_p]),
    "pg_get_atom_charges": (ctypes.c_int, [_ctx, _c_double_p]),
    "pg_set_pair_potentials": (ctypes.c_int, [_ctx, ctypes.c_int32, ctypes.c_int32, _c_int_p, _c_double_p,
                                              _c_double_p, _c_double_p, _c_u64_p, _c_u64_p, _c_int_p]),
    "pg_set_pair_products": (ctypes.c_int, [_ctx, ctypes.c_int32, _c_int_p, _c_int_p, ctypes.c_int32, _c_int_p,
                                            _c_double_p, _c_u64_p]),
    "pg_set_pair_tables": (ctypes.c_int, [_ctx, ctypes.c_int64, _c_double_p]),
    "pg_set_pair_first_targets": (ctypes.c_int, [_ctx, ctypes.c_int32, _c_u64_p]),
    "pg_set_triplet_potentials": (ctypes.c_int, [_ctx, ctypes.c_int32, _c_int_p, _c_double_p, _c_double_p,
                                                 _c_double_p, _c_u64_p, _c_u64_p, _c_u64_p, _c_u64_p]),
    "pg_set_quad_potentials": (ctypes.c_int, [_ctx, ctypes.c_int32, _c_int_p, _c_double_p, _c_double_p,
                                              _c_double_p, _c_u64_p, _c_u64_p]),
    "pg_set_single_potentials": (ctypes.c_int, [_ctx, ctypes.c_int32, _c_int_p, _c_double_p, _c_u64_p]),
    "pg_set_single_groups": (ctypes.c_int, [_ctx, ctypes.c_int32, _c_int_p]),
    "pg_set_pair_lanes": (ctypes.c_int, [_ctx, ctypes.c_int32]),
    "pg_get_atom_factors": (ctypes.c_int, [_ctx, ctypes.c_int32, ctypes.c_int32, _c_double_p]),
    "pg_get_atom_factor_gradients": (ctypes.c_int, [_ctx, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                    ctypes.c_int32, _c_double_p]),
    "pg_set_atom_factors": (ctypes.c_int, [_ctx, ctypes.c_int32, _c_int_p, _c_double_p, _c_double_p, _c_double_p,
                                           _c_u64_p, _c_u64_p, _c_int_p]),
    "pg_set_bond_order_factors": (ctypes.c_int, [_ctx, ctypes.c_int32, _c_double_p, _c_double_p, _c_double_p,
                                                 _c_u64_p, _c_u64_p, _c_u64_p, _c_int_p]),
    "pg_set_ewald": (ctypes.c_int, [_ctx, ctypes.c_double, ctypes.c_double, _c_int_p, ctypes.c_double,
                                    ctypes.c_double, _c_double_p]),
    "pg_clear_ewald": (ctypes.c_int, [_ctx]),
    "pg_generate_neighbor_lists": (ctypes.c_int, [_ctx, _c_double_p, ctypes.c_double]),
    "pg_generate_all_pairs_lists": (ctypes.c_int, [_ctx, _c_double_p, ctypes.c_double]),
    "pg_get_neighbor_counts": (ctypes.c_int, [_ctx, _c_int_p]),
    "pg_get_neighbor_lists": (ctypes.c_int, [_ctx, _c_int_p, _c_int_p]),
    "pg_create_neighbor_lists": (ctypes.c_int, [_ctx, _c_int_p, _c_int_p, _c_int_p, ctypes.c_double]),
    "pg_calculate_energy": (ctypes.c_int, [_ctx, ctypes.c_int32, _c_double_p]),
    "pg_calculate_forces": (ctypes.c_int, [_ctx, ctypes.c_int32, _c_double_p, _c_double_p]),
    "pg_calculate_electronegativities": (ctypes.c_int, [_ctx, ctypes.c_int32, _c_double_p]),
    "pg_calculate": (ctypes.c_int, [_ctx, ctypes.c_int32, ctypes.c_int32, _c_double_p, _c_double_p, _c_double_p,
                                    _c_double_p]),
    "pg_relax_charges": (ctypes.c_int, [_ctx, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, _c_double_p, _c_double_p, _c_int_p,
                                        _c_double_p, _c_double_p]),
    "pg_md_set_state": (ctypes.c_int, [_ctx, _c_double_p, _c_double_p]),
    "pg_md_run": (ctypes.c_int, [_ctx, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double, _c_int_p,
                                  _c_int_p]),
    "pg_get_list_positions": (ctypes.c_int, [_ctx, _c_double_p]),
    "pg_md_verlet": (ctypes.c_int, [_ctx, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                    _c_int_p, _c_int_p]),
    "pg_md_get_state": (ctypes.c_int, [_ctx, _c_double_p, _c_double_p]),
    "pg_optimize_charges": (ctypes.c_int, [_ctx, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, _c_double_p,
                                           _c_int_p, _c_double_p]),
    "pg_relax_charges_potentiostat": (ctypes.c_int, [_ctx, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                                     ctypes.c_double, ctypes.c_double, _c_double_p, _c_double_p,
                                                     _c_double_p]),
    "pg_get_bond_zeta": (ctypes.c_int, [_ctx, _c_double_p, ctypes.c_int64, _c_i64_p]),
    "pg_set_lanes_per_atom": (ctypes.c_int, [_ctx, ctypes.c_int32]),
    "pg_get_lanes_per_atom": (ctypes.c_int, [_ctx, _c_int_p]),
    "pg_device_evaluate": (ctypes.c_int, [_ctx, ctypes.c_int32, ctypes.c_int32]),
    "pg_device_synchronize": (ctypes.c_int, [_ctx]),
    "pg_device_results": (ctypes.c_int, [_ctx, _c_double_p, _c_double_p, _c_double_p, _c_double_p]),
    "pg_device_positions": (ctypes.c_int, [_ctx, ctypes.POINTER(_c_double_p)]),
    "pg_get_stream": (ctypes.c_int, [_ctx, ctypes.POINTER(ctypes.c_void_p)]),
    "pg_bond_order_noalloc": (ctypes.c_int, [_ctx, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]),
    "pg_device_allocation_count": (ctypes.c_int, [_c_u64_p]),
    "pg_measure_fp32_peak": (ctypes.c_int, [ctypes.c_int32, _c_double_p, _c_double_p]),
    "pg_last_launch_count": (ctypes.c_int, [_ctx, _c_int_p]),
    "pg_set_kernel_timing": (ctypes.c_int, [_ctx, ctypes.c_int32]),
    "pg_get_kernel_times": (ctypes.c_int, [_ctx, ctypes.POINTER(ctypes.c_float)]),
    "pg_set_graphs": (ctypes.c_int, [_ctx, ctypes.c_int32]),
    "pg_batch_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32]),
    "pg_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pg_batch_add": (ctypes.c_int, [ctypes.c_void_p, _ctx]),
    "pg_batch_set_lanes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]),
    "pg_batch_get_lanes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _c_int_p, _c_int_p]),
    "pg_batch_set_tile_blocks": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "pg_batch_get_tiles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, _c_int_p, _c_int_p, _c_int_p]),
    "pg_batch_test_stall": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double]),
    "pg_batch_evaluate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "pg_batch_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "pg_batch_get_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "pg_batch_last_launch_count": (ctypes.c_int, [ctypes.c_void_p, _c_int_p]),
    "pg_descriptors": (ctypes.c_int, [_ctx, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double, _c_float_p]),
    "pg_mlp_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32, ctypes.c_int32,
                                     ctypes.c_int32, ctypes.c_int32]),
    "pg_mlp_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pg_mlp_param_count": (ctypes.c_int, [ctypes.c_void_p, _c_i64_p]),
    "pg_mlp_set_params": (ctypes.c_int, [ctypes.c_void_p, _c_float_p, ctypes.c_int64]),
    "pg_mlp_get_params": (ctypes.c_int, [ctypes.c_void_p, _c_float_p, ctypes.c_int64]),
    "pg_mlp_add_samples": (ctypes.c_int, [ctypes.c_void_p, _c_float_p, _c_float_p, ctypes.c_int64]),
    "pg_mlp_clear_samples": (ctypes.c_int, [ctypes.c_void_p]),
    "pg_mlp_train": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_float, ctypes.c_uint64,
                                    _c_float_p]),
    "pg_mlp_gradients": (ctypes.c_int, [ctypes.c_void_p, _c_float_p, _c_float_p, ctypes.c_int64, _c_float_p,
                                        _c_double_p]),
    "pg_mlp_predict": (ctypes.c_int, [ctypes.c_void_p, _c_float_p, ctypes.c_int64, _c_float_p]),
    "pg_mlp_predict_charges": (ctypes.c_int, [ctypes.c_void_p, _ctx, ctypes.c_int32, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                              _c_int_p, _c_float_p, _c_float_p, ctypes.c_double, ctypes.c_double,
                                              ctypes.c_double, _c_double_p]),
}

# The two calls of a force-evaluation step, bound a second time with plain
# addresses (c_void_p) so that a step passes integers instead of building a
# ctypes pointer object per array (about 2 us each).
_ADDR_SIGNATURES = {
    "pg_update_atom_coordinates": (ctypes.c_int, [_ctx, ctypes.c_void_p]),
    "pg_calculate": (ctypes.c_int, [_ctx, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p]),
}

_lib = None
_addr_lib = None


def exported_symbols():
    return list(_SIGNATURES.keys())


def load(path=LIB_PATH):
    """Load the engine library (once).  Raises ImportError if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("GB300 engine library not found at {0}; build it with "
                          "`python -m pysic_gb300.build` (needs nvcc)".format(path))
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    global _addr_lib
    alib = ctypes.CDLL(path)  # separate function objects with their own argument types
    for name, (res, args) in _ADDR_SIGNATURES.items():
        fn = getattr(alib, name)
        fn.restype = res
        fn.argtypes = args
    _addr_lib = alib
    _lib = lib
    return lib


def addr_lib():
    """The step calls bound with plain addresses (see _ADDR_SIGNATURES)."""
    load()
    return _addr_lib


class AddressCache:
    """Data addresses of float64 C-contiguous arrays passed again and again
    (a caller's step buffers), looked up by identity through weak references,
    so that the arrays are not kept alive here and a recycled id is never
    mistaken for the old array."""

    def __init__(self, size=8):
        self.size = size
        self._d = {}

    def __call__(self, a):
        if a is None:
            return None
        e = self._d.get(id(a))
        if e is not None and e[0]() is a:
            return e[1]
        if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
            raise TypeError("expected a C-contiguous float64 array")
        addr = a.__array_interface__["data"][0]
        if len(self._d) >= self.size:
            self._d.pop(next(iter(self._d)))
        try:
            self._d[id(a)] = (weakref.ref(a), addr)
        except TypeError:  # not weak-referenceable: no caching
            pass
        return addr


def check(status):
    if status != PG_OK:
        msg = _lib.pg_last_error().decode(errors="replace") if _lib is not None else ""
        raise EngineError(status, msg)


def dptr(a):
    return a.ctypes.data_as(_c_double_p)


def fptr(a):
    return a.ctypes.data_as(_c_float_p)


def iptr(a):
    return a.ctypes.data_as(_c_int_p)


def u64ptr(a):
    return a.ctypes.data_as(_c_u64_p)


def as_f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


def as_i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def as_u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)

"""Many independent systems evaluated together (no counterpart in the
reference, which holds one system per process).

    batch = BatchedPysic([calc_1, calc_2, ...])
    batch.evaluate(precision="mixed")          # one persistent launch for all
    results = batch.results()                  # energy, forces, stress per system

Every calculator is set up as usual (atoms, potentials, neighbour lists); the
batch borrows their engine contexts and evaluates all of them in one
persistent launch that walks a work list of (phase, system, cells) tiles
(pg_batch_* in the C ABI).  ``mode="phases"`` uses one launch per phase
instead and ``mode="each"`` evaluates the systems one by one, for comparison.
"""
import ctypes

import numpy as np

from . import _lib as L

_PREC = {"fp64": L.PREC_FP64, "mixed": L.PREC_MIXED}
_MODE = {"batched": 0, "each": 1, "phases": 2}


class BatchedPysic:
    def __init__(self, calculators, device=-1, pair_lanes=0, bond_lanes=0):
        self.lib = L.load()
        self.calculators = list(calculators)
        h = ctypes.c_void_p()
        L.check(self.lib.pg_batch_create(ctypes.byref(h), int(device)))
        self.h = h
        for c in self.calculators:
            c.set_core()
            L.check(self.lib.pg_batch_add(self.h, c.engine.ctx))
        if pair_lanes or bond_lanes:
            self.set_lanes(pair_lanes, bond_lanes)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.lib.pg_batch_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def set_lanes(self, pair_lanes=0, bond_lanes=0):
        L.check(self.lib.pg_batch_set_lanes(self.h, int(pair_lanes), int(bond_lanes)))

    def get_lanes(self, precision="mixed"):
        p, q = ctypes.c_int32(0), ctypes.c_int32(0)
        L.check(self.lib.pg_batch_get_lanes(self.h, _PREC[precision], ctypes.byref(p), ctypes.byref(q)))
        return p.value, q.value

    def set_tile_blocks(self, blocks=0):
        """Cells (blocks of 128 threads' atoms) per work tile of the persistent
        launch; 0 lets the batch time the candidates."""
        L.check(self.lib.pg_batch_set_tile_blocks(self.h, int(blocks)))

    def get_tiles(self, precision="mixed", mode="batched"):
        """(pair lanes, bond lanes, cells per tile) in use for `mode`."""
        p, q, c = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_int32(0)
        L.check(self.lib.pg_batch_get_tiles(self.h, _PREC[precision], _MODE[mode], ctypes.byref(p), ctypes.byref(q),
                                            ctypes.byref(c)))
        return p.value, q.value, c.value

    def test_stall(self, system, wait_seconds=0.05):
        """Test hook of the persistent launch's bounded waits: the tiles of
        `system` wait for work that never comes (-1 ends the test); the next
        results() raises EngineError with PG_ERR_TIMEOUT."""
        L.check(self.lib.pg_batch_test_stall(self.h, int(system), float(wait_seconds)))

    def evaluate(self, precision="mixed", forces=True, mode="batched"):
        """Enqueue one energy (+ forces and virial) evaluation of every system;
        returns without waiting.  mode: "batched" (one persistent launch),
        "phases" (one launch per phase) or "each" (system by system)."""
        flags = L.WANT_ENERGY | (L.WANT_FORCES if forces else 0)
        L.check(self.lib.pg_batch_evaluate(self.h, _PREC[precision], flags, _MODE[mode]))

    def synchronize(self):
        L.check(self.lib.pg_batch_synchronize(self.h))

    def stream_handle(self):
        s = ctypes.c_void_p()
        L.check(self.lib.pg_batch_get_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def launch_count(self):
        v = ctypes.c_int32(0)
        L.check(self.lib.pg_batch_last_launch_count(self.h, ctypes.byref(v)))
        return v.value

    def results(self):
        self.synchronize()
        return [c.engine.device_results() for c in self.calculators]

    def energies(self):
        return np.array([r["energy"] for r in self.results()])

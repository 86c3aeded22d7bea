"""Learned warm start for ChargeRelaxation (no counterpart in the reference).

A small network maps per-atom radial descriptors to a starting charge; the
plain damped relaxation (pysic/charges/relaxation.py:394-450) then runs from
there to the same tolerance, so the converged charges are the reference's
own.  Descriptors, forward pass, backward pass and Adam run on the GPU in the
engine (csrc/mlp.cu); this module holds the settings, the file format of a
trained network and the glue to a calculator.

Descriptors: for each element type t and Gaussian k (``n_gauss`` centres
evenly spaced on [r0, r1], width ``width``), the sum over neighbours j of type
t within ``cutoff`` of exp(-(r_ij - mu_k)^2 / 2 w^2) times the cosine cutoff
1/2 (1 + cos(pi r_ij / cutoff)).  Network: n_in -> n_h1 -> n_h2 -> 1, tanh,
BF16 weights, FP32 arithmetic.
"""
import ctypes
import os

import numpy as np

from . import _lib as L

DEFAULT_DESCRIPTOR = {"n_gauss": 16, "r0": 0.8, "r1": 5.0, "width": 0.35, "cutoff": 5.0}
DEFAULT_LAYERS = (64, 64)
DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")


def inputs_from_types(raw, types, type_elements, elements, n_gauss):
    """Fold per-type descriptor columns into per-element columns and append
    the one-hot element code of each atom."""
    E = len(elements)
    out = np.zeros((raw.shape[0], E * n_gauss + E), dtype=np.float32)
    for t, el in enumerate(type_elements):
        if el not in elements:
            raise ValueError("the network was not trained for element " + str(el))
        e = elements.index(el)
        out[:, e * n_gauss:(e + 1) * n_gauss] += raw[:, t * n_gauss:(t + 1) * n_gauss]
        out[np.asarray(types) == t, E * n_gauss + e] = 1.0
    return out


class ChargeNetwork:
    """The warm-start network on the GPU (pg_mlp_* of the C ABI)."""

    def __init__(self, n_in, n_h1=DEFAULT_LAYERS[0], n_h2=DEFAULT_LAYERS[1], device=-1, descriptor=None,
                 elements=None):
        self.lib = L.load()
        self.n_in, self.n_h1, self.n_h2 = int(n_in), int(n_h1), int(n_h2)
        self.descriptor = dict(DEFAULT_DESCRIPTOR if descriptor is None else descriptor)
        self.elements = list(elements) if elements is not None else None
        # normalisation of inputs (per feature) and of the target, fixed at training time
        self.x_mean = np.zeros(self.n_in, dtype=np.float32)
        self.x_scale = np.ones(self.n_in, dtype=np.float32)
        self.y_mean, self.y_scale = 0.0, 1.0
        h = ctypes.c_void_p()
        L.check(self.lib.pg_mlp_create(ctypes.byref(h), self.n_in, self.n_h1, self.n_h2, int(device)))
        self.h = h
        n = ctypes.c_int64(0)
        L.check(self.lib.pg_mlp_param_count(self.h, ctypes.byref(n)))
        self.n_params = n.value

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.lib.pg_mlp_destroy(self.h)
                self.h = None
        except Exception:
            pass

    # ---- parameters ----------------------------------------------------------
    def get_params(self):
        p = np.zeros(self.n_params, dtype=np.float32)
        L.check(self.lib.pg_mlp_get_params(self.h, L.fptr(p), self.n_params))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        L.check(self.lib.pg_mlp_set_params(self.h, L.fptr(p), p.size))

    def save(self, path):
        np.savez(path, params=self.get_params(), layers=np.array([self.n_in, self.n_h1, self.n_h2]),
                 x_mean=self.x_mean, x_scale=self.x_scale, y_norm=np.array([self.y_mean, self.y_scale]),
                 descriptor=np.array([self.descriptor[k] for k in ("n_gauss", "r0", "r1", "width", "cutoff")]),
                 elements=np.array(self.elements if self.elements else []))

    @classmethod
    def load(cls, path, device=-1):
        d = np.load(path)
        n_in, n_h1, n_h2 = (int(v) for v in d["layers"])
        g, r0, r1, w, rc = (float(v) for v in d["descriptor"])
        net = cls(n_in, n_h1, n_h2, device=device,
                  descriptor={"n_gauss": int(g), "r0": r0, "r1": r1, "width": w, "cutoff": rc},
                  elements=[str(e) for e in d["elements"]])
        net.set_params(d["params"])
        net.x_mean, net.x_scale = d["x_mean"].astype(np.float32), d["x_scale"].astype(np.float32)
        net.y_mean, net.y_scale = float(d["y_norm"][0]), float(d["y_norm"][1])
        return net

    # ---- data, training, inference -----------------------------------------------
    def normalise_from(self, x, y):
        self.x_mean = x.mean(axis=0).astype(np.float32)
        self.x_scale = (x.std(axis=0) + 1e-6).astype(np.float32)
        self.y_mean, self.y_scale = float(y.mean()), float(y.std() + 1e-6)

    def _nx(self, x):
        return np.ascontiguousarray((x - self.x_mean) / self.x_scale, dtype=np.float32)

    def add_samples(self, x, y):
        xn = self._nx(x)
        yn = np.ascontiguousarray((y - self.y_mean) / self.y_scale, dtype=np.float32)
        L.check(self.lib.pg_mlp_add_samples(self.h, L.fptr(xn), L.fptr(yn), len(yn)))

    def clear_samples(self):
        L.check(self.lib.pg_mlp_clear_samples(self.h))

    def train(self, epochs, batch=4096, learning_rate=1e-3, seed=0):
        losses = np.zeros(max(epochs, 1), dtype=np.float32)
        L.check(self.lib.pg_mlp_train(self.h, int(epochs), int(batch), float(learning_rate), int(seed),
                                      L.fptr(losses)))
        return losses[:epochs]

    def predict(self, x):
        xn = self._nx(x)
        y = np.zeros(len(xn), dtype=np.float32)
        L.check(self.lib.pg_mlp_predict(self.h, L.fptr(xn), len(xn), L.fptr(y)))
        return y.astype(np.float64) * self.y_scale + self.y_mean

    def gradients(self, x, y):
        """Loss and gradient of the mean squared error on raw (already
        normalised) inputs and targets, without an update."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = ctypes.c_double(0)
        L.check(self.lib.pg_mlp_gradients(self.h, L.fptr(x), L.fptr(y), len(y), L.fptr(g), ctypes.byref(loss)))
        return loss.value, g

    # ---- calculators ---------------------------------------------------------------
    def descriptors(self, calc):
        """Network inputs of every atom of the calculator's structure: the
        radial features per neighbour element (in the order of
        ``self.elements``) followed by a one-hot code of the atom's own
        element."""
        d = self.descriptor
        calc.set_core()
        model = calc._model
        g = d["n_gauss"]
        raw = calc.engine.descriptors(model.n_types, g, d["r0"], d["r1"], d["width"], d["cutoff"])
        return inputs_from_types(raw, model.types, [sig[0] for sig in model.type_signatures], self.elements, g)

    def predict_charges(self, calc, total_charge=0.0):
        """Starting charges for the calculator's structure, shifted so that
        they add up to total_charge (the relaxation conserves the sum).  The
        whole prediction runs on the device (pg_mlp_predict_charges) and the
        engine keeps the predicted charges; a copy is returned."""
        d = self.descriptor
        calc.set_core()
        model = calc._model
        type_el = np.array([self._element_index(sig[0]) for sig in model.type_signatures], dtype=np.int32)
        q = np.zeros(len(model.types))
        xm = np.ascontiguousarray(self.x_mean, dtype=np.float32)
        xs = np.ascontiguousarray(self.x_scale, dtype=np.float32)
        L.check(self.lib.pg_mlp_predict_charges(
            self.h, calc.engine.ctx, int(d["n_gauss"]), float(d["r0"]), float(d["r1"]), float(d["width"]),
            float(d["cutoff"]), len(self.elements), L.iptr(type_el), L.fptr(xm), L.fptr(xs),
            float(self.y_mean), float(self.y_scale), float(total_charge), L.dptr(q)))
        return q

    def predict_charges_host(self, calc, total_charge=0.0):
        """The same prediction through the host: descriptors copied out, folded
        and normalised with NumPy, the network on the device, the shift in
        NumPy.  For comparisons with predict_charges."""
        q = self.predict(self.descriptors(calc))
        return q - (q.sum() - total_charge) / len(q)

    def _element_index(self, el):
        if not self.elements or el not in self.elements:
            raise ValueError("the network was not trained for element " + str(el))
        return self.elements.index(el)

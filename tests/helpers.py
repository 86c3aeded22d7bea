"""Shared helpers: run the oracle and the engine on the same structure and records."""
import numpy as np

import oracle
from pysic_gb300.model import compile_model, individual_cutoffs

SKIN = 0.5


def oracle_lists(atoms, pots, coulomb=None, skin=SKIN):
    cuts = np.array(individual_cutoffs(atoms, pots, coulomb)) + skin
    return oracle.neighbors(atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(), cuts)


def oracle_all(atoms, pots, coulomb=None, lists=None, threads=1):
    model = compile_model(atoms, pots, coulomb)
    c, i, o = lists if lists is not None else oracle_lists(atoms, pots, coulomb)
    args = (atoms.get_positions(), atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc(), model, c, i, o)
    e = oracle.evaluate(*args, what="energy", threads=threads)
    f, s = oracle.evaluate(*args, what="forces", threads=threads)
    chi = oracle.evaluate(*args, what="enegs", threads=threads)
    return {"energy": e, "forces": f, "stress": s, "enegs": chi, "model": model, "lists": (c, i, o)}


def engine_all(atoms, pots, coulomb=None, precision="fp64", lanes=0):
    import pysic_gb300 as pysic

    calc = pysic.Pysic(atoms, pots, coulomb=coulomb, precision=precision)
    calc.set_core()
    if lanes:
        calc.engine.set_lanes(lanes)
    r = calc.engine.calculate(calc._prec(), energy=True, forces=True, enegs=True)
    r["calc"] = calc
    return r

"""Regenerate the golden fixtures of this directory.

    python tests/golden/make_golden.py [--reference-root DIR]

reference_docs.json
    The known answers printed in the reference's documentation, read from the
    documentation files themselves when the reference tree is available
    (default location: the REFERENCE_ROOT environment variable):
      * He2 Lennard-Jones, doc/run examples.rst:141-145 (energy and forces),
      * C-O-H with two LJ potentials, doc/pysic class.rst:130-157 (energies
        and forces of pot1 alone, pot2 alone, and both in one calculator),
      * the COMB10 default parameters of pysic/interactions/comb.py:81-517
        (read from the source text: literal values, and the mixed Si-O values
        from the two rules used there, geometric mean and arithmetic mean).
    Without the reference tree the committed file is kept as it is.

oracle_cases.npz
    The FP64 oracle's neighbour lists, energy, forces, virial,
    electronegativities (and, for the SiO2 case, relaxed charges) for the
    seeded cases of cases.py.  The oracle is pinned by the documented values
    above and by the tests in tests/test_oracle.py; these arrays let the GPU
    tests compare against stored numbers and let the CPU tests detect any
    later drift of the oracle itself.
"""
import argparse
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle"), HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

FLOAT = r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?"


def _floats(lines):
    return [float(x) for line in lines for x in re.findall(FLOAT, line)]


def _block(lines, start, count):
    """`count` lines of a printed numpy array starting at 1-based line `start`."""
    return np.array(_floats(lines[start - 1:start - 1 + count])).reshape(count, 3)


def reference_docs(ref_root):
    doc = os.path.join(ref_root, "doc")
    run = open(os.path.join(doc, "run examples.rst")).read().splitlines()
    cls = open(os.path.join(doc, "pysic class.rst")).read().splitlines()

    def line(lines, i, must):
        text = lines[i - 1]
        assert must in text, (i, text)
        return text

    he2_e = float(line(run, 142, "-0.0222").strip())
    he2_f = np.array(_floats([line(run, 144, "array"), line(run, 145, "0.")])).reshape(2, 3)
    out = {
        "he2_lj": {
            "source": "doc/run examples.rst:106-145",
            "symbols": ["He", "He"],
            "positions": [[0.0, 0.0, 0.0], [0.0, 0.0, 3.0]],
            "potential": {"kind": "LJ", "symbols": ["He", "He"], "epsilon": 0.1, "sigma": 2.5, "cutoff": 10.0},
            "energy": he2_e,
            "forces": he2_f.tolist(),
            "printed_digits": 8,
        },
        "coh_lj": {
            "source": "doc/pysic class.rst:88-157",
            "symbols": ["C", "O", "H"],
            "positions": [[0.0, 0.0, 0.0], [2.0, 0.0, 0.0], [2.0, 2.0, 2.0]],
            "pot1": {"kind": "LJ", "symbols": ["C", "O"], "parameters": [1, 1], "cutoff": 10.0},
            "pot2": {"kind": "LJ", "symbols": ["O", "H"], "parameters": [1, 1], "cutoff": 10.0},
            "energy_pot1": float(line(cls, 133, "-0.0153").strip()),
            "forces_pot1": _block(cls, 134, 3).tolist(),
            "energy_pot2": float(line(cls, 140, "-0.0019").strip()),
            "forces_pot2": _block(cls, 141, 3).tolist(),
            "energy_both": float(line(cls, 154, "-0.0173").strip()),
            "forces_both": _block(cls, 155, 3).tolist(),
            "printed_digits": 8,
        },
    }
    out["comb10_parameters"] = {"source": "pysic/interactions/comb.py:81-517",
                                "values": comb10_parameters(ref_root)}
    return out


def comb10_parameters(ref_root):
    """name -> default value of CombPotential's parameter table, parsed from
    the reference's source text (no code of it is run)."""
    text = open(os.path.join(ref_root, "pysic", "interactions", "comb.py")).read()
    body = text[text.index("def __init__"):text.index("def get_parameter_value")]
    values, name = {}, None
    for m in re.finditer(r"newparam = '([^']+)'|self\.params\[newparam\] = (.*?)\n\s*self\.n_params", body, re.S):
        if m.group(1):
            name = m.group(1)
            continue
        expr = " ".join(m.group(2).replace("\\", " ").split())
        refs = re.findall(r"self\.params\['([^']+)'\]", expr)
        if not refs:
            values[name] = float(expr)
        elif expr.startswith("math.sqrt(") and len(refs) == 2 and "*" in expr:
            values[name] = float(np.sqrt(values[refs[0]] * values[refs[1]]))
        elif expr.endswith("* 0.5") and len(refs) == 2 and "+" in expr:
            values[name] = (values[refs[0]] + values[refs[1]]) * 0.5
        else:
            raise ValueError("unexpected parameter expression for %r: %s" % (name, expr))
    return values


def oracle_cases():
    import oracle
    from cases import CASES, RELAX
    from pysic_gb300.model import compile_model, individual_cutoffs

    oracle.build()
    arrays = {}
    for name, make in CASES.items():
        atoms, pots, coul = make()
        cuts = np.array(individual_cutoffs(atoms, pots, coul)) + 0.5
        pos, q, cell, pbc = atoms.get_positions(), atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc()
        c, i, o = oracle.neighbors(pos, cell, pbc, cuts)
        model = compile_model(atoms, pots, coul)
        args = (pos, q, cell, pbc, model, c, i, o)
        e = oracle.evaluate(*args, what="energy")
        f, s = oracle.evaluate(*args, what="forces")
        chi = oracle.evaluate(*args, what="enegs")
        pre = name + "/"
        arrays.update({
            pre + "symbols": np.array(atoms.get_chemical_symbols()),
            pre + "positions": pos, pre + "cell": cell, pre + "pbc": np.array(pbc, dtype=np.int8),
            pre + "charges": q, pre + "cutoffs": cuts,
            pre + "nb_counts": c.astype(np.int32), pre + "nb_index": i.astype(np.int32),
            pre + "nb_offset": o.astype(np.int32),
            pre + "energy": np.array(e), pre + "forces": f, pre + "stress": s, pre + "enegs": chi,
        })
        if name == "sio2_120":
            r = oracle.relax_charges(pos, q, cell, pbc, model, c, i, o, **RELAX)
            arrays.update({pre + "relaxed_charges": r["charges"], pre + "relaxed_rates": r["rates"],
                           pre + "relax_steps": np.array(r["steps"]), pre + "relax_error": np.array(r["error"])})
        print("%-16s n=%4d E=% .12f  list entries %d" % (name, len(atoms), e, len(i)))
    return arrays


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-root", default=os.environ.get("REFERENCE_ROOT"),
                    help="checkout of the reference (thynnine/pysic) whose doc/ holds the documented values; "
                         "default: the REFERENCE_ROOT environment variable")
    args = ap.parse_args()
    if args.reference_root and os.path.isdir(os.path.join(args.reference_root, "doc")):
        docs = reference_docs(args.reference_root)
        with open(os.path.join(HERE, "reference_docs.json"), "w") as fh:
            json.dump(docs, fh, indent=1)
        print("reference_docs.json written from", args.reference_root)
    else:
        print("reference tree not found: reference_docs.json kept")
    np.savez_compressed(os.path.join(HERE, "oracle_cases.npz"), **oracle_cases())
    print("oracle_cases.npz written")


if __name__ == "__main__":
    main()

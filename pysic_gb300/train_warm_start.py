"""Train the charge-relaxation warm-start network on relaxed SiO2 boxes.

    python -m pysic_gb300.train_warm_start [--configs 2000] [--out FILE]

Every training configuration is a seeded random SiO2 box (1000 Si + 2000 O at
2.2 g/cm^3, rejection below 1.5 A; seeds from --seed-base upwards, disjoint
from the evaluation seeds 0..999 that bench.py uses) relaxed to the tolerance
by the plain 'dynamic' ChargeRelaxation on the GPU.  The per-atom descriptors
of the relaxed structure and its relaxed charges are the samples; the network
is trained on the GPU by the engine's own forward, backward and Adam kernels.
Five percent of the configurations are held out for validation.  The trained
network and a JSON report (timings, losses, validation error) are written next
to each other.
"""
import argparse
import json
import multiprocessing as mp
import os
import time

import numpy as np

# Damped-dynamics settings for these boxes: the charge Hessian's largest
# eigenvalue reaches ~400 eV/e^2 (Si-O pairs at 1.5-1.6 A), so the time step
# must stay below ~2/sqrt(400) = 0.1; 0.05 with friction 3 converges in ~140
# steps from zero charges, and 0.08 already diverges.
RELAX = {"n_steps": 4000, "timestep": 0.05, "inertia": 1.0, "friction": 3.0, "tolerance": 1e-4}


def _structure(args):
    seed, n_si = args
    from pysic_gb300 import workloads as W

    a = W.sio2_box(n_si, seed=seed)
    return a.get_positions(), a.get_cell()[0, 0]


def relax(calc, params=RELAX, network=None):
    """The plain 'dynamic' relaxation of the calculator's structure from zero
    charges (network None) or from the network's prediction."""
    import pysic_gb300 as pysic

    s = calc.get_atoms()
    s.set_initial_charges(np.zeros(len(s)))
    rel = pysic.ChargeRelaxation("dynamic", calculator=calc, warm_start=network,
                                 parameters=[params[k] for k in ("n_steps", "timestep", "inertia", "friction",
                                                                 "tolerance")])
    q = rel.charge_relaxation()
    return q, rel


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--configs", type=int, default=2000)
    ap.add_argument("--n-si", type=int, default=1000)
    ap.add_argument("--seed-base", type=int, default=100000)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--workers", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                                                  "sio2_warm_start.npz"))
    args = ap.parse_args()

    # structures first, in worker processes started before any GPU use
    t0 = time.perf_counter()
    jobs = [(args.seed_base + k, args.n_si) for k in range(args.configs)]
    with mp.get_context("spawn").Pool(max(1, args.workers)) as pool:
        structures = pool.map(_structure, jobs, chunksize=8)
    t_struct = time.perf_counter() - t0

    import pysic_gb300 as pysic
    from pysic_gb300 import workloads as W
    from pysic_gb300.mlp import ChargeNetwork

    symbols = ["Si"] * args.n_si + ["O"] * (2 * args.n_si)
    pots, coul = W.sio2_potentials()
    pos0, L0 = structures[0]
    atoms = pysic.Atoms(symbols, pos0, cell=np.eye(3) * L0, pbc=True)
    calc = pysic.Pysic(atoms, pots, coulomb=coul, precision="mixed")
    net = ChargeNetwork(n_in=2 * 16 + 2, elements=["Si", "O"])

    t0 = time.perf_counter()
    xs, ys, steps = [], [], []
    for k, (pos, L) in enumerate(structures):
        a = pysic.Atoms(symbols, pos, cell=np.eye(3) * L, pbc=True)
        calc.set_atoms(a)
        q, rel = relax(calc)
        if not rel.last_converged:
            continue
        steps.append(rel.last_steps)
        xs.append(net.descriptors(calc))
        ys.append(q.astype(np.float32))
    t_relax = time.perf_counter() - t0
    n_cfg = len(xs)
    n_val = max(1, n_cfg // 20)
    x_tr, y_tr = np.concatenate(xs[n_val:]), np.concatenate(ys[n_val:])
    x_va, y_va = np.concatenate(xs[:n_val]), np.concatenate(ys[:n_val])

    net.normalise_from(x_tr, y_tr)
    net.add_samples(x_tr, y_tr)
    t0 = time.perf_counter()
    losses = []
    for stage, lr in enumerate((args.lr, args.lr / 4, args.lr / 16)):
        losses += [float(v) for v in net.train(max(1, args.epochs // 3), batch=args.batch, learning_rate=lr,
                                               seed=stage)]
    t_train = time.perf_counter() - t0
    pred = net.predict(x_va)
    rmse = float(np.sqrt(np.mean((pred - y_va) ** 2)))
    mae = float(np.mean(np.abs(pred - y_va)))

    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    net.save(args.out)
    report = {"configs_relaxed": n_cfg, "configs_requested": args.configs, "atoms_per_config": len(symbols),
              "train_samples": int(len(y_tr)), "validation_samples": int(len(y_va)),
              "relax_steps_mean": float(np.mean(steps)), "relax_settings": RELAX,
              "seconds": {"structures": t_struct, "relaxation_and_descriptors": t_relax, "training": t_train,
                          "per_epoch": t_train / max(1, len(losses))},
              "training_kernels": "tensor cores (mma.sync m16n8k16, BF16 operands, FP32 accumulation)"
                                  if net.n_h1 == 64 and net.n_h2 == 64 and net.n_in <= 64 else "scalar FP32",
              "epoch_loss_normalised": losses, "validation_rmse_e": rmse, "validation_mae_e": mae,
              "charge_std_e": float(np.std(y_va)), "epochs": len(losses), "batch": args.batch}
    with open(os.path.splitext(args.out)[0] + ".json", "w") as fh:
        json.dump(report, fh, indent=1)
    print(json.dumps({k: v for k, v in report.items() if k != "epoch_loss_normalised"}))


if __name__ == "__main__":
    main()

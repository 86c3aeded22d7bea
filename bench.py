#!/usr/bin/env python
"""Benchmark of the GB300 engine: Tersoff-silicon atom-steps/s, mixed precision
against the plain FP64 kernels, on the 16x16x16 diamond cell (32768 atoms).

One step = one energy + forces + virial evaluation of the whole structure
(neighbour list built once; positions fixed, as in the benchmark definition:
repeated evaluations at fixed positions).  The L2 cache (126 MB) is flushed
between timed steps by writing a 256 MB buffer; steps are timed with CUDA
events on the engine's stream.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload NAME]

--impl reference times the CPU restatement of the reference's Fortran core
(the Fortran itself cannot be compiled on these machines: no Fortran
compiler) on all host cores, on the same workload.  With torchrun (N > 1) each
rank runs an independent replica on its own GPU (the workload does not shard:
replicas only).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Tersoff-Si atom-steps/s mixed vs FP64 on GPU @1e-5 eV/atom; charge-relax gain"

# algorithmic cost per atom of one Tersoff energy + force evaluation: positions
# (16 B), neighbour entries (4 x 8 B), forces (24 B) = 72 B/atom; ~2.0 kFLOP/atom
TERSOFF_BYTES_PER_ATOM = 72.0
TERSOFF_FLOP_PER_ATOM = 2.0e3


def fp32_peak(device):
    """FP32 TFLOP/s of this GPU, measured now: the engine's FMA-chain kernel on
    every SM (pg_measure_fp32_peak), best of six timed launches."""
    import ctypes

    from pysic_gb300 import _lib as L

    lib = L.load()
    tf, ms = ctypes.c_double(0.0), ctypes.c_double(0.0)
    L.check(lib.pg_measure_fp32_peak(int(device), ctypes.byref(tf), ctypes.byref(ms)))
    return tf.value


def workload(name):
    from pysic_gb300 import workloads as W

    if name == "tersoff_si_32768":
        return W.diamond_si(16, seed=0), W.tersoff_si_potentials(), None, "diamond Si 16x16x16 cells, a=5.431, noise 0.10"
    if name == "tersoff_si_4096":
        return W.diamond_si(8, seed=0), W.tersoff_si_potentials(), None, "diamond Si 8x8x8 cells, a=5.431, noise 0.10"
    if name == "lj_fcc_864":
        return W.lj_fcc(), W.lj_potentials(), None, "LJ fcc 6x6x6 cells, a=5.26, noise 0.05, cutoff 8.5"
    if name == "ewald_nacl_8000":
        pots, coul = W.nacl_potentials()
        return W.rocksalt_nacl(), pots, coul, "rock salt 10x10x10 cells, Buckingham + Ewald (rc 10, sigma 2.5)"
    if name == "sutton_chen_cu_32000":
        from pysic_gb300 import Pysic

        calc = Pysic()
        calc.add_potential(W.sutton_chen_potentials(("Cu",), cutoff=5.0, cutoff_margin=0.5))
        return (W.fcc_alloy(20, symbols=("Cu",), noise=0.05, seed=0), calc.get_potentials(), None,
                "fcc Cu 20x20x20 cells, a=3.61, noise 0.05, Sutton-Chen (cutoff 5.0, margin 0.5)")
    if name == "comb_sio2_3000":
        # the COMB compound (COMB10 parameters, 12 A Coulomb and field ranges,
        # screened real-space Ewald) on a random SiO2 box with random charges
        from pysic_gb300 import CombPotential, Pysic

        atoms = W.sio2_box(1000, seed=81)
        q = np.random.default_rng(82).normal(0.0, 0.4, len(atoms))
        atoms.set_initial_charges(q - q.mean())
        calc = Pysic()
        CombPotential().set_calculator(calc, True)
        return (atoms, calc.get_potentials(), calc.get_coulomb_summation(),
                "random SiO2 1000 Si + 2000 O at 2.2 g/cm^3, random charges (0.4 e), COMB10 compound "
                "(40 pieces, 12 A ranges)")
    raise SystemExit("unknown workload " + name)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_traffic(kernel, workload_name):
    """dram bytes per launch from the committed ncu summary, if there is one."""
    kernel = {"kspace": "ew_field", "pair": "pair_kernel"}.get(kernel, kernel)
    path = os.path.join(ROOT, "profiles", "{0}_{1}.md".format(kernel, workload_name))
    try:
        for line in open(path):
            if line.lower().startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def setup(name, precision, device):
    import pysic_gb300 as pysic
    from pysic_gb300.engine import Engine

    atoms, pots, coul, desc = workload(name)
    calc = pysic.Pysic(atoms, pots, coulomb=coul, precision=precision)
    calc._engine = Engine(device=device)
    calc.set_core()
    return atoms, calc, desc


def device_time(torch, engine, prec, flags, steps, warmup, flush):
    """Per-step CUDA-event times (ms) on the engine's stream, L2 flushed before each step."""
    stream = torch.cuda.ExternalStream(engine.stream_handle())
    for _ in range(warmup):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        engine.device_evaluate(prec, flags)
    engine.device_synchronize()
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    launches = 0
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))
            ev0[k].record(stream)
        engine.device_evaluate(prec, flags)
        launches += engine.launch_count()
        with torch.cuda.stream(stream):
            ev1[k].record(stream)
    stream.synchronize()
    return [a.elapsed_time(b) for a, b in zip(ev0, ev1)], launches


def kernel_time(torch, engine, prec, flags, steps, flush):
    """Average duration of each kernel group, from events recorded by the engine
    around its own launches (same stream)."""
    engine.set_kernel_timing(True)
    stream = torch.cuda.ExternalStream(engine.stream_handle())
    acc = {}
    for k in range(steps + 2):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))
        engine.device_evaluate(prec, flags)
        t = engine.kernel_times()
        if k >= 2:
            for key, v in t.items():
                acc.setdefault(key, []).append(v)
    engine.set_kernel_timing(False)
    return {k: statistics.mean(v) for k, v in acc.items()}


def e2e_time(torch, engine, atoms, prec, flags, steps, warmup):
    """The C-ABI call a user makes, with host buffers: every step copies the
    positions in from pinned host memory and the energy, forces and virial out."""
    from pysic_gb300 import _lib as L

    n = len(atoms)
    pos = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    pos[:] = atoms.get_positions()
    e = torch.empty(1, dtype=torch.float64, pin_memory=True).numpy()
    f = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    s = torch.empty(6, dtype=torch.float64, pin_memory=True).numpy()
    c = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    for _ in range(warmup):
        engine.update_positions(pos)
        engine.calculate_into(prec, flags, e, f, s, c)
    t0 = time.perf_counter()
    for _ in range(steps):
        engine.update_positions(pos)
        engine.calculate_into(prec, flags, e, f, s, c)
    dt = time.perf_counter() - t0
    h2d = pos.nbytes
    d2h = e.nbytes + f.nbytes + s.nbytes
    del L
    return dt, h2d, d2h


def cpu_baseline(name, seconds, threads):
    """The oracle (FP64 CPU restatement of the reference loops) on a bounded
    sample: whole energy + force evaluations of the same structure."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from pysic_gb300.model import compile_model, individual_cutoffs

    atoms, pots, coul, _ = workload(name)
    model = compile_model(atoms, pots, coul)
    cuts = np.array(individual_cutoffs(atoms, pots, coul)) + 0.5
    lists = oracle.neighbors(atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(), cuts)
    args = (atoms.get_positions(), atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc(), model) + tuple(lists)
    evals = 0
    t0 = time.perf_counter()
    while True:
        e = oracle.evaluate(*args, what="energy", threads=threads)
        f, st = oracle.evaluate(*args, what="forces", threads=threads)
        evals += 1
        dt = time.perf_counter() - t0
        if dt >= seconds:
            break
    return len(atoms) * evals / dt, evals, dt, len(atoms), {"energy": e, "forces": f, "stress": st}


def accuracy(r, ref, n):
    """Errors of an engine result against a reference result (energy per atom,
    largest force component, virial relative to its largest component)."""
    return {"energy_err_eV_per_atom": abs(r["energy"] - ref["energy"]) / n,
            "max_force_err_eV_per_A": float(np.abs(r["forces"] - ref["forces"]).max()),
            "virial_rel_err": float(np.abs(r["stress"] - ref["stress"]).max() /
                                    max(1e-30, np.abs(ref["stress"]).max()))}


def common_config(name, atoms_n, desc, precision, implementation):
    """The config object both arms print (the same keys and values apart from
    precision and implementation), so that their lines can be matched."""
    return {"workload": name, "atoms": atoms_n, "structure": desc,
            "neighbor_list": "built once before timing (fixed positions)",
            "l2": "GPU arm: flushed before every step (256 MB write); CPU arm: not applicable",
            "precision": precision, "implementation": implementation}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        if rank != 0:
            dist.barrier()
            dist.destroy_process_group()
            return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from pysic_gb300.model import compile_model, individual_cutoffs

    threads = os.cpu_count() or 1
    atoms, pots, coul, desc = workload(args.workload)
    model = compile_model(atoms, pots, coul)
    cuts = np.array(individual_cutoffs(atoms, pots, coul)) + 0.5
    lists = oracle.neighbors(atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(), cuts)
    a = (atoms.get_positions(), atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc(), model) + tuple(lists)
    for _ in range(args.warmup):
        oracle.evaluate(*a, what="energy", threads=threads)
        oracle.evaluate(*a, what="forces", threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.evaluate(*a, what="energy", threads=threads)
        oracle.evaluate(*a, what="forces", threads=threads)
    dt = time.perf_counter() - t0
    value = len(atoms) * args.steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": common_config(args.workload, len(atoms), desc, "fp64",
                                    "C restatement of the Fortran core loops (oracle/oracle.c), energy pass + "
                                    "force pass per step, as the reference does"),
            "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                             "sample": "{0} full energy+force evaluations of {1} atoms".format(args.steps,
                                                                                                len(atoms)),
                             "mpi_ranks": 0},
            "e2e": {"value": value, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    sys.stdout.flush()
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()


RELAX_REPEATS = 3


def md_throughput(name, precision, device, steps):
    """Velocity Verlet of the benchmark structure at 1000 K (dt 1 fs): the
    device loop (pysic_gb300.VelocityVerlet, neighbour rebuilds included)
    against ASE's update driven from the host around Pysic.get_forces, the way
    the reference runs MD.  Wall-clock atom-steps/s of each."""
    import pysic_gb300 as pysic

    fs = 0.09822694788464063
    atoms, pots, coul, _ = workload(name)
    kT = 8.617333262e-5 * 1000.0
    m = atoms.get_masses()[:, None]
    p0 = np.random.default_rng(1).normal(0.0, 1.0, (len(atoms), 3)) * np.sqrt(m * kT)
    p0 -= p0.mean(axis=0)

    def fresh():
        a = atoms.copy()
        a.set_momenta(p0)
        a.set_calculator(pysic.Pysic(a, pots, coulomb=coul, precision=precision))
        return a

    a = fresh()
    dyn = pysic.VelocityVerlet(a, fs)
    dyn.run(5)  # warm-up: lists, tables, graphs
    t0 = time.perf_counter()
    dyn.run(steps)
    t_dev = time.perf_counter() - t0
    rebuilds = a.get_calculator().get_neighbor_lists().nupdates
    b = fresh()
    f = b.get_forces()
    host_steps = max(5, steps // 10)
    t0 = time.perf_counter()
    for _ in range(host_steps):
        p = b.get_momenta()
        p += 0.5 * fs * f
        b.set_positions(b.get_positions() + fs * p / m)
        b.set_momenta(p)
        f = b.get_forces()
        b.set_momenta(b.get_momenta() + 0.5 * fs * f)
    t_host = time.perf_counter() - t0
    n = len(atoms)
    return {"steps": steps, "temperature_K": 1000.0, "timestep_fs": 1.0, "precision": precision,
            "device_atom_steps_per_s": n * steps / t_dev, "device_us_per_step": 1e6 * t_dev / steps,
            "list_builds": rebuilds,
            "host_driven_atom_steps_per_s": n * host_steps / t_host, "host_driven_us_per_step": 1e6 * t_host / host_steps,
            "note": "wall clock; the host-driven loop is ASE's VelocityVerlet update around Pysic.get_forces"}


def relax_cpu_baseline(threads):
    """The reference's 'dynamic' loop (relaxation.py:417-450) as the oracle
    restates it, FP64 on the host cores, on the first held-out SiO2 box from
    zero charges to the same tolerance: steps and wall time."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from pysic_gb300 import workloads as W
    from pysic_gb300.model import compile_model, individual_cutoffs
    from pysic_gb300.train_warm_start import RELAX

    atoms = W.sio2_box(1000, seed=0)
    pots, coul = W.sio2_potentials()
    model = compile_model(atoms, pots, coul)
    cuts = np.array(individual_cutoffs(atoms, pots, coul)) + 0.5
    lists = oracle.neighbors(atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(), cuts)
    t0 = time.perf_counter()
    r = oracle.relax_charges(atoms.get_positions(), np.zeros(len(atoms)), atoms.get_cell(), atoms.get_pbc(), model,
                             *lists, threads=threads, **RELAX)
    dt = time.perf_counter() - t0
    return {"steps": r["steps"], "wall_ms": 1e3 * dt, "cores": threads, "kind": "port", "precision": "fp64",
            "sample": "one 3000-atom box (seed 0), 'dynamic' relaxation from zero charges to the same tolerance "
                      "(oracle: the reference's loop restated, every step a full electronegativity evaluation)",
            "mpi_ranks": 0}


def charge_relax_gain(n_configs, device, cpu_threads=0):
    """The metric's second part: plain 'dynamic' charge relaxation of SiO2
    boxes (1000 Si + 2000 O, seeds 0.. held out from training) from zero
    charges against the same relaxation started from the trained network's
    charges; steps and wall time (prediction included) to the same tolerance."""
    import pysic_gb300 as pysic
    from pysic_gb300 import workloads as W
    from pysic_gb300.mlp import ChargeNetwork
    from pysic_gb300.train_warm_start import RELAX, relax

    path = os.path.join(ROOT, "pysic_gb300", "data", "sio2_warm_start.npz")
    if not os.path.exists(path):
        return {"unavailable": "no trained network at pysic_gb300/data/sio2_warm_start.npz"}
    net = ChargeNetwork.load(path, device=device)
    pots, coul = W.sio2_potentials()
    cold_s, warm_s, cold_t, warm_t, rmse, dq = [], [], [], [], [], []
    opt_t, opt_it, opt_dq = [], [], []
    for seed in range(n_configs):
        atoms = W.sio2_box(1000, seed=seed)
        calc = pysic.Pysic(atoms, pots, coulomb=coul, precision="mixed")
        calc.set_core()
        relax(calc)  # warm-up: kernels, graphs, buffers
        relax(calc, network=net)
        tc, tw = [], []
        for _ in range(RELAX_REPEATS):  # wall times: the median of a few repeats
            t0 = time.perf_counter()
            q_cold, rc = relax(calc)
            tc.append(time.perf_counter() - t0)
            t0 = time.perf_counter()
            q_warm, rw = relax(calc, network=net)
            tw.append(time.perf_counter() - t0)
        cold_t.append(float(np.median(tc)))
        warm_t.append(float(np.median(tw)))
        # the same minimum by 'optimize' (conjugate gradients on the device), from zero charges
        opt = pysic.ChargeRelaxation("optimize", calculator=calc, parameters=[RELAX["n_steps"], RELAX["tolerance"]])
        to = []
        for _ in range(RELAX_REPEATS):
            calc.get_atoms().set_initial_charges(np.zeros(len(atoms)))
            t0 = time.perf_counter()
            q_opt = opt.charge_relaxation()
            to.append(time.perf_counter() - t0)
        opt_t.append(float(np.median(to)))
        opt_it.append(opt.last_steps)
        opt_dq.append(float(np.abs(q_opt - q_cold).max()))
        if not (rc.last_converged and rw.last_converged):
            return {"unavailable": "relaxation did not converge for seed {0}".format(seed)}
        cold_s.append(rc.last_steps)
        warm_s.append(rw.last_steps)
        calc.get_atoms().set_initial_charges(np.zeros(len(atoms)))
        rmse.append(float(np.sqrt(np.mean((net.predict_charges(calc) - q_cold) ** 2))))
        dq.append(float(np.abs(q_warm - q_cold).max()))
    # steps against the starting error: the converged charges of box 0 plus
    # seeded Gaussian noise (sum kept at zero), relaxed again to the same tolerance
    calc = pysic.Pysic(W.sio2_box(1000, seed=0), pots, coulomb=coul, precision="mixed")
    calc.set_core()
    q_exact, rc0 = relax(calc)
    curve = []
    for sigma in (0.1, 0.05, 0.02, 0.01, 0.005, 0.002, 0.001, 0.0005, 0.0002, 0.0001):
        st = []
        for rep in range(2):
            dq = np.random.default_rng(1000 + rep).normal(0.0, sigma, len(q_exact))
            q0 = q_exact + dq - dq.mean()
            calc.get_atoms().set_initial_charges(q0)
            rel = pysic.ChargeRelaxation("dynamic", calculator=calc,
                                         parameters=[RELAX[k] for k in ("n_steps", "timestep", "inertia", "friction",
                                                                        "tolerance")])
            rel.charge_relaxation()
            st.append(rel.last_steps)
        curve.append({"start_rmse_e": sigma, "steps": float(np.mean(st)),
                      "step_gain": rc0.last_steps / float(np.mean(st))})
    # the starting error at which the step gain reaches 3 (log-linear between the measured points)
    need = None
    for a, b in zip(curve, curve[1:]):
        if a["step_gain"] < 3.0 <= b["step_gain"]:
            t = (3.0 - a["step_gain"]) / (b["step_gain"] - a["step_gain"])
            need = float(np.exp(np.log(a["start_rmse_e"]) + t * (np.log(b["start_rmse_e"]) - np.log(a["start_rmse_e"]))))
            break
    gain_curve = {"box": "seed 0", "cold_steps": rc0.last_steps, "points": curve,
                  "start_rmse_for_3x_step_gain_e": need,
                  "network_rmse_e": float(np.mean(rmse)),
                  "note": "white noise on the converged charges; the damped dynamics converge linearly at the rate "
                          "of the softest charge mode, so steps grow with log(start error / tolerance)"}
    cpu = relax_cpu_baseline(cpu_threads) if cpu_threads > 0 else None
    if cpu is not None:
        cpu["gpu_cold_ms_same_box"] = 1e3 * cold_t[0]
        cpu["gpu_cold_steps_same_box"] = cold_s[0]
    return {"configs": n_configs, "atoms": 3000, "settings": RELAX, "precision": "mixed",
            "cpu_baseline": cpu, "gain_vs_start_error": gain_curve,
            "cold_steps_mean": float(np.mean(cold_s)), "warm_steps_mean": float(np.mean(warm_s)),
            "cold_ms_mean": 1e3 * float(np.mean(cold_t)), "warm_ms_mean": 1e3 * float(np.mean(warm_t)),
            "wall_time_gain": float(np.sum(cold_t) / np.sum(warm_t)),
            "step_gain": float(np.sum(cold_s) / np.sum(warm_s)),
            "prediction_rmse_e": float(np.mean(rmse)), "max_charge_difference_e": float(np.max(dq)),
            "repeats": RELAX_REPEATS,
            "optimize": {"iterations_mean": float(np.mean(opt_it)), "ms_mean": 1e3 * float(np.mean(opt_t)),
                         "max_charge_difference_e": float(np.max(opt_dq)),
                         "note": "'optimize' mode: projected conjugate gradients on the device to the same "
                                 "tolerance on max |chi - mean(chi)|, from zero charges"},
            "note": "the warm relaxation runs to the same tolerance; its wall time includes descriptors "
                    "and the network's prediction (on the device); wall times are medians of the repeats"}


def run_ours(args):
    import torch

    world, rank, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from pysic_gb300 import _lib as L

    prec = L.PREC_MIXED if args.precision == "mixed" else L.PREC_FP64
    flags = L.WANT_ENERGY | L.WANT_FORCES
    atoms, calc, desc = setup(args.workload, args.precision, local)
    engine = calc.engine
    n = len(atoms)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda:%d" % local)  # 256 MB > L2

    # warm-up (includes the lane-count autotuner and the graph capture)
    engine.calculate(prec)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    t_wall0 = time.perf_counter()
    times, launches = device_time(torch, engine, prec, flags, args.steps, args.warmup, flush)
    t_wall = time.perf_counter() - t_wall0
    clocks = sampler.stop()
    total_ms = sum(times)
    if dist is not None:
        t = torch.tensor([total_ms], dtype=torch.float64, device="cuda:%d" % local)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * n * args.steps / (total_ms / 1e3)

    extra = {}
    # the FP64 kernels on the same workload (the metric's denominator)
    prec64 = L.PREC_FP64
    engine.calculate(prec64)
    t64, _ = device_time(torch, engine, prec64, flags, max(10, args.steps // 4), args.warmup, flush)
    v64 = n * len(t64) / (sum(t64) / 1e3)
    r_mixed = engine.calculate(prec)
    r_64 = engine.calculate(prec64)
    extra["fp64"] = {"value": v64, "unit": "atom-steps/s", "ms_per_step": statistics.mean(t64)}
    extra["speedup_vs_fp64"] = value / world / v64
    extra["accuracy_vs_fp64"] = {
        "energy_err_eV_per_atom": abs(r_mixed["energy"] - r_64["energy"]) / n,
        "max_force_err_eV_per_A": float(np.abs(r_mixed["forces"] - r_64["forces"]).max()),
        "virial_rel_err": float(np.abs(r_mixed["stress"] - r_64["stress"]).max() /
                                max(1e-30, np.abs(r_64["stress"]).max()))}

    # kernel-level times and the roofline of the dominant kernel
    kt = kernel_time(torch, engine, prec, flags, min(50, args.steps), flush)
    dominant = max(kt, key=kt.get)
    peak, peak_kind = peaks()
    if args.workload.startswith("tersoff"):
        alg_bytes = TERSOFF_BYTES_PER_ATOM * n
        alg_flop = TERSOFF_FLOP_PER_ATOM * n
        kname = "bond_pass"
    else:
        alg_bytes = 48.0 * n
        alg_flop = None
        kname = dominant
    t_k = kt.get(kname, kt[dominant]) / 1e3
    achieved = alg_bytes / t_k / 1e9
    traffic = profile_traffic(kname, args.workload)
    hbm = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
           "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind}
    if alg_flop:
        # the bond-order pass is bound by FP32 issue and dependency latency (its
        # working set stays in L2): its roofline is the FP32 rate measured now
        p32 = fp32_peak(local)
        a32 = alg_flop / t_k / 1e12
        roof = {"bound": "fp32", "kernel": kname, "achieved": a32, "peak": p32, "unit": "TFLOP/s",
                "frac": a32 / p32, "traffic": traffic,
                "peak_source": "measured in this run: independent FMA chains on every SM (pg_measure_fp32_peak)",
                "algorithmic": "{0:.0f} FLOP/atom x {1} atoms per launch".format(TERSOFF_FLOP_PER_ATOM, n),
                "hbm": hbm}
    else:
        roof = hbm
    extra["kernel_ms"] = kt

    # end to end through the C ABI with host buffers
    e2e_dt, h2d, d2h = e2e_time(torch, engine, atoms, prec, flags, args.steps, args.warmup)
    if world == 1 and args.workload.startswith("tersoff_si_32768") and args.relax_configs > 0:
        extra["charge_relax"] = charge_relax_gain(args.relax_configs, local,
                                                  0 if args.no_cpu_baseline else (os.cpu_count() or 1))
    if world == 1 and args.workload.startswith("tersoff_si") and args.md_steps > 0:
        extra["md"] = md_throughput(args.workload, args.precision, local, args.md_steps)
    if world == 1 and args.workload.startswith("tersoff_si_32768") and not args.no_other_configs:
        extra["other_configs"] = other_configs(local, min(args.steps, 50), args.warmup, os.cpu_count() or 1)
        extra["batched"] = batch_measure(args.precision, min(args.steps, 20), args.warmup)
    e2e = {"value": n * args.steps / e2e_dt, "unit": "atom-steps/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e2e_dt / args.steps}

    cpu = None
    if world == 1 and rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, evals, dt, natoms, ref = cpu_baseline(args.workload, args.cpu_seconds, threads)
        cpu = {"value": v, "unit": "atom-steps/s", "cores": threads, "kind": "port",
               "sample": "{0} full energy+force evaluations of {1} atoms in {2:.1f} s (oracle, FP64)".format(
                   evals, natoms, dt), "mpi_ranks": 0}
        # the engine against the CPU restatement of the reference path on the same structure
        extra["accuracy_vs_oracle"] = {"mixed": accuracy(r_mixed, ref, n), "fp64": accuracy(r_64, ref, n),
                                       "note": "engine results against the FP64 oracle (the reference's loops "
                                               "restated in C) evaluated in the cpu_baseline sample"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32" if prec == L.PREC_MIXED else "f64",
                "data": "synthetic",
                "config": common_config(args.workload, n, desc,
                                        args.precision + (" (FP32 per pair/triplet, exact fixed-point accumulation)"
                                                          if prec == L.PREC_MIXED else ""),
                                        "sm_103a CUDA kernels through the C ABI (pysic_gb300)"),
                "tiles": {"lanes_per_atom": engine.get_lanes()}, "replicas": world,
                "e2e": e2e, "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu, "clocks": clocks,
                "wall_s_timed_region": t_wall}
        line.update(extra)
        print(json.dumps(line))
        sys.stdout.flush()
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def _batched_structure(k):
    import math

    from pysic_gb300 import workloads as W

    rng = np.random.default_rng(0)
    counts = np.floor(np.exp(rng.uniform(math.log(64), math.log(2048), 512))).astype(int)
    a = W.random_box(["Si"] * int(counts[k]), W.SI_DENSITY, 2.0, k)
    return a.get_positions(), a.get_cell()[0, 0]


def _build_batch(precision, systems=512):
    """The first `systems` of the 512 systems of the many-system workload, set
    up and batched (structures made in worker processes for the full set)."""
    if systems >= 512:
        import multiprocessing as mp

        with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
            structs = pool.map(_batched_structure, range(512), chunksize=8)
    else:
        structs = [_batched_structure(k) for k in range(systems)]
    import pysic_gb300 as pysic
    from pysic_gb300 import workloads as W
    from pysic_gb300.batch import BatchedPysic

    pots = W.batched_potentials()
    calcs = []
    for pos, L_ in structs:
        atoms = pysic.Atoms(["Si"] * len(pos), pos, cell=np.eye(3) * L_, pbc=True)
        c = pysic.Pysic(atoms, pots, precision=precision)
        c.set_core()
        calcs.append(c)
    return BatchedPysic(calcs), sum(len(p) for p, _ in structs)


def batch_measure(precision, steps, warmup):
    """512 uneven silicon boxes (Tersoff + LJ): one persistent launch for all
    systems (graph replay) against one launch per phase and one evaluation per
    system.  Device-timed
    ms per evaluation of all systems (L2 flushed before each), wall-clock
    comparison with per-system evaluation, and the FP64 kernels."""
    batch, n_atoms = _build_batch(precision)
    import torch

    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    stream = torch.cuda.ExternalStream(batch.stream_handle())

    def timed(prec, k_steps, mode="batched"):
        for _ in range(warmup):
            batch.evaluate(prec, mode=mode)
        batch.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k_steps)]
        for k in range(k_steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(k))
                ev[k][0].record(stream)
            batch.evaluate(prec, mode=mode)
            with torch.cuda.stream(stream):
                ev[k][1].record(stream)
        batch.synchronize()
        return [a.elapsed_time(b) for a, b in ev]

    sampler = ClockSampler(0)
    sampler.start()
    times = timed(precision, steps)
    clocks = sampler.stop()
    launches = batch.launch_count()
    ms = statistics.mean(times)

    def wall(mode):
        for _ in range(warmup):
            batch.evaluate(precision, mode=mode)
        batch.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            batch.evaluate(precision, mode=mode)
        batch.synchronize()
        return (time.perf_counter() - t0) / steps

    wall_each = wall("each")
    launches_each = batch.launch_count()
    wall_batched = wall("batched")
    t_phases = timed(precision, steps, "phases")
    launches_phases = batch.launch_count()
    t64 = timed("fp64", max(5, steps // 4))
    pl, bl, cells = batch.get_tiles(precision)
    ppl, pbl, _ = batch.get_tiles(precision, "phases")
    out = {"systems": 512, "atoms": n_atoms, "precision": precision, "ms_per_step": ms,
           "atom_steps_per_s": n_atoms / (ms / 1e3), "systems_per_s": 512 / (ms / 1e3),
           "launches_per_step": launches, "batched_wall_ms_per_step": 1e3 * wall_batched,
           "per_system": {"wall_ms_per_step": 1e3 * wall_each, "atom_steps_per_s": n_atoms / wall_each,
                          "launches_per_step": launches_each,
                          "note": "every system evaluated on its own: its own captured graph on its own stream"},
           "batched_vs_per_system_wall": wall_each / wall_batched,
           "fp64": {"atom_steps_per_s": n_atoms / (statistics.mean(t64) / 1e3), "ms_per_step": statistics.mean(t64)},
           "phase_launches": {"ms_per_step": statistics.mean(t_phases), "launches_per_step": launches_phases,
                              "tiles": {"pair_lanes": ppl, "bond_lanes": pbl},
                              "note": "the same tiles with one launch per phase (displacement, pair, bond, gather)"},
           "tiles": {"pair_lanes": pl, "bond_lanes": bl, "cells_per_tile": cells,
                     "note": "one persistent launch; chosen by the batch's autotuner over pair lanes {8, 16} x bond "
                             "lanes {4, 8, triplet tile} x cells per tile {1, 2, 4}"},
           "clocks": clocks,
           "structure": "Si boxes, atom counts log-uniform in [64, 2048], 2.33 g/cm^3, random with rejection below "
                        "2.0 A; Tersoff + LJ (0.01 eV, 2.1 A, cutoff 5)",
           "l2": "flushed before every step (256 MB write)"}
    out["speedup_vs_fp64"] = out["atom_steps_per_s"] / out["fp64"]["atom_steps_per_s"]
    return out


def run_batch(args):
    """The many-system workload as the line's own metric."""
    b = batch_measure(args.precision, args.steps, args.warmup)
    line = {"metric": METRIC, "value": b["atom_steps_per_s"], "unit": "atom-steps/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": b["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision == "mixed" else "f64",
            "data": "synthetic",
            "config": {"workload": "batched_si_512", "systems": 512, "atoms": b["atoms"],
                       "structure": b["structure"], "precision": args.precision, "l2": b["l2"]},
            "gpu_launches": b["launches_per_step"] * args.steps, "clocks": b["clocks"], "batched": b}
    print(json.dumps(line))


def other_configs(device, steps, warmup, threads):
    """The other single-system benchmark configurations, device-timed the same
    way (L2 flushed before every step), each against the oracle on the same
    structure: LJ fcc 864 atoms in FP64 (config 1), rock-salt NaCl 8000
    ions with Buckingham + Ewald (config 3) and the COMB compound on a
    3000-atom SiO2 box, in mixed precision and FP64."""
    import torch

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from pysic_gb300 import _lib as L
    from pysic_gb300.model import compile_model, individual_cutoffs

    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda:%d" % device)
    out = {}
    for name, precisions in (("lj_fcc_864", ("fp64",)), ("ewald_nacl_8000", ("mixed", "fp64")),
                             ("comb_sio2_3000", ("mixed", "fp64"))):
        atoms, pots, coul, desc = workload(name)
        model = compile_model(atoms, pots, coul)
        cuts = np.array(individual_cutoffs(atoms, pots, coul)) + 0.5
        lists = oracle.neighbors(atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(), cuts)
        a = (atoms.get_positions(), atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc(), model) + \
            tuple(lists)
        t0 = time.perf_counter()
        ref = {"energy": oracle.evaluate(*a, what="energy", threads=threads)}
        ref["forces"], ref["stress"] = oracle.evaluate(*a, what="forces", threads=threads)
        t_cpu = time.perf_counter() - t0
        n = len(atoms)
        block = {"atoms": n, "structure": desc,
                 "cpu_baseline": {"atom_steps_per_s": n / t_cpu, "cores": threads, "kind": "port",
                                  "sample": "one energy + force evaluation (oracle, FP64)"}}
        for prec_name in precisions:
            _, calc, _ = setup(name, prec_name, device)
            eng = calc.engine
            prec = L.PREC_MIXED if prec_name == "mixed" else L.PREC_FP64
            r = eng.calculate(prec)
            t, _ = device_time(torch, eng, prec, L.WANT_ENERGY | L.WANT_FORCES, steps, warmup, flush)
            ms = statistics.mean(t)
            block[prec_name] = {"ms_per_step": ms, "atom_steps_per_s": n / (ms / 1e3),
                                "accuracy_vs_oracle": accuracy(r, ref, n)}
        if "mixed" in block:
            block["speedup_vs_fp64"] = block["mixed"]["atom_steps_per_s"] / block["fp64"]["atom_steps_per_s"]
        out[name] = block
    return out


def run_profile(args):
    """Short fixed sequence for ncu: build, then `--steps` evaluations with a
    fixed lanes-per-atom tile (no autotuner launches)."""
    from pysic_gb300 import _lib as L

    prec = L.PREC_MIXED if args.precision == "mixed" else L.PREC_FP64
    if args.workload == "relax_sio2_3000":
        # plain 'dynamic' relaxations of the first held-out SiO2 box (3000 atoms) from zero charges
        import pysic_gb300 as pysic
        from pysic_gb300 import workloads as W
        from pysic_gb300.train_warm_start import relax

        pots, coul = W.sio2_potentials()
        calc = pysic.Pysic(W.sio2_box(1000, seed=0), pots, coulomb=coul, precision=args.precision)
        calc.set_core()
        steps = []
        for _ in range(max(1, args.steps)):
            _, rel = relax(calc)
            steps.append(rel.last_steps)
        print(json.dumps({"profile_run": args.workload, "precision": args.precision, "relax_steps": steps}))
        return
    if args.workload == "batched_si_512":
        # the batched launches only: set-up, then `--steps` evaluations of all 512 systems
        batch, n_atoms = _build_batch(args.precision, args.systems)
        if args.bond_lanes:  # fixed tiles: no autotuner launches
            batch.set_lanes(args.lanes, args.bond_lanes)
            batch.set_tile_blocks(args.cells)
        for _ in range(args.steps):
            batch.evaluate(args.precision, mode=args.batch_mode)
        batch.synchronize()
        print(json.dumps({"profile_run": args.workload, "precision": args.precision, "systems": args.systems,
                          "atoms": n_atoms, "mode": args.batch_mode, "tiles": batch.get_tiles(args.precision,
                                                                                             args.batch_mode)}))
        return
    atoms, calc, _ = setup(args.workload, args.precision, 0)
    eng = calc.engine
    eng.set_lanes(args.lanes)
    for _ in range(args.steps):
        eng.device_evaluate(prec, L.WANT_ENERGY | L.WANT_FORCES)
    eng.device_synchronize()
    r = eng.calculate(prec)
    print(json.dumps({"profile_run": args.workload, "precision": args.precision, "lanes": args.lanes,
                      "energy_per_atom": r["energy"] / len(atoms)}))


def main():
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("--profile", action="store_true", help="short fixed run for ncu captures")
    p.add_argument("--lanes", type=int, default=8, help="lanes per atom in --profile mode")
    p.add_argument("--systems", type=int, default=512, help="systems of the many-system workload in --profile mode")
    p.add_argument("--bond-lanes", type=int, default=0,
                   help="--profile of the many-system workload: bond lanes (with --lanes as pair lanes; 0: autotune)")
    p.add_argument("--cells", type=int, default=1, help="--profile of the many-system workload: cells per tile")
    p.add_argument("--batch-mode", default="batched", choices=("batched", "phases"),
                   help="--profile of the many-system workload: one persistent launch or one launch per phase")
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", default="tersoff_si_32768")
    p.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-other-configs", action="store_true",
                   help="skip the LJ 864, NaCl 8000 and 512-system blocks of the default line")
    p.add_argument("--relax-configs", type=int, default=3, help="SiO2 boxes for the charge-relax gain (0: skip)")
    p.add_argument("--md-steps", type=int, default=300, help="device velocity Verlet steps reported beside the metric "
                                                              "(0: skip)")
    args = p.parse_args()
    args.warmup = max(3, args.warmup)
    if args.profile:
        run_profile(args)
    elif args.workload == "batched_si_512" and args.impl != "reference":
        run_batch(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

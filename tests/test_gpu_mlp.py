"""GPU checks of the learned warm start (csrc/mlp.cu) against the FP64 NumPy
oracle (oracle/mlp_oracle.py).

Tolerances: the engine reads BF16 weights, rounds inputs and first-layer
activations to BF16 and sums in FP32; the oracle does the same in FP64, so
forward values agree to ~1e-6 relative except where a first-layer activation
falls on the other side of a BF16 rounding boundary (one BF16 step, rare), and
gradients (sums over the batch) to 1e-4 relative to the largest component.
Descriptors: FP32 against FP64, 1e-5 relative.
"""
import os
import sys

import numpy as np
import pytest

import mlp_oracle as MO
import pysic_gb300 as pysic
from pysic_gb300 import workloads as W
from pysic_gb300.mlp import ChargeNetwork

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _net(n_in=10, h1=12, h2=8, seed=0):
    net = ChargeNetwork(n_in, h1, h2)
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.4, net.n_params).astype(np.float32)
    net.set_params(p)
    return net, MO.bf16(p)


@pytest.mark.parametrize("sizes", [(10, 12, 8), (40, 33, 50), (64, 128, 128)])
def test_forward_matches_oracle(sizes):
    n_in, h1, h2 = sizes
    net, pb = _net(n_in, h1, h2)
    rng = np.random.default_rng(1)
    x = rng.normal(0, 1, (2001, n_in)).astype(np.float32)
    got = net.predict(x)  # identity normalisation
    ref, _, _ = MO.forward(pb, x, n_in, h1, h2)
    # the first-layer activations are rounded to BF16: where FP32 tanh (device)
    # and FP64 tanh (oracle) fall on either side of a rounding boundary, one
    # activation differs by one BF16 step (2^-8 relative); everything else agrees
    close = np.abs(got - ref) <= 1e-5 + 1e-5 * np.abs(ref)
    assert close.mean() >= 0.99
    assert np.abs(got - ref).max() <= 1e-2 * max(1.0, np.abs(ref).max())


def test_device_warm_start_matches_host_path():
    """pg_mlp_predict_charges (descriptors, fold, normalisation, network and
    total-charge shift on the device) against the host route with the
    shipped SiO2 network."""
    net = ChargeNetwork.load(os.path.join(os.path.dirname(pysic.__file__), "data", "sio2_warm_start.npz"))
    pots, coul = W.sio2_potentials(real_cutoff=5.5, sigma=1.6)
    for seed, total in ((31, 0.0), (32, 0.3)):
        calc = pysic.Pysic(W.sio2_box(60, seed=seed), pots, coulomb=coul, precision="mixed")
        calc.set_core()
        host = net.predict_charges_host(calc, total_charge=total)
        dev = net.predict_charges(calc, total_charge=total)
        np.testing.assert_allclose(dev, host, rtol=0, atol=1e-12)
        assert dev.sum() == pytest.approx(total, abs=1e-12)
        # the engine holds the predicted charges
        np.testing.assert_array_equal(calc.engine.get_charges(), dev)


def test_gradients_match_oracle():
    net, pb = _net(seed=2)
    rng = np.random.default_rng(3)
    x = rng.normal(0, 1, (300, 10)).astype(np.float32)
    y = rng.normal(0, 1, 300).astype(np.float32)
    loss, g = net.gradients(x, y)
    ref_loss, ref_g = MO.loss_and_grad(pb, x, y, 10, 12, 8)
    assert loss == pytest.approx(ref_loss, rel=1e-5)
    assert np.abs(g - ref_g).max() <= 1e-4 * np.abs(ref_g).max()


@pytest.mark.parametrize("n_in", [34, 35, 64])
def test_tensor_core_gradients_match_oracle(n_in):
    """Networks of two 64-unit layers train on the tensor cores (BF16 products,
    FP32 sums): against the oracle with the same BF16 layer errors to 1e-4 of
    the largest component, against the oracle without them to 2e-2."""
    net, pb = _net(n_in, 64, 64, seed=6)
    rng = np.random.default_rng(7)
    x = rng.normal(0, 1, (1000, n_in)).astype(np.float32)  # 15 full tiles of 64 samples and a ragged one
    y = rng.normal(0, 1, 1000).astype(np.float32)
    loss, g = net.gradients(x, y)
    ref_loss, ref_g = MO.loss_and_grad(pb, x, y, n_in, 64, 64, tensor_core=True)
    assert loss == pytest.approx(ref_loss, rel=1e-5)
    assert np.abs(g - ref_g).max() <= 1e-4 * np.abs(ref_g).max()
    _, plain = MO.loss_and_grad(pb, x, y, n_in, 64, 64)
    assert np.abs(g - plain).max() <= 2e-2 * np.abs(plain).max()
    loss2, g2 = net.gradients(x, y)  # deterministic
    assert loss2 == loss and np.array_equal(g2, g)


def test_tensor_core_training_reduces_loss_and_is_deterministic():
    rng = np.random.default_rng(8)
    x = rng.normal(0, 1, (20000, 34)).astype(np.float32)
    w = rng.normal(0, 1, 34)
    y = np.tanh(x @ w / 6.0).astype(np.float32)
    runs = []
    for _ in range(2):
        net, _ = _net(34, 64, 64, seed=9)
        net.add_samples(x, y)
        losses = net.train(6, batch=1024, learning_rate=2e-3, seed=13)
        runs.append((losses, net.get_params()))
    assert runs[0][0][-1] < 0.3 * runs[0][0][0]
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])


@pytest.mark.parametrize("n_gauss", [8, 16])
def test_descriptors_match_oracle(n_gauss):
    sys.path.insert(0, GOLDEN)
    import cases

    g = np.load(os.path.join(GOLDEN, "oracle_cases.npz"))
    atoms, pots, coul = cases.restore("sio2_120", g)
    calc = pysic.Pysic(atoms, pots, coulomb=coul)
    calc.set_core()
    c, i, o = calc.engine.neighbor_lists()
    d = dict(n_gauss=n_gauss, r0=0.8, r1=5.0, width=0.35, cutoff=5.0)
    got = calc.engine.descriptors(calc._model.n_types, **d)
    ref = MO.descriptors(atoms.get_positions(), atoms.get_cell(), calc._model.types, calc._model.n_types,
                         c, i, o, **d)
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())


def test_training_reduces_loss_and_is_deterministic():
    rng = np.random.default_rng(4)
    x = rng.normal(0, 1, (6000, 10)).astype(np.float32)
    w = rng.normal(0, 1, 10)
    y = np.tanh(x @ w / 3.0).astype(np.float32)
    runs = []
    for _ in range(2):
        net, _ = _net(seed=5)
        net.add_samples(x, y)
        losses = net.train(8, batch=512, learning_rate=3e-3, seed=11)
        runs.append((losses, net.get_params()))
    losses, p = runs[0]
    assert losses[-1] < 0.25 * losses[0]
    assert np.array_equal(p, runs[1][1])


def test_shipped_network_cuts_relaxation_steps_on_a_held_out_box():
    """The shipped SiO2 network (trained on boxes of seeds 100000 and up) on a
    held-out 3000-atom box with the benchmark's relaxation settings: strictly
    fewer damped-dynamics steps to the same tolerance, the same charges."""
    from pysic_gb300.train_warm_start import RELAX, relax

    net = ChargeNetwork.load(os.path.join(os.path.dirname(pysic.__file__), "data", "sio2_warm_start.npz"))
    pots, coul = W.sio2_potentials()
    calc = pysic.Pysic(W.sio2_box(1000, seed=1), pots, coulomb=coul, precision="mixed")
    q_cold, cold = relax(calc, RELAX)
    q_warm, warm = relax(calc, RELAX, network=net)
    assert cold.last_converged and warm.last_converged
    print("held-out box: cold %d steps, warm %d steps, prediction RMSE %.4f e" % (
        cold.last_steps, warm.last_steps,
        float(np.sqrt(np.mean((net.predict_charges(calc) - q_cold) ** 2)))))
    assert warm.last_steps < cold.last_steps
    np.testing.assert_allclose(q_warm, q_cold, atol=2e-4)


def test_warm_start_relaxation_reaches_the_same_charges():
    from pysic_gb300.train_warm_start import relax

    params = {"n_steps": 4000, "timestep": 0.1, "inertia": 1.0, "friction": 4.0, "tolerance": 1e-4}
    pots, coul = W.sio2_potentials(real_cutoff=5.5, sigma=1.6)
    net = ChargeNetwork(2 * 16 + 2, 32, 32, elements=["Si", "O"])
    xs, ys = [], []
    calc = None
    for seed in range(200, 216):  # training boxes
        atoms = W.sio2_box(40, seed=seed)
        calc = pysic.Pysic(atoms, pots, coulomb=coul, precision="mixed")
        q, rel = relax(calc, params)
        assert rel.last_converged
        xs.append(net.descriptors(calc))
        ys.append(q)
    x, y = np.concatenate(xs), np.concatenate(ys)
    net.normalise_from(x, y)
    net.add_samples(x, y)
    net.train(60, batch=256, learning_rate=3e-3, seed=1)
    test_atoms = W.sio2_box(40, seed=7)  # held out
    calc = pysic.Pysic(test_atoms, pots, coulomb=coul, precision="mixed")
    q_cold, cold = relax(calc, params)
    q_warm, warm = relax(calc, params, network=net)
    assert cold.last_converged and warm.last_converged
    assert warm.last_steps <= cold.last_steps
    np.testing.assert_allclose(q_warm, q_cold, atol=2e-4)
    assert abs(q_warm.sum()) < 1e-9

"""Velocity Verlet on the device (pg_md_run, pg_md_verlet) against ASE's
update written out on the host around the same force evaluations.

The host loop is VelocityVerlet.step of ase/md/verlet.py in NumPy:
p += 0.5 dt F; r = r + dt p / m; F = calc.get_forces(); p += 0.5 dt F, with
the calculator updating its neighbour list by the skin/2 rule.  The device
loop uses the same force kernels on the same coordinates and the same
rounding, so the trajectories agree bit for bit, list rebuilds included.
"""
import numpy as np
import pytest

import pysic_gb300 as pysic
from pysic_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FS = 0.09822694788464063  # one femtosecond in ASE time units


def _hot_silicon(seed=3, temperature=3000.0):
    atoms = W.diamond_si(3, noise=0.05, seed=seed)
    kT = 8.617333262e-5 * temperature
    m = atoms.get_masses()[:, None]
    p = np.random.default_rng(seed).normal(0.0, 1.0, (len(atoms), 3)) * np.sqrt(m * kT)
    p -= p.mean(axis=0)
    atoms.set_momenta(p)
    return atoms


def _host_verlet(atoms, calc, dt, steps):
    atoms.set_calculator(calc)
    f = atoms.get_forces()
    m = atoms.get_masses()[:, None]
    for _ in range(steps):
        p = atoms.get_momenta()
        p += 0.5 * dt * f
        r = atoms.get_positions()
        atoms.set_positions(r + dt * p / m)
        atoms.set_momenta(p)
        f = atoms.get_forces()
        atoms.set_momenta(atoms.get_momenta() + 0.5 * dt * f)
    return atoms.get_positions(), atoms.get_momenta()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_device_verlet_matches_the_host_loop_with_rebuilds(precision):
    dt, steps = 2.0 * FS, 40
    a_host = _hot_silicon()
    calc_h = pysic.Pysic(a_host, W.tersoff_si_potentials(), precision=precision)
    # one tile for both contexts: the autotuner times its candidates per
    # context, and another lanes-per-atom split sums in another order
    calc_h.set_core()
    calc_h.engine.set_lanes(4)
    r_h, p_h = _host_verlet(a_host, calc_h, dt, steps)
    rebuilds_host = calc_h.get_neighbor_lists().nupdates

    a_dev = _hot_silicon()
    calc_d = pysic.Pysic(a_dev, W.tersoff_si_potentials(), precision=precision)
    calc_d.set_core()
    calc_d.engine.set_lanes(4)
    a_dev.set_calculator(calc_d)
    dyn = pysic.VelocityVerlet(a_dev, dt)
    dyn.run(steps)
    assert dyn.nsteps == steps
    assert calc_d.get_neighbor_lists().nupdates == rebuilds_host > 1
    np.testing.assert_array_equal(a_dev.get_positions(), r_h)
    np.testing.assert_array_equal(a_dev.get_momenta(), p_h)
    # the calculator answers for the final positions without a stale result
    np.testing.assert_array_equal(a_dev.get_forces(), calc_h.get_forces(a_host))


def test_stop_at_rebuild_loop_matches_the_rebuilding_loop():
    """pg_md_verlet (stops when a rebuild is due; the host rebuilds and calls
    again) gives the trajectory of pg_md_run (rebuilds on the device), bit for
    bit; lists installed from the host are refused by pg_md_run."""
    from pysic_gb300 import _lib as L

    dt, steps = 2.0 * FS, 30

    def fresh():
        a = _hot_silicon(seed=11)
        c = pysic.Pysic(a, W.tersoff_si_potentials(), precision="mixed")
        c.set_core()
        c.engine.set_lanes(4)
        c.get_forces()
        eng = c.engine
        eng.md_set_state(a.get_masses(), a.get_momenta())
        return c, eng

    c1, e1 = fresh()
    nl = c1.get_neighbor_lists()
    left, host_rebuilds = steps, 0
    while left > 0:
        done, rebuild = e1.md_verlet(L.PREC_MIXED, left, dt, nl.skin)
        left -= done
        if rebuild:
            e1.build_neighbors(nl.cutoffs, nl.skin)
            host_rebuilds += 1
    p1, r1 = e1.md_get_state()

    c2, e2 = fresh()
    done, rebuilds = e2.md_run(L.PREC_MIXED, steps, dt, c2.get_neighbor_lists().skin)
    p2, r2 = e2.md_get_state()
    assert done == steps and rebuilds == host_rebuilds > 0
    np.testing.assert_array_equal(r1, r2)
    np.testing.assert_array_equal(p1, p2)
    # the reference positions of the last list generation
    lp = e2.list_positions()
    assert np.abs(lp - r2).max() <= 0.5 * c2.get_neighbor_lists().skin

    counts, idx, off = e2.neighbor_lists()
    e2.install_neighbors(counts, idx, off, c2.get_neighbor_lists().skin)
    with pytest.raises(L.EngineError) as err:
        e2.md_run(L.PREC_MIXED, 2, dt, c2.get_neighbor_lists().skin)
    assert err.value.status == L.PG_ERR_NOT_READY


def test_observers_cut_the_run_without_changing_it():
    dt = 2.0 * FS
    def calc_for(a):
        c = pysic.Pysic(a, W.tersoff_si_potentials())
        c.set_core()
        c.engine.set_lanes(4)
        return c

    a1 = _hot_silicon(seed=5)
    a1.set_calculator(calc_for(a1))
    pysic.VelocityVerlet(a1, dt).run(30)

    a2 = _hot_silicon(seed=5)
    a2.set_calculator(calc_for(a2))
    dyn = pysic.VelocityVerlet(a2, dt)
    seen = []
    dyn.attach(lambda: seen.append((dyn.nsteps, a2.get_positions().copy())), interval=7)
    dyn.run(30)
    assert [s for s, _ in seen] == [0, 7, 14, 21, 28]
    np.testing.assert_array_equal(a2.get_positions(), a1.get_positions())
    np.testing.assert_array_equal(a2.get_momenta(), a1.get_momenta())


def test_energy_is_conserved():
    """NVE: total energy drifts by far less than its thermal fluctuation."""
    atoms = _hot_silicon(seed=7, temperature=600.0)
    calc = pysic.Pysic(atoms, W.tersoff_si_potentials())
    atoms.set_calculator(calc)
    dyn = pysic.VelocityVerlet(atoms, 1.0 * FS)
    m = atoms.get_masses()[:, None]

    def total():
        return atoms.get_potential_energy() + 0.5 * float((atoms.get_momenta() ** 2 / m).sum())

    e0 = total()
    energies = []
    dyn.attach(lambda: energies.append(total()), interval=50)
    dyn.run(400)
    kinetic = 0.5 * float((atoms.get_momenta() ** 2 / m).sum())
    assert max(abs(e - e0) for e in energies) < 2e-3 * kinetic


def test_verlet_relaxes_the_charges_at_every_step():
    """With a ChargeRelaxation on the calculator every force call relaxes the
    charges first (Pysic.get_forces); the dynamics do the same at every step:
    the same trajectory and charges as ASE's update around get_forces, and the
    final charges equalise the electronegativities."""
    from pysic_gb300 import workloads as W

    def make():
        atoms = W.sio2_box(60, seed=31)
        atoms.set_initial_charges(np.zeros(len(atoms)))
        rng = np.random.default_rng(31)
        m = atoms.get_masses()[:, None]
        p = rng.normal(0.0, 1.0, (len(atoms), 3)) * np.sqrt(m * 8.617333e-5 * 300.0)
        atoms.set_momenta(p - p.mean(axis=0))
        pots, coul = W.sio2_potentials(real_cutoff=5.5, sigma=1.6)
        calc = pysic.Pysic(atoms, pots, coulomb=coul, precision="fp64")
        calc.set_charge_relaxation(pysic.ChargeRelaxation("dynamic", parameters=[2000, 0.05, 1.0, 3.0, 1e-7]))
        return atoms, calc

    dt, steps = 0.5 * FS, 6
    a_host, c_host = make()
    r_h, p_h = _host_verlet(a_host, c_host, dt, steps)
    a_dev, c_dev = make()
    a_dev.set_calculator(c_dev)
    seen = []
    dyn = pysic.VelocityVerlet(a_dev, dt)
    dyn.attach(lambda: seen.append(c_dev.get_atoms().get_initial_charges().copy()), interval=2)
    dyn.run(steps)
    assert np.array_equal(a_dev.get_positions(), r_h)
    assert np.array_equal(a_dev.get_momenta(), p_h)
    q = c_dev.get_atoms().get_initial_charges()
    assert np.array_equal(q, c_host.get_atoms().get_initial_charges())
    assert np.abs(q).max() > 0.1 and len(seen) == 4
    assert not np.array_equal(seen[1], seen[3])  # the charges follow the moving atoms
    chi = c_dev.get_electronegativities()
    assert np.abs(chi - chi.mean()).max() < 1e-6

"""GPU parity of the optimisation-loop callers of the hot path against runs of the reference's own code.

`Measurements.train` (measure.py:473-553) runs on the device (adjoint energy and gradient, QNG through the
device QFIM); its trajectories -- energy, Renyi-2 magic, Meyer-Wallach Q and GKP at every iteration -- are
compared with the reference's `train` on the same circuit, angles and `gates.rng` seed
(tests/golden/make_golden.py section 8).  `find_overparam_point` (measure.py:101-121) and `find_eff_H`
(measure.py:199-224) are compared with the reference's values the same way.
"""
import numpy as np
import pytest

import recipes
import pyramaterised_gb300 as pq
from pyramaterised_gb300 import gates

pytestmark = pytest.mark.gpu
TOL = 1e-9  # energies, Q and magic after hundreds of iterations of double-float arithmetic


def _circuit(L=2):
    c = recipes.he_ladder(pq, 4, L)
    c.set_H(pq.templates.TFIM_hamiltonian(4, 1.0))
    return c


@pytest.mark.parametrize("tag,angles_kind,method,rate,eps", [("grad_fixed", "fixed", "gradient", 0.05, 1e-4),
                                                             ("grad_random", "random", "gradient", 0.1, 1e-3),
                                                             ("qng_fixed", "fixed", "QNG", 0.05, 1e-4)])
def test_train_matches_reference_trajectories(cuda, golden, golden_meta, tag, angles_kind, method, rate, eps):
    key = f"train/{tag}"
    meta = golden_meta["meta"][key]
    gates.rng = np.random.default_rng(1)
    c = _circuit(meta["layers"])
    P = c.n_columns()
    angles = list(np.random.default_rng(meta["seed"]).random(P) * 2 * np.pi) if angles_kind == "fixed" else "random"
    energy, traj, magics, ents, gkps = pq.measure.Measurements(c).train(epsilon=eps, rate=rate, method=method,
                                                                        angles=angles)
    gates.rng = np.random.default_rng(1)
    its = meta["iterations"]
    if method == "QNG":
        # QNG steps with pinv of the QFIM, whose condition number grows to about 1e4 along this run, so
        # rounding-level differences of F (1e-13) are amplified: the trajectories agree to 1e-6 and the stop
        # point to a few iterations
        n = min(len(traj), len(golden[f"{key}/traj"]))
        for name, got in (("traj", traj), ("magics", magics), ("ents", ents), ("gkps", gkps)):
            np.testing.assert_allclose(np.asarray(got[:n]), golden[f"{key}/{name}"][:n], atol=1e-6, rtol=0,
                                       err_msg=name)
        print(f"QNG: {len(traj) - 1} iterations (reference {its}), final energy {energy} "
              f"(reference {float(golden[f'{key}/energy'])})")
        assert abs((len(traj) - 1) - its) <= 3
        assert abs(energy - float(golden[f"{key}/energy"])) < 1e-6
        return
    assert len(traj) - 1 == its
    assert abs(energy - float(golden[f"{key}/energy"])) < TOL
    for name, got in (("traj", traj), ("magics", magics), ("ents", ents), ("gkps", gkps)):
        np.testing.assert_allclose(np.asarray(got), golden[f"{key}/{name}"], atol=TOL, rtol=0, err_msg=name)
    np.testing.assert_allclose(np.asarray(c.get_params(), dtype=np.float64), golden[f"{key}/final_theta"],
                               atol=1e-8, rtol=0)


def test_train_lower_case_qng_runs_the_natural_gradient(cuda, golden):
    # the reference raises NameError for "qng"; here it is the same method as "QNG"
    c = _circuit(1)
    angles = list(np.random.default_rng(7).random(c.n_columns()) * 2 * np.pi)
    energy = pq.measure.Measurements(c).train(epsilon=1e-4, rate=0.05, method="qng", angles=angles)[0]
    assert abs(energy - float(golden["train/qng_fixed/energy"])) < 1e-6


def test_train_with_a_scipy_method_lowers_the_energy(cuda):
    c = _circuit()
    angles = list(np.random.default_rng(5).random(c.n_columns()) * 2 * np.pi)
    energy, traj, magics, ents, gkps = pq.measure.Measurements(c).train(epsilon=1e-6, method="BFGS", angles=angles)
    assert energy < traj[0] and len(traj) == len(magics) == len(ents) == len(gkps) > 1


def test_find_overparam_point_matches_reference(cuda, golden):
    gates.rng = np.random.default_rng(1)
    c = recipes.he_ladder(pq, 3, 1)
    count = pq.measure.Measurements(c).find_overparam_point([0])
    gates.rng = np.random.default_rng(1)
    assert count == int(golden["overparam/he3/count"])
    assert len(c.layers) == int(golden["overparam/he3/layers"])


def test_find_eff_H_matches_reference(cuda, golden):
    c = recipes.he_ladder(pq, 3, 2)
    got = pq.measure.Measurements(c).find_eff_H(list(golden["eff_h/he3/samples"]), 3)
    assert abs(got - float(golden["eff_h/he3/value"])) < 1e-6 * abs(float(golden["eff_h/he3/value"]))

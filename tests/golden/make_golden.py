"""Generate golden vectors by running the reference's own Python code.

The reference (rmdocherty/pyramaterised) depends on QuTiP 4.7.2, which is not
installed here; `oracle/qutip_shim` restates the QuTiP subset it calls.  This
script imports the reference package from its checkout with that shim on
`sys.path`, evaluates the circuits in `recipes.py` with the reference's own
`PQC` / `Measurements` code, and writes `reference_golden.npz` next to it.

Usage (development container only; the reference is not shipped):
    python tests/golden/make_golden.py /path/to/reference/checkout
"""
import json
import os
import random
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def main(ref_root):
    sys.path.insert(0, os.path.join(REPO, "oracle", "qutip_shim"))
    sys.path.insert(0, ref_root)
    sys.path.insert(0, HERE)
    import pyramaterised as ref  # the reference package
    import qutip as qt
    import recipes

    out = {}
    meta = {}

    def reset_rng():
        ref.gates.rng = np.random.default_rng(1)
        # circuit.py / measure.py see `rng` through `from .gates import *`
        ref.circuit.rng = ref.gates.rng

    def ket(q):
        return q.data.toarray()[:, 0]

    def record_circuit(key, c, theta, with_grads=True, H=None):
        N = c.n_qubits
        state = c.run(list(theta))
        out[f"{key}/theta"] = np.asarray(theta, dtype=np.float64)
        out[f"{key}/state"] = ket(state)
        out[f"{key}/init"] = ket(c.initial_state)
        info = {"N": N, "n_params": int(len(theta))}
        if N >= 2:
            out[f"{key}/energy_ZZ"] = np.array(float(c.cost(list(theta))))
        if H is not None:
            c.set_H(H)
            out[f"{key}/energy_H"] = np.array(float(c.cost(list(theta))))
        if with_grads:
            try:
                c.state = c.run(list(theta))
                grads = c.get_gradients()
                out[f"{key}/grads"] = np.array([ket(g) for g in grads])
                m = ref.measure.Measurements(c)
                out[f"{key}/qfim"] = np.asarray(m.get_QFI(), dtype=np.float64)
                info["grads"] = "ok"
            except Exception as e:  # the reference itself fails on some gate types
                info["grads"] = f"reference raised {type(e).__name__}: {e}"[:200]
            if N >= 2 and info.get("grads") == "ok":
                try:
                    m = ref.measure.Measurements(c)
                    out[f"{key}/grad_vector"] = np.asarray(m.get_gradient_vector(list(theta)), dtype=np.float64)
                except Exception as e:
                    info["grad_vector"] = f"reference raised {type(e).__name__}"
        meta[key] = info

    # 1. the reference's own qg-circuit test (tests.py:158-213)
    c = recipes.qg_test_circuit(ref)
    record_circuit("qg_test", c, recipes.QG_DEFAULT_ANGLES)
    m = ref.measure.Measurements(c)
    c.cost(recipes.QG_DEFAULT_ANGLES)
    out["qg_test/eqd"] = np.array(m.get_effective_quantum_dimension(10 ** -12))

    # 2. templates: gate signatures + state, gradients, QFIM at seeded angles
    sigs = {}
    for name, N, p in recipes.TEMPLATES:
        key = f"tpl/{name}/{N}/{p}"
        reset_rng()
        c = recipes.template_circuit(ref, name, N, p)
        sigs[key] = recipes.gate_signature(c)
        P = len([g for g in c.gates if g.is_param for _ in range(g.param_count)])
        theta = np.random.default_rng(11).random(P) * 2 * np.pi
        record_circuit(key, c, theta, H=ref.templates.TFIM_hamiltonian(N, 1.0, 0.5))

    # 3. NPQC identity QFIM (tests.py:103-128) at its reference angles
    for N in (4, 6):
        for P in (1, 2, 2 ** (N // 2)):
            layers, theta_ref = ref.templates.NPQC_layers(P, N)
            c = ref.PQC(N)
            for l in layers:
                c.add_layer(l)
            c.state = qt.Qobj(c.run(angles=theta_ref))
            out[f"npqc/{N}/{P}/qfim"] = np.asarray(ref.measure.Measurements(c).get_QFI(), dtype=np.float64)
            out[f"npqc/{N}/{P}/theta"] = np.asarray(theta_ref, dtype=np.float64)

    # 4. benchmark ansaetze at small N
    for rname, N, L in (("he_ladder", 4, 4), ("he_ladder", 5, 2), ("tfim_style", 4, 2), ("npqc_style", 4, 4),
                        ("npqc_style", 5, 3)):
        c = getattr(recipes, rname)(ref, N, L)
        P = len([g for g in c.gates if g.is_param])
        theta = np.random.default_rng(0).random(P) * 2 * np.pi
        record_circuit(f"ansatz/{rname}/{N}/{L}", c, theta, H=ref.templates.TFIM_hamiltonian(N, 1.0, 0.0))

    # 5. every gate class and the fSim gradient quirk
    for rname in ("every_gate", "fsim_mix"):
        c = getattr(recipes, rname)(ref, 4)
        P = len([g for g in c.gates if g.is_param for _ in range(g.param_count)])
        theta = np.random.default_rng(3).random(P) * 2 * np.pi
        record_circuit(f"special/{rname}", c, theta)

    # 6. measures on random states: efficient_measurements with the global rng (measure.py:370-459)
    reset_rng()
    c = recipes.he_ladder(ref, 4, 4)
    m = ref.measure.Measurements(c)
    em = m.efficient_measurements(101)
    reset_rng()
    full = m.efficient_measurements(101, full_data=True)
    out["em/he4/expr"] = np.array(em["Expr"])
    out["em/he4/ent"] = np.array(em["Ent"], dtype=np.float64)
    out["em/he4/magic"] = np.array(em["Magic"], dtype=np.float64)
    out["em/he4/gkp"] = np.array(em["GKP"], dtype=np.float64)
    out["em/he4/overlaps"] = np.array(full["Expr"], dtype=np.float64)
    out["em/he4/q"] = np.array(full["Ent"], dtype=np.float64)
    out["em/he4/magics"] = np.array(full["Magic"], dtype=np.float64)
    out["em/he4/gkps"] = np.array(full["GKP"], dtype=np.float64)
    # expressibility(150) on generic_HE (measure.py:182-197), and the Clifford-angle mode
    reset_rng()
    c = ref.templates.generate_circuit("generic_HE", 3, 3)
    out["expr/generic_HE3/value"] = np.array(ref.measure.Measurements(c).expressibility(150))
    reset_rng()
    random.seed(5)
    c = recipes.he_ladder(ref, 3, 2)
    cl = ref.measure.Measurements(c).efficient_measurements(20, angles="clifford")
    out["em/clifford3/magic"] = np.array(cl["Magic"], dtype=np.float64)
    out["em/clifford3/ent"] = np.array(cl["Ent"], dtype=np.float64)
    out["em/clifford3/expr"] = np.array(cl["Expr"])
    # idle (I gate) and 1-qubit circuits of test_expressibility (tests.py:217-247)
    reset_rng()
    idle = ref.PQC(1)
    idle.add_layer([ref.I(0, 1)])
    out["em/idle/expr"] = np.array(ref.measure.Measurements(idle).efficient_measurements(
        400, measure_ent=False, measure_eom=False, measure_GKP=False)["Expr"])
    reset_rng()
    ca = ref.PQC(1)
    ca.add_layer([ref.H(0, 1), ref.R_z(0, 1)])
    out["em/circA/expr"] = np.array(ref.measure.Measurements(ca).efficient_measurements(
        400, measure_ent=False, measure_eom=False, measure_GKP=False)["Expr"])

    # 7. Bell state (tests.py:284-295) and magic on seeded random kets
    bell = qt.states.bell_state("11")
    mb = ref.measure.Measurements(ref.PQC(2))
    out["bell/magic"] = np.array(mb.renyi_entropy_fast(bell))
    out["bell/gkp"] = np.array(mb.gkp_fast(bell))
    out["bell/q"] = np.array(mb.single_Q(bell, 2))
    rs = np.random.default_rng(21)
    for N in (1, 2, 3, 4, 5, 6):
        v = rs.standard_normal(2 ** N) + 1j * rs.standard_normal(2 ** N)
        v /= np.linalg.norm(v)
        q = qt.Qobj(v.reshape(-1, 1), dims=[[2] * N, [1] * N])
        mq = ref.measure.Measurements(ref.PQC(N))
        out[f"ket/{N}/psi"] = v
        out[f"ket/{N}/magic"] = np.array(mq.renyi_entropy_fast(q))
        out[f"ket/{N}/gkp"] = np.array(mq.gkp_fast(q))
        out[f"ket/{N}/q"] = np.array(mq.single_Q(q, N))

    # 9. shared_parameter(commute=False) over members that do not commute (gates.py:459-466): derivative
    #    states and QFIM by the reference's own dense form
    for N in (3, 4):
        c = recipes.shared_noncommuting(ref, N)
        P = len([g for g in c.gates if g.is_param])
        theta = np.random.default_rng(40 + N).random(P) * 2 * np.pi
        record_circuit(f"shared_nc/{N}", c, theta, H=ref.templates.TFIM_hamiltonian(N, 1.0, 0.0))

    # 8. training trajectories (measure.py:473-553), the overparameterisation point (measure.py:101-121) and the
    #    effective Hilbert-space dimension (measure.py:199-224), each run by the reference's own code
    #    (the QNG case uses one layer, whose QFIM stays well conditioned along the run: pinv of a near-singular
    #    QFIM turns rounding-level differences into different trajectories)
    for tag, angles_kind, method, rate, eps, L, seed in (("grad_fixed", "fixed", "gradient", 0.05, 1e-4, 2, 5),
                                                         ("grad_random", "random", "gradient", 0.1, 1e-3, 2, 5),
                                                         ("qng_fixed", "fixed", "QNG", 0.05, 1e-4, 1, 7)):
        reset_rng()
        c = recipes.he_ladder(ref, 4, L)
        c.set_H(ref.templates.TFIM_hamiltonian(4, 1.0))
        P = len([g for g in c.gates if g.is_param])
        angles = list(np.random.default_rng(seed).random(P) * 2 * np.pi) if angles_kind == "fixed" else "random"
        m = ref.measure.Measurements(c)
        energy, traj, magics, ents, gkps = m.train(epsilon=eps, rate=rate, method=method, angles=angles)
        key = f"train/{tag}"
        out[f"{key}/energy"] = np.array(float(energy))
        for name, v in (("traj", traj), ("magics", magics), ("ents", ents), ("gkps", gkps)):
            out[f"{key}/{name}"] = np.asarray(v, dtype=np.float64)
        out[f"{key}/final_theta"] = np.asarray(c.get_params(), dtype=np.float64)
        meta[key] = {"method": method, "rate": rate, "epsilon": eps, "angles": angles_kind, "layers": L,
                     "seed": seed, "iterations": len(traj) - 1}
    reset_rng()
    c = recipes.he_ladder(ref, 3, 1)
    m = ref.measure.Measurements(c)
    out["overparam/he3/count"] = np.array(m.find_overparam_point([0]))
    out["overparam/he3/layers"] = np.array(len(c.layers))
    reset_rng()
    c = recipes.he_ladder(ref, 3, 2)
    m = ref.measure.Measurements(c)
    F = m._gen_f_samples(60)
    out["eff_h/he3/samples"] = np.asarray(F, dtype=np.float64)
    out["eff_h/he3/value"] = np.array(float(m.find_eff_H(F, 3)))

    np.savez_compressed(os.path.join(HERE, "reference_golden.npz"), **out)
    with open(os.path.join(HERE, "reference_golden.json"), "w") as f:
        json.dump({"meta": meta, "signatures": {k: [list(map(_j, s)) for s in v] for k, v in sigs.items()}}, f,
                  indent=1, sort_keys=True)
    print(f"wrote {len(out)} arrays")


def _j(x):
    if isinstance(x, tuple):
        return [_j(y) for y in x]
    if isinstance(x, (np.integer,)):
        return int(x)
    return x


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout>")
    main(sys.argv[1])

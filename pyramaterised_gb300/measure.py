"""`Measurements`: the reference's capacity measures on the GB300 engine.

Mirrors `pyramaterised/measure.py` (reference).  Every state-sized
computation runs on the device: fidelities/histograms (`pqc_fidelity_hist`),
Meyer-Wallach (`pqc_mw`), magic (`pqc_magic`), QFIM (`pqc_qfim` over
`pqc_derivative_states`), energies and adjoint gradients.  What stays on the
host is what the reference does with O(P^2) or O(bins) numbers: `eigh` of the
QFIM (scipy, so the eigenvalue cutoff behaves identically), the optimiser
loops, and the final means/standard deviations.
"""
import random
from itertools import combinations  # noqa: F401  (reference import surface)
from typing import Callable, Dict, Tuple, Union  # noqa: F401

import numpy as np
import scipy
import scipy.linalg
import scipy.optimize
import scipy.special
import torch

from . import engine
from .circuit import PQC


def _as_states(x):
    if isinstance(x, (list, tuple)):
        return torch.stack([engine._c128(s, engine.device()).reshape(-1) for s in x])
    t = x if isinstance(x, torch.Tensor) else engine._c128(x.full() if hasattr(x, "full") else x, engine.device())
    return t


class Measurements:
    def __init__(self, QC: PQC):
        self.QC = QC
        try:
            self.minimize_function = QC.cost
        except AttributeError:
            self.minimize_function = lambda x: x
        self._grad_theta = None

    def set_minimise_function(self, function: Callable) -> None:
        self.minimize_function = function

    # ------------------------------------------------------------------ QFIM
    def get_QFI(self, grad_list=[], max_state_bytes=None) -> np.ndarray:
        """F_pq = 4 Re(<d_p|d_q> - <d_p|psi><psi|d_q>) (measure.py:33-71), psi = QC.state.

        When the P derivative states would take more than `max_state_bytes` of device memory (default: half of
        the free memory), they are produced and contracted in row blocks (`engine.qfim_blocked`)."""
        return self._qfim_device(grad_list, max_state_bytes).cpu().numpy()

    def _qfim_device(self, grad_list=(), max_state_bytes=None):
        """The QFIM of `get_QFI` as a device tensor."""
        if grad_list is None or len(grad_list) == 0:
            P = self.QC.program.lowered.gradient_runs()[2] if self.QC.program._grad_cache is None \
                else self.QC.program._grad_cache[2]
            need = P * 16 * (1 << self.QC.n_qubits)
            budget = max_state_bytes if max_state_bytes is not None else torch.cuda.mem_get_info()[0] // 2
            if need > budget:
                rows = max(1, int(budget // (2 * 16 * (1 << self.QC.n_qubits))))
                return engine.qfim_blocked(self.QC.program, self.QC._current_theta()[None, :], self.QC.state, rows,
                                           self.QC._psi0())
            grads = self.QC.get_gradients()
        else:
            grads = _as_states(grad_list)
        return engine.qfim(self.QC.state, grads)

    def get_eigenvalues(self, QFI: np.ndarray):
        return scipy.linalg.eigh(QFI)

    def get_effective_quantum_dimension(self, cutoff_eigvals: float) -> int:
        """Number of QFIM eigenvalues above the cutoff (measure.py:77-87)."""
        QFI = self.get_QFI()
        eigvals, eigvecs = scipy.linalg.eigh(QFI)
        return len(eigvals[eigvals > cutoff_eigvals])

    def new_measure(self, QFI: np.ndarray = None):
        """Sum of eigenvalues capped at 1 (measure.py:89-99)."""
        if QFI is None:
            QFI = self.get_QFI()
        eigvals, eigvecs = self.get_eigenvalues(QFI)
        return sum(1 if v > 1 else v for v in eigvals)

    def find_overparam_point(self, layer_index_list, epsilon: float = 1e-3) -> int:
        """Rounds of added layers after which the QFIM rank stops growing (measure.py:101-121).

        Each round appends copies of the layers `layer_index_list` to the circuit, draws new angles from
        `gates.rng` for the whole circuit and takes the rank of the QFIM of the new state on the device
        (torch.linalg.matrix_rank: singular values above max(M, N) eps sigma_max, numpy's matrix_rank rule).
        That tolerance (~1e-14 relative) is below the double-float error of the fused kernels, so the QFIM
        for the rank is formed in FP64 throughout: the one-kernel-per-op FP64 state and derivative states and
        the FP64 Gram (`pqc_qfim_fp64`).  It stops after the first round whose rank differs from the previous
        round's by at most epsilon (or after 10^6 rounds) and returns the number of rounds; the circuit keeps
        the added layers."""
        blocks = [self.QC.get_layer(i) for i in layer_index_list]
        ranks = [0]
        while len(ranks) == 1 or (abs(ranks[-1] - ranks[-2]) > epsilon and len(ranks) - 1 < 1e6):
            for layer in blocks:
                self.QC.add_layer(layer)
            self.QC.update_state("random")
            prog, th = self.QC.program, self.QC._current_theta()[None, :]
            psi = prog.run(th, self.QC._psi0(), mode="plain")
            dpsi = prog.gradient_states(th, self.QC._psi0(), plain=True)
            rank = int(torch.linalg.matrix_rank(engine.qfim(psi, dpsi, fp64=True)))
            print(f"Iteration {len(ranks) - 1}, r0={ranks[-1]}, r1={rank}, delta = {abs(rank - ranks[-1])}")
            ranks.append(rank)
        return len(ranks) - 1

    # ------------------------------------------------------------------ expressibility
    def _random_states(self, sample_N: int):
        thetas = self.QC.random_params(sample_N)
        return self.QC.run_batch(thetas)

    def _gen_f_samples(self, sample_N: int):
        """All-pairs |<psi_a|psi_b>|^2 of sample_N random states, combinations order (measure.py:123-137)."""
        states = self._random_states(sample_N)
        F, _, _ = engine.allpairs_fidelity_hist(states, 0, keep_samples=True)
        return F.cpu().numpy()

    def _gen_histo(self, F_samples, filt: float = 0):
        """Probability histogram and bin midpoints (measure.py:139-159; `filt` is ignored there too)."""
        n = len(F_samples)
        nbins = int((75 / 10000) * n)
        counts, edges = engine.histogram(np.asarray(F_samples, dtype=np.float64), nbins)
        counts = counts.cpu().numpy()
        edges = edges.cpu().numpy()
        prob = counts / sum(counts)
        F = np.array([(edges[i - 1] + edges[i]) / 2 for i in range(1, len(edges))])
        return prob, F

    def expr(self, F_samples, N, filt: int = 0) -> float:
        """KL(histogram || Haar) with Hilbert-space dimension N (measure.py:161-180)."""
        if len(F_samples) == 0:
            return 0
        nbins = int((75 / 10000) * len(F_samples))
        counts, edges = engine.histogram(np.asarray(F_samples, dtype=np.float64), nbins)
        return float(engine.expr_kl(counts, edges, N)[0])

    def expressibility(self, sample_N: int, nbins: int = None) -> float:
        """Expressibility of the circuit from sample_N random states (measure.py:182-197).

        `nbins` defaults to the reference's int(0.0075 * number of pairs)."""
        d = 2 ** self.QC.n_qubits
        states = self._random_states(sample_N)
        M = sample_N * (sample_N - 1) // 2
        if M == 0:
            return 0
        nb = int((75 / 10000) * M) if nbins is None else int(nbins)
        _, counts, edges = engine.allpairs_fidelity_hist(states, nb, keep_samples=False)
        return float(engine.expr_kl(counts, edges, d)[0])

    def find_eff_H(self, circuit_f_samples, n) -> float:
        """The Hilbert-space dimension d that minimises expr(F_samples, d) (measure.py:199-224).

        The samples are binned once on the device (np.histogram's rule, int(0.0075 M) bins on (0, 1)); the
        objective KL(histogram || (d - 1)(1 - F)^(d - 2)) then needs only the bin counts, so scipy's BFGS
        (started at d = 4, as in the reference) evaluates it on the host.  The reference sends n > 10 to an
        undefined `log_expr`; that case raises NotImplementedError here."""
        if n > 10:
            raise NotImplementedError("the reference's n > 10 branch calls an undefined log_expr")
        F = np.asarray(circuit_f_samples, dtype=np.float64)
        if len(F) == 0:
            objective = lambda d: 0.0  # noqa: E731  (expr of no samples is 0)
        else:
            counts, edges = engine.histogram(F, int((75 / 10000) * len(F)))
            counts, edges = counts.cpu().numpy(), edges.cpu().numpy()
            # the reference's own normalisations (builtin sum, in bin order) so that BFGS sees the same numbers
            prob = counts / sum(counts)
            mid = (edges[:-1] + edges[1:]) / 2

            def objective(d):
                haar = (d - 1) * (1 - mid) ** (d - 2)
                return np.sum(scipy.special.kl_div(prob, haar / sum(haar)))
        out = scipy.optimize.minimize(objective, [4], method="BFGS")
        if out.success is True:
            return out.x[0]
        print(out)
        return 0

    # ------------------------------------------------------------------ entanglement
    def single_Q(self, system, n=None) -> float:
        """Meyer-Wallach Q of one state (measure.py:226-237)."""
        return float(engine.mw(_as_states(system))[0])

    def entanglement(self, sample_N: int):
        """Q of sample_N random states (measure.py:239-249)."""
        return list(engine.mw(self._random_states(sample_N)).cpu().numpy())

    # ------------------------------------------------------------------ magic
    def theta_to_magic(self, angles) -> float:
        state = self.QC.run(angles=angles)
        return -1 * self.renyi_entropy_fast(state)

    def theta_to_gkp(self, angles):
        state = self.QC.run(angles=angles)
        return -1 * self.gkp_fast(state)

    def get_conversion_matrices(self):
        """The reference precomputes O(4^N) index/sign matrices here (measure.py:304-313);
        the Walsh-Hadamard kernel needs none, so this returns None."""
        return None

    def set_converstion_matrices(self, conv_mats) -> None:
        self.conversion_matrices = conv_mats

    def renyi_entropy_fast(self, state, conversion_matrices=None, alpha: float = 2) -> float:
        """Renyi-alpha stabiliser entropy (measure.py:318-349)."""
        return float(engine.magic(_as_states(state), alpha)[0])

    def entropy_of_magic(self, sample_N: int):
        """Mean magic of sample_N random states (measure.py:351-359)."""
        return float(np.mean(engine.magic(self._random_states(sample_N)).cpu().numpy()))

    def gkp_fast(self, state, conversion_matrices=None) -> float:
        """1/(2 ln 2) M_{1/2} (measure.py:361-368)."""
        return 1 / (2 * np.log(2)) * self.renyi_entropy_fast(state, conversion_matrices, alpha=1 / 2)

    # ------------------------------------------------------------------ combined
    def efficient_measurements(self, sample_N: int, measure_expr: bool = True, measure_ent: bool = True,
                               measure_eom: bool = True, measure_GKP: bool = True, full_data: bool = False,
                               angles="random", lift_limits: bool = False, nbins: int = None) -> Dict:
        """Shared states for Expr/Ent/Magic/GKP (measure.py:370-459); unmeasured values are -1.

        The reference computes overlaps only for n < 12 and the KL only for
        n < 7; `lift_limits=True` removes both limits (GPU-sized inputs)."""
        n = self.QC.n_qubits
        if sample_N == 0:
            measure_expr = measure_ent = measure_eom = measure_GKP = False
        if angles == "clifford":
            clifford_angles = (0, np.pi / 2, np.pi, 3 * np.pi / 2, 2 * np.pi)
            P = self.QC.n_columns()
            rows = [[random.choice(clifford_angles) for i in range(self.QC.n_params)] for i in range(sample_N)]
            thetas = np.asarray([r[:P] for r in rows], dtype=np.float64).reshape(sample_N, P)
            if sample_N:
                self.QC.set_params(list(thetas[-1]))
            states = self.QC.run_batch(thetas) if sample_N else None
        else:
            states = self._random_states(sample_N) if sample_N else None
        overlaps, magics, gkps, q_vals = [], [], [], []
        expr_max_n = 10 ** 9 if lift_limits else 12
        kl_max_n = 10 ** 9 if lift_limits else 7
        if measure_expr and n < expr_max_n and sample_N >= 2:
            M = sample_N * (sample_N - 1) // 2
            nb = int((75 / 10000) * M) if nbins is None else int(nbins)
            F, counts, edges = engine.allpairs_fidelity_hist(states, max(nb, 1), keep_samples=full_data)
            if full_data:
                overlaps = list(F.cpu().numpy())
            if n < kl_max_n:
                expr = float(engine.expr_kl(counts, edges, 2 ** n)[0]) if nb >= 1 else float("nan")
            else:
                expr = -1
        else:
            expr = -1
        if measure_ent:
            q_vals = list(engine.mw(states).cpu().numpy())
            q, std = np.mean(q_vals), np.std(q_vals)
        else:
            q, std = -1, -1
        if measure_eom:
            magics = list(engine.magic(states, 2.0).cpu().numpy())
            magic_bar, magic_std = np.mean(magics), np.std(magics)
        else:
            magic_bar, magic_std = -1, -1
        if measure_GKP:
            gkps = list((1 / (2 * np.log(2)) * engine.magic(states, 0.5)).cpu().numpy())
            gkp_bar, gkp_std = np.mean(gkps), np.std(gkps)
        else:
            gkp_bar, gkp_std = -1, -1
        if full_data is True:
            return {"Expr": overlaps, "Ent": q_vals, "Magic": magics, "GKP": gkps}
        return {"Expr": expr, "Ent": [q, std], "Magic": [magic_bar, magic_std], "GKP": [gkp_bar, gkp_std]}

    # ------------------------------------------------------------------ gradients / training
    def get_gradient_vector(self, theta):
        """dE/dtheta_i = 2 Re <psi|H|d_i psi> (measure.py:461-471), by the adjoint sweep."""
        self.QC.state = self.QC.run(angles=theta)
        self._grad_theta = list(theta)
        prog = self.QC.program
        try:
            E, g = prog.energy_grad(self.QC._current_theta()[None, :], self.QC.H, self.QC._psi0())
            return list(g[0].cpu().numpy())
        except NotImplementedError:
            # fSim circuits: the reference's rows are not true derivatives; use its derivative states
            return list(_grad_from_states(self.QC, self.QC.get_gradients()))

    @property
    def gradient_list(self):
        """Derivative states of the last `get_gradient_vector` call (measure.py:464)."""
        return self.QC.get_gradients()

    def train(self, epsilon: float = 1e-6, rate: float = 0.001, method: str = "gradient", angles="random",
              verbose: bool = False):
        """Minimise the energy (measure.py:473-553); returns (energy, traj, magics, ents, gkps).

        method "gradient" or "QNG" (any case): the descent runs on the device (`training.Descent`) and the
        per-iteration Renyi-2 magic, Meyer-Wallach Q and GKP of the visited states are evaluated afterwards in
        batches.  The lists follow the reference's bookkeeping: entry 0 holds the magic of the first state and
        the energy, Q and GKP after the callback's own cost call (with angles="random" those are two different
        draws from `gates.rng`, and the descent starts from a third), then one entry per iteration.  Other
        methods go to scipy.optimize.minimize with the same callback.  The reference raises NameError for
        method "qng" in lower case; here it means QNG."""
        qc = self.QC
        mf = self.minimize_function
        default_cost = getattr(mf, "__self__", None) is qc and getattr(mf, "__func__", None) is PQC.cost
        if isinstance(method, str) and method.lower() in ("gradient", "qng") and default_cost:
            return self._train_on_device(epsilon, rate, method, angles, verbose)
        return self._train_on_host(epsilon, rate, method, angles, verbose)

    def _train_on_device(self, epsilon, rate, method, angles, verbose):
        from .training import Descent, batched_measures

        qc = self.QC
        if isinstance(angles, str):
            if angles != "random":
                raise Exception("No parameters supplied!")
            rows = qc.random_params(3)
        else:
            rows = np.repeat(np.asarray(qc.set_params(angles), dtype=np.float64)[None, :], 3, axis=0)
        # rows: the first state's angles (magic), the callback's cost call (energy, Q, GKP), the start point
        run = Descent(qc, rate, method)
        thetas, energies, T = run.run(rows[2], epsilon, verbose)
        head = torch.as_tensor(rows[:2], device=thetas.device)
        mags, qs, gkps = batched_measures(qc, torch.cat([head, thetas[1:]]))
        E_first = float(qc.cost_batch(head[1:2])[0])
        traj = [E_first] + list(energies[1:])
        magics = [mags[0]] + list(mags[2:])
        ents = [qs[1]] + list(qs[2:])
        gkp_l = [gkps[1]] + list(gkps[2:])
        final = thetas[-1].cpu().numpy()
        qc.state = qc.run(list(final))
        return (float(energies[-1]), traj, magics, ents, gkp_l)

    def _train_on_host(self, epsilon, rate, method, angles, verbose):
        """A user-supplied cost function, or a scipy.optimize method: the loop evaluates through the caller's
        function on the host, with the callback measures of each visited state."""
        qc = self.QC
        traj, magics, ents, gkps = [], [], [], []

        def record(x):
            magics.append(self.renyi_entropy_fast(qc.state))
            traj.append(self.minimize_function(x))
            ents.append(self.single_Q(qc.state, qc.n_qubits))
            gkps.append(self.gkp_fast(qc.state))

        qc.state = qc.run(angles=angles)
        record(angles)
        if not (isinstance(method, str) and method.lower() in ("gradient", "qng")):
            res = scipy.optimize.minimize(self.minimize_function, x0=angles, method=method, callback=record,
                                          tol=epsilon)
            return (res.fun, traj, magics, ents, gkps)
        qng = method.lower() == "qng"
        prev = self.minimize_function(angles)
        diff, count, energy = 1.0, 0, prev
        while diff > epsilon and count < 100000:
            theta = np.asarray(qc.get_params(), dtype=np.float64)
            g = np.asarray(self.get_gradient_vector(list(theta)))
            step = np.linalg.pinv(self.get_QFI()).dot(g) if qng else g
            if verbose and count % 100 == 0:
                print(f"On iteration {count}, energy = {prev}, diff is {diff}")
            nxt = list(theta - rate * step)
            energy = self.minimize_function(nxt)
            diff = abs(energy - prev)
            record(nxt)
            count += 1
            prev = energy
        return (energy, traj, magics, ents, gkps)


def _grad_from_states(QC, grads):
    """2 Re <psi|H|d_i psi> from explicit derivative states (used when no adjoint form exists)."""
    psi = QC.state.reshape(1, -1)
    # polarisation of the Hermitian form: 2 Re<psi|H|d> = (E(psi + d) - E(psi - d)) / 2
    plus = engine.expect(psi + grads, QC.H)
    minus = engine.expect(psi - grads, QC.H)
    return list(((plus - minus) / 2).cpu().numpy())

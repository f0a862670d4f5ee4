"""Device-resident descent of the energy <H> for `Measurements.train`.

The reference (`pyramaterised/measure.py:473-553`) runs plain gradient descent
(or quantum natural gradient, QNG) one iteration at a time on the host: it
re-runs the circuit for the derivative states, forms 2 Re <psi|H|d_i psi>,
steps theta, re-runs the circuit for the new energy and, through its callback,
for the Renyi-2 magic, Meyer-Wallach Q and GKP of every visited state.

Here the whole iteration stays on the GPU: one adjoint sweep
(`Program.energy_grad`) gives both E(theta_t) and its gradient, QNG solves with
the pseudo-inverse of the device QFIM (`torch.linalg.pinv`, numpy's cutoff rule
rcond = 1e-15 relative to the largest singular value), and the update is a
device op.  The host reads the energies once per block of `check_every`
iterations to apply the stopping rule |E_{t+1} - E_t| <= epsilon; iterations
computed past the stop are dropped (each depends only on earlier ones, so the
kept ones are those the reference computes).  The callback measures of the
visited states run afterwards, batched over the parameter history.
"""
import numpy as np
import torch

from . import engine


class Descent:
    """Gradient or QNG descent of <H> for one circuit (a `PQC`) on the device."""

    def __init__(self, qc, rate, method="gradient", check_every=32, max_iter=100000):
        self.qc = qc
        self.program = qc.program
        self.rate = float(rate)
        self.qng = method.lower() == "qng"
        self.check_every = int(check_every)
        self.max_iter = int(max_iter)
        self.psi0 = qc._psi0()
        self._adjoint = True

    def energy_grad(self, theta):
        """(E [1], dE/dtheta [1, P]) at a device parameter row [1, P]."""
        if self._adjoint:
            try:
                return self.program.energy_grad(theta, self.qc.H, self.psi0)
            except NotImplementedError:
                self._adjoint = False  # fSim rows: the reference's derivative states instead
        E = self.program.energy_grad(theta, self.qc.H, self.psi0, want_grad=False)[0]
        psi = self.program.run(theta, self.psi0)
        d = self.program.gradient_states(theta, self.psi0)
        plus = engine.expect(psi + d, self.qc.H)
        minus = engine.expect(psi - d, self.qc.H)
        return E, ((plus - minus) / 2).reshape(1, -1)

    def step(self, theta, g):
        """theta - rate * (g, or pinv(F) g for QNG with F the QFIM at theta)."""
        if not self.qng:
            return theta - self.rate * g
        psi = self.program.run(theta, self.psi0)
        F = engine.qfim(psi, self.program.gradient_states(theta, self.psi0))
        Finv = torch.linalg.pinv(F, atol=0.0, rtol=1e-15, hermitian=False)
        return theta - self.rate * (Finv @ g.reshape(-1, 1)).reshape(1, -1)

    def run(self, theta0, epsilon, verbose=False):
        """Iterate from theta0 (host [P]); returns (thetas [T+1, P] device, energies [T+1] host, T).

        Row t of the history is theta_t (row 0 the start); iteration t (1-based) produced row t, and the run
        stops after the first iteration with |E_t - E_{t-1}| <= epsilon or after max_iter iterations."""
        dev = self.program.dev
        theta = torch.as_tensor(np.asarray(theta0, dtype=np.float64), device=dev).reshape(1, -1)
        E, g = self.energy_grad(theta)
        thetas, energies_dev = [theta], [E]
        energies = [float(E[0])]  # one read for the starting energy
        T = 0
        diff = 1.0
        while True:
            block_start = len(thetas)
            for _ in range(min(self.check_every, self.max_iter - T)):
                theta = self.step(thetas[-1], g)
                E, g = self.energy_grad(theta)
                thetas.append(theta)
                energies_dev.append(E)
            new = torch.cat(energies_dev[block_start:]).cpu().numpy()
            stop = None
            for j, e in enumerate(new):
                if verbose and T % 100 == 0:  # the reference's progress line, before iteration T's energy
                    print(f"On iteration {T}, energy = {energies[-1]}, diff is {diff}")
                T += 1
                diff = abs(float(e) - energies[-1])
                energies.append(float(e))
                if diff <= epsilon or T >= self.max_iter:
                    stop = block_start + j
                    break
            if stop is not None:
                del thetas[stop + 1:]
                return torch.cat(thetas), np.asarray(energies), T


def batched_measures(qc, thetas, rows=256):
    """(magic, Q, GKP) [R] host arrays of the states of parameter rows `thetas` [R, P] (device), evaluated
    `rows` states at a time: Renyi-2 magic (measure.py:318-349), Meyer-Wallach Q (measure.py:226-237) and GKP
    = M_1/2 / (2 ln 2) (measure.py:361-368)."""
    mags, qs, gkps = [], [], []
    for i in range(0, thetas.shape[0], rows):
        psi = qc.program.run(thetas[i:i + rows], qc._psi0())
        mags.append(engine.magic(psi, 2.0))
        qs.append(engine.mw(psi))
        gkps.append(engine.magic(psi, 0.5) / (2 * np.log(2)))
    out = torch.stack([torch.cat(mags), torch.cat(qs), torch.cat(gkps)]).cpu().numpy()
    return out[0], out[1], out[2]

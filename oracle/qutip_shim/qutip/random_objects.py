"""qutip.random_objects subset (Haar kets/unitaries via QR of a Ginibre matrix)."""
import numpy as np

from . import Qobj

_rng = np.random.default_rng(12345)


def rand_unitary_haar(N=2, dims=None):
    z = (_rng.standard_normal((N, N)) + 1j * _rng.standard_normal((N, N))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    q = q * (d / np.abs(d))
    return Qobj(q, dims=dims if dims is not None else [[N], [N]])


def rand_ket_haar(N=2, dims=None):
    v = _rng.standard_normal(N) + 1j * _rng.standard_normal(N)
    v /= np.linalg.norm(v)
    return Qobj(v.reshape(-1, 1), dims=dims if dims is not None else [[N], [1]])

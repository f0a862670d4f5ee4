"""qutip.states subset."""
import numpy as np

from . import basis, tensor


def bell_state(state="00"):
    s = 1 / np.sqrt(2)
    z, o = basis(2, 0), basis(2, 1)
    if state == "00":
        return (tensor(z, z) + tensor(o, o)) * s
    if state == "01":
        return (tensor(z, z) - tensor(o, o)) * s
    if state == "10":
        return (tensor(z, o) + tensor(o, z)) * s
    if state == "11":
        return (tensor(z, o) - tensor(o, z)) * s
    raise ValueError(state)

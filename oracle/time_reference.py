"""Time the reference's own `PQC.run` (circuit.py:118-125) on the CPU, over the QuTiP restatement in
`oracle/qutip_shim` (QuTiP 4.7.2 itself is not installable here).  Test infrastructure: a CPU baseline row for
the hardware-efficient ladder at sizes the reference's per-gate operator rebuild can hold, beside the numpy
oracle on the same circuits.

Usage (development container only; the reference is not shipped):
    OMP_NUM_THREADS=1 python oracle/time_reference.py /path/to/reference/checkout
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def main(ref_root):
    sys.path.insert(0, os.path.join(HERE, "qutip_shim"))
    sys.path.insert(0, ref_root)
    sys.path.insert(0, REPO)
    sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
    import pyramaterised as ref
    import recipes
    from oracle import pqc_oracle as O

    rows = []
    for N in (8, 10, 12):
        c = recipes.he_ladder(ref, N, N)
        ours = recipes.he_ladder(__import__("pyramaterised_gb300"), N, N)
        rng = np.random.default_rng(N)
        P = len(c.get_params()) if hasattr(c, "get_params") else 2 * N * N
        thetas = rng.random((3, 2 * N * N)) * 2 * np.pi
        c.run(list(thetas[0]))  # warm-up
        t0 = time.perf_counter()
        for th in thetas:
            c.run(list(th))
        ref_s = (time.perf_counter() - t0) / len(thetas)
        t0 = time.perf_counter()
        for th in thetas:
            O.run(ours.gates, N, th)
        orc_s = (time.perf_counter() - t0) / len(thetas)
        rows.append({"N": N, "L": N, "params": P, "reference_evals_per_s": 1.0 / ref_s,
                     "oracle_evals_per_s": 1.0 / orc_s})
        print(json.dumps(rows[-1]), flush=True)
    return rows


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(__doc__)
    main(sys.argv[1])

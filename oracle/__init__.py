"""CPU oracle for the pyramaterised hot path -- TEST INFRASTRUCTURE ONLY.

Nothing in the product package (`pyramaterised_gb300`) imports this package.
Only `tests/`, `__graft_entry__.smoke()` and the CPU-baseline legs of
`bench.py` use it, and only as the checker / the timed CPU baseline.

Contents
--------
* ``pqc_oracle``      -- numpy FP64 restatement of the reference's gate
  semantics, ``PQC.run``, ``take_derivative``/``get_gradients``, ``cost``,
  ``get_QFI`` and ``get_gradient_vector`` (citations per function).
* ``measures_oracle`` -- restatement of the capacity measures: the
  fidelity histogram + KL expressibility, Meyer-Wallach Q, Renyi/GKP magic
  (both the reference's conversion-matrix form and a Walsh-Hadamard form).
* ``qutip_shim``      -- a restatement of the QuTiP 4.7.2 subset the
  reference calls, used in a development container to execute the
  reference's own Python and generate the golden vectors under
  ``tests/golden``.  It cannot travel to machines without the reference.

Parity anchoring: the oracle reproduces the reference's own known answers
(`tests.py:158-213` qg-circuit energy 0.46135870050914374 and effective
dimension 12; `tests.py:103-128` NPQC QFIM identity; `tests.py:284-295`
Bell-state magic/GKP 0 and Q 1; `tests.py:64-87` gate amplitudes) and the
golden vectors produced by the reference code itself on the shim.
"""

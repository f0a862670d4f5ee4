"""pyramaterised_gb300: the pyramaterised hot path on a GB300 GPU.

Same surface as the reference package (`pyramaterised/__init__.py`):
`from .circuit import *` plus the `measure`, `gates` and `templates`
modules.  States live on the GPU as torch complex128 tensors; the
arithmetic runs in hand-written sm_103a kernels behind the C ABI declared in
`include/pyramaterised_gb300.h`.
"""
from .circuit import *  # noqa: F401,F403
from .circuit import PQC, BasisState, basis_product  # noqa: F401
from . import measure  # noqa: F401
from . import gates  # noqa: F401
from . import templates  # noqa: F401
from . import hamiltonian  # noqa: F401
from .hamiltonian import PauliSum  # noqa: F401

__version__ = "0.1.0"

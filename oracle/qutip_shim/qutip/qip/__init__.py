"""qutip.qip subset: only ``operations`` is used by pyramaterised."""
from . import operations  # noqa: F401

"""Stand-in for cupyx: only the jit submodule is provided."""
from . import jit  # noqa: F401

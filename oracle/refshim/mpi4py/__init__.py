"""Stand-in for mpi4py: a single-rank communicator."""
from . import MPI  # noqa: F401

"""Single-rank stand-in for mpi4py (oracle test infrastructure only)."""

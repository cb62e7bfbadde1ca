"""CPU oracle for the GPU path (test infrastructure only; see oracle.py)."""

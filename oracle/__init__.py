"""CPU oracle for the simpois path (test infrastructure only; see oracle.py)."""

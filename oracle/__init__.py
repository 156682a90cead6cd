"""CPU checkers for the CUDA path (test infrastructure; see oracle.py)."""

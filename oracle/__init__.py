"""CPU oracle for the Jaccard hot path -- test infrastructure only (see oracle.py)."""
